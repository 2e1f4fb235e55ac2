"""Log_Det's device probe generator on the CPU (tests/cpp/mt_probe_phases.cpp restates it)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_log_det_probe_generator_phases_match_std_mt19937(tmp_path):
    """Log_Det's device probe generator, restated on the host (tests/cpp/mt_probe_phases.cpp):
    the three-phase twist into a second state copy and the top bit of each tempered word give,
    draw for draw over calls of lengths that are not multiples of 624, what std::mt19937(seed)
    with uniform_int_distribution<>(0, 1) gives (the library's Lemire mapping of range 2)."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "mt_probe_phases")
    subprocess.check_call(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cpp", "mt_probe_phases.cpp"), "-o", exe])
    assert subprocess.check_output([exe], text=True).strip() == "ok"
