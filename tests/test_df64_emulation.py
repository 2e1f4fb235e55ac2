"""The double-float arithmetic's error bounds, on the CPU: tests/cpp/df64_fft_emulation.cpp
restates in float32 the 128- and 256-point transforms of the FP64 evaluation, once with the
renormalising double-word operations and once as the device computes them (sums without the
closing FastTwoSum, fused two-term twiddle products, renormalisation only where values leave
the transform), against a long-double DFT. Both stay normwise at the 2^-48 level: the lazy
scheme within 4x of the renormalising one and below 1e-13 of max |output| on random,
near-constant and DC-dominated inputs."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "df64_fft_emulation.cpp")


def test_lazy_double_float_transforms_stay_normwise(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "df64_fft_emulation")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", SRC, "-o", exe])
    rows = [line.split() for line in subprocess.check_output([exe], text=True).splitlines() if line.strip()]
    assert len(rows) == 12  # 2 lengths x 3 input kinds x 2 directions
    for n, kind, direction, err_r, err_l in rows:
        err_r, err_l = float(err_r), float(err_l)
        assert err_r < 3e-14, (n, kind, direction, err_r)
        assert err_l < 1e-13, (n, kind, direction, err_l)
        assert err_l < 4 * err_r, (n, kind, direction, err_r, err_l)


def test_double_float_logarithm_and_reciprocal(tmp_path):
    """tests/cpp/df64_log_emulation.cpp restates df_log1p, df_log and df_rcp operation for
    operation, with the generated table, over 200,000 arguments of each (eta-like, tiny,
    around the reduction threshold; densities from 1e-30 to 1e25; reciprocals of both
    signs from 1e-20 to 1e20): relative errors at the 2^-48 level."""
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "df64_log_emulation")
    src = os.path.join(ROOT, "tests", "cpp", "df64_log_emulation.cpp")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I",
                           os.path.join(ROOT, "classicaldft_gb300", "csrc"), src, "-o", exe])
    e_log1p, e_log, e_rcp = (float(v) for v in subprocess.check_output([exe], text=True).split())
    assert e_log1p < 2e-14, e_log1p
    assert e_log < 1.5e-14, e_log
    assert e_rcp < 1e-14, e_rcp

