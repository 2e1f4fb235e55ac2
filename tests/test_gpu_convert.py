"""The integer-pipe FP64 <-> FP32 conversions used by the row passes are
bit-identical to the hardware round-to-nearest-even conversions: every float
bit pattern, and every double exponent with fractions at the rounding
boundaries (normal and subnormal results), checked on the GPU by a small
standalone program compiled from tests/gpu_checks/convert_check.cu."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.gpu
def test_integer_conversions_match_hardware():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "convert_check")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        os.path.join(HERE, "gpu_checks", "convert_check.cu"), "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout
    counts = {m.group(1): (int(m.group(2)), int(m.group(3))) for m in re.finditer(r"(\S+)_checked (\d+) mismatches (\d+)", out)}
    assert counts["f32_to_f64"] == (1 << 32, 0), out
    assert counts["f64_to_f32"][0] == (1 << 16) * 4096 and counts["f64_to_f32"][1] == 0, out
