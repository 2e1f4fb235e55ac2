"""CPU checks of the product library: it loads, exports every entry point
include/cdft.h declares, and its host-only maths agrees with the oracle."""
import ctypes

import numpy as np
import os
import re

import pytest

from conftest import ROOT, golden


def declared_functions():
    with open(os.path.join(ROOT, "include", "cdft.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(cdft_\w+)\s*\(", text, re.M)))


def test_header_lists_match_binding():
    import classicaldft_gb300 as cd
    assert declared_functions() == sorted(cd.C_FUNCTIONS)


def test_library_exports_every_declared_symbol():
    import classicaldft_gb300 as cd
    if not os.path.exists(cd.LIB_PATH):
        cd_build = __import__("classicaldft_gb300.build", fromlist=["build"])
        cd_build.build()
    L = ctypes.CDLL(cd.LIB_PATH)
    for name in declared_functions():
        assert hasattr(L, name), name


def test_bh_diameter_matches_reference(oracle):
    import classicaldft_gb300 as cd
    g = golden("bulk")
    # the same integral to 1e-15; the product and the oracle sum in the same order
    assert cd.bh_diameter(1.0, 1.0, 3.0, 0.8) == pytest.approx(g["bulk.lj_hsd_kT0.8"][0], rel=1e-15)
    assert cd.bh_diameter(1.0, 1.0, 3.0, 1.0) == pytest.approx(g["bulk.lj_hsd_kT1.0"][0], rel=1e-15)
    assert cd.bh_diameter(1.0, 1.0, 2.5, 0.7) == oracle.bh_diameter(2.5, 0.7)


def test_lattice_rules():
    import classicaldft_gb300 as cd
    L = cd.Lattice(0.2, [6.4, 6.4, 6.4])
    assert (L.Nx(), L.Ny(), L.Nz()) == (32, 32, 32)
    assert L.getX(0) == pytest.approx(-3.2)
    with pytest.raises(RuntimeError):
        cd.Lattice(0.3, [1.0, 1.0, 1.0])


@pytest.mark.parametrize("tag,dx,n,hsd", [("w_d1_dx0.2_n16", 0.2, 16, 1.0), ("w_d0.9786_dx0.1_n16", 0.1, 16, 0.9786),
                                          ("w_d1.3_dx0.25_n12", 0.25, 12, 1.3)])
def test_product_weights_match_reference(tag, dx, n, hsd):
    import numpy as np
    import classicaldft_gb300 as cd
    g = golden("weights")
    w = cd.fmt_weights((n, n, n), dx, hsd)
    for a in range(11):
        np.testing.assert_allclose(w[a].ravel(), g[tag + ".w%d" % a], rtol=0, atol=1e-14)


@pytest.mark.parametrize("n", [7, 16, 30, 48, 64, 80, 96, 112, 128, 144, 160, 256])
def test_radix_candidates(n):
    """Every plan the FFT autotuner tries is a factorisation of n into supported radices, the default first."""
    import classicaldft_gb300 as cd
    cands = cd.radix_candidates(n)
    assert 1 <= len(cands) <= 12
    assert len({tuple(c) for c in cands}) == len(cands)
    for c in cands:
        assert int(np.prod(c)) == n
        assert all(r in (2, 4, 8) or (r % 2 == 1 and all(r % q for q in range(3, r, 2))) for r in c)


def test_create_rejects_bad_systems_before_touching_the_gpu():
    """Grid lengths with a prime factor above 31 and hsd < dx are refused (CDFT_ERR_ARG = 4)
    before any device allocation, as the reference refuses them in its constructors."""
    import classicaldft_gb300 as cd
    L = cd.lib()
    for nx, hsd in ((37, 1.0), (32, 0.05)):
        p = cd.Params(nx, 32, 32, 0.1, cd.WHITEBEAR_I, 1.0, 0.0, hsd, 0, 1.0, 1.0, 3.0, 1.0, 0.0, -1.0, cd.FP64)
        h = ctypes.c_void_p()
        assert L.cdft_create(ctypes.byref(p), ctypes.byref(h)) == 4
        assert not h.value


def test_double_float_log_table_is_the_generated_one():
    """cdft_df_log_table.h (the df64 logarithm's table of log F and 1/F, F = 1 + j/128) is
    what its generator writes, and every entry's float pair carries its value to 2^-48."""
    import subprocess
    import sys
    from decimal import Decimal, getcontext
    csrc = os.path.join(ROOT, "classicaldft_gb300", "csrc")
    out = subprocess.run([sys.executable, os.path.join(csrc, "gen_df_log_table.py")], capture_output=True, text=True, check=True).stdout
    with open(os.path.join(csrc, "cdft_df_log_table.h")) as f:
        assert f.read() == out
    rows = re.findall(r"^\s*\{([^}]*)\}", out, re.M)
    assert len(rows) == 97
    getcontext().prec = 50
    for i, r in enumerate(rows):
        v = [np.float32(x.strip().rstrip("f")) for x in r.split(",")]
        F = 1 + Decimal(i - 32) / 128
        for (h, l), exact in (((v[0], v[1]), F.ln()), ((v[2], v[3]), 1 / F)):
            assert abs(Decimal(float(h)) + Decimal(float(l)) - exact) <= abs(exact) * Decimal(2) ** -48
            assert abs(float(l)) <= abs(float(h)) * 2.0 ** -23 or h == 0
