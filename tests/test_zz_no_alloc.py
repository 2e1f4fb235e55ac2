"""The allocation-free entry point, cdft_number_of_atoms_noalloc.

Callers that cannot call cudaMalloc (they hand this library only device memory
from their own pool, whose budget a cudaMalloc would bypass) use it to get
sum(rho) * dV of a device density. Its scratch is a static device array, so this
test checks, through the C ABI, that two calls in a row each agree with the
number of atoms the regular evaluation entry point (cdft_eval) reports, within
the FP64 tolerance of the parity tests; that the full capacity (2^25 points,
4096 blocks filling the scratch up to its result slot) agrees with an exactly
rounded host sum; that a call on a side stream agrees too; and that sizes beyond
the array are rejected. The file is named to be collected last.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, dev, n, dV, stream):
    out = ctypes.c_double(-1.0)
    rc = lib.cdft_number_of_atoms_noalloc(ctypes.c_void_p(dev.data_ptr()), n, dV, stream, ctypes.byref(out))
    return rc, out.value


def test_number_of_atoms_noalloc_matches_eval():
    import torch
    import classicaldft_gb300 as cd
    from oracle import pyoracle
    shape, dx = (40, 36, 30), 0.15
    c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=1.0)
    lib = cd.lib()
    for seed in (7, 8):  # two calls in a row, each on fresh data
        rho = pyoracle.fill_noise(shape, 0.5, 0.3, seed)
        c.set_density(rho)
        terms, _ = c.eval(want_dF=False)
        dev = torch.from_numpy(rho.ravel()).to("cuda")
        torch.cuda.synchronize()
        rc, val = _call(lib, dev, rho.size, c.info.dV, None)
        assert rc == 0
        assert abs(val - terms["N"]) <= 1e-13 * abs(terms["N"]), (val, terms["N"])
    c.close()


def test_number_of_atoms_noalloc_full_capacity_and_side_stream():
    import torch
    import classicaldft_gb300 as cd
    lib = cd.lib()
    n, dV = 1 << 25, 1e-3
    g = torch.Generator().manual_seed(11)
    host = (torch.rand(n, generator=g, dtype=torch.float64) * 0.9 + 0.05).numpy()
    exact = math.fsum(host) * dV
    dev = torch.from_numpy(host).to("cuda")
    torch.cuda.synchronize()
    for _ in range(2):  # the largest size, twice in a row
        rc, val = _call(lib, dev, n, dV, None)
        assert rc == 0
        assert abs(val - exact) <= 1e-13 * abs(exact), (val, exact)
    side = torch.cuda.Stream()
    small = dev[: 1000003]
    exact_small = math.fsum(host[: 1000003]) * dV
    with torch.cuda.stream(side):
        rc, val = _call(lib, small, small.numel(), dV, ctypes.c_void_p(side.cuda_stream))
    assert rc == 0
    assert abs(val - exact_small) <= 1e-13 * abs(exact_small), (val, exact_small)
    del dev
    torch.cuda.empty_cache()


def test_number_of_atoms_noalloc_rejects_oversize_and_bad_args():
    import classicaldft_gb300 as cd
    lib = cd.lib()
    out = ctypes.c_double()
    assert lib.cdft_number_of_atoms_noalloc(ctypes.c_void_p(16), (1 << 25) + 1, 1.0, None, ctypes.byref(out)) == cd.ERR_ARG
    assert lib.cdft_number_of_atoms_noalloc(None, 10, 1.0, None, ctypes.byref(out)) == cd.ERR_ARG
