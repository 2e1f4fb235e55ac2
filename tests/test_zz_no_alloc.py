"""The allocation-free entry point, cdft_number_of_atoms_noalloc.

Callers that cannot call cudaMalloc (they pass only device pointers from their
own memory pool, or must not allocate between launches they record into a CUDA
graph) use it to get sum(rho) * dV of a device density. Its scratch is a static
device array, so this test checks, through the C ABI, that two calls in a row
each agree with the number of atoms the regular evaluation entry point
(cdft_eval) reports, within the FP64 tolerance of the parity tests. The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
        out = ctypes.c_double(-1.0)
        rc = lib.cdft_number_of_atoms_noalloc(ctypes.c_void_p(dev.data_ptr()), rho.size, c.info.dV, None,
                                              ctypes.byref(out))
        assert rc == 0
        assert abs(out.value - terms["N"]) <= 1e-13 * abs(terms["N"]), (out.value, terms["N"])


def test_number_of_atoms_noalloc_rejects_oversize_and_bad_args():
    import classicaldft_gb300 as cd
    lib = cd.lib()
    out = ctypes.c_double()
    assert lib.cdft_number_of_atoms_noalloc(ctypes.c_void_p(16), (1 << 25) + 1, 1.0, None, ctypes.byref(out)) == cd.ERR_ARG
    assert lib.cdft_number_of_atoms_noalloc(None, 10, 1.0, None, ctypes.byref(out)) == cd.ERR_ARG
