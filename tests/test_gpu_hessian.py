"""Hessian-vector products (cdft_hessian_dot_v) on the GPU against the
reference's own DFT::matrix_dot_v1 (tests/golden/hessian.npz) and the oracle.

Tolerances: FP64 mode 1e-12 of max|Hv| (FFT roundoff); FP32 bulk mode 2e-5."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

MODELS = [("Rosenfeld", "ROSENFELD", 1, 0), ("RSLT", "RSLT_MODEL", 1, 0), ("esFMT", "ESFMT", 1, 0), ("esFMT_A1_Bm1", "ESFMT", 1, -1),
          ("WhiteBearI", "WHITEBEAR_I", 1, 0), ("WhiteBearII", "WHITEBEAR_II", 1, 0)]


@pytest.fixture(scope="module")
def cd():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import classicaldft_gb300 as m
    m.lib()
    return m


def _v(oracle, shape, seed=77):
    return 0.3 * (oracle.fill_noise(shape, 1.0, 1.0, seed) - 1.0)


@pytest.mark.parametrize("tag,model,A,B", MODELS)
def test_hessian_models_vs_reference(cd, oracle, tag, model, A, B):
    g = golden("hessian")
    shape = (16, 16, 16)
    c = cd.Context(shape, 0.2, getattr(cd, model), hsd=1.0, es_A=A, es_B=B)
    rho = oracle.fill_noise(shape, 0.6, 0.2, 11)
    c.set_density(rho)
    c.set_chem_potential(0.0)
    c.eval()
    hv = c.hessian_dot_v(_v(oracle, shape))
    ref = g["h16.%s.Hv" % tag].reshape(shape)
    assert np.max(np.abs(hv - ref)) <= 1e-12 * np.max(np.abs(ref))
    c.close()


def test_hessian_lj_vs_reference(cd, oracle):
    g = golden("hessian")
    shape = (16, 16, 16)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=float(g["hlj16.hsd"][0]), lj=True, kT=0.8)
    c.set_density(oracle.fill_noise(shape, 0.3, 0.1, 5))
    hv = c.hessian_dot_v(_v(oracle, shape))
    ref = g["hlj16.Hv"].reshape(shape)
    assert np.max(np.abs(hv - ref)) <= 1e-12 * np.max(np.abs(ref))
    c.close()


@pytest.mark.parametrize("shape,prec,tol", [((48, 48, 48), "FP64", 1e-12), ((40, 36, 30), "FP64", 1e-12),
                                            ((48, 48, 48), "FP32", 2e-5), ((128, 32, 128), "FP32", 2e-5),
                                            ((128, 32, 128), "FP64", 1e-12), ((32, 16, 256), "FP32", 2e-5),
                                            ((128, 128, 128), "FP64", 1e-12), ((128, 128, 256), "FP64", 1e-12)])
def test_hessian_vs_oracle(cd, oracle, shape, prec, tol):
    """The last two shapes take the double-float-spectra path of FP64 (compile-time plans on
    every axis), the second with 256-point z rows copied in two boxes."""
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=getattr(cd, prec))
    rho = oracle.fill_noise(shape, 0.4, 0.3, 9)
    c.set_density(rho)
    v = _v(oracle, shape, 21) * rho
    hv = c.hessian_dot_v(v)
    o = oracle.Oracle(shape, 0.1, "WhiteBearI", hsd=hsd, lj=True, kT=0.8)
    ref = o.hessian_dot_v(rho, v)
    assert np.max(np.abs(hv - ref)) <= tol * np.max(np.abs(ref))
    c.close()


def test_hessian_symmetric_and_derivative_of_dF(cd, oracle):
    """u.Hv = v.Hu, and a central difference of dF along v gives Hv."""
    shape = (32, 32, 32)
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    rho = oracle.fill_noise(shape, 0.4, 0.3, 2)
    u = _v(oracle, shape, 31) * rho
    v = _v(oracle, shape, 32) * rho
    c.set_chem_potential(0.0)
    c.set_density(rho)
    hu = c.hessian_dot_v(u)
    hv = c.hessian_dot_v(v)
    assert abs(np.dot(u.ravel(), hv.ravel()) - np.dot(v.ravel(), hu.ravel())) <= 1e-12 * abs(np.dot(u.ravel(), hv.ravel()))
    eps = 1e-5
    c.set_density(rho + eps * v)
    dp = c.eval()[1]
    c.set_density(rho - eps * v)
    dm = c.eval()[1]
    fd = (dp - dm) / (2 * eps)
    assert np.max(np.abs(fd - hv)) <= 1e-7 * np.max(np.abs(hv))
    c.close()


def test_ddft_dynamical_matrix_vs_reference(cd, oracle):
    g = golden("hessian")
    shape = (16, 16, 16)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=float(g["hlj16.hsd"][0]), lj=True, kT=0.8)
    rho = oracle.fill_noise(shape, 0.3, 0.1, 5)
    c.set_density(rho)
    out = c.ddft_matrix_dot_v(_v(oracle, shape))
    ref = g["hlj16.GHv"].reshape(shape)
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))
    # and at a size the golden does not cover, against the oracle
    shape = (40, 36, 30)
    c2 = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=float(g["hlj16.hsd"][0]), lj=True, kT=0.8)
    rho = oracle.fill_noise(shape, 0.3, 0.2, 6)
    v = _v(oracle, shape, 8) * rho
    c2.set_density(rho)
    out = c2.ddft_matrix_dot_v(v)
    o = oracle.Oracle(shape, 0.1, "WhiteBearI", hsd=float(g["hlj16.hsd"][0]), lj=True, kT=0.8)
    ref = o.ddft_matrix_dot_v(rho, v)
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))
    c.close()
    c2.close()
