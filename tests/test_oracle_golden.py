"""Pins the FP64 CPU oracle to outputs of the reference's own sources.

The golden arrays come from oracle/_ref/ref_driver (the reference compiled as
it lies, with stand-ins for its absent third-party libraries). Tolerances:
weights, pointwise Phi and bulk thermodynamics agree to the last bits; full
evaluations to FFT roundoff (F 1e-12 relative, dF 1e-12 absolute, well inside
the 1e-12 / 1e-10 bar the GPU FP64 path is held to).
"""
import numpy as np
import pytest

from conftest import golden

MODELS = ["Rosenfeld", "RSLT", "esFMT", "WhiteBearI", "WhiteBearII"]


@pytest.mark.parametrize("tag,dx,n,hsd", [("w_d1_dx0.2_n16", 0.2, 16, 1.0), ("w_d0.9786_dx0.1_n16", 0.1, 16, 0.9786),
                                          ("w_d1.3_dx0.25_n12", 0.25, 12, 1.3)])
def test_fmt_weights(oracle, tag, dx, n, hsd):
    g = golden("weights")
    W = oracle.Oracle(n, dx, "WhiteBearI", hsd=hsd).weights()
    for a in range(11):
        np.testing.assert_allclose(W[a].ravel(), g[tag + ".w%d" % a], rtol=0, atol=1e-14)


def test_weight_sum_rules(oracle):
    # sum w_eta = pi d^3/6, sum w_s = pi d^2 = trace of sum w_T, odd weights sum to 0
    for n, dx, d in [(16, 0.2, 1.0), (16, 0.1, 0.9786)]:
        W = oracle.Oracle(n, dx, "WhiteBearI", hsd=d).weights()
        s = W.reshape(11, -1).sum(axis=1)
        assert abs(s[0] - np.pi * d ** 3 / 6) < 1e-8
        assert abs(s[1] - np.pi * d ** 2) < 1e-7
        assert abs(s[5] + s[8] + s[10] - np.pi * d ** 2) < 1e-7
        assert np.all(np.abs(s[[2, 3, 4, 6, 7, 9]]) < 1e-14)


@pytest.mark.parametrize("model,name,A,B", [("Rosenfeld", "Rosenfeld", 1, 0), ("RSLT", "RSLT", 1, 0), ("esFMT", "esFMT", 1, 0),
                                            ("esFMT_A1_Bm1", "esFMT", 1, -1), ("WhiteBearI", "WhiteBearI", 1, 0),
                                            ("WhiteBearII", "WhiteBearII", 1, 0)])
def test_phi_pointwise(oracle, model, name, A, B):
    g = golden("phi")
    inp = g["phi.inputs"].reshape(-1, 19)
    P = g["phi.%s.phi" % model]
    D = g["phi.%s.dphi" % model].reshape(-1, 19)
    for i in range(len(inp)):
        v, d = oracle.phi(name, inp[i], A, B)
        assert v == P[i]
        np.testing.assert_array_equal(d, D[i])


@pytest.mark.parametrize("model", MODELS)
def test_bulk_thermodynamics(oracle, model):
    g = golden("bulk")
    o = oracle.Oracle(16, 0.2, model, hsd=1.0)
    for key, f in [("mu", o.mu_times_beta), ("omega", o.omega_times_beta_over_volume),
                   ("fhelm", o.fhelmholtz_times_beta_over_volume)]:
        got = np.array([f(r) for r in g["bulk.rho"]])
        np.testing.assert_allclose(got, g["bulk.%s.%s" % (model, key)], rtol=1e-15, atol=1e-15)


def test_bh_diameter(oracle):
    g = golden("bulk")
    assert oracle.bh_diameter(3.0, 0.8) == pytest.approx(g["bulk.lj_hsd_kT0.8"][0], abs=1e-15)
    assert oracle.bh_diameter(3.0, 1.0) == pytest.approx(g["bulk.lj_hsd_kT1.0"][0], abs=1e-15)


def _check_eval(terms, dF, g, tag, full=True, pos=None):
    for k in ("Omega", "F_id", "F_hs", "F_mf", "F_ext", "mu"):
        ref = g[tag + "." + k][0]
        assert abs(terms[k] - ref) <= 1e-12 * max(1.0, abs(ref)), (k, terms[k], ref)
    if full:
        np.testing.assert_allclose(dF.ravel(), g[tag + ".dF"], rtol=0, atol=1e-13)
    else:
        np.testing.assert_allclose(dF.ravel()[pos], g[tag + ".dF.sample"], rtol=0, atol=1e-13)
        assert abs(dF.sum() - g[tag + ".dF.sum"][0]) < 1e-11


@pytest.mark.parametrize("model", MODELS)
def test_eval_models_16(oracle, model):
    g = golden("eval_models16")
    o = oracle.Oracle(16, 0.2, model, hsd=1.0)
    rho = oracle.fill_noise((16, 16, 16), 0.6, 0.2, 11)
    np.testing.assert_array_equal(rho.ravel(), g["m16.%s.rho" % model])
    o.set_mu(o.mu_times_beta(0.6))
    st, t, dF, _ = o.eval(rho)
    assert st == 0
    _check_eval(t, dF, g, "m16." + model)


def test_eval_hs32_config1(oracle):
    g = golden("eval_hs32")
    o = oracle.Oracle(32, 0.2, "WhiteBearI", hsd=1.0)
    rho = oracle.fill_noise((32, 32, 32), 0.7, 0.05, 20240601)
    o.set_mu(o.mu_times_beta(0.7))
    st, t, dF, _ = o.eval(rho)
    assert st == 0
    _check_eval(t, dF, g, "hs32", full=False, pos=g["hs32.pos"].astype(np.int64))


def test_eval_lj(oracle):
    g = golden("eval_lj")
    o = oracle.Oracle(24, 0.2, "WhiteBearI", hsd=None, lj=True, kT=0.8)
    assert o.hsd == g["lj24.hsd"][0]
    assert abs(o.a_vdw - g["lj24.a_vdw"][0]) < 1e-13
    np.testing.assert_allclose(o.w_att().ravel(), g["lj24.w_att"], rtol=0, atol=1e-14)
    o.set_mu(o.mu_times_beta(0.01))
    st, t, dF, _ = o.eval(g["lj24.rho"])
    _check_eval(t, dF, g, "lj24")
    o = oracle.Oracle(16, 0.1, "WhiteBearI", hsd=None, lj=True, kT=0.8)
    rho = oracle.fill_noise((16, 16, 16), 0.3, 0.1, 5)
    o.set_mu(o.mu_times_beta(0.3))
    st, t, dF, _ = o.eval(rho)
    _check_eval(t, dF, g, "lj16")
    o = oracle.Oracle(24, 0.2, "WhiteBearI", hsd=None, lj=True, kT=0.8, fixed_mass=g["lj24fm.fixed_mass"][0])
    st, t, dF, r = o.eval(g["lj24.rho"])
    _check_eval(t, dF, g, "lj24fm")
    np.testing.assert_allclose(r.ravel(), g["lj24fm.rho"], rtol=1e-15, atol=0)


def test_fire_hs32_200_steps(oracle):
    g = golden("fire_hs32")
    o = oracle.Oracle(32, 0.2, "WhiteBearI", hsd=1.0)
    rho = oracle.fill_noise((32, 32, 32), 0.7, 0.05, 20240601)
    o.set_mu(o.mu_times_beta(0.7))
    n, rec, r = o.fire(rho, 200)
    assert n == 200
    np.testing.assert_array_equal(rec["dt"], g["fire32.dt"])
    np.testing.assert_array_equal(rec["alpha"], g["fire32.alpha"])
    np.testing.assert_allclose(rec["F"], g["fire32.F"], rtol=1e-14)
    np.testing.assert_allclose(rec["fmax"], g["fire32.fmax"], rtol=1e-9)
    np.testing.assert_allclose(rec["vv"], g["fire32.vv"], rtol=1e-5, atol=1e-12)
    pos = g["fire32.pos"].astype(np.int64)
    np.testing.assert_allclose(r.ravel()[pos], g["fire32.rho_final.sample"], rtol=0, atol=1e-13)


def test_fire_lj24_fixed_mass(oracle):
    g = golden("fire_lj24")
    rho = golden("eval_lj")["lj24.rho"].reshape(24, 24, 24)
    o = oracle.Oracle(24, 0.2, "WhiteBearI", hsd=None, lj=True, kT=0.8, fixed_mass=rho.sum() * 0.2 ** 3)
    n, rec, r = o.fire(rho, 60)
    np.testing.assert_array_equal(rec["dt"], g["firelj.dt"])
    np.testing.assert_allclose(rec["F"], g["firelj.F"], rtol=1e-14)
    np.testing.assert_allclose(rec["fmax"], g["firelj.fmax"], rtol=1e-12)
    np.testing.assert_allclose(r.ravel(), g["firelj.rho_final"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("case,tag,nsteps,dt,dtmax", [("ddft_lj16", "ddft16", 10, 1e-4, 1e-4),
                                                       ("ddft_adapt16", "ddfta", 14, 1e-5, 4e-5)])
def test_ddft(oracle, case, tag, nsteps, dt, dtmax):
    g = golden(case)
    o = oracle.Oracle(16, 0.1, "WhiteBearI", hsd=None, lj=True, kT=0.8)
    rho = oracle.fill_noise((16, 16, 16), 0.3, 0.1, 5)
    n, rec, r = o.ddft(rho, nsteps, dt, dtmax)
    assert n == nsteps
    np.testing.assert_array_equal(rec["dt"], g[tag + ".dt"])
    np.testing.assert_allclose(rec["t"], g[tag + ".t"], rtol=1e-15)
    np.testing.assert_allclose(rec["F"], g[tag + ".F"], rtol=1e-14)
    np.testing.assert_allclose(rec["mass"], g[tag + ".mass"], rtol=1e-15)
    np.testing.assert_allclose(r.ravel(), g[tag + ".rho_final"], rtol=0, atol=1e-14)


def test_fft_roundtrip_and_numpy(oracle):
    rng = np.random.default_rng(0)
    for shape in [(16, 16, 16), (12, 10, 9), (8, 6, 15)]:
        a = rng.standard_normal(shape)
        A = oracle.r2c(a)
        np.testing.assert_allclose(A, np.fft.rfftn(a), rtol=0, atol=1e-12)
        np.testing.assert_allclose(oracle.c2r(A, shape[2]) / a.size, a, rtol=0, atol=1e-13)


def _hess_v(oracle, shape):
    # the reference driver's v_i = 0.3 (2u - 1) from splitmix64(77)
    return 0.3 * (oracle.fill_noise(shape, 1.0, 1.0, 77) - 1.0)


@pytest.mark.parametrize("model,name,A,B", [("Rosenfeld", "Rosenfeld", 1, 0), ("RSLT", "RSLT", 1, 0), ("esFMT", "esFMT", 1, 0),
                                            ("esFMT_A1_Bm1", "esFMT", 1, -1), ("WhiteBearI", "WhiteBearI", 1, 0),
                                            ("WhiteBearII", "WhiteBearII", 1, 0)])
def test_hessian_dot_v_models(oracle, model, name, A, B):
    """Full Hessian times v (DFT::matrix_dot_v1) of every FMT model against the reference."""
    g = golden("hessian")
    shape = (16, 16, 16)
    o = oracle.Oracle(16, 0.2, name, hsd=1.0, es_A=A, es_B=B)
    rho = oracle.fill_noise(shape, 0.6, 0.2, 11)
    h = o.hessian_dot_v(rho, _hess_v(oracle, shape))
    ref = g["h16.%s.Hv" % model].reshape(shape)
    assert np.max(np.abs(h - ref)) <= 1e-15 * max(1.0, np.max(np.abs(ref))) + 1e-16


def test_hessian_dot_v_lj(oracle):
    g = golden("hessian")
    shape = (16, 16, 16)
    hsd = float(g["hlj16.hsd"][0])
    o = oracle.Oracle(16, 0.1, "WhiteBearI", hsd=hsd, lj=True, kT=0.8)
    rho = oracle.fill_noise(shape, 0.3, 0.1, 5)
    h = o.hessian_dot_v(rho, _hess_v(oracle, shape))
    ref = g["hlj16.Hv"].reshape(shape)
    assert np.max(np.abs(h - ref)) <= 1e-15


def test_hessian_is_the_derivative_of_dF(oracle):
    """Central difference of dF along v equals H.v (second-order accurate)."""
    shape = (12, 12, 12)
    o = oracle.Oracle(12, 0.2, "WhiteBearI", hsd=1.0)
    o.set_mu(0.0)
    rho = oracle.fill_noise(shape, 0.5, 0.2, 3)
    v = _hess_v(oracle, shape) * rho
    hv = o.hessian_dot_v(rho, v)
    eps = 1e-5
    dp = o.eval(rho + eps * v)[2]
    dm = o.eval(rho - eps * v)[2]
    fd = (dp - dm) / (2 * eps)
    assert np.max(np.abs(fd - hv)) <= 1e-8 * np.max(np.abs(hv))


def test_ddft_dynamical_matrix_dot_v(oracle):
    """DDFT::matrix_dot_v1 (g . H v) of the LJ fluid against the reference."""
    g = golden("hessian")
    shape = (16, 16, 16)
    o = oracle.Oracle(16, 0.1, "WhiteBearI", hsd=float(g["hlj16.hsd"][0]), lj=True, kT=0.8)
    rho = oracle.fill_noise(shape, 0.3, 0.1, 5)
    out = o.ddft_matrix_dot_v(rho, _hess_v(oracle, shape))
    ref = g["hlj16.GHv"].reshape(shape)
    assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("tag,order,seed,samples,has_zero,dynamic",
                         [("o10", 10, 1234, 3, False, False), ("o40", 40, 1234, 3, False, False),
                          ("zero", 20, 77, 2, True, False), ("ddft", 16, 4321, 2, True, True)])
def test_log_det_vs_reference(oracle, tag, order, seed, samples, has_zero, dynamic):
    """Log_Det::calculate_log_det (src/Log_Det.cpp:84-166), compiled from the reference,
    against the oracle's restatement: same seed, same +-1 probes, same recurrence."""
    g = golden("spectral")
    o = oracle.Oracle(16, 0.2, "WhiteBearI", hsd=1.0)
    rho = oracle.fill_noise((16, 16, 16), 0.6, 0.2, 11)
    lo, hi = g["sp16.logdet.ddft.bounds" if dynamic else "sp16.logdet.bounds"]
    val, var = o.log_det(rho, order, hi, lo, seed, samples, has_zero=has_zero, dynamic=dynamic)
    ref = g["sp16.logdet." + tag]
    assert abs(val - ref[0]) <= 1e-12 * abs(ref[0])
    assert abs(var - ref[1]) <= 1e-9 * abs(ref[1])


@pytest.mark.parametrize("tag,dx,rho0,amp,seed,lj", [("sp16", 0.2, 0.6, 0.2, 11, False), ("splj16", 0.1, 0.3, 0.1, 5, True)])
def test_spectrum_pins_oracle_hessian(oracle, tag, dx, rho0, amp, seed, lj):
    """The reference's dense Hessians (their LAPACK eigenpairs in the golden file) and the
    oracle's Hessian product: H y = lambda y for the isolated extreme pairs."""
    g = golden("spectral")
    kw = dict(hsd=float(g["splj16.hsd"][0]), lj=True, kT=0.8) if lj else dict(hsd=1.0)
    o = oracle.Oracle(16, dx, "WhiteBearI", **kw)
    rho = oracle.fill_noise((16, 16, 16), rho0, amp, seed)
    eig = g[tag + ".eig"]
    assert g[tag + ".asym"][0] <= 1e-15 * np.abs(eig).max()
    for name, lam in (("evec_min", eig[0]), ("evec_max", eig[-1])):
        y = g[tag + "." + name]
        hy = o.hessian_dot_v(rho, y.reshape(16, 16, 16)).ravel()
        assert np.linalg.norm(hy - lam * y) <= 1e-12 * np.abs(eig).max()
