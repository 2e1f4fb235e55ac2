"""GPU parity: the CUDA path through the C ABI against the reference's golden
vectors (tests/golden) and the FP64 CPU oracle.

Every comparison feeds both sides the same hard-sphere diameter: the
reference's analytic cell-averaged weights are so ill-conditioned near the
sphere surface that a one-ulp change of the diameter moves Omega by ~1e-9
relative (the diameter itself is checked separately, to 1e-15).

Tolerances (FP64 mode): Omega within 1e-12 relative, dF/drho within 1e-10
absolute (dF carries the reference's x dV, so the bar on dF is 1e-10 * dV).
FP32 mode: Omega within 2e-6 relative, dF within 2e-6 of max|dF|.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

MODELS = ["Rosenfeld", "RSLT", "esFMT", "WhiteBearI", "WhiteBearII"]


@pytest.fixture(scope="module")
def cd():
    import classicaldft_gb300 as cd
    cd.lib()
    return cd


def model_id(cd, name):
    return {"Rosenfeld": cd.ROSENFELD, "RSLT": cd.RSLT_MODEL, "esFMT": cd.ESFMT, "WhiteBearI": cd.WHITEBEAR_I,
            "WhiteBearII": cd.WHITEBEAR_II}[name]


def check_terms(terms, g, tag, rtol=1e-12):
    for k in ("Omega", "F_id", "F_hs", "F_mf", "F_ext", "mu"):
        ref = g[tag + "." + k][0]
        assert abs(terms[k] - ref) <= rtol * max(1.0, abs(ref)), (tag, k, terms[k], ref)


def dF_tol(dx):
    return 1e-10 * dx ** 3


def test_weights_match_reference(cd):
    g = golden("weights")
    for tag, dx, n, hsd in [("w_d1_dx0.2_n16", 0.2, 16, 1.0), ("w_d0.9786_dx0.1_n16", 0.1, 16, 0.9786),
                            ("w_d1.3_dx0.25_n12", 0.25, 12, 1.3)]:
        c = cd.Context(n, dx, cd.WHITEBEAR_I, hsd=hsd)
        w, _ = c.weights()
        for a in range(11):
            np.testing.assert_allclose(w[a].ravel(), g[tag + ".w%d" % a], rtol=0, atol=1e-14)


@pytest.mark.parametrize("model", MODELS)
def test_eval_models_fp64(cd, oracle, model):
    g = golden("eval_models16")
    c = cd.Context(16, 0.2, model_id(cd, model), hsd=1.0)
    rho = oracle.fill_noise((16, 16, 16), 0.6, 0.2, 11)
    c.set_chem_potential(c.bulk(0.6)["mu"])
    c.set_density(rho)
    terms, dF = c.eval()
    check_terms(terms, g, "m16." + model)
    np.testing.assert_allclose(dF.ravel(), g["m16.%s.dF" % model], rtol=0, atol=dF_tol(0.2))


def test_eval_config1_hs32(cd, oracle):
    g = golden("eval_hs32")
    c = cd.Context(32, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_chem_potential(c.bulk(0.7)["mu"])
    c.set_density(oracle.fill_noise((32, 32, 32), 0.7, 0.05, 20240601))
    terms, dF = c.eval()
    check_terms(terms, g, "hs32")
    pos = g["hs32.pos"].astype(np.int64)
    np.testing.assert_allclose(dF.ravel()[pos], g["hs32.dF.sample"], rtol=0, atol=dF_tol(0.2))
    assert abs(dF.sum() - g["hs32.dF.sum"][0]) < 1e-9


def test_eval_lj_fp64(cd, oracle):
    g = golden("eval_lj")
    assert cd.bh_diameter(1.0, 1.0, 3.0, 0.8) == pytest.approx(g["lj24.hsd"][0], rel=1e-15)
    hsd = g["lj24.hsd"][0]
    c = cd.Context(24, 0.2, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    assert abs(c.info.a_vdw - g["lj24.a_vdw"][0]) < 1e-12
    _, watt = c.weights()
    np.testing.assert_allclose(watt.ravel(), g["lj24.w_att"], rtol=0, atol=1e-14)
    c.set_chem_potential(c.bulk(0.01)["mu"])
    c.set_density(g["lj24.rho"])
    terms, dF = c.eval()
    check_terms(terms, g, "lj24")
    np.testing.assert_allclose(dF.ravel(), g["lj24.dF"], rtol=0, atol=dF_tol(0.2))
    c2 = cd.Context(16, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    c2.set_chem_potential(c2.bulk(0.3)["mu"])
    c2.set_density(oracle.fill_noise((16, 16, 16), 0.3, 0.1, 5))
    terms, dF = c2.eval()
    check_terms(terms, g, "lj16")
    np.testing.assert_allclose(dF.ravel(), g["lj16.dF"], rtol=0, atol=dF_tol(0.1))
    c3 = cd.Context(24, 0.2, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, fixed_mass=g["lj24fm.fixed_mass"][0])
    c3.set_density(g["lj24.rho"])
    terms, dF = c3.eval()
    check_terms(terms, g, "lj24fm")
    np.testing.assert_allclose(dF.ravel(), g["lj24fm.dF"], rtol=0, atol=dF_tol(0.2))
    np.testing.assert_allclose(c3.get_density().ravel(), g["lj24fm.rho"], rtol=1e-14, atol=0)


@pytest.mark.parametrize("shape,dx,model,lj", [((48, 48, 48), 0.1, "WhiteBearI", True), ((20, 24, 30), 0.15, "RSLT", True),
                                               ((15, 12, 9), 0.2, "WhiteBearII", False), ((40, 40, 40), 0.1, "esFMT", True)])
def test_eval_vs_oracle_fp64(cd, oracle, shape, dx, model, lj):
    hsd = oracle.bh_diameter(3.0, 0.9) if lj else 1.0
    o = oracle.Oracle(shape, dx, model, hsd=hsd, lj=lj, kT=0.9)
    c = cd.Context(shape, dx, model_id(cd, model), hsd=hsd, lj=lj, kT=0.9)
    rho = oracle.fill_noise(shape, 0.4, 0.3, 1234)
    mu = c.bulk(0.4)["mu"]
    assert abs(mu - o.mu_times_beta(0.4)) < 1e-13
    o.set_mu(mu)
    c.set_chem_potential(mu)
    c.set_density(rho)
    terms, dF = c.eval()
    st, t, dFo, _ = o.eval(rho)
    for k in ("Omega", "F_id", "F_hs", "F_mf", "F_ext"):
        assert abs(terms[k] - t[k]) <= 1e-12 * max(1.0, abs(t[k])), (k, terms[k], t[k])
    np.testing.assert_allclose(dF, dFo, rtol=0, atol=dF_tol(dx))


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("lj", [False, True])
def test_double_float_path_models_vs_oracle(cd, oracle, model, lj):
    """At 128^3 FP64 takes the double-float-spectra path (compile-time plans on every axis;
    RSLT with its per-point FP64 branch): every model, with and without the mean field, at the
    reference bars, and its Hessian product against the oracle's to 1e-12 of its maximum."""
    shape, dx = (128, 128, 128), 0.1
    hsd = oracle.bh_diameter(3.0, 0.9) if lj else 1.0
    o = oracle.Oracle(shape, dx, model, hsd=hsd, lj=lj, kT=0.9)
    c = cd.Context(shape, dx, model_id(cd, model), hsd=hsd, lj=lj, kT=0.9)
    rho = oracle.fill_noise(shape, 0.4, 0.3, 4321)
    mu = c.bulk(0.4)["mu"]
    o.set_mu(mu)
    c.set_chem_potential(mu)
    c.set_density(rho)
    terms, dF = c.eval()
    st, t, dFo, _ = o.eval(rho)
    for k in ("Omega", "F_id", "F_hs", "F_mf", "F_ext"):
        assert abs(terms[k] - t[k]) <= 1e-12 * max(1.0, abs(t[k])), (k, terms[k], t[k])
    np.testing.assert_allclose(dF, dFo, rtol=0, atol=dF_tol(dx))
    if lj:
        v = (oracle.fill_noise(shape, 1.0, 1.0, 99) - 1.0) * rho  # signed, of the size of rho
        hv = c.hessian_dot_v(v)
        ref = o.hessian_dot_v(rho, v)
        assert np.max(np.abs(hv - ref)) <= 1e-12 * np.max(np.abs(ref))
    c.close()


@pytest.mark.parametrize("shape", [(32, 128, 128), (128, 48, 128), (128, 128, 32)])
def test_mixed_plan_lattices_vs_oracle(cd, oracle, shape):
    """Lattices mixing a runtime-plan axis with 128-point axes (double-float transforms on
    those, FP64 spectra between passes): FP64 at the reference bars against the oracle."""
    dx = 0.1
    rho = oracle.fill_noise(shape, 0.3, 0.1, 11)
    o = oracle.Oracle(shape, dx, "WhiteBearI", hsd=1.0)
    c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=1.0)
    mu = c.bulk(0.25)["mu"]
    c.set_chem_potential(mu)
    o.set_mu(mu)
    c.set_density(rho)
    terms, dF = c.eval()
    st, t, dFo, _ = o.eval(rho)
    for k in ("Omega", "F_id", "F_hs"):
        assert abs(terms[k] - t[k]) <= 1e-12 * max(1.0, abs(t[k])), (k, terms[k], t[k])
    np.testing.assert_allclose(dF, dFo, rtol=0, atol=dF_tol(dx))
    c.close()


def test_double_float_path_only_fex_and_external_field(cd, oracle):
    """The double-float final pass (ln rho, dF and the sums in df64) without the ideal gas and
    with an external field, at 128^3 FP64: the differences are ln(rho) dV and V dV."""
    shape = (128, 128, 128)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=cd.bh_diameter(1.0, 1.0, 3.0, 0.9), lj=True, kT=0.9, mu=0.2)
    rho = oracle.fill_noise(shape, 0.4, 0.3, 7)
    c.set_density(rho)
    dV = c.info.dV
    t0, d0 = c.eval()
    t3, d3 = c.eval(only_fex=True)
    assert t3["F_id"] == 0.0
    np.testing.assert_allclose(d0 - d3, np.log(rho) * dV, rtol=0, atol=1e-15)
    V = np.sin(np.arange(np.prod(shape)).reshape(shape) * 1e-3)
    c.set_external_field(V)
    t1, d1 = c.eval()
    np.testing.assert_allclose(d1 - d0, V * dV, rtol=0, atol=1e-15)
    assert abs((t1["F_ext"] - t0["F_ext"]) - np.sum(V * rho) * dV) <= 1e-10 * max(1.0, abs(t1["F_ext"]))
    c.close()


def droplet(shape, dx, rho_v=0.01, rho_l=0.75, R=4.0, w=0.5):
    n = np.array(shape)
    ax = [dx * (np.arange(m) - m / 2.0) for m in shape]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    return rho_v + (rho_l - rho_v) * 0.5 * (1 - np.tanh((r - R) / w))


def test_config2_128_fp64_and_fp32_vs_oracle(cd, oracle):
    shape, dx = (128, 128, 128), 0.1
    rho = droplet(shape, dx)
    hsd = oracle.bh_diameter(3.0, 0.8)
    o = oracle.Oracle(shape, dx, "WhiteBearI", hsd=hsd, lj=True, kT=0.8)
    mu = o.mu_times_beta(0.01)
    o.set_mu(mu)
    st, t, dFo, _ = o.eval(rho)
    c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, mu=mu)
    c.set_density(rho)
    terms, dF = c.eval()
    for k in ("Omega", "F_id", "F_hs", "F_mf", "F_ext"):
        assert abs(terms[k] - t[k]) <= 1e-12 * max(1.0, abs(t[k])), (k, terms[k], t[k])
    np.testing.assert_allclose(dF, dFo, rtol=0, atol=dF_tol(dx))
    c.set_precision(cd.FP32)
    terms32, dF32 = c.eval()
    assert abs(terms32["Omega"] - t["Omega"]) <= 2e-6 * abs(t["Omega"])
    assert np.abs(dF32 - dFo).max() <= 2e-6 * np.abs(dFo).max()


@pytest.mark.parametrize("shape", [(256, 16, 256), (16, 256, 24), (128, 128, 256)])
def test_256_point_axes_vs_oracle(cd, oracle, shape):
    """Axes of 256 points run the compile-time 256-point plans (x and z in the first shape,
    y in the second; every axis in the third, whose FP64 spectra stay in double-float between
    passes and whose 256-point z rows reach the Phi pass in two tensor copies): FP64 at the
    reference bars. In FP32 the error of dF is relative to the
    terms that cancel in it near equilibrium (ln rho + c1 against mu, each of order |mu| dV),
    so the FP32 bar on dF is 2e-6 of the larger of max|dF| and |mu| dV."""
    dx = 0.1
    hsd = oracle.bh_diameter(3.0, 0.9)
    o = oracle.Oracle(shape, dx, "WhiteBearI", hsd=hsd, lj=True, kT=0.9)
    rho = oracle.fill_noise(shape, 0.4, 0.3, 77)
    mu = o.mu_times_beta(0.4)
    o.set_mu(mu)
    st, t, dFo, _ = o.eval(rho)
    c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.9, mu=mu)
    c.set_density(rho)
    terms, dF = c.eval()
    for k in ("Omega", "F_id", "F_hs", "F_mf", "F_ext"):
        assert abs(terms[k] - t[k]) <= 1e-12 * max(1.0, abs(t[k])), (k, terms[k], t[k])
    np.testing.assert_allclose(dF, dFo, rtol=0, atol=dF_tol(dx))
    c.set_precision(cd.FP32)
    terms32, dF32 = c.eval()
    assert abs(terms32["Omega"] - t["Omega"]) <= 2e-6 * abs(t["Omega"])
    assert np.abs(dF32 - dFo).max() <= 2e-6 * max(np.abs(dFo).max(), abs(mu) * dx ** 3)
    c.close()


def test_bulk_limit(cd):
    # uniform density: Omega/V equals the bulk grand potential density and dF/dV equals mu(rho) - mu,
    # up to the lattice weights' own sum-rule error (sum w_eta = pi d^3/6 only to ~3e-9 relative)
    for lj in (False, True):
        c = cd.Context(32, 0.1, cd.WHITEBEAR_I, hsd=None if lj else 1.0, lj=lj, kT=0.9)
        rho0 = 0.5
        mu = c.bulk(0.3)["mu"]
        c.set_chem_potential(mu)
        c.set_density(np.full((32, 32, 32), rho0))
        terms, dF = c.eval()
        b = c.bulk(rho0)
        V = c.info.volume
        assert abs(terms["Omega"] / V - (b["fhelmholtz"] - rho0 * mu)) < 1e-8
        np.testing.assert_allclose(dF / c.info.dV, b["mu"] - mu, rtol=0, atol=1e-7)
        assert np.ptp(dF) < 1e-13  # uniform in space to roundoff


def test_eta_too_large_is_reported(cd):
    c = cd.Context(16, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    rho = np.full((16, 16, 16), 0.5)
    rho[4:9, 4:9, 4:9] = 3.0  # eta ~ 1.5 around the block
    c.set_density(rho)
    with pytest.raises(cd.Eta_Too_Large_Exception):
        c.eval()
    c.set_density(np.full((16, 16, 16), 0.5))  # the context stays usable
    terms, _ = c.eval()
    assert np.isfinite(terms["Omega"])


def test_determinism_and_only_fex(cd, oracle):
    c = cd.Context(32, 0.1, cd.WHITEBEAR_I, hsd=0.97, lj=True, kT=0.8)
    rho = oracle.fill_noise((32, 32, 32), 0.4, 0.2, 3)
    c.set_density(rho)
    t1, d1 = c.eval()
    t2, d2 = c.eval()
    assert t1 == t2 and np.array_equal(d1, d2)
    t3, d3 = c.eval(only_fex=True)
    assert t3["F_id"] == 0.0
    np.testing.assert_allclose(d1 - d3, np.log(rho) * c.info.dV, rtol=0, atol=1e-15)


def test_pinned_host_dF_matches_copied_dF(cd, oracle):
    """cdft_eval with a page-locked host dF (the final row pass writes it directly) gives the
    same bits as the copy into pageable memory, for grand-canonical and fixed-mass systems
    (the latter takes the copy path), in both precisions."""
    import torch
    shape = (128, 128, 128)
    rho = oracle.fill_noise(shape, 0.4, 0.3, 5)
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    for kw in ({"mu": 0.3}, {"fixed_mass": float(rho.sum()) * 1e-3}):
        for prec in (cd.FP64, cd.FP32):
            c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=prec, **kw)
            c.set_density(rho)
            t0, d0 = c.eval()
            pinned = torch.full(shape, float("nan"), dtype=torch.float64).pin_memory()
            # at fixed mass every evaluation rescales rho to the mass again (a factor within
            # rounding of 1), so there the bar is rounding, not bits
            same = (lambda a, b: np.array_equal(a, b)) if "mu" in kw else \
                (lambda a, b: np.allclose(a, b, rtol=1e-13, atol=1e-13 * np.abs(b).max()))
            for _ in range(2):  # the second reuses the graph captured with this buffer
                t1, _ = c.eval(dF_out=pinned)
                assert same(pinned.numpy(), d0), (kw, prec)
                assert same(np.array(t1["Omega"]), np.array(t0["Omega"]))
            t2, d2 = c.eval()  # and the device dF stays the same for the next copy
            assert same(d2, d0)
            c.close()


def test_external_field(cd, oracle):
    c = cd.Context(24, 0.2, cd.WHITEBEAR_I, hsd=1.0, mu=0.3)
    rho = oracle.fill_noise((24, 24, 24), 0.5, 0.1, 8)
    V = np.sin(np.arange(24 ** 3).reshape(24, 24, 24) * 0.01)
    c.set_density(rho)
    t0, d0 = c.eval()
    c.set_external_field(V)
    t1, d1 = c.eval()
    dV = c.info.dV
    np.testing.assert_allclose(d1 - d0, V * dV, rtol=0, atol=1e-15)
    assert abs((t1["F_ext"] - t0["F_ext"]) - np.sum(V * rho) * dV) < 1e-10


def test_fire_config1_200_steps_matches_reference(cd, oracle):
    g = golden("fire_hs32")
    c = cd.Context(32, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_chem_potential(c.bulk(0.7)["mu"])
    c.set_density(oracle.fill_noise((32, 32, 32), 0.7, 0.05, 20240601))
    c.fire_init(force_limit=0.0)
    F, dt, alpha, fmax = [], [], [], []
    for _ in range(200):
        r = c.fire_step(1)
        F.append(r["F"]); dt.append(r["dt"]); alpha.append(r["alpha"]); fmax.append(r["fmax"])
    np.testing.assert_array_equal(dt, g["fire32.dt"])
    np.testing.assert_array_equal(alpha, g["fire32.alpha"])
    np.testing.assert_allclose(F, g["fire32.F"], rtol=1e-12)
    np.testing.assert_allclose(fmax, g["fire32.fmax"], rtol=1e-8)
    pos = g["fire32.pos"].astype(np.int64)
    np.testing.assert_allclose(c.get_density().ravel()[pos], g["fire32.rho_final.sample"], rtol=0, atol=1e-12)


def test_fire_lj_fixed_mass_matches_reference(cd):
    g = golden("fire_lj24")
    rho = golden("eval_lj")["lj24.rho"].reshape(24, 24, 24)
    hsd = golden("eval_lj")["lj24.hsd"][0]
    c = cd.Context(24, 0.2, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, fixed_mass=rho.sum() * 0.2 ** 3)
    c.set_density(rho)
    c.fire_init(force_limit=0.0)
    F, dt = [], []
    for _ in range(60):
        r = c.fire_step(1)
        F.append(r["F"]); dt.append(r["dt"])
    np.testing.assert_array_equal(dt, g["firelj.dt"])
    np.testing.assert_allclose(F, g["firelj.F"], rtol=1e-12)
    np.testing.assert_allclose(c.get_density().ravel(), g["firelj.rho_final"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case,tag,nsteps,dt,dtmax", [("ddft_lj16", "ddft16", 10, 1e-4, 1e-4),
                                                       ("ddft_adapt16", "ddfta", 14, 1e-5, 4e-5)])
def test_ddft_matches_reference(cd, oracle, case, tag, nsteps, dt, dtmax):
    g = golden(case)
    c = cd.Context(16, 0.1, cd.WHITEBEAR_I, hsd=golden("eval_lj")["lj24.hsd"][0], lj=True, kT=0.8)
    c.set_density(oracle.fill_noise((16, 16, 16), 0.3, 0.1, 5))
    c.ddft_init(dt, dtmax)
    F, t, dts, mass = [], [], [], []
    for _ in range(nsteps):
        r = c.ddft_step(1)
        F.append(r["F"]); t.append(r["time"]); dts.append(r["dt"]); mass.append(r["mass"])
    np.testing.assert_array_equal(dts, g[tag + ".dt"])
    np.testing.assert_allclose(t, g[tag + ".t"], rtol=1e-14)
    np.testing.assert_allclose(F, g[tag + ".F"], rtol=1e-12)
    np.testing.assert_allclose(mass, g[tag + ".mass"], rtol=1e-13)
    np.testing.assert_allclose(c.get_density().ravel(), g[tag + ".rho_final"], rtol=0, atol=1e-12)


def test_ddft_128_fp64_vs_oracle(cd, oracle):
    """Two DDFT steps at 128^3 in FP64: the evaluations run on double-float spectra and the
    propagator's own transforms on the compile-time 128-point plans, against the oracle's
    restatement of DDFT::step on the same density (time steps exactly, F and mass to 1e-12,
    the densities to 1e-12 absolute)."""
    shape = (128, 128, 128)
    hsd = oracle.bh_diameter(3.0, 0.8)
    rho = oracle.fill_noise(shape, 0.3, 0.1, 17)
    dt, dtmax = 1e-4, 1e-3
    o = oracle.Oracle(shape, 0.1, "WhiteBearI", hsd=hsd, lj=True, kT=0.8)
    n, rec, rfin = o.ddft(rho, 2, dt, dtmax)
    assert n == 2
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    c.set_density(rho)
    c.ddft_init(dt, dtmax)
    for i in range(2):
        r = c.ddft_step(1)
        assert r["dt"] == rec["dt"][i]
        assert abs(r["F"] - rec["F"][i]) <= 1e-12 * abs(rec["F"][i])
        assert abs(r["mass"] - rec["mass"][i]) <= 1e-12 * abs(rec["mass"][i])
    assert np.max(np.abs(c.get_density() - rfin)) <= 1e-12
    c.close()


def test_reference_shaped_api(cd, oracle):
    # The reference's own call sequence, on the GPU (config 1 evaluation).
    d = cd.Density(0.2, [6.4, 6.4, 6.4])
    s = cd.FMT_Species(d, 1.0, 0.0)
    fmt = cd.WhiteBearI()
    dft = cd.DFT(s)
    dft.addHardCoreContribution(fmt)
    d.set(oracle.fill_noise((32, 32, 32), 0.7, 0.05, 20240601))
    s.setChemPotential(dft.mu_times_beta(0.7))
    F = dft.calculateFreeEnergyAndDerivatives(False)
    g = golden("eval_hs32")
    assert abs(F - g["hs32.Omega"][0]) < 1e-12 * abs(F)
    assert abs(dft.get_f_hs() - g["hs32.F_hs"][0]) < 1e-12 * abs(dft.get_f_hs())
    fire = cd.fireMinimizer2(dft)
    fire.setForceTerminationCriterion(0.0)
    fire.run(5)
    assert fire.report["total_steps"] == 5


def test_bulk_coexistence_matches_reference(cd):
    g = golden("coex")
    for i, kT in enumerate(g["coex.kT"]):
        tag = "%.1f" % kT
        c = cd.Context(16, 0.1, cd.WHITEBEAR_I, hsd=g["coex.hsd_kT" + tag][0], lj=True, kT=kT)
        assert abs(c.info.a_vdw - g["coex.avdw_kT" + tag][0]) < 1e-12
        r = c.find_coex(1.0, 1e-3, 1e-8)
        assert abs(r["x_vap"] - g["coex.x_vap"][i]) < 1e-9
        assert abs(r["x_liq"] - g["coex.x_liq"][i]) < 1e-9
        assert abs(r["mu"] - g["coex.mu"][i]) < 1e-9
        assert abs(r["spinodal1"] - g["coex.spinodal1"][i]) < 1e-8
        assert abs(r["spinodal2"] - g["coex.spinodal2"][i]) < 1e-8


def test_large_grid_properties(cd, oracle):
    """Sizes past what the oracle finishes quickly: 256^3 (FP32) and 192 x 160 x 144 (FP64).
    A uniform density gives the bulk values everywhere; translating the density by whole
    lattice sites translates dF (periodic), in both precisions."""
    for shape, prec, tol in (((256, 256, 256), cd.FP32, 1e-5), ((192, 160, 144), cd.FP64, 1e-12)):
        c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=None, lj=True, kT=0.9, precision=prec)
        mu = c.bulk(0.3)["mu"]
        c.set_chem_potential(mu)
        c.set_density(np.full(shape, 0.4))
        terms, dF = c.eval()
        b = c.bulk(0.4)
        assert abs(dF.mean() / c.info.dV - (b["mu"] - mu)) < (1e-6 if prec == cd.FP32 else 1e-7)
        assert np.ptp(dF) / c.info.dV < (1e-5 if prec == cd.FP32 else 1e-12)
        rho = oracle.fill_noise(shape, 0.3, 0.3, 21)
        c.set_density(rho)
        _, d0 = c.eval()
        c.set_density(np.roll(rho, (3, -5, 7), axis=(0, 1, 2)))
        _, d1 = c.eval()
        assert np.max(np.abs(np.roll(d0, (3, -5, 7), axis=(0, 1, 2)) - d1)) <= tol * np.max(np.abs(d0))
        c.close()
