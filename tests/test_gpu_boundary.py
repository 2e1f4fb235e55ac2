"""Species::setFixedBackground / setHomogeneousBoundary (src/Species.cpp:74-95) on the GPU
against the reference's own outputs (tests/golden/boundary.npz, oracle/ref_driver case
"boundary": the hard-sphere WhiteBearI 16^3 state at dx = 0.2, rho = 0.6 (1 +- 0.2)).

Tolerances as for the other evaluations: FP64 Omega within 1e-12 relative, dF within
1e-10 dV; the Hessian product within 1e-12 of max|Hv|; Log_Det within 1e-10; FIRE2's F
sequence within 1e-12 relative."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

SHAPE = (16, 16, 16)
DV = 0.2 ** 3


@pytest.fixture(scope="module")
def cd():
    import classicaldft_gb300 as m
    m.lib()
    return m


def boundary_mask():
    i, j, k = np.meshgrid(*(np.arange(16),) * 3, indexing="ij")
    return ((i == 0) | (j == 0) | (k == 0)).ravel()


def context(cd, oracle, fixed=False, homo=False, precision="FP64", seed=11):
    c = cd.Context(SHAPE, 0.2, cd.WHITEBEAR_I, hsd=1.0, precision=getattr(cd, precision))
    c.set_density(oracle.fill_noise(SHAPE, 0.6, 0.2, seed))
    c.set_chem_potential(c.bulk(0.6)["mu"])
    c.set_boundary(fixed_background=fixed, homogeneous=homo)
    return c


@pytest.mark.parametrize("tag,fixed,homo", [("bfix", True, False), ("bhom", False, True)])
def test_eval_with_boundary_mode(cd, oracle, tag, fixed, homo):
    g = golden("boundary")
    c = context(cd, oracle, fixed, homo)
    terms, dF = c.eval()
    assert abs(terms["Omega"] - g[tag + ".Omega"][0]) <= 1e-12 * abs(g[tag + ".Omega"][0])
    np.testing.assert_allclose(dF.ravel(), g[tag + ".dF"], rtol=0, atol=1e-10 * DV)
    b = boundary_mask()
    if fixed:
        assert np.all(dF.ravel()[b] == 0.0)
    else:
        assert np.ptp(dF.ravel()[b]) == 0.0
    assert abs(terms["resid"] - np.abs(g[tag + ".dF"]).max() / DV) <= 1e-10
    c.close()


def test_eval_fixed_background_fp32(cd, oracle):
    g = golden("boundary")
    c = context(cd, oracle, fixed=True, precision="FP32")
    terms, dF = c.eval()
    ref = g["bfix.dF"]
    assert np.all(dF.ravel()[boundary_mask()] == 0.0)
    assert np.abs(dF.ravel() - ref).max() <= 2e-6 * max(np.abs(ref).max(), abs(c.chem_potential()) * DV)
    c.close()


def test_homogeneous_boundary_with_fixed_mass(cd, oracle):
    g = golden("boundary")
    c = cd.Context(SHAPE, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_density(oracle.fill_noise(SHAPE, 0.6, 0.2, 11))
    c.set_fixed_mass(float(g["bhomfm.fixed_mass"][0]))
    c.set_boundary(homogeneous=True)
    terms, dF = c.eval()
    assert abs(terms["Omega"] - g["bhomfm.Omega"][0]) <= 1e-12 * abs(g["bhomfm.Omega"][0])
    assert abs(terms["mu"] - g["bhomfm.mu"][0]) <= 1e-12 * abs(g["bhomfm.mu"][0])
    np.testing.assert_allclose(dF.ravel(), g["bhomfm.dF"], rtol=0, atol=1e-10 * DV)
    c.close()


def test_fixed_background_with_fixed_mass_is_refused(cd, oracle):
    c = context(cd, oracle, fixed=True)
    c.set_fixed_mass(10.0)
    with pytest.raises(cd.CDFTError) as e:
        c.eval()
    assert e.value.code == cd.ERR_ARG
    c.close()


def test_hessian_and_log_det_with_fixed_background(cd, oracle):
    """Dynamical_Matrix::matrix_dot_v1 zeroes the input's boundary and DFT::matrix_dot_v_intern
    the output's; Log_Det zeroes its probes there and counts only the inner points."""
    g = golden("boundary")
    c = context(cd, oracle, fixed=True)
    c.eval()
    v = 0.3 * (oracle.fill_noise(SHAPE, 1.0, 1.0, 77) - 1.0)
    hv = c.hessian_dot_v(v)
    ref = g["bfix.Hv"]
    assert np.max(np.abs(hv.ravel() - ref)) <= 1e-12 * np.max(np.abs(ref))
    val, var = c.log_det(10, 0.16, 0.008, 1234, 2)
    assert abs(val - g["bfix.logdet"][0]) <= 1e-10 * abs(g["bfix.logdet"][0])
    assert abs(var - g["bfix.logdet"][1]) <= 1e-6 * g["bfix.logdet"][1]
    lam, y, rep = c.eigenvalue(tol=1e-8, change_sign=True)
    assert rep["converged"] and np.all(y.ravel()[boundary_mask()] == 0.0)
    c.close()


def test_fire_with_fixed_background(cd, oracle):
    """30 host-stepped FIRE2 steps (the reference's F sequence and final density: the
    boundary densities do not move beyond the alias map's round-trip roundoff), then the
    device-resident steps from the same start."""
    g = golden("boundary")
    c = context(cd, oracle, fixed=True)
    c.fire_init(force_limit=0.0)
    F = [c.fire_step(1)["F"] for _ in range(30)]
    np.testing.assert_allclose(F, g["bfix.fire.F"], rtol=1e-12, atol=0)
    rho = c.get_density().ravel()
    np.testing.assert_allclose(rho, g["bfix.fire.rho"], rtol=1e-10, atol=0)
    rho0 = oracle.fill_noise(SHAPE, 0.6, 0.2, 11).ravel()
    np.testing.assert_allclose(rho[boundary_mask()], rho0[boundary_mask()], rtol=1e-13, atol=0)
    c.close()
    c = context(cd, oracle, fixed=True)
    c.fire_init(force_limit=0.0)
    r = c.fire_run_device(0.0, max_steps=30)
    assert r["total_steps"] == 30 and abs(r["F"] - g["bfix.fire.F"][-1]) <= 1e-12 * abs(r["F"])
    np.testing.assert_allclose(c.get_density().ravel()[boundary_mask()], rho0[boundary_mask()], rtol=1e-13, atol=0)
    c.close()


@pytest.mark.parametrize("tag,fixed", [("bddft_fix", True), ("bddft_hom", False)])
def test_ddft_with_boundary_mode(cd, oracle, tag, fixed):
    """10 DDFT steps of the LJ system of ddft_lj16 (dt = 1e-4 fixed) with each mode: g . dF
    vanishes on a fixed boundary and its densities stay (the mass then changes); the
    homogeneous boundary only changes dF."""
    g = golden("boundary")
    c = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=golden("eval_lj")["lj24.hsd"][0], lj=True, kT=0.8)
    rho0 = oracle.fill_noise(SHAPE, 0.3, 0.1, 5)
    c.set_density(rho0)
    c.set_boundary(fixed_background=fixed, homogeneous=not fixed)
    c.ddft_init(1e-4, 1e-4)
    F, mass = [], []
    for _ in range(10):
        r = c.ddft_step(1)
        F.append(r["F"]); mass.append(r["mass"])
    np.testing.assert_allclose(F, g[tag + ".F"], rtol=1e-12)
    np.testing.assert_allclose(mass, g[tag + ".mass"], rtol=1e-13)
    rho = c.get_density().ravel()
    np.testing.assert_allclose(rho, g[tag + ".rho_final"], rtol=1e-10)
    if fixed:
        assert np.all(rho[boundary_mask()] == rho0.ravel()[boundary_mask()])
    c.close()


@pytest.mark.parametrize("fixed_mass", [False, True])
def test_device_fire_with_homogeneous_boundary_matches_host_steps(cd, oracle, fixed_mass):
    """The homogeneous boundary in the device-resident FIRE2 step (the boundary mean of dF,
    then, at fixed mass, mu from sum dF . rho over the averaged dF) against the host-stepped
    FIRE2, whose evaluation follows Species::endForceCalculation (pinned by the bhom and
    bhomfm goldens): the same dt and alpha after 30 steps, F and the density to roundoff."""
    g = golden("boundary")
    runs = []
    for device in (False, True):
        c = context(cd, oracle, homo=True)
        if fixed_mass:
            c.set_fixed_mass(float(g["bhomfm.fixed_mass"][0]))
        c.fire_init(force_limit=0.0)
        r = c.fire_run_device(0.0, max_steps=30) if device else c.fire_step(30)
        runs.append((r, c.get_density()))
        c.close()
    (rh, dh), (rd, dd) = runs
    assert rh["dt"] == rd["dt"] and rh["alpha"] == rd["alpha"]
    assert abs(rh["F"] - rd["F"]) <= 1e-12 * abs(rh["F"])
    np.testing.assert_allclose(dd, dh, rtol=1e-11, atol=0)


def test_newton_with_fixed_background(cd, oracle):
    """Newton-Krylov (mixed = 3) with a fixed background: the correction lives on the
    interior, the boundary densities stay, and it reaches the minimum plain FP64 FIRE2
    finds (Omega within 1e-10, max|dOmega/drho| <= 1e-8)."""
    res = {}
    rho0 = oracle.fill_noise(SHAPE, 0.6, 0.2, 11).ravel()
    for mixed in (0, 3):
        c = context(cd, oracle, fixed=True)
        c.fire_init(force_limit=0.0)
        r = c.fire_run_device(1e-8, max_steps=40000, mixed=mixed)
        t, _ = c.eval(want_dF=False)
        assert t["resid"] <= 1e-8, (mixed, r, t["resid"])
        rho = c.get_density().ravel()
        np.testing.assert_allclose(rho[boundary_mask()], rho0[boundary_mask()], rtol=1e-13, atol=0)
        res[mixed] = (t["Omega"], rho, r)
        c.close()
    assert res[3][2]["newton"] >= 1
    assert abs(res[3][0] - res[0][0]) <= 1e-10 * abs(res[0][0])
    np.testing.assert_allclose(res[3][1], res[0][1], rtol=0, atol=1e-6)


def test_batch_with_boundary_modes(cd, oracle):
    """The batched driver takes contexts with boundary modes: two fixed-background contexts
    under Newton-Krylov (mixed = 3), and a homogeneous-boundary one, for which the batch
    takes the FIRE2 policy (mixed = 1); each reaches the state it reaches alone with the
    same settings (with a homogeneous boundary only the boundary mean of dF vanishes, so the
    end state depends on the path, and the two runs must take the same one)."""
    for modes, mixed_alone in (((dict(fixed=True, seed=11), dict(fixed=True, seed=12)), 3), ((dict(homo=True, seed=11),), 1)):
        ctxs = [context(cd, oracle, **m) for m in modes]
        for c in ctxs:
            c.fire_init(force_limit=0.0)
        reps, status = cd.fire_run_batch(ctxs, 1e-8, max_steps=40000, mixed=3, switch_tol=1e-4)
        assert not any(status), (status, reps)
        batched = [c.eval(want_dF=False)[0] for c in ctxs]
        for c in ctxs:
            c.close()
        for m, b in zip(modes, batched):
            c = context(cd, oracle, **m)
            c.fire_init(force_limit=0.0)
            c.fire_run_device(1e-8, max_steps=40000, mixed=mixed_alone, switch_tol=1e-4)
            a = c.eval(want_dF=False)[0]
            c.close()
            assert b["resid"] <= 1e-8 and a["resid"] <= 1e-8, (m, b["resid"], a["resid"])
            assert abs(b["Omega"] - a["Omega"]) <= 1e-10 * abs(a["Omega"])


def test_boundary_modes_report_what_is_not_built(cd, oracle):
    c = context(cd, oracle, homo=True)
    with pytest.raises(cd.CDFTError) as e:
        c.newton_refine(1e-8)
    assert e.value.code == cd.ERR_ARG
    c.close()
