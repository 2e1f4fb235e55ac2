"""Device-resident, graph-captured FIRE2 (cdft_fire_run_device): the same
steps as the host-driven path (which matches the reference's trajectory), and
the mixed FP32 -> FP64 policy reaching the same minimum as plain FP64."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def droplet(shape, dx, R, rho_v=0.01, rho_l=0.75, w=0.5):
    ax = [dx * (np.arange(m) - m / 2.0) for m in shape]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    return rho_v + (rho_l - rho_v) * 0.5 * (1 - np.tanh((r - R) / w))


def test_device_fire_matches_reference_trajectory():
    import classicaldft_gb300 as cd
    from oracle import pyoracle
    g = golden("fire_hs32")
    c = cd.Context(32, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_chem_potential(c.bulk(0.7)["mu"])
    c.set_density(pyoracle.fill_noise((32, 32, 32), 0.7, 0.05, 20240601))
    c.fire_init(force_limit=0.0)
    r = c.fire_run_device(0.0, max_steps=200)
    assert r["total_steps"] == 200
    assert r["dt"] == g["fire32.dt"][199] and r["alpha"] == g["fire32.alpha"][199]
    assert abs(r["F"] - g["fire32.F"][199]) <= 1e-12 * abs(r["F"])
    pos = g["fire32.pos"].astype(np.int64)
    np.testing.assert_allclose(c.get_density().ravel()[pos], g["fire32.rho_final.sample"], rtol=0, atol=1e-12)


def test_device_fire_fixed_mass_matches_host_path():
    import classicaldft_gb300 as cd
    rho = golden("eval_lj")["lj24.rho"].reshape(24, 24, 24)
    hsd = golden("eval_lj")["lj24.hsd"][0]
    runs = []
    for device in (False, True):
        c = cd.Context(24, 0.2, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, fixed_mass=rho.sum() * 0.2 ** 3)
        c.set_density(rho)
        c.fire_init(force_limit=0.0)
        r = c.fire_run_device(0.0, max_steps=60) if device else c.fire_step(60)
        runs.append((r, c.get_density()))
    (rh, dh), (rd, dd) = runs
    assert rh["dt"] == rd["dt"] and rh["alpha"] == rd["alpha"]
    assert abs(rh["F"] - rd["F"]) <= 1e-12 * abs(rh["F"])
    np.testing.assert_allclose(dd, dh, rtol=0, atol=1e-12)


def test_mixed_precision_reaches_fp64_minimum():
    import classicaldft_gb300 as cd
    shape, dx = (32, 32, 32), 0.2
    rho = droplet(shape, dx, R=1.8)
    mass = rho.sum() * dx ** 3
    hsd = cd.bh_diameter(1, 1, 3, 0.8)
    res = {}
    for mixed in (False, True):
        c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, fixed_mass=mass)
        c.set_density(rho)
        c.fire_init(force_limit=0.0, dt=1e-3, dt_max=1e-2)
        r = c.fire_run_device(1e-8, max_steps=40000, mixed=mixed, switch_tol=2e-6)
        assert r["resid"] <= 1e-8, r
        t, dF = c.eval()
        assert t["resid"] <= 1e-8
        res[mixed] = (t["Omega"], c.get_density(), r["total_steps"])
    assert abs(res[True][0] - res[False][0]) <= 1e-10 * abs(res[False][0])
    np.testing.assert_allclose(res[True][1], res[False][1], rtol=0, atol=1e-6)
    # both minima checked by the FP64 oracle (the reference's arithmetic): Omega within
    # 1e-10 relative and the oracle's own max|dOmega/drho| at most 1e-8 (+ the 1e-10 dF bar)
    from oracle import pyoracle
    o = pyoracle.Oracle(shape, dx, "WhiteBearI", hsd=hsd, lj=True, kT=0.8, fixed_mass=mass)
    for mixed in (False, True):
        _, t, dFo, _ = o.eval(res[mixed][1])
        assert abs(res[mixed][0] - t["Omega"]) <= 1e-10 * abs(t["Omega"]), (mixed, res[mixed][0], t["Omega"])
        assert np.abs(dFo).max() / dx ** 3 <= 1e-8 + 1e-10, (mixed, np.abs(dFo).max() / dx ** 3)


def test_ddft_fp32_conserves_mass_and_tracks_fp64():
    import classicaldft_gb300 as cd
    from oracle import pyoracle
    shape, dx = (48, 48, 48), 0.1
    rho = pyoracle.fill_noise(shape, 0.3, 0.1, 21)
    hsd = cd.bh_diameter(1, 1, 3, 0.8)
    out = {}
    for prec in (cd.FP64, cd.FP32):
        c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=prec)
        c.set_density(rho)
        c.ddft_init(1e-4, 1e-4)
        m0 = np.sum(rho) * dx ** 3
        masses = [c.ddft_step(1)["mass"] for _ in range(10)]
        out[prec] = (c.get_density(), masses, m0)
    d64, m64, m0 = out[cd.FP64]
    d32, m32, _ = out[cd.FP32]
    assert max(abs(m - m0) for m in m32) <= 1e-12 * m0
    assert max(abs(m - m0) for m in m64) <= 1e-12 * m0
    assert np.abs(d32 - d64).max() <= 1e-5


def test_ddft_fp32_64cubed_tracks_fp64_50_steps():
    """50 DDFT steps at 64^3 (dt = 1e-4, the LJ droplet functional) in FP32 bulk against
    the FP64 step (the reference's arithmetic, pinned to it at 16^3): with the mass
    restore the FP32 trajectory stays within 2e-5 of FP64 and keeps the mass to 1e-12;
    without it the FP32 propagator's own drift is reported and stays below 1e-5."""
    import classicaldft_gb300 as cd
    from oracle import pyoracle
    shape, dx = (64, 64, 64), 0.1
    rho = pyoracle.fill_noise(shape, 0.3, 0.1, 64)
    hsd = cd.bh_diameter(1, 1, 3, 0.8)
    m0 = np.sum(rho) * dx ** 3
    out = {}
    for name, prec, restore in (("fp64", cd.FP64, True), ("fp32", cd.FP32, True), ("fp32_raw", cd.FP32, False)):
        c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=prec)
        c.set_chem_potential(c.bulk(0.3)["mu"])
        c.set_density(rho)
        c.ddft_init(1e-4, 1e-4)
        c.ddft_set_mass_restore(restore)
        r = c.ddft_step(50)
        out[name] = (c.get_density(), r["mass"], c.ddft_mass_deviation(), r["time"])
        c.close()
    d64, m64, dev64, t64 = out["fp64"]
    d32, m32, dev32, t32 = out["fp32"]
    dr, mr, devr, tr = out["fp32_raw"]
    assert t64 == t32 == tr
    assert abs(m64 - m0) <= 1e-12 * m0 and dev64 == 0.0
    assert abs(m32 - m0) <= 1e-12 * m0
    assert 0.0 < dev32 <= 1e-5 and 0.0 < devr <= 1e-5
    assert abs(mr - m0) <= 1e-5 * m0
    assert np.abs(d32 - d64).max() <= 2e-5, np.abs(d32 - d64).max()
    assert np.abs(dr - d64).max() <= 2e-5, np.abs(dr - d64).max()


def test_fire_state_saved_and_resumed_matches_reference(tmp_path):
    """fireMinimizer2's serialised state: 30 fixed-mass FIRE2 steps of the LJ droplet, the
    state saved, a fresh context resumes it for 30 more (host-stepped) and the device-resident
    driver from a second copy; both land on the reference's 60-step trajectory (dt, alpha,
    F, the final density)."""
    import classicaldft_gb300 as cd
    g = golden("fire_lj24")
    rho = golden("eval_lj")["lj24.rho"].reshape(24, 24, 24)
    hsd = golden("eval_lj")["lj24.hsd"][0]
    mass = rho.sum() * 0.2 ** 3

    def ctx():
        return cd.Context(24, 0.2, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, fixed_mass=mass)
    a = ctx()
    a.set_density(rho)
    a.fire_init(force_limit=0.0)
    a.fire_step(30)
    path = str(tmp_path / "fire.state")
    a.fire_save(path)
    a.close()
    for device in (False, True):
        b = ctx()
        b.fire_load(path)
        if device:
            r = b.fire_run_device(0.0, max_steps=30)
        else:
            reps = [b.fire_step(1) for _ in range(30)]
            np.testing.assert_allclose([q["F"] for q in reps], g["firelj.F"][30:], rtol=1e-12)
            np.testing.assert_array_equal([q["dt"] for q in reps], g["firelj.dt"][30:])
            r = reps[-1]
        assert r["total_steps"] == 60
        assert r["dt"] == g["firelj.dt"][59] and r["alpha"] == g["firelj.alpha"][59]
        assert abs(r["F"] - g["firelj.F"][59]) <= 1e-12 * abs(g["firelj.F"][59])
        np.testing.assert_allclose(b.get_density().ravel(), g["firelj.rho_final"], rtol=0, atol=1e-12)
        b.close()
