"""Neural-operator warm start on the GPU at a small size: training lowers the
loss, the prediction is a positive density, and the solver started from it
lands on the same minimum as the solver started from the tanh profile."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (64, 64, 64)


@pytest.fixture(scope="module")
def mods():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import classicaldft_gb300 as cd
    from classicaldft_gb300 import fno
    return cd, fno


def test_fno_train_predict_and_warm_start(mods):
    cd, fno = mods
    pts = fno.sample_droplets(4, seed=5, R=(1.8, 2.4))
    samples = fno.solve_droplets(pts, SHAPE, 0.1)
    assert len(samples) == 4
    model = fno.FNO3d()
    log = []
    fno.train(model, samples[:3], SHAPE, steps=60, lr=3e-3, log=log)
    assert log[-1][1] < log[0][1]
    seed, kT, rho = samples[3]
    pred = fno.predict(model, seed, kT, SHAPE)
    assert pred.shape == SHAPE and np.all(pred > 0) and np.isfinite(pred).all()
    # warm start converges to the cold start's minimum
    p = pts[3]
    from classicaldft_gb300.statepoints import droplet
    rho0 = droplet(SHAPE, 0.1, p["rho_v"], p["rho_l"], p["R"])
    mass = float(rho0.sum()) * 1e-3
    om = []
    for start in (rho0, pred):
        c = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=cd.bh_diameter(1.0, 1.0, 3.0, p["kT"]), lj=True, kT=p["kT"], fixed_mass=mass)
        c.set_density(start)
        c.fire_init(force_limit=0.0)
        r = c.fire_run_device(1e-8, max_steps=20000, mixed=3)
        t, _ = c.eval(want_dF=False)
        assert r["stop"] == 2 and t["resid"] <= 1e-8
        om.append(t["Omega"])
        c.close()
    assert abs(om[1] - om[0]) <= 1e-10 * abs(om[0])


def test_warm_start_needs_fewer_newton_corrections(mods):
    """Trained on eight converged 64^3 droplets, the operator's prediction for a held-out
    droplet of the same family needs fewer Newton-Krylov corrections than the tanh start
    (the solver's own guess) to reach max|dOmega/drho| <= 1e-8, and lands on the same Omega."""
    cd, fno = mods
    pts = fno.sample_droplets(9, seed=21, R=(1.8, 2.6))
    samples = fno.solve_droplets(pts, SHAPE, 0.1)
    assert len(samples) == 9
    model = fno.FNO3d()
    fno.train(model, samples[:8], SHAPE, steps=400, lr=3e-3)
    seed, kT, rho = samples[8]
    p = pts[8]
    from classicaldft_gb300.statepoints import droplet
    rho0 = droplet(SHAPE, 0.1, p["rho_v"], p["rho_l"], p["R"])
    mass = float(rho0.sum()) * 1e-3
    res = {}
    for name, start in (("cold", rho0), ("warm", fno.predict(model, seed, kT, SHAPE))):
        c = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=cd.bh_diameter(1.0, 1.0, 3.0, p["kT"]), lj=True, kT=p["kT"], fixed_mass=mass)
        c.set_density(start)
        c.fire_init(force_limit=0.0)
        r = c.fire_run_device(1e-8, max_steps=20000, mixed=3)
        t, _ = c.eval(want_dF=False)
        assert r["stop"] == 2 and t["resid"] <= 1e-8
        res[name] = (r["newton"], t["Omega"])
        c.close()
    assert res["warm"][0] < res["cold"][0], res
    assert abs(res["warm"][1] - res["cold"][1]) <= 1e-10 * abs(res["cold"][1])
