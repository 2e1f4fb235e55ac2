"""Newton-Krylov refinement (cdft_newton_refine and the mixed = 2 policy of
cdft_fire_run_device / cdft_fire_run_batch) on the GPU: FP32 Hessian products,
FP64 residuals. It must land on the minimum plain FP64 FIRE2 finds
(Omega to 1e-10 relative) with max|dOmega/drho| <= 1e-8 taken from FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cd():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import classicaldft_gb300 as m
    m.lib()
    return m


def _droplet_ctx(cd, n=48):
    from classicaldft_gb300 import statepoints as sp
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    rho = sp.droplet((n,) * 3, 0.1, 0.02, 0.65, 1.6)
    c = cd.Context((n,) * 3, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, fixed_mass=float(rho.sum() * 1e-3))
    c.set_density(rho)
    c.fire_init(force_limit=0.0)
    return c


def test_mixed_newton_reaches_fp64_minimum(cd):
    a = _droplet_ctx(cd)
    ra = a.fire_run_device(1e-8, max_steps=20000, mixed=0)
    ta, _ = a.eval(want_dF=False)
    b = _droplet_ctx(cd)
    rb = b.fire_run_device(1e-8, max_steps=20000, mixed=2, switch_tol=1e-4)
    tb, _ = b.eval(want_dF=False)
    assert ra["stop"] == 2 and rb["stop"] == 2
    assert rb["newton"] >= 1 and rb["cg_iters"] >= 1
    assert tb["resid"] <= 1e-8 and ta["resid"] <= 1e-8
    assert abs(tb["Omega"] - ta["Omega"]) <= 1e-10 * abs(ta["Omega"])
    assert abs(tb["N"] - ta["N"]) <= 1e-12 * ta["N"]  # fixed mass kept
    np.testing.assert_allclose(b.get_density(), a.get_density(), rtol=0, atol=1e-6)
    # both minima checked by the FP64 oracle: Omega within 1e-10 relative, its own
    # max|dOmega/drho| at most 1e-8 (+ the 1e-10 dF bar)
    from oracle import pyoracle
    from classicaldft_gb300 import statepoints as sp
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    mass = float(sp.droplet((48,) * 3, 0.1, 0.02, 0.65, 1.6).sum() * 1e-3)
    o = pyoracle.Oracle((48,) * 3, 0.1, "WhiteBearI", hsd=hsd, lj=True, kT=0.8, fixed_mass=mass)
    for ctx, t in ((a, ta), (b, tb)):
        _, to, dFo, _ = o.eval(ctx.get_density())
        assert abs(t["Omega"] - to["Omega"]) <= 1e-10 * abs(to["Omega"]), (t["Omega"], to["Omega"])
        assert np.abs(dFo).max() / 1e-3 <= 1e-8 + 1e-10
    a.close()
    b.close()


def test_newton_refine_grand_canonical(cd, oracle):
    """Fixed chemical potential, a noisy uniform fluid: Newton alone converges to the bulk state."""
    shape = (32, 32, 32)
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 1.2)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=1.2)
    c.set_chem_potential(c.bulk(0.3)["mu"])
    c.set_density(oracle.fill_noise(shape, 0.3, 0.05, 4))
    r = c.newton_refine(1e-10, max_newton=20)
    assert r["stop"] == 2 and r["resid"] <= 1e-10
    rho = c.get_density()
    assert np.max(np.abs(rho - 0.3)) <= 1e-8
    c.close()


def test_batch_newton_matches_sequential(cd):
    from classicaldft_gb300 import statepoints as sp
    pts = sp.sample_state_points(3, seed=5, grids=(48, 64))
    alone = []
    for p in pts:
        (c,) = sp.build_contexts([dict(p)])
        alone.append(c.fire_run_device(1e-8, max_steps=20000, mixed=2, switch_tol=1e-4))
        c.close()
    ctxs = sp.build_contexts([dict(p) for p in pts])
    reps, status = cd.fire_run_batch(ctxs, 1e-8, max_steps=20000, mixed=2, switch_tol=1e-4)
    assert status == [0, 0, 0], [r.get("error") for r in reps]
    for a, b in zip(alone, reps):
        assert b["stop"] == 2 and b["resid"] <= 1e-8
        assert b["F"] == a["F"] and b["newton"] == a["newton"] and b["cg_iters"] == a["cg_iters"]
    for c in ctxs:
        c.close()


def test_direct_newton_policy(cd):
    """mixed = 3: Newton-Krylov from the tanh profile lands on the FP64 FIRE2 minimum."""
    a = _droplet_ctx(cd)
    a.fire_run_device(1e-8, max_steps=20000, mixed=0)
    ta, _ = a.eval(want_dF=False)
    b = _droplet_ctx(cd)
    rb = b.fire_run_device(1e-8, max_steps=20000, mixed=3)
    tb, _ = b.eval(want_dF=False)
    assert rb["stop"] == 2 and tb["resid"] <= 1e-8 and rb["newton"] >= 1
    assert abs(tb["Omega"] - ta["Omega"]) <= 1e-10 * abs(ta["Omega"])
    a.close()
    b.close()


def test_batch_direct_newton_matches_sequential(cd):
    from classicaldft_gb300 import statepoints as sp
    pts = sp.sample_state_points(4, seed=8, grids=(48, 64))
    alone = []
    for p in pts:
        (c,) = sp.build_contexts([dict(p)])
        alone.append(c.fire_run_device(1e-8, max_steps=20000, mixed=3))
        c.close()
    ctxs = sp.build_contexts([dict(p) for p in pts])
    reps, status = cd.fire_run_batch(ctxs, 1e-8, max_steps=20000, mixed=3)
    assert status == [0] * 4, [r.get("error") for r in reps]
    for a, b in zip(alone, reps):
        assert b["stop"] == 2 and b["resid"] <= 1e-8
        assert b["F"] == a["F"] and b["newton"] == a["newton"] and b["cg_iters"] == a["cg_iters"]
    for c in ctxs:
        c.close()
