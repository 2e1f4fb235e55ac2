"""Batched state points (cdft_fire_run_batch) on the GPU.

Every kernel of the device FIRE step reduces in a fixed order, so a context
run inside a batch must take exactly the steps it takes alone and end on the
same state; the batch only changes what runs concurrently."""
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


def _points():
    from classicaldft_gb300 import statepoints as sp
    pts = sp.sample_state_points(4, seed=11, grids=(48, 64))
    # one point repeated with the other grid: uneven sizes in one batch
    n = 64 if pts[0]["n"] == 48 else 48
    pts.append(dict(pts[0], n=n, R=min(pts[0]["R"], 0.4 * n * 0.1)))
    return pts


@pytest.mark.parametrize("mixed", [False, True])
def test_batch_matches_sequential(cd, mixed):
    from classicaldft_gb300 import statepoints as sp
    pts = _points()
    tol = 1e-7
    alone = []
    for p in pts:
        (c,) = sp.build_contexts([dict(p)])
        r = c.fire_run_device(tol, max_steps=4000, mixed=mixed, switch_tol=2e-6)
        alone.append((r, c.get_density()))
        c.close()
    ctxs = sp.build_contexts([dict(p) for p in pts])
    reps, status = cd.fire_run_batch(ctxs, tol, max_steps=4000, mixed=mixed, switch_tol=2e-6)
    assert status == [0] * len(pts), [r.get("error") for r in reps]
    for (ra, rho_a), rb, c in zip(alone, reps, ctxs):
        assert rb["stop"] == 2 and rb["resid"] <= tol
        assert rb["steps"] == ra["steps"] and rb["steps_fp32"] == ra["steps_fp32"]
        assert rb["F"] == ra["F"]
        np.testing.assert_array_equal(c.get_density(), rho_a)
        c.close()


def test_sweep_converges_to_fp64_minimum(cd):
    """Mixed FP32/FP64 batch and FP64 batch reach the same minima (Omega to 1e-10 relative)."""
    from classicaldft_gb300 import statepoints as sp
    pts = sp.sample_state_points(6, seed=3, grids=(48, 64))
    _, r64, s64 = sp.solve([dict(p) for p in pts], tol=1e-8, max_steps=6000, mixed=False)
    ctxs, rmx, smx = sp.solve([dict(p) for p in pts], tol=1e-8, max_steps=6000, mixed=True)
    assert s64 == [0] * 6 and smx == [0] * 6
    for a, b, c in zip(r64, rmx, ctxs):
        assert a["resid"] <= 1e-8 and b["resid"] <= 1e-8
        assert abs(a["F"] - b["F"]) <= 1e-10 * abs(a["F"])
        rho = c.get_density()
        assert np.all(rho > 0) and np.isfinite(rho).all()


def test_batch_rejects_duplicates_and_uninitialised(cd):
    c = cd.Context((32, 32, 32), 0.1, cd.WHITEBEAR_I, hsd=1.0)
    c.set_density(np.full((32, 32, 32), 0.3))
    with pytest.raises(cd.CDFTError):
        cd.fire_run_batch([c], 1e-8)  # no fire_init
    c.set_chem_potential(c.bulk(0.3)["mu"])
    c.fire_init()
    with pytest.raises(cd.CDFTError):
        cd.fire_run_batch([c, c], 1e-8)
