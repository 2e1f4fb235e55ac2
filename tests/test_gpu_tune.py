"""FFT-plan autotuner (cdft_autotune) on the GPU: a retuned context evaluates
the same functional (FFT roundoff apart), keeps the fastest plan it timed, and
later contexts of the same shape start from the tuned plans."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (40, 48, 36)  # used by no other test: the tuned plans persist in the process


@pytest.fixture(scope="module")
def cd():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import classicaldft_gb300 as m
    m.lib()
    return m


def test_autotune_keeps_results_and_is_remembered(cd, oracle):
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    rho = oracle.fill_noise(SHAPE, 0.3, 0.1, 17)
    c = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    c.set_chem_potential(-3.0)
    c.set_density(rho)
    t0, d0 = c.eval()
    before = c.radices()
    assert before == {ax: cd.radix_candidates(n)[0] for ax, n in zip("xyz", SHAPE)}
    plans, ms0, ms1 = c.autotune(reps=3)
    assert ms1 <= ms0 and ms1 > 0
    assert c.radices() == plans
    for ax, n in zip("xyz", SHAPE):
        assert plans[ax] in cd.radix_candidates(n)
    t1, d1 = c.eval()
    assert abs(t1["Omega"] - t0["Omega"]) <= 1e-12 * abs(t0["Omega"])
    assert np.max(np.abs(d1 - d0)) <= 1e-13
    o = oracle.Oracle(SHAPE, 0.1, "WhiteBearI", hsd=hsd, lj=True, kT=0.8, mu=-3.0)
    st, terms, dfo, _ = o.eval(rho)
    om = terms["Omega"]
    assert st == 0
    assert abs(t1["Omega"] - om) <= 1e-12 * abs(om)
    assert np.max(np.abs(d1 - dfo)) <= 1e-10
    # a new context of the same shape, model and precision starts tuned; FP32 does not
    c2 = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    assert c2.radices() == plans
    c3 = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=cd.FP32)
    assert c3.radices() == before
    for x in (c, c2, c3):
        x.close()


def test_autotune_fp32_then_fire(cd):
    """Tuning in FP32 and then running device FIRE on the retuned plans (graphs are captured after the swap)."""
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    shape = (48, 48, 48)
    from classicaldft_gb300 import statepoints as sp
    rho = sp.droplet(shape, 0.1, 0.02, 0.65, 1.6)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=cd.FP32)
    c.set_fixed_mass(float(rho.sum() * 1e-3))
    c.set_density(rho)
    plans, ms0, ms1 = c.autotune(reps=3)
    assert ms1 <= ms0
    c.fire_init()
    r = c.fire_run_device(1e-7, max_steps=4000, mixed=True, switch_tol=2e-6)
    assert r["stop"] == 2 and r["resid"] <= 1e-7
    c.close()
