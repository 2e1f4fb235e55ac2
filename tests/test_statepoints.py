"""State-point sampler and bulk-branch solver (host logic, no GPU).

The branch densities are checked against the oracle's DFT::mu_times_beta at the
coexistence points the reference itself computed (tests/golden/coex.npz)."""
import numpy as np
import pytest

from conftest import golden

sp = pytest.importorskip("classicaldft_gb300.statepoints")


def test_sampler_is_seeded_and_in_range():
    a = sp.sample_state_points(64, seed=7)
    b = sp.sample_state_points(64, seed=7)
    c = sp.sample_state_points(64, seed=8)
    assert a == b and a != c
    for p in a:
        assert 0.7 <= p["kT"] <= 0.94
        assert -0.2 <= p["dmu"] <= 0.2
        assert p["n"] in sp.GRIDS and p["dx"] == 0.1
        assert 0 < p["R"] <= 0.4 * p["n"] * p["dx"] + 1e-12
    assert len({p["n"] for p in a}) > 4  # uneven grids


def test_radius_clamped_on_small_boxes():
    pts = sp.sample_state_points(200, seed=1, grids=(48,), R_range=(5.0, 6.0))
    assert all(abs(p["R"] - 0.4 * 4.8) < 1e-12 for p in pts)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_branch_densities_against_reference_coex(oracle, k):
    g = golden("coex")
    kT = float(g["coex.kT"][k])
    tag = "%.1f" % kT
    o = oracle.Oracle(16, 0.1, "WhiteBearI", hsd=float(g["coex.hsd_kT" + tag][0]), lj=True, kT=kT)
    assert abs(o.a_vdw - float(g["coex.avdw_kT" + tag][0])) < 1e-12 * abs(o.a_vdw)
    coex = {"mu": float(g["coex.mu"][k]), "spinodal1": float(g["coex.spinodal1"][k]), "spinodal2": float(g["coex.spinodal2"][k])}
    # dmu = 0 returns the reference's coexisting pair
    mu, rv, rl = sp.coexisting_densities(o.mu_times_beta, coex, 0.0)
    assert abs(rv - g["coex.x_vap"][k]) < 1e-6 and abs(rl - g["coex.x_liq"][k]) < 1e-6
    for dmu in (-0.2, -0.05, 0.05, 0.2):
        mu, rv, rl = sp.coexisting_densities(o.mu_times_beta, coex, dmu)
        assert abs(o.mu_times_beta(rv) - mu) < 1e-9 and abs(o.mu_times_beta(rl) - mu) < 1e-9
        assert rv < coex["spinodal1"] < coex["spinodal2"] < rl
        # clamped inside the metastable window, else exactly mu_coex + dmu
        mu_hi = o.mu_times_beta(coex["spinodal1"])
        mu_lo = o.mu_times_beta(coex["spinodal2"])
        assert mu_lo < mu < mu_hi
        if mu_lo + 0.1 * (coex["mu"] - mu_lo) < coex["mu"] + dmu < mu_hi - 0.1 * (mu_hi - coex["mu"]):
            assert abs(mu - (coex["mu"] + dmu)) < 1e-15


def test_droplet_profile():
    rho = sp.droplet((48, 48, 48), 0.1, 0.02, 0.7, 1.5)
    assert rho.shape == (48, 48, 48)
    # centre (r = 0) and corner (r = 2.4 sqrt 3) from the formula
    assert abs(rho[24, 24, 24] - (0.02 + 0.68 * 0.5 * (1 + np.tanh(3.0)))) < 1e-15
    r = 2.4 * np.sqrt(3.0)
    assert abs(rho[0, 0, 0] - (0.02 + 0.68 * 0.5 * (1 - np.tanh((r - 1.5) / 0.5)))) < 1e-15
    assert np.all(rho >= 0.02 - 1e-15) and np.all(rho <= 0.7 + 1e-15)
