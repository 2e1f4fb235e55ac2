"""The Asakura-Oosawa species (FMT_AO_Species: hard-sphere colloids with ideal polymers,
src/FMT_Species.cpp:645-738, src/FMT.cpp:340-421) against the reference's own outputs
(tests/golden/ao.npz from oracle/ref_driver, case "ao": 16^3, dx = 0.2, d = 1,
Rp = 0.35, reservoir density 0.4, Rosenfeld and WhiteBearI), and the bulk limit on
larger grids (uniform density: dF/dV = mu_bulk(rho) - mu, with the AO terms of the
bulk chemical potential).

Tolerances as for the other evaluations: FP64 Omega and its terms within 1e-12
relative, dF within 1e-10 dV absolute; FP32 Omega within 2e-6 relative and dF within
2e-6 of the larger of max|dF| and |mu| dV."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

RP, RES = 0.35, 0.4


@pytest.fixture(scope="module")
def cd():
    import classicaldft_gb300 as cd
    cd.lib()
    return cd


def model_id(cd, name):
    return {"Rosenfeld": cd.ROSENFELD, "WhiteBearI": cd.WHITEBEAR_I}[name]


@pytest.mark.parametrize("model", ["Rosenfeld", "WhiteBearI"])
def test_ao_eval_matches_reference(cd, model):
    g = golden("ao")
    tag = "ao16." + model
    c = cd.Context(16, 0.2, model_id(cd, model), hsd=1.0, ao_rp=RP, ao_reservoir=RES)
    mu = c.bulk(0.4)["mu"]
    assert abs(mu - g[tag + ".mu"][0]) <= 1e-13 * abs(mu)
    for r, m_ref, o_ref in zip((0.05, 0.2, 0.4, 0.6), g[tag + ".bulk_mu"], g[tag + ".bulk_omega"]):
        b = c.bulk(r)
        assert abs(b["mu"] - m_ref) <= 1e-12 * max(1.0, abs(m_ref))
        assert abs(b["omega"] - o_ref) <= 1e-12 * max(1.0, abs(o_ref))
    c.set_chem_potential(mu)
    c.set_density(g[tag + ".rho"].reshape(16, 16, 16))
    terms, dF = c.eval()
    for k in ("Omega", "F_id", "F_hs", "F_ext"):
        ref = g[tag + "." + k][0]
        assert abs(terms[k] - ref) <= 1e-12 * max(1.0, abs(ref)), (k, terms[k], ref)
    dV = 0.2 ** 3
    np.testing.assert_allclose(dF.ravel(), g[tag + ".dF"], rtol=0, atol=1e-10 * dV)
    c.set_precision(cd.FP32)
    t32, dF32 = c.eval()
    assert abs(t32["Omega"] - g[tag + ".Omega"][0]) <= 2e-6 * abs(g[tag + ".Omega"][0])
    bar = 2e-6 * max(np.abs(g[tag + ".dF"]).max(), abs(mu) * dV)
    assert np.abs(dF32.ravel() - g[tag + ".dF"]).max() <= bar
    c.close()


@pytest.mark.parametrize("shape,prec", [((128, 32, 128), "FP64"), ((128, 32, 128), "FP32"), ((40, 36, 30), "FP64")])
def test_ao_bulk_limit(cd, shape, prec):
    """Uniform density: the AO passes give dF/dV = mu_bulk(rho) - mu everywhere and
    Omega/V = omega_bulk(rho) (128-point axes run the compile-time plans)."""
    dx, rho0 = 0.1, 0.3
    c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=1.0, ao_rp=RP, ao_reservoir=RES, precision=getattr(cd, prec))
    mu = c.bulk(0.25)["mu"]
    c.set_chem_potential(mu)
    c.set_density(np.full(shape, rho0))
    terms, dF = c.eval()
    b = c.bulk(rho0)
    V = np.prod(shape) * dx ** 3
    tol = 1e-8 if prec == "FP64" else 1e-5  # the lattice weights meet the bulk sum rules to ~1e-10
    assert abs(dF.mean() / dx ** 3 - (b["mu"] - mu)) <= tol * max(1.0, abs(b["mu"]))
    assert np.ptp(dF) / dx ** 3 <= tol * max(1.0, abs(b["mu"]))
    omega_v = b["fhelmholtz"] - rho0 * mu  # Omega / V of the uniform state at this mu
    assert abs(terms["Omega"] / V - omega_v) <= (1e-8 if prec == "FP64" else 2e-6) * max(1.0, abs(omega_v))
    c.close()


def test_ao_fp64_128_point_y_axis_matches_the_transposed_lattice(cd, oracle):
    """FP64 with AO keeps FP64 spectra between passes, so a 128-point y axis runs the
    double-float y transform that joins to doubles, including its partial last column
    tile; the lattice with x and y exchanged (32-point y axis, runtime plan) gives the same
    Omega and the transposed dF. The reference's lattice weights themselves depend on the
    axis order at ~3e-9 of max|dF| (the oracle shows the same difference between these two
    lattices without AO), hence the dF bar."""
    dx = 0.1
    rho = oracle.fill_noise((32, 128, 128), 0.3, 0.1, 11)
    out = []
    for shape, r in (((32, 128, 128), rho), ((128, 32, 128), np.ascontiguousarray(rho.transpose(1, 0, 2)))):
        c = cd.Context(shape, dx, cd.WHITEBEAR_I, hsd=1.0, ao_rp=RP, ao_reservoir=RES, precision=cd.FP64)
        c.set_chem_potential(c.bulk(0.25)["mu"])
        c.set_density(r)
        out.append(c.eval())
        c.close()
    (t0, d0), (t1, d1) = out
    for k in ("Omega", "F_id", "F_hs"):
        assert abs(t0[k] - t1[k]) <= 1e-12 * max(1.0, abs(t1[k])), (k, t0[k], t1[k])
    np.testing.assert_allclose(d0, d1.transpose(1, 0, 2), rtol=0, atol=2e-8 * np.abs(d1).max())


@pytest.mark.parametrize("model", ["Rosenfeld", "WhiteBearI"])
@pytest.mark.parametrize("prec", ["FP64", "FP32"])
def test_ao_hessian_product_matches_reference(cd, model, prec):
    """Dynamical_Matrix::matrix_dot_v1 of the AO system against the reference's own product
    (golden ao16.<model>.Hv: its FMT::add_second_derivative, src/FMT.cpp:437-567, takes the
    AO species through the hard-sphere branch); v_i = 0.3 (2u - 1) from splitmix64(77).
    FP64 within 1e-12 of max|Hv|, FP32 within 2e-6."""
    from oracle import pyoracle
    g = golden("ao")
    tag = "ao16." + model
    c = cd.Context(16, 0.2, getattr(cd, {"Rosenfeld": "ROSENFELD", "WhiteBearI": "WHITEBEAR_I"}[model]), hsd=1.0, ao_rp=RP,
                   ao_reservoir=RES, precision=getattr(cd, prec))
    c.set_chem_potential(c.bulk(0.4)["mu"])
    c.set_density(g[tag + ".rho"].reshape(16, 16, 16))
    c.eval()
    v = 0.3 * (pyoracle.fill_noise((16, 16, 16), 1.0, 1.0, 77) - 1.0)
    hv = c.hessian_dot_v(v)
    ref = g[tag + ".Hv"]
    tol = 1e-12 if prec == "FP64" else 2e-6
    assert np.abs(hv.ravel() - ref).max() <= tol * np.abs(ref).max(), np.abs(hv.ravel() - ref).max() / np.abs(ref).max()
    c.close()


def test_ao_reports_what_it_does_not_build(cd):
    c = cd.Context(16, 0.2, cd.WHITEBEAR_I, hsd=1.0, ao_rp=RP, ao_reservoir=RES)
    c.set_density(np.full((16, 16, 16), 0.3))
    c.eval()
    with pytest.raises(cd.CDFTError):
        c.newton_refine(1e-8)
    c.close()
    with pytest.raises(cd.CDFTError):
        cd.Context(16, 0.2, cd.MODEL_NONE, hsd=1.0, lj=True, kT=1.0, ao_rp=RP, ao_reservoir=RES)


def test_ao_fire_lowers_omega(cd):
    """The minimizers run on the AO functional (device FIRE2; Newton-Krylov is not built
    for it, so mixed = 3 takes the FIRE2 policy)."""
    g = golden("ao")
    c = cd.Context(16, 0.2, cd.WHITEBEAR_I, hsd=1.0, ao_rp=RP, ao_reservoir=RES)
    c.set_chem_potential(c.bulk(0.4)["mu"])
    c.set_density(g["ao16.WhiteBearI.rho"].reshape(16, 16, 16))
    t0, _ = c.eval(want_dF=False)
    c.fire_init(force_limit=0.0)
    r = c.fire_run_device(1e-8, max_steps=300, mixed=3)
    t1, _ = c.eval(want_dF=False)
    assert r["newton"] == 0 and t1["Omega"] < t0["Omega"] and t1["resid"] < t0["resid"]
    c.close()


def test_ao_ddft_conserves_mass(cd):
    """DDFT steps on the AO functional: the integrating-factor step keeps the mass."""
    g = golden("ao")
    c = cd.Context(16, 0.2, cd.WHITEBEAR_I, hsd=1.0, ao_rp=RP, ao_reservoir=RES)
    c.set_chem_potential(c.bulk(0.4)["mu"])
    rho = g["ao16.WhiteBearI.rho"].reshape(16, 16, 16)
    c.set_density(rho)
    c.ddft_init(1e-4, 1e-3)
    r = c.ddft_step(20)
    m0 = rho.sum() * 0.2 ** 3
    assert abs(r["mass"] - m0) <= 1e-12 * m0 and np.isfinite(r["F"])
    c.close()
