"""The spectral drivers (cdft_log_det, cdft_eigenvalue, cdft_arnoldi_largest) on the GPU.

Pins (tests/golden/spectral.npz, from oracle/ref_driver case "spectral"):
* Log_Det::calculate_log_det compiled from the reference (src/Log_Det.cpp), at the
  hard-sphere 16^3 state, for the DFT matrix and the DDFT matrix: the same seed gives
  the same +-1 probes, so the estimate itself must agree (1e-10 relative; FFT roundoff
  through the Chebyshev recurrence).
* The eigenvalues of the reference's dense Hessians (every column a matrix_dot_v1 of a
  unit vector), taken with LAPACK: the hard-sphere state (spectrum 0.00904 ... 0.1528,
  a tight cluster at the bottom) and the LJ state at kT = 0.8 (one unstable mode,
  -0.002004, below a band 0.0025 ... 0.0057).
Larger grids are checked against the oracle (log det) and by the eigen-residual
|H y - lambda y| computed with the GPU's own Hessian product."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

SHAPE = (16, 16, 16)


@pytest.fixture(scope="module")
def cd():
    import classicaldft_gb300 as m
    m.lib()
    return m


def hs_context(cd, oracle):
    c = cd.Context(SHAPE, 0.2, cd.WHITEBEAR_I, hsd=1.0)
    c.set_density(oracle.fill_noise(SHAPE, 0.6, 0.2, 11))
    return c


def lj_context(cd, oracle, g):
    c = cd.Context(SHAPE, 0.1, cd.WHITEBEAR_I, hsd=float(g["splj16.hsd"][0]), lj=True, kT=0.8)
    c.set_density(oracle.fill_noise(SHAPE, 0.3, 0.1, 5))
    return c


@pytest.mark.parametrize("tag,order,seed,samples,has_zero,matrix",
                         [("o10", 10, 1234, 3, False, 0), ("o40", 40, 1234, 3, False, 0),
                          ("zero", 20, 77, 2, True, 0), ("ddft", 16, 4321, 2, True, 1)])
def test_log_det_matches_reference(cd, oracle, tag, order, seed, samples, has_zero, matrix):
    g = golden("spectral")
    c = hs_context(cd, oracle)
    lo, hi = g["sp16.logdet.ddft.bounds" if matrix else "sp16.logdet.bounds"]
    val, var = c.log_det(order, hi, lo, seed, samples, has_zero_eigenvalue=has_zero, matrix=matrix)
    ref = g["sp16.logdet." + tag]
    assert abs(val - ref[0]) <= 1e-10 * abs(ref[0]), (val, ref[0])
    assert abs(var - ref[1]) <= 1e-6 * abs(ref[1]), (var, ref[1])
    c.close()


def test_log_det_estimates_the_exact_log_det(cd, oracle):
    """With many probes the estimate approaches sum(log lambda) of the reference's spectrum."""
    g = golden("spectral")
    c = hs_context(cd, oracle)
    lo, hi = g["sp16.logdet.bounds"]
    val, var = c.log_det(40, hi, lo, 99, 64)
    exact = np.sum(np.log(g["sp16.eig"]))
    assert abs(val - exact) <= 4 * var / np.sqrt(64) + 1e-3 * abs(exact), (val, exact, var)
    c.close()


@pytest.mark.parametrize("shape,matrix,prec", [((40, 36, 30), 0, "FP64"), ((64, 64, 64), 0, "FP64"), ((48, 48, 48), 1, "FP64"),
                                               ((64, 64, 64), 0, "FP32")])
def test_log_det_vs_oracle(cd, oracle, shape, matrix, prec):
    """An LJ state on larger (and uneven) grids: the GPU estimator against the oracle's
    restatement, same probes (FP32 bulk passes: 2e-4)."""
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    rho = oracle.fill_noise(shape, 0.3, 0.1, 5)
    o = oracle.Oracle(shape, 0.1, "WhiteBearI", hsd=hsd, lj=True, kT=0.8)
    lo, hi = (1e-4, 0.02) if matrix == 0 else (1e-3, 60.0)
    ref, rvar = o.log_det(rho, 8, hi, lo, 2024, 1, has_zero=bool(matrix), dynamic=bool(matrix))
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8, precision=getattr(cd, prec))
    c.set_density(rho)
    val, var = c.log_det(8, hi, lo, 2024, 1, has_zero_eigenvalue=bool(matrix), matrix=matrix)
    tol = 1e-10 if prec == "FP64" else 2e-4
    assert abs(val - ref) <= tol * abs(ref), (val, ref)
    c.close()


def _residual(c, lam, y):
    hy = c.hessian_dot_v(y.reshape(c.shape))
    return np.linalg.norm(hy.ravel() - lam * y.ravel())


def test_eigenvalue_unstable_mode_lj(cd, oracle):
    """Eigenvalues::calculate_eigenvector: the LJ state's one negative eigenvalue."""
    g = golden("spectral")
    c = lj_context(cd, oracle, g)
    lam, y, rep = c.eigenvalue(tol=1e-10)
    ref = g["splj16.eig"][0]
    assert rep["converged"] and abs(lam - ref) <= 1e-9 * abs(ref), (lam, ref, rep)
    assert abs(np.dot(y.ravel(), g["splj16.evec_min"])) >= 1 - 1e-9
    assert abs(np.linalg.norm(y) - 1) <= 1e-12
    assert _residual(c, lam, y) <= 1e-8 * abs(lam)
    c.close()


def test_eigenvalue_change_sign_and_scale(cd, oracle):
    """change_sign gives the largest eigenvalue (hard spheres: 0.15275, isolated); the
    scale only scales the objective."""
    g = golden("spectral")
    c = hs_context(cd, oracle)
    ref = g["sp16.eig"][-1]
    for scale in (1e6, 1.0):
        lam, y, rep = c.eigenvalue(scale=scale, tol=1e-10, change_sign=True)
        assert rep["converged"] and abs(lam - ref) <= 1e-9 * ref, (scale, lam, ref, rep)
        assert abs(np.dot(y.ravel(), g["sp16.evec_max"])) >= 1 - 1e-9
    c.close()


@pytest.mark.parametrize("tag", ["splj16", "sp16"])
def test_eigenvalue_with_vshift(cd, oracle, tag):
    """set_vshift: the smallest eigenvalue of H + vshift vshift^T / 2 (the hard-sphere
    one sits in a cluster 2e-5 wide, so it takes more products)."""
    g = golden("spectral")
    c = lj_context(cd, oracle, g) if tag == "splj16" else hs_context(cd, oracle)
    lam, y, rep = c.eigenvalue(tol=1e-8, vshift=g[tag + ".vshift"], max_matvecs=40000)
    ref = g[tag + ".eig_vshift"][0]
    assert rep["converged"] and abs(lam - ref) <= 1e-8 * abs(ref), (lam, ref, rep)
    c.close()


def test_eigenvalue_bottom_of_a_cluster(cd, oracle):
    g = golden("spectral")
    c = hs_context(cd, oracle)
    lam, y, rep = c.eigenvalue(tol=1e-8, max_matvecs=40000)
    ref = g["sp16.eig"][0]
    assert rep["converged"] and abs(lam - ref) <= 1e-8 * ref, (lam, ref, rep)
    assert _residual(c, lam, y) <= 2e-8 * lam
    c.close()


def test_arnoldi_largest_pairs(cd, oracle):
    """Arnoldi::determine_largest_eigenpairs(0, 4, 12): the four largest eigenvalues of
    the hard-sphere Hessian, each its own value (in magnitude order)."""
    g = golden("spectral")
    c = hs_context(cd, oracle)
    vals, vecs, rep = c.arnoldi(0.0, 4, 12, tol=1e-8)
    ref = g["sp16.eig"][::-1][:4]
    assert rep["converged"]
    np.testing.assert_allclose(vals, ref, rtol=1e-9, atol=0)
    for lam, y in zip(vals, vecs):
        assert _residual(c, lam, y) <= 1e-7 * abs(lam)
    c.close()


def test_arnoldi_shift_selects_the_unstable_mode(cd, oracle):
    """With shift = -0.006 the largest |lambda + shift| is the LJ state's negative mode."""
    g = golden("spectral")
    c = lj_context(cd, oracle, g)
    vals, vecs, rep = c.arnoldi(-0.006, 1, 15, tol=1e-10, all_k=False)
    ref = g["splj16.eig"][0]
    assert rep["converged"] and abs(vals[0] - ref) <= 1e-9 * abs(ref), (vals, ref, rep)
    assert abs(np.dot(vecs[0].ravel(), g["splj16.evec_min"])) >= 1 - 1e-9
    c.close()


def test_arnoldi_reports_max_steps(cd, oracle):
    """The reference throws after maxSteps restarts; here CDFT_ERR_TIMEOUT."""
    c = hs_context(cd, oracle)
    with pytest.raises(cd.CDFTError) as e:
        c.arnoldi(-0.2, 3, 2, max_steps=2, tol=1e-14)
    assert e.value.code == cd.ERR_TIMEOUT
    c.close()


def test_eigen_drivers_at_128_uniform_state(cd):
    """A uniform LJ fluid at 128^3 (rho = 0.3, kT = 0.8, inside the spinodal): the Hessian
    is translation invariant, so plane waves diagonalise it and its whole spectrum is the
    FFT of one column, H e_0 (taken with the GPU's own product). Eigenvalues must find the
    smallest of those values and Arnoldi the largest in magnitude."""
    shape = (128, 128, 128)
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, 0.8)
    c = cd.Context(shape, 0.1, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=0.8)
    c.set_density(np.full(shape, 0.3))
    e0 = np.zeros(shape)
    e0[0, 0, 0] = 1.0
    spec = np.fft.fftn(c.hessian_dot_v(e0))
    assert np.abs(spec.imag).max() <= 1e-12 * np.abs(spec.real).max()
    spec = np.sort(spec.real.ravel())
    lam, y, rep = c.eigenvalue(tol=1e-8, max_matvecs=3000)
    assert rep["converged"] and abs(lam - spec[0]) <= 1e-9 * np.abs(spec).max(), (lam, spec[:3], rep)
    assert _residual(c, lam, y) <= 1e-7 * abs(lam)
    vals, vecs, rep = c.arnoldi(0.0, 2, 14, all_k=False, tol=1e-8)
    top = spec[np.argmax(np.abs(spec))]
    assert rep["converged"] and abs(vals[0] - top) <= 1e-9 * abs(top), (vals, top, rep)
    assert _residual(c, vals[0], vecs[0]) <= 1e-7 * abs(vals[0])
    c.close()


def test_spectral_drivers_on_ao_system(cd, oracle):
    """The reference's Hessian of an FMT_AO_Species system is its hard-sphere FMT Hessian plus
    the ideal gas (FMT::add_second_derivative takes the AO species through the plain branch),
    so the spectral drivers on an AO system give what they give on the same density without
    polymers: Log_Det with the same probes, and the smallest eigenvalue."""
    rho = oracle.fill_noise(SHAPE, 0.6, 0.2, 11)
    out = []
    for ao in (True, False):
        kw = dict(ao_rp=0.35, ao_reservoir=0.4) if ao else {}
        c = cd.Context(SHAPE, 0.2, cd.WHITEBEAR_I, hsd=1.0, **kw)
        c.set_density(rho)
        c.eval()
        ld, _ = c.log_det(10, 0.16, 0.008, 1234, 2)
        lam, _, rep = c.eigenvalue(tol=1e-9, max_matvecs=40000)
        assert rep["converged"]
        out.append((ld, lam))
        c.close()
    assert abs(out[0][0] - out[1][0]) <= 1e-12 * abs(out[1][0])
    assert abs(out[0][1] - out[1][1]) <= 1e-9 * abs(out[1][1])


def _ddft_residual(c, lam, y):
    gy = c.ddft_matrix_dot_v(y)
    return float(np.linalg.norm(gy.ravel() - lam * y.ravel()))


def test_arnoldi_ddft_matrix_largest_pairs(cd, oracle):
    """Arnoldi(ddft).determine_largest_eigenpairs(0, 4, 16) on the DDFT dynamical matrix
    g.H of the hard-sphere state: the four eigenvalues of largest magnitude (the fastest
    relaxing modes) of the reference's dense g.H (every column a DDFT::matrix_dot_v1,
    eigenvalues by LAPACK), and unit eigenvectors with g.H y = lambda y."""
    g = golden("spectral")
    c = hs_context(cd, oracle)
    vals, vecs, rep = c.arnoldi(0.0, 4, 16, tol=1e-9, matrix=cd.MATRIX_DDFT)
    ref = g["sp16.G.eig"]
    ref = ref[np.argsort(-np.abs(ref))][:4]
    assert rep["converged"], rep
    np.testing.assert_allclose(vals, ref, rtol=1e-9, atol=0)
    for lam, y in zip(vals, vecs):
        assert abs(np.linalg.norm(y) - 1) <= 1e-12
        assert _ddft_residual(c, lam, y) <= 1e-7 * abs(lam)
    # the isolated fastest mode: the reference's eigenvector, up to sign
    assert abs(np.dot(vecs[0].ravel(), g["sp16.G.evec_top0"])) >= 1 - 1e-8
    c.close()


def test_arnoldi_ddft_matrix_shift_selects_slow_modes_and_mass_mode(cd, oracle):
    """With shift = 2.5 the largest |lambda + shift| are the conserved-mass mode (lambda = 0,
    eigenvector H^-1 1) and then the slowest relaxing modes of g.H, as in the reference's
    spectrum."""
    g = golden("spectral")
    c = hs_context(cd, oracle)
    vals, vecs, rep = c.arnoldi(2.5, 3, 20, tol=1e-9, matrix=cd.MATRIX_DDFT)
    ref = g["sp16.G.eig"]
    ref = ref[np.argsort(-np.abs(ref + 2.5))][:3]
    assert rep["converged"], rep
    assert vals[0] == 0.0 and abs(ref[0]) <= 1e-12
    np.testing.assert_allclose(vals[1:], ref[1:], rtol=1e-9, atol=0)
    assert _ddft_residual(c, 0.0, vecs[0]) <= 1e-9
    for lam, y in zip(vals[1:], vecs[1:]):
        assert _ddft_residual(c, lam, y) <= 1e-7 * abs(lam)
    c.close()


def test_arnoldi_ddft_matrix_fixed_background(cd, oracle):
    """With a fixed background the boundary is held (g and H act on interior points only),
    so there is no mass mode: every returned pair satisfies g.H y = lambda y with y zero on
    the boundary planes."""
    c = hs_context(cd, oracle)
    c.set_boundary(fixed_background=True)
    vals, vecs, rep = c.arnoldi(2.5, 2, 20, tol=1e-9, matrix=cd.MATRIX_DDFT)
    assert rep["converged"] and np.all(vals < 0)
    for lam, y in zip(vals, vecs):
        assert np.abs(y[0, :, :]).max() == 0 and np.abs(y[:, 0, :]).max() == 0 and np.abs(y[:, :, 0]).max() == 0
        assert _ddft_residual(c, lam, y) <= 1e-7 * abs(lam)
    c.close()
