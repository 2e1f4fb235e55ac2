"""The factorisation behind the eigen drivers on the DDFT matrix (CPU, numpy).

DDFT::g_dot_x (src/DDFT.cpp:320-351, forward differences) is
    (g x)_p = sum_ax D [(rho_p+ + rho_p)(x_p+ - x_p) - (rho_p + rho_p-)(x_p - x_p-)],
D = 1/(2 dx^2). With C the edge-weighted difference operator of the GPU kernels
(k_mob_c / k_mob_ct: (C x)_(ax, p) = sqrt(D (rho_p + rho_p+)) (x_p+ - x_p)), g = -C^T C, and
g.H shares its non-zero eigenvalues with the symmetric -C H C^T; an eigenvector w of the
latter gives the eigenvector C^T w of g.H. Checked here on a small periodic lattice with a
random symmetric H."""
import numpy as np


def _lattice(n):
    idx = np.arange(n ** 3).reshape(n, n, n)
    return idx


def g_matrix(rho, dx):
    n = rho.shape[0]
    N = n ** 3
    idx = _lattice(n)
    D = 1.0 / (2 * dx * dx)
    G = np.zeros((N, N))
    r = rho.ravel()
    for ax in range(3):
        plus = np.roll(idx, -1, axis=ax).ravel()
        minus = np.roll(idx, 1, axis=ax).ravel()
        for p in range(N):
            q, m = plus[p], minus[p]
            G[p, q] += D * (r[q] + r[p])
            G[p, p] -= D * (r[q] + r[p])
            G[p, p] -= D * (r[p] + r[m])
            G[p, m] += D * (r[p] + r[m])
    return G


def c_matrix(rho, dx):
    n = rho.shape[0]
    N = n ** 3
    idx = _lattice(n)
    D = 1.0 / (2 * dx * dx)
    C = np.zeros((3 * N, N))
    r = rho.ravel()
    for ax in range(3):
        plus = np.roll(idx, -1, axis=ax).ravel()
        for p in range(N):
            q = plus[p]
            c = np.sqrt(D * (r[p] + r[q]))
            C[ax * N + p, q] += c
            C[ax * N + p, p] -= c
    return C


def test_mobility_is_minus_ct_c_and_spectra_match():
    rng = np.random.default_rng(3)
    n, dx = 4, 0.2
    rho = 0.3 + 0.1 * rng.random((n, n, n))
    G, C = g_matrix(rho, dx), c_matrix(rho, dx)
    np.testing.assert_allclose(G, -C.T @ C, rtol=0, atol=1e-12 * np.abs(G).max())
    N = n ** 3
    A = rng.standard_normal((N, N))
    H = A @ A.T / N + 0.5 * np.eye(N)  # symmetric positive definite
    lam = np.sort(np.linalg.eigvals(G @ H).real)
    S = -C @ H @ C.T
    mu = np.linalg.eigvalsh(S)
    nz = np.sort(mu[np.abs(mu) > 1e-9 * np.abs(mu).max()])
    # g.H: N - 1 non-zero eigenvalues (the mass mode is the zero one), the same as -C H C^T's
    assert np.sum(np.abs(lam) <= 1e-9 * np.abs(lam).max()) == 1
    np.testing.assert_allclose(np.sort(lam[np.abs(lam) > 1e-9 * np.abs(lam).max()]), nz, rtol=1e-9)
    # eigenvectors: w of -C H C^T gives C^T w of g.H
    w_mu, W = np.linalg.eigh(S)
    i = np.argmax(np.abs(w_mu))
    v = C.T @ W[:, i]
    np.testing.assert_allclose(G @ H @ v, w_mu[i] * v, rtol=0, atol=1e-10 * np.abs(w_mu[i]) * np.linalg.norm(v))
    # the mass mode: g 1 = 0, so g.H (H^-1 1) = 0
    z = np.linalg.solve(H, np.ones(N))
    assert np.abs(G @ H @ z).max() <= 1e-10 * np.abs(G).max() * np.abs(z).max()
