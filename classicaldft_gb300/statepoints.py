"""State-point sweeps: many LJ droplets at once on one GPU.

A sweep draws state points (temperature, chemical-potential offset from bulk
coexistence, droplet radius, cubic grid size), builds one context per point
with the reference's droplet setup (LJ cut-and-shifted, Barker-Henderson
diameter, WhiteBearI + QF mean field; legacy_lib/examples/Droplet/droplet.cpp),
and minimises all of them together with cdft_fire_run_batch.

The bulk densities of a point come from the reference's bulk thermodynamics
(DFT::findCoex, src/DFT_Coex.cpp:159-196; DFT::mu_times_beta, src/DFT.cpp:58-115):
mu = mu_coex(kT) + dmu, the vapour density is the root of mu(rho) = mu below the
first spinodal and the liquid density the root above the second. The droplet
is the reference's tanh profile between the two, and the point is solved at
fixed mass (Species::setFixedMass), where a droplet is a minimum.
"""
import math

import numpy as np

from . import Context, WHITEBEAR_I, bh_diameter, fire_run_batch

GRIDS = tuple(range(48, 161, 16))


def sample_state_points(n, seed, kT_range=(0.7, 0.94), dmu_range=(-0.2, 0.2), R_range=(2.0, 6.0), grids=GRIDS,
                        dx=0.1, R_max_frac=0.4):
    """Seeded draws: kT ~ U[kT_range], dmu ~ U[dmu_range], R ~ U[R_range] clamped to
    R_max_frac * L, grid size uniform over `grids` (cubic, spacing dx).

    The default upper temperature is 0.94: this functional's liquid-vapour
    critical point lies near kT = 0.975, and from kT ~ 0.947 up the reference's
    coexistence search (vapour density divided by 1.1 per step until the
    pressure difference changes sign) steps past the end of the liquid branch
    and fails."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        kT = float(rng.uniform(*kT_range))
        dmu = float(rng.uniform(*dmu_range))
        R = float(rng.uniform(*R_range))
        g = int(grids[int(rng.integers(len(grids)))])
        L = g * dx
        out.append({"kT": kT, "dmu": dmu, "R": min(R, R_max_frac * L), "n": g, "dx": dx})
    return out


def branch_density(mu_of_rho, mu, lo, hi, tol=1e-13, iters=200):
    """Root of mu_of_rho(rho) = mu on [lo, hi], where mu_of_rho is monotone (one bulk branch)."""
    flo = mu_of_rho(lo) - mu
    fhi = mu_of_rho(hi) - mu
    if flo * fhi > 0:
        raise ValueError("mu = %g is not bracketed on [%g, %g]" % (mu, lo, hi))
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        fm = mu_of_rho(mid) - mu
        if (fm < 0) == (flo < 0):
            lo, flo = mid, fm
        else:
            hi = mid
        if hi - lo <= tol * max(1.0, abs(mid)):
            break
    return 0.5 * (lo + hi)


def coexisting_densities(mu_of_rho, coex, dmu, margin=0.1):
    """(mu, rho_vapour, rho_liquid) at mu = mu_coex + dmu.

    dmu is clamped so that mu stays inside both metastable branches: below
    mu(spinodal 1) (the vapour branch ends there) and above mu(spinodal 2),
    with `margin` of that window kept free on each side."""
    mu_hi = mu_of_rho(coex["spinodal1"])
    mu_lo = mu_of_rho(coex["spinodal2"])
    mu0 = coex["mu"]
    w_hi, w_lo = mu_hi - mu0, mu0 - mu_lo
    d = min(max(dmu, -(1 - margin) * w_lo), (1 - margin) * w_hi)
    mu = mu0 + d
    rv = branch_density(mu_of_rho, mu, 1e-12, coex["spinodal1"])
    rl = branch_density(mu_of_rho, mu, coex["spinodal2"], 0.99 * 6 / math.pi)
    return mu, rv, rl


def droplet(shape, dx, rho_v, rho_l, R, width=0.5):
    """rho = rho_v + (rho_l - rho_v) (1 - tanh((r - R)/width))/2, r from the box centre,
    x_i = dx (i - N/2) (Lattice::getX, include/Lattice.h:113-115)."""
    ax = [dx * (np.arange(n) - n / 2.0) for n in shape]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    return rho_v + (rho_l - rho_v) * 0.5 * (1.0 - np.tanh((r - R) / width))


def build_contexts(points, sigma=1.0, eps=1.0, rc=3.0, model=WHITEBEAR_I, precision=0):
    """One fixed-mass droplet context per state point, FIRE-initialised."""
    ctxs = []
    for sp in points:
        kT = sp["kT"]
        hsd = bh_diameter(sigma, eps, rc, kT)
        c = Context((sp["n"],) * 3, sp["dx"], model, hsd=hsd, lj=True, sigma=sigma, eps=eps, rc=rc, kT=kT,
                    precision=precision)
        coex = c.find_coex()

        def mu_of(rho, c=c):
            return c.bulk(rho)["mu"]

        mu, rv, rl = coexisting_densities(mu_of, coex, sp["dmu"])
        rho = droplet((sp["n"],) * 3, sp["dx"], rv, rl, sp["R"])
        sp.update({"mu": mu, "rho_v": rv, "rho_l": rl, "hsd": hsd, "mu_coex": coex["mu"]})
        dV = sp["dx"] ** 3
        c.set_fixed_mass(float(rho.sum() * dV))
        c.set_density(rho)
        c.fire_init()
        ctxs.append(c)
    return ctxs


def solve(points, tol=1e-8, max_steps=-1, mixed=True, switch_tol=2e-6, **kw):
    """Builds the contexts of `points` and minimises them together. Returns (contexts, reports, statuses)."""
    ctxs = build_contexts(points, **kw)
    reps, status = fire_run_batch(ctxs, tol, max_steps=max_steps, mixed=mixed, switch_tol=switch_tol)
    return ctxs, reps, status


def shard(points, rank, world):
    """Replicas-only split of a sweep over `world` GPUs: longest-processing-time
    greedy on the grid cost N^3 log N (largest first, each to the least-loaded
    rank, ties to the lowest rank). Deterministic; every point lands on exactly
    one rank. Returns the indices of `rank`'s points, in sweep order."""
    cost = [p["n"] ** 3 * math.log2(p["n"]) for p in points]
    order = sorted(range(len(points)), key=lambda i: (-cost[i], i))
    load = [0.0] * world
    owner = [0] * len(points)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += cost[i]
    return [i for i in range(len(points)) if owner[i] == rank]
