"""Benchmark: F+dF evaluations per second at 128^3 (the LJ droplet system:
WhiteBearI FMT + QF mean field of the cut-and-shifted LJ, kT = 0.8, dx = 0.1),
one JSON line on stdout.

`value`  FP64 evaluations/s (the reference's precision) with the density resident
         in HBM, timed with CUDA events per step; L2 flushed between steps.
`e2e`    the same FP64 evaluation through the public C ABI from host buffers
         (host density in, host dF out, copies inside the timed region).
`roofline`  the dominant pass of the FP64 evaluation (the Phi pass), which does its
         arithmetic in double-float on the FP32 pipe: its executed FP32 work (ncu count
         per launch) over its event-timed duration against the FP32 FMA rate measured in
         the same run, with its HBM fraction and its FP64-equivalent rate (the all-FP64
         form's work over this time, against the measured FP64 unit rate) beside it.
`fp32`   the FP32-bulk evaluation of the same system (FP64 reductions): its rate,
         its error against FP64 on the same density, its HBM roofline.
Extra keys: per-pass breakdowns, the time-to-residual legs (their converged
densities checked by the FP64 oracle in the CPU leg), the 256^3 evaluation and
DDFT legs (FP32 against an FP64 run of the same trajectory), the state-point
sweep, the spectral drivers, the learned warm start, and the oracle CPU baseline.
With --impl reference the FP64 CPU oracle (the port of the reference's path; the
reference itself needs FFTW/GSL/Boost/Armadillo, absent on the GPU machines) is
timed on all host cores.
Multi-GPU: replicas only (each rank evaluates its own system); value is the sum.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FMT F+dF evals/s at 128^3; s to resid 1e-8: warm-start mixed vs plain FP64"
SHAPE, DX, KT, R_DROP, W_DROP, RHO_V, RHO_L = (128, 128, 128), 0.1, 0.8, 4.0, 0.5, 0.01, 0.75


def droplet():
    ax = [DX * (np.arange(m) - m / 2.0) for m in SHAPE]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    return RHO_V + (RHO_L - RHO_V) * 0.5 * (1 - np.tanh((r - R_DROP) / W_DROP))


def workload():
    return {"workload": "LJ droplet F+dF evaluation, 128^3, dx=0.1, WhiteBearI + QF mean field, kT=0.8, "
                        "rho_v=0.01, rho_l=0.75, R=4, w=0.5, grand canonical at mu(rho_v)",
            "grid": list(SHAPE), "model": "WhiteBearI", "interaction": "QF", "precision": "fp64 throughout",
            "l2": "flushed between timed steps (256 MB write)"}


# DRAM bytes per launch (read + write) from one ncu capture of the named kernel on
# this workload; None where none was taken.
NCU_TRAFFIC = {("phi_rows", "fp32"): 98.1e6 + 40.0e6, ("phi_rows", "fp64"): 196.20e6 + 131.81e6}
# FP64-equivalent work per launch of a pass: the FP64 add/mul/fma instructions (fma = 2)
# the pass executes when all its arithmetic is FP64 (ncu on that build:
# smsp__sass_thread_inst_executed_op_{dadd,dmul}_pred_on.sum + 2 x ..._dfma_pred_on.sum).
NCU_FP64_FLOPS = {"phi_rows": 424.27e6 + 266.25e6 + 2 * 306.44e6}
# What the shipped FP64 pass executes instead: its arithmetic runs in double-float on the
# FP32 pipe. FP32 work per launch (ncu: smsp__sass_thread_inst_executed_op_{fadd,fmul}_pred_on.sum
# + 2 x ..._ffma_pred_on.sum), how busy it keeps the FMA pipe
# (sm__inst_executed_pipe_fma.avg.pct_of_peak_sustained_active) and the issue slots
# (smsp__issue_active.avg.pct_of_peak_sustained_active); None where none was taken.
NCU_FP32_FLOPS = {"phi_rows": 5663.90e6 + 551.00e6 + 2 * 1457.09e6}
NCU_FMA_PIPE_BUSY = {"phi_rows": 0.503}
NCU_ISSUE_ACTIVE = {"phi_rows": 0.655}
# FP64 instructions the shipped pass still executes (same counters)
NCU_FP64_EXECUTED = {"phi_rows": 0.703e6 + 0.078e6 + 2 * 0.778e6}


def fma_peak(cd, fn):
    """The device's sustained FMA rate in TFLOP/s for one precision, measured now."""
    import ctypes
    v = ctypes.c_double()
    if getattr(cd.lib(), fn)(ctypes.byref(v), None) != 0:
        return None
    return v.value


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def __enter__(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,"
                                          "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                                          "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                    vals = [v.strip() for v in out.stdout.strip().split(",")]
                    if len(vals) >= 6:
                        self.samples.append(vals)
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def cpu_baseline(budget_s=15.0, steps=None):
    # every host core: torchrun sets OMP_NUM_THREADS=1 for its ranks, and only one rank runs this
    os.environ["OMP_NUM_THREADS"] = str(os.cpu_count())
    from oracle import pyoracle
    o = pyoracle.Oracle(SHAPE, DX, "WhiteBearI", hsd=None, lj=True, kT=KT)
    o.set_mu(o.mu_times_beta(RHO_V))
    rho = droplet()
    o.eval(rho)  # warm-up (plans, threads)
    n, t0 = 0, time.perf_counter()
    while True:
        o.eval(rho)
        n += 1
        el = time.perf_counter() - t0
        if (steps is not None and n >= steps) or (steps is None and el > budget_s):
            break
    return n / el, n, el


def oracle_pins(kept):
    """The CPU leg's check of the converged 128^3 droplets: one FP64 oracle evaluation
    (fixed mass, the same hard-sphere diameter) of each end density the time-to-residual
    legs reached, its Omega against the GPU's and its own max|dOmega/drho|."""
    from oracle import pyoracle
    out = {}
    for name, (rho, omega_gpu, mass, hsd) in kept.items():
        o = pyoracle.Oracle(SHAPE, DX, "WhiteBearI", hsd=hsd, lj=True, kT=KT, fixed_mass=mass)
        _, t, dF, _ = o.eval(rho)
        out[name] = {"omega_oracle": t["Omega"], "omega_gpu": omega_gpu,
                     "omega_rel_vs_oracle": abs(omega_gpu - t["Omega"]) / abs(t["Omega"]),
                     "oracle_resid": float(np.abs(dF).max() / DX ** 3)}
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps = max(1, args.steps)
    rate, n, el = cpu_baseline(steps=steps)  # its first evaluation is an untimed warm-up
    cores = int(os.environ["OMP_NUM_THREADS"])
    line = {"metric": METRIC, "impl": "reference", "value": rate, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload(),
            "cpu_baseline": {"value": rate, "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": "%d FP64 F+dF evaluations of the 128^3 LJ droplet (OpenMP, %d threads)" % (n, cores)},
            "e2e": {"value": rate, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ddft_initial_density(n=256, dx=0.1, seed=3, rho0=0.3, amp=0.1, ell=1.0):
    """rho = rho0 (1 + amp g), g Gaussian-filtered white noise (exp(-k^2 ell^2/2)), unit std, seeded."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n))
    k = 2 * np.pi * np.fft.fftfreq(n, d=dx)
    kz = 2 * np.pi * np.fft.rfftfreq(n, d=dx)
    K2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
    g = np.fft.irfftn(np.fft.rfftn(w) * np.exp(-K2 * ell ** 2 / 2), s=(n, n, n), axes=(0, 1, 2))
    g /= g.std()
    return np.maximum(rho0 * (1 + amp * g), 1e-6)


def ddft_leg(cd, n=256, steps=2000, compare_at=101):
    """Integrating-factor DDFT of the LJ system at 256^3, dx = 0.1, dt = 1e-4 fixed.
    FP32 bulk with the FP64 mass restore: one warm-up step, then 2000 timed steps (wall
    time, ms per step, and the largest mass deviation the restore corrected). The same
    FP32 run without the restore gives the propagator's own FP32 mass drift over the
    whole run. An FP64 run of the first `compare_at` steps (the reference's arithmetic)
    gives the FP32 trajectory's error at that step, with and without the restore."""
    import torch
    rho = ddft_initial_density(n)
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, KT)
    m0 = float(np.sum(rho)) * DX ** 3

    def ctx(prec, restore=True):
        c = cd.Context((n, n, n), DX, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=KT, precision=prec)
        c.set_chem_potential(c.bulk(0.3)["mu"])
        c.set_density(rho)
        c.ddft_init(1e-4, 1e-4)
        c.ddft_set_mass_restore(restore)
        return c

    c = ctx(cd.FP32)
    c.ddft_step(1)  # warm-up: step 1 of the trajectory
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    c.ddft_step(compare_at - 1)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    d32 = c.get_density()  # outside the timing
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = c.ddft_step(steps - (compare_at - 1))
    torch.cuda.synchronize()
    el = (el + time.perf_counter() - t0) / steps
    out = {"grid": [n, n, n], "dt": 1e-4, "ms_per_step": 1e3 * el, "steps_timed": steps,
           "run_s": steps * el, "precision": "fp32 bulk, fp64 mass restore",
           "mass_rel_drift": abs(r["mass"] - m0) / m0,
           "mass_note": "zero by construction: each propagated density is shifted back to the starting mass",
           "restore_max_rel_correction": c.ddft_mass_deviation()}
    c.close()
    c = ctx(cd.FP32, restore=False)
    c.ddft_step(compare_at)
    d32n = c.get_density()
    r = c.ddft_step(steps + 1 - compare_at)
    out["no_restore"] = {"steps": steps + 1, "mass_rel_drift": abs(r["mass"] - m0) / m0,
                         "max_rel_mass_deviation": c.ddft_mass_deviation()}
    c.close()
    c = ctx(cd.FP64)
    t0 = time.perf_counter()
    r64 = c.ddft_step(compare_at)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    d64 = c.get_density()
    c.close()
    out["vs_fp64"] = {"step": compare_at, "fp64_ms_per_step": 1e3 * t64 / compare_at,
                      "fp64_mass_rel_drift": abs(r64["mass"] - m0) / m0,
                      "max_abs_rho_diff": float(np.abs(d32 - d64).max()),
                      "max_abs_rho_diff_no_restore": float(np.abs(d32n - d64).max()),
                      "max_rho": float(d64.max()), "min_rho": float(d64.min())}
    return out


def eval_256_leg(cd, steps=10):
    """The FP32 evaluation at 256^3 (dx = 0.1, the same droplet functional), where the
    working set (~1.4 GB of spectra) cannot stay in L2 between passes: evals/s and the
    fraction of the measured HBM bandwidth against B_DFT."""
    import torch
    n = 256
    c = cd.Context((n, n, n), DX, cd.WHITEBEAR_I, hsd=cd.bh_diameter(1.0, 1.0, 3.0, KT), lj=True, kT=KT, precision=cd.FP32)
    c.set_chem_potential(c.bulk(RHO_V)["mu"])
    c.set_density(ddft_initial_density(n))
    for _ in range(3):
        c.eval(want_dF=False)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        c.eval(want_dF=False)
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    passes = c.time_passes(reps=3)
    N, Nc = n ** 3, n * n * (n // 2 + 1)
    B = 4 * (N * (4 * 11 + 3) + Nc * (2 * 11 + 11))
    peak = measured_peaks()[0]
    c.close()
    return {"grid": [n, n, n], "evals_per_s": 1e3 / ms, "ms": ms, "algorithmic_bytes": B,
            "achieved_gbs": B / (ms * 1e-3) / 1e9, "frac": B / (ms * 1e-3) / 1e9 / peak,
            "passes": [{"pass": p["pass"], "ms": round(p["ms"], 4), "GBs": round(p["bytes"] / max(p["ms"], 1e-9) / 1e6, 1)}
                       for p in passes]}


def spectral_leg(cd, rho):
    """The spectral drivers at 128^3 on the droplet functional (host clock around each
    call; every call synchronises): Log_Det (order 20, 2 probes = 40 Hessian products) on
    the droplet density in FP64 and FP32, and Eigenvalues on the uniform fluid at
    rho = 0.3 (its smallest eigenvalue, the unstable k = 0 mode, to a residual of 1e-8)."""
    n = 128
    out = {"grid": [n, n, n]}
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, KT)
    for prec in ("FP64", "FP32"):
        c = cd.Context((n, n, n), DX, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=KT, precision=getattr(cd, prec))
        c.set_density(rho)
        c.log_det(2, 0.2, 1e-4, 1, 1)  # warm-up (buffers, weighted densities)
        t0 = time.perf_counter()
        val, var = c.log_det(20, 0.2, 1e-4, 1234, 2)
        el = time.perf_counter() - t0
        out["log_det_" + prec.lower()] = {"seconds": el, "hessian_products": 40, "products_per_s": 40 / el, "log_det": val}
        c.close()
    c = cd.Context((n, n, n), DX, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=KT)
    c.set_density(np.full((n, n, n), 0.3))
    t0 = time.perf_counter()
    lam, _, rep = c.eigenvalue(tol=1e-8, max_matvecs=3000)
    out["eigenvalue_uniform_fp64"] = {"seconds": time.perf_counter() - t0, "eigenvalue": lam, **rep}
    c.close()
    return out


def fire_legs(cd, rho, tol=1e-8, max_steps=20000, legs=("newton", "mixed_newton", "mixed_fire", "plain_fp64"), keep=None):
    """Wall seconds to reach max|dOmega/drho| <= tol on the droplet at fixed mass,
    every leg device-resident and starting from the same tanh profile, FIRE2 with
    the reference defaults (dt = 1e-3, dt_max = 1e-2):
      plain_fp64    FIRE2 with FP64 evaluations throughout;
      mixed_fire    FP32 FIRE2 bulk phase to its noise floor, then FP64 FIRE2;
      mixed_newton  FP32 FIRE2 bulk phase to resid 1e-4, then Newton-Krylov
                    refinement (FP32 Hessian products, FP64 residuals);
      newton        Newton-Krylov from the start (FP32 Hessian products, FP64
                    residuals and line search).
    Each end state is re-evaluated in FP64; with `keep` (a dict) each end density is
    kept there for the oracle's check of the converged state."""
    import torch
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, KT)
    mass = float(rho.sum()) * DX ** 3
    out = {"start": "tanh droplet (no learned warm start)", "ensemble": "fixed mass", "tol": tol,
           "mixed_fire": "FP32 FIRE2 until resid <= 2e-6 or 96 steps without a 2% improvement, then FP64 FIRE2",
           "mixed_newton": "FP32 FIRE2 until resid <= 1e-4, then Newton-Krylov (CG to 1e-3, FP32 Hessian products)",
           "newton": "Newton-Krylov from the tanh profile (CG to 1e-3, FP32 Hessian products, FP64 residuals)"}
    res = {}
    for name, mixed, sw in (("newton", 3, 1e-4), ("mixed_newton", 2, 1e-4), ("mixed_fire", 1, 2e-6), ("plain_fp64", 0, 2e-6)):
        if name not in legs:
            continue
        c = cd.Context(SHAPE, DX, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=KT, fixed_mass=mass)
        c.set_density(rho)
        c.fire_init(force_limit=0.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = c.fire_run_device(tol, max_steps=max_steps, mixed=mixed, switch_tol=sw)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        t, _ = c.eval(want_dF=False)  # FP64 re-evaluation of the end state
        res[name] = {"seconds": el, "fire_steps": r["total_steps"], "fp32_steps": r["steps_fp32"],
                     "newton": r["newton"], "cg_iters": r["cg_iters"], "resid": t["resid"],
                     "Omega": t["Omega"], "converged": bool(t["resid"] <= tol)}
        if keep is not None:
            keep[name] = (c.get_density(), t["Omega"], mass, hsd)
        c.close()
    out.update(res)
    if len(res) < 4:  # a subset of the legs (e.g. for a profile): no ratios
        return out
    plain = res["plain_fp64"]
    out["speedup_mixed_vs_plain"] = plain["seconds"] / res["newton"]["seconds"]
    out["speedup_mixed_newton_vs_plain"] = plain["seconds"] / res["mixed_newton"]["seconds"]
    out["speedup_mixed_fire_vs_plain"] = plain["seconds"] / res["mixed_fire"]["seconds"]
    out["omega_rel_diff"] = max(abs(res[k]["Omega"] - plain["Omega"]) / abs(plain["Omega"])
                                for k in ("newton", "mixed_newton", "mixed_fire"))
    return out


def batch_leg(cd, n=64, seed=2024, tol=1e-8, max_steps=20000, grids=(48, 64, 80, 96, 112, 128, 144, 160), rank=0, world=1, dist=None):
    """State-point sweep: n LJ droplets (kT ~ U[0.7, 0.94], mu = mu_coex(kT) + U[-0.2, 0.2],
    R ~ U[2, 6] clamped to 0.4 L, cubic grids drawn from `grids`, dx = 0.1, fixed mass),
    all minimised to max|dOmega/drho| <= tol by Newton-Krylov (FIRE2 fallback). Batched
    (cdft_fire_run_batch: contexts spread over host threads, each on its own stream)
    vs one after another (cdft_fire_run_device); context set-up is outside both timings."""
    import torch
    from classicaldft_gb300 import statepoints as sp
    pts_all = sp.sample_state_points(n, seed=seed, grids=grids)
    # replicas only: with several GPUs each rank takes its share of the points (no exchange)
    pts = [pts_all[i] for i in sp.shard(pts_all, rank, world)] if world > 1 else pts_all
    out = {"points": n, "ranks": world, "seed": seed, "tol": tol, "grids": sorted(p["n"] for p in pts),
           "ensemble": "fixed mass droplets",
           "precision": "Newton-Krylov from the tanh profile (FP32 Hessian products, FP64 residuals), FIRE2 fallback"}
    ctxs = sp.build_contexts([dict(p) for p in pts])
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    reps, status = cd.fire_run_batch(ctxs, tol, max_steps=max_steps, mixed=3, switch_tol=1e-4)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t0
    conv = sum(1 for r, s in zip(reps, status) if s == 0 and r["resid"] <= tol)
    steps = sum(r["total_steps"] for r in reps)
    nk = sum(r["newton"] for r in reps)
    ncg = sum(r["cg_iters"] for r in reps)
    if dist:  # the job's time is the slowest rank's; tallies add up
        t = torch.tensor([tb, conv, steps, nk, ncg], dtype=torch.float64, device="cuda")
        tmax = t[:1].clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        tb, conv, steps, nk, ncg = float(tmax.item()), int(t[1].item()), int(t[2].item()), int(t[3].item()), int(t[4].item())
    out["batched_s"] = tb
    out["converged"] = int(conv)
    out["total_steps"] = int(steps)
    out["newton_corrections"] = int(nk)
    out["cg_iters"] = int(ncg)
    out["state_points_per_s"] = n / tb
    omega_b = [r["F"] for r in reps]
    for c in ctxs:
        c.close()
    if world > 1:  # the one-after-another comparison is a single-GPU measurement
        return out
    ctxs = sp.build_contexts([dict(p) for p in pts])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq = [c.fire_run_device(tol, max_steps=max_steps, mixed=3, switch_tol=1e-4) for c in ctxs]
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    for c in ctxs:
        c.close()
    out["sequential_s"] = ts
    out["speedup_batched_vs_sequential"] = ts / tb
    out["same_minima"] = bool(all(a == r["F"] for a, r in zip(omega_b, seq)))
    return out


def warm_start_leg(cd, n_train=120, n_test=8, steps=600, tol=1e-8, plain_fp64_s=None):
    """Neural-operator warm start: converged 128^3 droplets around the benchmark
    point (kT ~ U[0.75, 0.9], rho_v ~ U[0.005, 0.04], rho_l ~ U[0.6, 0.8],
    R ~ U[3, 5], fixed mass) from the Newton-Krylov solver, a 4-layer FNO (width 32,
    12 modes per axis, BF16 tcgen05 GEMMs) trained on them, then the benchmark
    droplet solved from the operator's prediction vs from the tanh profile, by
    Newton-Krylov and by the mixed FP32 -> FP64 FIRE2 policy (the latter against
    plain FP64 FIRE2 from the tanh profile, plain_fp64_s, when given)."""
    import torch
    from classicaldft_gb300 import fno
    out = {"train": n_train, "test": n_test, "steps": steps, "width": fno.WIDTH, "modes": fno.MODES, "layers": fno.LAYERS}
    t0 = time.perf_counter()
    samples = fno.solve_droplets(fno.sample_droplets(n_train + n_test, seed=11), SHAPE, DX)
    out["data_s"] = time.perf_counter() - t0
    train, test = samples[:n_train], samples[n_train:]
    # one-time costs of the first training steps in a process (library kernels compiled for
    # this GPU on first use, allocator growth), kept out of train_s and reported apart
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fno.train(fno.FNO3d(), train[:1], SHAPE, steps=2)
    torch.cuda.synchronize()
    out["first_use_s"] = time.perf_counter() - t0
    model = fno.FNO3d()
    log = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fno.train(model, train, SHAPE, steps=steps, log=log)
    torch.cuda.synchronize()
    out["train_s"] = time.perf_counter() - t0
    out["loss"] = [round(l, 6) for _, l in log]
    # held-out error of log rho: operator vs the seed alone
    e_seed, e_fno = [], []
    for seed, kT, rho in test:
        pred = fno.predict(model, seed, kT, SHAPE)
        up = np.exp(fno.upsample(np.log(seed), SHAPE).numpy())
        lr = np.log(rho)
        e_fno.append(float(np.sqrt(np.mean((np.log(pred) - lr) ** 2))))
        e_seed.append(float(np.sqrt(np.mean((np.log(up) - lr) ** 2))))
    out["test_rms_log_error"] = {"operator": e_fno, "seed": e_seed}
    # the benchmark droplet, cold (tanh) vs warm (operator) start, Newton-Krylov both
    rho0 = droplet()
    mass = float(rho0.sum()) * DX ** 3
    hsd = cd.bh_diameter(1.0, 1.0, 3.0, KT)
    res = {}
    for name in ("cold", "warm"):
        c = cd.Context(SHAPE, DX, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=KT, fixed_mass=mass)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        start = rho0 if name == "cold" else fno.predict(model, fno.coarse_seed(SHAPE, DX, RHO_V, RHO_L, R_DROP), KT, SHAPE,
                                                        on_device=True)
        c.set_density(start)
        c.fire_init(force_limit=0.0)
        r = c.fire_run_device(tol, max_steps=20000, mixed=3)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        t, _ = c.eval(want_dF=False)
        res[name] = {"seconds": el, "newton": r["newton"], "cg_iters": r["cg_iters"], "fire_steps": r["total_steps"],
                     "resid": t["resid"], "Omega": t["Omega"]}
        c.close()
    # warm start + mixed FIRE2 (FP32 bulk phase, then FP64 FIRE2): the warm-started mixed-precision FIRE2 policy
    c = cd.Context(SHAPE, DX, cd.WHITEBEAR_I, hsd=hsd, lj=True, kT=KT, fixed_mass=mass)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    c.set_density(fno.predict(model, fno.coarse_seed(SHAPE, DX, RHO_V, RHO_L, R_DROP), KT, SHAPE, on_device=True))
    c.fire_init(force_limit=0.0)
    r = c.fire_run_device(tol, max_steps=20000, mixed=1, switch_tol=2e-6)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    t, _ = c.eval(want_dF=False)
    res["warm_mixed_fire"] = {"seconds": el, "fire_steps": r["total_steps"], "fp32_steps": r["steps_fp32"], "resid": t["resid"],
                              "Omega": t["Omega"]}
    if plain_fp64_s:
        res["warm_mixed_fire"]["speedup_vs_plain_fp64_fire_from_tanh"] = plain_fp64_s / el
    c.close()
    out.update(res)
    out["speedup_warm_vs_cold"] = res["cold"]["seconds"] / res["warm"]["seconds"]
    seed = fno.coarse_seed(SHAPE, DX, RHO_V, RHO_L, R_DROP)
    for _ in range(2):
        fno.predict(model, seed, KT, SHAPE, on_device=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fno.predict(model, seed, KT, SHAPE, on_device=True)
    torch.cuda.synchronize()
    out["predict_ms"] = (time.perf_counter() - t0) * 1e3  # inside the warm timing above
    # the operator's pointwise layer on the tensor cores: Y = GELU(X W + b + add), 128^3 rows, K = N = 32
    M, K, N = int(np.prod(SHAPE)), fno.WIDTH, fno.WIDTH
    x = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    w = (torch.randn(K, N, device="cuda") / K ** 0.5).to(torch.bfloat16)
    b = torch.zeros(N, device="cuda")
    add = torch.randn(M, N, device="cuda")
    for _ in range(3):
        fno.tc_gemm(x, w, b, add, act=1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    e0.record()
    for _ in range(reps):
        fno.tc_gemm(x, w, b, add, act=1)
    e1.record()
    e1.synchronize()
    fno.check_status()
    ms = e0.elapsed_time(e1) / reps
    by = M * K * 2 + M * N * 4 * 2 + K * N * 2 + N * 4  # X in, add in, Y out
    peaks = measured_peaks()
    out["tc_gemm"] = {"kernel": "k_gemm_bf16<32,32> (tcgen05.mma kind::f16, TMEM accumulator)", "rows": M, "K": K, "N": N,
                      "ms": ms, "GBs": by / (ms * 1e-3) / 1e9, "TFLOPs": 2.0 * M * K * N / (ms * 1e-3) / 1e12,
                      "hbm_frac": by / (ms * 1e-3) / 1e9 / peaks[0], "bound": "hbm (16 flop/byte)"}
    out["omega_rel_diff"] = max(abs(res[k]["Omega"] - res["cold"]["Omega"]) for k in ("warm", "warm_mixed_fire")) / abs(res["cold"]["Omega"])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fire", action="store_true", help="skip the time-to-residual legs")
    ap.add_argument("--fire-legs", default="newton,mixed_newton,mixed_fire,plain_fp64",
                    help="time-to-residual legs to run (a subset reports no speed-ups)")
    ap.add_argument("--no-ddft", action="store_true", help="skip the 256^3 DDFT leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the state-point sweep leg")
    ap.add_argument("--sweep-points", type=int, default=64, help="state points in the sweep leg")
    ap.add_argument("--no-fno", action="store_true", help="skip the neural-operator warm-start leg")
    ap.add_argument("--fno-train", type=int, default=120, help="converged 128^3 droplets the operator trains on")
    ap.add_argument("--no-spectral", action="store_true", help="skip the Log_Det / Eigenvalues leg")
    ap.add_argument("--sweep-grids", default="48,64,80,96,112,128,144,160",
                    help="grid sizes the sweep draws from (the full range is 48,64,...,160)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import classicaldft_gb300 as cd

    rho = droplet()
    c = cd.Context(SHAPE, DX, cd.WHITEBEAR_I, hsd=None, lj=True, kT=KT, precision=cd.FP64)
    c.set_chem_potential(c.bulk(RHO_V)["mu"])
    c.set_density(rho)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(K, W, fn):
        for _ in range(W):
            fn()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        total = 0.0
        for _ in range(K):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            total += a.elapsed_time(b)
        torch.cuda.synchronize()
        t = torch.tensor([total], device="cuda")
        if dist:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return t.item() / K  # ms per step, max over ranks

    # the headline: FP64 evaluations, the reference's own precision
    with Clocks(local) as clk:
        ms64 = timed(args.steps, max(3, args.warmup), lambda: c.eval(want_dF=False))
    clocks = clk.summary()
    passes64 = c.time_passes(reps=3)
    # e2e through the public API, FP64: the density from pinned host memory in, dF to pinned
    # host memory out, every step (cdft_set_density + cdft_eval with host pointers)
    host_rho = torch.from_numpy(rho.copy()).pin_memory()
    host_dF = torch.empty(rho.shape, dtype=torch.float64).pin_memory()
    K2 = max(5, args.steps // 2)
    for _ in range(3):
        c.set_density(host_rho)
        c.eval(dF_out=host_dF)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K2):
        c.set_density(host_rho)
        c.eval(dF_out=host_dF)
    e2e_s = (time.perf_counter() - t0) / K2
    # the FP32-bulk evaluation of the same system, and its error against FP64 on the same density
    t64, dF64 = c.eval()
    c.set_precision(cd.FP32)
    ms32 = timed(args.steps, max(3, args.warmup), lambda: c.eval(want_dF=False))
    passes32 = c.time_passes(reps=5)
    t32, dF32 = c.eval()
    c.set_precision(cd.FP64)
    fp32_err = {"omega_rel": abs(t32["Omega"] - t64["Omega"]) / abs(t64["Omega"]),
                "dF_max_abs_over_max_dF64": float(np.abs(dF32 - dF64).max() / np.abs(dF64).max()),
                "dF_max_abs_over_dV": float(np.abs(dF32 - dF64).max() / DX ** 3)}
    n_per_eval = 11  # kernels per evaluation: 9 passes, one finish of the sums, one finish of the residual norms
    peak, peak_kind = measured_peaks()
    fp64_peak = fma_peak(cd, "cdft_fp64_fma_rate")
    fp32_peak = fma_peak(cd, "cdft_fp32_fma_rate")
    N = int(np.prod(SHAPE))
    Nc = SHAPE[0] * SHAPE[1] * (SHAPE[2] // 2 + 1)
    M = 11
    B64 = 8 * (N * (4 * M + 3) + Nc * (2 * M + 11))
    B32 = 4 * (N * (4 * M + 3) + Nc * (2 * M + 11))
    top64 = max(passes64, key=lambda p: p["ms"])
    top32 = max(passes32, key=lambda p: p["ms"])
    ops = NCU_FP64_FLOPS.get(top64["pass"])
    f32ops = NCU_FP32_FLOPS.get(top64["pass"])
    t64s = top64["ms"] * 1e-3
    hbm64 = top64["bytes"] / (top64["ms"] * 1e-3) / 1e9  # the pass's algorithmic bytes at FP64 width
    line = {"metric": METRIC, "value": world * 1e3 / ms64, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload(),
            "gpu_launches": n_per_eval * args.steps,
            "e2e": {"value": world / e2e_s, "unit": "evals/s", "h2d_bytes_per_step": int(N * 8),
                    "d2h_bytes_per_step": int(N * 8 + 8 * 8)},
            "roofline": {"bound": "fp32", "kernel": top64["pass"] + " (FP64 evaluation, double-float arithmetic on the FP32 pipe)",
                         "achieved": (f32ops / t64s / 1e12) if f32ops else None, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": (f32ops / t64s / 1e12 / fp32_peak) if (f32ops and fp32_peak) else None,
                         "flops_per_launch": f32ops,
                         "flops_source": "executed FP32 add/mul/fma (fma = 2) per launch, ncu",
                         "peak_source": "measured in this run: cdft_fp32_fma_rate (independent FMA chains on every SM)",
                         "fma_pipe_busy": NCU_FMA_PIPE_BUSY.get(top64["pass"]),
                         "issue_active": NCU_ISSUE_ACTIVE.get(top64["pass"]),
                         "traffic": NCU_TRAFFIC.get((top64["pass"], "fp64")),
                         "hbm": {"achieved_gbs": hbm64, "peak_gbs": peak, "frac": hbm64 / peak, "peak_source": peak_kind},
                         "fp64_equivalent": {"flops_per_launch": ops, "achieved_tflops": (ops / t64s / 1e12) if ops else None,
                                             "fp64_fma_peak_tflops": fp64_peak,
                                             "ratio": (ops / t64s / 1e12 / fp64_peak) if (ops and fp64_peak) else None,
                                             "fp64_executed_per_launch": NCU_FP64_EXECUTED.get(top64["pass"]),
                                             "note": "the work of the all-FP64 form of the pass over this pass's time, against the "
                                                     "FP64 unit's measured rate: the margin the double-float arithmetic buys"}},
            "eval_roofline": {"algorithmic_bytes_per_eval": B64, "achieved_gbs": B64 / (ms64 * 1e-3) / 1e9,
                              "frac": B64 / (ms64 * 1e-3) / 1e9 / peak},
            "passes_fp64": [{"pass": p["pass"], "ms": round(p["ms"], 4)} for p in passes64],
            "fp32": {"evals_per_s": world * 1e3 / ms32, "ms_per_step": ms32, "dtype": "f32 transforms, f64 reductions",
                     "error_vs_fp64_same_density": fp32_err,
                     "roofline": {"bound": "hbm", "kernel": top32["pass"],
                                  "achieved": top32["bytes"] / (top32["ms"] * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                                  "frac": top32["bytes"] / (top32["ms"] * 1e-3) / 1e9 / peak, "peak_source": peak_kind,
                                  "traffic": NCU_TRAFFIC.get((top32["pass"], "fp32"))},
                     "eval_roofline": {"algorithmic_bytes_per_eval": B32, "achieved_gbs": B32 / (ms32 * 1e-3) / 1e9,
                                       "frac": B32 / (ms32 * 1e-3) / 1e9 / peak},
                     "passes": [{"pass": p["pass"], "ms": round(p["ms"], 5),
                                 "GBs": round(p["bytes"] / max(p["ms"], 1e-9) / 1e6, 1)} for p in passes32]},
            "clocks": clocks}
    if not args.no_batch:  # sharded over the ranks when there are several
        sweep = batch_leg(cd, n=args.sweep_points, grids=tuple(int(g) for g in args.sweep_grids.split(",")),
                          rank=rank, world=world, dist=dist)
        if rank == 0:
            line["statepoint_sweep"] = sweep
    # the single-GPU legs below are reported by rank 0 only (the other replicas skip them)
    kept = {}
    if rank == 0 and not args.no_fire:
        line["fire_to_resid_1e-8"] = fire_legs(cd, rho, legs=tuple(args.fire_legs.split(",")), keep=kept)
    if rank == 0 and not args.no_ddft:
        line["eval_256"] = eval_256_leg(cd)
        line["ddft_256"] = ddft_leg(cd)
    if rank == 0 and not args.no_spectral:
        line["spectral_128"] = spectral_leg(cd, rho)
    if rank == 0 and not args.no_fno:
        fr = line.get("fire_to_resid_1e-8", {})
        plain = fr.get("plain_fp64", {}).get("seconds") if isinstance(fr, dict) else None
        line["warm_start"] = warm_start_leg(cd, n_train=args.fno_train, plain_fp64_s=plain)
    if rank == 0 and not args.no_cpu_baseline:
        rate, n, el = cpu_baseline()
        line["cpu_baseline"] = {"value": rate, "unit": "evals/s", "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                                "sample": "%d FP64 F+dF evaluations of the same 128^3 system by the oracle in %.1f s" % (n, el)}
        fr = line.get("fire_to_resid_1e-8")
        if fr and kept:  # the converged droplets checked by the oracle (FP64, CPU)
            fr["oracle_pins"] = oracle_pins(kept)
        if fr and "plain_fp64" in fr:  # the CPU time to resid 1e-8, extrapolated: one FP64 evaluation per FIRE2 step
            steps = fr["plain_fp64"]["fire_steps"]
            fr["cpu_oracle_plain_fp64_extrapolated_s"] = steps / rate
            fr["cpu_note"] = ("%d FIRE2 steps of the GPU's plain FP64 run x the oracle's seconds per FP64 evaluation "
                              "(the BLAS-1 work of a step left out), labelled extrapolated" % steps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
