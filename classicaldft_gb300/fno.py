"""Fourier neural operator warm start for the density solver.

A learned map from the solver's cheap initial guess (the tanh droplet profile,
carried on a coarse 32^3 grid, and the temperature) to the converged 128^3
density, used as the starting point of the Newton-Krylov solve. No
counterpart in the reference.

Layout (channels-last, one row per lattice point, so every pointwise layer is a
GEMM over the N = 128^3 rows):
  lift      [seed, kT, 1, 0 ...] (16 channels) -> width 32      tensor-core GEMM
  4 blocks  v <- GELU(v W + b + SpectralConv(v))                 tensor-core GEMM + truncated DFTs
  project   32 -> 32 (GELU) -> 32 (column 0 used)                tensor-core GEMMs
  output    log rho = log seed_up + out  (positive by construction)
The pointwise GEMMs run on the BF16 tcgen05 kernel (cdft_tc_gemm_bf16, FP32
accumulation in tensor memory) forward and, for the activations' gradient,
backward; the spectral convolutions (12 modes per axis, as truncated DFTs in
library GEMMs) and the weight gradients are plain library operations.
"""
import ctypes
import math

import numpy as np
import torch

from . import lib

WIDTH = 32
MODES = 12
LAYERS = 4
K_IN = 16


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


_STATUS = {}


def _status(dev):
    if dev not in _STATUS:
        _STATUS[dev] = torch.zeros(1, dtype=torch.int32, device=dev)
    return _STATUS[dev]


def tc_gemm(x, w, bias=None, add=None, act=0, want_z=False):
    """Y = act(x . w + bias + add) on the tensor cores. x: (M, K) BF16, w: (K, N) BF16."""
    x = x.contiguous()
    w = w.contiguous()
    M, K = x.shape
    N = w.shape[1]
    y = torch.empty(M, N, device=x.device, dtype=torch.float32)
    z = torch.empty(M, N, device=x.device, dtype=torch.float32) if want_z else None
    st = _status(x.device)
    rc = lib().cdft_tc_gemm_bf16(_vp(x), _vp(w), _vp(bias), _vp(add.contiguous() if add is not None else None), _vp(y), _vp(z), M, K,
                                 N, act, _vp(st), ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream))
    if rc:
        raise RuntimeError("cdft_tc_gemm_bf16: bad shape or arguments (%d)" % rc)
    return y, z


def check_status():
    for st in _STATUS.values():
        if int(st.item()):
            raise RuntimeError("tensor-core GEMM: a device wait ran out (status %d)" % int(st.item()))


def _gelu_grad(z):
    cdf = 0.5 * (1.0 + torch.erf(z * (1.0 / math.sqrt(2.0))))
    pdf = torch.exp(-0.5 * z * z) * (1.0 / math.sqrt(2.0 * math.pi))
    return cdf + z * pdf


class _TCLinear(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, w, b, add, act):
        xb = x.to(torch.bfloat16)
        wb = w.to(torch.bfloat16)
        y, z = tc_gemm(xb, wb, b, add, act, want_z=bool(act))
        ctx.save_for_backward(xb, wb, z)
        ctx.act = act
        ctx.has_add = add is not None
        return y

    @staticmethod
    def backward(ctx, gy):
        xb, wb, z = ctx.saved_tensors
        g = gy * _gelu_grad(z) if ctx.act else gy
        gx = None
        if ctx.needs_input_grad[0]:
            gx, _ = tc_gemm(g.to(torch.bfloat16), wb.t().contiguous())  # (M, N) . (N, K) on the tensor cores
        gw = xb.float().t() @ g  # weight gradient: a plain (K x M) . (M x N) product
        gb = g.sum(0)
        return gx, gw, gb, (g if ctx.has_add else None), None


def tc_linear(x, w, b, add=None, act=0):
    return _TCLinear.apply(x, w, b, add, act)


_DFT_CACHE = {}


def _dft_mats(shape, m, device):
    """Truncated DFT matrices of a (n0, n1, n2) grid keeping kx, ky in [0, m) and [n - m, n)
    and kz in [0, m): forward Fz (2m x n2, real: cos rows then -sin rows), Fy (2m x n1) and
    Fx (2m x n0) complex; inverse Gx (n0 x 2m), Gy (n1 x 2m) complex and Gz (n2 x 2m, real),
    Gz carrying the half-spectrum weights (1 for kz = 0, 2 above) and the 1/N of the inverse."""
    key = (tuple(shape), m, str(device))
    if key not in _DFT_CACHE:
        n0, n1, n2 = shape

        def full(n):  # kept wave numbers along a full axis, and the phases
            k = np.concatenate([np.arange(m), np.arange(n - m, n)])
            return np.exp(-2j * np.pi * np.outer(k, np.arange(n)) / n)

        th = 2 * np.pi * np.outer(np.arange(m), np.arange(n2)) / n2  # (m, n2)
        Fz = np.concatenate([np.cos(th), -np.sin(th)], axis=0)
        w = np.where(np.arange(m) == 0, 1.0, 2.0)[:, None] / float(n0 * n1 * n2)
        Gz = np.concatenate([w * np.cos(th), -w * np.sin(th)], axis=0).T  # (n2, 2m)
        Fx, Fy = full(n0), full(n1)
        c = lambda a: torch.as_tensor(a, dtype=torch.complex64, device=device)
        r = lambda a: torch.as_tensor(a, dtype=torch.float32, device=device)
        _DFT_CACHE[key] = (r(Fz), c(Fy), c(Fx), c(Fx.conj().T), c(Fy.conj().T), r(Gz))
    return _DFT_CACHE[key]


class SpectralConv3d(torch.nn.Module):
    """Fourier layer: complex channel mixing on the 4 x MODES^3 lowest modes of the real 3D
    transform (the four (kx, ky) corners, kz < MODES), back to real space.

    Only the kept modes are ever formed: the transform is three truncated DFTs taken as GEMMs
    straight on the channels-last (N, C) activations (z, then y, then x; and back), so a layer
    reads and writes its activations once, with no full-grid FFT and no transposed copies.
    The result equals irfftn(mix(rfftn(v))) with every other mode zero."""

    def __init__(self, width, modes):
        super().__init__()
        scale = 1.0 / (width * width)
        self.m = modes
        self.w = torch.nn.Parameter(scale * torch.randn(4, width, width, modes, modes, modes, 2))

    def mixing(self):
        """The weights as (2m, 2m, m, C_in, C_out) complex, corners in the kept-mode order."""
        W = torch.view_as_complex(self.w).permute(0, 3, 4, 5, 1, 2)  # (4, x, y, z, i, o)
        top = torch.cat([W[0], W[2]], dim=1)  # kx < m: ky < m, then ky >= n - m
        bot = torch.cat([W[1], W[3]], dim=1)  # kx >= n - m
        return torch.cat([top, bot], dim=0)

    def forward(self, v, shape):  # v: (N, C) channels-last
        n0, n1, n2 = shape
        m = self.m
        C = v.shape[1]
        Fz, Fy, Fx, Gx, Gy, Gz = _dft_mats(shape, m, v.device)
        a = torch.matmul(Fz, v.reshape(n0 * n1, n2, C))                       # (n0 n1, 2m, C)
        xz = torch.complex(a[:, :m], a[:, m:]).reshape(n0, n1, m * C)          # z: kz < m
        xy = torch.matmul(Fy, xz)                                              # y: (n0, 2m, m C)
        xx = torch.matmul(Fx, xy.reshape(n0, 2 * m * m * C)).reshape(2 * m, 2 * m, m, 1, C)
        out = torch.matmul(xx, self.mixing()).reshape(2 * m, 2 * m * m * C)   # channel mixing per mode
        y1 = torch.matmul(Gx, out).reshape(n0, 2 * m, m * C)                   # x back: (n0, 2m, m C)
        y2 = torch.matmul(Gy, y1).reshape(n0 * n1, m, C)                       # y back: (n0, n1, m C)
        b = torch.cat([y2.real, y2.imag], dim=1)                               # (n0 n1, 2m, C)
        return torch.matmul(Gz, b).reshape(n0 * n1 * n2, C)                    # z back, real


class FNO3d(torch.nn.Module):
    def __init__(self, width=WIDTH, modes=MODES, layers=LAYERS):
        super().__init__()
        g = torch.Generator().manual_seed(1234)
        self.lift_w = torch.nn.Parameter(torch.randn(K_IN, width, generator=g) / math.sqrt(K_IN))
        self.lift_b = torch.nn.Parameter(torch.zeros(width))
        self.spec = torch.nn.ModuleList([SpectralConv3d(width, modes) for _ in range(layers)])
        self.ws = torch.nn.ParameterList([torch.nn.Parameter(torch.randn(width, width, generator=g) / math.sqrt(width)) for _ in range(layers)])
        self.bs = torch.nn.ParameterList([torch.nn.Parameter(torch.zeros(width)) for _ in range(layers)])
        self.p1_w = torch.nn.Parameter(torch.randn(width, width, generator=g) / math.sqrt(width))
        self.p1_b = torch.nn.Parameter(torch.zeros(width))
        self.p2_w = torch.nn.Parameter(torch.zeros(width, 32))  # only column 0 is used; zero init = identity warm start
        self.p2_b = torch.nn.Parameter(torch.zeros(32))

    def forward(self, feats, shape):
        """feats: (N, K_IN) features per lattice point; returns the log-density correction (N,)."""
        v = tc_linear(feats, self.lift_w, self.lift_b)
        for spec, w, b in zip(self.spec, self.ws, self.bs):
            v = tc_linear(v, w, b, add=spec(v, shape), act=1)
        h = tc_linear(v, self.p1_w, self.p1_b, act=1)
        out = tc_linear(h, self.p2_w, self.p2_b)
        return out[:, 0]


def upsample(coarse, shape, device="cpu"):
    """Spectral (zero-padded Fourier) interpolation of a periodic coarse field to `shape`."""
    c = torch.as_tensor(coarse, dtype=torch.float64, device=device)
    C = torch.fft.rfftn(c)
    n = c.shape
    F = torch.zeros(shape[0], shape[1], shape[2] // 2 + 1, dtype=C.dtype, device=C.device)
    hx, hy = n[0] // 2, n[1] // 2
    kz = min(C.shape[2], F.shape[2])
    F[:hx, :hy, :kz] = C[:hx, :hy, :kz]
    F[-hx:, :hy, :kz] = C[-hx:, :hy, :kz]
    F[:hx, -hy:, :kz] = C[:hx, -hy:, :kz]
    F[-hx:, -hy:, :kz] = C[-hx:, -hy:, :kz]
    scale = np.prod(shape) / np.prod(n)
    return torch.fft.irfftn(F * scale, s=shape)


def features(seed_coarse, kT, shape, device):
    """Per-point input features: [log seed (upsampled), kT, 1, 0, ...] as an (N, K_IN) FP32 tensor,
    and the upsampled seed itself."""
    # interpolate log(seed): smooth, and positive after exp whatever the interpolant's ringing
    up = torch.exp(upsample(np.log(seed_coarse), shape, device)).to(dtype=torch.float32)
    N = up.numel()
    f = torch.zeros(N, K_IN, device=device)
    f[:, 0] = torch.log(up).reshape(-1)
    f[:, 1] = kT
    f[:, 2] = 1.0
    return f, up


def coarse_seed(shape_fine, dx, rho_v, rho_l, R, width=0.5, factor=4):
    """The tanh droplet sampled on the coarse lattice (spacing factor*dx) the operator takes as its seed."""
    from .statepoints import droplet
    n = tuple(s // factor for s in shape_fine)
    return droplet(n, dx * factor, rho_v, rho_l, R, width)


def predict(model, seed_coarse, kT, shape, device="cuda", on_device=False):
    """Warm-start density for the fine grid: numpy FP64, or (on_device) a CUDA FP64
    tensor that Context.set_density takes without a host round trip."""
    with torch.no_grad():
        f, up = features(seed_coarse, kT, shape, device)
        out = model(f, shape)
        rho = (up.reshape(-1) * torch.exp(out)).reshape(shape).double()
    check_status()
    return rho if on_device else rho.cpu().numpy()


def train(model, samples, shape, steps=300, lr=3e-3, device="cuda", log=None):
    """samples: list of (seed_coarse, kT, rho_converged). Loss: mean squared error of log rho."""
    model.to(device)
    opt = torch.optim.Adam(model.parameters(), lr=lr)
    # per sample only the coarse seed and the FP32 target stay resident (N floats); the
    # (N, K_IN) features are rebuilt for each step, so thousands of samples fit on the device
    data = []
    for seed, kT, rho in samples:
        _, up = features(seed, kT, shape, device)
        target = torch.log(torch.as_tensor(rho, device=device, dtype=torch.float32).reshape(-1)) - torch.log(up.reshape(-1))
        data.append((seed, kT, target))
    g = torch.Generator().manual_seed(7)
    for it in range(steps):
        seed, kT, target = data[int(torch.randint(len(data), (1,), generator=g))]
        f, _ = features(seed, kT, shape, device)
        out = model(f, shape)
        loss = torch.mean((out - target) ** 2)
        opt.zero_grad()
        loss.backward()
        opt.step()
        if log is not None and (it % 50 == 0 or it == steps - 1):
            log.append((it, float(loss.detach())))
    check_status()
    return model


# ------------------------------------------------------------ training data ---
def sample_droplets(n, seed, kT=(0.75, 0.9), rho_v=(0.005, 0.04), rho_l=(0.6, 0.8), R=(3.0, 5.0)):
    """Seeded droplet parameters around the 128^3 benchmark droplet (kT 0.8, rho 0.01 / 0.75, R = 4)."""
    rng = np.random.default_rng(seed)
    return [{"kT": float(rng.uniform(*kT)), "rho_v": float(rng.uniform(*rho_v)), "rho_l": float(rng.uniform(*rho_l)),
             "R": float(rng.uniform(*R))} for _ in range(n)]


def solve_droplets(points, shape=(128, 128, 128), dx=0.1, tol=1e-8, chunk=8):
    """Converged fixed-mass droplets (Newton-Krylov, cdft_fire_run_batch with mixed = 3).
    Returns [(coarse seed, kT, converged rho)] for the points that converged."""
    from . import Context, WHITEBEAR_I, bh_diameter, fire_run_batch
    from .statepoints import droplet
    out = []
    for i0 in range(0, len(points), chunk):
        ctxs, seeds = [], []
        for p in points[i0:i0 + chunk]:
            rho = droplet(shape, dx, p["rho_v"], p["rho_l"], p["R"])
            c = Context(shape, dx, WHITEBEAR_I, hsd=bh_diameter(1.0, 1.0, 3.0, p["kT"]), lj=True, kT=p["kT"],
                        fixed_mass=float(rho.sum()) * dx ** 3)
            c.set_density(rho)
            c.fire_init(force_limit=0.0)
            ctxs.append(c)
            seeds.append((coarse_seed(shape, dx, p["rho_v"], p["rho_l"], p["R"]), p["kT"]))
        reps, status = fire_run_batch(ctxs, tol, max_steps=20000, mixed=3)
        for c, r, s, (seed, kT) in zip(ctxs, reps, status, seeds):
            if s == 0 and r["resid"] <= tol:
                out.append((seed, kT, c.get_density()))
            c.close()
    return out
