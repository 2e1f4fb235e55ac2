"""The neural operator's gradients on the GPU (BF16 tcgen05 GEMMs for the pointwise layers,
the truncated-DFT Fourier layers) against an FP64 CPU restatement of the same network.

The CPU network is written independently here: plain float64 matrix products for the
pointwise layers and the Fourier layers as irfftn(mix(rfftn(v))) with only the kept modes.
Both take the same weights and the same input; the loss and the gradient of every
parameter must agree to the precision of BF16 operands (2^-9 relative rounding of every
GEMM operand, FP32 accumulation). Forward, that is 1e-2 on the loss; backward, the
rounding of activations and gradients compounds through the six GEMM layers of the chain
(the lift weights, deepest in it, come out ~4% off in norm), so each gradient must lie
within 6e-2 of the FP64 gradient's norm and point the same way (cosine >= 0.998). A bias
gradient is a sum over all points of terms of both signs, whose cancellation makes its norm
a poor yardstick: each entry must lie within 3e-2 of the size of its terms (the sum of their
magnitudes, from the FP64 network)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _gelu64(z):
    return 0.5 * z * (1.0 + torch.erf(z / math.sqrt(2.0)))


def _spectral64(v, W, shape, m):
    """irfftn(mix(rfftn(v))) on the kept modes: the four (kx, ky) corners, kz < m."""
    n0, n1, n2 = shape
    C = v.shape[1]
    X = torch.fft.rfftn(v.t().reshape(C, n0, n1, n2), dim=(1, 2, 3))
    out = torch.zeros_like(X)
    for q, (sx, sy) in enumerate(((slice(0, m), slice(0, m)), (slice(n0 - m, n0), slice(0, m)),
                                  (slice(0, m), slice(n1 - m, n1)), (slice(n0 - m, n0), slice(n1 - m, n1)))):
        out[:, sx, sy, :m] = torch.einsum("ixyz,ioxyz->oxyz", X[:, sx, sy, :m], W[q])
    return torch.fft.irfftn(out, s=shape, dim=(1, 2, 3)).reshape(C, -1).t()


def _forward64(p, feats, shape, m, pre=None):
    """The network in FP64; pre (a dict) receives each bias's layer output (points x
    channels, gradients retained), whose column sums are the bias gradients."""
    def keep(name, z):
        if pre is not None:
            z.retain_grad()
            pre[name] = z
        return z
    v = keep("lift_b", feats @ p["lift_w"] + p["lift_b"])
    for k in range(len(p["ws"])):
        W = torch.view_as_complex(p["spec"][k])
        v = _gelu64(keep("bs%d" % k, v @ p["ws"][k] + p["bs"][k] + _spectral64(v, W, shape, m)))
    h = _gelu64(keep("p1_b", v @ p["p1_w"] + p["p1_b"]))
    return (h @ p["p2_w"] + p["p2_b"])[:, 0]


def test_fno_gradients_match_fp64_cpu_network():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from classicaldft_gb300 import fno
    shape = (16, 16, 16)
    m = 4
    model = fno.FNO3d(modes=m).cuda()
    g = torch.Generator().manual_seed(9)
    with torch.no_grad():  # a trained-looking state: no zero output layer
        model.p2_w.copy_(torch.randn(model.p2_w.shape, generator=g) * 0.2)
        for s in model.spec:
            s.w.mul_(20.0)
    seed = fno.coarse_seed((64, 64, 64), 0.1, 0.02, 0.7, 2.0)
    feats, up = fno.features(seed, 0.8, shape, "cuda")
    feats = feats + 0.1 * torch.randn(feats.shape, generator=g).cuda()  # every input channel live
    target = 0.3 * torch.randn(int(np.prod(shape)), generator=g).cuda()
    out = model(feats, shape)
    loss = torch.mean((out - target) ** 2)
    model.zero_grad()
    loss.backward()
    fno.check_status()
    # the same network in FP64 on the CPU, from the same weights and input
    p = {"lift_w": model.lift_w, "lift_b": model.lift_b, "p1_w": model.p1_w, "p1_b": model.p1_b, "p2_w": model.p2_w,
         "p2_b": model.p2_b}
    p = {k: v.detach().double().cpu().requires_grad_(True) for k, v in p.items()}
    p["ws"] = [w.detach().double().cpu().requires_grad_(True) for w in model.ws]
    p["bs"] = [b.detach().double().cpu().requires_grad_(True) for b in model.bs]
    p["spec"] = [s.w.detach().double().cpu().requires_grad_(True) for s in model.spec]
    pre = {}
    out64 = _forward64(p, feats.double().cpu(), shape, m, pre)
    loss64 = torch.mean((out64 - target.double().cpu()) ** 2)
    loss64.backward()
    # a bias gradient is a sum over all points of terms of both signs; its error is judged
    # per channel against the size of those terms (the sum of their magnitudes)
    terms = {name: torch.sum(torch.abs(z.grad), dim=0) for name, z in pre.items()}
    bias_name = {id(model.lift_b): "lift_b", id(model.p1_b): "p1_b"}
    bias_name.update({id(b): "bs%d" % k for k, b in enumerate(model.bs)})
    assert abs(float(loss.detach()) - float(loss64.detach())) <= 1e-2 * float(loss64.detach())
    pairs = [(model.lift_w, p["lift_w"]), (model.lift_b, p["lift_b"]), (model.p1_w, p["p1_w"]), (model.p1_b, p["p1_b"]),
             (model.p2_w, p["p2_w"]), (model.p2_b, p["p2_b"])]
    pairs += list(zip(model.ws, p["ws"])) + list(zip(model.bs, p["bs"])) + [(s.w, w) for s, w in zip(model.spec, p["spec"])]
    for gpu, cpu in pairs:
        a = gpu.grad.double().cpu()
        b = cpu.grad
        if gpu is model.p2_b:
            # one live entry, 2 mean(out - target): a sum of terms of both signs, so its
            # error is judged against the size of the terms, 2 mean|out - target|
            scale = 2 * float(torch.mean(torch.abs(out64 - target.double().cpu())))
            assert abs(float(a[0] - b[0])) <= 2e-2 * scale and float(torch.abs(a[1:]).max()) == 0.0
            continue
        if id(gpu) in bias_name:
            name = bias_name[id(gpu)]
            t = terms[name]
            assert torch.allclose(pre[name].grad.sum(dim=0), b)  # the terms are this bias's
            worst = float(torch.max(torch.abs(a - b) / torch.clamp(t, min=1e-300)))
            assert worst <= 3e-2, (name, worst)
            continue
        rel = float(torch.linalg.norm(a - b) / max(float(torch.linalg.norm(b)), 1e-300))
        cos = float(torch.sum(a * b) / max(float(torch.linalg.norm(a) * torch.linalg.norm(b)), 1e-300))
        assert rel <= 6e-2 and cos >= 0.998, (tuple(gpu.shape), rel, cos)
