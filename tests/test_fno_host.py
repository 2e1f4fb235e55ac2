"""Host-side pieces of the neural-operator warm start (no GPU): the coarse seed,
its spectral upsampling and the training-point sampler."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_upsample_is_exact_for_band_limited_fields():
    from classicaldft_gb300 import fno
    n, N = 16, 64
    x = np.arange(n) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    f = 1.0 + 0.3 * np.cos(2 * np.pi * 2 * X) * np.sin(2 * np.pi * 3 * Y) + 0.1 * np.cos(2 * np.pi * Z)
    up = fno.upsample(f, (N, N, N)).numpy()
    xf = np.arange(N) / N
    Xf, Yf, Zf = np.meshgrid(xf, xf, xf, indexing="ij")
    ref = 1.0 + 0.3 * np.cos(2 * np.pi * 2 * Xf) * np.sin(2 * np.pi * 3 * Yf) + 0.1 * np.cos(2 * np.pi * Zf)
    assert np.max(np.abs(up - ref)) < 1e-12


def test_seed_and_features():
    from classicaldft_gb300 import fno
    seed = fno.coarse_seed((128, 128, 128), 0.1, 0.01, 0.75, 4.0)
    assert seed.shape == (32, 32, 32) and seed.min() > 0.009 and seed.max() < 0.751
    f, up = fno.features(seed, 0.8, (64, 64, 64), "cpu")
    assert f.shape == (64 ** 3, fno.K_IN) and torch.all(up > 0)
    assert torch.allclose(f[:, 1], torch.full((64 ** 3,), 0.8))


def test_droplet_sampler_is_seeded():
    from classicaldft_gb300 import fno
    a = fno.sample_droplets(8, 3)
    assert a == fno.sample_droplets(8, 3) and a != fno.sample_droplets(8, 4)
    for p in a:
        assert 0.75 <= p["kT"] <= 0.9 and 3.0 <= p["R"] <= 5.0 and p["rho_v"] < p["rho_l"]


def test_spectral_conv_equals_fft_formulation():
    """The truncated-DFT Fourier layer equals irfftn(mix(rfftn(v))) with only the kept modes."""
    from classicaldft_gb300 import fno
    torch.manual_seed(3)
    shape, C, m = (12, 10, 16), 4, 3
    layer = fno.SpectralConv3d(C, m)
    with torch.no_grad():
        layer.w.mul_(50.0)
    v = torch.randn(int(np.prod(shape)), C)
    y = layer(v, shape)
    n0, n1, n2 = shape
    X = torch.fft.rfftn(v.t().reshape(1, C, n0, n1, n2), dim=(2, 3, 4))
    out = torch.zeros_like(X)
    W = torch.view_as_complex(layer.w.detach())
    for q, (sx, sy) in enumerate(((slice(0, m), slice(0, m)), (slice(n0 - m, n0), slice(0, m)),
                                  (slice(0, m), slice(n1 - m, n1)), (slice(n0 - m, n0), slice(n1 - m, n1)))):
        out[:, :, sx, sy, :m] = torch.einsum("bixyz,ioxyz->boxyz", X[:, :, sx, sy, :m], W[q])
    ref = torch.fft.irfftn(out, s=shape, dim=(2, 3, 4)).reshape(C, -1).t()
    assert torch.max(torch.abs(y.detach() - ref)) <= 1e-5 * torch.max(torch.abs(ref))
    # gradients flow to the input and to the weights
    v.requires_grad_(True)
    layer(v, shape).square().sum().backward()
    assert v.grad is not None and layer.w.grad is not None and torch.isfinite(layer.w.grad).all()
