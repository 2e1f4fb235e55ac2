"""BF16 tcgen05 GEMM (cdft_tc_gemm_bf16) against a plain PyTorch FP32 product of
the same BF16 inputs: FP32 accumulation, so agreement to ~1e-6 relative."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fno():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from classicaldft_gb300 import fno as m
    return m


@pytest.mark.parametrize("M,K,N,act", [(256, 32, 32, 0), (1000, 16, 32, 1), (1000, 32, 64, 1), (777, 64, 128, 1), (129, 48, 32, 0),
                                       (300000, 32, 32, 1)])
def test_tc_gemm_matches_fp32_product(fno, M, K, N, act):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M + K + N)
    x = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    w = (torch.randn(K, N, device="cuda", generator=g) / K ** 0.5).to(torch.bfloat16)
    b = torch.randn(N, device="cuda", generator=g)
    a = torch.randn(M, N, device="cuda", generator=g)
    y, z = fno.tc_gemm(x, w, b, a, act=act, want_z=True)
    torch.cuda.synchronize()
    fno.check_status()
    ref = x.float() @ w.float() + b + a
    assert (z - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
    out = torch.nn.functional.gelu(ref) if act else ref
    assert (y - out).abs().max().item() <= 1e-5 * out.abs().max().item()


def test_tc_linear_gradients(fno):
    """Backward of the tensor-core layer (activation gradient on the tensor cores) vs autograd of the FP32 reference."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(4096, 32, device="cuda", generator=g).to(torch.bfloat16).float().requires_grad_(True)
    w = (torch.randn(32, 32, device="cuda", generator=g) / 32 ** 0.5).to(torch.bfloat16).float().requires_grad_(True)
    b = torch.randn(32, device="cuda", generator=g).requires_grad_(True)
    y = fno.tc_linear(x, w, b, act=1)
    gy = torch.randn_like(y)
    (y * gy).sum().backward()
    x2 = x.detach().clone().requires_grad_(True)
    w2 = w.detach().clone().requires_grad_(True)
    b2 = b.detach().clone().requires_grad_(True)
    y2 = torch.nn.functional.gelu(x2 @ w2 + b2)
    (y2 * gy).sum().backward()
    assert (y - y2).abs().max().item() <= 1e-5 * y2.abs().max().item()
    # the activation gradient passes through BF16 once on the tensor cores
    assert (x.grad - x2.grad).abs().max().item() <= 1e-2 * x2.grad.abs().max().item()
    assert (w.grad - w2.grad).abs().max().item() <= 1e-4 * w2.grad.abs().max().item()
    assert (b.grad - b2.grad).abs().max().item() <= 1e-4 * b2.grad.abs().max().item()
