"""The tcgen05 BF16 GEMM building block against an fp32 product of the same
bf16 operands (bf16 x bf16 products are exact in fp32, so only the
accumulation order differs)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch

    from partapp_gb300 import build
    import partapp_gb300 as pa

    build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = pa.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 320), (200, 130, 104),
                                   (1024, 512, 1024)])
def test_gemm_bf16_matches_fp32_reference(ctx, M, N, K):
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(M * 7 + N * 3 + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)
    C = ctx.gemm_bf16(A, B)
    ref = A.float() @ B.float().T
    err = (C - ref).abs().max().item()
    scale = ref.abs().max().item()
    assert err <= 1e-5 * scale * max(1.0, K / 64), (err, scale)


def test_gemm_bf16_strided_operands(ctx):
    """Row strides larger than K (a view into a wider buffer): the columns
    past K must not enter the product."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    Aw = torch.randn((256, 200), generator=g, device="cuda").to(torch.bfloat16)
    Bw = torch.randn((128, 200), generator=g, device="cuda").to(torch.bfloat16)
    A, B = Aw[:, :136], Bw[:, :136]
    C = ctx.gemm_bf16(A, B)
    ref = A.float() @ B.float().T
    assert (C - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()


@pytest.mark.parametrize("M,N,K,band", [(1024, 3072, 1024, 72), (384, 520, 296, 20),
                                        (128, 256, 128, 0)])
def test_banded_gemm_matches_dense_product(ctx, M, N, K, band):
    """A banded A (zero outside |k - m| <= band), the persistent band kernel:
    equals the dense product."""
    import torch

    import partapp_gb300 as pa

    g = torch.Generator(device="cuda")
    g.manual_seed(M + N + K + band)
    A = torch.randn((M, K), generator=g, device="cuda")
    i = torch.arange(M, device="cuda")[:, None]
    k = torch.arange(K, device="cuda")[None, :]
    A = torch.where((k - i).abs() <= band, A, torch.zeros_like(A)).to(torch.bfloat16)
    B = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)
    C = ctx.gemm_bf16_banded(A, B, band)
    ref = A.float() @ B.float().T
    assert (C - ref).abs().max().item() <= 1e-5 * max(1.0, ref.abs().max().item()) * 4
