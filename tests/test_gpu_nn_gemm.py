"""tcgen05 BF16 GEMM (the learned warm start's convolution engine) against an FP32 reference of
the same bf16 operands. Tolerance: FP32 accumulation of bf16 products, |err| <= 1e-5 * K * max|a||b|
(accumulation order differs); bf16 outputs within one bf16 ulp of the rounded reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref(A, B):
    return A.float().cpu() @ B.float().cpu().T


# the last three have more tiles than a GB300 has SMs: each persistent CTA runs two or three tiles
# through both TMEM accumulators
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 128, 128), (300, 77, 200), (1000, 3, 32), (128, 256, 512),
                                   (4096, 64, 288), (77, 130, 8), (8269, 1300, 200), (40000, 96, 72),
                                   (2048, 2560, 1000)])
def test_gemm_fp32_out(ps, M, N, K):
    import torch

    from ps_gb300 import nn

    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    nn.gemm_bf16(A, B, C)
    ref = _ref(A, B)
    err = (C.cpu() - ref).abs().max().item()
    assert err <= 1e-5 * K * 16, (M, N, K, err)


def test_gemm_bias_relu_bf16(ps):
    import torch

    from ps_gb300 import nn

    M, N, K = 9000, 520, 576  # 213 tiles of 128 x 256: more than one per SM
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = (0.05 * torch.randn(N, K, device="cuda", generator=g)).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    C = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    nn.gemm_bf16(A, B, C, bias=bias, flags=nn.RELU | nn.OUT_BF16)
    ref = torch.relu(_ref(A, B) + bias.cpu())
    got = C.float().cpu()
    # one bf16 rounding of the output (relative 2^-8) plus FP32 accumulation-order differences
    assert torch.all((got - ref).abs() <= ref.abs() * 2.0 ** -8 + 1e-3), (got - ref).abs().max()
    assert (got == 0).any() and (got > 0).any()


@pytest.mark.parametrize("split,M,N,K", [(1, 64, 288, 8192), (3, 64, 288, 8192), (8, 64, 288, 8192),
                                         (2, 4096, 1024, 1024)])
def test_gemm_split_k_accumulate(ps, split, M, N, K):
    """The weight-gradient shape (few output tiles, long K) and a split over 256 tiles."""
    import torch

    from ps_gb300 import nn

    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.ones(M, N, device="cuda")
    nn.gemm_bf16(A, B, C, flags=nn.ACCUMULATE, split=split)
    ref = _ref(A, B) + 1.0
    err = (C.cpu() - ref).abs().max().item()
    assert err <= 1e-5 * K * 16, err
