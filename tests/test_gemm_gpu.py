"""tcgen05/TMA BF16 GEMM against a plain PyTorch FP32 matmul of the same BF16 values."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ref(A, B, M, N):
    return A[:M].float() @ B[:N].float().T


@pytest.mark.parametrize("M,N,K,splits,arows,brows", [
    (128, 64, 64, 1, 128, 64),
    (256, 64, 128, 1, 256, 64),
    (389, 200, 4096, 8, 512, 256),
    (64, 64, 8192, 16, 128, 64),
    (1000, 130, 200, 1, 1024, 192),
    (2048, 4096, 64, 1, 2048, 4096),
])
def test_gemm_matches_fp32(M, N, K, splits, arows, brows):
    from optifax_gb300.gemm import gemm_bf16, tc_error
    g = torch.Generator().manual_seed(M + N + K)
    A = torch.randn(arows, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(brows, K, generator=g).to(torch.bfloat16).cuda()
    C = gemm_bf16(A, B, M=M, N=N, splits=splits)
    torch.cuda.synchronize()
    assert tc_error() == 0
    R = _ref(A, B, M, N)
    err = (C - R).abs().max().item() / R.abs().max().item()
    assert err < 1e-5, err


def test_gemm_accumulate_and_strided():
    from optifax_gb300.gemm import gemm_bf16, tc_error
    g = torch.Generator().manual_seed(7)
    big = torch.randn(256, 192, generator=g).to(torch.bfloat16).cuda()
    A = big[:, :128]                       # leading dimension 192, K = 128
    B = torch.randn(64, 128, generator=g).to(torch.bfloat16).cuda()
    C0 = torch.randn(256, 64, generator=g).cuda()
    C = C0.clone()
    gemm_bf16(A, B, C, accumulate=True)
    torch.cuda.synchronize()
    assert tc_error() == 0
    R = C0 + A.float() @ B.float().T
    assert (C - R).abs().max().item() < 1e-3
