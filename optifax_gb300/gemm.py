"""BF16 tensor-core GEMM (optifax_gemm_bf16): C[M, N] (+)= A[M, K] . B[N, K]^T."""
from __future__ import annotations

import ctypes
from typing import Optional

import torch

from . import _native as nat


def gemm_bf16(A: torch.Tensor, B: torch.Tensor, C: Optional[torch.Tensor] = None, *, M: Optional[int] = None,
              N: Optional[int] = None, splits: int = 1, accumulate: bool = False, stream=None) -> torch.Tensor:
    """A: (a_rows >= max(M, 128), K) bf16; B: (b_rows >= max(N, 64), K) bf16; rows
    past M (N) are read but not used.  Returns C (M, N) float32."""
    if A.dtype != torch.bfloat16 or B.dtype != torch.bfloat16 or not A.is_cuda or not B.is_cuda:
        raise TypeError("A and B must be CUDA bfloat16")
    if A.dim() != 2 or B.dim() != 2 or A.stride(1) != 1 or B.stride(1) != 1 or A.shape[1] != B.shape[1]:
        raise ValueError("A and B must be row-major 2-D with the same K")
    M = A.shape[0] if M is None else M
    N = B.shape[0] if N is None else N
    K = A.shape[1]
    if C is None:
        C = torch.zeros((M, N), dtype=torch.float32, device=A.device) if accumulate else \
            torch.empty((M, N), dtype=torch.float32, device=A.device)
    if stream is None:
        stream = torch.cuda.current_stream(A.device)
    lib = nat.load()
    rc = lib.optifax_gemm_bf16(A.data_ptr(), A.stride(0), A.shape[0], B.data_ptr(), B.stride(0), B.shape[0],
                               C.data_ptr(), C.stride(0), M, N, K, int(splits), int(accumulate),
                               int(stream.cuda_stream))
    nat.check(rc, None, "optifax_gemm_bf16")
    return C


def tc_error(clear: bool = True) -> int:
    v = ctypes.c_int32(0)
    nat.check(nat.load().optifax_tc_error(ctypes.byref(v), int(clear)), None, "optifax_tc_error")
    return int(v.value)
