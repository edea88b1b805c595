"""Learned warm start for the Stokes2D PT solver: a BF16 conv encoder-decoder whose convolutions
run as tcgen05 tensor-core GEMMs in libps_b200.so (no counterpart in the reference).

``gemm_bf16`` exposes the GEMM on its own (C = A B^T, bf16 operands, FP32 accumulation)."""
from __future__ import annotations

import ctypes

from . import _lib

RELU, OUT_BF16, ACCUMULATE = 1, 2, 4

_lib.register("ps_nn_gemm_bf16", [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p])


def gemm_bf16(A, B, C, bias=None, flags=0, split=1, stream=None):
    """C[M][N] (FP32, or bf16 with OUT_BF16) = A[M][K] @ B[N][K]^T (+ bias, ReLU) on the tensor cores.
    A, B, C, bias: contiguous CUDA tensors (torch)."""
    from .core import stream_handle

    M, K = A.shape
    N = B.shape[0]
    if B.shape[1] != K:
        raise ValueError("A and B must have the same K")
    _lib.call("ps_nn_gemm_bf16", ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
              ctypes.c_void_p(C.data_ptr()), M, N, K, ctypes.c_void_p(bias.data_ptr() if bias is not None else 0),
              int(flags), int(split), stream_handle(stream))
