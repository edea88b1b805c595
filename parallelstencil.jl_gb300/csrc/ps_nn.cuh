// ps_nn.cuh -- internal interface of the learned warm start's kernels (tcgen05 GEMM and the
// convolution / training kernels around it).
#pragma once
#include <cuda_bf16.h>

#include "ps_common.cuh"

namespace ps {

// What the GEMM does with each FP32 accumulator value x = alpha * (A B^T)[m][n]:
// x += bias[n] (if bias), x = max(x, 0) (if relu), then out[m*ldc + n] = x as bf16 (out_bf16),
// out[...] += x with an FP32 atomic (atomic; required for split-K), or out[...] = x.
struct GemmEpilogue {
    const float* bias;
    int relu, out_bf16, atomic;
    float alpha;
    float* outf;
    __nv_bfloat16* outh;
    int64_t ldc, M, N;
};

// D = A[M][K] * B[N][K]^T (bf16, row-major, K % 8 == 0), split-K over `split` CTAs per tile.
int nn_gemm(const void* A, int64_t M, const void* B, int64_t N, int64_t K, const GemmEpilogue& e, int split,
            cudaStream_t s, int* d_err);

}  // namespace ps
