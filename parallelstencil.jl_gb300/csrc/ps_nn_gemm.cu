// ps_nn_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05) for the learned warm
// start's convolutions: D[M][N] = A[M][K] * B[N][K]^T, A and B bf16 row-major (K contiguous), FP32
// accumulation in tensor memory (TMEM).
//
// Persistent: one CTA of 192 threads per SM walks the 128 x BN output tiles of D (BN = 128, or 256
// when N > 128; K splits as further tiles), in bands of 16 m blocks for L2 reuse:
//   - warp 0 (one thread) streams 128 x 64 / BN x 64 tiles of A and B into a 6-stage (BN = 256: 4)
//     ring with TMA (cp.async.bulk.tensor.2d, 128-byte swizzle, zero fill past the matrix edges, so
//     M, N and K need no padding beyond K % 8 == 0), across tile boundaries, refilling a stage as
//     soon as its "empty" mbarrier says the MMAs that read it are done;
//   - warp 1 (one thread) waits for each stage's "full" mbarrier and issues tcgen05.mma
//     (kind::f16, M = 128, N = BN, K = 16) into one of two TMEM accumulators; tcgen05.commit
//     arrives on the stage's "empty" mbarrier when those MMAs have read it, and on the
//     accumulator's "full" mbarrier when the tile is done;
//   - warps 2-5 read the other accumulator with tcgen05.ld (warp w owns TMEM lanes / tile rows
//     32 (w % 4) .. + 31) and apply the epilogue -- + bias[n], ReLU, store as bf16 or FP32 (vector
//     stores where aligned), or add into FP32 output with atomics (split-K) -- while the next
//     tile's MMAs run, then release the accumulator.
// Every mbarrier wait is bounded: on a timeout the kernel raises DEV_ERR_TMA_TIMEOUT, drains
// the copies it issued, frees its TMEM columns and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "ps_common.cuh"
#include "ps_nn.cuh"

namespace ps {

constexpr int G_BM = 128, G_BK = 64;
constexpr int G_ABYTES = G_BM * G_BK * 2;  // 16 KB
// Tile N = 128 (6-stage ring) or 256 (4 stages; an MMA then reads A once for twice the work, which
// keeps the instruction off the shared-memory bandwidth limit a 128 x 128 x 16 MMA sits at).
template <int BN>
struct GCfg {
    static constexpr int S = BN == 256 ? 4 : 6;
    static constexpr int BBYTES = BN * G_BK * 2;
    static constexpr int STAGE = G_ABYTES + BBYTES;
    static constexpr int SMEM = S * STAGE + 1024 + 256;  // ring (1024-aligned) + barriers, TMEM slot, counters
    static constexpr uint32_t TMEM = BN;                 // FP32 accumulator: one column per n (two are allocated)
};

// tcgen05 instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// Shared-memory matrix descriptor of a K-major tile stored by TMA with 128-byte swizzle: rows of
// 128 bytes, 8-row (1024-byte) swizzle atoms; start address in 16-byte units.
__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}
__device__ __forceinline__ void tc_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_arrive1(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One output tile of the persistent schedule. Tiles go in bands of G_GROUP m blocks: within a
// band, m block fastest, then n block; then the next band; the K split outermost. The CTAs in
// flight then share a band of A (G_GROUP x 128 rows) and a few B blocks, which stay in L2
// (m-fastest over the whole of M re-read all of A from DRAM for every n block of a large problem).
constexpr int G_GROUP = 16;
struct GTile {
    int m0, n0, kb0, nkb;
};
__device__ __forceinline__ GTile gemm_tile(int t, int tiles_m, int tiles_n, int BN, int KB, int per) {
    GTile g;
    const int plane = tiles_m * tiles_n, zi = t / plane, r = t % plane;
    const int band = r / (G_GROUP * tiles_n), in_band = r % (G_GROUP * tiles_n);
    const int gm = min(G_GROUP, tiles_m - band * G_GROUP);  // m blocks in this band
    const int mi = band * G_GROUP + in_band % gm, ni = in_band / gm;
    g.m0 = mi * G_BM;
    g.n0 = ni * BN;
    g.kb0 = zi * per;
    g.nkb = min(KB, g.kb0 + per) - g.kb0;
    return g;
}

// Persistent, warp-specialised: one CTA per SM walks the tiles t = blockIdx.x, +gridDim.x, ...
// warp 0 (one thread) feeds the shared-memory ring across tile boundaries, warp 1 (one thread)
// issues the MMAs into one of two TMEM accumulators, and warps 2-5 drain the other accumulator
// (tcgen05.ld, epilogue, global stores) while the next tile's MMAs run.
template <int BN>
__global__ void __launch_bounds__(192, 1)
    nn_gemm_tc(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, int64_t K,
               int kb_per_split, int tiles_m, int tiles_n, int ntiles, GemmEpilogue e, int* __restrict__ err) {
    using C = GCfg<BN>;
    constexpr int G_S = C::S, G_STAGE = C::STAGE;
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + G_S * G_STAGE);
    uint64_t* empty = full + G_S;
    uint64_t* tfull = empty + G_S;  // [2] accumulator ready (MMA -> epilogue)
    uint64_t* tempty = tfull + 2;   // [2] accumulator drained (epilogue warps -> MMA)
    uint64_t* done = tempty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    int* counts = reinterpret_cast<int*>(tmem_slot + 1);  // [0] stages filled, [1] stages consumed
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int KB = (int)((K + G_BK - 1) / G_BK);
    const int per = kb_per_split;

    if (threadIdx.x == 0) {
        prefetch_tensormap(&mA);
        prefetch_tensormap(&mB);
        for (int s = 0; s < G_S; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], 4);  // one arrival per epilogue warp
        }
        mbar_init(done, 1);
        counts[0] = counts[1] = 0;
        fence_mbar_init();
    }
    if (warp == 0) tc_alloc(tmem_slot, 2 * C::TMEM);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 0) {  // TMA producer
        int it = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            const GTile g = gemm_tile(t, tiles_m, tiles_n, BN, KB, per);
            for (int i = 0; i < g.nkb; i++, it++) {
                const int s = it % G_S;
                // stage s was last read by the MMAs of ring step it - G_S: its empty barrier's (it/G_S - 1)th phase
                if (it >= G_S && !mbar_wait_bounded(&empty[s], ((it / G_S) - 1) & 1)) {
                    ok = false;
                    break;
                }
                unsigned char* st = smem + s * G_STAGE;
                mbar_arrive_expect_tx(&full[s], G_STAGE);
                tma_load_2d(st, &mA, &full[s], (g.kb0 + i) * G_BK, g.m0);
                tma_load_2d(st + G_ABYTES, &mB, &full[s], (g.kb0 + i) * G_BK, g.n0);
            }
        }
        counts[0] = it;
        if (!ok) atomicOr(err, DEV_ERR_TMA_TIMEOUT);
    } else if (threadIdx.x == 32) {  // MMA issuer
        constexpr uint32_t idesc = umma_idesc_bf16(G_BM, BN);
        int it = 0, j = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, j++) {
            const GTile g = gemm_tile(t, tiles_m, tiles_n, BN, KB, per);
            const int acc = j & 1, use = j >> 1;
            // the epilogue must have drained this accumulator's previous tile (its (use-1)th phase)
            if (use >= 1 && !mbar_wait_bounded(&tempty[acc], (use - 1) & 1)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(acc * BN);
            for (int i = 0; i < g.nkb; i++, it++) {
                const int s = it % G_S;
                if (!mbar_wait_bounded(&full[s], (it / G_S) & 1)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + s * G_STAGE);
                const uint64_t da = umma_desc_sw128(sa), db = umma_desc_sw128(sa + G_ABYTES);
#pragma unroll
                for (int k = 0; k < G_BK / 16; k++)  // K = 16 per MMA: +32 bytes along the swizzled row
                    tc_mma(d, da + 2 * k, db + 2 * k, idesc, (i > 0 || k > 0) ? 1u : 0u);
                tc_commit(&empty[s]);
            }
            if (!ok) break;
            tc_commit(&tfull[acc]);  // arrives when this tile's MMAs have completed
        }
        counts[1] = it;
        if (!ok) atomicOr(err, DEV_ERR_TMA_TIMEOUT);
        tc_commit(done);  // arrives when every MMA issued above has completed
    } else if (warp >= 2) {  // epilogue: warp w reads TMEM lanes (tile rows) 32 (w % 4) .. + 31
        const int q = warp & 3, row = q * 32 + lane;
        int j = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, j++) {
            const GTile g = gemm_tile(t, tiles_m, tiles_n, BN, KB, per);
            const int acc = j & 1, use = j >> 1;
            // warp-uniform: tcgen05.ld below is a warp-collective instruction
            if (!__all_sync(0xffffffffu, mbar_wait_bounded(&tfull[acc], use & 1))) {
                if (lane == 0) atomicOr(err, DEV_ERR_TMA_TIMEOUT);
                break;
            }
            tc_fence_after();
            const int64_t gm = (int64_t)g.m0 + row;
            const bool row_ok = gm < e.M && g.nkb > 0;
            const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN);
            for (int c = 0; c < BN; c += 16) {
                float v[16];
                tc_ld16(tl + (uint32_t)c, v);  // whole warp, no divergence
                if (!row_ok) continue;
                const int64_t gn0 = (int64_t)g.n0 + c;
#pragma unroll
                for (int jj = 0; jj < 16; jj++) {
                    float x = v[jj] * e.alpha;
                    if (e.bias && gn0 + jj < e.N) x += e.bias[gn0 + jj];
                    if (e.relu) x = fmaxf(x, 0.0f);
                    v[jj] = x;
                }
                const int64_t o = gm * e.ldc + gn0;
                if (gn0 + 16 <= e.N && !e.atomic) {  // 16 columns in range: vector stores where aligned
                    if (e.out_bf16) {
                        __nv_bfloat16* p = e.outh + o;
                        if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
                            uint4 w[2];
                            __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(w);
#pragma unroll
                            for (int jj = 0; jj < 8; jj++) h[jj] = __floats2bfloat162_rn(v[2 * jj], v[2 * jj + 1]);
                            reinterpret_cast<uint4*>(p)[0] = w[0];
                            reinterpret_cast<uint4*>(p)[1] = w[1];
                            continue;
                        }
                    } else {
                        float* p = e.outf + o;
                        if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
#pragma unroll
                            for (int jj = 0; jj < 4; jj++)
                                reinterpret_cast<float4*>(p)[jj] =
                                    make_float4(v[4 * jj], v[4 * jj + 1], v[4 * jj + 2], v[4 * jj + 3]);
                            continue;
                        }
                    }
                }
#pragma unroll
                for (int jj = 0; jj < 16; jj++) {
                    if (gn0 + jj >= e.N) break;
                    if (e.out_bf16)
                        e.outh[o + jj] = __float2bfloat16_rn(v[jj]);
                    else if (e.atomic)
                        atomicAdd(e.outf + o + jj, v[jj]);
                    else
                        e.outf[o + jj] = v[jj];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive1(&tempty[acc]);
        }
    }
    __syncwarp();
    if (!mbar_wait_bounded(done, 0) && threadIdx.x == 0) atomicOr(err, DEV_ERR_TMA_TIMEOUT);
    tc_fence_after();
    __syncthreads();  // counts[] visible
    if (threadIdx.x == 0 && counts[1] < counts[0])  // a wait gave up: drain the copies still in flight
        for (int j = counts[1]; j < counts[0]; j++) mbar_wait_bounded(&full[j % G_S], (j / G_S) & 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, 2 * C::TMEM);
}

template <int BN>
static int nn_gemm_bn(const void* A, int64_t M, const void* B, int64_t N, int64_t K, const GemmEpilogue& e,
                      int split, cudaStream_t s, int* d_err) {
    using C = GCfg<BN>;
    CUtensorMap mA, mB;
    PS_TRY(encode_bf16_rows_sw128(&mA, A, (uint64_t)K, (uint64_t)M, G_BK, G_BM));
    PS_TRY(encode_bf16_rows_sw128(&mB, B, (uint64_t)K, (uint64_t)N, G_BK, BN));
    static bool attr = false;
    if (!attr) {
        PS_CUDA_TRY(cudaFuncSetAttribute(nn_gemm_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
        attr = true;
    }
    const int KB = (int)((K + G_BK - 1) / G_BK);
    split = std::max(1, std::min(split, KB));
    if (split > 1 && (!e.atomic || e.out_bf16 || e.bias || e.relu))
        return fail(PS_ERR_ARG, "nn_gemm: split-K needs a plain FP32 atomic epilogue");
    const int per = (KB + split - 1) / split;
    const int64_t tiles_m = (M + G_BM - 1) / G_BM, tiles_n = (N + BN - 1) / BN, splits = (KB + per - 1) / per;
    const int64_t ntiles = tiles_m * tiles_n * splits;
    if (ntiles > 0x7FFFFFFF - 65536) return fail(PS_ERR_SHAPE, "nn_gemm: matrix too large");
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<int64_t>(ntiles, std::max(1, sms));  // one CTA per SM (shared memory)
    nn_gemm_tc<BN><<<grid, 192, C::SMEM, s>>>(mA, mB, K, per, (int)tiles_m, (int)tiles_n, (int)ntiles, e, d_err);
    PS_CUDA_TRY(cudaGetLastError());
    return PS_OK;
}

int nn_gemm(const void* A, int64_t M, const void* B, int64_t N, int64_t K, const GemmEpilogue& e, int split,
            cudaStream_t s, int* d_err) {
    if (M <= 0 || N <= 0 || K <= 0) return PS_OK;
    if (K % 8) return fail(PS_ERR_SHAPE, "nn_gemm: K = %lld must be a multiple of 8", (long long)K);
    return N > 128 ? nn_gemm_bn<256>(A, M, B, N, K, e, split, s, d_err)
                   : nn_gemm_bn<128>(A, M, B, N, K, e, split, s, d_err);
}

}  // namespace ps

using namespace ps;

extern "C" int ps_nn_gemm_bf16(const void* A, const void* B, void* C, int64_t M, int64_t N, int64_t K,
                               const float* bias, int32_t flags, int32_t split, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (!A || !B || !C) return fail(PS_ERR_NULL, "ps_nn_gemm_bf16: NULL matrix");
    GemmEpilogue e{};
    e.M = M;
    e.N = N;
    e.ldc = N;
    e.alpha = 1.0f;
    e.bias = bias;
    e.relu = (flags & PS_NN_RELU) != 0;
    e.out_bf16 = (flags & PS_NN_OUT_BF16) != 0;
    e.atomic = (flags & PS_NN_ACCUMULATE) != 0;
    e.outf = static_cast<float*>(C);
    e.outh = static_cast<__nv_bfloat16*>(C);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(nn_gemm(A, M, B, N, K, e, split < 1 ? 1 : split, s, st->d_err));
    return finish_launch(s, 1, "ps_nn_gemm_bf16");
}
