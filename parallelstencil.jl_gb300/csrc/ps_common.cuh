// ps_common.cuh -- shared host/device helpers of libps_b200.so.
#pragma once

#include <cuda.h>  // CUtensorMap and its enums only; the driver is reached through cudart
#include <cuda_runtime.h>
#include <stdint.h>

#include "ps_gb300.h"

namespace ps {

// ---------------------------------------------------------------------------------------
// Error state (thread-local message, status codes of ps_gb300.h).
// ---------------------------------------------------------------------------------------
int fail(int status, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
void clear_error();

#define PS_CUDA_TRY(call)                                       \
    do {                                                        \
        cudaError_t _ps_e = (call);                             \
        if (_ps_e != cudaSuccess) return ps::cuda_fail(_ps_e, #call); \
    } while (0)

#define PS_TRY(expr)                      \
    do {                                  \
        int _ps_rc = (expr);              \
        if (_ps_rc != PS_OK) return _ps_rc; \
    } while (0)

// Device-side error word bits (kernels OR them in; the host reads and clears the word).
enum : int { DEV_ERR_NONE = 0, DEV_ERR_TMA_TIMEOUT = 1, DEV_ERR_GRID_TIMEOUT = 2, DEV_ERR_RANGE = 4 };

// Per-device library state.
struct DeviceState {
    bool ready = false;
    int* d_err = nullptr;        // device error word (DEV_ERR_*)
    double* d_scratch = nullptr;  // small reduction scratch (library-owned)
    size_t scratch_bytes = 0;
    int num_sms = 0;
};

// Returns PS_ERR_NOT_INIT unless ps_init succeeded for the current device.
int current_state(DeviceState** st);
// Frees library-owned solver scratch (ps_finalize).
void stokes2d_free_scratch();
void stokes2d_static_forget();  // drop the cached device addresses of the static scratch array
void diffusion_free_scratch();
void adjoint_free_scratch();

// Copies `bytes` (<= 256 through pinned staging) from device memory on stream s and synchronises s.
int read_device_words(void* dst, const void* src, size_t bytes, cudaStream_t s);
// Reads (and clears) the device error word after a synchronisation.
int check_device_error(DeviceState* st, cudaStream_t s);

// After a launch: report launch errors; if sync, synchronise and report execution errors.
int finish_launch(cudaStream_t s, int sync, const char* what);

// ---------------------------------------------------------------------------------------
// Array validation.
// ---------------------------------------------------------------------------------------
inline int64_t numel(const ps_array& a) { return a.n[0] * a.n[1] * a.n[2]; }
inline size_t elsize(int32_t dtype) { return dtype == PS_F64 ? 8 : dtype == PS_F32 ? 4 : 2; }
int check_array(const ps_array& a, const char* name);
int check_same_dtype(const ps_array& a, const ps_array& b, const char* na, const char* nb);
int check_shape(const ps_array& a, int64_t nx, int64_t ny, int64_t nz, const char* name);

// Thread-index box of one call: full grid unless cfg gives a non-empty range.
struct Box {
    int64_t lo[3];
    int64_t hi[3];
};
Box launch_box(const ps_launch* cfg, const int64_t grid[3]);

// ---------------------------------------------------------------------------------------
// TMA tensor maps (cuTensorMapEncodeTiled through cudaGetDriverEntryPointByVersion).
// ---------------------------------------------------------------------------------------
// Encodes a 3-D tiled map over a dense column-major array with box (bx, by, 1), zero OOB
// fill. Returns PS_ERR_ALIGN if the array does not meet TMA's 16-byte rules.
int encode_plane_map(CUtensorMap* map, const ps_array& a, uint32_t bx, uint32_t by);
bool tma_eligible(const ps_array& a);
// 2-D map of a row-major bf16 matrix [rows][cols] with 128-byte swizzle; box = box_rows x 64
// columns (one 128-byte swizzle row). Reads past the matrix are zero-filled.
int encode_bf16_rows_sw128(CUtensorMap* map, const void* ptr, uint64_t cols, uint64_t rows, uint32_t box_cols,
                           uint32_t box_rows);

// z-sweep length for loopsize = 0: a launch of cta_xy CTAs per z-block over wz planes with
// `slots` CTAs resident at once (occupancy x SMs) loses the idle part of its last wave and
// re-reads two halo planes per z-block; the candidate with the best product wins (ties: longer).
// Results do not depend on the choice (every cell is computed the same way).
inline int auto_loopsize(int64_t cta_xy, int64_t wz, int64_t slots) {
    static const int cand[] = {64, 56, 48, 40, 32, 28, 24, 20, 16};
    int best = 64;
    double best_score = -1.0;
    for (int L : cand) {
        const int64_t ctas = cta_xy * ((wz + L - 1) / L);
        const int64_t waves = (ctas + slots - 1) / slots;
        const double score = (double)ctas / (double)(waves * slots) * (double)L / (L + 2.0);
        if (score > best_score + 1e-9) {
            best_score = score;
            best = L;
        }
    }
    return best;
}

// CTAs of `kernel` resident per SM (queried once per kernel by the caller's static cache).
template <typename K>
inline int resident_ctas(K kernel, int threads, int smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

// ---------------------------------------------------------------------------------------
// Device helpers.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int64_t idx3(int64_t x, int64_t y, int64_t z, int64_t nx, int64_t ny) {
    return x + nx * (y + ny * z);
}

// Julia's Base.max / Base.min for IEEE floats (NaN-propagating; -0.0 < 0.0).
template <typename T>
__device__ __forceinline__ T jl_max(T x, T y) {
    T diff = x - y;
    T r = signbit(diff) ? y : x;
    return (isnan(x) || isnan(y)) ? diff : r;
}
template <typename T>
__device__ __forceinline__ T jl_min(T x, T y) {
    T diff = x - y;
    T r = signbit(diff) ? x : y;
    return (isnan(x) || isnan(y)) ? diff : r;
}

// --- mbarrier / TMA inline PTX (sm_90+; used on sm_103a) ---------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's generic-proxy shared-memory writes before later async-proxy (TMA) accesses
// of the same bytes (a staged slot rewritten in place and later refilled by a TMA load).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after ~2^22 polls (each poll may itself suspend briefly).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}
__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

}  // namespace ps
