// ps_common.cuh -- shared host/device helpers of libps_b200.so.
#pragma once

#include <cuda.h>  // CUtensorMap and its enums only; the driver is reached through cudart
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

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
void acoustic_free_scratch();
void stokes3d_free_scratch();

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
// Boundary-first tile order (`@hide_communication` in one launch).
// ---------------------------------------------------------------------------------------
// A z-sweep launch over TX x TY x TZ tiles (x tile columns, y tile rows, z chunks) can run as a
// 1-D grid whose first `nb` CTAs take the tiles holding boundary cells -- bx0 / bx1 tile columns
// at the low / high x end, by0 / by1 rows, bz0 / bz1 chunks -- and the rest the inner block. Each
// boundary CTA, once its stores are done, increments `counter` (host-mapped memory); the host
// calls the communication when the counter reaches nb, while the inner tiles still run. The
// kernel never waits on the host. counter == NULL: an ordinary launch (blockIdx is the tile).
struct TileOrder {
    unsigned* counter;
    int TX, TY, TZ;
    int bx0, bx1, by0, by1, bz0, bz1;
    int nb;
};
// Host: the order of a TX x TY x TZ tile launch whose tiles start at cell lo + t * tile (per
// axis) over the cells [lo, end); boundary cells are c < lo_end or c >= hi_start.
TileOrder make_tile_order(const int64_t ntiles[3], const int64_t lo[3], const int64_t tile[3], const int64_t end[3],
                          const int64_t lo_end[3], const int64_t hi_start[3], unsigned* counter);
// What a caller asks of a boundary-first launch (the launcher fills nb).
struct HideReq {
    int64_t lo_end[3], hi_start[3];
    unsigned* counter;
    int nb;
};
// Host: the thread's host-mapped progress word (allocated on first use; NULL pointers if the
// device cannot map host memory).
int progress_word(volatile unsigned** host, unsigned** dev);

__device__ __forceinline__ uint3 ordered_tile(const TileOrder& o) {
    if (!o.counter) return make_uint3(blockIdx.x, blockIdx.y, blockIdx.z);
    int i = (int)blockIdx.x;
    const int IX = o.TX - o.bx0 - o.bx1, IY = o.TY - o.by0 - o.by1;
    if (i >= o.nb) {  // the inner block, x fastest
        i -= o.nb;
        return make_uint3(o.bx0 + i % IX, o.by0 + (i / IX) % IY, o.bz0 + i / (IX * IY));
    }
    const int layer = o.TX * o.TY;
    const int nzfull = (o.bz0 + o.bz1) * layer;
    if (i < nzfull) {  // whole layers at both z ends
        const int l = i / layer, r = i % layer;
        return make_uint3(r % o.TX, r / o.TX, l < o.bz0 ? l : o.TZ - o.bz1 + (l - o.bz0));
    }
    i -= nzfull;  // the frames of the middle layers: whole rows at both y ends, then column ends
    const int frame = layer - IX * IY;
    const int z = o.bz0 + i / frame;
    int r = i % frame;
    const int nyfull = (o.by0 + o.by1) * o.TX;
    if (r < nyfull) {
        const int row = r / o.TX;
        return make_uint3(r % o.TX, row < o.by0 ? row : o.TY - o.by1 + (row - o.by0), z);
    }
    r -= nyfull;
    const int ex = o.bx0 + o.bx1, c = r % ex;
    return make_uint3(c < o.bx0 ? c : o.TX - o.bx1 + (c - o.bx0), o.by0 + r / ex, z);
}

// Called by every thread of a CTA after its last global store (plain stores only).
__device__ __forceinline__ void ordered_tile_done(const TileOrder& o) {
    if (!o.counter || (int)blockIdx.x >= o.nb) return;  // uniform over the CTA
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        __threadfence_system();
        atomicAdd_system(o.counter, 1u);
    }
}

// ---------------------------------------------------------------------------------------
// Division by a number known on the host, correctly rounded.
// ---------------------------------------------------------------------------------------
// Markstein's method (P. W. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34 (1990) 111-119): with y = RN(1/b) and a quotient
// q within one ulp of a/b, the remainder r = a - b q is exact in one FMA and RN(q + r y) = RN(a/b).
// The first quotient RN(a y) can be 1.5 ulps off, so one FMA correction brings it within an ulp and
// a second gives the correctly rounded quotient: 1 multiply + 4 FMAs against the general division's
// reciprocal iteration and slow-path test. Dividends outside [lo, hi] (tiny, huge, non-finite; zero
// is a * y, with the quotient's sign) take the IEEE division; for divisors outside [2^-20, 2^20]
// (FP32) or [2^-60, 2^60] (FP64) the host sets lo > hi and every division takes it. lo keeps the
// quotient normal and the remainder a - bq, a multiple of 2^(e(a) - 2p + 1), representable
// (subnormal remainders are exact); hi keeps a*y and the quotient finite. Results equal a / b bit
// for bit (checked against the IEEE division by ps_check_division).
template <typename T>
struct DivC {
    T b, y, lo, hi;
};
template <typename T>
inline DivC<T> make_div(T b) {
    const T lim = sizeof(T) == 4 ? (T)0x1p20 : (T)0x1p60;
    const T a = b < 0 ? -b : b;
    DivC<T> d;
    d.b = b;
    if (a >= 1 / lim && a <= lim) {
        d.y = (T)1 / b;
        d.lo = sizeof(T) == 4 ? (T)0x1p-100 : (T)0x1p-960;
        d.hi = sizeof(T) == 4 ? (T)0x1p70 : (T)0x1p900;
    } else {
        d.y = 0;
        d.lo = 1;
        d.hi = 0;
    }
    return d;
}
__device__ __forceinline__ float div_c(float a, const DivC<float>& d) {
    const float aa = fabsf(a);
    if (aa >= d.lo && aa <= d.hi) {
        float q = a * d.y;
        float r = fmaf(-q, d.b, a);
        q = fmaf(r, d.y, q);
        r = fmaf(-q, d.b, a);
        return fmaf(r, d.y, q);
    }
    return (aa == 0.0f && d.lo <= d.hi) ? a * d.y : a / d.b;
}
__device__ __forceinline__ double div_c(double a, const DivC<double>& d) {
    const double aa = fabs(a);
    if (aa >= d.lo && aa <= d.hi) {
        double q = a * d.y;
        double r = fma(-q, d.b, a);
        q = fma(r, d.y, q);
        r = fma(-q, d.b, a);
        return fma(r, d.y, q);
    }
    return (aa == 0.0 && d.lo <= d.hi) ? a * d.y : a / d.b;
}

// a / h for statement helpers used with a plain divisor (host or device) or a DivC (device)
template <typename T>
__host__ __device__ __forceinline__ T dvd(T a, T h) {
    return a / h;
}
template <typename T>
__device__ __forceinline__ T dvd(T a, const DivC<T>& h) {
    return div_c(a, h);
}

// ---------------------------------------------------------------------------------------
// Programmatic dependent launch: a kernel launched with launch_dependent() may start while the
// kernel before it on the stream finishes its last wave; it waits in grid_dependency_wait() (a
// no-op in an ordinary launch) until that kernel has completed and its stores are visible, so
// every read of data the previous kernel wrote must come after the wait.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dependents_may_launch() { asm volatile("griddepcontrol.launch_dependents;"); }
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                    Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
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
// The same for doubles without FP64 instructions (GB300 issues FP64 at 2 per clock per SM): the
// bits of a double with the magnitude bits flipped for negative values order as the values do,
// with -0.0 below 0.0, so for non-NaN operands the larger key is the result above, bit for bit
// (equal keys are equal values); a NaN operand is returned itself, as Julia's max and min do (a
// NaN either way: its payload is the operand's instead of the difference's).
__device__ __forceinline__ long long jl_key(long long b) { return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL); }
__device__ __forceinline__ bool jl_nan_bits(long long b) { return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL; }
template <>
__device__ __forceinline__ double jl_max<double>(double x, double y) {
    const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
    const double r = jl_key(bx) >= jl_key(by) ? x : y;
    return jl_nan_bits(bx) ? x : jl_nan_bits(by) ? y : r;
}
template <>
__device__ __forceinline__ double jl_min<double>(double x, double y) {
    const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
    const double r = jl_key(bx) < jl_key(by) ? x : y;
    return jl_nan_bits(bx) ? x : jl_nan_bits(by) ? y : r;
}
// Floats: max.NaN / min.NaN order -0.0 below 0.0 and give the canonical NaN when an operand is NaN,
// as the subtraction above does on the GPU (checked over signed zeros, subnormals, infinities and
// NaNs against Julia's rules): one instruction instead of six.
template <>
__device__ __forceinline__ float jl_max<float>(float x, float y) {
    float d;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(x), "f"(y));
    return d;
}
template <>
__device__ __forceinline__ float jl_min<float>(float x, float y) {
    float d;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(x), "f"(y));
    return d;
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
