// ps_core.cu -- device state, errors, memory, streams and TMA descriptors of libps_b200.so.
//
// Replaces the CUDA-extension plumbing of ParallelStencil.jl: device selection at
// `@init_parallel_stencil` (src/init_parallel_stencil.jl:36-51), `@zeros`/`@fill!`
// allocation (src/ParallelKernel/CUDAExt/allocators.jl:3-8), and the priority / normal
// stream pools of `@hide_communication` (src/ParallelKernel/CUDAExt/shared.jl:17-31).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "ps_common.cuh"

namespace ps {

static thread_local char g_errmsg[512] = "";
static constexpr int kMaxDevices = 64;
static DeviceState g_dev[kMaxDevices];
static std::mutex g_mutex;

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn g_encode = nullptr;

int fail(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(PS_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

void clear_error() { g_errmsg[0] = '\0'; }

int current_state(DeviceState** st) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices || !g_dev[dev].ready)
        return fail(PS_ERR_NOT_INIT, "ps_init has not been called for the current device");
    *st = &g_dev[dev];
    return PS_OK;
}

// A small pinned staging buffer per host thread for reading device flags and norms: a copy into
// pageable memory goes through the driver's own staging and can queue behind large copies of other
// streams. Freed when the thread exits.
namespace {
struct PinnedWords {
    void* p = nullptr;
    bool tried = false;
    ~PinnedWords() {
        if (p) cudaFreeHost(p);
    }
};
thread_local PinnedWords t_pinned;
constexpr size_t kPinnedWordBytes = 256;
}  // namespace

namespace {
struct MappedWord {
    unsigned* h = nullptr;
    bool tried = false;
    ~MappedWord() {
        if (h) cudaFreeHost(h);
    }
};
thread_local MappedWord t_mapped;
}  // namespace

int progress_word(volatile unsigned** host, unsigned** dev) {
    *host = nullptr;
    *dev = nullptr;
    if (!t_mapped.tried) {
        t_mapped.tried = true;
        void* p = nullptr;
        if (cudaHostAlloc(&p, 64, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
            cudaGetLastError();
            return PS_OK;
        }
        t_mapped.h = static_cast<unsigned*>(p);
    }
    if (!t_mapped.h) return PS_OK;
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, t_mapped.h, 0) != cudaSuccess) {
        cudaGetLastError();
        return PS_OK;
    }
    *host = t_mapped.h;
    *dev = static_cast<unsigned*>(d);
    return PS_OK;
}

TileOrder make_tile_order(const int64_t ntiles[3], const int64_t lo[3], const int64_t tile[3], const int64_t end[3],
                          const int64_t lo_end[3], const int64_t hi_start[3], unsigned* counter) {
    int64_t b0[3], b1[3];
    for (int d = 0; d < 3; ++d) {
        // tiles holding a cell c < lo_end[d], and tiles holding a cell c >= hi_start[d]
        b0[d] = lo_end[d] > lo[d] ? (lo_end[d] - lo[d] + tile[d] - 1) / tile[d] : 0;
        const int64_t first_hi = hi_start[d] > lo[d] ? (hi_start[d] - lo[d]) / tile[d] : 0;
        b1[d] = hi_start[d] < end[d] ? ntiles[d] - first_hi : 0;
        if (b0[d] > ntiles[d]) b0[d] = ntiles[d];
        if (b1[d] < 0) b1[d] = 0;
        if (b0[d] + b1[d] >= ntiles[d]) {  // every tile along this axis holds boundary cells
            b0[d] = ntiles[d];
            b1[d] = 0;
        }
    }
    TileOrder o{};
    o.counter = counter;
    o.TX = (int)ntiles[0];
    o.TY = (int)ntiles[1];
    o.TZ = (int)ntiles[2];
    o.bx0 = (int)b0[0];
    o.bx1 = (int)b1[0];
    o.by0 = (int)b0[1];
    o.by1 = (int)b1[1];
    o.bz0 = (int)b0[2];
    o.bz1 = (int)b1[2];
    const int64_t inner = (ntiles[0] - b0[0] - b1[0]) * (ntiles[1] - b0[1] - b1[1]) * (ntiles[2] - b0[2] - b1[2]);
    o.nb = (int)(ntiles[0] * ntiles[1] * ntiles[2] - inner);
    return o;
}

int read_device_words(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    if (!t_pinned.tried) {
        t_pinned.tried = true;
        if (cudaMallocHost(&t_pinned.p, kPinnedWordBytes) != cudaSuccess) {
            cudaGetLastError();
            t_pinned.p = nullptr;
        }
    }
    void* stage = (t_pinned.p && bytes <= kPinnedWordBytes) ? t_pinned.p : dst;
    PS_CUDA_TRY(cudaMemcpyAsync(stage, src, bytes, cudaMemcpyDeviceToHost, s));
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    if (stage != dst) memcpy(dst, stage, bytes);
    return PS_OK;
}

int check_device_error(DeviceState* st, cudaStream_t s) {
    int h = 0;
    PS_TRY(read_device_words(&h, st->d_err, sizeof(int), s));
    if (h != DEV_ERR_NONE) {
        int zero = 0;
        PS_CUDA_TRY(cudaMemcpyAsync(st->d_err, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
        PS_CUDA_TRY(cudaStreamSynchronize(s));
        if (h & (DEV_ERR_TMA_TIMEOUT | DEV_ERR_GRID_TIMEOUT))
            return fail(PS_ERR_TIMEOUT, "a bounded device-side wait gave up (device error bits %d)", h);
        return fail(PS_ERR_UNSUPPORTED, "an FP64 value outside the split-arithmetic range (|x| >= 2^128 or "
                    "non-finite) was seen; rerun with fp64_mode = PS_FP64_IEEE (device error bits %d)", h);
    }
    return PS_OK;
}

int finish_launch(cudaStream_t s, int sync, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (sync) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, what);
        DeviceState* st = nullptr;
        PS_TRY(current_state(&st));
        PS_TRY(check_device_error(st, s));
    }
    return PS_OK;
}

int check_array(const ps_array& a, const char* name) {
    if (a.ptr == nullptr) return fail(PS_ERR_NULL, "array %s: NULL device pointer", name);
    if (a.dtype != PS_F64 && a.dtype != PS_F32) return fail(PS_ERR_DTYPE, "array %s: unsupported dtype %d", name, a.dtype);
    for (int d = 0; d < 3; d++)
        if (a.n[d] < 1) return fail(PS_ERR_SHAPE, "array %s: extent n[%d] = %lld < 1", name, d, (long long)a.n[d]);
    if ((reinterpret_cast<uintptr_t>(a.ptr) % elsize(a.dtype)) != 0)
        return fail(PS_ERR_ALIGN, "array %s: pointer not aligned to its element size", name);
    return PS_OK;
}

int check_same_dtype(const ps_array& a, const ps_array& b, const char* na, const char* nb) {
    if (a.dtype != b.dtype) return fail(PS_ERR_DTYPE, "arrays %s and %s have different dtypes", na, nb);
    return PS_OK;
}

int check_shape(const ps_array& a, int64_t nx, int64_t ny, int64_t nz, const char* name) {
    if (a.n[0] != nx || a.n[1] != ny || a.n[2] != nz)
        return fail(PS_ERR_SHAPE, "array %s: size (%lld,%lld,%lld), expected (%lld,%lld,%lld)", name,
                    (long long)a.n[0], (long long)a.n[1], (long long)a.n[2], (long long)nx, (long long)ny,
                    (long long)nz);
    return PS_OK;
}

Box launch_box(const ps_launch* cfg, const int64_t grid[3]) {
    Box b;
    bool use = cfg != nullptr;
    if (use) {
        bool any = false;
        for (int d = 0; d < 3; d++) any |= cfg->range_hi[d] > cfg->range_lo[d];
        use = any;
    }
    for (int d = 0; d < 3; d++) {
        b.lo[d] = use ? cfg->range_lo[d] : 0;
        b.hi[d] = use ? cfg->range_hi[d] : grid[d];
        if (b.lo[d] < 0) b.lo[d] = 0;
        if (b.hi[d] > grid[d]) b.hi[d] = grid[d];
    }
    return b;
}

bool tma_eligible(const ps_array& a) {
    size_t es = elsize(a.dtype);
    if (reinterpret_cast<uintptr_t>(a.ptr) % 16 != 0) return false;
    if ((a.n[0] * es) % 16 != 0) return false;
    if ((a.n[0] * a.n[1] * es) % 16 != 0) return false;
    if (a.n[0] >= (1ll << 32) || a.n[1] >= (1ll << 32) || a.n[2] >= (1ll << 32)) return false;
    return g_encode != nullptr;
}

int encode_plane_map(CUtensorMap* map, const ps_array& a, uint32_t bx, uint32_t by) {
    if (!tma_eligible(a)) return fail(PS_ERR_ALIGN, "array not eligible for TMA (16-byte base/stride rule)");
    size_t es = elsize(a.dtype);
    if ((bx * es) % 16 != 0 || bx > 256 || by > 256) return fail(PS_ERR_ARG, "invalid TMA box (%u, %u)", bx, by);
    cuuint64_t dims[3] = {(cuuint64_t)a.n[0], (cuuint64_t)a.n[1], (cuuint64_t)a.n[2]};
    cuuint64_t strides[2] = {(cuuint64_t)(a.n[0] * es), (cuuint64_t)(a.n[0] * a.n[1] * es)};
    cuuint32_t box[3] = {bx, by, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUtensorMapDataType dt = a.dtype == PS_F64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    CUresult r = g_encode(map, dt, 3, a.ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(PS_ERR_CUDA, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
    return PS_OK;
}

int encode_bf16_rows_sw128(CUtensorMap* map, const void* ptr, uint64_t cols, uint64_t rows, uint32_t box_cols,
                           uint32_t box_rows) {
    if (!g_encode) return fail(PS_ERR_NOT_INIT, "TMA encoder unavailable (ps_init not called)");
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (cols * 2) % 16 || cols == 0 || rows == 0)
        return fail(PS_ERR_ALIGN, "bf16 matrix not TMA-eligible (16-byte base and row stride)");
    if (box_cols * 2 != 128 || box_rows == 0 || box_rows > 256) return fail(PS_ERR_ARG, "invalid bf16 TMA box");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(cols * 2)};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(PS_ERR_CUDA, "cuTensorMapEncodeTiled (bf16) failed (CUresult %d)", (int)r);
    return PS_OK;
}

// ps_check_division: div_c against the IEEE division. Dividend i: FP32 -- significand i mod 2^23,
// exponent and sign from i / 2^23 (every significand in each listed binade, both signs); FP64 --
// a hashed 52-bit significand, exponent and sign from the hash too. The first 64 indices are
// special values (zeros, subnormals, extremes, infinities, NaN).
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
__constant__ int c_exp32[12] = {-126, -101, -100, -99, -70, -1, 0, 1, 69, 70, 71, 127};
__constant__ int c_exp64[12] = {-1022, -961, -960, -959, -900, -1, 0, 1, 899, 900, 901, 1023};

template <typename T>
__device__ T special_dividend(int i) {
    const T v[16] = {(T)0, -(T)0, (T)1, -(T)1, (T)INFINITY, -(T)INFINITY, (T)NAN,
                     sizeof(T) == 4 ? (T)1e-40f : (T)1e-310, sizeof(T) == 4 ? (T)-1e-45f : (T)-4e-324,
                     sizeof(T) == 4 ? (T)3.4e38f : (T)1.7e308, sizeof(T) == 4 ? (T)1.17549435e-38f : (T)2.2250738585072014e-308,
                     (T)3, (T)0.1, (T)-7.5, (T)1e10, (T)-1e-10};
    return v[i & 15];
}

__global__ void check_div32_kernel(DivC<float> d, unsigned long long* bad) {
    const int64_t n = 12LL * 2 * (1LL << 23);
    unsigned long long local = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float a;
        if (i < 64) {
            a = special_dividend<float>((int)i);
        } else {
            const unsigned m = (unsigned)(i & ((1 << 23) - 1));
            const int64_t k = i >> 23;
            const int e = c_exp32[(k >> 1) % 12];
            a = ldexpf(1.0f + (float)m * 0x1p-23f, e) * ((k & 1) ? -1.0f : 1.0f);
        }
        const float q1 = div_c(a, d), q2 = a / d.b;
        if (__float_as_uint(q1) != __float_as_uint(q2) && !(isnan(q1) && isnan(q2))) ++local;
    }
    if (local) atomicAdd(bad, local);
}

__global__ void check_div64_kernel(DivC<double> d, int64_t n, uint64_t seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a;
        if (i < 64) {
            a = special_dividend<double>((int)i);
        } else {
            const uint64_t h = mix64(seed ^ (uint64_t)i * 0x9e3779b97f4a7c15ull);
            const int e = c_exp64[(h >> 52) % 12];
            a = ldexp(1.0 + (double)(h & ((1ull << 52) - 1)) * 0x1p-52, e) * ((h >> 63) ? -1.0 : 1.0);
        }
        const double q1 = div_c(a, d), q2 = a / d.b;
        if (__double_as_longlong(q1) != __double_as_longlong(q2) && !(isnan(q1) && isnan(q2))) ++local;
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_check_division(double b, int32_t dtype, int64_t n, uint64_t seed, int64_t* mismatches, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (!mismatches) return fail(PS_ERR_NULL, "ps_check_division: NULL output");
    if (dtype != PS_F32 && dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_check_division: dtype %d", dtype);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long* bad = nullptr;
    PS_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&bad), sizeof(*bad), s));
    PS_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(*bad), s));
    const unsigned grid = (unsigned)st->num_sms * 8;
    if (dtype == PS_F32)
        check_div32_kernel<<<grid, 256, 0, s>>>(make_div<float>((float)b), bad);
    else
        check_div64_kernel<<<grid, 256, 0, s>>>(make_div<double>(b), n, seed, bad);
    unsigned long long h = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(bad, s);
    if (e != cudaSuccess) return cuda_fail(e, "ps_check_division");
    *mismatches = (int64_t)h;
    return PS_OK;
}

int ps_abi_version(void) { return PS_ABI_VERSION; }

const char* ps_last_error(void) { return g_errmsg; }

int ps_device_count(int* count) {
    if (!count) return fail(PS_ERR_NULL, "ps_device_count: NULL output");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return PS_OK;
}

int ps_init(int device) {
    std::lock_guard<std::mutex> lock(g_mutex);
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(PS_ERR_CUDA, "ps_init: no CUDA device available (%s)", cudaGetErrorString(e));
    }
    if (device < 0 || device >= n || device >= kMaxDevices)
        return fail(PS_ERR_ARG, "ps_init: device %d out of range (0..%d)", device, n - 1);
    PS_CUDA_TRY(cudaSetDevice(device));
    DeviceState& st = g_dev[device];
    if (st.ready) return PS_OK;
    cudaDeviceProp prop;
    PS_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) return fail(PS_ERR_UNSUPPORTED, "ps_init: device %d is sm_%d%d; this build targets sm_103a", device, prop.major, prop.minor);
    st.num_sms = prop.multiProcessorCount;
    PS_CUDA_TRY(cudaMalloc(&st.d_err, sizeof(int)));
    PS_CUDA_TRY(cudaMemset(st.d_err, 0, sizeof(int)));
    st.scratch_bytes = 64 * 1024;
    PS_CUDA_TRY(cudaMalloc(&st.d_scratch, st.scratch_bytes));
    if (g_encode == nullptr) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<EncodeTiledFn>(fn);
        cudaGetLastError();
    }
    PS_CUDA_TRY(cudaDeviceSynchronize());
    st.ready = true;
    clear_error();
    return PS_OK;
}

int ps_finalize(void) {
    std::lock_guard<std::mutex> lock(g_mutex);
    int cur = 0;
    cudaGetDevice(&cur);
    stokes2d_free_scratch();
    diffusion_free_scratch();
    adjoint_free_scratch();
    acoustic_free_scratch();
    stokes3d_free_scratch();
    stokes2d_static_forget();
    for (int d = 0; d < kMaxDevices; d++) {
        DeviceState& st = g_dev[d];
        if (!st.ready) continue;
        cudaSetDevice(d);
        cudaDeviceSynchronize();
        cudaFree(st.d_err);
        cudaFree(st.d_scratch);
        st = DeviceState();
    }
    cudaSetDevice(cur);
    cudaGetLastError();
    return PS_OK;
}

int ps_alloc(ps_array* a, int32_t dtype, int64_t nx, int64_t ny, int64_t nz) {
    if (!a) return fail(PS_ERR_NULL, "ps_alloc: NULL descriptor");
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (dtype != PS_F64 && dtype != PS_F32 && dtype != PS_BF16) return fail(PS_ERR_DTYPE, "ps_alloc: dtype %d", dtype);
    if (nx < 1 || ny < 1 || nz < 1) return fail(PS_ERR_SHAPE, "ps_alloc: extents must be >= 1");
    size_t bytes = (size_t)nx * (size_t)ny * (size_t)nz * elsize(dtype);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(PS_ERR_NOMEM, "ps_alloc: cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    PS_CUDA_TRY(cudaMemset(p, 0, bytes));
    a->ptr = p;
    a->n[0] = nx;
    a->n[1] = ny;
    a->n[2] = nz;
    a->dtype = dtype;
    a->reserved = 0;
    return PS_OK;
}

int ps_free(ps_array* a) {
    if (!a) return fail(PS_ERR_NULL, "ps_free: NULL descriptor");
    if (a->ptr) PS_CUDA_TRY(cudaFree(a->ptr));
    a->ptr = nullptr;
    return PS_OK;
}

int ps_copy_h2d(ps_array dst, const void* host_src, void* stream) {
    PS_TRY(check_array(dst, "dst"));
    if (!host_src) return fail(PS_ERR_NULL, "ps_copy_h2d: NULL host pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_CUDA_TRY(cudaMemcpyAsync(dst.ptr, host_src, numel(dst) * elsize(dst.dtype), cudaMemcpyHostToDevice, s));
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    return PS_OK;
}

int ps_copy_d2h(void* host_dst, ps_array src, void* stream) {
    PS_TRY(check_array(src, "src"));
    if (!host_dst) return fail(PS_ERR_NULL, "ps_copy_d2h: NULL host pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_CUDA_TRY(cudaMemcpyAsync(host_dst, src.ptr, numel(src) * elsize(src.dtype), cudaMemcpyDeviceToHost, s));
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    return PS_OK;
}

int ps_copy_h2d_async(ps_array dst, const void* host_src, void* stream) {
    PS_TRY(check_array(dst, "dst"));
    if (!host_src) return fail(PS_ERR_NULL, "ps_copy_h2d_async: NULL host pointer");
    PS_CUDA_TRY(cudaMemcpyAsync(dst.ptr, host_src, numel(dst) * elsize(dst.dtype), cudaMemcpyHostToDevice,
                                static_cast<cudaStream_t>(stream)));
    return PS_OK;
}

int ps_copy_d2h_async(void* host_dst, ps_array src, void* stream) {
    PS_TRY(check_array(src, "src"));
    if (!host_dst) return fail(PS_ERR_NULL, "ps_copy_d2h_async: NULL host pointer");
    PS_CUDA_TRY(cudaMemcpyAsync(host_dst, src.ptr, numel(src) * elsize(src.dtype), cudaMemcpyDeviceToHost,
                                static_cast<cudaStream_t>(stream)));
    return PS_OK;
}

int ps_copy_d2d_async(ps_array dst, ps_array src, void* stream) {
    PS_TRY(check_array(dst, "dst"));
    PS_TRY(check_array(src, "src"));
    PS_TRY(check_same_dtype(dst, src, "dst", "src"));
    PS_TRY(check_shape(src, dst.n[0], dst.n[1], dst.n[2], "src"));
    PS_CUDA_TRY(cudaMemcpyAsync(dst.ptr, src.ptr, numel(dst) * elsize(dst.dtype), cudaMemcpyDeviceToDevice,
                                static_cast<cudaStream_t>(stream)));
    return PS_OK;
}

int ps_stream_create(int priority, void** stream) {
    if (!stream) return fail(PS_ERR_NULL, "ps_stream_create: NULL output");
    int lo = 0, hi = 0;
    PS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    cudaStream_t s;
    PS_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, priority > 0 ? hi : lo));
    *stream = s;
    return PS_OK;
}

int ps_stream_destroy(void* stream) {
    if (stream) PS_CUDA_TRY(cudaStreamDestroy(static_cast<cudaStream_t>(stream)));
    return PS_OK;
}

int ps_synchronize(void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    return check_device_error(st, s);
}

}  // extern "C"
