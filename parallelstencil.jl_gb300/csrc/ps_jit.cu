// ps_jit.cu -- run-time compiled `@parallel` / `@parallel_indices` kernels.
//
// The host side (ps_gb300/jit.py) translates a kernel body written with the FiniteDifferences
// macros (or with explicit indexing, for `@parallel_indices`) into CUDA C following the same rules
// as the library's fixed kernels: the grid is the largest extent of the array arguments, every
// statement is masked by `@within` of its left-hand selection, literals take the number type, and
// there is no FMA contraction. Unless the kernel is defined with `inbounds=true`, every array access
// is bounds-checked: an index outside the array skips the access and sets the kernel's error flag,
// which a synchronous launch reads back and reports (Julia raises a BoundsError there). This file compiles that source with NVRTC for sm_103a
// (`--fmad=false`), loads the cubin into the current context and launches its entry point with one
// by-value argument block (ps_jit_args below; the generated source declares the same layout).
//
// Driver-API entry points (module load / launch) are looked up through the runtime like the TMA
// encoder, so the library still links only the static runtime and NVRTC.
#include <nvrtc.h>
#include <string.h>

#include <chrono>
#include <mutex>
#include <string>
#include <vector>

#include "ps_common.cuh"

namespace ps {

// By-value argument block of every generated kernel (identical layout in the generated source).
constexpr int kJitMaxArrays = 32, kJitMaxScalars = 32;
struct ps_jit_args {
    void* a[kJitMaxArrays];
    long long n[kJitMaxArrays][3];
    double s[kJitMaxScalars];
    long long lo[3];   // first thread index (0-based) per dimension
    long long cnt[3];  // threads per dimension
    int* err;          // error flags of the kernel (device memory, one int): 1 out of bounds, 2 partial block,
                       // 4 a value outside the split FP64 range
    long long smem;    // dynamic shared memory bytes of this launch (@sharedMem views are checked against it)
    long long loop;    // indices per thread along the sweep dimension of a sweep (memopt) kernel; 1 otherwise
    unsigned* ocnt;    // boundary-first launch (ps_jit_hide_communication): host-mapped count of finished
                       // boundary blocks; NULL for an ordinary launch
    int ord[10];       // its tile order: blocks per axis, boundary blocks at both ends of each axis, their count
};

typedef CUresult (*ModuleLoadDataFn)(CUmodule*, const void*);
typedef CUresult (*ModuleGetFunctionFn)(CUfunction*, CUmodule, const char*);
typedef CUresult (*ModuleUnloadFn)(CUmodule);
typedef CUresult (*LaunchKernelFn)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                                   CUstream, void**, void**);
typedef CUresult (*FuncSetAttributeFn)(CUfunction, CUfunction_attribute, int);
static ModuleLoadDataFn g_load = nullptr;
static ModuleGetFunctionFn g_getfn = nullptr;
static ModuleUnloadFn g_unload = nullptr;
static LaunchKernelFn g_launch = nullptr;
static FuncSetAttributeFn g_setattr = nullptr;
static std::mutex g_jit_mutex;

template <typename F>
static int driver_fn(const char* name, F* out) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return fail(PS_ERR_CUDA, "driver entry point %s unavailable", name);
    }
    *out = reinterpret_cast<F>(fn);
    return PS_OK;
}

static int jit_driver() {
    std::lock_guard<std::mutex> l(g_jit_mutex);
    if (g_launch) return PS_OK;
    PS_TRY(driver_fn("cuModuleLoadData", &g_load));
    PS_TRY(driver_fn("cuModuleGetFunction", &g_getfn));
    PS_TRY(driver_fn("cuModuleUnload", &g_unload));
    PS_TRY(driver_fn("cuFuncSetAttribute", &g_setattr));
    PS_TRY(driver_fn("cuLaunchKernel", &g_launch));
    return PS_OK;
}

struct JitKernel {
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    int device = -1;
    int* err = nullptr;
    int smem_opt_in = 48 * 1024;  // dynamic shared memory the function is currently allowed
};

}  // namespace ps

using namespace ps;

extern "C" {

int ps_jit_compile(const char* source, const char* entry, void** kernel) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (!source || !entry || !kernel) return fail(PS_ERR_NULL, "ps_jit_compile: NULL argument");
    *kernel = nullptr;
    PS_TRY(jit_driver());
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source, "ps_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        return fail(PS_ERR_CUDA, "ps_jit_compile: nvrtcCreateProgram failed");
    const char* opts[] = {"--gpu-architecture=sm_103a", "--fmad=false", "-std=c++17"};
    const nvrtcResult rc = nvrtcCompileProgram(prog, 3, opts);
    if (rc != NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        nvrtcDestroyProgram(&prog);
        return fail(PS_ERR_ARG, "ps_jit_compile: %s: %.400s", nvrtcGetErrorString(rc), log.c_str());
    }
    size_t nbin = 0;
    std::vector<char> bin;
    if (nvrtcGetCUBINSize(prog, &nbin) == NVRTC_SUCCESS && nbin) {
        bin.resize(nbin);
        nvrtcGetCUBIN(prog, bin.data());
    }
    nvrtcDestroyProgram(&prog);
    if (bin.empty()) return fail(PS_ERR_CUDA, "ps_jit_compile: NVRTC produced no cubin");
    JitKernel* k = new JitKernel();
    if (cudaMalloc(&k->err, sizeof(int)) != cudaSuccess || cudaMemset(k->err, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        if (k->err) cudaFree(k->err);
        delete k;
        return fail(PS_ERR_NOMEM, "ps_jit_compile: cannot allocate the error flag");
    }
    CUresult r = g_load(&k->mod, bin.data());
    if (r == CUDA_SUCCESS) r = g_getfn(&k->fn, k->mod, entry);
    if (r != CUDA_SUCCESS) {
        if (k->mod) g_unload(k->mod);
        cudaFree(k->err);
        delete k;
        return fail(PS_ERR_CUDA, "ps_jit_compile: loading the module or entry %s failed (CUresult %d)", entry, (int)r);
    }
    cudaGetDevice(&k->device);
    *kernel = k;
    return PS_OK;
}

int ps_jit_launch(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                  const int64_t lo[3], const int64_t count[3], void* stream, int sync) {
    const int32_t threads[3] = {32, 8, 1};
    return ps_jit_launch_ex(kernel, arrays, narrays, scalars, nscalars, lo, count, threads, 0, nullptr, stream, sync);
}

}  // extern "C"

namespace ps {

// Validates a launch and fills its argument block and grid (gd: blocks per axis; all zero when a
// count is zero).
static int jit_prepare(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                       const int64_t lo[3], const int64_t count[3], const int32_t threads[3], int64_t shmem,
                       const int32_t loop[3], JitKernel** kout, ps_jit_args* g, int64_t gd[3], int32_t lp[3]) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (!kernel || !lo || !count || !threads) return fail(PS_ERR_NULL, "ps_jit_launch: NULL argument");
    if (threads[0] < 1 || threads[1] < 1 || threads[2] < 1 || threads[2] > 64 ||
        (int64_t)threads[0] * threads[1] * threads[2] > 1024 || threads[0] > 1024 || threads[1] > 1024)
        return fail(PS_ERR_ARG, "ps_jit_launch: threads per block must be >= 1 and at most 1024 (z <= 64)");
    if (shmem < 0 || shmem > 227 * 1024)
        return fail(PS_ERR_ARG, "ps_jit_launch: shmem must be 0 to 232448 bytes (227 KB)");
    lp[0] = lp[1] = lp[2] = 1;
    int nsweep = 0;
    for (int d = 0; d < 3 && loop; d++) {
        lp[d] = loop[d];
        if (lp[d] < 1 || (lp[d] > 1 && threads[d] != 1))
            return fail(PS_ERR_ARG, "ps_jit_launch: loop[%d] must be >= 1, with threads[%d] == 1 when > 1", d, d);
        nsweep += lp[d] > 1;
    }
    if (nsweep > 1) return fail(PS_ERR_ARG, "ps_jit_launch: a sweep kernel loops along one dimension only");
    if (narrays < 0 || narrays > kJitMaxArrays || nscalars < 0 || nscalars > kJitMaxScalars ||
        (narrays && !arrays) || (nscalars && !scalars))
        return fail(PS_ERR_ARG, "ps_jit_launch: at most %d arrays and %d scalars", kJitMaxArrays, kJitMaxScalars);
    JitKernel* k = static_cast<JitKernel*>(kernel);
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != k->device) return fail(PS_ERR_ARG, "ps_jit_launch: kernel compiled for device %d", k->device);
    memset(g, 0, sizeof(*g));
    for (int i = 0; i < narrays; i++) {
        PS_TRY(check_array(arrays[i], "jit argument"));
        if (i && arrays[i].dtype != arrays[0].dtype) return fail(PS_ERR_DTYPE, "ps_jit_launch: mixed dtypes");
        g->a[i] = arrays[i].ptr;
        for (int d = 0; d < 3; d++) g->n[i][d] = arrays[i].n[d];
    }
    for (int i = 0; i < nscalars; i++) g->s[i] = scalars[i];
    for (int d = 0; d < 3; d++) {
        if (lo[d] < 0 || count[d] < 0) return fail(PS_ERR_ARG, "ps_jit_launch: negative range");
        g->lo[d] = lo[d];
        g->cnt[d] = count[d];
    }
    g->err = k->err;
    g->smem = shmem;
    g->loop = lp[0] * lp[1] * lp[2];  // the one loop count > 1, if any
    for (int d = 0; d < 3; d++)
        gd[d] = count[0] == 0 || count[1] == 0 || count[2] == 0
                    ? 0
                    : (count[d] + (int64_t)threads[d] * lp[d] - 1) / ((int64_t)threads[d] * lp[d]);
    if (shmem > k->smem_opt_in) {
        if (g_setattr(k->fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)shmem) != CUDA_SUCCESS)
            return fail(PS_ERR_ARG, "ps_jit_launch: %lld bytes of dynamic shared memory not available", (long long)shmem);
        k->smem_opt_in = (int)shmem;
    }
    *kout = k;
    return PS_OK;
}

// Reads (and clears) the kernel's error flags; the stream is idle.
static int jit_flags(JitKernel* k, const char* what) {
    int flag = 0;
    if (cudaMemcpy(&flag, k->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(PS_ERR_CUDA, "%s: reading the error flag failed", what);
    if (flag) {
        cudaMemset(k->err, 0, sizeof(int));
        if (flag & 1) return fail(PS_ERR_ARG, "%s: out-of-bounds array access in the kernel (BoundsError)", what);
        if (flag & 4)
            return fail(PS_ERR_UNSUPPORTED, "%s: a value outside the split FP64 arithmetic's range "
                                            "(|x| >= 2^128); run the kernel with fp64 = ieee", what);
        if (flag & 8)
            return fail(PS_ERR_TIMEOUT, "%s: a bounded wait for a staged plane gave up (the kernel stopped)", what);
        return fail(PS_ERR_ARG, "%s: a kernel with @sync_threads, shuffles or votes needs ranges that are "
                                "a multiple of the thread block; a partial block did not run", what);
    }
    return PS_OK;
}

// Argument block of a TMA-staged sweep kernel (ps_jit_launch_tma): the tensor maps of its staged
// arrays beside the ordinary block (identical layout in the generated source).
constexpr int kJitMaxMaps = 8;
struct alignas(64) ps_jit_targs {
    CUtensorMap tm[kJitMaxMaps];
    ps_jit_args g;
};

static int jit_cu_launch(JitKernel* k, unsigned gx, unsigned gy, unsigned gz, const int32_t threads[3], int64_t shmem,
                         void* g, void* stream) {
    void* params[] = {g};
    const CUresult r = g_launch(k->fn, gx, gy, gz, (unsigned)threads[0], (unsigned)threads[1], (unsigned)threads[2],
                                (unsigned)shmem, static_cast<CUstream>(stream), params, nullptr);
    if (r != CUDA_SUCCESS) return fail(PS_ERR_CUDA, "ps_jit_launch: cuLaunchKernel failed (CUresult %d)", (int)r);
    return PS_OK;
}

}  // namespace ps

extern "C" {

int ps_jit_launch_ex(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                     const int64_t lo[3], const int64_t count[3], const int32_t threads[3], int64_t shmem,
                     const int32_t loop[3], void* stream, int sync) {
    JitKernel* k = nullptr;
    ps_jit_args g;
    int64_t gd[3];
    int32_t lp[3];
    PS_TRY(jit_prepare(kernel, arrays, narrays, scalars, nscalars, lo, count, threads, shmem, loop, &k, &g, gd, lp));
    if (gd[0] == 0) return PS_OK;
    if (gd[0] > 2147483647LL || gd[1] > 65535 || gd[2] > 65535) return fail(PS_ERR_SHAPE, "ps_jit_launch: grid too large");
    PS_TRY(jit_cu_launch(k, (unsigned)gd[0], (unsigned)gd[1], (unsigned)gd[2], threads, shmem, &g, stream));
    PS_TRY(finish_launch(static_cast<cudaStream_t>(stream), sync, "ps_jit_launch"));
    if (!sync) return PS_OK;
    return jit_flags(k, "ps_jit_launch");  // flags of earlier asynchronous launches are reported too
}

int ps_jit_launch_tma(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                      const int64_t count[3], const int32_t threads[3], int64_t shmem, int32_t loop_z,
                      const int32_t* maps, int32_t nmaps, void* stream, int sync) {
    const int64_t lo[3] = {0, 0, 0};
    const int32_t loop[3] = {1, 1, loop_z};
    JitKernel* k = nullptr;
    ps_jit_targs t;
    int64_t gd[3];
    int32_t lp[3];
    PS_TRY(jit_prepare(kernel, arrays, narrays, scalars, nscalars, lo, count, threads, shmem, loop, &k, &t.g, gd, lp));
    if (nmaps < 0 || nmaps > kJitMaxMaps || (nmaps && !maps))
        return fail(PS_ERR_ARG, "ps_jit_launch_tma: at most %d staged arrays", kJitMaxMaps);
    memset(t.tm, 0, sizeof(t.tm));
    for (int i = 0; i < nmaps; i++) {
        const int32_t a = maps[3 * i], bx = maps[3 * i + 1], by = maps[3 * i + 2];
        if (a < 0 || a >= narrays || bx < 1 || by < 1)
            return fail(PS_ERR_ARG, "ps_jit_launch_tma: staged array %d: index %d, box (%d, %d)", i, a, bx, by);
        PS_TRY(encode_plane_map(&t.tm[i], arrays[a], (uint32_t)bx, (uint32_t)by));
    }
    if (gd[0] == 0) return PS_OK;
    if (gd[0] > 2147483647LL || gd[1] > 65535 || gd[2] > 65535)
        return fail(PS_ERR_SHAPE, "ps_jit_launch_tma: grid too large");
    PS_TRY(jit_cu_launch(k, (unsigned)gd[0], (unsigned)gd[1], (unsigned)gd[2], threads, shmem, &t, stream));
    PS_TRY(finish_launch(static_cast<cudaStream_t>(stream), sync, "ps_jit_launch_tma"));
    if (!sync) return PS_OK;
    return jit_flags(k, "ps_jit_launch_tma");
}

int ps_jit_hide_communication(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars,
                              int32_t nscalars, const int64_t count[3], const int32_t threads[3], const int32_t loop[3],
                              const int64_t bw[3], ps_comm_fn comm, void* comm_ctx, void* stream) {
    const int64_t lo[3] = {0, 0, 0};
    JitKernel* k = nullptr;
    ps_jit_args g;
    int64_t gd[3];
    int32_t lp[3];
    PS_TRY(jit_prepare(kernel, arrays, narrays, scalars, nscalars, lo, count, threads, 0, loop, &k, &g, gd, lp));
    if (!bw) return fail(PS_ERR_NULL, "ps_jit_hide_communication: NULL boundary width");
    if ((int64_t)threads[0] * threads[1] * threads[2] > 256)
        return fail(PS_ERR_ARG, "ps_jit_hide_communication: blocks of at most 256 threads");
    for (int d = 0; d < 3; d++) {  // validate_ranges_args (src/ParallelKernel/hide_communication.jl:396-403)
        if (bw[d] < 0) return fail(PS_ERR_ARG, "boundary width must be >= 0");
        if (!(count[d] > 2 * bw[d]))
            return fail(PS_ERR_SHAPE, "@hide_communication: length(ranges) > 2*boundary_width violated");
        if (count[d] > 1 && bw[d] == 0)
            return fail(PS_ERR_SHAPE, "@hide_communication: boundary_width 0 in a dimension of length > 1");
    }
    if (gd[0] == 0) return PS_OK;
    if (gd[0] * gd[1] * gd[2] > 2147483647LL) return fail(PS_ERR_SHAPE, "ps_jit_hide_communication: grid too large");
    volatile unsigned* hc = nullptr;
    unsigned* dc = nullptr;
    PS_TRY(progress_word(&hc, &dc));
    if (!dc) return fail(PS_ERR_UNSUPPORTED, "ps_jit_hide_communication: no host-mapped memory on this device");
    // tiles: thread blocks (times the sweep length); boundary: thread indices t < bw or t >= count - bw,
    // the reference's ranges_outer (src/ParallelKernel/hide_communication.jl:350-394)
    const int64_t tl[3] = {(int64_t)threads[0] * lp[0], (int64_t)threads[1] * lp[1], (int64_t)threads[2] * lp[2]};
    const int64_t end[3] = {count[0], count[1], count[2]}, hi[3] = {count[0] - bw[0], count[1] - bw[1], count[2] - bw[2]};
    const TileOrder o = make_tile_order(gd, lo, tl, end, bw, hi, dc);
    g.ocnt = dc;
    const int ov[10] = {o.TX, o.TY, o.TZ, o.bx0, o.bx1, o.by0, o.by1, o.bz0, o.bz1, o.nb};
    memcpy(g.ord, ov, sizeof(ov));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned need = (unsigned)o.nb;  // each boundary block counts itself once
    *hc = 0u;
    PS_TRY(jit_cu_launch(k, (unsigned)(gd[0] * gd[1] * gd[2]), 1, 1, threads, 0, &g, stream));
    PS_TRY(finish_launch(s, 0, "ps_jit_hide_communication"));
    const auto t0 = std::chrono::steady_clock::now();
    for (unsigned spin = 1; *hc < need; ++spin) {
        if (spin % 256 == 0) {
            cudaError_t q = cudaStreamQuery(s);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return cuda_fail(q, "ps_jit_hide_communication");
            if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60)) {
                PS_CUDA_TRY(cudaStreamSynchronize(s));
                break;
            }
        }
    }
    const bool boundary_done = *hc >= need;
    int crc = PS_OK;
    if (comm && boundary_done) crc = comm(comm_ctx);
    PS_TRY(finish_launch(s, 1, "ps_jit_hide_communication(sync)"));
    PS_TRY(jit_flags(k, "ps_jit_hide_communication"));
    if (!boundary_done) return fail(PS_ERR_TIMEOUT, "ps_jit_hide_communication: boundary blocks not reported done");
    if (crc != PS_OK) return fail(crc, "ps_jit_hide_communication: communication callback returned %d", crc);
    return PS_OK;
}

int ps_jit_check(void* kernel, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    if (!kernel) return fail(PS_ERR_NULL, "ps_jit_check: NULL kernel");
    JitKernel* k = static_cast<JitKernel*>(kernel);
    PS_TRY(finish_launch(static_cast<cudaStream_t>(stream), 1, "ps_jit_check"));
    return jit_flags(k, "ps_jit_check");
}

int ps_jit_destroy(void* kernel) {
    if (!kernel) return PS_OK;
    JitKernel* k = static_cast<JitKernel*>(kernel);
    if (k->mod && g_unload) g_unload(k->mod);
    if (k->err) cudaFree(k->err);
    delete k;
    return PS_OK;
}

}  // extern "C"
