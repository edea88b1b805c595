// ps_stencil3d.cu -- FD operators, memcopy3D and diffusion3D kernels of libps_b200.so.
//
// Kernels:
//   fd_sweep_kernel      one-statement `@parallel` kernels of every 3-D and 2-D FiniteDifferences
//                        macro (src/FiniteDifferences.jl:160-185, 328-394): z sweeps with a register
//                        window of the planes the macro reads (2-D: the same over (nx, 1, ny))
//   fd_apply_kernel      the same for 1-D macros (src/FiniteDifferences.jl:54-61), FD_ZB points
//                        per thread
//   memcopy_flat/_box    `@all(T2) = @all(T) + @all(Ci)` (examples/memcopy3D.jl:10-13)
//   diff3d_plain         diffusion step, one thread per cell (`memopt=false`, and boxes under half
//                        a sweep tile, e.g. @hide_communication's thin boundary slabs)
//   diff3d_zsweep_tma    diffusion step, z-sweep with TMA-staged x-y planes in a shared-memory
//                        ring and register-rotated z neighbours (`memopt=true`; the reference's
//                        memopt codegen is src/memopt.jl:190-573)
//   diff3d_zsweep_smem   the same sweep with thread-loaded planes, for arrays whose extents break
//                        TMA's 16-byte stride rule (odd nx, e.g. the reference's 31/33/127 sizes)
// All arithmetic is compiled without FMA contraction (--fmad=false) in the macros' operation
// order, so FP64 results are bit-identical to the reference's CPU path.
#include <algorithm>

#include <chrono>

#include "ps_common.cuh"

namespace ps {

// =======================================================================================
// Fill
// =======================================================================================
template <typename T>
__global__ void fill_kernel(T* __restrict__ a, int64_t n, T v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

// =======================================================================================
// Generic FD operator kernel
// =======================================================================================
struct FdDesc {
    int kind, opdims, inn, ndims, lhs_inn;
    int64_t nR[3], nA[3], tmax[3];
};

// The operator of one macro, specialised at compile time on its kind and operated dimensions
// (src/FiniteDifferences.jl: index patterns and operation orders), so the corners unroll into
// register-indexed loads and the averaging weights are literals.
__host__ __device__ constexpr int fd_dim(int opd, int j) {  // the j-th operated dimension
    int n = 0;
    for (int k = 0; k < 3; k++)
        if ((opd >> k) & 1) {
            if (n == j) return k;
            n++;
        }
    return 0;
}
__host__ __device__ constexpr int fd_popc(int opd) { return (opd & 1) + ((opd >> 1) & 1) + ((opd >> 2) & 1); }

// The macro's value from an accessor at(ox, oy, oz) of A relative to the point (offsets are
// compile-time constants once the loops unroll).
// RCP_DONE: at() already gives the reciprocals of a harmonic mean's corners.
template <typename T, int KIND, int OPD, bool RCP_DONE = false, class F>
__device__ __forceinline__ T fd_eval_f(F at) {
    if constexpr (KIND == PS_FD_SEL) {
        return at(0, 0, 0);
    } else if constexpr (KIND == PS_FD_DIFF) {
        constexpr int k = fd_dim(OPD, 0);
        return at(k == 0, k == 1, k == 2) - at(0, 0, 0);
    } else if constexpr (KIND == PS_FD_DIFF2) {
        constexpr int k = fd_dim(OPD, 0);
        const T m = at(0, 0, 0);
        return (at(k == 0, k == 1, k == 2) - m) - (m - at(-(k == 0), -(k == 1), -(k == 2)));
    } else if constexpr (KIND == PS_FD_AV || KIND == PS_FD_HARM) {
        constexpr int ND = fd_popc(OPD), NC = 1 << ND;
        T s = T(0);
#pragma unroll
        for (int cc = 0; cc < NC; cc++) {  // first operated dimension fastest, as the macros list them
            int o[3] = {0, 0, 0};
#pragma unroll
            for (int j = 0; j < ND; j++) o[fd_dim(OPD, j)] = (cc >> j) & 1;
            T v = at(o[0], o[1], o[2]);
            if constexpr (KIND == PS_FD_HARM && !RCP_DONE) v = T(1.0) / v;
            s = cc == 0 ? v : s + v;
        }
        if constexpr (KIND == PS_FD_AV) return s * T(1.0 / NC);  // 0.5, 0.25, 0.125: exact literals
        else return (T(1.0) / s) * T(NC);
    } else {  // maxloc / minloc; OPD = ndims, or 5: a 2-D macro laid out as (nx, 1, ny) (y as z)
        constexpr bool MX = KIND == PS_FD_MAXLOC;
        const auto f = [](T a, T b) { return MX ? jl_max(a, b) : jl_min(a, b); };
        T m = f(f(at(-1, 0, 0), at(1, 0, 0)), at(0, 0, 0));
        if constexpr (OPD == 5) {
            m = f(m, f(at(0, 0, -1), at(0, 0, 1)));
        } else {
#pragma unroll
            for (int k = 1; k < OPD; k++) m = f(m, f(at(0, -(k == 1), -(k == 2)), at(0, k == 1, k == 2)));
        }
        return m;
    }
}

// z offsets the macro reads (3-D): [fd_zlo, fd_zhi]; a window of zhi - zlo + 1 planes when > 1.
template <int KIND, int OPD>
__host__ __device__ constexpr int fd_zlo() {
    return ((KIND == PS_FD_DIFF2 && OPD == 4) || ((KIND == PS_FD_MAXLOC || KIND == PS_FD_MINLOC) && (OPD == 3 || OPD == 5)))
               ? -1 : 0;
}
template <int KIND, int OPD>
__host__ __device__ constexpr int fd_zhi() {
    return ((KIND == PS_FD_DIFF || KIND == PS_FD_DIFF2 || KIND == PS_FD_AV || KIND == PS_FD_HARM) && (OPD & 4)) ||
                   ((KIND == PS_FD_MAXLOC || KIND == PS_FD_MINLOC) && (OPD == 3 || OPD == 5))
               ? 1 : 0;
}
// Whether the macro reads the point (ox, oy) of some plane (offsets -1..1).
template <int KIND, int OPD>
__host__ __device__ constexpr bool fd_reads_xy(int ox, int oy) {
    if (KIND == PS_FD_SEL) return ox == 0 && oy == 0;
    if (KIND == PS_FD_DIFF || KIND == PS_FD_AV || KIND == PS_FD_HARM)
        return ox >= 0 && oy >= 0 && (ox == 0 || (OPD & 1)) && (oy == 0 || (OPD & 2));
    if (KIND == PS_FD_DIFF2) return (ox == 0 || OPD == 1) && (oy == 0 || OPD == 2);
    return OPD == 5 ? oy == 0 : (ox == 0 || oy == 0);  // maxloc / minloc: the cross
}

// Each thread evaluates FD_ZB consecutive z indices, their loads issued together (with one value
// per thread in flight a one-point-per-thread kernel keeps too few bytes in flight for HBM).
constexpr int FD_ZB = 4;

template <typename T, int KIND, int OPD>
__global__ void fd_apply_kernel(T* __restrict__ R, const T* __restrict__ A, FdDesc d) {
    const int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx >= d.tmax[0] || ty >= d.tmax[1]) return;
    const int64_t st[3] = {1, d.nA[0], d.nA[0] * d.nA[1]};
    const int64_t bx = tx + (d.inn & 1), by = ty + ((d.inn >> 1) & 1), dz = (d.inn >> 2) & 1;
    const int64_t rx = tx + (d.lhs_inn & 1), ry = ty + ((d.lhs_inn >> 1) & 1), rz0 = (d.lhs_inn >> 2) & 1;
    const int64_t rs = d.nR[0] * d.nR[1];
    for (int64_t z0 = (int64_t)blockIdx.z * FD_ZB; z0 < d.tmax[2]; z0 += (int64_t)gridDim.z * FD_ZB) {
        T v[FD_ZB];
#pragma unroll
        for (int u = 0; u < FD_ZB; u++)
            if (z0 + u < d.tmax[2]) {
                const T* p = A + bx + st[1] * by + st[2] * (z0 + u + dz);
                v[u] = fd_eval_f<T, KIND, OPD>([&](int ox, int oy, int oz) { return __ldg(p + ox + st[1] * oy + st[2] * oz); });
            }
#pragma unroll
        for (int u = 0; u < FD_ZB; u++)
            if (z0 + u < d.tmax[2]) R[rx + d.nR[0] * ry + rs * (z0 + u + rz0)] = v[u];
    }
}

// 3-D macros: each thread sweeps `zl` consecutive z indices, keeping a window of the planes' points
// in registers, so every plane is loaded once per thread (4 loads per point instead of 8 for @av,
// 5 instead of 7 for @maxloc); the same values in the same operation order as fd_apply_kernel.
// Selections and differences (a few loads, little arithmetic) unroll the sweep 4 times to keep
// more loads in flight; averages and extrema keep the compiler's own unrolling (each measured
// fastest at 512^3 that way, against forced unrolling by 1, 2 and 4).
// Harmonic means keep reciprocals in the window: each plane's corners are inverted once when
// loaded and reused by the next z step. In FP64 (division bound), with x among the operated
// dimensions, a warp outputs FD_HX = 31 columns, lane 31 only loading, and takes the x + 1
// corners' reciprocals from the next lane (9 divisions per point -> 3 for @harm, 5 -> 3 for
// @harm_xya; same operations, same order: FP64 @harm_xya 315 -> 442 GB/s at 512^3). FP32 keeps
// 32 columns per warp: its rows would straddle cache lines for no gain (2886 -> 2205 GB/s).
constexpr int FD_HX = 31;
template <typename T, int KIND, int OPD>
__host__ __device__ constexpr bool fd_xshare() {
    return KIND == PS_FD_HARM && (OPD & 1) && sizeof(T) == 8;
}

template <typename T, int KIND, int OPD>
__global__ void fd_sweep_kernel(T* __restrict__ R, const T* __restrict__ A, FdDesc d, int64_t zl) {
    constexpr int ZLO = fd_zlo<KIND, OPD>(), ZN = fd_zhi<KIND, OPD>() - ZLO + 1;
    constexpr bool UNR4 = KIND == PS_FD_SEL || KIND == PS_FD_DIFF || KIND == PS_FD_DIFF2;
    constexpr bool HARM = KIND == PS_FD_HARM, XSH = fd_xshare<T, KIND, OPD>();
    // @d2_zi (and the 2-D @d2_yi, swept as z): (A[z+1] - A[z]) - (A[z] - A[z-1]); the step's first
    // difference is the next step's second one (same operands, same operation), so the sweep carries
    // it: 2 subtractions per point, not 3
    constexpr bool D2Z = KIND == PS_FD_DIFF2 && OPD == 4;
    const int lane = (int)(threadIdx.x & 31);
    const int64_t tx = XSH ? ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * FD_HX + lane
                           : blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    const int64_t z0 = (int64_t)blockIdx.z * zl;
    // XSH: warps leave whole (ty is the warp's own, blockDim.x being a multiple of 32); a lane past
    // the last column stays for the shuffles, loading column tmax[0] (the last point's x + 1 corner)
    // at most, and writes nothing
    if ((XSH ? tx - lane : tx) >= d.tmax[0] || ty >= d.tmax[1] || z0 >= d.tmax[2]) return;
    const bool out = !XSH || (lane < FD_HX && tx < d.tmax[0]);
    const bool ld = !XSH || tx <= d.tmax[0];
    const int64_t z1 = min(z0 + zl, d.tmax[2]);
    const int64_t s1 = d.nA[0], s2 = d.nA[0] * d.nA[1];
    const int64_t dz = (d.inn >> 2) & 1;
    const T* p = A + tx + (d.inn & 1) + s1 * (ty + ((d.inn >> 1) & 1));
    T* r = R + tx + (d.lhs_inn & 1) + d.nR[0] * (ty + ((d.lhs_inn >> 1) & 1));
    const int64_t rs = d.nR[0] * d.nR[1], rz0 = (d.lhs_inn >> 2) & 1;
    T W[ZN][9] = {};
    auto load_plane = [&](T* w, int64_t z) {  // the points of plane z + dz the macro reads
        const T* q = p + s2 * (z + dz);
#pragma unroll
        for (int oy = -1; oy <= 1; oy++)
#pragma unroll
            for (int ox = -1; ox <= 1; ox++)
                if (fd_reads_xy<KIND, OPD>(ox, oy) && !(XSH && ox == 1))
                    w[(oy + 1) * 3 + ox + 1] = ld ? __ldg(q + ox + s1 * oy) : T(1);
        if constexpr (HARM) {  // after all the plane's loads, so that they are in flight together
#pragma unroll
            for (int k = 0; k < 9; k++)
                if (fd_reads_xy<KIND, OPD>(k % 3 - 1, k / 3 - 1) && !(XSH && k % 3 == 2)) w[k] = T(1.0) / w[k];
        }
        if constexpr (XSH) {
#pragma unroll
            for (int oy = 0; oy <= 1; oy++)
                if (fd_reads_xy<KIND, OPD>(1, oy)) w[(oy + 1) * 3 + 2] = __shfl_down_sync(0xffffffffu, w[(oy + 1) * 3 + 1], 1);
        }
    };
#pragma unroll
    for (int k = 1; k < ZN; k++) load_plane(W[k], z0 + ZLO + k - 1);
    T d2_prev = T(0);  // D2Z: A[z] - A[z-1] of the coming step (planes z0 - 1 and z0 here)
    if constexpr (D2Z) d2_prev = W[2][4] - W[1][4];
#define PS_FD_SWEEP_STEP                                                                                 \
    {                                                                                                    \
        _Pragma("unroll") for (int k = 0; k + 1 < ZN; k++)                                               \
            _Pragma("unroll") for (int q = 0; q < 9; q++) W[k][q] = W[k + 1][q];                         \
        load_plane(W[ZN - 1], z + ZLO + ZN - 1);                                                         \
        T v_;                                                                                            \
        if constexpr (D2Z) {                                                                             \
            const T f_ = W[2][4] - W[1][4];                                                              \
            v_ = f_ - d2_prev;                                                                           \
            d2_prev = f_;                                                                                \
        } else {                                                                                         \
            v_ = fd_eval_f<T, KIND, OPD, HARM>(                                                          \
                [&](int ox, int oy, int oz) { return W[oz - ZLO][(oy + 1) * 3 + ox + 1]; });             \
        }                                                                                                \
        if (out) r[rs * (z + rz0)] = v_;                                                                 \
    }
    if constexpr (UNR4) {
#pragma unroll 4
        for (int64_t z = z0; z < z1; z++) PS_FD_SWEEP_STEP
    } else {
        for (int64_t z = z0; z < z1; z++) PS_FD_SWEEP_STEP  // the compiler's own unrolling
    }
#undef PS_FD_SWEEP_STEP
}

// Threads a GB300 holds at once (152 SMs x 2048): sweeps are shortened until a launch fills them.
constexpr int64_t kResidentThreads = 152 * 2048;

template <typename T, int K, int O>
static void fd_launch_one(const FdDesc& d, T* R, const T* A, cudaStream_t s) {
    // a 2-D macro arrives here as a 3-D one over (nx, 1, ny): rows of 128 threads sweep "z" (= y)
    const dim3 blk = d.tmax[1] == 1 ? dim3(128, 1, 1) : dim3(32, 8, 1);
    const unsigned gy = (unsigned)((d.tmax[1] + blk.y - 1) / blk.y);
    unsigned gx = (unsigned)((d.tmax[0] + blk.x - 1) / blk.x);
    if (d.ndims == 3) {  // every 3-D macro sweeps z; 1-D and 2-D ones keep fd_apply_kernel
        if (fd_xshare<T, K, O>()) {  // FD_HX output columns per warp
            const int64_t cols = (int64_t)FD_HX * (blk.x / 32);
            gx = (unsigned)((d.tmax[0] + cols - 1) / cols);
        }
        int64_t zl = 64;
        while (zl > 2 && d.tmax[0] * d.tmax[1] * ((d.tmax[2] + zl - 1) / zl) < kResidentThreads) zl /= 2;
        zl = std::max<int64_t>(zl, (d.tmax[2] + 65534) / 65535);
        fd_sweep_kernel<T, K, O><<<dim3(gx, gy, (unsigned)((d.tmax[2] + zl - 1) / zl)), blk, 0, s>>>(R, A, d, zl);
        return;
    }
    const unsigned gz = (unsigned)std::min<int64_t>((d.tmax[2] + FD_ZB - 1) / FD_ZB, 65535);
    fd_apply_kernel<T, K, O><<<dim3(gx, gy, gz), blk, 0, s>>>(R, A, d);
}

template <typename T>
static int launch_fd(const FdDesc& d, T* R, const T* A, cudaStream_t s) {
#define PS_FD_CASE(K, O) \
    case O: fd_launch_one<T, K, O>(d, R, A, s); return PS_OK;
#define PS_FD_ONE_DIM(K) switch (d.opdims) { PS_FD_CASE(K, 1) PS_FD_CASE(K, 2) PS_FD_CASE(K, 4) }
#define PS_FD_ANY_DIMS(K) \
    switch (d.opdims) { PS_FD_CASE(K, 1) PS_FD_CASE(K, 2) PS_FD_CASE(K, 3) PS_FD_CASE(K, 4) PS_FD_CASE(K, 5) \
                        PS_FD_CASE(K, 6) PS_FD_CASE(K, 7) }
#define PS_FD_NDIMS(K) \
    switch (d.ndims) { case 1: fd_launch_one<T, K, 1>(d, R, A, s); return PS_OK; \
                       case 2: fd_launch_one<T, K, 2>(d, R, A, s); return PS_OK; \
                       case 3: fd_launch_one<T, K, 3>(d, R, A, s); return PS_OK; }
    switch (d.kind) {
    case PS_FD_SEL: fd_launch_one<T, PS_FD_SEL, 0>(d, R, A, s); return PS_OK;
    case PS_FD_DIFF: PS_FD_ONE_DIM(PS_FD_DIFF) break;
    case PS_FD_DIFF2: PS_FD_ONE_DIM(PS_FD_DIFF2) break;
    case PS_FD_AV: PS_FD_ANY_DIMS(PS_FD_AV) break;
    case PS_FD_HARM: PS_FD_ANY_DIMS(PS_FD_HARM) break;
    case PS_FD_MAXLOC:
        if (d.opdims == 5) { fd_launch_one<T, PS_FD_MAXLOC, 5>(d, R, A, s); return PS_OK; }
        PS_FD_NDIMS(PS_FD_MAXLOC) break;
    case PS_FD_MINLOC:
        if (d.opdims == 5) { fd_launch_one<T, PS_FD_MINLOC, 5>(d, R, A, s); return PS_OK; }
        PS_FD_NDIMS(PS_FD_MINLOC) break;
    }
#undef PS_FD_CASE
#undef PS_FD_ONE_DIM
#undef PS_FD_ANY_DIMS
#undef PS_FD_NDIMS
    return fail(PS_ERR_ARG, "ps_fd_apply: unsupported operator (kind %d, dims %d)", d.kind, d.opdims);
}

// =======================================================================================
// memcopy3D
// =======================================================================================
template <typename T>
struct Vec;
template <>
struct Vec<double> {
    static constexpr int N = 2;
    using type = double2;
};
template <>
struct Vec<float> {
    static constexpr int N = 4;
    using type = float4;
};

template <typename T>
__device__ __forceinline__ typename Vec<T>::type vadd(typename Vec<T>::type a, typename Vec<T>::type b);
template <>
__device__ __forceinline__ double2 vadd<double>(double2 a, double2 b) {
    return make_double2(a.x + b.x, a.y + b.y);
}
template <>
__device__ __forceinline__ float4 vadd<float>(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// Flat streaming form over whole arrays (the full `@parallel` grid): 128-bit loads and
// stores, 4 independent vectors in flight per thread per iteration.
template <typename T>
__global__ void __launch_bounds__(256) memcopy_flat(T* __restrict__ T2, const T* __restrict__ Tin,
                                                    const T* __restrict__ Ci, int64_t n) {
    using V = typename Vec<T>::type;
    constexpr int VN = Vec<T>::N;
    constexpr int U = 4;
    const int64_t nv = n / VN;
    const V* a = reinterpret_cast<const V*>(Tin);
    const V* b = reinterpret_cast<const V*>(Ci);
    V* o = reinterpret_cast<V*>(T2);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < nv; i += U * stride) {
        V x[U], y[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            x[u] = __ldcs(a + i + u * stride);
            y[u] = __ldcs(b + i + u * stride);
        }
#pragma unroll
        for (int u = 0; u < U; u++) __stcs(o + i + u * stride, vadd<T>(x[u], y[u]));
    }
    for (; i < nv; i += stride) __stcs(o + i, vadd<T>(__ldcs(a + i), __ldcs(b + i)));
    // scalar tail
    int64_t t = nv * VN + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) T2[t] = Tin[t] + Ci[t];
}

template <typename T>
__global__ void memcopy_box(T* __restrict__ T2, const T* __restrict__ Tin, const T* __restrict__ Ci, int64_t nx,
                            int64_t ny, Box b) {
    int64_t x = b.lo[0] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t y = b.lo[1] + blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (x >= b.hi[0] || y >= b.hi[1]) return;
    for (int64_t z = b.lo[2] + blockIdx.z; z < b.hi[2]; z += gridDim.z) {
        int64_t i = x + nx * (y + ny * z);
        T2[i] = Tin[i] + Ci[i];
    }
}

// =======================================================================================
// diffusion3D
// =======================================================================================
template <typename T>
struct DiffParams {
    T lam, dt, hx, hy, hz;
    DivC<T> q[3];  // the divisors hx*hx, hy*hy, hz*hz of the `/dx^2` form
};

// One cell of the diffusion statement in form FORM (see ps_diffusion_form). Operation order
// follows the Julia expression exactly; negation is exact so (-a)*b == -(a*b).
template <typename T, int FORM>
__device__ __forceinline__ T diff_cell(const DiffParams<T>& p, T Tc, T Txm, T Txp, T Tym, T Typ, T Tzm, T Tzp, T ci,
                                       T lc, T lxm, T lxp, T lym, T lyp, T lzm, T lzp) {
    if constexpr (FORM == PS_DIFF_DIV || FORM == PS_DIFF_MUL) {
        T d2x = (Txp - Tc) - (Tc - Txm);
        T d2y = (Typ - Tc) - (Tc - Tym);
        T d2z = (Tzp - Tc) - (Tc - Tzm);
        T s;
        if constexpr (FORM == PS_DIFF_DIV)
            s = (div_c(d2x, p.q[0]) + div_c(d2y, p.q[1])) + div_c(d2z, p.q[2]);
        else
            s = (d2x * (p.hx * p.hx) + d2y * (p.hy * p.hy)) + d2z * (p.hz * p.hz);
        return Tc + p.dt * ((p.lam * ci) * s);
    } else {
        T kxp, kxm, kyp, kym, kzp, kzm;
        if constexpr (FORM == PS_DIFF_FLUX) {
            kxp = kxm = kyp = kym = kzp = kzm = p.lam;
        } else {
            kxp = (lc + lxp) * T(0.5);
            kxm = (lxm + lc) * T(0.5);
            kyp = (lc + lyp) * T(0.5);
            kym = (lym + lc) * T(0.5);
            kzp = (lc + lzp) * T(0.5);
            kzm = (lzm + lc) * T(0.5);
        }
        T qxp = ((-kxp) * (Txp - Tc)) * p.hx, qxm = ((-kxm) * (Tc - Txm)) * p.hx;
        T qyp = ((-kyp) * (Typ - Tc)) * p.hy, qym = ((-kym) * (Tc - Tym)) * p.hy;
        T qzp = ((-kzp) * (Tzp - Tc)) * p.hz, qzm = ((-kzm) * (Tc - Tzm)) * p.hz;
        T dTdt = ci * (((-(qxp - qxm)) * p.hx - (qyp - qym) * p.hy) - (qzp - qzm) * p.hz);
        return Tc + p.dt * dTdt;
    }
}

// The flux forms with face fluxes carried: a cell's x-face flux qxm is its left neighbour's qxp and
// its z-face flux qzm the qzp of the cell below -- the same operations on the same operands, so a
// sweep passes them on instead of recomputing them (bit-identical; about a fifth fewer operations
// per cell, which the FP64 pipe bounds). qx: in, qxm when xin; out, qxp. qz: in, qzm; out, qzp.
template <typename T, int FORM>
__device__ __forceinline__ T diff_cell_carry(const DiffParams<T>& p, T Tc, T Txm, T Txp, T Tym, T Typ, T Tzp, T ci,
                                             T lc, T lxm, T lxp, T lym, T lyp, T lzp, bool xin, T& qx, T& qz) {
    static_assert(FORM == PS_DIFF_FLUX || FORM == PS_DIFF_FLUX_LAM, "flux forms only");
    const bool L = FORM == PS_DIFF_FLUX_LAM;
    const T kxp = L ? (lc + lxp) * T(0.5) : p.lam, kyp = L ? (lc + lyp) * T(0.5) : p.lam;
    const T kym = L ? (lym + lc) * T(0.5) : p.lam, kzp = L ? (lc + lzp) * T(0.5) : p.lam;
    T qxm;
    if (xin) {
        qxm = qx;
    } else {
        const T kxm = L ? (lxm + lc) * T(0.5) : p.lam;
        qxm = ((-kxm) * (Tc - Txm)) * p.hx;
    }
    const T qxp = ((-kxp) * (Txp - Tc)) * p.hx;
    const T qyp = ((-kyp) * (Typ - Tc)) * p.hy, qym = ((-kym) * (Tc - Tym)) * p.hy;
    const T qzp = ((-kzp) * (Tzp - Tc)) * p.hz, qzm = qz;
    const T dTdt = ci * (((-(qxp - qxm)) * p.hx - (qyp - qym) * p.hy) - (qzp - qzm) * p.hz);
    qx = qxp;
    qz = qzp;
    return Tc + p.dt * dTdt;
}
// qzm of the first cell of a sweep (the carried value's start)
template <typename T, int FORM>
__device__ __forceinline__ T diff_qzm(const DiffParams<T>& p, T Tc, T Tzm, T lc, T lzm) {
    const T kzm = FORM == PS_DIFF_FLUX_LAM ? (lzm + lc) * T(0.5) : p.lam;
    return ((-kzm) * (Tc - Tzm)) * p.hz;
}

// --- plain: one thread per cell, (32, 8, 1) threads like the reference's default --------
template <typename T, int FORM>
__global__ void __launch_bounds__(256) diff3d_plain(T* __restrict__ T2, const T* __restrict__ Tin,
                                                    const T* __restrict__ Ci, const T* __restrict__ lam,
                                                    DiffParams<T> p, int64_t nx, int64_t ny, Box cb) {
    int64_t cx = cb.lo[0] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t cy = cb.lo[1] + blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (cx >= cb.hi[0] || cy >= cb.hi[1]) return;
    const int64_t sy = nx, sz = nx * ny;
    constexpr bool L = FORM == PS_DIFF_FLUX_LAM;
    for (int64_t cz = cb.lo[2] + blockIdx.z; cz < cb.hi[2]; cz += gridDim.z) {
        int64_t c = cx + sy * cy + sz * cz;
        T Tc = __ldg(Tin + c);
        T lc = L ? __ldg(lam + c) : T(0);
        T r = diff_cell<T, FORM>(p, Tc, __ldg(Tin + c - 1), __ldg(Tin + c + 1), __ldg(Tin + c - sy), __ldg(Tin + c + sy),
                                 __ldg(Tin + c - sz), __ldg(Tin + c + sz), __ldg(Ci + c), lc,
                                 L ? __ldg(lam + c - 1) : T(0), L ? __ldg(lam + c + 1) : T(0),
                                 L ? __ldg(lam + c - sy) : T(0), L ? __ldg(lam + c + sy) : T(0),
                                 L ? __ldg(lam + c - sz) : T(0), L ? __ldg(lam + c + sz) : T(0));
        T2[c] = r;
    }
}

// --- z-sweep with TMA-staged planes -----------------------------------------------------
// A CTA owns a TX x TY column of cells and sweeps `L` planes in z. Plane z of T (and lam)
// is staged with its x-y halo by one TMA copy into slot (z mod S) of a shared-memory ring;
// an mbarrier per slot signals completion. Each thread keeps the z-1 / z / z+1 values of
// its VEC cells in registers (rotated every step) and reads x-y neighbours from the staged
// plane. Ci is staged without halo in the same slot. T2 is written with 128-bit stores.
template <typename T, int FORM, int TY, int S>
struct ZSweep {
    static constexpr int VEC = 16 / (int)sizeof(T);
    static constexpr int TX = 32 * VEC;
    static constexpr int H = VEC;  // x halo: keeps every TMA x coordinate 16-byte aligned
    static constexpr int PW = TX + 2 * H;
    static constexpr int PH = TY + 2;
    static constexpr bool HAS_LAM = FORM == PS_DIFF_FLUX_LAM;
    static constexpr int PLANE_BYTES = ((PW * PH * (int)sizeof(T) + 127) / 128) * 128;
    static constexpr int CI_BYTES = ((TX * TY * (int)sizeof(T) + 127) / 128) * 128;
    static constexpr int STAGE_BYTES = PLANE_BYTES * (HAS_LAM ? 2 : 1) + CI_BYTES;
    static constexpr uint32_t TX_BYTES =
        (uint32_t)(PW * PH * sizeof(T) * (HAS_LAM ? 2 : 1) + TX * TY * sizeof(T));
    static constexpr int SMEM = S * STAGE_BYTES + 8 * S;
};

template <typename T, int FORM, int TY, int S>
__global__ void __launch_bounds__(32 * TY) diff3d_zsweep_tma(const __grid_constant__ CUtensorMap mT,
                                                             const __grid_constant__ CUtensorMap mL,
                                                             const __grid_constant__ CUtensorMap mC,
                                                             T* __restrict__ T2, DiffParams<T> p, int64_t nx,
                                                             int64_t ny, Box cb, int L, int* __restrict__ err,
                                                             TileOrder ord) {
    using Z = ZSweep<T, FORM, TY, S>;
    constexpr int VEC = Z::VEC;
    using V = typename Vec<T>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + S * Z::STAGE_BYTES);

    const int lx = threadIdx.x, ly = threadIdx.y, tid = ly * 32 + lx;
    const uint3 tile = ordered_tile(ord);
    const int X0 = (int)(cb.lo[0] & ~(int64_t)(VEC - 1)) + (int)tile.x * Z::TX;
    const int Y0 = (int)cb.lo[1] + (int)tile.y * TY;
    const int Z0 = (int)cb.lo[2] + (int)tile.z * L;
    const int nk = min(L, (int)cb.hi[2] - Z0);
    const int nq = nk + 2;  // planes Z0-1 .. Z0+nk

    auto tplane = [&](int q) { return reinterpret_cast<T*>(smem + (q % S) * Z::STAGE_BYTES); };
    auto lplane = [&](int q) { return reinterpret_cast<T*>(smem + (q % S) * Z::STAGE_BYTES + Z::PLANE_BYTES); };
    auto cplane = [&](int q) {
        return reinterpret_cast<T*>(smem + (q % S) * Z::STAGE_BYTES + Z::PLANE_BYTES * (Z::HAS_LAM ? 2 : 1));
    };

    if (tid == 0) {
        prefetch_tensormap(&mT);
        if constexpr (Z::HAS_LAM) prefetch_tensormap(&mL);
        prefetch_tensormap(&mC);
        for (int s = 0; s < S; s++) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();

    int next_q = 0;
    auto issue = [&](int q) {
        int s = q % S, z = Z0 - 1 + q;
        mbar_arrive_expect_tx(&bar[s], Z::TX_BYTES);
        tma_load_3d(tplane(q), &mT, &bar[s], X0 - Z::H, Y0 - 1, z);
        if constexpr (Z::HAS_LAM) tma_load_3d(lplane(q), &mL, &bar[s], X0 - Z::H, Y0 - 1, z);
        tma_load_3d(cplane(q), &mC, &bar[s], X0, Y0, z);
    };
    if (tid == 0)
        for (; next_q < min(S, nq); ++next_q) issue(next_q);

    const int px = Z::H + lx * VEC;  // staged-plane column of this thread's first cell
    const int py = 1 + ly;
    const int64_t gx = X0 + lx * VEC, gy = Y0 + ly;
    const bool row_in = gy >= cb.lo[1] && gy < cb.hi[1];
    bool full_vec = row_in && gx >= cb.lo[0] && gx + VEC <= cb.hi[0];

    T Tzm[VEC], Tc[VEC], Tzp[VEC], lzm[VEC], lc[VEC], lzp[VEC];
    constexpr bool CARRY = FORM == PS_DIFF_FLUX || FORM == PS_DIFF_FLUX_LAM;
    T qzc[VEC];  // CARRY: each cell's qzm, the qzp of the cell below
    bool timed_out = false;
    timed_out |= !mbar_wait_bounded(&bar[0], 0);
    timed_out |= !mbar_wait_bounded(&bar[1 % S], (1 / S) & 1);
    if (!timed_out) {
        const V a = *reinterpret_cast<const V*>(tplane(0) + py * Z::PW + px);
        const V b = *reinterpret_cast<const V*>(tplane(1) + py * Z::PW + px);
        const T* av = reinterpret_cast<const T*>(&a);
        const T* bv = reinterpret_cast<const T*>(&b);
#pragma unroll
        for (int j = 0; j < VEC; j++) {
            Tzm[j] = av[j];
            Tc[j] = bv[j];
        }
        if constexpr (Z::HAS_LAM) {
            const V la = *reinterpret_cast<const V*>(lplane(0) + py * Z::PW + px);
            const V lb = *reinterpret_cast<const V*>(lplane(1) + py * Z::PW + px);
            const T* lav = reinterpret_cast<const T*>(&la);
            const T* lbv = reinterpret_cast<const T*>(&lb);
#pragma unroll
            for (int j = 0; j < VEC; j++) {
                lzm[j] = lav[j];
                lc[j] = lbv[j];
            }
        }
        if constexpr (CARRY) {
#pragma unroll
            for (int j = 0; j < VEC; j++) qzc[j] = diff_qzm<T, FORM>(p, Tc[j], Tzm[j], Z::HAS_LAM ? lc[j] : T(0),
                                                                   Z::HAS_LAM ? lzm[j] : T(0));
        }
    }

    for (int k = 0; k < nk; ++k) {
        const int q = k + 2;
        timed_out |= !mbar_wait_bounded(&bar[q % S], (q / S) & 1);
        if (!timed_out) {
            const T* tp = tplane(k + 1);
            {
                const V zp = *reinterpret_cast<const V*>(tplane(q) + py * Z::PW + px);
                const T* zv = reinterpret_cast<const T*>(&zp);
#pragma unroll
                for (int j = 0; j < VEC; j++) Tzp[j] = zv[j];
            }
            const V ym = *reinterpret_cast<const V*>(tp + (py - 1) * Z::PW + px);
            const V yp = *reinterpret_cast<const V*>(tp + (py + 1) * Z::PW + px);
            const T xm = tp[py * Z::PW + px - 1];
            const T xp = tp[py * Z::PW + px + VEC];
            const V cv = *reinterpret_cast<const V*>(cplane(k + 1) + ly * Z::TX + lx * VEC);
            const T* ymv = reinterpret_cast<const T*>(&ym);
            const T* ypv = reinterpret_cast<const T*>(&yp);
            const T* civ = reinterpret_cast<const T*>(&cv);
            T lym_[VEC], lyp_[VEC], lxm = T(0), lxp = T(0);
            if constexpr (Z::HAS_LAM) {
                const T* lp = lplane(k + 1);
                const V zp = *reinterpret_cast<const V*>(lplane(q) + py * Z::PW + px);
                const T* zv = reinterpret_cast<const T*>(&zp);
                const V a = *reinterpret_cast<const V*>(lp + (py - 1) * Z::PW + px);
                const V b = *reinterpret_cast<const V*>(lp + (py + 1) * Z::PW + px);
                const T* av = reinterpret_cast<const T*>(&a);
                const T* bv = reinterpret_cast<const T*>(&b);
#pragma unroll
                for (int j = 0; j < VEC; j++) {
                    lzp[j] = zv[j];
                    lym_[j] = av[j];
                    lyp_[j] = bv[j];
                }
                lxm = lp[py * Z::PW + px - 1];
                lxp = lp[py * Z::PW + px + VEC];
            } else {
#pragma unroll
                for (int j = 0; j < VEC; j++) lym_[j] = lyp_[j] = lzp[j] = lc[j] = lzm[j] = T(0);
            }
            T out[VEC];
            T qxc = T(0);  // CARRY: the previous cell's qxp
#pragma unroll
            for (int j = 0; j < VEC; j++) {
                T txm = j == 0 ? xm : Tc[j - 1];
                T txp = j == VEC - 1 ? xp : Tc[j + 1];
                T lxm_j = j == 0 ? lxm : lc[j - 1];
                T lxp_j = j == VEC - 1 ? lxp : lc[j + 1];
                if constexpr (CARRY)
                    out[j] = diff_cell_carry<T, FORM>(p, Tc[j], txm, txp, ymv[j], ypv[j], Tzp[j], civ[j], lc[j], lxm_j,
                                                      lxp_j, lym_[j], lyp_[j], lzp[j], j > 0, qxc, qzc[j]);
                else
                    out[j] = diff_cell<T, FORM>(p, Tc[j], txm, txp, ymv[j], ypv[j], Tzm[j], Tzp[j], civ[j], lc[j],
                                                lxm_j, lxp_j, lym_[j], lyp_[j], lzm[j], lzp[j]);
            }
            const int64_t gz = Z0 + k;
            T* dst = T2 + gx + nx * (gy + ny * gz);
            if (full_vec) {
                V o;
                T* ov = reinterpret_cast<T*>(&o);
#pragma unroll
                for (int j = 0; j < VEC; j++) ov[j] = out[j];
                *reinterpret_cast<V*>(dst) = o;
            } else if (row_in) {
#pragma unroll
                for (int j = 0; j < VEC; j++)
                    if (gx + j >= cb.lo[0] && gx + j < cb.hi[0]) dst[j] = out[j];
            }
#pragma unroll
            for (int j = 0; j < VEC; j++) {
                Tzm[j] = Tc[j];
                Tc[j] = Tzp[j];
                if constexpr (Z::HAS_LAM) {
                    lzm[j] = lc[j];
                    lc[j] = lzp[j];
                }
            }
        }
        // Every thread is done with plane k+1: its slot may be refilled.
        if (__syncthreads_or(timed_out)) {
            if (tid == 0) {
                atomicOr(err, DEV_ERR_TMA_TIMEOUT);
                for (int r = q + 1; r < next_q; ++r) mbar_wait_bounded(&bar[r % S], (r / S) & 1);
            }
            return;
        }
        if (tid == 0)
            for (; next_q < min(nq, k + 2 + S); ++next_q) issue(next_q);
    }
    ordered_tile_done(ord);
}

// --- z-sweep with thread-loaded planes (fallback for non-TMA-eligible arrays) ----------
// The reference's memopt structure: per z step, the x-y halo plane of T (and lam) is loaded
// into shared memory between two barriers; z neighbours rotate through registers.
template <typename T, int FORM, int TY>
__global__ void __launch_bounds__(32 * TY) diff3d_zsweep_smem(T* __restrict__ T2, const T* __restrict__ Tin,
                                                              const T* __restrict__ Ci, const T* __restrict__ lam,
                                                              DiffParams<T> p, int64_t nx, int64_t ny, int64_t nz,
                                                              Box cb, int L) {
    constexpr bool HAS_LAM = FORM == PS_DIFF_FLUX_LAM;
    constexpr int PW = 32 + 2, PH = TY + 2;
    __shared__ T sT[PH][PW];
    __shared__ T sL[HAS_LAM ? PH : 1][HAS_LAM ? PW : 1];
    const int lx = threadIdx.x, ly = threadIdx.y, tid = ly * 32 + lx;
    const int64_t X0 = cb.lo[0] + blockIdx.x * 32, Y0 = cb.lo[1] + blockIdx.y * TY;
    const int64_t Z0 = cb.lo[2] + blockIdx.z * (int64_t)L;
    const int64_t Z1 = min(Z0 + L, cb.hi[2]);
    const int64_t gx = X0 + lx, gy = Y0 + ly;
    const bool active = gx < cb.hi[0] && gy < cb.hi[1];
    const int64_t sy = nx, sz = nx * ny;
    auto ld = [&](const T* A, int64_t x, int64_t y, int64_t z) -> T {
        return (x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz) ? __ldg(A + x + sy * y + sz * z) : T(0);
    };
    T Tzm = active ? ld(Tin, gx, gy, Z0 - 1) : T(0), Tc = active ? ld(Tin, gx, gy, Z0) : T(0), Tzp;
    T lzm = (HAS_LAM && active) ? ld(lam, gx, gy, Z0 - 1) : T(0), lc = (HAS_LAM && active) ? ld(lam, gx, gy, Z0) : T(0),
      lzp = T(0);
    for (int64_t z = Z0; z < Z1; ++z) {
        __syncthreads();
        for (int i = tid; i < PW * PH; i += 32 * TY) {
            int hx = i % PW, hy = i / PW;
            sT[hy][hx] = ld(Tin, X0 - 1 + hx, Y0 - 1 + hy, z);
            if constexpr (HAS_LAM) sL[hy][hx] = ld(lam, X0 - 1 + hx, Y0 - 1 + hy, z);
        }
        __syncthreads();
        Tzp = active ? ld(Tin, gx, gy, z + 1) : T(0);
        if constexpr (HAS_LAM) lzp = active ? ld(lam, gx, gy, z + 1) : T(0);
        if (active) {
            const int sx = lx + 1, sy_ = ly + 1;
            T r = diff_cell<T, FORM>(p, Tc, sT[sy_][sx - 1], sT[sy_][sx + 1], sT[sy_ - 1][sx], sT[sy_ + 1][sx], Tzm, Tzp,
                                     __ldg(Ci + gx + sy * gy + sz * z), lc, HAS_LAM ? sL[sy_][sx - 1] : T(0),
                                     HAS_LAM ? sL[sy_][sx + 1] : T(0), HAS_LAM ? sL[sy_ - 1][sx] : T(0),
                                     HAS_LAM ? sL[sy_ + 1][sx] : T(0), lzm, lzp);
            T2[gx + sy * gy + sz * z] = r;
        }
        Tzm = Tc;
        Tc = Tzp;
        lzm = lc;
        lc = lzp;
    }
}

// =======================================================================================
// acoustic3D (miniapps/acoustic3D.jl:11-21)
// =======================================================================================
template <typename T>
__global__ void acoustic_v_kernel(T* __restrict__ Vx, T* __restrict__ Vy, T* __restrict__ Vz, const T* __restrict__ P,
                                  int64_t nx, int64_t ny, int64_t nz, T dtr, DivC<T> dx, DivC<T> dy, DivC<T> dz) {
    // grid = (nx+1, ny+1, nz+1); each statement masked by @inn of its left-hand array.
    int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx > nx || ty > ny) return;
    const int64_t sy = nx, sz = nx * ny;
    for (int64_t tz = blockIdx.z; tz <= nz; tz += gridDim.z) {
        if (tx < nx - 1 && ty < ny - 2 && tz < nz - 2) {  // @inn(Vx): Vx is (nx+1, ny, nz)
            int64_t v = (tx + 1) + (nx + 1) * ((ty + 1) + ny * (tz + 1));
            int64_t pc = (tx + 1) + sy * (ty + 1) + sz * (tz + 1);
            Vx[v] = Vx[v] - div_c(dtr * (P[pc] - P[pc - 1]), dx);
        }
        if (tx < nx - 2 && ty < ny - 1 && tz < nz - 2) {  // @inn(Vy): Vy is (nx, ny+1, nz)
            int64_t v = (tx + 1) + nx * ((ty + 1) + (ny + 1) * (tz + 1));
            int64_t pc = (tx + 1) + sy * (ty + 1) + sz * (tz + 1);
            Vy[v] = Vy[v] - div_c(dtr * (P[pc] - P[pc - sy]), dy);
        }
        if (tx < nx - 2 && ty < ny - 2 && tz < nz - 1) {  // @inn(Vz): Vz is (nx, ny, nz+1)
            int64_t v = (tx + 1) + nx * ((ty + 1) + ny * (tz + 1));
            int64_t pc = (tx + 1) + sy * (ty + 1) + sz * (tz + 1);
            Vz[v] = Vz[v] - div_c(dtr * (P[pc] - P[pc - sz]), dz);
        }
    }
}

template <typename T>
__global__ void acoustic_p_kernel(T* __restrict__ P, const T* __restrict__ Vx, const T* __restrict__ Vy,
                                  const T* __restrict__ Vz, int64_t nx, int64_t ny, int64_t nz, T dtk, DivC<T> dx,
                                  DivC<T> dy, DivC<T> dz) {
    int64_t ix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t iy = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (ix >= nx || iy >= ny) return;
    for (int64_t iz = blockIdx.z; iz < nz; iz += gridDim.z) {
        T ax = Vx[(ix + 1) + (nx + 1) * (iy + ny * iz)] - Vx[ix + (nx + 1) * (iy + ny * iz)];
        T ay = Vy[ix + nx * ((iy + 1) + (ny + 1) * iz)] - Vy[ix + nx * (iy + (ny + 1) * iz)];
        T az = Vz[ix + nx * (iy + ny * (iz + 1))] - Vz[ix + nx * (iy + ny * iz)];
        int64_t pc = ix + nx * (iy + ny * iz);
        P[pc] = P[pc] - dtk * ((div_c(ax, dx) + div_c(ay, dy)) + div_c(az, dz));
    }
}

// =======================================================================================
// Host launchers
// =======================================================================================
static dim3 grid3(int64_t wx, int64_t wy, int64_t wz, dim3 blk) {
    return dim3((unsigned)((wx + blk.x - 1) / blk.x), (unsigned)((wy + blk.y - 1) / blk.y),
                (unsigned)std::min<int64_t>(std::max<int64_t>(wz, 1), 65535));
}

template <typename T>
static DiffParams<T> diff_params(double lam, double dt, double hx, double hy, double hz) {
    const T x = (T)hx, y = (T)hy, z = (T)hz;
    return DiffParams<T>{(T)lam, (T)dt, x, y, z, {make_div((T)(x * x)), make_div((T)(y * y)), make_div((T)(z * z))}};
}

int launch_diffusion_split(int form, const ps_array& T2, const ps_array& Tin, const ps_array& Ci, const ps_array* lam,
                           double lam_s, double dt, double hx, double hy, double hz, const Box& cb, int L,
                           cudaStream_t s, int* d_err, HideReq* hr = nullptr);

// z-sweep length (`loopsize`) of the shared-memory fallback when none is given: the reference
// uses 64 on compute capability >= 9 (src/parallel.jl:532-543). The TMA z-sweeps choose theirs
// from the wave count (auto_loopsize).
static constexpr int kDefaultLoopsize = 64;

template <typename T, int FORM, int TY, int S>
static int launch_zsweep_tma(const ps_array& T2, const ps_array& Tin, const ps_array& Ci, const ps_array* lam,
                             const DiffParams<T>& p, const Box& cb, int L, cudaStream_t s, int* d_err,
                             HideReq* hr = nullptr) {
    using Z = ZSweep<T, FORM, TY, S>;
    CUtensorMap mT, mL, mC;
    PS_TRY(encode_plane_map(&mT, Tin, Z::PW, Z::PH));
    if (Z::HAS_LAM)
        PS_TRY(encode_plane_map(&mL, *lam, Z::PW, Z::PH));
    else
        mL = mT;
    PS_TRY(encode_plane_map(&mC, Ci, Z::TX, TY));
    static bool attr_set = false;
    if (!attr_set) {
        PS_CUDA_TRY(cudaFuncSetAttribute(diff3d_zsweep_tma<T, FORM, TY, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Z::SMEM));
        attr_set = true;
    }
    int64_t x0 = cb.lo[0] & ~(int64_t)(Z::VEC - 1);
    dim3 blk(32, TY, 1);
    const int64_t bx = (cb.hi[0] - x0 + Z::TX - 1) / Z::TX, by = (cb.hi[1] - cb.lo[1] + TY - 1) / TY;
    if (L <= 0) {
        static const int occ = resident_ctas(diff3d_zsweep_tma<T, FORM, TY, S>, 32 * TY, Z::SMEM);
        DeviceState* st = nullptr;
        PS_TRY(current_state(&st));
        L = auto_loopsize(bx * by, cb.hi[2] - cb.lo[2], (int64_t)occ * st->num_sms);
    }
    const int64_t bz = (cb.hi[2] - cb.lo[2] + L - 1) / L;
    dim3 grd((unsigned)bx, (unsigned)by, (unsigned)bz);
    TileOrder ord{};
    if (hr) {  // boundary tiles first, as one 1-D grid
        const int64_t nt[3] = {bx, by, bz}, lo[3] = {x0, cb.lo[1], cb.lo[2]}, tl[3] = {Z::TX, TY, L};
        const int64_t end[3] = {cb.hi[0], cb.hi[1], cb.hi[2]};
        ord = make_tile_order(nt, lo, tl, end, hr->lo_end, hr->hi_start, hr->counter);
        hr->nb = ord.nb;
        grd = dim3((unsigned)(bx * by * bz), 1, 1);
    }
    diff3d_zsweep_tma<T, FORM, TY, S><<<grd, blk, Z::SMEM, s>>>(mT, mL, mC, static_cast<T*>(T2.ptr), p, T2.n[0],
                                                                T2.n[1], cb, L, d_err, ord);
    return PS_OK;
}

template <typename T, int FORM>
static int launch_diffusion(const ps_array& T2, const ps_array& Tin, const ps_array& Ci, const ps_array* lam,
                            const DiffParams<T>& p, const Box& cb, int memopt, int loopsize, cudaStream_t s,
                            int* d_err, HideReq* hr = nullptr) {
    const int64_t wx = cb.hi[0] - cb.lo[0], wy = cb.hi[1] - cb.lo[1], wz = cb.hi[2] - cb.lo[2];
    if (wx <= 0 || wy <= 0 || wz <= 0) return hr ? PS_ERR_UNSUPPORTED : PS_OK;
    if (hr) {  // boundary-first launches exist for the TMA z-sweep only
        const bool tma = tma_eligible(T2) && tma_eligible(Tin) && tma_eligible(Ci) && (!lam || tma_eligible(*lam));
        if (!memopt || !tma) return PS_ERR_UNSUPPORTED;
        return launch_zsweep_tma<T, FORM, 8, 4>(T2, Tin, Ci, lam, p, cb, loopsize, s, d_err, hr);
    }
    const T* lp = lam ? static_cast<const T*>(lam->ptr) : nullptr;
    int L = loopsize > 0 ? loopsize : kDefaultLoopsize;
    // A box under half a z-sweep tile wide (x) or high (y) -- e.g. 16-cell boundary slabs of
    // @hide_communication -- would leave most of each tile's threads idle; those run one point per
    // thread instead, in blocks no wider than the box (same results: every kernel here is
    // bit-identical).
    constexpr int64_t kSweepTileX = 32 * (16 / (int64_t)sizeof(T));
    if (memopt && 2 * wx >= kSweepTileX && wy >= 4) {
        bool tma = tma_eligible(T2) && tma_eligible(Tin) && tma_eligible(Ci) && (!lam || tma_eligible(*lam));
        if (tma) return launch_zsweep_tma<T, FORM, 8, 4>(T2, Tin, Ci, lam, p, cb, loopsize, s, d_err);
        dim3 blk(32, 4, 1);
        dim3 grd((unsigned)((wx + 31) / 32), (unsigned)((wy + 3) / 4), (unsigned)((wz + L - 1) / L));
        diff3d_zsweep_smem<T, FORM, 4><<<grd, blk, 0, s>>>(static_cast<T*>(T2.ptr), static_cast<const T*>(Tin.ptr),
                                                            static_cast<const T*>(Ci.ptr), lp, p, T2.n[0], T2.n[1],
                                                            T2.n[2], cb, L);
        return PS_OK;
    }
    unsigned bxw = 32;  // full warps for boxes narrower than 32 in x: a warp spans several y rows
    while (bxw > 1 && bxw / 2 >= wx) bxw /= 2;
    dim3 blk(bxw, 256 / bxw, 1);
    diff3d_plain<T, FORM><<<grid3(wx, wy, wz, blk), blk, 0, s>>>(static_cast<T*>(T2.ptr),
                                                                 static_cast<const T*>(Tin.ptr),
                                                                 static_cast<const T*>(Ci.ptr), lp, p, T2.n[0],
                                                                 T2.n[1], cb);
    return PS_OK;
}

template <typename T>
static int dispatch_diffusion(int form, const ps_array& T2, const ps_array& Tin, const ps_array& Ci,
                              const ps_array* lam, double lam_s, double dt, double hx, double hy, double hz,
                              const Box& cb, int memopt, int loopsize, cudaStream_t s, int* d_err,
                              HideReq* hr = nullptr) {
    DiffParams<T> p = diff_params<T>(lam_s, dt, hx, hy, hz);
    switch (form) {
    case PS_DIFF_DIV:
        return launch_diffusion<T, PS_DIFF_DIV>(T2, Tin, Ci, nullptr, p, cb, memopt, loopsize, s, d_err, hr);
    case PS_DIFF_MUL:
        return launch_diffusion<T, PS_DIFF_MUL>(T2, Tin, Ci, nullptr, p, cb, memopt, loopsize, s, d_err, hr);
    case PS_DIFF_FLUX:
        return launch_diffusion<T, PS_DIFF_FLUX>(T2, Tin, Ci, nullptr, p, cb, memopt, loopsize, s, d_err, hr);
    case PS_DIFF_FLUX_LAM:
        return launch_diffusion<T, PS_DIFF_FLUX_LAM>(T2, Tin, Ci, lam, p, cb, memopt, loopsize, s, d_err, hr);
    }
    return fail(PS_ERR_ARG, "ps_diffusion3d_step: unknown form %d", form);
}

// Validates the diffusion arguments and converts the thread box into the box of written
// cells (`@inn(T2)` mask: c = t + 1 for 0 <= t < n - 2).
int diffusion_args(int32_t form, const ps_array& T2, const ps_array& Tin, const ps_array& Ci,
                          const ps_array& lam) {
    PS_TRY(check_array(T2, "T2"));
    PS_TRY(check_array(Tin, "T"));
    PS_TRY(check_array(Ci, "Ci"));
    PS_TRY(check_same_dtype(T2, Tin, "T2", "T"));
    PS_TRY(check_same_dtype(T2, Ci, "T2", "Ci"));
    PS_TRY(check_shape(Tin, T2.n[0], T2.n[1], T2.n[2], "T"));
    PS_TRY(check_shape(Ci, T2.n[0], T2.n[1], T2.n[2], "Ci"));
    if (form < 0 || form > 3) return fail(PS_ERR_ARG, "diffusion: unknown form %d", form);
    if (form == PS_DIFF_FLUX_LAM) {
        PS_TRY(check_array(lam, "lam"));
        PS_TRY(check_same_dtype(T2, lam, "T2", "lam"));
        PS_TRY(check_shape(lam, T2.n[0], T2.n[1], T2.n[2], "lam"));
    }
    if (T2.ptr == Tin.ptr) return fail(PS_ERR_ARG, "diffusion: T2 and T must be distinct arrays");
    return PS_OK;
}

static Box inner_cells(const Box& tb, const int64_t n[3]) {
    Box cb;
    for (int d = 0; d < 3; d++) {
        int64_t lo = std::max<int64_t>(tb.lo[d], 0), hi = std::min<int64_t>(tb.hi[d], n[d] - 2);
        cb.lo[d] = lo + 1;
        cb.hi[d] = std::max(hi, lo) + 1;
    }
    return cb;
}

int diffusion_box(int32_t form, const ps_array& T2, const ps_array& Tin, const ps_array& Ci, const ps_array& lam,
                  double lam_s, double dt, double hx, double hy, double hz, const Box& thread_box, int memopt,
                  int loopsize, int fp64_mode, cudaStream_t s, int* d_err, HideReq* hr = nullptr) {
    Box cb = inner_cells(thread_box, T2.n);
    const ps_array* lp = form == PS_DIFF_FLUX_LAM ? &lam : nullptr;
    if (cb.hi[0] <= cb.lo[0] || cb.hi[1] <= cb.lo[1] || cb.hi[2] <= cb.lo[2]) return hr ? PS_ERR_UNSUPPORTED : PS_OK;
    if (T2.dtype == PS_F64 && fp64_mode == PS_FP64_SPLIT) {
        int rc = launch_diffusion_split(form, T2, Tin, Ci, lp, lam_s, dt, hx, hy, hz, cb, loopsize, s, d_err, hr);
        if (rc != PS_ERR_UNSUPPORTED || hr) return rc;  // not TMA-eligible: IEEE kernels below
    }
    if (T2.dtype == PS_F64)
        return dispatch_diffusion<double>(form, T2, Tin, Ci, lp, lam_s, dt, hx, hy, hz, cb, memopt, loopsize, s, d_err,
                                          hr);
    return dispatch_diffusion<float>(form, T2, Tin, Ci, lp, lam_s, dt, hx, hy, hz, cb, memopt, loopsize, s, d_err, hr);
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_fill(ps_array a, double value, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(a, "A"));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int64_t n = numel(a);
    unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)st->num_sms * 32);
    if (a.dtype == PS_F64)
        fill_kernel<double><<<g, 256, 0, s>>>(static_cast<double*>(a.ptr), n, value);
    else
        fill_kernel<float><<<g, 256, 0, s>>>(static_cast<float*>(a.ptr), n, (float)value);
    return finish_launch(s, 1, "ps_fill");
}

int ps_fd_apply(ps_fd_op op, int32_t lhs_inn, ps_array R, ps_array A, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(R, "R"));
    PS_TRY(check_array(A, "A"));
    PS_TRY(check_same_dtype(R, A, "R", "A"));
    if (op.kind < PS_FD_SEL || op.kind > PS_FD_MINLOC) return fail(PS_ERR_ARG, "ps_fd_apply: unknown kind %d", op.kind);
    if (op.ndims < 1 || op.ndims > 3) return fail(PS_ERR_ARG, "ps_fd_apply: ndims %d", op.ndims);
    int dmask = (1 << op.ndims) - 1;
    if ((op.opdims & ~dmask) || (op.inn & ~dmask) || (lhs_inn & ~dmask))
        return fail(PS_ERR_ARG, "ps_fd_apply: dimension masks exceed ndims");
    if ((op.kind == PS_FD_DIFF || op.kind == PS_FD_DIFF2) && __builtin_popcount(op.opdims) != 1)
        return fail(PS_ERR_ARG, "ps_fd_apply: a difference acts along exactly one dimension");
    if ((op.kind == PS_FD_AV || op.kind == PS_FD_HARM) && op.opdims == 0)
        return fail(PS_ERR_ARG, "ps_fd_apply: an average needs at least one dimension");
    for (int d = op.ndims; d < 3; d++)
        if (R.n[d] != 1 || A.n[d] != 1) return fail(PS_ERR_SHAPE, "ps_fd_apply: array has more dimensions than ndims");
    FdDesc d;
    d.kind = op.kind;
    d.opdims = op.opdims;
    d.inn = op.inn;
    d.ndims = op.ndims;
    d.lhs_inn = lhs_inn;
    for (int k = 0; k < 3; k++) {
        d.nR[k] = R.n[k];
        d.nA[k] = A.n[k];
        d.tmax[k] = R.n[k] - 2 * ((lhs_inn >> k) & 1);
        int rlo = 0, rhi = 0;
        if (op.kind == PS_FD_DIFF || op.kind == PS_FD_AV || op.kind == PS_FD_HARM) rhi = (op.opdims >> k) & 1;
        if (op.kind == PS_FD_DIFF2 || op.kind == PS_FD_MAXLOC || op.kind == PS_FD_MINLOC)
            rlo = rhi = (op.opdims >> k) & 1;
        int64_t lo = ((op.inn >> k) & 1) - rlo, hi = ((op.inn >> k) & 1) + rhi;
        if (d.tmax[k] > 0 && (lo < 0 || d.tmax[k] - 1 + hi > A.n[k] - 1))
            return fail(PS_ERR_SHAPE, "ps_fd_apply: the operator reads outside A along dimension %d", k);
    }
    if (d.tmax[0] <= 0 || d.tmax[1] <= 0 || d.tmax[2] <= 0) return PS_OK;
    if (op.ndims == 2) {
        // (nx, ny) is laid out as (nx, 1, ny): the 2-D macro is the 3-D one with y as z (the same
        // points in the same operation order; @maxloc / @minloc as OPD 5), so it runs as a sweep
        // along y with a register window
        auto yz = [](int m) { return (m & 1) | ((m & 2) << 1); };
        d.ndims = 3;
        d.opdims = yz(d.opdims);
        d.inn = yz(d.inn);
        d.lhs_inn = yz(d.lhs_inn);
        d.nR[2] = d.nR[1], d.nA[2] = d.nA[1], d.tmax[2] = d.tmax[1];
        d.nR[1] = d.nA[1] = d.tmax[1] = 1;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (R.dtype == PS_F64)
        PS_TRY(launch_fd<double>(d, static_cast<double*>(R.ptr), static_cast<const double*>(A.ptr), s));
    else
        PS_TRY(launch_fd<float>(d, static_cast<float*>(R.ptr), static_cast<const float*>(A.ptr), s));
    return finish_launch(s, sync, "ps_fd_apply");
}

int ps_memcopy3d(ps_array T2, ps_array T, ps_array Ci, const ps_launch* cfg, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(T2, "T2"));
    PS_TRY(check_array(T, "T"));
    PS_TRY(check_array(Ci, "Ci"));
    PS_TRY(check_same_dtype(T2, T, "T2", "T"));
    PS_TRY(check_same_dtype(T2, Ci, "T2", "Ci"));
    PS_TRY(check_shape(T, T2.n[0], T2.n[1], T2.n[2], "T"));
    PS_TRY(check_shape(Ci, T2.n[0], T2.n[1], T2.n[2], "Ci"));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Box b = launch_box(cfg, T2.n);
    bool full = b.lo[0] == 0 && b.lo[1] == 0 && b.lo[2] == 0 && b.hi[0] == T2.n[0] && b.hi[1] == T2.n[1] &&
                b.hi[2] == T2.n[2];
    bool aligned = (reinterpret_cast<uintptr_t>(T2.ptr) | reinterpret_cast<uintptr_t>(T.ptr) |
                    reinterpret_cast<uintptr_t>(Ci.ptr)) % 16 == 0;
    int64_t n = numel(T2);
    if (full && aligned) {
        int64_t vn = n / (T2.dtype == PS_F64 ? 2 : 4);
        unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((vn + 1023) / 1024, (int64_t)st->num_sms * 16));
        if (T2.dtype == PS_F64)
            memcopy_flat<double><<<g, 256, 0, s>>>(static_cast<double*>(T2.ptr), static_cast<const double*>(T.ptr),
                                                   static_cast<const double*>(Ci.ptr), n);
        else
            memcopy_flat<float><<<g, 256, 0, s>>>(static_cast<float*>(T2.ptr), static_cast<const float*>(T.ptr),
                                                  static_cast<const float*>(Ci.ptr), n);
    } else {
        int64_t wx = b.hi[0] - b.lo[0], wy = b.hi[1] - b.lo[1], wz = b.hi[2] - b.lo[2];
        if (wx > 0 && wy > 0 && wz > 0) {
            dim3 blk(32, 8, 1);
            if (T2.dtype == PS_F64)
                memcopy_box<double><<<grid3(wx, wy, wz, blk), blk, 0, s>>>(
                    static_cast<double*>(T2.ptr), static_cast<const double*>(T.ptr),
                    static_cast<const double*>(Ci.ptr), T2.n[0], T2.n[1], b);
            else
                memcopy_box<float><<<grid3(wx, wy, wz, blk), blk, 0, s>>>(
                    static_cast<float*>(T2.ptr), static_cast<const float*>(T.ptr), static_cast<const float*>(Ci.ptr),
                    T2.n[0], T2.n[1], b);
        }
    }
    return finish_launch(s, sync, "ps_memcopy3d");
}

int ps_diffusion3d_step(int32_t form, ps_array T2, ps_array T, ps_array Ci, ps_array lam_arr, double lam, double dt,
                        double hx, double hy, double hz, const ps_launch* cfg, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(diffusion_args(form, T2, T, Ci, lam_arr));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Box tb = launch_box(cfg, T2.n);
    int memopt = cfg ? cfg->memopt : 0;
    int loopsize = cfg ? cfg->loopsize : 0;
    int fp64_mode = cfg ? cfg->fp64_mode : PS_FP64_IEEE;
    if (loopsize < 0) return fail(PS_ERR_ARG, "ps_diffusion3d_step: loopsize must be >= 0");
    if (fp64_mode < PS_FP64_IEEE || fp64_mode > PS_FP64_SPLIT_GRID)
        return fail(PS_ERR_ARG, "unknown fp64_mode %d", fp64_mode);
    if (fp64_mode != PS_FP64_IEEE) fp64_mode = PS_FP64_SPLIT;  // one step: the state stays IEEE
    PS_TRY(diffusion_box(form, T2, T, Ci, lam_arr, lam, dt, hx, hy, hz, tb, memopt, loopsize, fp64_mode, s, st->d_err));
    return finish_launch(s, sync, "ps_diffusion3d_step");
}

}  // extern "C"

namespace ps {
namespace {
thread_local cudaEvent_t t_order_event = nullptr;
}

// The boundary-first launch of ps_diffusion3d_step_split (memopt, TMA-eligible arrays); returns
// PS_ERR_UNSUPPORTED (nothing launched) when it does not apply.
static int ordered_step(int32_t form, const ps_array& T2, const ps_array& T, const ps_array& Ci,
                        const ps_array& lam_arr, double lam, double dt, double hx, double hy, double hz,
                        const int64_t bw[3], int fp64_mode, cudaStream_t sb, cudaStream_t si, ps_comm_fn comm,
                        void* comm_ctx, DeviceState* st) {
    volatile unsigned* hc = nullptr;
    unsigned* dc = nullptr;
    PS_TRY(progress_word(&hc, &dc));
    if (!dc) return PS_ERR_UNSUPPORTED;
    HideReq hr{};
    for (int d = 0; d < 3; ++d) {
        hr.lo_end[d] = bw[d] + 1;
        hr.hi_start[d] = T2.n[d] - 1 - bw[d];
    }
    hr.counter = dc;
    if (sb != si) {  // the launch follows the work already queued on both streams
        if (!t_order_event) PS_CUDA_TRY(cudaEventCreateWithFlags(&t_order_event, cudaEventDisableTiming));
        PS_CUDA_TRY(cudaEventRecord(t_order_event, sb));
        PS_CUDA_TRY(cudaStreamWaitEvent(si, t_order_event, 0));
    }
    *hc = 0u;
    const Box full = {{0, 0, 0}, {T2.n[0], T2.n[1], T2.n[2]}};
    int rc = diffusion_box(form, T2, T, Ci, lam_arr, lam, dt, hx, hy, hz, full, 1, 0, fp64_mode, si, st->d_err, &hr);
    if (rc != PS_OK) return rc;
    PS_TRY(finish_launch(si, 0, "ps_diffusion3d_step_split"));
    // wait for the boundary tiles (bounded; a kernel that ended early is reported by the sync below)
    const auto t0 = std::chrono::steady_clock::now();
    for (unsigned spin = 1; *hc < (unsigned)hr.nb; ++spin) {
        if (spin % 256 == 0) {
            cudaError_t q = cudaStreamQuery(si);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return cuda_fail(q, "ps_diffusion3d_step_split");
            if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60)) {
                PS_CUDA_TRY(cudaStreamSynchronize(si));
                break;
            }
        }
    }
    const bool boundary_done = *hc >= (unsigned)hr.nb;
    int crc = PS_OK;
    if (comm && boundary_done) crc = comm(comm_ctx);
    PS_TRY(finish_launch(si, 1, "ps_diffusion3d_step_split(sync)"));
    if (!boundary_done) return fail(PS_ERR_TIMEOUT, "ps_diffusion3d_step_split: boundary tiles not reported done");
    if (crc != PS_OK) return fail(crc, "ps_diffusion3d_step_split: communication callback returned %d", crc);
    return PS_OK;
}

}  // namespace ps

extern "C" {

int ps_diffusion3d_step_split(int32_t form, ps_array T2, ps_array T, ps_array Ci, ps_array lam_arr, double lam,
                              double dt, double hx, double hy, double hz, const ps_launch* cfg, const int64_t bw[3],
                              void* s_boundary, void* s_inner, ps_comm_fn comm, void* comm_ctx) {
    DeviceState* st = nullptr;
    const int memopt = cfg ? cfg->memopt : 0, fp64_mode = cfg ? cfg->fp64_mode : PS_FP64_IEEE;
    PS_TRY(current_state(&st));
    PS_TRY(diffusion_args(form, T2, T, Ci, lam_arr));
    if (!bw) return fail(PS_ERR_NULL, "ps_diffusion3d_step_split: NULL boundary width");
    const int64_t* ms = T2.n;  // the kernel's `@parallel` grid: all arguments are n^3
    // validate_ranges_args (src/ParallelKernel/hide_communication.jl:396-403)
    bool any_gt1 = false;
    for (int d = 0; d < 3; d++) {
        if (bw[d] < 0) return fail(PS_ERR_ARG, "boundary width must be >= 0");
        if (!(ms[d] > 2 * bw[d])) return fail(PS_ERR_SHAPE, "@hide_communication: length(ranges) > 2*boundary_width violated");
        if (ms[d] > 1 && bw[d] == 0) return fail(PS_ERR_SHAPE, "@hide_communication: boundary_width 0 in a dimension of length > 1");
        any_gt1 |= ms[d] > 1;
    }
    if (!any_gt1) return fail(PS_ERR_SHAPE, "@hide_communication: all ranges have length 1");
    cudaStream_t sb = static_cast<cudaStream_t>(s_boundary), si = static_cast<cudaStream_t>(s_inner);
    if (memopt) {
        // One TMA z-sweep launch on s_inner whose first CTAs take the tiles holding boundary cells
        // (cells 1 .. bw and n-1-bw .. n-2 of each axis: the reference's boundary ranges, whose
        // high end in @inn(T2) cells is n-bw+1 .. n-2, plus the planes a halo exchange sends).
        // Each such CTA counts itself in host-mapped memory after its stores; `comm` runs once
        // all have, while the inner tiles still run. No second launch, no tile cut twice.
        int rc = ordered_step(form, T2, T, Ci, lam_arr, lam, dt, hx, hy, hz, bw, fp64_mode, sb, si, comm, comm_ctx,
                              st);
        if (rc != PS_ERR_UNSUPPORTED) return rc;  // otherwise the boundary slabs as separate launches below
    }
    // Boundary widths below (lw) and above (hw) the inner box. With the z-sweep kernels the x and y
    // slabs are widened to whole sweep tiles (x: 64 FP64 / 128 FP32 cells from an even cell, y: 8
    // rows): a slab narrower than a tile costs the whole tile anyway, and an inner box that starts
    // mid-tile costs one more tile column. The boundary boxes then hold a superset of the requested
    // boundary cells (all computed before `comm`), the inner box the rest; each cell is computed once.
    int64_t lw[3] = {bw[0], bw[1], bw[2]}, hw[3] = {bw[0], bw[1], bw[2]};
    if (memopt) {
        const int64_t W = (T2.dtype == PS_F64 || fp64_mode != PS_FP64_IEEE) ? 64 : 128;
        const int64_t a = ((bw[0] + W) / W) * W - 1;           // cells [1, a + 1): ends at a tile edge
        const int64_t b = ms[0] + 1 - ((ms[0] + 1 - bw[0]) / W) * W;  // first cell on a tile edge
        if (bw[0] > 0 && a >= bw[0] && b >= bw[0] && ms[0] > a + b) {
            lw[0] = a;
            hw[0] = b;
        }
        const int64_t y = ((bw[1] + 7) / 8) * 8;
        if (bw[1] > 0 && ms[1] > 2 * y) lw[1] = hw[1] = y;
    }
    // get_ranges_outer / get_ranges_inner (src/ParallelKernel/hide_communication.jl:350-394), 3-D case,
    // converted to 0-based half-open boxes.
    Box outer[6] = {
        {{0, lw[1], lw[2]}, {lw[0], ms[1] - hw[1], ms[2] - hw[2]}},
        {{0, 0, 0}, {ms[0], ms[1], lw[2]}},
        {{0, 0, ms[2] - hw[2]}, {ms[0], ms[1], ms[2]}},
        {{ms[0] - hw[0], lw[1], lw[2]}, {ms[0], ms[1] - hw[1], ms[2] - hw[2]}},
        {{0, 0, lw[2]}, {ms[0], lw[1], ms[2] - hw[2]}},
        {{0, ms[1] - hw[1], lw[2]}, {ms[0], ms[1], ms[2] - hw[2]}},
    };
    Box inner = {{lw[0], lw[1], lw[2]}, {ms[0] - hw[0], ms[1] - hw[1], ms[2] - hw[2]}};
    for (int i = 0; i < 6; i++) {
        bool empty = false;
        for (int d = 0; d < 3; d++) empty |= outer[i].hi[d] <= outer[i].lo[d];
        if (empty) continue;
        PS_TRY(diffusion_box(form, T2, T, Ci, lam_arr, lam, dt, hx, hy, hz, outer[i], memopt, 0, fp64_mode, sb, st->d_err));
    }
    PS_TRY(finish_launch(sb, 0, "ps_diffusion3d_step_split(boundary)"));
    PS_TRY(diffusion_box(form, T2, T, Ci, lam_arr, lam, dt, hx, hy, hz, inner, memopt, 0, fp64_mode, si, st->d_err));
    PS_TRY(finish_launch(si, 0, "ps_diffusion3d_step_split(inner)"));
    PS_TRY(finish_launch(sb, 1, "ps_diffusion3d_step_split(boundary sync)"));
    int crc = PS_OK;
    if (comm) crc = comm(comm_ctx);
    PS_TRY(finish_launch(si, 1, "ps_diffusion3d_step_split(inner sync)"));
    if (crc != PS_OK) return fail(crc, "ps_diffusion3d_step_split: communication callback returned %d", crc);
    return PS_OK;
}

int ps_acoustic3d_v(ps_array Vx, ps_array Vy, ps_array Vz, ps_array P, double dt, double rho, double dx, double dy,
                    double dz, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(P, "P"));
    PS_TRY(check_array(Vx, "Vx"));
    PS_TRY(check_array(Vy, "Vy"));
    PS_TRY(check_array(Vz, "Vz"));
    PS_TRY(check_same_dtype(P, Vx, "P", "Vx"));
    PS_TRY(check_same_dtype(P, Vy, "P", "Vy"));
    PS_TRY(check_same_dtype(P, Vz, "P", "Vz"));
    int64_t nx = P.n[0], ny = P.n[1], nz = P.n[2];
    PS_TRY(check_shape(Vx, nx + 1, ny, nz, "Vx"));
    PS_TRY(check_shape(Vy, nx, ny + 1, nz, "Vy"));
    PS_TRY(check_shape(Vz, nx, ny, nz + 1, "Vz"));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8, 1);
    dim3 grd = grid3(nx + 1, ny + 1, nz + 1, blk);
    if (P.dtype == PS_F64)
        acoustic_v_kernel<double><<<grd, blk, 0, s>>>(static_cast<double*>(Vx.ptr), static_cast<double*>(Vy.ptr),
                                                      static_cast<double*>(Vz.ptr), static_cast<const double*>(P.ptr),
                                                      nx, ny, nz, dt / rho, make_div(dx), make_div(dy),
                                                      make_div(dz));
    else
        acoustic_v_kernel<float><<<grd, blk, 0, s>>>(static_cast<float*>(Vx.ptr), static_cast<float*>(Vy.ptr),
                                                     static_cast<float*>(Vz.ptr), static_cast<const float*>(P.ptr), nx,
                                                     ny, nz, (float)dt / (float)rho, make_div((float)dx),
                                                     make_div((float)dy), make_div((float)dz));
    return finish_launch(s, sync, "ps_acoustic3d_v");
}

int ps_acoustic3d_p(ps_array P, ps_array Vx, ps_array Vy, ps_array Vz, double dt, double k, double dx, double dy,
                    double dz, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(P, "P"));
    PS_TRY(check_array(Vx, "Vx"));
    PS_TRY(check_array(Vy, "Vy"));
    PS_TRY(check_array(Vz, "Vz"));
    PS_TRY(check_same_dtype(P, Vx, "P", "Vx"));
    PS_TRY(check_same_dtype(P, Vy, "P", "Vy"));
    PS_TRY(check_same_dtype(P, Vz, "P", "Vz"));
    int64_t nx = P.n[0], ny = P.n[1], nz = P.n[2];
    PS_TRY(check_shape(Vx, nx + 1, ny, nz, "Vx"));
    PS_TRY(check_shape(Vy, nx, ny + 1, nz, "Vy"));
    PS_TRY(check_shape(Vz, nx, ny, nz + 1, "Vz"));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8, 1);
    dim3 grd = grid3(nx, ny, nz, blk);
    if (P.dtype == PS_F64)
        acoustic_p_kernel<double><<<grd, blk, 0, s>>>(static_cast<double*>(P.ptr), static_cast<const double*>(Vx.ptr),
                                                      static_cast<const double*>(Vy.ptr),
                                                      static_cast<const double*>(Vz.ptr), nx, ny, nz, dt * k,
                                                      make_div(dx), make_div(dy), make_div(dz));
    else
        acoustic_p_kernel<float><<<grd, blk, 0, s>>>(static_cast<float*>(P.ptr), static_cast<const float*>(Vx.ptr),
                                                     static_cast<const float*>(Vy.ptr), static_cast<const float*>(Vz.ptr),
                                                     nx, ny, nz, (float)dt * (float)k, make_div((float)dx),
                                                     make_div((float)dy), make_div((float)dz));
    return finish_launch(s, sync, "ps_acoustic3d_p");
}

}  // extern "C"
