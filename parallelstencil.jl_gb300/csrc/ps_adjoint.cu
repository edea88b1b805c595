// ps_adjoint.cu -- hand-written adjoint of the 3-D diffusion step (flux form, conductivity array)
// and the checkpointed gradient of an inverse-conductivity misfit.
//
// The reference differentiates `@parallel` kernels with Enzyme (`@parallel ∇=...`,
// src/ParallelKernel/parallel.jl:265-301; src/ParallelKernel/EnzymeExt/autodiff_gpu.jl:35-40).
// Here the reverse step is written out: with μ = dt*Ci*λ2 on inner cells (0 elsewhere),
//   λ[c]     = λ2[c] + Σ_d h_d² (k_d+(μ[c+e] - μ[c]) - k_d-(μ[c] - μ[c-e]))      (inner cells)
//   glam[c] += 0.5 Σ_faces(a,b=a+e) of c (μ[a] - μ[b]) h_d² (T[b] - T[a])          (all cells)
// i.e. the transpose of the step's Jacobian in T (a symmetric operator) and its derivative in
// lam through the face conductivities k = (lam_a + lam_b)/2.
//
// ps_diffusion3d_misfit_gradient runs nt forward steps keeping a checkpoint every `ce` steps,
// forms L = 0.5 ||T_nt - T_obs||^2, then sweeps the segments in reverse: each segment is
// recomputed from its checkpoint into device buffers and differentiated backwards.
#include <math.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "ps_common.cuh"
#include "ps_dd.cuh"

namespace ps {

int diffusion_box(int32_t form, const ps_array& T2, const ps_array& Tin, const ps_array& Ci, const ps_array& lam,
                  double lam_s, double dt, double hx, double hy, double hz, const Box& thread_box, int memopt,
                  int loopsize, int fp64_mode, cudaStream_t s, int* d_err, HideReq* hr = nullptr);
int grid_misfit_gradient(const ps_array& T0, const ps_array& Tobs, const ps_array& Ci, const ps_array& lam, double dt,
                         double hx, double hy, double hz, int64_t nt, int64_t ce, const ps_array& glam,
                         const ps_array& T_final, double* loss, int64_t* recomputed, bool* redo, cudaStream_t s);

template <typename T>
__global__ void __launch_bounds__(256) adjoint_step_kernel(T* __restrict__ lamT, const T* __restrict__ lamT2,
                                                           const T* __restrict__ Tn, const T* __restrict__ Ci,
                                                           const T* __restrict__ lam, T* __restrict__ glam, T dt,
                                                           T hx, T hy, T hz, int64_t nx, int64_t ny, int64_t nz) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t j = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    const T hh[3] = {hx * hx, hy * hy, hz * hz};
    const int64_t st[3] = {1, nx, nx * ny};
    const int64_t ext[3] = {nx, ny, nz};
    auto inner = [&](int64_t a, int64_t b, int64_t c) {
        return a >= 1 && a <= nx - 2 && b >= 1 && b <= ny - 2 && c >= 1 && c <= nz - 2;
    };
    for (int64_t k = blockIdx.z; k < nz; k += gridDim.z) {
        const int64_t c = i + nx * (j + ny * k);
        const int64_t idx[3] = {i, j, k};
        const bool inner_c = inner(i, j, k);
        const T mu_c = inner_c ? dt * Ci[c] * lamT2[c] : T(0);
        const T lc = lam[c], Tc = Tn[c];
        T acc = T(0), g = T(0);
#pragma unroll
        for (int d = 0; d < 3; d++) {
#pragma unroll
            for (int sgn = -1; sgn <= 1; sgn += 2) {
                const int64_t q = idx[d] + sgn;
                if (q < 0 || q >= ext[d]) continue;
                const int64_t nb = c + sgn * st[d];
                const bool inner_n = inner(d == 0 ? q : i, d == 1 ? q : j, d == 2 ? q : k);
                const T mu_n = inner_n ? dt * Ci[nb] * lamT2[nb] : T(0);
                const T kf = (lc + lam[nb]) * T(0.5);
                const T mua = sgn > 0 ? mu_c : mu_n, mub = sgn > 0 ? mu_n : mu_c;
                const T Ta = sgn > 0 ? Tc : Tn[nb], Tb = sgn > 0 ? Tn[nb] : Tc;
                acc += hh[d] * kf * (mu_n - mu_c);
                g += T(0.5) * (mua - mub) * hh[d] * (Tb - Ta);
            }
        }
        lamT[c] = inner_c ? lamT2[c] + acc : T(0);
        glam[c] += g;
    }
}

// The same reverse step with FP64 arrays evaluated in split-FP32 arithmetic (fp64_mode != IEEE):
// every input is split into an FP32 pair with integer operations, the sums and products of the
// IEEE kernel above run on pairs (47-bit significands), and the results are applied in FP64 as
// λ = (λ2 + acc.h) + acc.l and glam = (glam + g.h) + g.l. Same statement order as the IEEE kernel.
// Two passes: adjoint_pairs_kernel splits T and lam and forms μ = (dt Ci) λT2 once per cell into
// pair arrays; adjoint_step_split_kernel reads the seven points' pairs from them (each value was
// split and each μ multiplied seven times when one pass did everything: 1.35 ms per 256^3 step).
__global__ void __launch_bounds__(256) adjoint_pairs_kernel(float2* __restrict__ Tp, float2* __restrict__ Lp,
                                                            float2* __restrict__ Mp, const double* __restrict__ lamT2,
                                                            const double* __restrict__ Tn, const double* __restrict__ Ci,
                                                            const double* __restrict__ lam, dd dt, int64_t nx,
                                                            int64_t ny, int64_t nz, int* err) {
    bool big = false;
    const int64_t n = nx * ny * nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
        const bool inner = i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2;
        const dd t = dd_split(__ldg(Tn + c), big), l = dd_split(__ldg(lam + c), big);
        dd mu = {0.0f, 0.0f};
        if (inner) mu = dd_mul(dd_mul(dt, dd_split(__ldg(Ci + c), big)), dd_split(__ldg(lamT2 + c), big));
        Tp[c] = make_float2(t.h, t.l);
        Lp[c] = make_float2(l.h, l.l);
        Mp[c] = make_float2(mu.h, mu.l);
    }
    if (big) atomicOr(err, DEV_ERR_RANGE);  // a magnitude outside the split range: reported at the next sync
}

__global__ void __launch_bounds__(256) adjoint_step_split_kernel(double* __restrict__ lamT,
                                                                 const double* __restrict__ lamT2,
                                                                 const float2* __restrict__ Tp,
                                                                 const float2* __restrict__ Lp,
                                                                 const float2* __restrict__ Mp,
                                                                 double* __restrict__ glam, dd hh0, dd hh1, dd hh2,
                                                                 int64_t nx, int64_t ny, int64_t nz) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t j = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    const dd hh[3] = {hh0, hh1, hh2};
    const int64_t st[3] = {1, nx, nx * ny};
    const int64_t ext[3] = {nx, ny, nz};
    const dd zero = {0.0f, 0.0f};
    auto pr = [](const float2* a, int64_t c) {
        const float2 v = __ldg(a + c);
        return dd{v.x, v.y};
    };
    for (int64_t k = blockIdx.z; k < nz; k += gridDim.z) {
        const int64_t c = i + nx * (j + ny * k);
        const int64_t idx[3] = {i, j, k};
        const bool inner_c = i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2;
        const dd mu_c = pr(Mp, c), lc = pr(Lp, c), Tc = pr(Tp, c);
        dd acc = zero, g = zero;
#pragma unroll
        for (int d = 0; d < 3; d++) {
#pragma unroll
            for (int sgn = -1; sgn <= 1; sgn += 2) {
                const int64_t q = idx[d] + sgn;
                if (q < 0 || q >= ext[d]) continue;
                const int64_t nb = c + sgn * st[d];
                const dd mu_n = pr(Mp, nb);  // zero off the inner cells
                const dd kf = dd_scale(dd_add(lc, pr(Lp, nb)), 0.5f);
                const dd Tnb = pr(Tp, nb);
                const dd mua = sgn > 0 ? mu_c : mu_n, mub = sgn > 0 ? mu_n : mu_c;
                const dd Ta = sgn > 0 ? Tc : Tnb, Tb = sgn > 0 ? Tnb : Tc;
                acc = dd_add(acc, dd_mul(dd_mul(hh[d], kf), dd_sub(mu_n, mu_c)));
                g = dd_add(g, dd_mul(dd_mul(dd_scale(dd_sub(mua, mub), 0.5f), hh[d]), dd_sub(Tb, Ta)));
            }
        }
        lamT[c] = inner_c ? (__ldg(lamT2 + c) + f32_to_f64(acc.h)) + f32_to_f64(acc.l) : 0.0;
        glam[c] = (glam[c] + f32_to_f64(g.h)) + f32_to_f64(g.l);
    }
}

// λ = (T - T_obs) on inner cells (0 on the boundary); loss += 0.5 Σ (T - T_obs)^2 over all cells.
__global__ void misfit_kernel(double* __restrict__ lamT, const double* __restrict__ Tn, const double* __restrict__ Tobs,
                              int64_t nx, int64_t ny, int64_t nz, double* loss) {
    double s = 0.0;
    const int64_t n = nx * ny * nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
        const double r = Tn[c] - Tobs[c];
        s += 0.5 * r * r;
        const bool inner = i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 2 && k >= 1 && k <= nz - 2;
        lamT[c] = inner ? r : 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

static int check3(const ps_array& a, const ps_array& ref, const char* name) {
    PS_TRY(check_array(a, name));
    PS_TRY(check_same_dtype(a, ref, name, "T"));
    return check_shape(a, ref.n[0], ref.n[1], ref.n[2], name);
}

// Library-owned scratch of the gradient (checkpoints, segment states, forward and adjoint buffers),
// kept between calls (an inverse problem asks for many gradients of one size); freed by
// ps_finalize.
static void* g_adj_scratch = nullptr;
static size_t g_adj_bytes = 0;

// Pair arrays of the split reverse step (T, lam, μ: 3 x 8 bytes per cell), grow-only.
static void* g_adj_pairs = nullptr;
static size_t g_adj_pairs_bytes = 0;

void adjoint_free_scratch() {
    if (g_adj_scratch) cudaFree(g_adj_scratch);
    g_adj_scratch = nullptr;
    g_adj_bytes = 0;
    if (g_adj_pairs) cudaFree(g_adj_pairs);
    g_adj_pairs = nullptr;
    g_adj_pairs_bytes = 0;
}

static int adjoint_pairs(size_t bytes, char** p) {
    if (bytes > g_adj_pairs_bytes) {
        if (g_adj_pairs) cudaFree(g_adj_pairs);
        g_adj_pairs = nullptr;
        g_adj_pairs_bytes = 0;
        if (cudaMalloc(&g_adj_pairs, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(PS_ERR_NOMEM, "adjoint step: pair scratch of %zu bytes failed", bytes);
        }
        g_adj_pairs_bytes = bytes;
    }
    *p = static_cast<char*>(g_adj_pairs);
    return PS_OK;
}

static int adjoint_scratch(size_t bytes, char** p) {
    if (bytes > g_adj_bytes) {
        adjoint_free_scratch();
        if (cudaMalloc(&g_adj_scratch, bytes) != cudaSuccess) {
            cudaGetLastError();
            g_adj_scratch = nullptr;
            return fail(PS_ERR_NOMEM, "ps_diffusion3d_misfit_gradient: scratch allocation of %zu bytes failed", bytes);
        }
        g_adj_bytes = bytes;
    }
    *p = static_cast<char*>(g_adj_scratch);
    return PS_OK;
}

static dd host_split(double x) {  // x = h + l to ~2^-48 relative (host side, for the coefficients)
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

static int launch_adjoint_step(const ps_array& lamT, const ps_array& lamT2, const ps_array& Tn, const ps_array& Ci,
                               const ps_array& lam, const ps_array& glam, double dt, double hx, double hy, double hz,
                               cudaStream_t s, int fp64_mode = PS_FP64_IEEE, int* d_err = nullptr) {
    dim3 blk(32, 8);
    dim3 grd((unsigned)((Tn.n[0] + 31) / 32), (unsigned)((Tn.n[1] + 7) / 8), (unsigned)std::min<int64_t>(Tn.n[2], 65535));
    if (Tn.dtype == PS_F64 && fp64_mode != PS_FP64_IEEE && d_err) {
        const int64_t n = Tn.n[0] * Tn.n[1] * Tn.n[2];
        char* pp = nullptr;
        PS_TRY(adjoint_pairs((size_t)n * 3 * sizeof(float2), &pp));
        float2* Tp = reinterpret_cast<float2*>(pp);
        float2 *Lp = Tp + n, *Mp = Lp + n;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8));
        adjoint_pairs_kernel<<<g, 256, 0, s>>>(Tp, Lp, Mp, static_cast<const double*>(lamT2.ptr),
                                               static_cast<const double*>(Tn.ptr), static_cast<const double*>(Ci.ptr),
                                               static_cast<const double*>(lam.ptr), host_split(dt), Tn.n[0], Tn.n[1],
                                               Tn.n[2], d_err);
        adjoint_step_split_kernel<<<grd, blk, 0, s>>>(
            static_cast<double*>(lamT.ptr), static_cast<const double*>(lamT2.ptr), Tp, Lp, Mp,
            static_cast<double*>(glam.ptr), host_split(hx * hx), host_split(hy * hy), host_split(hz * hz), Tn.n[0],
            Tn.n[1], Tn.n[2]);
    } else if (Tn.dtype == PS_F64)
        adjoint_step_kernel<double><<<grd, blk, 0, s>>>(
            static_cast<double*>(lamT.ptr), static_cast<const double*>(lamT2.ptr), static_cast<const double*>(Tn.ptr),
            static_cast<const double*>(Ci.ptr), static_cast<const double*>(lam.ptr), static_cast<double*>(glam.ptr), dt,
            hx, hy, hz, Tn.n[0], Tn.n[1], Tn.n[2]);
    else
        adjoint_step_kernel<float><<<grd, blk, 0, s>>>(
            static_cast<float*>(lamT.ptr), static_cast<const float*>(lamT2.ptr), static_cast<const float*>(Tn.ptr),
            static_cast<const float*>(Ci.ptr), static_cast<const float*>(lam.ptr), static_cast<float*>(glam.ptr),
            (float)dt, (float)hx, (float)hy, (float)hz, Tn.n[0], Tn.n[1], Tn.n[2]);
    return PS_OK;
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_diffusion3d_adjoint_step(ps_array lamT, ps_array lamT2, ps_array T, ps_array Ci, ps_array lam, ps_array glam,
                                double dt, double hx, double hy, double hz, void* stream, int sync) {
    return ps_diffusion3d_adjoint_step_ex(lamT, lamT2, T, Ci, lam, glam, dt, hx, hy, hz, PS_FP64_IEEE, stream, sync);
}

int ps_diffusion3d_adjoint_step_ex(ps_array lamT, ps_array lamT2, ps_array T, ps_array Ci, ps_array lam,
                                   ps_array glam, double dt, double hx, double hy, double hz, int32_t fp64_mode,
                                   void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(T, "T"));
    PS_TRY(check3(lamT, T, "λT"));
    PS_TRY(check3(lamT2, T, "λT2"));
    PS_TRY(check3(Ci, T, "Ci"));
    PS_TRY(check3(lam, T, "lam"));
    PS_TRY(check3(glam, T, "glam"));
    if (lamT.ptr == lamT2.ptr) return fail(PS_ERR_ARG, "λT and λT2 must be distinct arrays");
    if (fp64_mode < PS_FP64_IEEE || fp64_mode > PS_FP64_SPLIT_GRID) return fail(PS_ERR_ARG, "unknown fp64_mode %d", fp64_mode);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(launch_adjoint_step(lamT, lamT2, T, Ci, lam, glam, dt, hx, hy, hz, s, fp64_mode, st->d_err));
    return finish_launch(s, sync, "ps_diffusion3d_adjoint_step");
}

int ps_diffusion3d_misfit_gradient(ps_array T0, ps_array Tobs, ps_array Ci, ps_array lam, double dt, double hx,
                                   double hy, double hz, int64_t nt, int64_t checkpoint_every, const ps_launch* cfg,
                                   ps_array dL_dlam, ps_array T_final, ps_adjoint_stats* stats, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(T0, "T0"));
    if (T0.dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_diffusion3d_misfit_gradient: FP64 arrays required");
    PS_TRY(check3(Tobs, T0, "T_obs"));
    PS_TRY(check3(Ci, T0, "Ci"));
    PS_TRY(check3(lam, T0, "lam"));
    PS_TRY(check3(dL_dlam, T0, "dL_dlam"));
    if (T_final.ptr) PS_TRY(check3(T_final, T0, "T_final"));
    if (!stats) return fail(PS_ERR_NULL, "NULL stats");
    if (nt < 1 || checkpoint_every < 1) return fail(PS_ERR_ARG, "nt and checkpoint_every must be >= 1");
    const int memopt = cfg ? cfg->memopt : 1;
    int fp64_mode = cfg ? cfg->fp64_mode : PS_FP64_IEEE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    if (fp64_mode == PS_FP64_SPLIT_GRID) {
        // forward and reverse sweeps on fixed power-of-two grids (TMA-eligible arrays with inner
        // cells); a value that leaves its grid makes the gradient run again with split pairs
        const bool ok = tma_eligible(T0) && tma_eligible(Ci) && tma_eligible(lam) && T0.n[0] > 2 && T0.n[1] > 2 &&
                        T0.n[2] > 2;
        if (ok) {
            double loss = 0.0;
            int64_t rec = 0;
            bool redo = false;
            PS_TRY(grid_misfit_gradient(T0, Tobs, Ci, lam, dt, hx, hy, hz, nt, checkpoint_every, dL_dlam, T_final,
                                        &loss, &rec, &redo, s));
            if (!redo) {
                PS_TRY(finish_launch(s, 1, "ps_diffusion3d_misfit_gradient"));
                stats->loss = loss;
                stats->checkpoints = (nt + checkpoint_every - 1) / checkpoint_every;
                stats->recomputed_steps = rec;
                stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                return PS_OK;
            }
        }
        fp64_mode = PS_FP64_SPLIT;
    }
    const int64_t ce = checkpoint_every, nseg = (nt + ce - 1) / ce;
    const size_t bytes = (size_t)numel(T0) * 8;
    // scratch: nseg checkpoints, ce segment states, two forward buffers, two adjoint buffers, the loss
    const int64_t nbuf = nseg + ce + 4;
    const size_t stride = (bytes + 255) / 256 * 256;
    char* scr = nullptr;
    PS_TRY(adjoint_scratch(stride * nbuf + 256, &scr));
    double* d_loss = reinterpret_cast<double*>(scr + stride * nbuf);
    int rc = PS_OK;
    auto arr = [&](int64_t b) {
        ps_array a = T0;
        a.ptr = scr + stride * b;
        return a;
    };
    auto ckpt = [&](int64_t sidx) { return arr(sidx); };
    auto seg = [&](int64_t j) { return arr(nseg + j); };
    ps_array fA = arr(nseg + ce), fB = arr(nseg + ce + 1), lA = arr(nseg + ce + 2), lB = arr(nseg + ce + 3);
    const Box full = {{0, 0, 0}, {T0.n[0], T0.n[1], T0.n[2]}};
    auto step = [&](const ps_array& out, const ps_array& in) {
        return diffusion_box(PS_DIFF_FLUX_LAM, out, in, Ci, lam, 0.0, dt, hx, hy, hz, full, memopt, 0, fp64_mode, s,
                             st->d_err);
    };
    auto copy = [&](const ps_array& dst, const ps_array& src) {
        return cudaMemcpyAsync(dst.ptr, src.ptr, bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? PS_OK
                   : fail(PS_ERR_CUDA, "device copy failed");
    };
    int64_t recomputed = 0;
    double loss = 0.0;
    // ---- forward with checkpoints ----
    // the steps write inner cells only: every state buffer gets T0's boundary values once
    if (rc == PS_OK) rc = copy(fA, T0);
    if (rc == PS_OK) rc = copy(fB, T0);
    for (int64_t j = 1; j < ce && j < nt && rc == PS_OK; j++) rc = copy(seg(j), T0);
    for (int64_t n = 0; n < nt && rc == PS_OK; n++) {
        if (n % ce == 0) rc = copy(ckpt(n / ce), fA);
        if (rc == PS_OK) rc = step(fB, fA);
        std::swap(fA, fB);
    }
    // ---- loss and λ_nt ----
    if (rc == PS_OK) {
        cudaMemsetAsync(d_loss, 0, sizeof(double), s);
        misfit_kernel<<<std::max(1, st->num_sms * 4), 256, 0, s>>>(static_cast<double*>(lA.ptr),
                                                                   static_cast<const double*>(fA.ptr),
                                                                   static_cast<const double*>(Tobs.ptr), T0.n[0],
                                                                   T0.n[1], T0.n[2], d_loss);
        if (T_final.ptr) rc = copy(T_final, fA);
        cudaMemsetAsync(dL_dlam.ptr, 0, bytes, s);
    }
    // ---- reverse sweep over segments ----
    for (int64_t sidx = nseg - 1; sidx >= 0 && rc == PS_OK; sidx--) {
        const int64_t n0 = sidx * ce, n1 = std::min(nt, n0 + ce);
        rc = copy(seg(0), ckpt(sidx));
        for (int64_t j = 1; j < n1 - n0 && rc == PS_OK; j++) {
            rc = step(seg(j), seg(j - 1));  // seg(j) holds the boundary values already
            recomputed++;
        }
        for (int64_t nn = n1 - 1; nn >= n0 && rc == PS_OK; nn--) {
            rc = launch_adjoint_step(lB, lA, seg(nn - n0), Ci, lam, dL_dlam, dt, hx, hy, hz, s, fp64_mode, st->d_err);
            std::swap(lA, lB);
        }
    }
    if (rc == PS_OK) {
        cudaError_t e = cudaMemcpyAsync(&loss, d_loss, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_fail(e, "ps_diffusion3d_misfit_gradient");
    }
    if (rc == PS_OK) rc = finish_launch(s, 1, "ps_diffusion3d_misfit_gradient");
    cudaStreamSynchronize(s);
    stats->loss = loss;
    stats->checkpoints = nseg;
    stats->recomputed_steps = recomputed;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

}  // extern "C"
