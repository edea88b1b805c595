// ps_stokes2d_apt.cu -- accelerated pseudo-transient (APT) Stokes 2-D with pseudo-time steps from
// the local viscosity maximum, and its FP64 and mixed-precision solvers.
//
// The reference's Stokes2D miniapp (miniapps/Stokes2D.jl:11-55) relaxes the momentum equations
// with damped pseudo-time steps from @av_xi(Mus); at a viscosity contrast of 1e-3 (a soft circular
// inclusion) that iteration diverges. This scheme keeps the miniapp's staggered arrays and
// statements (∇V, P, τ, R, V, the free-slip copies bc_x!/bc_y!) but
//   - takes every local pseudo-time step from Musτ = @maxloc(Mus), the reference's own idiom for
//     heterogeneous coefficients (miniapps/HydroMech2D.jl:27: min_dxy2/@maxloc(K_muf)/4.1);
//   - relaxes the stresses in pseudo-time (τ is state: τ = aτ τ + bτ ε̇') so that the pseudo-time
//     "wave speed" Vpdτ is the same in every cell (dτρ ∝ 1/Musτ, Gdτ ∝ Musτ); the face steps are
//     the smaller of the two cells' dτρ and the corner moduli the smallest of the four cells' Gdτ,
//     which keeps every face-cell and face-corner coupling within the CFL limit across the
//     inclusion's edge.
// Written as the reference's kernels would be:
//   @parallel function compute_apt_params!(...)        # once: Musτ, kP, aτ, bτ, aτc, bτc, dτVx, dτVy
//   @parallel function compute_P_τ!(∇V, Pt, τxx, τyy, τxy, Vx, Vy, kP, aτ, bτ, aτc, bτc, _dx, _dy)
//       @all(∇V)  = @d_xa(Vx)*_dx + @d_ya(Vy)*_dy
//       @all(Pt)  = @all(Pt) - @all(kP)*@all(∇V)
//       @all(τxx) = @all(aτ)*@all(τxx) + @all(bτ)*(@d_xa(Vx)*_dx - @all(∇V)*(1.0/3.0))
//       @all(τyy) = @all(aτ)*@all(τyy) + @all(bτ)*(@d_ya(Vy)*_dy - @all(∇V)*(1.0/3.0))
//       @all(τxy) = @all(aτc)*@all(τxy) + @all(bτc)*(0.5*(@d_yi(Vx)*_dy + @d_xi(Vy)*_dx))
//   @parallel function compute_R_V!(Rx, Ry, Vx, Vy, Pt, τxx, τyy, τxy, Rog, dτVx, dτVy, _dx, _dy)
//       @all(Rx)  = (@d_xi(τxx)*_dx + @d_ya(τxy)*_dy) - @d_xi(Pt)*_dx
//       @all(Ry)  = ((@d_yi(τyy)*_dy + @d_xa(τxy)*_dx) - @d_yi(Pt)*_dy) + @av_yi(Rog)
//       @inn(Vx)  = @inn(Vx) + @all(dτVx)*@all(Rx)
//       @inn(Vy)  = @inn(Vy) + @all(dτVy)*@all(Ry)
//   bc_y!(Vx); bc_x!(Vy)
// The CPU oracle's orc_stokes2d_apt_* functions are the same statements; every kernel here is
// bit-identical to them (FP64 and FP32; built with --fmad=false).
//
// Solvers (ps_stokes2d_apt_solve) stop on the FP64 residual of the state (V, P) with the stresses
// at their steady state τ = 2μ(ε̇ - ∇V/3), err = max(mean|Rx|, mean|Ry|, mean|∇V|)
// (Stokes2D.jl:119-120):
//   mode 0  FP64 APT iterations, the residual checked every `nout` iterations;
//   mode 1  defect correction: FP32 APT sweeps on the correction (δV, δP, δτ) with the FP64
//           residual of the state as source, FP64 update of V and P, FP64 residual check.
// Iterations run as CUDA graphs of `nout` iterations (two kernels each).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>

#include "ps_common.cuh"

namespace ps {

#define A2(a, i, j, n0) (a)[(int64_t)(i) + (int64_t)(n0) * (int64_t)(j)]

static double apt_now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------------------
// Coefficients (FP64 arithmetic on the values the arrays hold; stored rounded to T)
// ---------------------------------------------------------------------------------------
struct AptCoeffParams {
    double c0;   // (Vpdτ * max_lxy) / Re
    double v2;   // Vpdτ * Vpdτ
    double rp2;  // r + 2
    double r;
};

__device__ __forceinline__ void apt_cell_coeffs(double mt, const AptCoeffParams& p, double* R, double* G) {
    *R = p.c0 / mt;
    *G = (p.v2 / *R) / p.rp2;
}

template <typename T>
__global__ void apt_must_k(const T* __restrict__ Mus, T* __restrict__ Must, int64_t nx, int64_t ny) {
    const int64_t ix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, iy = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (ix >= nx || iy >= ny) return;
    double m = (double)A2(Mus, ix, iy, nx);
    if (ix > 0 && iy > 0 && ix < nx - 1 && iy < ny - 1) {
        double a = jl_max((double)A2(Mus, ix - 1, iy, nx), (double)A2(Mus, ix + 1, iy, nx));
        a = jl_max(a, m);
        m = jl_max(a, jl_max((double)A2(Mus, ix, iy - 1, nx), (double)A2(Mus, ix, iy + 1, nx)));
    }
    A2(Must, ix, iy, nx) = (T)m;
}

// Cell, corner and face coefficients from Musτ, in FP64 arithmetic on the values the arrays hold
// (FP32 fields: their own FP32 Mus widened), stored rounded to T.
template <typename T>
__global__ void apt_coeffs_k(const T* __restrict__ Mus, const T* __restrict__ Must, T* kP, T* aT, T* bT, T* aTc, T* bTc,
                             T* dtVx, T* dtVy, int64_t nx, int64_t ny, AptCoeffParams p) {
    const int64_t ix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, iy = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (ix >= nx || iy >= ny) return;
    auto RG = [&](int64_t x, int64_t y, double* R, double* G) { apt_cell_coeffs((double)A2(Must, x, y, nx), p, R, G); };
    double R, G;
    RG(ix, iy, &R, &G);
    const double mu = (double)A2(Mus, ix, iy, nx);
    const double a = 1.0 / (G / mu + 1.0);
    A2(kP, ix, iy, nx) = (T)(p.r * G);
    A2(aT, ix, iy, nx) = (T)a;
    A2(bT, ix, iy, nx) = (T)((2.0 * G) * a);
    if (ix < nx - 1 && iy < ny - 1) {
        double R1, G1, R2, G2, R3, G3;
        RG(ix + 1, iy, &R1, &G1);
        RG(ix, iy + 1, &R2, &G2);
        RG(ix + 1, iy + 1, &R3, &G3);
        const double g = jl_min(jl_min(G, G1), jl_min(G2, G3));
        const double mc = ((((double)A2(Mus, ix, iy, nx) + (double)A2(Mus, ix + 1, iy, nx)) +
                            (double)A2(Mus, ix, iy + 1, nx)) +
                           (double)A2(Mus, ix + 1, iy + 1, nx)) *
                          0.25;
        const double ac = 1.0 / (g / mc + 1.0);
        A2(aTc, ix, iy, nx - 1) = (T)ac;
        A2(bTc, ix, iy, nx - 1) = (T)((2.0 * g) * ac);
    }
    if (ix < nx - 1 && iy < ny - 2) {
        double Ra, Ga, Rb, Gb;
        RG(ix, iy + 1, &Ra, &Ga);
        RG(ix + 1, iy + 1, &Rb, &Gb);
        A2(dtVx, ix, iy, nx - 1) = (T)jl_min(Ra, Rb);
    }
    if (ix < nx - 2 && iy < ny - 1) {
        double Ra, Ga, Rb, Gb;
        RG(ix + 1, iy, &Ra, &Ga);
        RG(ix + 1, iy + 1, &Rb, &Gb);
        A2(dtVy, ix, iy, nx - 2) = (T)jl_min(Ra, Rb);
    }
}

// ---------------------------------------------------------------------------------------
// Iteration kernels
// ---------------------------------------------------------------------------------------
template <typename T>
struct AptArrays {
    T *Vx, *Vy, *Pt, *txx, *tyy, *txy, *divV, *Rx, *Ry;
    const T *kP, *aT, *bT, *aTc, *bTc, *dtVx, *dtVy, *Rog;
    const T *div0, *rx0, *ry0;  // DEFECT: the FP64 residual of the outer state (as T)
    double* red;                // Σ|Rx|, Σ|Ry|, Σ|∇V| of this iteration (or nullptr)
    int64_t nx, ny;
    T _dx, _dy;
};

// Block sums of two values (v1/out1 optional), one atomicAdd per block and value. Every thread
// of the block calls it (block-uniform condition).
__device__ __forceinline__ void apt_block_add(double v0, double* out0, double v1 = 0.0, double* out1 = nullptr) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        v0 += __shfl_xor_sync(0xFFFFFFFFu, v0, o);
        v1 += __shfl_xor_sync(0xFFFFFFFFu, v1, o);
    }
    __shared__ double part[2][32];
    const int t = threadIdx.y * blockDim.x + threadIdx.x, lane = t & 31, warp = t >> 5;
    if (lane == 0) {
        part[0][warp] = v0;
        part[1][warp] = v1;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x * blockDim.y + 31) >> 5;
        double s0 = lane < nw ? part[0][lane] : 0.0, s1 = lane < nw ? part[1][lane] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            s0 += __shfl_xor_sync(0xFFFFFFFFu, s0, o);
            s1 += __shfl_xor_sync(0xFFFFFFFFu, s1, o);
        }
        if (lane == 0) {
            if (s0 != 0.0) atomicAdd(out0, s0);
            if (out1 && s1 != 0.0) atomicAdd(out1, s1);
        }
    }
}

#define A2I(a, i, j, n0) (a)[(i) + (n0) * (j)]  // index arithmetic in the index type I

// compute_P_τ!: cells (∇V, Pt, τxx, τyy) and corners (τxy). DEFECT: the correction's sweep
// (pressure driven by ∇δV + ∇V of the outer state). STORE: write ∇V (and add Σ|∇V| to red).
// I: index type (int where every array has fewer than 2^31 elements).
template <typename T, bool DEFECT, bool STORE, typename I>
__global__ void __launch_bounds__(256) apt_cells_k(AptArrays<T> a) {
    grid_dependency_wait();  // V of the previous iteration's faces kernel
    grid_dependents_may_launch();
    const I ix = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x, iy = (I)blockIdx.y * (I)blockDim.y + (I)threadIdx.y;
    const I nx = (I)a.nx, ny = (I)a.ny;
    const T third = (T)(1.0 / 3.0), h = (T)0.5;
    double sabs = 0.0;
    if (ix < nx && iy < ny) {
        const I c = ix + nx * iy;
        const T dvx = A2I(a.Vx, ix + 1, iy, nx + 1) - A2I(a.Vx, ix, iy, nx + 1);
        const T dvy = A2I(a.Vy, ix, iy + 1, nx) - A2I(a.Vy, ix, iy, nx);
        const T d = dvx * a._dx + dvy * a._dy;
        const T td = d * third;
        T dp = d;
        if constexpr (DEFECT) dp = d + a.div0[c];
        a.Pt[c] = a.Pt[c] - a.kP[c] * dp;
        a.txx[c] = a.aT[c] * a.txx[c] + a.bT[c] * (dvx * a._dx - td);
        a.tyy[c] = a.aT[c] * a.tyy[c] + a.bT[c] * (dvy * a._dy - td);
        if constexpr (STORE) {
            a.divV[c] = dp;
            sabs = fabs((double)dp);
        }
        if (ix < nx - 1 && iy < ny - 1) {
            const I k = ix + (nx - 1) * iy;
            const T e = h * ((A2I(a.Vx, ix + 1, iy + 1, nx + 1) - A2I(a.Vx, ix + 1, iy, nx + 1)) * a._dy +
                             (A2I(a.Vy, ix + 1, iy + 1, nx) - A2I(a.Vy, ix, iy + 1, nx)) * a._dx);
            a.txy[k] = a.aTc[k] * a.txy[k] + a.bTc[k] * e;
        }
    }
    if constexpr (STORE) {
        if (a.red) apt_block_add(sabs, a.red + 2);
    }
}

// compute_R_V! and the free-slip copies: face residuals, V += dτV R (UPDATE) and bc_y!(Vx),
// bc_x!(Vy). DEFECT adds the outer state's FP64 residual as source. STORE: write Rx, Ry (and add
// Σ|Rx|, Σ|Ry| to red).
template <typename T, bool DEFECT, bool STORE, bool UPDATE, typename I>
__global__ void __launch_bounds__(256) apt_faces_k(AptArrays<T> a) {
    grid_dependency_wait();  // τ and Pt of the cells kernel
    grid_dependents_may_launch();
    const I ix = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x, iy = (I)blockIdx.y * (I)blockDim.y + (I)threadIdx.y;
    const I nx = (I)a.nx, ny = (I)a.ny;
    const T h = (T)0.5;
    double sx = 0.0, sy = 0.0;
    if (ix < nx - 1 && iy < ny - 2) {
        const I k = ix + (nx - 1) * iy;
        T R = ((A2I(a.txx, ix + 1, iy + 1, nx) - A2I(a.txx, ix, iy + 1, nx)) * a._dx +
               (A2I(a.txy, ix, iy + 1, nx - 1) - A2I(a.txy, ix, iy, nx - 1)) * a._dy) -
              (A2I(a.Pt, ix + 1, iy + 1, nx) - A2I(a.Pt, ix, iy + 1, nx)) * a._dx;
        if constexpr (DEFECT) R = R + a.rx0[k];
        if constexpr (STORE) {
            a.Rx[k] = R;
            sx = fabs((double)R);
        }
        if constexpr (UPDATE) {
            const T v = A2I(a.Vx, ix + 1, iy + 1, nx + 1) + a.dtVx[k] * R;
            A2I(a.Vx, ix + 1, iy + 1, nx + 1) = v;
            if (iy == 0) A2I(a.Vx, ix + 1, 0, nx + 1) = v;
            if (iy == ny - 3) A2I(a.Vx, ix + 1, ny - 1, nx + 1) = v;
        }
    }
    if (ix < nx - 2 && iy < ny - 1) {
        const I k = ix + (nx - 2) * iy;
        T R = (((A2I(a.tyy, ix + 1, iy + 1, nx) - A2I(a.tyy, ix + 1, iy, nx)) * a._dy +
                (A2I(a.txy, ix + 1, iy, nx - 1) - A2I(a.txy, ix, iy, nx - 1)) * a._dx) -
               (A2I(a.Pt, ix + 1, iy + 1, nx) - A2I(a.Pt, ix + 1, iy, nx)) * a._dy);
        if constexpr (DEFECT)
            R = R + a.ry0[k];
        else
            R = R + (A2I(a.Rog, ix + 1, iy, nx) + A2I(a.Rog, ix + 1, iy + 1, nx)) * h;
        if constexpr (STORE) {
            a.Ry[k] = R;
            sy = fabs((double)R);
        }
        if constexpr (UPDATE) {
            const T v = A2I(a.Vy, ix + 1, iy + 1, nx) + a.dtVy[k] * R;
            A2I(a.Vy, ix + 1, iy + 1, nx) = v;
            if (ix == 0) A2I(a.Vy, 0, iy + 1, nx) = v;
            if (ix == nx - 3) A2I(a.Vy, nx - 1, iy + 1, nx) = v;
        }
    }
    if constexpr (UPDATE) {
        if (ix == 0 && iy == 0) {  // the copies of the lines that are never updated
            A2I(a.Vx, 0, 0, nx + 1) = A2I(a.Vx, 0, 1, nx + 1);
            A2I(a.Vx, 0, ny - 1, nx + 1) = A2I(a.Vx, 0, ny - 2, nx + 1);
            A2I(a.Vx, nx, 0, nx + 1) = A2I(a.Vx, nx, 1, nx + 1);
            A2I(a.Vx, nx, ny - 1, nx + 1) = A2I(a.Vx, nx, ny - 2, nx + 1);
            A2I(a.Vy, 0, 0, nx) = A2I(a.Vy, 1, 0, nx);
            A2I(a.Vy, nx - 1, 0, nx) = A2I(a.Vy, nx - 2, 0, nx);
            A2I(a.Vy, 0, ny, nx) = A2I(a.Vy, 1, ny, nx);
            A2I(a.Vy, nx - 1, ny, nx) = A2I(a.Vy, nx - 2, ny, nx);
        }
    }
    if constexpr (STORE) {
        if (a.red) apt_block_add(sx, a.red, sy, a.red + 1);
    }
}

// FP64 residual of the state: τ at its steady state 2μ(ε̇ - ∇V/3) into txx/tyy/txy (the given
// arrays), ∇V into divV; then apt_faces_k<double, false, true, false, I> gives Rx, Ry.
__global__ void __launch_bounds__(256) apt_res_cells_k(AptArrays<double> a, const double* __restrict__ Mus) {
    const int64_t ix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, iy = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    const int64_t nx = a.nx, ny = a.ny;
    double sabs = 0.0;
    if (ix < nx && iy < ny) {
        const int64_t c = ix + nx * iy;
        const double dvx = A2(a.Vx, ix + 1, iy, nx + 1) - A2(a.Vx, ix, iy, nx + 1);
        const double dvy = A2(a.Vy, ix, iy + 1, nx) - A2(a.Vy, ix, iy, nx);
        const double d = dvx * a._dx + dvy * a._dy;
        const double td = d * (1.0 / 3.0);
        a.divV[c] = d;
        sabs = fabs(d);
        a.txx[c] = (2.0 * Mus[c]) * (dvx * a._dx - td);
        a.tyy[c] = (2.0 * Mus[c]) * (dvy * a._dy - td);
        if (ix < nx - 1 && iy < ny - 1) {
            const double mc = (((A2(Mus, ix, iy, nx) + A2(Mus, ix + 1, iy, nx)) + A2(Mus, ix, iy + 1, nx)) +
                               A2(Mus, ix + 1, iy + 1, nx)) *
                              0.25;
            const double e = 0.5 * ((A2(a.Vx, ix + 1, iy + 1, nx + 1) - A2(a.Vx, ix + 1, iy, nx + 1)) * a._dy +
                                    (A2(a.Vy, ix + 1, iy + 1, nx) - A2(a.Vy, ix, iy + 1, nx)) * a._dx);
            a.txy[ix + (nx - 1) * iy] = (2.0 * mc) * e;
        }
    }
    if (a.red) apt_block_add(sabs, a.red + 2);
}

// out = (D)in elementwise; x += d (FP64 += FP32)
template <typename D, typename S>
__global__ void apt_convert_k(D* __restrict__ out, const S* __restrict__ in, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (D)in[i];
}
__global__ void apt_add_k(double* __restrict__ x, const float* __restrict__ d, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = x[i] + (double)d[i];
}

// ---------------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------------
template <typename T>
static T* AP(const ps_array& a) {
    return static_cast<T*>(a.ptr);
}

static int check2(const ps_array& a, int64_t n0, int64_t n1, int32_t dt, const char* name) {
    PS_TRY(check_array(a, name));
    if (a.dtype != dt) return fail(PS_ERR_DTYPE, "%s: all Stokes2D arrays must have the same dtype", name);
    return check_shape(a, n0, n1, 1, name);
}

static int check_apt(const ps_stokes2d_apt_fields* f, int64_t* nx, int64_t* ny) {
    if (!f) return fail(PS_ERR_NULL, "NULL fields");
    const int64_t X = f->Pt.n[0], Y = f->Pt.n[1];
    if (X < 3 || Y < 3) return fail(PS_ERR_SHAPE, "Stokes2D needs nx, ny >= 3 (got %lld x %lld)", (long long)X, (long long)Y);
    const int32_t dt = f->Pt.dtype;
    if (dt != PS_F64 && dt != PS_F32) return fail(PS_ERR_DTYPE, "Stokes2D arrays must be FP64 or FP32");
    const struct {
        const ps_array* a;
        int64_t n0, n1;
        const char* name;
    } spec[] = {{&f->Pt, X, Y, "Pt"},         {&f->divV, X, Y, "divV"},         {&f->Vx, X + 1, Y, "Vx"},
                {&f->Vy, X, Y + 1, "Vy"},     {&f->txx, X, Y, "txx"},           {&f->tyy, X, Y, "tyy"},
                {&f->txy, X - 1, Y - 1, "txy"}, {&f->Rx, X - 1, Y - 2, "Rx"},   {&f->Ry, X - 2, Y - 1, "Ry"},
                {&f->Mus, X, Y, "Mus"},       {&f->Rog, X, Y, "Rog"},           {&f->Must, X, Y, "Must"},
                {&f->kP, X, Y, "kP"},         {&f->aT, X, Y, "aT"},             {&f->bT, X, Y, "bT"},
                {&f->aTc, X - 1, Y - 1, "aTc"}, {&f->bTc, X - 1, Y - 1, "bTc"}, {&f->dtVx, X - 1, Y - 2, "dtVx"},
                {&f->dtVy, X - 2, Y - 1, "dtVy"}};
    for (const auto& s : spec) PS_TRY(check2(*s.a, s.n0, s.n1, dt, s.name));
    *nx = X;
    *ny = Y;
    return PS_OK;
}

static int check_apt_params(const ps_stokes2d_apt_params* p) {
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    if (!(p->dx > 0) || !(p->dy > 0) || !(p->Vpdt > 0) || !(p->Re > 0) || !(p->r > 0) || !(p->max_lxy > 0))
        return fail(PS_ERR_ARG, "Stokes2D APT parameters must be positive");
    return PS_OK;
}

static dim3 apt_grid(int64_t wx, int64_t wy, dim3 b) {
    return dim3((unsigned)((wx + b.x - 1) / b.x), (unsigned)((wy + b.y - 1) / b.y), 1);
}

template <typename T>
static AptArrays<T> apt_arrays(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p) {
    AptArrays<T> a{};
    a.Vx = AP<T>(f->Vx);
    a.Vy = AP<T>(f->Vy);
    a.Pt = AP<T>(f->Pt);
    a.txx = AP<T>(f->txx);
    a.tyy = AP<T>(f->tyy);
    a.txy = AP<T>(f->txy);
    a.divV = AP<T>(f->divV);
    a.Rx = AP<T>(f->Rx);
    a.Ry = AP<T>(f->Ry);
    a.kP = AP<T>(f->kP);
    a.aT = AP<T>(f->aT);
    a.bT = AP<T>(f->bT);
    a.aTc = AP<T>(f->aTc);
    a.bTc = AP<T>(f->bTc);
    a.dtVx = AP<T>(f->dtVx);
    a.dtVy = AP<T>(f->dtVy);
    a.Rog = AP<T>(f->Rog);
    a.nx = f->Pt.n[0];
    a.ny = f->Pt.n[1];
    a._dx = (T)(1.0 / p->dx);
    a._dy = (T)(1.0 / p->dy);
    return a;
}

static bool apt_i32(int64_t nx, int64_t ny) {  // 32-bit indices: every array and offset below 2^31
    return (nx + 1 + 32) * (ny + 1 + 8) < ((int64_t)1 << 31);
}

template <typename T, bool DEFECT, bool STORE, typename I>
static void apt_launch_iteration_i(const AptArrays<T>& a, cudaStream_t s, bool after_kernel) {
    const dim3 blk(32, 8);
    const dim3 grd = apt_grid(a.nx, a.ny, blk);
    // each kernel may start while the kernel before it ends (programmatic dependent launch; it waits
    // for that kernel's stores before reading); after_kernel = false: the stream's last operation
    // is not one of these kernels (a memset, a copy, the start of a captured graph)
    if (!after_kernel) {
        apt_cells_k<T, DEFECT, STORE, I><<<grd, blk, 0, s>>>(a);
    } else if (launch_dependent(apt_cells_k<T, DEFECT, STORE, I>, grd, blk, 0, s, a) != cudaSuccess) {
        cudaGetLastError();
        apt_cells_k<T, DEFECT, STORE, I><<<grd, blk, 0, s>>>(a);
    }
    if (launch_dependent(apt_faces_k<T, DEFECT, STORE, true, I>, grd, blk, 0, s, a) != cudaSuccess) {
        cudaGetLastError();
        apt_faces_k<T, DEFECT, STORE, true, I><<<grd, blk, 0, s>>>(a);
    }
}

template <typename T, bool DEFECT, bool STORE>
static void apt_launch_iteration(const AptArrays<T>& a, cudaStream_t s, bool after_kernel = true) {
    if (apt_i32(a.nx, a.ny))
        apt_launch_iteration_i<T, DEFECT, STORE, int>(a, s, after_kernel);
    else
        apt_launch_iteration_i<T, DEFECT, STORE, int64_t>(a, s, after_kernel);
}

template <typename T>
static int apt_coefficients(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, cudaStream_t s) {
    const int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    AptCoeffParams c{(p->Vpdt * p->max_lxy) / p->Re, p->Vpdt * p->Vpdt, p->r + 2.0, p->r};
    const dim3 blk(32, 8);
    const dim3 grd = apt_grid(nx, ny, blk);
    apt_must_k<T><<<grd, blk, 0, s>>>(AP<T>(f->Mus), AP<T>(f->Must), nx, ny);
    apt_coeffs_k<T><<<grd, blk, 0, s>>>(AP<T>(f->Mus), AP<T>(f->Must), AP<T>(f->kP), AP<T>(f->aT), AP<T>(f->bT),
                                        AP<T>(f->aTc), AP<T>(f->bTc), AP<T>(f->dtVx), AP<T>(f->dtVy), nx, ny, c);
    return PS_OK;
}

// FP64 residual of (Vx, Vy, Pt): τ* into tau[3], ∇V / Rx / Ry into the given arrays, sums into red.
static void apt_residual64(AptArrays<double> a, const double* Mus, double* const tau[3], double* red, cudaStream_t s) {
    a.txx = tau[0];
    a.tyy = tau[1];
    a.txy = tau[2];
    a.red = red;
    const dim3 blk(32, 8);
    const dim3 grd = apt_grid(a.nx, a.ny, blk);
    cudaMemsetAsync(red, 0, 3 * sizeof(double), s);
    apt_res_cells_k<<<grd, blk, 0, s>>>(a, Mus);
    if (apt_i32(a.nx, a.ny))
        apt_faces_k<double, false, true, false, int><<<grd, blk, 0, s>>>(a);
    else
        apt_faces_k<double, false, true, false, int64_t><<<grd, blk, 0, s>>>(a);
}

static double apt_err(const double h[3], int64_t nx, int64_t ny) {
    const double nrx = (double)((nx - 1) * (ny - 2)), nry = (double)((nx - 2) * (ny - 1)), nd = (double)(nx * ny);
    if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2])) return NAN;
    return std::max(std::max(h[0] / nrx, h[1] / nry), h[2] / nd);
}

// Graph of `nout` iterations; with store_last the last one stores ∇V, Rx, Ry and their sums.
template <typename T, bool DEFECT>
struct AptGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int build(const AptArrays<T>& a, int64_t nout, bool store_last, double* red, cudaStream_t s) {
        PS_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        if (store_last) cudaMemsetAsync(red, 0, 3 * sizeof(double), s);
        for (int64_t it = 0; it < nout; ++it) {
            if (store_last && it == nout - 1) {
                AptArrays<T> b = a;
                b.red = red;
                apt_launch_iteration<T, DEFECT, true>(b, s, it > 0);
            } else {
                apt_launch_iteration<T, DEFECT, false>(a, s, it > 0);
            }
        }
        PS_CUDA_TRY(cudaStreamEndCapture(s, &graph));
        PS_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
        return PS_OK;
    }
    ~AptGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t bytes) {
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return fail(PS_ERR_NOMEM, "Stokes2D APT solver: scratch allocation of %zu bytes failed", bytes);
        }
        return PS_OK;
    }
};

static int apt_solve_fp64(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, double tol,
                          int64_t max_iter, int64_t nout, double max_seconds, ps_solve_stats* st, cudaStream_t s) {
    const int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    const size_t bc = ((size_t)nx * ny * 8 + 255) / 256 * 256, bk = (size_t)(nx - 1) * (ny - 1) * 8;
    DevBuf buf;
    PS_TRY(buf.alloc(256 + 2 * bc + bk));
    char* c = static_cast<char*>(buf.p);
    double* red = reinterpret_cast<double*>(c);
    double* const tau[3] = {reinterpret_cast<double*>(c + 256), reinterpret_cast<double*>(c + 256 + bc),
                            reinterpret_cast<double*>(c + 256 + 2 * bc)};
    AptArrays<double> a = apt_arrays<double>(f, p);
    AptGraph<double, false> g;
    PS_TRY(g.build(a, nout, false, nullptr, s));
    const double t0 = apt_now();
    double h[3], err = INFINITY;
    int64_t it = 0;
    int rc = PS_OK;
    for (;;) {
        apt_residual64(a, AP<double>(f->Mus), tau, red, s);
        PS_TRY(read_device_words(h, red, sizeof(h), s));
        err = apt_err(h, nx, ny);
        if (std::isnan(err)) {
            rc = fail(PS_ERR_NONFINITE, "ps_stokes2d_apt_solve: non-finite residual after %lld iterations", (long long)it);
            break;
        }
        if (err < tol) break;
        if (it >= max_iter) {
            rc = fail(PS_ERR_NOT_CONVERGED, "ps_stokes2d_apt_solve: err %.3e after %lld iterations", err, (long long)it);
            break;
        }
        if (max_seconds > 0 && apt_now() - t0 > max_seconds) {
            rc = fail(PS_ERR_TIMEOUT, "ps_stokes2d_apt_solve: wall-clock limit reached (err %.3e)", err);
            break;
        }
        PS_CUDA_TRY(cudaGraphLaunch(g.exec, s));
        it += nout;
    }
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    st->iters = it;
    st->outer = 1;
    st->err = err;
    st->seconds = apt_now() - t0;
    st->converged = rc == PS_OK;
    return rc;
}

// Defect correction: FP32 APT sweeps on (δV, δP, δτ) with the FP64 residual of the state as
// source, then V += δV, P += δP in FP64.
static int apt_solve_mixed(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, double tol,
                           int64_t max_iter, int64_t nout, double max_seconds, double inner_rtol, ps_solve_stats* st,
                           cudaStream_t s) {
    const int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    const int64_t n_c = nx * ny, n_k = (nx - 1) * (ny - 1), n_x = (nx - 1) * (ny - 2), n_y = (nx - 2) * (ny - 1),
                  n_vx = (nx + 1) * ny, n_vy = nx * (ny + 1);
    // float arrays: coefficients (7), correction state (6), stored ∇V / Rx / Ry (3), sources (3)
    const int64_t counts[] = {n_c,  n_c,  n_c, n_k, n_k, n_x, n_y,  // kP aT bT aTc bTc dtVx dtVy
                              n_vx, n_vy, n_c, n_c, n_c, n_k,       // δVx δVy δP δτxx δτyy δτxy
                              n_c,  n_x,  n_y,                      // ∇V Rx Ry
                              n_c,  n_x,  n_y};                     // div0 rx0 ry0
    constexpr int NA = sizeof(counts) / sizeof(counts[0]);
    size_t off[NA + 1];
    off[0] = 256;
    for (int i = 0; i < NA; i++) off[i + 1] = off[i] + ((size_t)counts[i] * 4 + 255) / 256 * 256;
    DevBuf buf;
    PS_TRY(buf.alloc(off[NA]));
    char* c = static_cast<char*>(buf.p);
    auto F = [&](int i) { return reinterpret_cast<float*>(c + off[i]); };
    double* red_out = reinterpret_cast<double*>(c);
    double* red_in = red_out + 4;
    const int g = 1024;
    const ps_array* src[7] = {&f->kP, &f->aT, &f->bT, &f->aTc, &f->bTc, &f->dtVx, &f->dtVy};
    for (int i = 0; i < 7; i++) apt_convert_k<float, double><<<g, 256, 0, s>>>(F(i), AP<double>(*src[i]), counts[i]);

    AptArrays<double> a64 = apt_arrays<double>(f, p);
    AptArrays<float> d{};
    d.kP = F(0);
    d.aT = F(1);
    d.bT = F(2);
    d.aTc = F(3);
    d.bTc = F(4);
    d.dtVx = F(5);
    d.dtVy = F(6);
    d.Vx = F(7);
    d.Vy = F(8);
    d.Pt = F(9);
    d.txx = F(10);
    d.tyy = F(11);
    d.txy = F(12);
    d.divV = F(13);
    d.Rx = F(14);
    d.Ry = F(15);
    d.div0 = F(16);
    d.rx0 = F(17);
    d.ry0 = F(18);
    d.Rog = nullptr;
    d.nx = nx;
    d.ny = ny;
    d._dx = (float)(1.0 / p->dx);
    d._dy = (float)(1.0 / p->dy);
    AptGraph<float, true> gr;
    PS_TRY(gr.build(d, nout, true, red_in, s));
    // the residual's stresses go to the caller's τ arrays (this solver keeps no stress state)
    double* const tau[3] = {AP<double>(f->txx), AP<double>(f->tyy), AP<double>(f->txy)};

    const double t0 = apt_now();
    double h[3], err = INFINITY;
    int64_t it = 0, outer = 0;
    int rc = PS_OK;
    for (;;) {
        apt_residual64(a64, AP<double>(f->Mus), tau, red_out, s);
        PS_TRY(read_device_words(h, red_out, sizeof(h), s));
        err = apt_err(h, nx, ny);
        if (std::isnan(err)) {
            rc = fail(PS_ERR_NONFINITE, "ps_stokes2d_apt_solve: non-finite FP64 residual");
            break;
        }
        if (err < tol) break;
        if (it >= max_iter) {
            rc = fail(PS_ERR_NOT_CONVERGED, "ps_stokes2d_apt_solve: err %.3e after %lld iterations", err, (long long)it);
            break;
        }
        if (max_seconds > 0 && apt_now() - t0 > max_seconds) {
            rc = fail(PS_ERR_TIMEOUT, "ps_stokes2d_apt_solve: wall-clock limit reached (err %.3e)", err);
            break;
        }
        ++outer;
        apt_convert_k<float, double><<<g, 256, 0, s>>>(F(16), AP<double>(f->divV), n_c);
        apt_convert_k<float, double><<<g, 256, 0, s>>>(F(17), AP<double>(f->Rx), n_x);
        apt_convert_k<float, double><<<g, 256, 0, s>>>(F(18), AP<double>(f->Ry), n_y);
        cudaMemsetAsync(c + off[7], 0, off[13] - off[7], s);  // δVx, δVy, δP, δτ from zero
        const double target = std::max(err * inner_rtol, tol * 0.25);
        // APT residuals oscillate while they decay, and pseudo-time waves need ~n iterations to
        // cross the grid: the sweep stops at the target, or -- after at least 20 n iterations --
        // when the best error has not improved by 2 % over the last 4 n iterations (FP32
        // stagnation), n = max(nx, ny)
        const int64_t nmax = std::max(nx, ny), min_sweep = 20 * nmax;
        const int64_t stale_checks = std::max<int64_t>(10, (4 * nmax + nout - 1) / nout);
        double ierr = INFINITY, best = INFINITY;
        int64_t stale = 0, swept = 0;
        while (it < max_iter) {
            PS_CUDA_TRY(cudaGraphLaunch(gr.exec, s));
            it += nout;
            swept += nout;
            PS_TRY(read_device_words(h, red_in, sizeof(h), s));
            ierr = apt_err(h, nx, ny);
            if (std::isnan(ierr)) break;
            if (ierr < target) break;
            if (ierr < 0.98 * best) {
                best = ierr;
                stale = 0;
            } else if (++stale >= stale_checks && swept >= min_sweep) {
                break;
            }
            if (max_seconds > 0 && apt_now() - t0 > max_seconds) break;
        }
        if (std::isnan(ierr)) {
            rc = fail(PS_ERR_NONFINITE, "ps_stokes2d_apt_solve: non-finite FP32 correction");
            break;
        }
        apt_add_k<<<g, 256, 0, s>>>(AP<double>(f->Vx), F(7), n_vx);
        apt_add_k<<<g, 256, 0, s>>>(AP<double>(f->Vy), F(8), n_vy);
        apt_add_k<<<g, 256, 0, s>>>(AP<double>(f->Pt), F(9), n_c);
    }
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    st->iters = it;
    st->outer = outer;
    st->err = err;
    st->seconds = apt_now() - t0;
    st->converged = rc == PS_OK;
    return rc;
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_stokes2d_apt_coefficients(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, void* stream,
                                 int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_apt(f, &nx, &ny));
    PS_TRY(check_apt_params(p));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PS_TRY(f->Pt.dtype == PS_F64 ? apt_coefficients<double>(f, p, s) : apt_coefficients<float>(f, p, s));
    return finish_launch(s, sync, "ps_stokes2d_apt_coefficients");
}

int ps_stokes2d_apt_iterate(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, int64_t n_iter,
                            void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_apt(f, &nx, &ny));
    PS_TRY(check_apt_params(p));
    if (n_iter < 0) return fail(PS_ERR_ARG, "n_iter must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int64_t it = 0; it < n_iter; ++it) {
        if (f->Pt.dtype == PS_F64)
            apt_launch_iteration<double, false, true>(apt_arrays<double>(f, p), s, it > 0);
        else
            apt_launch_iteration<float, false, true>(apt_arrays<float>(f, p), s, it > 0);
    }
    return finish_launch(s, 1, "ps_stokes2d_apt_iterate");
}

int ps_stokes2d_apt_residual(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, double out_mean_abs[3],
                             void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_apt(f, &nx, &ny));
    PS_TRY(check_apt_params(p));
    if (!out_mean_abs) return fail(PS_ERR_NULL, "NULL output");
    if (f->Pt.dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_stokes2d_apt_residual: FP64 fields only");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* red = st->d_scratch;
    double* const tau[3] = {AP<double>(f->txx), AP<double>(f->tyy), AP<double>(f->txy)};
    apt_residual64(apt_arrays<double>(f, p), AP<double>(f->Mus), tau, red, s);
    PS_CUDA_TRY(cudaGetLastError());
    double h[3];
    PS_TRY(read_device_words(h, red, sizeof(h), s));
    out_mean_abs[0] = h[0] / (double)((nx - 1) * (ny - 2));
    out_mean_abs[1] = h[1] / (double)((nx - 2) * (ny - 1));
    out_mean_abs[2] = h[2] / (double)(nx * ny);
    return finish_launch(s, 1, "ps_stokes2d_apt_residual");
}

int ps_stokes2d_apt_solve(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, int32_t mode, double tol,
                          int64_t max_iter, int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_apt(f, &nx, &ny));
    PS_TRY(check_apt_params(p));
    if (!stats) return fail(PS_ERR_NULL, "NULL stats");
    if (f->Pt.dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_stokes2d_apt_solve: FP64 fields (mode 1 sweeps FP32 itself)");
    if (nout < 1) return fail(PS_ERR_ARG, "nout must be >= 1");
    if (!(tol > 0) || max_iter < 0) return fail(PS_ERR_ARG, "invalid tol / max_iter");
    if (mode != 0 && mode != 1) return fail(PS_ERR_ARG, "mode must be 0 (FP64) or 1 (FP32 + FP64 defect correction)");
    memset(stats, 0, sizeof(*stats));
    // graphs are captured on a private stream ordered after `stream`
    cudaStream_t user = static_cast<cudaStream_t>(stream), s;
    PS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t ev;
    PS_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(s, ev, 0);
    int rc = apt_coefficients<double>(f, p, s);
    if (rc == PS_OK)
        rc = mode == 0 ? apt_solve_fp64(f, p, tol, max_iter, nout, max_seconds, stats, s)
                       : apt_solve_mixed(f, p, tol, max_iter, nout, max_seconds, 1e-3, stats, s);
    cudaStreamSynchronize(s);
    cudaEventDestroy(ev);
    cudaStreamDestroy(s);
    cudaGetLastError();
    return rc;
}

}  // extern "C"
