// ps_stokes2d.cu -- pseudo-transient (PT) viscous Stokes 2-D kernels and solvers of libps_b200.so.
//
// Reference: miniapps/Stokes2D.jl:11-55 (kernels), :107-125 (PT loop), :117-123 (error check).
//
//   s2_* device functions     the arithmetic of each reference statement, shared by every kernel
//                             below so all paths round identically
//   one-to-one kernels        compute_timesteps!, compute_P!, compute_τ!, compute_dV!, compute_V!,
//                             bc_x!, bc_y! -- the drop-in replacements of the six `@parallel` calls
//   s2_fused                  one whole PT iteration in one kernel: a CTA stages its tile of
//                             Vx, Vy, Pt, Mus (+1-2 cell halo) in shared memory, recomputes the halo
//                             of ∇V / Pt / τ, updates dVdτ and V of its own faces and applies the
//                             free-slip copies. Old/new V and Pt are ping-pong buffers, so results are
//                             identical to the six-kernel sequence. Optional fused FP64 reduction of
//                             Σ|Rx|, Σ|Ry|, Σ|∇V| (warp shuffles + one atomicAdd per block).
//   s2_residual64             FP64 residuals of the current state (no pseudo-time update) for the
//                             defect-correction outer loop.
//   ps_stokes2d_solve         PT solve to `tol` in FP64 (mode 0) or with FP32 PT sweeps on the
//                             correction and an FP64 residual / update / convergence check (mode 1).
//                             Iterations run as CUDA graphs of `nout` fused kernels.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <vector>

#include "ps_common.cuh"

namespace ps {

// =======================================================================================
// Statement arithmetic (Stokes2D.jl:11-37); literals cast to T like the reference does.
// =======================================================================================
template <typename T>
__host__ __device__ __forceinline__ T s2_dtV(T Vsc, T min_dxy2, T m0, T m1) {
    T av = (m0 + m1) * T(0.5);
    return ((Vsc * min_dxy2) / av) / T(4.1);
}
template <typename T>
__host__ __device__ __forceinline__ T s2_dtPt(T Ptsc, T mus, T max_nxy) {
    return ((Ptsc * T(4.1)) * mus) / max_nxy;
}
// H: the divisor's type -- T, or DivC<T> (the correctly rounded division by a host-known number)
template <typename T, typename H>
__host__ __device__ __forceinline__ T s2_divV(T vx0, T vx1, T vy0, T vy1, H dx, H dy) {
    return dvd(vx1 - vx0, dx) + dvd(vy1 - vy0, dy);
}
template <typename T, typename H>
__host__ __device__ __forceinline__ T s2_tau_nn(T mus, T v0, T v1, T divV, H h) {
    return (T(2.0) * mus) * (dvd(v1 - v0, h) - (T(1.0) / T(3.0)) * divV);
}
template <typename T, typename H>
__host__ __device__ __forceinline__ T s2_tau_xy(T m00, T m10, T m01, T m11, T dyVx, T dxVy, H dx, H dy) {
    T av = (((m00 + m10) + m01) + m11) * T(0.25);
    return (T(2.0) * av) * (T(0.5) * (dvd(dyVx, dy) + dvd(dxVy, dx)));
}
template <typename T, typename H>
__host__ __device__ __forceinline__ T s2_Rx(T txx_l, T txx_r, T txy_b, T txy_t, T p_l, T p_r, H dx, H dy) {
    return (dvd(txx_r - txx_l, dx) + dvd(txy_t - txy_b, dy)) - dvd(p_r - p_l, dx);
}
template <typename T, typename H>
__host__ __device__ __forceinline__ T s2_Ry_core(T tyy_b, T tyy_t, T txy_l, T txy_r, T p_b, T p_t, H dx, H dy) {
    return (dvd(tyy_t - tyy_b, dy) + dvd(txy_r - txy_l, dx)) - dvd(p_t - p_b, dy);
}

template <typename T>
struct S2P {
    DivC<T> dx, dy;
    T dampX, dampY, Vsc, Ptsc, min_dxy2, max_nxy;
};

template <typename T>
static S2P<T> s2p(const ps_stokes2d_params& p) {
    return S2P<T>{make_div((T)p.dx), make_div((T)p.dy), (T)p.dampX,    (T)p.dampY,
                  (T)p.Vsc,          (T)p.Ptsc,         (T)p.min_dxy2, (T)p.max_nxy};
}

#define A2(a, i, j, n0) (a)[(int64_t)(i) + (int64_t)(n0) * (int64_t)(j)]

// =======================================================================================
// One-to-one kernels (grid = max extents of the kernel's array arguments).
// =======================================================================================
template <typename T>
__global__ void s2_timesteps_k(T* dtVx, T* dtVy, T* dtPt, const T* __restrict__ Mus, int64_t nx, int64_t ny, S2P<T> p) {
    int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx >= nx || ty >= ny) return;
    if (tx < nx - 1 && ty < ny - 2)
        A2(dtVx, tx, ty, nx - 1) = s2_dtV(p.Vsc, p.min_dxy2, A2(Mus, tx, ty + 1, nx), A2(Mus, tx + 1, ty + 1, nx));
    if (tx < nx - 2 && ty < ny - 1)
        A2(dtVy, tx, ty, nx - 2) = s2_dtV(p.Vsc, p.min_dxy2, A2(Mus, tx + 1, ty, nx), A2(Mus, tx + 1, ty + 1, nx));
    A2(dtPt, tx, ty, nx) = s2_dtPt(p.Ptsc, A2(Mus, tx, ty, nx), p.max_nxy);
}

template <typename T>
__global__ void s2_P_k(T* divV, T* Pt, const T* __restrict__ Vx, const T* __restrict__ Vy, const T* __restrict__ dtPt,
                       int64_t nx, int64_t ny, S2P<T> p) {
    int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx >= nx || ty >= ny) return;
    T d = s2_divV(A2(Vx, tx, ty, nx + 1), A2(Vx, tx + 1, ty, nx + 1), A2(Vy, tx, ty, nx), A2(Vy, tx, ty + 1, nx), p.dx, p.dy);
    A2(divV, tx, ty, nx) = d;
    A2(Pt, tx, ty, nx) = A2(Pt, tx, ty, nx) - A2(dtPt, tx, ty, nx) * d;
}

template <typename T>
__global__ void s2_tau_k(const T* __restrict__ divV, T* txx, T* tyy, T* txy, const T* __restrict__ Vx,
                         const T* __restrict__ Vy, const T* __restrict__ Mus, int64_t nx, int64_t ny, S2P<T> p) {
    int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx >= nx || ty >= ny) return;
    T m = A2(Mus, tx, ty, nx), d = A2(divV, tx, ty, nx);
    A2(txx, tx, ty, nx) = s2_tau_nn(m, A2(Vx, tx, ty, nx + 1), A2(Vx, tx + 1, ty, nx + 1), d, p.dx);
    A2(tyy, tx, ty, nx) = s2_tau_nn(m, A2(Vy, tx, ty, nx), A2(Vy, tx, ty + 1, nx), d, p.dy);
    if (tx < nx - 1 && ty < ny - 1)
        A2(txy, tx, ty, nx - 1) =
            s2_tau_xy(A2(Mus, tx, ty, nx), A2(Mus, tx + 1, ty, nx), A2(Mus, tx, ty + 1, nx), A2(Mus, tx + 1, ty + 1, nx),
                      A2(Vx, tx + 1, ty + 1, nx + 1) - A2(Vx, tx + 1, ty, nx + 1),
                      A2(Vy, tx + 1, ty + 1, nx) - A2(Vy, tx, ty + 1, nx), p.dx, p.dy);
}

template <typename T>
__global__ void s2_dV_k(T* Rx, T* Ry, T* dVxdt, T* dVydt, const T* __restrict__ Pt, const T* __restrict__ Rog,
                        const T* __restrict__ txx, const T* __restrict__ tyy, const T* __restrict__ txy, int64_t nx,
                        int64_t ny, S2P<T> p) {
    int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx >= nx || ty >= ny) return;
    if (tx < nx - 1 && ty < ny - 2) {
        T r = s2_Rx(A2(txx, tx, ty + 1, nx), A2(txx, tx + 1, ty + 1, nx), A2(txy, tx, ty, nx - 1),
                    A2(txy, tx, ty + 1, nx - 1), A2(Pt, tx, ty + 1, nx), A2(Pt, tx + 1, ty + 1, nx), p.dx, p.dy);
        A2(Rx, tx, ty, nx - 1) = r;
        A2(dVxdt, tx, ty, nx - 1) = p.dampX * A2(dVxdt, tx, ty, nx - 1) + r;
    }
    if (tx < nx - 2 && ty < ny - 1) {
        T r = s2_Ry_core(A2(tyy, tx + 1, ty, nx), A2(tyy, tx + 1, ty + 1, nx), A2(txy, tx, ty, nx - 1),
                         A2(txy, tx + 1, ty, nx - 1), A2(Pt, tx + 1, ty, nx), A2(Pt, tx + 1, ty + 1, nx), p.dx, p.dy) +
              (A2(Rog, tx + 1, ty, nx) + A2(Rog, tx + 1, ty + 1, nx)) * T(0.5);
        A2(Ry, tx, ty, nx - 2) = r;
        A2(dVydt, tx, ty, nx - 2) = p.dampY * A2(dVydt, tx, ty, nx - 2) + r;
    }
}

template <typename T>
__global__ void s2_V_k(T* Vx, T* Vy, const T* __restrict__ dVxdt, const T* __restrict__ dVydt,
                       const T* __restrict__ dtVx, const T* __restrict__ dtVy, int64_t nx, int64_t ny) {
    int64_t tx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, ty = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    if (tx > nx || ty > ny) return;
    if (tx < nx - 1 && ty < ny - 2)
        A2(Vx, tx + 1, ty + 1, nx + 1) = A2(Vx, tx + 1, ty + 1, nx + 1) + A2(dtVx, tx, ty, nx - 1) * A2(dVxdt, tx, ty, nx - 1);
    if (tx < nx - 2 && ty < ny - 1)
        A2(Vy, tx + 1, ty + 1, nx) = A2(Vy, tx + 1, ty + 1, nx) + A2(dtVy, tx, ty, nx - 2) * A2(dVydt, tx, ty, nx - 2);
}

template <typename T>
__global__ void s2_bc_x_k(T* A, int64_t n0, int64_t n1) {
    int64_t iy = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (iy >= n1) return;
    A2(A, 0, iy, n0) = A2(A, 1, iy, n0);
    A2(A, n0 - 1, iy, n0) = A2(A, n0 - 2, iy, n0);
}
template <typename T>
__global__ void s2_bc_y_k(T* A, int64_t n0, int64_t n1) {
    int64_t ix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ix >= n0) return;
    A2(A, ix, 0, n0) = A2(A, ix, 1, n0);
    A2(A, ix, n1 - 1, n0) = A2(A, ix, n1 - 2, n0);
}

// =======================================================================================
// Fused PT iteration
// =======================================================================================
constexpr int S2_TX = 32;
// tile rows: FP64 16 (the halo it recomputes is FP64-pipe work: 0.366 -> 0.354 ms per 1023^2
// iteration), FP32 8 (16 measured slower there)
template <typename T>
__host__ __device__ constexpr int s2_ty() {
    return sizeof(T) == 8 ? 16 : 8;
}

template <typename T>
struct S2Fused {
    // state in / out (ping-pong) and in-place pseudo-velocities
    const T* Vx_in;
    const T* Vy_in;
    const T* P_in;
    T* Vx_out;
    T* Vy_out;
    T* P_out;
    T* dVxdt;
    T* dVydt;
    const T* Mus;
    const T* Rog;  // PLAIN: buoyancy (nx, ny); DEFECT: unused
    // pseudo-time steps read from arrays (drop-in) or recomputed from Mus (solver)
    const T* dtVx;
    const T* dtVy;
    const T* dtPt;
    // DEFECT sources (the FP64 residual of the outer state, rounded to T)
    const T* fp;  // (nx, ny)
    const T* fx;  // (nx-1, ny-2)
    const T* fy;  // (nx-2, ny-1)
    // temporaries of the reference (written only if STORE_TMP)
    T* divV;
    T* txx;
    T* tyy;
    T* txy;
    T* Rx;
    T* Ry;
    double* red;  // Σ|Rx|, Σ|Ry|, Σ|∇V| (NULL: no reduction)
    int64_t nx, ny;
};

template <typename T, typename I>
__device__ __forceinline__ T ldg_or0(const T* a, I i, I j, I n0, I n1) {
    return (i >= 0 && i < n0 && j >= 0 && j < n1) ? __ldg(a + i + n0 * j) : T(0);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// I: index type (int where every array has fewer than 2^31 elements: fewer instructions per cell).
// RED: a.red is set (the FP64 sums are compiled in only then: the conversions to double run on the
// FP64 pipe even when predicated off).
template <typename T, bool DEFECT, bool STORE_TMP, bool READ_DT, typename I, bool RED>
__global__ void __launch_bounds__(S2_TX* s2_ty<T>()) s2_fused(S2Fused<T> a, S2P<T> p) {
    constexpr int TX = S2_TX, TY = s2_ty<T>();
    constexpr int VW = TX + 2, VH = TY + 2;  // staged V / Mus window: [x0-1, x0+TX] x [y0-1, y0+TY]
    constexpr int CW = TX + 1, CH = TY + 1;  // computed cells / corners: [x0-1, x0+TX) x [y0-1, y0+TY)
    __shared__ T sVx[VH][VW], sVy[VH][VW], sMus[VH][VW];
    __shared__ T sP[CH][CW], sTxx[CH][CW], sTyy[CH][CW], sTxy[CH][CW];
    __shared__ double sred[3][TX * TY / 32];

    const I nx = (I)a.nx, ny = (I)a.ny;
    const int tid = threadIdx.y * TX + threadIdx.x;
    const I x0 = (I)blockIdx.x * TX, y0 = (I)blockIdx.y * TY;
    constexpr int NC = (CW * CH + TX * TY - 1) / (TX * TY);  // halo-window cells per thread

    // Every global load of the thread is issued before the first barrier (the staged window, the
    // cells' P / dtPt / defect source, the faces' dVdt / dt / sources), so one memory round trip
    // covers the iteration instead of three dependent ones.
    for (int k = tid; k < VW * VH; k += TX * TY) {
        int u = k % VW, v = k / VW;
        I gi = x0 - 1 + u, gj = y0 - 1 + v;
        sVx[v][u] = ldg_or0(a.Vx_in, gi, gj, nx + 1, ny);
        sVy[v][u] = ldg_or0(a.Vy_in, gi, gj, nx, ny + 1);
        sMus[v][u] = ldg_or0(a.Mus, gi, gj, nx, ny);
    }
    T c_p[NC], c_dt[NC], c_f[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const int k = tid + q * TX * TY;
        const I gi = x0 - 1 + k % CW, gj = y0 - 1 + k / CW;
        const bool in = k < CW * CH && gi >= 0 && gi < nx && gj >= 0 && gj < ny;
        c_p[q] = in ? __ldg(a.P_in + gi + nx * gj) : T(0);
        c_dt[q] = (READ_DT && in) ? __ldg(a.dtPt + gi + nx * gj) : T(0);
        c_f[q] = (DEFECT && in) ? __ldg(a.fp + gi + nx * gj) : T(0);
    }
    const int lx = threadIdx.x, ly = threadIdx.y;
    const I fi = x0 + lx, fj = y0 + ly;
    const bool xin = fi <= nx && fj < ny, xinner = fi >= 1 && fi <= nx - 1 && fj >= 1 && fj <= ny - 2;
    const bool yin = fi < nx && fj <= ny, yinner = fi >= 1 && fi <= nx - 2 && fj >= 1 && fj <= ny - 1;
    const I rxi = (fi - 1) + (nx - 1) * (fj - 1), ryi = (fi - 1) + (nx - 2) * (fj - 1);
    T x_dv = T(0), x_dt = T(0), x_f = T(0), y_dv = T(0), y_dt = T(0), y_f = T(0);
    if (xin && xinner) {
        x_dv = a.dVxdt[rxi];
        if constexpr (READ_DT) x_dt = __ldg(a.dtVx + rxi);
        if constexpr (DEFECT) x_f = __ldg(a.fx + rxi);
    }
    if (yin && yinner) {
        y_dv = a.dVydt[ryi];
        if constexpr (READ_DT) y_dt = __ldg(a.dtVy + ryi);
        if constexpr (DEFECT)
            y_f = __ldg(a.fy + ryi);
        else
            y_f = (__ldg(a.Rog + fi + nx * (fj - 1)) + __ldg(a.Rog + fi + nx * fj)) * T(0.5);
    }
    __syncthreads();

    double acc_div = 0.0;
    // cells and corners of the halo window
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const int k = tid + q * TX * TY;
        if (k >= CW * CH) break;
        int u = k % CW, v = k / CW;  // window cell (u, v) = global cell (x0-1+u, y0-1+v)
        I gi = x0 - 1 + u, gj = y0 - 1 + v;
        if (gi >= 0 && gi < nx && gj >= 0 && gj < ny) {
            T vx0 = sVx[v][u], vx1 = sVx[v][u + 1];  // Vx faces gi, gi+1 of row gj
            T vy0 = sVy[v][u], vy1 = sVy[v + 1][u];  // Vy faces gj, gj+1 of column gi
            T mus = sMus[v][u];
            T d = s2_divV(vx0, vx1, vy0, vy1, p.dx, p.dy);
            T dtp = READ_DT ? c_dt[q] : s2_dtPt(p.Ptsc, mus, p.max_nxy);
            T dp = d;
            if constexpr (DEFECT) dp = d + c_f[q];
            T pn = c_p[q] - dtp * dp;
            T txx = s2_tau_nn(mus, vx0, vx1, d, p.dx);
            T tyy = s2_tau_nn(mus, vy0, vy1, d, p.dy);
            sP[v][u] = pn;
            sTxx[v][u] = txx;
            sTyy[v][u] = tyy;
            bool own = u >= 1 && v >= 1;  // inside [x0, x0+TX) x [y0, y0+TY)
            if (own) {
                a.P_out[gi + nx * gj] = pn;
                if constexpr (STORE_TMP) {
                    a.divV[gi + nx * gj] = d;
                    a.txx[gi + nx * gj] = txx;
                    a.tyy[gi + nx * gj] = tyy;
                }
                if constexpr (RED) acc_div += fabs((double)dp);
            }
        }
        // corner (gi, gj): between cells gi..gi+1, gj..gj+1
        if (gi >= 0 && gi < nx - 1 && gj >= 0 && gj < ny - 1) {
            T t = s2_tau_xy(sMus[v][u], sMus[v][u + 1], sMus[v + 1][u], sMus[v + 1][u + 1],
                            sVx[v + 1][u + 1] - sVx[v][u + 1], sVy[v + 1][u + 1] - sVy[v + 1][u], p.dx, p.dy);
            sTxy[v][u] = t;
            if constexpr (STORE_TMP)
                if (u >= 1 && v >= 1) a.txy[gi + (nx - 1) * gj] = t;
        }
    }
    __syncthreads();

    // faces of this tile
    const int u = lx + 1, v = ly + 1;  // window coordinates of cell (fi, fj)
    double acc_rx = 0.0, acc_ry = 0.0;
    // ---- Vx face (fi, fj), Vx is (nx+1, ny) ----
    if (xin) {
        T vnew = sVx[v][u];
        if (xinner) {
            T r = s2_Rx(sTxx[v][u - 1], sTxx[v][u], sTxy[v - 1][u - 1], sTxy[v][u - 1], sP[v][u - 1], sP[v][u], p.dx, p.dy);
            if constexpr (DEFECT) r = r + x_f;
            T dv = p.dampX * x_dv + r;
            a.dVxdt[rxi] = dv;
            if constexpr (STORE_TMP) a.Rx[rxi] = r;
            if constexpr (RED) acc_rx += fabs((double)r);
            T dt = READ_DT ? x_dt : s2_dtV(p.Vsc, p.min_dxy2, sMus[v][u - 1], sMus[v][u]);
            vnew = vnew + dt * dv;
        }
        // bc_y!(Vx): rows 0 and ny-1 copy rows 1 and ny-2 (written by the owner of the inner row)
        if (fj >= 1 && fj <= ny - 2) a.Vx_out[fi + (nx + 1) * fj] = vnew;
        if (fj == 1) a.Vx_out[fi] = vnew;
        if (fj == ny - 2) a.Vx_out[fi + (nx + 1) * (ny - 1)] = vnew;
        if (ny <= 2 && (fj == 0 || fj == ny - 1)) a.Vx_out[fi + (nx + 1) * fj] = vnew;  // degenerate grid
    }
    // ---- Vy face (fi, fj), Vy is (nx, ny+1) ----
    if (yin) {
        T vnew = sVy[v][u];
        if (yinner) {
            T r = s2_Ry_core(sTyy[v - 1][u], sTyy[v][u], sTxy[v - 1][u - 1], sTxy[v - 1][u], sP[v - 1][u], sP[v][u], p.dx,
                             p.dy);
            r = r + y_f;  // the defect source, or the buoyancy average of the two cells
            T dv = p.dampY * y_dv + r;
            a.dVydt[ryi] = dv;
            if constexpr (STORE_TMP) a.Ry[ryi] = r;
            if constexpr (RED) acc_ry += fabs((double)r);
            T dt = READ_DT ? y_dt : s2_dtV(p.Vsc, p.min_dxy2, sMus[v - 1][u], sMus[v][u]);
            vnew = vnew + dt * dv;
        }
        // bc_x!(Vy): columns 0 and nx-1 copy columns 1 and nx-2
        if (fi >= 1 && fi <= nx - 2) a.Vy_out[fi + nx * fj] = vnew;
        if (fi == 1) a.Vy_out[nx * fj] = vnew;
        if (fi == nx - 2) a.Vy_out[(nx - 1) + nx * fj] = vnew;
        if (nx <= 2 && (fi == 0 || fi == nx - 1)) a.Vy_out[fi + nx * fj] = vnew;
    }
    if constexpr (RED) {
        double s0 = warp_sum(acc_rx), s1 = warp_sum(acc_ry), s2 = warp_sum(acc_div);
        int w = tid >> 5;
        if ((tid & 31) == 0) {
            sred[0][w] = s0;
            sred[1][w] = s1;
            sred[2][w] = s2;
        }
        __syncthreads();
        if (tid < 3) {
            double s = 0.0;
            for (int k = 0; k < TX * TY / 32; k++) s += sred[tid][k];
            atomicAdd(a.red + tid, s);
        }
    }
}

// =======================================================================================
// FP64 residual of the outer state (defect correction): no pseudo-time update.
// Outputs fp = ∇V, fx = Rx, fy = Ry rounded to float, and Σ|.| in FP64.
// =======================================================================================
__global__ void s2_residual64(const double* __restrict__ Vx, const double* __restrict__ Vy,
                              const double* __restrict__ P, const double* __restrict__ Mus,
                              const double* __restrict__ Rog, float* fp, float* fx, float* fy, double* red, int64_t nx,
                              int64_t ny, S2P<double> p) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, j = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;
    auto div_at = [&](int64_t ci, int64_t cj) {
        return s2_divV(A2(Vx, ci, cj, nx + 1), A2(Vx, ci + 1, cj, nx + 1), A2(Vy, ci, cj, nx), A2(Vy, ci, cj + 1, nx), p.dx,
                       p.dy);
    };
    auto txx_at = [&](int64_t ci, int64_t cj) {
        return s2_tau_nn(A2(Mus, ci, cj, nx), A2(Vx, ci, cj, nx + 1), A2(Vx, ci + 1, cj, nx + 1), div_at(ci, cj), p.dx);
    };
    auto tyy_at = [&](int64_t ci, int64_t cj) {
        return s2_tau_nn(A2(Mus, ci, cj, nx), A2(Vy, ci, cj, nx), A2(Vy, ci, cj + 1, nx), div_at(ci, cj), p.dy);
    };
    auto txy_at = [&](int64_t a_, int64_t b_) {
        return s2_tau_xy(A2(Mus, a_, b_, nx), A2(Mus, a_ + 1, b_, nx), A2(Mus, a_, b_ + 1, nx), A2(Mus, a_ + 1, b_ + 1, nx),
                         A2(Vx, a_ + 1, b_ + 1, nx + 1) - A2(Vx, a_ + 1, b_, nx + 1),
                         A2(Vy, a_ + 1, b_ + 1, nx) - A2(Vy, a_, b_ + 1, nx), p.dx, p.dy);
    };
    double ax = 0, ay = 0, ad = 0;
    if (i < nx && j < ny) {
        double d = div_at(i, j);
        fp[i + nx * j] = (float)d;
        ad = fabs(d);
    }
    if (i >= 1 && i <= nx - 1 && j >= 1 && j <= ny - 2) {
        double r = s2_Rx(txx_at(i - 1, j), txx_at(i, j), txy_at(i - 1, j - 1), txy_at(i - 1, j), A2(P, i - 1, j, nx),
                         A2(P, i, j, nx), p.dx, p.dy);
        fx[(i - 1) + (nx - 1) * (j - 1)] = (float)r;
        ax = fabs(r);
    }
    if (i >= 1 && i <= nx - 2 && j >= 1 && j <= ny - 1) {
        double r = s2_Ry_core(tyy_at(i, j - 1), tyy_at(i, j), txy_at(i - 1, j - 1), txy_at(i, j - 1), A2(P, i, j - 1, nx),
                              A2(P, i, j, nx), p.dx, p.dy) +
                   (A2(Rog, i, j - 1, nx) + A2(Rog, i, j, nx)) * 0.5;
        fy[(i - 1) + (nx - 2) * (j - 1)] = (float)r;
        ay = fabs(r);
    }
    __shared__ double sred[3][8];
    double s0 = warp_sum(ax), s1 = warp_sum(ay), s2 = warp_sum(ad);
    int tid = threadIdx.y * blockDim.x + threadIdx.x, w = tid >> 5;
    if ((tid & 31) == 0) {
        sred[0][w] = s0;
        sred[1][w] = s1;
        sred[2][w] = s2;
    }
    __syncthreads();
    if (tid < 3) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x * blockDim.y) / 32; k++) s += sred[tid][k];
        atomicAdd(red + tid, s);
    }
}

// x64 += (double) d32 over n elements
__global__ void s2_axpy32(double* x, const float* d, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += (double)d[i];
}

__global__ void s2_to_f32(float* y, const double* x, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}

// =======================================================================================
// Host side
// =======================================================================================
static int check2(const ps_array& a, int64_t n0, int64_t n1, int32_t dt, const char* name) {
    PS_TRY(check_array(a, name));
    if (a.dtype != dt) return fail(PS_ERR_DTYPE, "Stokes2D: array %s has a different dtype", name);
    return check_shape(a, n0, n1, 1, name);
}

static int check_fields(const ps_stokes2d_fields* f, int64_t* nx, int64_t* ny, bool need_dt) {
    if (!f) return fail(PS_ERR_NULL, "Stokes2D: NULL fields");
    PS_TRY(check_array(f->Pt, "Pt"));
    int64_t X = f->Pt.n[0], Y = f->Pt.n[1];
    int32_t dt = f->Pt.dtype;
    if (X < 3 || Y < 3 || f->Pt.n[2] != 1) return fail(PS_ERR_SHAPE, "Stokes2D: Pt must be 2-D with nx, ny >= 3");
    PS_TRY(check2(f->Vx, X + 1, Y, dt, "Vx"));
    PS_TRY(check2(f->Vy, X, Y + 1, dt, "Vy"));
    PS_TRY(check2(f->divV, X, Y, dt, "∇V"));
    PS_TRY(check2(f->txx, X, Y, dt, "τxx"));
    PS_TRY(check2(f->tyy, X, Y, dt, "τyy"));
    PS_TRY(check2(f->txy, X - 1, Y - 1, dt, "τxy"));
    PS_TRY(check2(f->Rx, X - 1, Y - 2, dt, "Rx"));
    PS_TRY(check2(f->Ry, X - 2, Y - 1, dt, "Ry"));
    PS_TRY(check2(f->dVxdtau, X - 1, Y - 2, dt, "dVxdτ"));
    PS_TRY(check2(f->dVydtau, X - 2, Y - 1, dt, "dVydτ"));
    PS_TRY(check2(f->Mus, X, Y, dt, "Mus"));
    PS_TRY(check2(f->Rog, X, Y, dt, "Rog"));
    if (need_dt) {
        PS_TRY(check2(f->dtauPt, X, Y, dt, "dτPt"));
        PS_TRY(check2(f->dtauVx, X - 1, Y - 2, dt, "dτVx"));
        PS_TRY(check2(f->dtauVy, X - 2, Y - 1, dt, "dτVy"));
    }
    *nx = X;
    *ny = Y;
    return PS_OK;
}

template <typename T>
static T* P_(const ps_array& a) {
    return static_cast<T*>(a.ptr);
}

static dim3 g2(int64_t wx, int64_t wy, dim3 b) {
    return dim3((unsigned)((wx + b.x - 1) / b.x), (unsigned)((wy + b.y - 1) / b.y), 1);
}

// Library-owned scratch for the ping-pong buffers and the solvers (freed by ps_finalize).
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};
static std::mutex g_scr_mutex;
static std::vector<void*> g_scratch_all;

static int scratch_alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(PS_ERR_NOMEM, "Stokes2D scratch allocation of %zu bytes failed", bytes);
    }
    std::lock_guard<std::mutex> l(g_scr_mutex);
    g_scratch_all.push_back(*p);
    return PS_OK;
}
static void scratch_free(void* p) {
    if (!p) return;
    cudaFree(p);
    std::lock_guard<std::mutex> l(g_scr_mutex);
    g_scratch_all.erase(std::remove(g_scratch_all.begin(), g_scratch_all.end(), p), g_scratch_all.end());
}

template <typename T, bool DEFECT, bool STORE_TMP, bool READ_DT>
static void launch_fused(const S2Fused<T>& a, const S2P<T>& p, cudaStream_t s) {
    constexpr int TY = s2_ty<T>();
    dim3 blk(S2_TX, TY);
    dim3 grd((unsigned)((a.nx + 1 + S2_TX - 1) / S2_TX), (unsigned)((a.ny + 1 + TY - 1) / TY));
    // 32-bit indices while the largest array and the tile origins stay below 2^31
    const bool i32 = (a.nx + 1 + S2_TX) * (a.ny + 1 + TY) < ((int64_t)1 << 31);
    if (a.red) {
        if (i32) s2_fused<T, DEFECT, STORE_TMP, READ_DT, int, true><<<grd, blk, 0, s>>>(a, p);
        else s2_fused<T, DEFECT, STORE_TMP, READ_DT, int64_t, true><<<grd, blk, 0, s>>>(a, p);
    } else {
        if (i32) s2_fused<T, DEFECT, STORE_TMP, READ_DT, int, false><<<grd, blk, 0, s>>>(a, p);
        else s2_fused<T, DEFECT, STORE_TMP, READ_DT, int64_t, false><<<grd, blk, 0, s>>>(a, p);
    }
}

template <typename T>
static int iterate_dropin(const ps_stokes2d_fields* f, const ps_stokes2d_params* pp, int64_t n_iter, cudaStream_t s) {
    int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    S2P<T> p = s2p<T>(*pp);
    size_t bx = (nx + 1) * ny * sizeof(T), by = nx * (ny + 1) * sizeof(T), bp = nx * ny * sizeof(T);
    void* buf = nullptr;
    PS_TRY(scratch_alloc(&buf, bx + by + bp + 256));
    T* Vx_b = static_cast<T*>(buf);
    T* Vy_b = reinterpret_cast<T*>(static_cast<char*>(buf) + bx);
    T* P_b = reinterpret_cast<T*>(static_cast<char*>(buf) + bx + by);
    S2Fused<T> a{};
    a.Mus = P_<T>(f->Mus);
    a.Rog = P_<T>(f->Rog);
    a.dtVx = P_<T>(f->dtauVx);
    a.dtVy = P_<T>(f->dtauVy);
    a.dtPt = P_<T>(f->dtauPt);
    a.dVxdt = P_<T>(f->dVxdtau);
    a.dVydt = P_<T>(f->dVydtau);
    a.divV = P_<T>(f->divV);
    a.txx = P_<T>(f->txx);
    a.tyy = P_<T>(f->tyy);
    a.txy = P_<T>(f->txy);
    a.Rx = P_<T>(f->Rx);
    a.Ry = P_<T>(f->Ry);
    a.red = nullptr;
    a.nx = nx;
    a.ny = ny;
    T* A[3] = {P_<T>(f->Vx), P_<T>(f->Vy), P_<T>(f->Pt)};
    T* B[3] = {Vx_b, Vy_b, P_b};
    for (int64_t it = 0; it < n_iter; ++it) {
        T** in = (it % 2 == 0) ? A : B;
        T** out = (it % 2 == 0) ? B : A;
        a.Vx_in = in[0];
        a.Vy_in = in[1];
        a.P_in = in[2];
        a.Vx_out = out[0];
        a.Vy_out = out[1];
        a.P_out = out[2];
        launch_fused<T, false, true, true>(a, p, s);
    }
    if (n_iter % 2 == 1) {
        cudaMemcpyAsync(A[0], B[0], bx, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(A[1], B[1], by, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(A[2], B[2], bp, cudaMemcpyDeviceToDevice, s);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    scratch_free(buf);
    if (e != cudaSuccess) return cuda_fail(e, "ps_stokes2d_iterate");
    return PS_OK;
}

// ---- solver ---------------------------------------------------------------------------
// Runs `nout` fused iterations per CUDA graph launch; the last one of each graph accumulates
// Σ|Rx|, Σ|Ry|, Σ|∇V| into `red`. `n_even` iterations keep the ping-pong parity.
template <typename T, bool DEFECT>
struct PTRunner {
    S2Fused<T> a{};
    S2P<T> p{};
    T* A[3];
    T* B[3];
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    int64_t nout = 0;

    int build(cudaStream_t s, int64_t nout_) {
        nout = nout_;
        PS_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(a.red, 0, 3 * sizeof(double), s);
        for (int64_t it = 0; it < nout; ++it) {
            T** in = (it % 2 == 0) ? A : B;
            T** out = (it % 2 == 0) ? B : A;
            S2Fused<T> k = a;
            k.Vx_in = in[0];
            k.Vy_in = in[1];
            k.P_in = in[2];
            k.Vx_out = out[0];
            k.Vy_out = out[1];
            k.P_out = out[2];
            if (it != nout - 1) k.red = nullptr;
            launch_fused<T, DEFECT, false, false>(k, p, s);
        }
        PS_CUDA_TRY(cudaStreamEndCapture(s, &graph));
        PS_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
        return PS_OK;
    }
    void destroy() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
};

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int solve_fp64(const ps_stokes2d_fields* f, const ps_stokes2d_params* pp, double tol, int64_t max_iter,
                      int64_t nout, double max_seconds, ps_solve_stats* st, cudaStream_t s) {
    int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    size_t bx = (nx + 1) * ny * 8, by = nx * (ny + 1) * 8, bp = nx * ny * 8;
    void* buf = nullptr;
    PS_TRY(scratch_alloc(&buf, bx + by + bp + 3 * sizeof(double) + 256));
    char* c = static_cast<char*>(buf);
    PTRunner<double, false> r;
    r.p = s2p<double>(*pp);
    r.a.Mus = P_<double>(f->Mus);
    r.a.Rog = P_<double>(f->Rog);
    r.a.dVxdt = P_<double>(f->dVxdtau);
    r.a.dVydt = P_<double>(f->dVydtau);
    r.a.red = reinterpret_cast<double*>(c + bx + by + bp);
    r.a.nx = nx;
    r.a.ny = ny;
    r.A[0] = P_<double>(f->Vx);
    r.A[1] = P_<double>(f->Vy);
    r.A[2] = P_<double>(f->Pt);
    r.B[0] = reinterpret_cast<double*>(c);
    r.B[1] = reinterpret_cast<double*>(c + bx);
    r.B[2] = reinterpret_cast<double*>(c + bx + by);
    int rc = r.build(s, nout);
    const double nrx = (double)((nx - 1) * (ny - 2)), nry = (double)((nx - 2) * (ny - 1)), nd = (double)(nx * ny);
    double t0 = now_s(), err = INFINITY, h[3];
    int64_t it = 0;
    while (rc == PS_OK && it < max_iter) {
        cudaError_t e = cudaGraphLaunch(r.exec, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, r.a.red, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "ps_stokes2d_solve(fp64)");
            break;
        }
        it += nout;
        err = std::max(std::max(h[0] / nrx, h[1] / nry), h[2] / nd);
        if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2])) {  // std::max drops a NaN
            err = NAN;
            rc = fail(PS_ERR_NONFINITE, "ps_stokes2d_solve: non-finite residual after %lld iterations", (long long)it);
            break;
        }
        if (err < tol) break;
        if (max_seconds > 0 && now_s() - t0 > max_seconds) {
            rc = fail(PS_ERR_TIMEOUT, "ps_stokes2d_solve: wall-clock limit reached (err %.3e)", err);
            break;
        }
    }
    // the state is in A after an even number of iterations (nout is even)
    r.destroy();
    cudaStreamSynchronize(s);
    scratch_free(buf);
    st->iters = it;
    st->outer = 1;
    st->err = err;
    st->seconds = now_s() - t0;
    st->converged = err < tol;
    if (rc == PS_OK && !(err < tol))
        rc = fail(PS_ERR_NOT_CONVERGED, "ps_stokes2d_solve: err %.3e after %lld iterations", err, (long long)it);
    return rc;
}

// Mixed precision: FP32 PT sweeps on the correction (δP, δV) with the FP64 residual of the
// outer state as source; FP64 residual, update and convergence check.
static int solve_mixed(const ps_stokes2d_fields* f, const ps_stokes2d_params* pp, double tol, int64_t max_iter,
                       int64_t nout, double max_seconds, double inner_rtol, ps_solve_stats* st, cudaStream_t s) {
    int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    const int64_t nVx = (nx + 1) * ny, nVy = nx * (ny + 1), nP = nx * ny, nRx = (nx - 1) * (ny - 2),
                  nRy = (nx - 2) * (ny - 1);
    // float buffers: δVx a/b, δVy a/b, δP a/b, dVxdτ, dVydτ, fx, fy, fp, Mus32
    int64_t counts[12] = {nVx, nVx, nVy, nVy, nP, nP, nRx, nRy, nRx, nRy, nP, nP};
    size_t off[13];
    off[0] = 0;
    for (int k = 0; k < 12; k++) off[k + 1] = off[k] + ((counts[k] * 4 + 255) / 256) * 256;
    size_t total = off[12] + 2 * 3 * sizeof(double) + 256;
    void* buf = nullptr;
    PS_TRY(scratch_alloc(&buf, total));
    char* c = static_cast<char*>(buf);
    auto F = [&](int k) { return reinterpret_cast<float*>(c + off[k]); };
    double* red_in = reinterpret_cast<double*>(c + off[12]);
    double* red_out = red_in + 3;
    int rc = PS_OK;
    cudaError_t e = cudaMemsetAsync(buf, 0, off[12], s);
    if (e != cudaSuccess) rc = cuda_fail(e, "memset");
    const double* Mus = P_<double>(f->Mus);
    s2_to_f32<<<256, 256, 0, s>>>(F(11), Mus, nP);
    // The corrections keep the free-slip copies (bc_y!(Vx), bc_x!(Vy)) of the state they are added
    // to, so a start state that violates them (an externally supplied guess) would keep its
    // violation: apply the copies once, as the first FP64 PT iteration would.
    s2_bc_y_k<double><<<(unsigned)((nx + 1 + 255) / 256), 256, 0, s>>>(P_<double>(f->Vx), nx + 1, ny);
    s2_bc_x_k<double><<<(unsigned)((ny + 1 + 255) / 256), 256, 0, s>>>(P_<double>(f->Vy), nx, ny + 1);

    PTRunner<float, true> r;
    r.p = s2p<float>(*pp);
    r.a.Mus = F(11);
    r.a.dVxdt = F(6);
    r.a.dVydt = F(7);
    r.a.fx = F(8);
    r.a.fy = F(9);
    r.a.fp = F(10);
    r.a.red = red_in;
    r.a.nx = nx;
    r.a.ny = ny;
    r.A[0] = F(0);
    r.A[1] = F(2);
    r.A[2] = F(4);
    r.B[0] = F(1);
    r.B[1] = F(3);
    r.B[2] = F(5);
    if (rc == PS_OK) rc = r.build(s, nout);

    S2P<double> p64 = s2p<double>(*pp);
    const double nrx = (double)nRx, nry = (double)nRy, nd = (double)nP;
    double t0 = now_s(), err = INFINITY, h[3];
    int64_t it = 0, outer = 0;
    dim3 blk(32, 8);
    dim3 grd = g2(nx + 1, ny + 1, blk);
    while (rc == PS_OK) {
        // FP64 residual of the outer state -> fx, fy, fp (float) and err
        cudaMemsetAsync(red_out, 0, 3 * sizeof(double), s);
        s2_residual64<<<grd, blk, 0, s>>>(P_<double>(f->Vx), P_<double>(f->Vy), P_<double>(f->Pt), Mus,
                                          P_<double>(f->Rog), F(10), F(8), F(9), red_out, nx, ny, p64);
        e = cudaMemcpyAsync(h, red_out, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "ps_stokes2d_solve(mixed residual)");
            break;
        }
        err = std::max(std::max(h[0] / nrx, h[1] / nry), h[2] / nd);
        if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2])) {
            err = NAN;
            rc = fail(PS_ERR_NONFINITE, "ps_stokes2d_solve: non-finite FP64 residual");
            break;
        }
        if (err < tol || it >= max_iter) break;
        if (max_seconds > 0 && now_s() - t0 > max_seconds) {
            rc = fail(PS_ERR_TIMEOUT, "ps_stokes2d_solve: wall-clock limit reached (err %.3e)", err);
            break;
        }
        ++outer;
        // inner FP32 PT on the correction, from zero
        cudaMemsetAsync(c, 0, off[8], s);  // δV, δP (a and b), dVxdτ, dVydτ
        double target = std::max(err * inner_rtol, tol * 0.25);
        double ierr = INFINITY;
        while (it < max_iter) {
            e = cudaGraphLaunch(r.exec, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(h, red_in, sizeof(h), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "ps_stokes2d_solve(mixed inner)");
                break;
            }
            it += nout;
            double prev = ierr;
            ierr = std::max(std::max(h[0] / nrx, h[1] / nry), h[2] / nd);
            if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2])) {
                rc = fail(PS_ERR_NONFINITE, "ps_stokes2d_solve: non-finite FP32 residual");
                break;
            }
            if (ierr < target) break;
            // FP32 floor: stop the sweep once it no longer reduces the residual
            if (ierr > 0.98 * prev && ierr < err * 0.5) break;
        }
        if (rc != PS_OK) break;
        // FP64 update of the outer state with the FP32 correction (in A after nout even)
        s2_axpy32<<<256, 256, 0, s>>>(P_<double>(f->Vx), F(0), nVx);
        s2_axpy32<<<256, 256, 0, s>>>(P_<double>(f->Vy), F(2), nVy);
        s2_axpy32<<<256, 256, 0, s>>>(P_<double>(f->Pt), F(4), nP);
    }
    r.destroy();
    cudaStreamSynchronize(s);
    scratch_free(buf);
    st->iters = it;
    st->outer = outer;
    st->err = err;
    st->seconds = now_s() - t0;
    st->converged = err < tol;
    if (rc == PS_OK && !(err < tol))
        rc = fail(PS_ERR_NOT_CONVERGED, "ps_stokes2d_solve(mixed): err %.3e after %lld iterations", err, (long long)it);
    return rc;
}

// Σ|a| (FP64 accumulation) -- used by ps_stokes2d_err.
__global__ void ps_sum_abs_f64(const double* a, int64_t n, double* out) {
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += fabs(a[i]);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}
__global__ void ps_sum_abs_f32(const float* a, int64_t n, double* out) {
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += fabs((double)a[i]);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

void stokes2d_free_scratch() {
    std::lock_guard<std::mutex> l(g_scr_mutex);
    for (void* p : g_scratch_all) cudaFree(p);
    g_scratch_all.clear();
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_stokes2d_timesteps(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8), grd = g2(nx, ny, blk);
    if (f->Pt.dtype == PS_F64)
        s2_timesteps_k<double><<<grd, blk, 0, s>>>(P_<double>(f->dtauVx), P_<double>(f->dtauVy), P_<double>(f->dtauPt),
                                                   P_<double>(f->Mus), nx, ny, s2p<double>(*p));
    else
        s2_timesteps_k<float><<<grd, blk, 0, s>>>(P_<float>(f->dtauVx), P_<float>(f->dtauVy), P_<float>(f->dtauPt),
                                                  P_<float>(f->Mus), nx, ny, s2p<float>(*p));
    return finish_launch(s, sync, "ps_stokes2d_timesteps");
}

int ps_stokes2d_compute_P(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8), grd = g2(nx, ny, blk);
    if (f->Pt.dtype == PS_F64)
        s2_P_k<double><<<grd, blk, 0, s>>>(P_<double>(f->divV), P_<double>(f->Pt), P_<double>(f->Vx), P_<double>(f->Vy),
                                           P_<double>(f->dtauPt), nx, ny, s2p<double>(*p));
    else
        s2_P_k<float><<<grd, blk, 0, s>>>(P_<float>(f->divV), P_<float>(f->Pt), P_<float>(f->Vx), P_<float>(f->Vy),
                                          P_<float>(f->dtauPt), nx, ny, s2p<float>(*p));
    return finish_launch(s, sync, "ps_stokes2d_compute_P");
}

int ps_stokes2d_compute_tau(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8), grd = g2(nx, ny, blk);
    if (f->Pt.dtype == PS_F64)
        s2_tau_k<double><<<grd, blk, 0, s>>>(P_<double>(f->divV), P_<double>(f->txx), P_<double>(f->tyy),
                                             P_<double>(f->txy), P_<double>(f->Vx), P_<double>(f->Vy),
                                             P_<double>(f->Mus), nx, ny, s2p<double>(*p));
    else
        s2_tau_k<float><<<grd, blk, 0, s>>>(P_<float>(f->divV), P_<float>(f->txx), P_<float>(f->tyy), P_<float>(f->txy),
                                            P_<float>(f->Vx), P_<float>(f->Vy), P_<float>(f->Mus), nx, ny,
                                            s2p<float>(*p));
    return finish_launch(s, sync, "ps_stokes2d_compute_tau");
}

int ps_stokes2d_compute_dV(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8), grd = g2(nx, ny, blk);
    if (f->Pt.dtype == PS_F64)
        s2_dV_k<double><<<grd, blk, 0, s>>>(P_<double>(f->Rx), P_<double>(f->Ry), P_<double>(f->dVxdtau),
                                            P_<double>(f->dVydtau), P_<double>(f->Pt), P_<double>(f->Rog),
                                            P_<double>(f->txx), P_<double>(f->tyy), P_<double>(f->txy), nx, ny,
                                            s2p<double>(*p));
    else
        s2_dV_k<float><<<grd, blk, 0, s>>>(P_<float>(f->Rx), P_<float>(f->Ry), P_<float>(f->dVxdtau),
                                           P_<float>(f->dVydtau), P_<float>(f->Pt), P_<float>(f->Rog), P_<float>(f->txx),
                                           P_<float>(f->tyy), P_<float>(f->txy), nx, ny, s2p<float>(*p));
    return finish_launch(s, sync, "ps_stokes2d_compute_dV");
}

int ps_stokes2d_compute_V(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    (void)p;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(32, 8), grd = g2(nx + 1, ny + 1, blk);
    if (f->Pt.dtype == PS_F64)
        s2_V_k<double><<<grd, blk, 0, s>>>(P_<double>(f->Vx), P_<double>(f->Vy), P_<double>(f->dVxdtau),
                                           P_<double>(f->dVydtau), P_<double>(f->dtauVx), P_<double>(f->dtauVy), nx, ny);
    else
        s2_V_k<float><<<grd, blk, 0, s>>>(P_<float>(f->Vx), P_<float>(f->Vy), P_<float>(f->dVxdtau),
                                          P_<float>(f->dVydtau), P_<float>(f->dtauVx), P_<float>(f->dtauVy), nx, ny);
    return finish_launch(s, sync, "ps_stokes2d_compute_V");
}

static int bc2(ps_array A, void* stream, int sync, bool xdir) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(A, "A"));
    if (A.n[2] != 1 || A.n[0] < 2 || A.n[1] < 2) return fail(PS_ERR_SHAPE, "bc: A must be 2-D with extents >= 2");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int64_t w = xdir ? A.n[1] : A.n[0];
    unsigned g = (unsigned)((w + 255) / 256);
    if (A.dtype == PS_F64) {
        if (xdir)
            s2_bc_x_k<double><<<g, 256, 0, s>>>(P_<double>(A), A.n[0], A.n[1]);
        else
            s2_bc_y_k<double><<<g, 256, 0, s>>>(P_<double>(A), A.n[0], A.n[1]);
    } else {
        if (xdir)
            s2_bc_x_k<float><<<g, 256, 0, s>>>(P_<float>(A), A.n[0], A.n[1]);
        else
            s2_bc_y_k<float><<<g, 256, 0, s>>>(P_<float>(A), A.n[0], A.n[1]);
    }
    return finish_launch(s, sync, xdir ? "ps_bc_x2d" : "ps_bc_y2d");
}

int ps_bc_x2d(ps_array A, void* stream, int sync) { return bc2(A, stream, sync, true); }
int ps_bc_y2d(ps_array A, void* stream, int sync) { return bc2(A, stream, sync, false); }

int ps_stokes2d_iterate(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, int64_t n_iter, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    if (n_iter < 0) return fail(PS_ERR_ARG, "n_iter must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = f->Pt.dtype == PS_F64 ? iterate_dropin<double>(f, p, n_iter, s) : iterate_dropin<float>(f, p, n_iter, s);
    PS_TRY(rc);
    return finish_launch(s, 1, "ps_stokes2d_iterate");
}

int ps_stokes2d_err(const ps_stokes2d_fields* f, double out_mean_abs[3], void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, false));
    if (!out_mean_abs) return fail(PS_ERR_NULL, "NULL output");
    // mean(abs.(Rx)), mean(abs.(Ry)), mean(abs.(∇V)) (Stokes2D.jl:119) on the stored arrays
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const ps_array* arrs[3] = {&f->Rx, &f->Ry, &f->divV};
    double* red = st->d_scratch;
    PS_CUDA_TRY(cudaMemsetAsync(red, 0, 3 * sizeof(double), s));
    for (int k = 0; k < 3; k++) {
        int64_t n = numel(*arrs[k]);
        if (f->Pt.dtype == PS_F64)
            ps_sum_abs_f64<<<std::max<int64_t>(1, std::min<int64_t>((n + 1023) / 1024, 1024)), 256, 0, s>>>(
                P_<double>(*arrs[k]), n, red + k);
        else
            ps_sum_abs_f32<<<std::max<int64_t>(1, std::min<int64_t>((n + 1023) / 1024, 1024)), 256, 0, s>>>(
                P_<float>(*arrs[k]), n, red + k);
    }
    double h[3];
    PS_CUDA_TRY(cudaMemcpyAsync(h, red, sizeof(h), cudaMemcpyDeviceToHost, s));
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    for (int k = 0; k < 3; k++) out_mean_abs[k] = h[k] / (double)numel(*arrs[k]);
    return finish_launch(s, 0, "ps_stokes2d_err");
}

int ps_stokes2d_solve(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, int32_t mode, double tol,
                      int64_t max_iter, int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, false));
    if (!p || !stats) return fail(PS_ERR_NULL, "NULL params / stats");
    if (f->Pt.dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_stokes2d_solve: the state arrays must be FP64");
    if (nout < 2 || nout % 2) return fail(PS_ERR_ARG, "nout must be even and >= 2");
    if (!(tol > 0) || max_iter < 0) return fail(PS_ERR_ARG, "invalid tol / max_iter");
    if (mode != 0 && mode != 1) return fail(PS_ERR_ARG, "mode must be 0 (FP64) or 1 (FP32 + FP64 defect correction)");
    memset(stats, 0, sizeof(*stats));
    // the solver captures CUDA graphs: run on a private stream ordered after `stream`
    cudaStream_t user = static_cast<cudaStream_t>(stream), s;
    PS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t ev;
    PS_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(s, ev, 0);
    int rc = mode == 0 ? solve_fp64(f, p, tol, max_iter, nout, max_seconds, stats, s)
                       : solve_mixed(f, p, tol, max_iter, nout, max_seconds, 1e-3, stats, s);
    cudaStreamSynchronize(s);
    cudaEventDestroy(ev);
    cudaStreamDestroy(s);
    cudaGetLastError();
    return rc;
}

}  // extern "C"


// =======================================================================================
// ps_stokes2d_iterate_static: the fused PT iteration without any device allocation.
//
// ps_stokes2d_iterate needs three ping-pong buffers (the old/new Vx, Vy, Pt) and allocates them
// per call. Some hosts cannot let a library allocate device memory: an application whose device
// memory is fully owned by its own pool allocator (CUDA.jl's memory pool, a framework caching
// allocator), where a cudaMalloc behind its back fails or fragments the pool, and code that must
// not call cudaFree, which synchronises the whole device. This variant takes its ping-pong buffers
// from a fixed device array compiled into the library instead.
//
// The array is file-scope, kStaticScratchBytes (16 MiB) on every device that loads the library,
// held until process exit. Host code must not pass the array's name to a kernel (on the host it
// is only a stand-in symbol): its device address is looked up once per device with
// cudaGetSymbolAddress, on the first call on that device, with that device current, and cached.
// The cache belongs to the device's current context: ps_finalize clears it, so that after a
// context is torn down (ps_finalize, then cudaDeviceReset) the next call looks the address up again.
// =======================================================================================
namespace ps {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static constexpr int kStaticMaxDevices = 64;
static void* g_static_scratch_addr[kStaticMaxDevices] = {};
static std::mutex g_static_mutex;

// Device address of g_static_scratch on the current device (looked up once per device).
static int static_scratch(void** out) {
    int dev = -1;
    PS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticMaxDevices) return fail(PS_ERR_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        g_static_scratch_addr[dev] = p;
    }
    *out = g_static_scratch_addr[dev];
    return PS_OK;
}

void stokes2d_static_forget() {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    for (int d = 0; d < kStaticMaxDevices; d++) g_static_scratch_addr[d] = nullptr;
}

static size_t round256(size_t b) { return (b + 255) / 256 * 256; }

template <typename T>
static int iterate_static(const ps_stokes2d_fields* f, const ps_stokes2d_params* pp, int64_t n_iter, cudaStream_t s) {
    const int64_t nx = f->Pt.n[0], ny = f->Pt.n[1];
    const size_t bx = (nx + 1) * ny * sizeof(T), by = nx * (ny + 1) * sizeof(T), bp = nx * ny * sizeof(T);
    const size_t need = round256(bx) + round256(by) + round256(bp);
    if (need > kStaticScratchBytes)
        return fail(PS_ERR_SHAPE,
                    "ps_stokes2d_iterate_static: a %lld x %lld grid needs %zu bytes of scratch; the static buffer "
                    "holds %zu bytes (use ps_stokes2d_iterate)",
                    (long long)nx, (long long)ny, need, kStaticScratchBytes);
    void* base = nullptr;
    PS_TRY(static_scratch(&base));
    char* c = static_cast<char*>(base);
    T* B[3] = {reinterpret_cast<T*>(c), reinterpret_cast<T*>(c + round256(bx)),
               reinterpret_cast<T*>(c + round256(bx) + round256(by))};
    T* A[3] = {P_<T>(f->Vx), P_<T>(f->Vy), P_<T>(f->Pt)};
    S2P<T> p = s2p<T>(*pp);
    S2Fused<T> a{};
    a.Mus = P_<T>(f->Mus);
    a.Rog = P_<T>(f->Rog);
    a.dtVx = P_<T>(f->dtauVx);
    a.dtVy = P_<T>(f->dtauVy);
    a.dtPt = P_<T>(f->dtauPt);
    a.dVxdt = P_<T>(f->dVxdtau);
    a.dVydt = P_<T>(f->dVydtau);
    a.divV = P_<T>(f->divV);
    a.txx = P_<T>(f->txx);
    a.tyy = P_<T>(f->tyy);
    a.txy = P_<T>(f->txy);
    a.Rx = P_<T>(f->Rx);
    a.Ry = P_<T>(f->Ry);
    a.red = nullptr;
    a.nx = nx;
    a.ny = ny;
    // every element of the buffers in use is written before it is read within a call, so the
    // contents left by the previous call never matter
    for (int64_t it = 0; it < n_iter; ++it) {
        T** in = (it % 2 == 0) ? A : B;
        T** out = (it % 2 == 0) ? B : A;
        a.Vx_in = in[0];
        a.Vy_in = in[1];
        a.P_in = in[2];
        a.Vx_out = out[0];
        a.Vy_out = out[1];
        a.P_out = out[2];
        launch_fused<T, false, true, true>(a, p, s);
    }
    if (n_iter % 2 == 1) {
        PS_CUDA_TRY(cudaMemcpyAsync(A[0], B[0], bx, cudaMemcpyDeviceToDevice, s));
        PS_CUDA_TRY(cudaMemcpyAsync(A[1], B[1], by, cudaMemcpyDeviceToDevice, s));
        PS_CUDA_TRY(cudaMemcpyAsync(A[2], B[2], bp, cudaMemcpyDeviceToDevice, s));
    }
    return PS_OK;
}

}  // namespace ps

extern "C" int ps_stokes2d_iterate_static(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, int64_t n_iter,
                                          void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    int64_t nx, ny;
    PS_TRY(check_fields(f, &nx, &ny, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    if (n_iter < 0) return fail(PS_ERR_ARG, "n_iter must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = f->Pt.dtype == PS_F64 ? iterate_static<double>(f, p, n_iter, s) : iterate_static<float>(f, p, n_iter, s);
    PS_TRY(rc);
    return finish_launch(s, 1, "ps_stokes2d_iterate_static");
}
