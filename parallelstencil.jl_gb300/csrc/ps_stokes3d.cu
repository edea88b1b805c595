// ps_stokes3d.cu -- pseudo-transient (PT) viscous Stokes 3-D kernels and solver of libps_b200.so.
//
// Reference: miniapps/Stokes3D.jl:11-68 (kernels), :131-149 (PT loop and error check).
//
//   s3_* device functions   the arithmetic of each reference statement (operation order and
//                           literals of the FD macros, src/FiniteDifferences.jl:328-388), shared
//                           by every kernel below so all paths round identically
//   one-to-one kernels      compute_timesteps!, compute_P!, compute_τ!, compute_dV!, compute_V!,
//                           bc_x!, bc_y!, bc_z! -- drop-in replacements of the `@parallel` calls
//   iteration kernels       one PT iteration in three launches:
//                             s3_Ptau_k  ∇V, Pt and the six stresses of a cell; the normal
//                                        stresses are indexed so that every thread uses the ∇V
//                                        of its own cell (no re-read of ∇V from memory),
//                             s3_dVV_k   residuals, pseudo-velocity and velocity updates,
//                             s3_bc_k    the six free-slip copies of the loop body at once: the
//                                        copies along different axes commute, so each boundary
//                                        value is the composed copy of an interior value.
//                           Results are bit-identical to the reference's ten-launch loop body.
//   ps_stokes3d_solve       the `while err > ε` loop in FP64: CUDA graphs of `nout` iterations
//                           followed by the FP64 residual norms, checked on the host.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <utility>
#include <mutex>
#include <map>

#include "ps_common.cuh"

namespace ps {

template <typename T>
struct S3P {
    DivC<T> dx, dy, dz;  // divisors of the statements (correctly rounded division by host numbers)
    T dampX, dampY, dampZ, Vsc, Ptsc, min_dxyz2, max_nxyz;
};

template <typename T>
static S3P<T> s3p(const ps_stokes3d_params& p) {
    return S3P<T>{make_div((T)p.dx), make_div((T)p.dy), make_div((T)p.dz), (T)p.dampX,     (T)p.dampY,
                  (T)p.dampZ,        (T)p.Vsc,          (T)p.Ptsc,         (T)p.min_dxyz2, (T)p.max_nxyz};
}

// Device pointers of the miniapp's arrays (sizes relative to (nx, ny, nz) = size(Pt) as in
// Stokes3D.jl:89-110).
template <typename T>
struct S3A {
    T *Pt, *dtPt, *divV, *Vx, *Vy, *Vz, *txx, *tyy, *tzz, *txy, *txz, *tyz, *Rx, *Ry, *Rz, *dVx, *dVy, *dVz, *dtVx,
        *dtVy, *dtVz;
    const T *Mus, *Rog;
    const T *fx, *fy, *fz, *fp;  // mode S3_DEFECT: FP64 residual of the outer state, rounded to T
    int64_t nx, ny, nz;
};

// Modes of the iteration kernels: the reference's iteration; the inner sweep of the mixed-precision
// solver (PT on a correction: the outer state's residual is the source, buoyancy included in it);
// the residual alone (no pseudo-time update) of the FP64 outer state.
enum { S3_PLAIN = 0, S3_DEFECT = 1, S3_RESIDUAL = 2 };

#define I3(a, b, c, n0, n1) ((int64_t)(a) + (int64_t)(n0) * ((int64_t)(b) + (int64_t)(n1) * (int64_t)(c)))
// the same in the index type I of the iteration kernels (32-bit where every array has < 2^31 elements)
#define I3T(a, b, c, n0, n1) ((I)(a) + (I)(n0) * ((I)(b) + (I)(n1) * (I)(c)))

// ---- statement arithmetic ------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T s3_dtV(T Vsc, T mdx2, T m0, T m1) {
    const T av = (m0 + m1) * T(0.5);
    return ((Vsc * mdx2) / av) / T(6.1);
}
template <typename T>
__device__ __forceinline__ T s3_dtPt(T Ptsc, T m, T mn) {
    return ((Ptsc * T(6.1)) * m) / mn;
}
// @d_xa(Vx)/dx + @d_ya(Vy)/dy + @d_za(Vz)/dz at cell (x, y, z)
template <typename T, typename I = int64_t>
__device__ __forceinline__ T s3_divV(const S3A<T>& a, const S3P<T>& p, I x, I y, I z) {
    const I nx = (I)a.nx, ny = (I)a.ny;
    return (div_c(a.Vx[I3T(x + 1, y, z, nx + 1, ny)] - a.Vx[I3T(x, y, z, nx + 1, ny)], p.dx) +
            div_c(a.Vy[I3T(x, y + 1, z, nx, ny + 1)] - a.Vy[I3T(x, y, z, nx, ny + 1)], p.dy)) +
           div_c(a.Vz[I3T(x, y, z + 1, nx, ny)] - a.Vz[I3T(x, y, z, nx, ny)], p.dz);
}
// 2.0*μ*(dV/h - 1.0/3.0*∇V)
template <typename T>
__device__ __forceinline__ T s3_tnn(T m, T v1, T v0, const DivC<T>& h, T d) {
    return (T(2.0) * m) * (div_c(v1 - v0, h) - (T(1.0) / T(3.0)) * d);
}
// 2.0*@av_..i(μ)*(0.5*(a/ha + b/hb)), the four μ in the macro's order
template <typename T>
__device__ __forceinline__ T s3_tsh(T m0, T m1, T m2, T m3, T a, const DivC<T>& ha, T b, const DivC<T>& hb) {
    const T av = (((m0 + m1) + m2) + m3) * T(0.25);
    return (T(2.0) * av) * (T(0.5) * (div_c(a, ha) + div_c(b, hb)));
}

template <typename T, typename I = int64_t>
__device__ __forceinline__ void s3_txy(const S3A<T>& a, const S3P<T>& p, I x, I y, I z) {
    const I nx = (I)a.nx, ny = (I)a.ny;
    const T* M = a.Mus;
    a.txy[I3T(x, y, z, nx - 1, ny - 1)] =
        s3_tsh(M[I3T(x, y, z + 1, nx, ny)], M[I3T(x + 1, y, z + 1, nx, ny)], M[I3T(x, y + 1, z + 1, nx, ny)],
               M[I3T(x + 1, y + 1, z + 1, nx, ny)],
               a.Vx[I3T(x + 1, y + 1, z + 1, nx + 1, ny)] - a.Vx[I3T(x + 1, y, z + 1, nx + 1, ny)], p.dy,
               a.Vy[I3T(x + 1, y + 1, z + 1, nx, ny + 1)] - a.Vy[I3T(x, y + 1, z + 1, nx, ny + 1)], p.dx);
}
template <typename T, typename I = int64_t>
__device__ __forceinline__ void s3_txz(const S3A<T>& a, const S3P<T>& p, I x, I y, I z) {
    const I nx = (I)a.nx, ny = (I)a.ny;
    const T* M = a.Mus;
    a.txz[I3T(x, y, z, nx - 1, ny - 2)] =
        s3_tsh(M[I3T(x, y + 1, z, nx, ny)], M[I3T(x + 1, y + 1, z, nx, ny)], M[I3T(x, y + 1, z + 1, nx, ny)],
               M[I3T(x + 1, y + 1, z + 1, nx, ny)],
               a.Vx[I3T(x + 1, y + 1, z + 1, nx + 1, ny)] - a.Vx[I3T(x + 1, y + 1, z, nx + 1, ny)], p.dz,
               a.Vz[I3T(x + 1, y + 1, z + 1, nx, ny)] - a.Vz[I3T(x, y + 1, z + 1, nx, ny)], p.dx);
}
template <typename T, typename I = int64_t>
__device__ __forceinline__ void s3_tyz(const S3A<T>& a, const S3P<T>& p, I x, I y, I z) {
    const I nx = (I)a.nx, ny = (I)a.ny;
    const T* M = a.Mus;
    a.tyz[I3T(x, y, z, nx - 2, ny - 1)] =
        s3_tsh(M[I3T(x + 1, y, z, nx, ny)], M[I3T(x + 1, y + 1, z, nx, ny)], M[I3T(x + 1, y, z + 1, nx, ny)],
               M[I3T(x + 1, y + 1, z + 1, nx, ny)],
               a.Vy[I3T(x + 1, y + 1, z + 1, nx, ny + 1)] - a.Vy[I3T(x + 1, y + 1, z, nx, ny + 1)], p.dz,
               a.Vz[I3T(x + 1, y + 1, z + 1, nx, ny)] - a.Vz[I3T(x + 1, y, z + 1, nx, ny)], p.dy);
}

// compute_dV! statements at residual index (x, y, z) and, with update_V, compute_V! at the same
// index (it reads only the pseudo-velocity just written)
template <typename T, int MODE = S3_PLAIN, typename I = int64_t>
__device__ __forceinline__ void s3_dV(const S3A<T>& a, const S3P<T>& p, I x, I y, I z, bool update_V) {
    const I nx = (I)a.nx, ny = (I)a.ny, nz = (I)a.nz;
    const T* Pt = a.Pt;
    if (x < nx - 1 && y < ny - 2 && z < nz - 2) {
        const I r = I3T(x, y, z, nx - 1, ny - 2);
        const T A = a.txx[I3T(x + 1, y, z, nx, ny - 2)] - a.txx[I3T(x, y, z, nx, ny - 2)];
        const T B = a.txy[I3T(x, y + 1, z, nx - 1, ny - 1)] - a.txy[I3T(x, y, z, nx - 1, ny - 1)];
        const T C = a.txz[I3T(x, y, z + 1, nx - 1, ny - 2)] - a.txz[I3T(x, y, z, nx - 1, ny - 2)];
        const T P = Pt[I3T(x + 1, y + 1, z + 1, nx, ny)] - Pt[I3T(x, y + 1, z + 1, nx, ny)];
        T R = ((div_c(A, p.dx) + div_c(B, p.dy)) + div_c(C, p.dz)) - div_c(P, p.dx);
        if constexpr (MODE == S3_DEFECT) R = R + a.fx[r];
        a.Rx[r] = R;
        if constexpr (MODE != S3_RESIDUAL) {
            const T dv = p.dampX * a.dVx[r] + R;
            a.dVx[r] = dv;
            if (update_V) {
                const I v = I3T(x + 1, y + 1, z + 1, nx + 1, ny);
                a.Vx[v] = a.Vx[v] + a.dtVx[r] * dv;
            }
        }
    }
    if (x < nx - 2 && y < ny - 1 && z < nz - 2) {
        const I r = I3T(x, y, z, nx - 2, ny - 1);
        const T A = a.tyy[I3T(x, y + 1, z, nx - 2, ny)] - a.tyy[I3T(x, y, z, nx - 2, ny)];
        const T B = a.txy[I3T(x + 1, y, z, nx - 1, ny - 1)] - a.txy[I3T(x, y, z, nx - 1, ny - 1)];
        const T C = a.tyz[I3T(x, y, z + 1, nx - 2, ny - 1)] - a.tyz[I3T(x, y, z, nx - 2, ny - 1)];
        const T P = Pt[I3T(x + 1, y + 1, z + 1, nx, ny)] - Pt[I3T(x + 1, y, z + 1, nx, ny)];
        T R = ((div_c(A, p.dy) + div_c(B, p.dx)) + div_c(C, p.dz)) - div_c(P, p.dy);
        if constexpr (MODE == S3_DEFECT) R = R + a.fy[r];
        a.Ry[r] = R;
        if constexpr (MODE != S3_RESIDUAL) {
            const T dv = p.dampY * a.dVy[r] + R;
            a.dVy[r] = dv;
            if (update_V) {
                const I v = I3T(x + 1, y + 1, z + 1, nx, ny + 1);
                a.Vy[v] = a.Vy[v] + a.dtVy[r] * dv;
            }
        }
    }
    if (x < nx - 2 && y < ny - 2 && z < nz - 1) {
        const I r = I3T(x, y, z, nx - 2, ny - 2);
        const T A = a.tzz[I3T(x, y, z + 1, nx - 2, ny - 2)] - a.tzz[I3T(x, y, z, nx - 2, ny - 2)];
        const T B = a.txz[I3T(x + 1, y, z, nx - 1, ny - 2)] - a.txz[I3T(x, y, z, nx - 1, ny - 2)];
        const T C = a.tyz[I3T(x, y + 1, z, nx - 2, ny - 1)] - a.tyz[I3T(x, y, z, nx - 2, ny - 1)];
        const T P = Pt[I3T(x + 1, y + 1, z + 1, nx, ny)] - Pt[I3T(x + 1, y + 1, z, nx, ny)];
        T R;
        if constexpr (MODE == S3_DEFECT) {  // the buoyancy is part of the outer residual fz
            R = (((div_c(A, p.dz) + div_c(B, p.dx)) + div_c(C, p.dy)) - div_c(P, p.dz)) + a.fz[r];
        } else {
            const T G = (a.Rog[I3T(x + 1, y + 1, z, nx, ny)] + a.Rog[I3T(x + 1, y + 1, z + 1, nx, ny)]) * T(0.5);
            R = (((div_c(A, p.dz) + div_c(B, p.dx)) + div_c(C, p.dy)) - div_c(P, p.dz)) + G;
        }
        a.Rz[r] = R;
        if constexpr (MODE != S3_RESIDUAL) {
            const T dv = p.dampZ * a.dVz[r] + R;
            a.dVz[r] = dv;
            if (update_V) {
                const I v = I3T(x + 1, y + 1, z + 1, nx, ny);
                a.Vz[v] = a.Vz[v] + a.dtVz[r] * dv;
            }
        }
    }
}

#define S3_IDX                                                                               \
    const int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;                        \
    const int64_t y = blockIdx.y * (int64_t)blockDim.y + threadIdx.y;                        \
    const int64_t z = blockIdx.z;                                                            \
    const int64_t nx = a.nx, ny = a.ny, nz = a.nz;                                           \
    if (x >= nx || y >= ny || z >= nz) return
#define S3_IDXT                                                                              \
    const I x = (I)(blockIdx.x * blockDim.x + threadIdx.x);                                  \
    const I y = (I)(blockIdx.y * blockDim.y + threadIdx.y);                                  \
    const I z = (I)blockIdx.z;                                                               \
    const I nx = (I)a.nx, ny = (I)a.ny, nz = (I)a.nz;                                        \
    if (x >= nx || y >= ny || z >= nz) return

// ---- one-to-one kernels (grid: max extents of the kernel's array arguments) ---------------
template <typename T>
__global__ void s3_timesteps_k(S3A<T> a, S3P<T> p) {
    S3_IDX;
    const T* M = a.Mus;
    if (x < nx - 1 && y < ny - 2 && z < nz - 2)
        a.dtVx[I3(x, y, z, nx - 1, ny - 2)] =
            s3_dtV(p.Vsc, p.min_dxyz2, M[I3(x, y + 1, z + 1, nx, ny)], M[I3(x + 1, y + 1, z + 1, nx, ny)]);
    if (x < nx - 2 && y < ny - 1 && z < nz - 2)
        a.dtVy[I3(x, y, z, nx - 2, ny - 1)] =
            s3_dtV(p.Vsc, p.min_dxyz2, M[I3(x + 1, y, z + 1, nx, ny)], M[I3(x + 1, y + 1, z + 1, nx, ny)]);
    if (x < nx - 2 && y < ny - 2 && z < nz - 1)
        a.dtVz[I3(x, y, z, nx - 2, ny - 2)] =
            s3_dtV(p.Vsc, p.min_dxyz2, M[I3(x + 1, y + 1, z, nx, ny)], M[I3(x + 1, y + 1, z + 1, nx, ny)]);
    a.dtPt[I3(x, y, z, nx, ny)] = s3_dtPt(p.Ptsc, M[I3(x, y, z, nx, ny)], p.max_nxyz);
}

template <typename T>
__global__ void s3_P_k(S3A<T> a, S3P<T> p) {
    S3_IDX;
    const int64_t c = I3(x, y, z, nx, ny);
    const T d = s3_divV(a, p, x, y, z);
    a.divV[c] = d;
    a.Pt[c] = a.Pt[c] - a.dtPt[c] * d;
}

template <typename T>
__global__ void s3_tau_k(S3A<T> a, S3P<T> p) {
    S3_IDX;
    const T* M = a.Mus;
    if (y < ny - 2 && z < nz - 2) {
        const int64_t c = I3(x, y + 1, z + 1, nx, ny);
        a.txx[I3(x, y, z, nx, ny - 2)] = s3_tnn(M[c], a.Vx[I3(x + 1, y + 1, z + 1, nx + 1, ny)],
                                                a.Vx[I3(x, y + 1, z + 1, nx + 1, ny)], p.dx, a.divV[c]);
    }
    if (x < nx - 2 && z < nz - 2) {
        const int64_t c = I3(x + 1, y, z + 1, nx, ny);
        a.tyy[I3(x, y, z, nx - 2, ny)] = s3_tnn(M[c], a.Vy[I3(x + 1, y + 1, z + 1, nx, ny + 1)],
                                                a.Vy[I3(x + 1, y, z + 1, nx, ny + 1)], p.dy, a.divV[c]);
    }
    if (x < nx - 2 && y < ny - 2) {
        const int64_t c = I3(x + 1, y + 1, z, nx, ny);
        a.tzz[I3(x, y, z, nx - 2, ny - 2)] = s3_tnn(M[c], a.Vz[I3(x + 1, y + 1, z + 1, nx, ny)],
                                                    a.Vz[I3(x + 1, y + 1, z, nx, ny)], p.dz, a.divV[c]);
    }
    if (x < nx - 1 && y < ny - 1 && z < nz - 2) s3_txy(a, p, x, y, z);
    if (x < nx - 1 && y < ny - 2 && z < nz - 1) s3_txz(a, p, x, y, z);
    if (x < nx - 2 && y < ny - 1 && z < nz - 1) s3_tyz(a, p, x, y, z);
}

template <typename T>
__global__ void s3_dV_k(S3A<T> a, S3P<T> p) {
    S3_IDX;
    s3_dV(a, p, x, y, z, false);
}

template <typename T>
__global__ void s3_V_k(S3A<T> a) {
    S3_IDX;
    if (x < nx - 1 && y < ny - 2 && z < nz - 2) {
        const int64_t v = I3(x + 1, y + 1, z + 1, nx + 1, ny), r = I3(x, y, z, nx - 1, ny - 2);
        a.Vx[v] = a.Vx[v] + a.dtVx[r] * a.dVx[r];
    }
    if (x < nx - 2 && y < ny - 1 && z < nz - 2) {
        const int64_t v = I3(x + 1, y + 1, z + 1, nx, ny + 1), r = I3(x, y, z, nx - 2, ny - 1);
        a.Vy[v] = a.Vy[v] + a.dtVy[r] * a.dVy[r];
    }
    if (x < nx - 2 && y < ny - 2 && z < nz - 1) {
        const int64_t v = I3(x + 1, y + 1, z + 1, nx, ny), r = I3(x, y, z, nx - 2, ny - 2);
        a.Vz[v] = a.Vz[v] + a.dtVz[r] * a.dVz[r];
    }
}

// bc_x! / bc_y! / bc_z! (Stokes3D.jl:52-68): the boundary planes of axis `ax` copy the first
// inner planes; threads run over the other two axes.
template <typename T>
__global__ void s3_bc_axis_k(T* A, int64_t n0, int64_t n1, int64_t n2, int ax) {
    const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, v = blockIdx.y;
    const int64_t n[3] = {n0, n1, n2};
    const int o0 = ax == 0 ? 1 : 0, o1 = ax == 2 ? 1 : 2;  // the two other axes
    if (u >= n[o0] || v >= n[o1]) return;
    int64_t i[3];
    i[o0] = u;
    i[o1] = v;
    i[ax] = 0;
    const int64_t lo = I3(i[0], i[1], i[2], n0, n1);
    i[ax] = 1;
    const int64_t lo1 = I3(i[0], i[1], i[2], n0, n1);
    i[ax] = n[ax] - 1;
    const int64_t hi = I3(i[0], i[1], i[2], n0, n1);
    i[ax] = n[ax] - 2;
    const int64_t hi1 = I3(i[0], i[1], i[2], n0, n1);
    A[lo] = A[lo1];
    A[hi] = A[hi1];
}

// ---- iteration kernels ---------------------------------------------------------------------
// compute_P! and compute_τ! of cell (x, y, z): τxx, τyy, τzz are written at the index whose ∇V
// is this cell's, τxy, τxz, τyz at the cell's own index.
template <typename T, int MODE = S3_PLAIN, typename I = int64_t>
__global__ void s3_Ptau_k(S3A<T> a, S3P<T> p) {
    S3_IDXT;
    const I c = I3T(x, y, z, nx, ny);
    const T d = s3_divV<T, I>(a, p, x, y, z);
    if constexpr (MODE == S3_DEFECT) {  // the correction's continuity residual includes the outer one
        const T dp = d + a.fp[c];
        a.divV[c] = dp;
        a.Pt[c] = a.Pt[c] - a.dtPt[c] * dp;
    } else {
        a.divV[c] = d;
        if constexpr (MODE == S3_PLAIN) a.Pt[c] = a.Pt[c] - a.dtPt[c] * d;
    }
    const T m = a.Mus[c];
    const bool iy = y >= 1 && y <= ny - 2, iz = z >= 1 && z <= nz - 2, ix = x >= 1 && x <= nx - 2;
    if (iy && iz)
        a.txx[I3T(x, y - 1, z - 1, nx, ny - 2)] =
            s3_tnn(m, a.Vx[I3T(x + 1, y, z, nx + 1, ny)], a.Vx[I3T(x, y, z, nx + 1, ny)], p.dx, d);
    if (ix && iz)
        a.tyy[I3T(x - 1, y, z - 1, nx - 2, ny)] =
            s3_tnn(m, a.Vy[I3T(x, y + 1, z, nx, ny + 1)], a.Vy[I3T(x, y, z, nx, ny + 1)], p.dy, d);
    if (ix && iy)
        a.tzz[I3T(x - 1, y - 1, z, nx - 2, ny - 2)] =
            s3_tnn(m, a.Vz[I3T(x, y, z + 1, nx, ny)], a.Vz[I3T(x, y, z, nx, ny)], p.dz, d);
    if (x < nx - 1 && y < ny - 1 && z < nz - 2) s3_txy<T, I>(a, p, x, y, z);
    if (x < nx - 1 && y < ny - 2 && z < nz - 1) s3_txz<T, I>(a, p, x, y, z);
    if (x < nx - 2 && y < ny - 1 && z < nz - 1) s3_tyz<T, I>(a, p, x, y, z);
}

template <typename T, int MODE = S3_PLAIN, typename I = int64_t>
__global__ void s3_dVV_k(S3A<T> a, S3P<T> p) {
    S3_IDXT;
    s3_dV<T, MODE, I>(a, p, x, y, z, true);
}

// The loop body's six copies (bc_x!(Vy), bc_x!(Vz), bc_y!(Vx), bc_y!(Vz), bc_z!(Vx), bc_z!(Vy)):
// velocity component c is copied along the two axes other than c. Job j = 4*c + face: faces 0/1
// are the low/high planes of the first copied axis, 2/3 of the second. The value written at a
// boundary cell is A[clamp(i)] with every copied axis clamped into [1, n-2]: that is what the
// sequence of two copies leaves, in either order, and no source is itself written here.
template <typename T>
__global__ void s3_bc_k(S3A<T> a) {
    const int job = blockIdx.y, c = job >> 2, face = job & 3;
    T* A = c == 0 ? a.Vx : c == 1 ? a.Vy : a.Vz;
    const int64_t n[3] = {a.nx + (c == 0), a.ny + (c == 1), a.nz + (c == 2)};
    const int ax0 = c == 0 ? 1 : 0, ax1 = c == 2 ? 1 : 2;  // the copied axes
    const int fa = face < 2 ? ax0 : ax1;                   // this face's axis
    const int u0 = fa == 0 ? 1 : 0, u1 = fa == 2 ? 1 : 2;  // axes spanning the face
    const int64_t cnt = n[u0] * n[u1];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t i[3];
        i[u0] = t % n[u0];
        i[u1] = t / n[u0];
        i[fa] = (face & 1) ? n[fa] - 1 : 0;
        int64_t s[3] = {i[0], i[1], i[2]};
        s[ax0] = s[ax0] < 1 ? 1 : s[ax0] > n[ax0] - 2 ? n[ax0] - 2 : s[ax0];
        s[ax1] = s[ax1] < 1 ? 1 : s[ax1] > n[ax1] - 2 ? n[ax1] - 2 : s[ax1];
        A[I3(i[0], i[1], i[2], n[0], n[1])] = A[I3(s[0], s[1], s[2], n[0], n[1])];
    }
}

// ---- one launch per iteration ----------------------------------------------------------------
// s3_fused_k runs compute_P!, compute_τ!, compute_dV!, compute_V! and the six free-slip copies of
// one iteration (Stokes3D.jl:131-137) as one z-sweep. The state moves from (V, Pt) to (V2, Pt2):
// neighbouring CTAs read each other's old V and Pt while writing their own. dVdτ is updated in
// place (each value only at its own face). The stresses, ∇V and R live in registers and shared
// memory only: per cell 20 words move (V, Pt, dτPt, Mus, Rog, dVdτ, dτV read, V2, Pt2, dVdτ
// written) against ~40 for the kernels that store them.
//
// Block: 32 x S3F_TY threads at positions X = 30 bx - 1 + tx, Y = (S3F_TY - 2) by - 1 + ty; the
// outer ring only computes the quantities its neighbours need. A position holds the cell (X, Y, k),
// the faces Vx (X, Y, k) (low x side of cell X), Vy (X, Y, k) and Vz (X, Y, k) (low z side), the
// x-y edge at the cell's low-x low-y corner (τxy) and, one level up, the x-z and y-z edges at its
// low-x / low-y side between planes k and k+1 (τxz, τyz). Per plane k: (1) every thread computes
// the plane-k quantities of its position and the level-(k+1/2) edges; (2) Rx, Ry of the faces in
// plane k and Rz of the Vz face k (between cells k-1 and k) from its own values and those of the
// neighbours in shared memory; (3) the updates and the free-slip copies: the thread of an inner
// face writes the boundary faces that copy it (s3_bc_k's clamped source), faces outside the
// updated range keep their old value. Bit-identical to the one-to-one kernels (same operations on
// the same operands, in the reference's order).
constexpr int S3F_TY = 16;

template <typename T>
struct S3Out {
    T *Vx, *Vy, *Vz, *Pt;
};

template <typename T, int MODE>
__global__ void __launch_bounds__(32 * S3F_TY) s3_fused_k(S3A<T> a, S3Out<T> o, S3P<T> p, int Lz) {
    static_assert(MODE == S3_PLAIN || MODE == S3_DEFECT, "update modes only");
    __shared__ T sPt[S3F_TY][32], sTxx[S3F_TY][32], sTyy[S3F_TY][32], sTxy[S3F_TY][32];
    __shared__ T sLxz[2][S3F_TY][32], sLyz[2][S3F_TY][32];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t nx = a.nx, ny = a.ny, nz = a.nz;
    const int64_t X = (int64_t)blockIdx.x * 30 - 1 + tx, Y = (int64_t)blockIdx.y * (S3F_TY - 2) - 1 + ty;
    const int64_t z0 = (int64_t)blockIdx.z * Lz, z1 = z0 + Lz < nz + 1 ? z0 + Lz : nz + 1;
    const bool own = tx >= 1 && tx <= 30 && ty >= 1 && ty <= S3F_TY - 2;
    const T* M = a.Mus;
    // existence of this position's objects in x-y
    const bool pos = X >= 0 && Y >= 0;
    const bool cell_xy = pos && X < nx && Y < ny;
    const bool vx_xy = pos && X <= nx && Y < ny, vy_xy = pos && X < nx && Y <= ny;
    const bool xin = X >= 1 && X <= nx - 2, yin = Y >= 1 && Y <= ny - 2;
    const bool txy_xy = X >= 1 && X <= nx - 1 && Y >= 1 && Y <= ny - 1;
    const bool txz_xy = X >= 1 && X <= nx - 1 && yin;  // τxz at (X-1, Y-1, .)
    const bool tyz_xy = xin && Y >= 1 && Y <= ny - 1;  // τyz at (X-1, Y-1, .)
    auto VX = [&](int64_t x, int64_t y, int64_t z) { return I3(x, y, z, nx + 1, ny); };
    auto VY = [&](int64_t x, int64_t y, int64_t z) { return I3(x, y, z, nx, ny + 1); };
    auto VZ = [&](int64_t x, int64_t y, int64_t z) { return I3(x, y, z, nx, ny); };
    auto C3 = [&](int64_t x, int64_t y, int64_t z) { return I3(x, y, z, nx, ny); };

    // carried along z: own V faces of plane k, Mus of plane k at (X,Y), (X-1,Y), (X,Y-1); from
    // plane k-1: τzz and the new Pt of the own cell, Rog; the own edges of level k-1/2
    T vx = 0, vy = 0, vz = 0, m00 = 0, m10 = 0, m01 = 0;
    T tzz_m = 0, pt_m = 0, rog_m = 0, lxz_m = 0, lyz_m = 0;
    const int64_t kb = z0 >= 1 ? z0 - 1 : 0;  // plane k0-1 is recomputed for Rz of face k0
    if (kb < nz) {
        if (vx_xy) vx = a.Vx[VX(X, Y, kb)];
        if (vy_xy) vy = a.Vy[VY(X, Y, kb)];
        if (cell_xy) vz = a.Vz[VZ(X, Y, kb)];
        if (cell_xy) m00 = M[C3(X, Y, kb)];
        if (X >= 1 && X <= nx && Y >= 0 && Y < ny) m10 = M[C3(X - 1, Y, kb)];
        if (Y >= 1 && Y <= ny && X >= 0 && X < nx) m01 = M[C3(X, Y - 1, kb)];
    }
    for (int64_t k = kb; k < z1; ++k) {
        const bool plane = k < nz;  // plane k holds cells (k = nz: only the Vz faces k)
        const bool out = own && k >= z0;
        // ---- loads of plane k+1 (own faces and Mus) and the neighbour values of plane k
        T vx_n = 0, vy_n = 0, vz_n = 0, m00_n = 0, m10_n = 0, m01_n = 0, m11 = 0;
        T vx_r = 0, vy_u = 0, vx_d = 0, vy_l = 0, vzl_n = 0, vzd_n = 0;
        if (plane) {
            if (vx_xy && k + 1 < nz) vx_n = a.Vx[VX(X, Y, k + 1)];
            if (vy_xy && k + 1 < nz) vy_n = a.Vy[VY(X, Y, k + 1)];
            if (cell_xy) vz_n = a.Vz[VZ(X, Y, k + 1)];  // face k+1 <= nz
            if (cell_xy && k + 1 < nz) m00_n = M[C3(X, Y, k + 1)];
            if (X >= 1 && X <= nx && Y >= 0 && Y < ny && k + 1 < nz) m10_n = M[C3(X - 1, Y, k + 1)];
            if (Y >= 1 && Y <= ny && X >= 0 && X < nx && k + 1 < nz) m01_n = M[C3(X, Y - 1, k + 1)];
            if (X >= 1 && Y >= 1 && X <= nx && Y <= ny) m11 = M[C3(X - 1, Y - 1, k)];
            if (cell_xy) {
                vx_r = a.Vx[VX(X + 1, Y, k)];
                vy_u = a.Vy[VY(X, Y + 1, k)];
            }
            if (txy_xy) {
                vx_d = a.Vx[VX(X, Y - 1, k)];
                vy_l = a.Vy[VY(X - 1, Y, k)];
            }
            if (txz_xy && k + 1 < nz) vzl_n = a.Vz[VZ(X - 1, Y, k + 1)];
            if (tyz_xy && k + 1 < nz) vzd_n = a.Vz[VZ(X, Y - 1, k + 1)];
        }
        // ---- plane-k quantities of this position and its level-(k+1/2) edges
        T pt_new = 0, d = 0, txx = 0, tyy = 0, tzz = 0, txy = 0, lxz = 0, lyz = 0, rog = 0;
        if (plane && cell_xy) {
            const int64_t c = C3(X, Y, k);
            d = (div_c(vx_r - vx, p.dx) + div_c(vy_u - vy, p.dy)) + div_c(vz_n - vz, p.dz);
            T dp = d;
            if constexpr (MODE == S3_DEFECT) dp = d + a.fp[c];
            pt_new = a.Pt[c] - a.dtPt[c] * dp;
            if constexpr (MODE == S3_PLAIN) rog = a.Rog[c];
            if (yin && k >= 1 && k <= nz - 2) txx = s3_tnn(m00, vx_r, vx, p.dx, d);
            if (xin && k >= 1 && k <= nz - 2) tyy = s3_tnn(m00, vy_u, vy, p.dy, d);
            if (xin && yin) tzz = s3_tnn(m00, vz_n, vz, p.dz, d);
        }
        if (plane && txy_xy && k >= 1 && k <= nz - 2)
            txy = s3_tsh(m11, m01, m10, m00, vx - vx_d, p.dy, vy - vy_l, p.dx);
        if (plane && txz_xy && k <= nz - 2) lxz = s3_tsh(m10, m00, m10_n, m00_n, vx_n - vx, p.dz, vz_n - vzl_n, p.dx);
        if (plane && tyz_xy && k <= nz - 2) lyz = s3_tsh(m01, m00, m01_n, m00_n, vy_n - vy, p.dz, vz_n - vzd_n, p.dy);
        __syncthreads();  // A: the previous plane's neighbour reads are done
        sPt[ty][tx] = pt_new;
        sTxx[ty][tx] = txx;
        sTyy[ty][tx] = tyy;
        sTxy[ty][tx] = txy;
        sLxz[k & 1][ty][tx] = lxz;
        sLyz[k & 1][ty][tx] = lyz;
        __syncthreads();  // B: plane k and level k+1/2 published
        if (out) {
            // compute_dV! / compute_V! of the faces of this position (r: index of R, dVdτ, dτV)
            const int64_t r = I3(X - 1, Y - 1, k - 1, nx - 1, ny - 2);
            T ux = vx;  // the updated Vx face (X, Y, k): old value outside @inn
            if (plane && X >= 1 && X <= nx - 1 && yin && k >= 1 && k <= nz - 2) {
                const T A = txx - sTxx[ty][tx - 1], B = sTxy[ty + 1][tx] - txy, Cc = lxz - lxz_m;
                const T P = pt_new - sPt[ty][tx - 1];
                T R = ((div_c(A, p.dx) + div_c(B, p.dy)) + div_c(Cc, p.dz)) - div_c(P, p.dx);
                if constexpr (MODE == S3_DEFECT) R = R + a.fx[r];
                const T dv = p.dampX * a.dVx[r] + R;
                a.dVx[r] = dv;
                ux = vx + a.dtVx[r] * dv;
            }
            T uy = vy;
            if (plane && xin && Y >= 1 && Y <= ny - 1 && k >= 1 && k <= nz - 2) {
                const int64_t ry = I3(X - 1, Y - 1, k - 1, nx - 2, ny - 1);
                const T A = tyy - sTyy[ty - 1][tx], B = sTxy[ty][tx + 1] - txy, Cc = lyz - lyz_m;
                const T P = pt_new - sPt[ty - 1][tx];
                T R = ((div_c(A, p.dy) + div_c(B, p.dx)) + div_c(Cc, p.dz)) - div_c(P, p.dy);
                if constexpr (MODE == S3_DEFECT) R = R + a.fy[ry];
                const T dv = p.dampY * a.dVy[ry] + R;
                a.dVy[ry] = dv;
                uy = vy + a.dtVy[ry] * dv;
            }
            T uz = vz;
            if (xin && yin && k >= 1 && k <= nz - 1) {
                const int64_t rz = I3(X - 1, Y - 1, k - 1, nx - 2, ny - 2);
                const T A = tzz - tzz_m;
                const T B = sLxz[(k - 1) & 1][ty][tx + 1] - lxz_m, Cc = sLyz[(k - 1) & 1][ty + 1][tx] - lyz_m;
                const T P = pt_new - pt_m;
                T R;
                if constexpr (MODE == S3_DEFECT) {
                    R = (((div_c(A, p.dz) + div_c(B, p.dx)) + div_c(Cc, p.dy)) - div_c(P, p.dz)) + a.fz[rz];
                } else {
                    const T G = (rog_m + rog) * T(0.5);
                    R = (((div_c(A, p.dz) + div_c(B, p.dx)) + div_c(Cc, p.dy)) - div_c(P, p.dz)) + G;
                }
                const T dv = p.dampZ * a.dVz[rz] + R;
                a.dVz[rz] = dv;
                uz = vz + a.dtVz[rz] * dv;
            }
            // the new state and the free-slip copies (bc_y!(Vx), bc_z!(Vx), bc_x!(Vy), bc_z!(Vy),
            // bc_x!(Vz), bc_y!(Vz)): the source of a copied face is the face with its copied axes
            // clamped into [1, n-2]; that source's thread writes it
            if (plane && vx_xy && yin && k >= 1 && k <= nz - 2) {
                const int ny0 = Y == 1 ? 1 : 0, ny1 = Y == ny - 2 ? 1 : 0, nz0 = k == 1 ? 1 : 0, nz1 = k == nz - 2 ? 1 : 0;
                for (int dy = -ny0; dy <= ny1; ++dy)
                    for (int dz = -nz0; dz <= nz1; ++dz) o.Vx[VX(X, Y + dy, k + dz)] = ux;
            }
            if (plane && vy_xy && xin && k >= 1 && k <= nz - 2) {
                const int nx0 = X == 1 ? 1 : 0, nx1 = X == nx - 2 ? 1 : 0, nz0 = k == 1 ? 1 : 0, nz1 = k == nz - 2 ? 1 : 0;
                for (int dx = -nx0; dx <= nx1; ++dx)
                    for (int dz = -nz0; dz <= nz1; ++dz) o.Vy[VY(X + dx, Y, k + dz)] = uy;
            }
            if (cell_xy && xin && yin) {  // Vz faces k = 0 .. nz
                const int nx0 = X == 1 ? 1 : 0, nx1 = X == nx - 2 ? 1 : 0, ny0 = Y == 1 ? 1 : 0, ny1 = Y == ny - 2 ? 1 : 0;
                for (int dx = -nx0; dx <= nx1; ++dx)
                    for (int dy = -ny0; dy <= ny1; ++dy) o.Vz[VZ(X + dx, Y + dy, k)] = uz;
            }
            if (plane && cell_xy) o.Pt[C3(X, Y, k)] = pt_new;
        }
        // ---- carry to plane k+1
        tzz_m = tzz;
        pt_m = pt_new;
        rog_m = rog;
        lxz_m = lxz;
        lyz_m = lyz;
        vx = vx_n;
        vy = vy_n;
        vz = vz_n;
        m00 = m00_n;
        m10 = m10_n;
        m01 = m01_n;
    }
}

template <typename T, int MODE>
static void s3_fused_launch(const S3A<T>& a, const S3Out<T>& o, const S3P<T>& p, cudaStream_t s) {
    static int occ = 0;
    if (!occ) occ = resident_ctas(s3_fused_k<T, MODE>, 32 * S3F_TY, 0);
    DeviceState* st = nullptr;
    current_state(&st);
    const int64_t gx = (a.nx + 1 + 29) / 30, gy = (a.ny + 1 + S3F_TY - 3) / (S3F_TY - 2);
    int Lz = auto_loopsize(gx * gy, a.nz + 1, (int64_t)occ * (st ? st->num_sms : 152));
    const dim3 grd((unsigned)gx, (unsigned)gy, (unsigned)((a.nz + 1 + Lz - 1) / Lz));
    s3_fused_k<T, MODE><<<grd, dim3(32, S3F_TY, 1), 0, s>>>(a, o, p, Lz);
}

// y32 = (float) x64 (rounding of the outer residual for the FP32 sweeps)
__global__ void s3_to_f32(float* y, const double* x, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}
// x64 += (double) d32 (FP64 update of the outer state with the FP32 correction)
__global__ void s3_axpy32(double* x, const float* d, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += (double)d[i];
}

__device__ __forceinline__ double s3_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// sum |a| of four arrays into out[0..3] (job = blockIdx.y)
template <typename T>
__global__ void s3_sum_abs_k(const T* a0, int64_t n0, const T* a1, int64_t n1, const T* a2, int64_t n2, const T* a3,
                             int64_t n3, double* out) {
    const T* a = blockIdx.y == 0 ? a0 : blockIdx.y == 1 ? a1 : blockIdx.y == 2 ? a2 : a3;
    const int64_t n = blockIdx.y == 0 ? n0 : blockIdx.y == 1 ? n1 : blockIdx.y == 2 ? n2 : n3;
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += fabs((double)a[i]);
    s = s3_warp_sum(s);
    if ((threadIdx.x & 31) == 0) atomicAdd(out + blockIdx.y, s);
}

// ---- host side -----------------------------------------------------------------------------
static int check3(const ps_array& a, int64_t n0, int64_t n1, int64_t n2, int32_t dt, const char* name) {
    PS_TRY(check_array(a, name));
    if (a.dtype != dt) return fail(PS_ERR_DTYPE, "Stokes3D: array %s has a different dtype", name);
    return check_shape(a, n0, n1, n2, name);
}

static int check_fields3(const ps_stokes3d_fields* f, bool need_dt) {
    if (!f) return fail(PS_ERR_NULL, "Stokes3D: NULL fields");
    PS_TRY(check_array(f->Pt, "Pt"));
    const int64_t X = f->Pt.n[0], Y = f->Pt.n[1], Z = f->Pt.n[2];
    const int32_t dt = f->Pt.dtype;
    if (X < 3 || Y < 3 || Z < 3) return fail(PS_ERR_SHAPE, "Stokes3D: Pt must have nx, ny, nz >= 3");
    if (X > (int64_t)INT32_MAX || Y > 65535 * 8 || Z > 65535) return fail(PS_ERR_SHAPE, "Stokes3D: grid too large");
    PS_TRY(check3(f->Vx, X + 1, Y, Z, dt, "Vx"));
    PS_TRY(check3(f->Vy, X, Y + 1, Z, dt, "Vy"));
    PS_TRY(check3(f->Vz, X, Y, Z + 1, dt, "Vz"));
    PS_TRY(check3(f->divV, X, Y, Z, dt, "∇V"));
    PS_TRY(check3(f->txx, X, Y - 2, Z - 2, dt, "τxx"));
    PS_TRY(check3(f->tyy, X - 2, Y, Z - 2, dt, "τyy"));
    PS_TRY(check3(f->tzz, X - 2, Y - 2, Z, dt, "τzz"));
    PS_TRY(check3(f->txy, X - 1, Y - 1, Z - 2, dt, "τxy"));
    PS_TRY(check3(f->txz, X - 1, Y - 2, Z - 1, dt, "τxz"));
    PS_TRY(check3(f->tyz, X - 2, Y - 1, Z - 1, dt, "τyz"));
    PS_TRY(check3(f->Rx, X - 1, Y - 2, Z - 2, dt, "Rx"));
    PS_TRY(check3(f->Ry, X - 2, Y - 1, Z - 2, dt, "Ry"));
    PS_TRY(check3(f->Rz, X - 2, Y - 2, Z - 1, dt, "Rz"));
    PS_TRY(check3(f->dVxdtau, X - 1, Y - 2, Z - 2, dt, "dVxdτ"));
    PS_TRY(check3(f->dVydtau, X - 2, Y - 1, Z - 2, dt, "dVydτ"));
    PS_TRY(check3(f->dVzdtau, X - 2, Y - 2, Z - 1, dt, "dVzdτ"));
    PS_TRY(check3(f->Mus, X, Y, Z, dt, "Mus"));
    PS_TRY(check3(f->Rog, X, Y, Z, dt, "Rog"));
    if (need_dt) {
        PS_TRY(check3(f->dtauPt, X, Y, Z, dt, "dτPt"));
        PS_TRY(check3(f->dtauVx, X - 1, Y - 2, Z - 2, dt, "dτVx"));
        PS_TRY(check3(f->dtauVy, X - 2, Y - 1, Z - 2, dt, "dτVy"));
        PS_TRY(check3(f->dtauVz, X - 2, Y - 2, Z - 1, dt, "dτVz"));
    }
    return PS_OK;
}

template <typename T>
static S3A<T> s3a(const ps_stokes3d_fields* f) {
    auto P = [](const ps_array& a) { return static_cast<T*>(a.ptr); };
    S3A<T> a;
    a.fx = a.fy = a.fz = a.fp = nullptr;
    a.Pt = P(f->Pt);
    a.dtPt = P(f->dtauPt);
    a.divV = P(f->divV);
    a.Vx = P(f->Vx);
    a.Vy = P(f->Vy);
    a.Vz = P(f->Vz);
    a.txx = P(f->txx);
    a.tyy = P(f->tyy);
    a.tzz = P(f->tzz);
    a.txy = P(f->txy);
    a.txz = P(f->txz);
    a.tyz = P(f->tyz);
    a.Rx = P(f->Rx);
    a.Ry = P(f->Ry);
    a.Rz = P(f->Rz);
    a.dVx = P(f->dVxdtau);
    a.dVy = P(f->dVydtau);
    a.dVz = P(f->dVzdtau);
    a.dtVx = P(f->dtauVx);
    a.dtVy = P(f->dtauVy);
    a.dtVz = P(f->dtauVz);
    a.Mus = P(f->Mus);
    a.Rog = P(f->Rog);
    a.nx = f->Pt.n[0];
    a.ny = f->Pt.n[1];
    a.nz = f->Pt.n[2];
    return a;
}

// grid over (wx, wy, wz) with (32, 8, 1) blocks
static dim3 g3(int64_t wx, int64_t wy, int64_t wz) {
    return dim3((unsigned)((wx + 31) / 32), (unsigned)((wy + 7) / 8), (unsigned)wz);
}

enum S3Kernel { S3_TIMESTEPS, S3_P, S3_TAU, S3_DV, S3_V, S3_PTAU, S3_DVV, S3_BC };

// The iteration kernels in 32-bit index arithmetic where every array index fits (the largest array,
// a staggered velocity, has fewer than (nx+1)(ny+1)(nz+1) < 2^31 elements), else 64-bit.
template <typename T>
static bool s3_idx32(const S3A<T>& a) {
    return (a.nx + 1) * (a.ny + 1) * (a.nz + 1) < (int64_t(1) << 31);
}
template <typename T, int MODE>
static void s3_iteration_kernels(const S3A<T>& a, const S3P<T>& p, dim3 gc, dim3 b, cudaStream_t s) {
    if (s3_idx32(a)) {
        s3_Ptau_k<T, MODE, int><<<gc, b, 0, s>>>(a, p);
        s3_dVV_k<T, MODE, int><<<gc, b, 0, s>>>(a, p);
    } else {
        s3_Ptau_k<T, MODE, int64_t><<<gc, b, 0, s>>>(a, p);
        s3_dVV_k<T, MODE, int64_t><<<gc, b, 0, s>>>(a, p);
    }
}

template <typename T>
static void s3_launch(S3Kernel k, const S3A<T>& a, const S3P<T>& p, cudaStream_t s) {
    const dim3 b(32, 8, 1);
    // The reference's grid is the max extent of the array arguments ((nx+1, ny+1, nz+1) where a
    // staggered velocity is one), but every statement's mask lies inside (nx, ny, nz): the
    // threads beyond it do nothing, so all kernels run on the cell grid.
    const dim3 gc = g3(a.nx, a.ny, a.nz);
    switch (k) {
    case S3_TIMESTEPS: s3_timesteps_k<T><<<gc, b, 0, s>>>(a, p); break;
    case S3_P: s3_P_k<T><<<gc, b, 0, s>>>(a, p); break;
    case S3_TAU: s3_tau_k<T><<<gc, b, 0, s>>>(a, p); break;
    case S3_DV: s3_dV_k<T><<<gc, b, 0, s>>>(a, p); break;
    case S3_V: s3_V_k<T><<<gc, b, 0, s>>>(a); break;
    case S3_PTAU:
        if (s3_idx32(a)) s3_Ptau_k<T, S3_PLAIN, int><<<gc, b, 0, s>>>(a, p);
        else s3_Ptau_k<T, S3_PLAIN, int64_t><<<gc, b, 0, s>>>(a, p);
        break;
    case S3_DVV:
        if (s3_idx32(a)) s3_dVV_k<T, S3_PLAIN, int><<<gc, b, 0, s>>>(a, p);
        else s3_dVV_k<T, S3_PLAIN, int64_t><<<gc, b, 0, s>>>(a, p);
        break;
    case S3_BC: {
        const int64_t face = std::max(std::max((a.nx + 1) * (a.ny + 1), (a.nx + 1) * (a.nz + 1)), (a.ny + 1) * (a.nz + 1));
        s3_bc_k<T><<<dim3((unsigned)std::min<int64_t>((face + 255) / 256, 1024), 12), 256, 0, s>>>(a);
        break;
    }
    }
}

// n iterations of MODE on the state (a.Vx, a.Vy, a.Vz, a.Pt): pairs of one-launch iterations
// through the second set B (the state is back in a's arrays after each pair), then the remaining
// one or two iterations as the three kernels that also store ∇V, τ and R (the reference's loop
// body leaves them, and the solvers' residual norms read them). With n >= 1 the last iteration
// always stores. B.Vx.. B.Pt: arrays of the shapes of a's.
template <typename T, int MODE>
static void s3_iterations(const S3A<T>& a, const S3Out<T>& B, const S3P<T>& p, int64_t n, cudaStream_t s,
                          bool one_launch) {
    if (n <= 0) return;
    const int64_t pairs = one_launch ? (n - 1) / 2 : 0;
    S3A<T> b = a;
    b.Vx = B.Vx;
    b.Vy = B.Vy;
    b.Vz = B.Vz;
    b.Pt = B.Pt;
    const S3Out<T> toB{B.Vx, B.Vy, B.Vz, B.Pt}, toA{a.Vx, a.Vy, a.Vz, a.Pt};
    for (int64_t i = 0; i < pairs; ++i) {
        s3_fused_launch<T, MODE>(a, toB, p, s);
        s3_fused_launch<T, MODE>(b, toA, p, s);
    }
    const dim3 b3(32, 8, 1), gc = g3(a.nx, a.ny, a.nz);
    for (int64_t i = 2 * pairs; i < n; ++i) {
        s3_iteration_kernels<T, MODE>(a, p, gc, b3, s);
        s3_launch(S3_BC, a, p, s);
    }
}

// divV, the stresses and Rx, Ry, Rz of the FP64 state (the reference's statements, no update)
static void s3_residual(const S3A<double>& a, const S3P<double>& p, cudaStream_t s) {
    const dim3 b(32, 8, 1), gc = g3(a.nx, a.ny, a.nz);
    s3_iteration_kernels<double, S3_RESIDUAL>(a, p, gc, b, s);
}

// Library scratch of the iterate entry point: grow-only, one per device and stream.
struct S3Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};
static std::mutex g_s3_mutex;
static std::map<std::pair<int, cudaStream_t>, S3Scratch> g_s3_scratch;

static int s3_scratch(size_t bytes, char** out, cudaStream_t s) {
    int dev = 0;
    PS_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_s3_mutex);
    S3Scratch& sc = g_s3_scratch[{dev, s}];
    if (sc.bytes < bytes) {
        if (sc.ptr) {
            PS_CUDA_TRY(cudaStreamSynchronize(s));
            PS_CUDA_TRY(cudaFree(sc.ptr));
            sc.ptr = nullptr;
            sc.bytes = 0;
        }
        PS_CUDA_TRY(cudaMalloc(&sc.ptr, bytes));
        sc.bytes = bytes;
    }
    *out = static_cast<char*>(sc.ptr);
    return PS_OK;
}

void stokes3d_free_scratch() {
    std::lock_guard<std::mutex> lk(g_s3_mutex);
    for (auto& kv : g_s3_scratch)
        if (kv.second.ptr) cudaFree(kv.second.ptr);
    g_s3_scratch.clear();
}

static int s3_entry(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, S3Kernel k, void* stream, int sync,
                    const char* what) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_fields3(f, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (f->Pt.dtype == PS_F64)
        s3_launch<double>(k, s3a<double>(f), s3p<double>(*p), s);
    else
        s3_launch<float>(k, s3a<float>(f), s3p<float>(*p), s);
    return finish_launch(s, sync, what);
}

static double now_s3() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Mixed precision (the precision extension of the PT solvers, as ps_stokes2d_solve mode 1): FP32 PT
// sweeps on the correction (δV, δP) with the FP64 residual of the outer state as source; FP64
// residual, update and convergence check. The outer residual uses the reference's FP64 statements
// (S3_RESIDUAL kernels) on the caller's arrays, so the final err is the reference's err of the
// returned state.
static int solve_mixed3(const ps_stokes3d_fields* f, const ps_stokes3d_params* pp, double tol, int64_t max_iter,
                        int64_t nout, double max_seconds, double inner_rtol, double* red, ps_solve_stats* st,
                        cudaStream_t s) {
    const int64_t nx = f->Pt.n[0], ny = f->Pt.n[1], nz = f->Pt.n[2];
    const int64_t nC = nx * ny * nz, nVx = (nx + 1) * ny * nz, nVy = nx * (ny + 1) * nz, nVz = nx * ny * (nz + 1);
    const int64_t nRx = (nx - 1) * (ny - 2) * (nz - 2), nRy = (nx - 2) * (ny - 1) * (nz - 2),
                  nRz = (nx - 2) * (ny - 2) * (nz - 1);
    // float buffers, in this order: δVx δVy δVz δP dVx dVy dVz (zeroed before every inner sweep),
    // txx tyy tzz txy txz tyz divV Rx Ry Rz, dtPt dtVx dtVy dtVz Mus, fx fy fz fp, and the second
    // set δVx δVy δVz δP of the one-launch sweeps
    const int64_t cnt[30] = {nVx, nVy, nVz, nC, nRx, nRy, nRz,
                             numel(f->txx), numel(f->tyy), numel(f->tzz), numel(f->txy), numel(f->txz), numel(f->tyz),
                             nC, nRx, nRy, nRz, nC, nRx, nRy, nRz, nC, nRx, nRy, nRz, nC, nVx, nVy, nVz, nC};
    size_t off[31];
    off[0] = 0;
    for (int k = 0; k < 30; k++) off[k + 1] = off[k] + ((cnt[k] * 4 + 255) / 256) * 256;
    float* base = nullptr;
    PS_CUDA_TRY(cudaMalloc(&base, off[30]));
    auto F = [&](int k) { return reinterpret_cast<float*>(reinterpret_cast<char*>(base) + off[k]); };
    S3A<float> a;
    a.Vx = F(0); a.Vy = F(1); a.Vz = F(2); a.Pt = F(3);
    a.dVx = F(4); a.dVy = F(5); a.dVz = F(6);
    a.txx = F(7); a.tyy = F(8); a.tzz = F(9); a.txy = F(10); a.txz = F(11); a.tyz = F(12);
    a.divV = F(13); a.Rx = F(14); a.Ry = F(15); a.Rz = F(16);
    a.dtPt = F(17); a.dtVx = F(18); a.dtVy = F(19); a.dtVz = F(20);
    a.Mus = F(21); a.Rog = nullptr;
    a.fx = F(22); a.fy = F(23); a.fz = F(24); a.fp = F(25);
    a.nx = nx; a.ny = ny; a.nz = nz;
    const S3P<float> p32 = s3p<float>(*pp);
    const S3P<double> p64 = s3p<double>(*pp);
    const S3A<double> a64 = s3a<double>(f);
    int rc = PS_OK;
    const S3Out<float> B32{F(26), F(27), F(28), F(29)};
    cudaError_t e = cudaMemsetAsync(base, 0, off[30], s);
    s3_to_f32<<<1024, 256, 0, s>>>(F(21), a64.Mus, nC);
    s3_timesteps_k<float><<<g3(nx, ny, nz), dim3(32, 8, 1), 0, s>>>(a, p32);
    // the corrections keep the free-slip copies of the state they are added to: give the state
    // those copies first, as the first FP64 iteration would
    s3_launch(S3_BC, a64, p64, s);
    double* red_in = red;       // Σ|.| of the inner sweep (Rx, Ry, Rz, divV)
    double* red_out = red + 4;  // of the FP64 outer residual
    const int64_t n4[4] = {nRx, nRy, nRz, nC};
    const dim3 gr((unsigned)std::max<int64_t>(1, std::min<int64_t>((nC + 1023) / 1024, 1024)), 4);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        s3_iterations<float, S3_DEFECT>(a, B32, p32, nout, s, false);
        cudaMemsetAsync(red_in, 0, 4 * sizeof(double), s);
        s3_sum_abs_k<float><<<gr, 256, 0, s>>>(a.Rx, nRx, a.Ry, nRy, a.Rz, nRz, a.divV, nC, red_in);
        e = cudaStreamEndCapture(s, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) rc = cuda_fail(e, "ps_stokes3d_solve_mixed: graph capture");
    const double t0 = now_s3();
    double err = INFINITY, h[4];
    int64_t it = 0, outer = 0;
    auto norm = [&](const double* v) {
        double m = 0;
        for (int k = 0; k < 4; k++) m = std::max(m, v[k] / (double)n4[k]);
        return m;
    };
    auto finite4 = [](const double* v) {
        return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]) && std::isfinite(v[3]);
    };
    while (rc == PS_OK) {
        // FP64 residual of the outer state; its rounding to FP32 is the inner sweeps' source
        s3_residual(a64, p64, s);
        cudaMemsetAsync(red_out, 0, 4 * sizeof(double), s);
        s3_sum_abs_k<double><<<gr, 256, 0, s>>>(a64.Rx, nRx, a64.Ry, nRy, a64.Rz, nRz, a64.divV, nC, red_out);
        s3_to_f32<<<1024, 256, 0, s>>>(F(22), a64.Rx, nRx);
        s3_to_f32<<<1024, 256, 0, s>>>(F(23), a64.Ry, nRy);
        s3_to_f32<<<1024, 256, 0, s>>>(F(24), a64.Rz, nRz);
        s3_to_f32<<<1024, 256, 0, s>>>(F(25), a64.divV, nC);
        e = cudaMemcpyAsync(h, red_out, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "ps_stokes3d_solve_mixed(residual)");
            break;
        }
        if (!finite4(h)) {
            err = NAN;
            rc = fail(PS_ERR_NONFINITE, "ps_stokes3d_solve_mixed: non-finite FP64 residual");
            break;
        }
        err = norm(h);
        if (err < tol || it >= max_iter) break;
        if (max_seconds > 0 && now_s3() - t0 > max_seconds) {
            rc = fail(PS_ERR_TIMEOUT, "ps_stokes3d_solve_mixed: wall-clock limit reached (err %.3e)", err);
            break;
        }
        ++outer;
        cudaMemsetAsync(base, 0, off[7], s);  // δV, δP and the pseudo-velocities from zero
        const double target = std::max(err * inner_rtol, tol * 0.25);
        double ierr = INFINITY;
        while (it < max_iter) {
            e = cudaGraphLaunch(exec, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(h, red_in, sizeof(h), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "ps_stokes3d_solve_mixed(inner)");
                break;
            }
            it += nout;
            if (!finite4(h)) {
                rc = fail(PS_ERR_NONFINITE, "ps_stokes3d_solve_mixed: non-finite FP32 residual");
                break;
            }
            const double prev = ierr;
            ierr = norm(h);
            if (ierr < target) break;
            if (ierr > 0.98 * prev && ierr < err * 0.5) break;  // FP32 floor reached
        }
        if (rc != PS_OK) break;
        s3_axpy32<<<1024, 256, 0, s>>>(a64.Vx, a.Vx, nVx);
        s3_axpy32<<<1024, 256, 0, s>>>(a64.Vy, a.Vy, nVy);
        s3_axpy32<<<1024, 256, 0, s>>>(a64.Vz, a.Vz, nVz);
        s3_axpy32<<<1024, 256, 0, s>>>(a64.Pt, a.Pt, nC);
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamSynchronize(s);
    cudaFree(base);
    cudaGetLastError();
    st->iters = it;
    st->outer = outer;
    st->err = err;
    st->seconds = now_s3() - t0;
    st->converged = err < tol;
    if (rc == PS_OK && !(err < tol))
        rc = fail(PS_ERR_NOT_CONVERGED, "ps_stokes3d_solve_mixed: err %.3e after %lld iterations", err, (long long)it);
    return rc;
}

}  // namespace ps

using namespace ps;

extern "C" {

int ps_stokes3d_timesteps(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync) {
    return s3_entry(f, p, S3_TIMESTEPS, stream, sync, "ps_stokes3d_timesteps");
}
int ps_stokes3d_compute_P(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync) {
    return s3_entry(f, p, S3_P, stream, sync, "ps_stokes3d_compute_P");
}
int ps_stokes3d_compute_tau(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync) {
    return s3_entry(f, p, S3_TAU, stream, sync, "ps_stokes3d_compute_tau");
}
int ps_stokes3d_compute_dV(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync) {
    return s3_entry(f, p, S3_DV, stream, sync, "ps_stokes3d_compute_dV");
}
int ps_stokes3d_compute_V(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync) {
    return s3_entry(f, p, S3_V, stream, sync, "ps_stokes3d_compute_V");
}

static int bc3(ps_array A, void* stream, int sync, int ax, const char* what) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_array(A, "A"));
    if (A.n[0] < 3 || A.n[1] < 3 || A.n[2] < 3) return fail(PS_ERR_SHAPE, "%s: A must be 3-D with extents >= 3", what);
    const int o0 = ax == 0 ? 1 : 0, o1 = ax == 2 ? 1 : 2;
    if (A.n[o1] > 65535) return fail(PS_ERR_SHAPE, "%s: extent too large", what);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 g((unsigned)((A.n[o0] + 127) / 128), (unsigned)A.n[o1]);
    if (A.dtype == PS_F64)
        s3_bc_axis_k<double><<<g, 128, 0, s>>>(static_cast<double*>(A.ptr), A.n[0], A.n[1], A.n[2], ax);
    else
        s3_bc_axis_k<float><<<g, 128, 0, s>>>(static_cast<float*>(A.ptr), A.n[0], A.n[1], A.n[2], ax);
    return finish_launch(s, sync, what);
}

int ps_bc_x3d(ps_array A, void* stream, int sync) { return bc3(A, stream, sync, 0, "ps_bc_x3d"); }
int ps_bc_y3d(ps_array A, void* stream, int sync) { return bc3(A, stream, sync, 1, "ps_bc_y3d"); }
int ps_bc_z3d(ps_array A, void* stream, int sync) { return bc3(A, stream, sync, 2, "ps_bc_z3d"); }

int ps_stokes3d_iterate(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, int64_t n_iter, void* stream) {
    return ps_stokes3d_iterate_ex(f, p, n_iter, 0, stream);
}

int ps_stokes3d_iterate_ex(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, int64_t n_iter,
                           int32_t one_launch, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_fields3(f, true));
    if (!p) return fail(PS_ERR_NULL, "NULL params");
    if (n_iter < 0) return fail(PS_ERR_ARG, "n_iter must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_iter == 0) return PS_OK;
    if (!one_launch) {  // the three storing kernels per iteration, in place
        for (int64_t it = 0; it < n_iter; ++it) {
            if (f->Pt.dtype == PS_F64)
                s3_iterations<double, S3_PLAIN>(s3a<double>(f), S3Out<double>{}, s3p<double>(*p), 1, s, false);
            else
                s3_iterations<float, S3_PLAIN>(s3a<float>(f), S3Out<float>{}, s3p<float>(*p), 1, s, false);
        }
        return finish_launch(s, 1, "ps_stokes3d_iterate");
    }
    // the second state set of the one-launch iterations (grow-only library scratch per device and stream)
    const size_t es = elsize(f->Pt.dtype);
    const size_t nb[4] = {(size_t)numel(f->Vx) * es, (size_t)numel(f->Vy) * es, (size_t)numel(f->Vz) * es,
                          (size_t)numel(f->Pt) * es};
    size_t off[4], total = 0;
    for (int i = 0; i < 4; ++i) {
        off[i] = total;
        total += (nb[i] + 255) / 256 * 256;
    }
    char* base = nullptr;
    PS_TRY(s3_scratch(total, &base, s));
    if (f->Pt.dtype == PS_F64) {
        const S3Out<double> B{reinterpret_cast<double*>(base + off[0]), reinterpret_cast<double*>(base + off[1]),
                              reinterpret_cast<double*>(base + off[2]), reinterpret_cast<double*>(base + off[3])};
        s3_iterations<double, S3_PLAIN>(s3a<double>(f), B, s3p<double>(*p), n_iter, s, one_launch != 0);
    } else {
        const S3Out<float> B{reinterpret_cast<float*>(base + off[0]), reinterpret_cast<float*>(base + off[1]),
                             reinterpret_cast<float*>(base + off[2]), reinterpret_cast<float*>(base + off[3])};
        s3_iterations<float, S3_PLAIN>(s3a<float>(f), B, s3p<float>(*p), n_iter, s, one_launch != 0);
    }
    return finish_launch(s, 1, "ps_stokes3d_iterate");
}

int ps_stokes3d_err(const ps_stokes3d_fields* f, double out_mean_abs[4], void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_fields3(f, false));
    if (!out_mean_abs) return fail(PS_ERR_NULL, "NULL output");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* red = st->d_scratch;
    const int64_t n[4] = {numel(f->Rx), numel(f->Ry), numel(f->Rz), numel(f->divV)};
    PS_CUDA_TRY(cudaMemsetAsync(red, 0, 4 * sizeof(double), s));
    const dim3 g((unsigned)std::max<int64_t>(1, std::min<int64_t>((n[3] + 1023) / 1024, 1024)), 4);
    if (f->Pt.dtype == PS_F64)
        s3_sum_abs_k<double><<<g, 256, 0, s>>>(static_cast<const double*>(f->Rx.ptr), n[0],
                                               static_cast<const double*>(f->Ry.ptr), n[1],
                                               static_cast<const double*>(f->Rz.ptr), n[2],
                                               static_cast<const double*>(f->divV.ptr), n[3], red);
    else
        s3_sum_abs_k<float><<<g, 256, 0, s>>>(static_cast<const float*>(f->Rx.ptr), n[0],
                                              static_cast<const float*>(f->Ry.ptr), n[1],
                                              static_cast<const float*>(f->Rz.ptr), n[2],
                                              static_cast<const float*>(f->divV.ptr), n[3], red);
    double h[4];
    PS_CUDA_TRY(cudaMemcpyAsync(h, red, sizeof(h), cudaMemcpyDeviceToHost, s));
    PS_CUDA_TRY(cudaStreamSynchronize(s));
    for (int k = 0; k < 4; k++) out_mean_abs[k] = h[k] / (double)n[k];
    return finish_launch(s, 0, "ps_stokes3d_err");
}

int ps_stokes3d_solve(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, double tol, int64_t max_iter,
                      int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_fields3(f, true));
    if (!p || !stats) return fail(PS_ERR_NULL, "NULL params / stats");
    if (f->Pt.dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_stokes3d_solve: the arrays must be FP64");
    if (nout < 1) return fail(PS_ERR_ARG, "nout must be >= 1");
    if (!(tol > 0) || max_iter < 0) return fail(PS_ERR_ARG, "invalid tol / max_iter");
    memset(stats, 0, sizeof(*stats));
    // graphs are captured on a private stream ordered after `stream`
    cudaStream_t user = static_cast<cudaStream_t>(stream), s;
    PS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t ev;
    PS_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(s, ev, 0);
    const S3A<double> a = s3a<double>(f);
    const S3P<double> pp = s3p<double>(*p);
    double* red = st->d_scratch;
    const int64_t n[4] = {numel(f->Rx), numel(f->Ry), numel(f->Rz), numel(f->divV)};
    const dim3 gr((unsigned)std::max<int64_t>(1, std::min<int64_t>((n[3] + 1023) / 1024, 1024)), 4);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // the second state set of the one-launch iterations
    const size_t nb[4] = {(size_t)numel(f->Vx) * 8, (size_t)numel(f->Vy) * 8, (size_t)numel(f->Vz) * 8,
                          (size_t)numel(f->Pt) * 8};
    char* bbase = nullptr;
    cudaError_t e = cudaMalloc(&bbase, (nb[0] + nb[1] + nb[2] + nb[3] + 1024));
    S3Out<double> B{};
    if (e == cudaSuccess) {
        size_t o = 0;
        double** dst[4] = {&B.Vx, &B.Vy, &B.Vz, &B.Pt};
        for (int i = 0; i < 4; ++i) {
            *dst[i] = reinterpret_cast<double*>(bbase + o);
            o += (nb[i] + 255) / 256 * 256;
        }
        e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    }
    if (e == cudaSuccess) {
        s3_iterations<double, S3_PLAIN>(a, B, pp, nout, s, false);
        cudaMemsetAsync(red, 0, 4 * sizeof(double), s);
        s3_sum_abs_k<double><<<gr, 256, 0, s>>>(a.Rx, n[0], a.Ry, n[1], a.Rz, n[2], a.divV, n[3], red);
        e = cudaStreamEndCapture(s, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    int rc = e == cudaSuccess ? PS_OK : cuda_fail(e, "ps_stokes3d_solve: graph capture");
    const double t0 = now_s3();
    double err = INFINITY, h[4];
    int64_t it = 0;
    while (rc == PS_OK && it < max_iter) {
        e = cudaGraphLaunch(exec, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, red, sizeof(h), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "ps_stokes3d_solve");
            break;
        }
        it += nout;
        err = 0;
        bool finite = true;
        for (int k = 0; k < 4; k++) {
            finite = finite && std::isfinite(h[k]);
            err = std::max(err, h[k] / (double)n[k]);
        }
        if (!finite) {
            err = NAN;
            rc = fail(PS_ERR_NONFINITE, "ps_stokes3d_solve: non-finite residual after %lld iterations", (long long)it);
            break;
        }
        if (err < tol) break;
        if (max_seconds > 0 && now_s3() - t0 > max_seconds) {
            rc = fail(PS_ERR_TIMEOUT, "ps_stokes3d_solve: wall-clock limit reached (err %.3e)", err);
            break;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamSynchronize(s);
    if (bbase) cudaFree(bbase);
    cudaEventDestroy(ev);
    cudaStreamDestroy(s);
    cudaGetLastError();
    stats->iters = it;
    stats->outer = 1;
    stats->err = err;
    stats->seconds = now_s3() - t0;
    stats->converged = err < tol;
    if (rc == PS_OK && !(err < tol))
        rc = fail(PS_ERR_NOT_CONVERGED, "ps_stokes3d_solve: err %.3e after %lld iterations", err, (long long)it);
    return rc;
}

int ps_stokes3d_solve_mixed(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, double tol, int64_t max_iter,
                            int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream) {
    DeviceState* st = nullptr;
    PS_TRY(current_state(&st));
    PS_TRY(check_fields3(f, false));
    if (!p || !stats) return fail(PS_ERR_NULL, "NULL params / stats");
    if (f->Pt.dtype != PS_F64) return fail(PS_ERR_DTYPE, "ps_stokes3d_solve_mixed: the arrays must be FP64");
    if (nout < 1) return fail(PS_ERR_ARG, "nout must be >= 1");
    if (!(tol > 0) || max_iter < 0) return fail(PS_ERR_ARG, "invalid tol / max_iter");
    memset(stats, 0, sizeof(*stats));
    cudaStream_t user = static_cast<cudaStream_t>(stream), s;
    PS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t ev;
    PS_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(s, ev, 0);
    const int rc = solve_mixed3(f, p, tol, max_iter, nout, max_seconds, 1e-3, st->d_scratch, stats, s);
    cudaStreamSynchronize(s);
    cudaEventDestroy(ev);
    cudaStreamDestroy(s);
    return rc;
}

}  // extern "C"
