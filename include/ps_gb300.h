/*
 * ps_gb300.h -- C ABI of libps_b200.so, the GB300 (sm_103a) stencil library.
 *
 * The library replaces the kernel-launch layer that ParallelStencil.jl uses for its
 * `@parallel` / `@parallel_indices` finite-difference kernels on CUDA:
 *   - `@parallel k!(args...)` lowers to `CUDA.@cuda blocks threads stream k!(args..., ranges,
 *     rlx, rly, rlz)` followed by `CUDA.synchronize(stream)`
 *     (src/ParallelKernel/parallel.jl:303-334, 883-918, 375);
 *   - `@parallel_async` omits the synchronisation (src/ParallelKernel/parallel.jl:884).
 * Every entry point below takes the same arrays and scalars as the reference kernel it
 * replaces, plus a stream and a `sync` flag (1 = `@parallel`, 0 = `@parallel_async`).
 *
 * Conventions
 *   - Arrays are dense, column-major (x fastest), caller-owned device memory: element
 *     (ix,iy,iz) (0-based) lives at ptr[ix + n[0]*(iy + n[1]*iz)]. 2-D arrays use n[2] = 1,
 *     1-D arrays n[1] = n[2] = 1. This is `Data.Array` of the reference
 *     (src/ParallelKernel/Data.jl:271) with `padding=false`.
 *   - Every call returns a ps_status; nothing aborts, traps or throws across the ABI.
 *     ps_last_error() gives a thread-local message for the last failing call.
 *   - FP arithmetic is IEEE without FMA contraction, in the operation order of the
 *     reference's macros, so FP64 results are bit-identical to the reference's CPU path.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).
 */
#ifndef PS_GB300_H
#define PS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PS_ABI_VERSION 1

/* Status codes. The reference raises typed Julia exceptions for the same conditions
 * (src/ParallelKernel/Exceptions.jl:5-15); here they are return codes. */
typedef enum {
    PS_OK                = 0,
    PS_ERR_ARG           = -1,  /* invalid scalar argument / enum value          (ArgumentError) */
    PS_ERR_NULL          = -2,  /* NULL pointer where an array is required                        */
    PS_ERR_SHAPE         = -3,  /* incoherent array sizes                     (IncoherentArgumentError) */
    PS_ERR_DTYPE         = -4,  /* unsupported or mixed element types                              */
    PS_ERR_ALIGN         = -5,  /* misaligned device pointer                                       */
    PS_ERR_CUDA          = -6,  /* a CUDA runtime call failed (message in ps_last_error)           */
    PS_ERR_NOT_CONVERGED = -7,  /* iteration cap reached before the tolerance                      */
    PS_ERR_TIMEOUT       = -8,  /* a bounded device-side wait gave up                              */
    PS_ERR_NOT_INIT      = -9,  /* ps_init not called                        (NotInitializedError) */
    PS_ERR_NOMEM         = -10, /* device allocation failed                                        */
    PS_ERR_NONFINITE     = -11, /* NaN/Inf detected in a residual                                  */
    PS_ERR_UNSUPPORTED   = -12  /* valid request that this build does not implement               */
} ps_status;

/* Element types (the reference's `numbertype`, src/ParallelKernel/shared.jl:59). */
typedef enum { PS_F64 = 0, PS_F32 = 1, PS_BF16 = 2 } ps_dtype;

/* Array descriptor: a device pointer plus its extents (`size(A)`) and element type. */
typedef struct ps_array {
    void*   ptr;
    int64_t n[3];
    int32_t dtype;
    int32_t reserved;
} ps_array;

/* Launch configuration of one kernel call (the `@parallel` keyword arguments). */
typedef struct ps_launch {
    int32_t memopt;       /* 0: one thread per cell (`memopt=false`);
                             1: z-sweep with TMA-staged planes (`memopt=true`, loopdim z) */
    int32_t loopsize;     /* z-planes swept by one CTA (`loopsize`); 0 = library default:
                             chosen per launch from the number of CTA waves (the results do
                             not depend on it) */
    int64_t range_lo[3];  /* `ranges` of the call as 0-based half-open thread-index boxes  */
    int64_t range_hi[3];  /* (hi <= lo in every dimension, or a NULL ps_launch = full grid) */
    int32_t fp64_mode;    /* FP64 arrays only. PS_FP64_IEEE: IEEE double arithmetic on the FP64
                             pipe, bit-identical to the reference. PS_FP64_SPLIT: arithmetic on
                             pairs of FP32 numbers (47-bit significand) on the FP32/integer pipes,
                             <= 1e-12 relative max-norm from the reference (see ps_diffusion3d_step) */
    int32_t reserved;
} ps_launch;

/* PS_FP64_SPLIT_STATE (multi-step runs only, see ps_diffusion3d_run): as PS_FP64_SPLIT, but the
 * state between steps is kept as split pairs (8 bytes per value, as FP64) in library scratch and
 * converted from / to IEEE doubles at the start / end of the run.
 * PS_FP64_SPLIT_GRID (multi-step runs only): the state and lam are kept as pairs of floats on a
 * power-of-two grid fixed for the run from max|T| and max|lam| (an integer-valued high part of at
 * most 2^23 grid units plus a low part), which makes differences and conductivity sums exact in
 * one FP32 operation. Rounding <= 1.5 * 2^-47 of max|T| per step. If a value leaves the grid's
 * range (max|T| growing past its initial power of two), the run is redone in
 * PS_FP64_SPLIT_STATE by kernels enqueued behind it that run only when the grid run flagged
 * that, so the call stays asynchronous.
 * Single steps (ps_diffusion3d_step) treat both multi-step modes as PS_FP64_SPLIT. */
enum { PS_FP64_IEEE = 0, PS_FP64_SPLIT = 1, PS_FP64_SPLIT_STATE = 2, PS_FP64_SPLIT_GRID = 3 };

/* ------------------------------------------------------------------------------------ */
/* Core: device, memory, streams.                                                        */
/* ------------------------------------------------------------------------------------ */

/* Select and initialise a device (the `@init_parallel_stencil(GB300, ...)` hook,
 * src/init_parallel_stencil.jl:36-51). Idempotent per device. */
int ps_init(int device);
/* Release library-owned resources (streams, scratch, cached descriptors). */
int ps_finalize(void);
/* Message of the last failing call on this host thread ("" if none). */
const char* ps_last_error(void);
int ps_abi_version(void);
/* Number of CUDA devices visible (0 without a driver). Needs no ps_init. */
int ps_device_count(int* count);
/* Self-check of the kernels' division by a number known on the host (Markstein's method: one
 * multiply and four FMAs, correctly rounded) against the IEEE division a / b on the device.
 * PS_F32: every significand of 12 binades (from 2^-126 to 2^127) with both signs plus special
 * values; PS_F64: n dividends from a seeded hash plus special values. *mismatches = the number
 * of results whose bits differ (NaNs compare equal). Synchronises. */
int ps_check_division(double b, int32_t dtype, int64_t n, uint64_t seed, int64_t* mismatches, void* stream);

/* `@zeros(nx,ny,nz)` allocation (src/ParallelKernel/allocators.jl:279-293,
 * CUDAExt/allocators.jl:3): zero-filled device array owned by the caller. */
int ps_alloc(ps_array* a, int32_t dtype, int64_t nx, int64_t ny, int64_t nz);
int ps_free(ps_array* a);
/* `@fill!(A, v)` / `A .= v` on the device (src/ParallelKernel/allocators.jl:327-375). */
int ps_fill(ps_array a, double value, void* stream);
/* Host <-> device copies of a whole array (`Data.Array(host)` / `Array(A)`). */
int ps_copy_h2d(ps_array dst, const void* host_src, void* stream);
int ps_copy_d2h(void* host_dst, ps_array src, void* stream);
/* The same without waiting (stream-ordered; the host buffer must be page-locked for the copy to
 * overlap other work), and a device-to-device copy of two arrays of one shape and dtype. */
int ps_copy_h2d_async(ps_array dst, const void* host_src, void* stream);
int ps_copy_d2h_async(void* host_dst, ps_array src, void* stream);
int ps_copy_d2d_async(ps_array dst, ps_array src, void* stream);

/* Streams of the `@hide_communication` split (CUDAExt/shared.jl:17-31): priority 1 =
 * high-priority non-blocking stream (boundary slabs), 0 = normal non-blocking stream. */
int ps_stream_create(int priority, void** stream);
int ps_stream_destroy(void* stream);
/* `@synchronize(stream)` (src/ParallelKernel/parallel.jl:175-184). */
int ps_synchronize(void* stream);

/* ------------------------------------------------------------------------------------ */
/* Finite-difference operators (src/FiniteDifferences.jl).                               */
/* ------------------------------------------------------------------------------------ */

/* Operator kinds of the FiniteDifferences{1,2,3}D macros. */
typedef enum {
    PS_FD_SEL    = 0, /* @all, @inn, @inn_x ... @inn_yz                                  */
    PS_FD_DIFF   = 1, /* @d_xa/@d_ya/@d_za, @d_xi/@d_yi/@d_zi (1-D: @d)                  */
    PS_FD_DIFF2  = 2, /* @d2_xa/@d2_ya (2-D), @d2_xi/@d2_yi/@d2_zi (1-D: @d2)            */
    PS_FD_AV     = 3, /* @av, @av_xa ... @av_yzi                                         */
    PS_FD_HARM   = 4, /* @harm, @harm_xa ... @harm_yzi                                   */
    PS_FD_MAXLOC = 5, /* @maxloc                                                         */
    PS_FD_MINLOC = 6  /* @minloc                                                         */
} ps_fd_kind;

/* One FD macro as a descriptor. Bit d of a mask refers to dimension d (x=1, y=2, z=4).
 *   opdims: dimensions the operator differences / averages over
 *   inn:    dimensions whose base index is the inner index (ixi = ix+1)
 * Examples (3-D): @d_xi = {DIFF, x, y|z}; @d2_yi = {DIFF2, y, x|y|z}; @av_xyi = {AV, x|y, z};
 * @inn_xz = {SEL, 0, x|z}; @maxloc = {MAXLOC, x|y|z, x|y|z}. */
typedef struct ps_fd_op {
    int32_t kind;
    int32_t opdims;
    int32_t inn;
    int32_t ndims;   /* 1, 2 or 3: the FiniteDifferences module the macro comes from */
} ps_fd_op;

/* `@<lhs>(R) = @<op>(A)` as a one-statement `@parallel` kernel: thread grid = max extents of
 * R and A (src/ParallelKernel/parallel.jl:795-798), statement masked by `@within` of the
 * left-hand selection (src/FiniteDifferences.jl:397-408; src/parallel.jl:654-680).
 * lhs_inn is the inn-mask of the left-hand macro (@all = 0, @inn = all dims, @inn_x = x ...).
 * Returns PS_ERR_SHAPE if a thread passing the mask would read outside A. */
int ps_fd_apply(ps_fd_op op, int32_t lhs_inn, ps_array R, ps_array A, void* stream, int sync);

/* ------------------------------------------------------------------------------------ */
/* 3-D kernels of the examples (examples/memcopy3D.jl, examples/diffusion3D_*.jl).       */
/* ------------------------------------------------------------------------------------ */

/* `@all(T2) = @all(T) + @all(Ci)` (examples/memcopy3D.jl:10-13;
 * `@parallel_indices` form examples/memcopy3D_parindices.jl:9-12). */
int ps_memcopy3d(ps_array T2, ps_array T, ps_array Ci, const ps_launch* cfg, void* stream, int sync);

/* Statement forms of the 3-D diffusion step. */
typedef enum {
    /* @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)/dx^2 + @d2_yi(T)/dy^2 + @d2_zi(T)/dz^2))
     * examples/diffusion3D_novis_noperf.jl:10-13; h = (dx, dy, dz) */
    PS_DIFF_DIV      = 0,
    /* @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))
     * examples/diffusion3D_multigpucpu_hidecomm_novis.jl:12-15; h = (_dx, _dy, _dz) */
    PS_DIFF_MUL      = 1,
    /* on-the-fly flux form with scalar lam (test/test_parallel.jl:420-426):
     *   @all(qx) = -lam*@d_xi(T)*_dx ... ;
     *   @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz);
     *   @inn(T2) = @inn(T) + dt*@all(dTdt)                        h = (_dx, _dy, _dz) */
    PS_DIFF_FLUX     = 2,
    /* the same flux form with a conductivity array and face values @av_xi(lam) etc.:
     *   @all(qx) = -@av_xi(lam)*@d_xi(T)*_dx ...                  h = (_dx, _dy, _dz) */
    PS_DIFF_FLUX_LAM = 3
} ps_diffusion_form;

/* One diffusion step `@parallel diffusion3D_step!(T2, T, Ci, lam, dt, h...)`. All arrays
 * n^3 of one dtype; lam_arr is used (and must be non-NULL) only for PS_DIFF_FLUX_LAM.
 * Scalars are cast to the array dtype first, as the reference's literal typing does
 * (src/ParallelKernel/parallel.jl:400-418). Boundary cells of T2 are not written. */
int ps_diffusion3d_step(int32_t form, ps_array T2, ps_array T, ps_array Ci, ps_array lam_arr,
                        double lam, double dt, double hx, double hy, double hz,
                        const ps_launch* cfg, void* stream, int sync);

/* The time loop of the examples, `for it = 1:nt; @parallel diffusion3D_step!(T2, T, ...);
 * T, T2 = T2, T; end` (examples/diffusion3D_novis_noperf.jl:43-46), as one call. On return T
 * holds the state after nt steps (the boundary values of T and T2 must agree, as in the
 * examples' `T2 .= T`); T2's interior is workspace. cfg->memopt and cfg->fp64_mode apply; with
 * PS_FP64_SPLIT / PS_FP64_SPLIT_STATE the static arrays lam and Ci are split once per call into
 * library scratch (grow-only, one per device and stream, freed by ps_finalize), so each step
 * converts only T (SPLIT) or nothing (SPLIT_STATE). Asynchronous on `stream` in every mode; runs
 * on different streams may overlap on the GPU. */
int ps_diffusion3d_run(int32_t form, ps_array T, ps_array T2, ps_array Ci, ps_array lam_arr, double lam, double dt,
                       double hx, double hy, double hz, int64_t nt, const ps_launch* cfg, void* stream);

/* Host callback run by the split launcher once the boundary slabs are complete: the
 * communication / boundary-condition slot of `@hide_communication`. */
typedef int (*ps_comm_fn)(void* ctx);

/* `@hide_communication bw begin @parallel diffusion3D_step!(...); comm(ctx) end`
 * (src/ParallelKernel/hide_communication.jl:177-258, ranges :350-394): the six boundary
 * slabs of width bw run on s_boundary, the inner box on s_inner; comm (may be NULL) runs
 * after the boundary slabs finish and before the inner box is waited for. On return both
 * streams are synchronised. cfg supplies memopt and fp64_mode (its ranges are ignored).
 * With memopt the x and y slabs are widened to whole z-sweep tiles when the grid allows it
 * (x: 64 cells for FP64 / 128 for FP32 from an even cell, y: 8 rows), so the boundary phase
 * computes a superset of the bw-wide boundary. Result identical to ps_diffusion3d_step. */
int ps_diffusion3d_step_split(int32_t form, ps_array T2, ps_array T, ps_array Ci, ps_array lam_arr,
                              double lam, double dt, double hx, double hy, double hz,
                              const ps_launch* cfg, const int64_t bw[3], void* s_boundary, void* s_inner,
                              ps_comm_fn comm, void* comm_ctx);

/* ------------------------------------------------------------------------------------ */
/* Adjoint of the diffusion step (replaces `@parallel ∇=(T->T̄, lam->lam̄) step!(...)`,     */
/* src/ParallelKernel/parallel.jl:265-301, for PS_DIFF_FLUX_LAM).                         */
/* ------------------------------------------------------------------------------------ */

/* One reverse step of T2 = step(T, lam) (PS_DIFF_FLUX_LAM with h = (_dx, _dy, _dz)):
 * lamT = (∂T2/∂T)^T lamT2 on inner cells (0 on boundary cells, whose values are constants) and
 * glam += (∂T2/∂lam)^T lamT2. T is the step's input state. All arrays n^3, one dtype. */
int ps_diffusion3d_adjoint_step(ps_array lamT, ps_array lamT2, ps_array T, ps_array Ci, ps_array lam, ps_array glam,
                                double dt, double hx, double hy, double hz, void* stream, int sync);
/* The same with fp64_mode (ps_launch.fp64_mode values): PS_FP64_IEEE is the function above; any
 * split mode evaluates the reverse step on FP32 pairs (FP64 arrays only; within ~1e-13 relative of
 * the IEEE step). ps_diffusion3d_misfit_gradient uses this form with its cfg's fp64_mode. */
int ps_diffusion3d_adjoint_step_ex(ps_array lamT, ps_array lamT2, ps_array T, ps_array Ci, ps_array lam,
                                   ps_array glam, double dt, double hx, double hy, double hz, int32_t fp64_mode,
                                   void* stream, int sync);

typedef struct ps_adjoint_stats {
    double loss;               /* 0.5 * ||T_nt - T_obs||^2                  */
    int64_t checkpoints;       /* forward states kept (one every ce steps)  */
    int64_t recomputed_steps;  /* forward steps recomputed in the reverse sweep */
    double seconds;
} ps_adjoint_stats;

/* Gradient of L(lam) = 0.5 ||T_nt - T_obs||^2, T_nt = nt diffusion steps (PS_DIFF_FLUX_LAM) from
 * T0, by the adjoint with a checkpoint every `checkpoint_every` steps and recomputation of each
 * segment. cfg selects memopt / fp64_mode of the forward steps (NULL: memopt, IEEE). FP64 arrays.
 * dL_dlam is overwritten; T_final (ptr may be NULL) receives T_nt. Synchronises. */
int ps_diffusion3d_misfit_gradient(ps_array T0, ps_array T_obs, ps_array Ci, ps_array lam, double dt, double hx,
                                   double hy, double hz, int64_t nt, int64_t checkpoint_every, const ps_launch* cfg,
                                   ps_array dL_dlam, ps_array T_final, ps_adjoint_stats* stats, void* stream);

/* ------------------------------------------------------------------------------------ */
/* acoustic3D (miniapps/acoustic3D.jl:11-21).                                            */
/* ------------------------------------------------------------------------------------ */

/* `@inn(Vx) = @inn(Vx) - dt/ρ*@d_xi(P)/dx` etc. Vx (n+1,n,n), Vy (n,n+1,n), Vz (n,n,n+1). */
int ps_acoustic3d_v(ps_array Vx, ps_array Vy, ps_array Vz, ps_array P,
                    double dt, double rho, double dx, double dy, double dz, void* stream, int sync);
/* `@all(P) = @all(P) - dt*k*(@d_xa(Vx)/dx + @d_ya(Vy)/dy + @d_za(Vz)/dz)`. */
int ps_acoustic3d_p(ps_array P, ps_array Vx, ps_array Vy, ps_array Vz,
                    double dt, double k, double dx, double dy, double dz, void* stream, int sync);
/* One time step of the miniapp's loop (acoustic3D.jl:55-56: compute_V! then compute_P!) as one
 * kernel that reads (Vx, Vy, Vz, P) and writes the new state into (Vx2, Vy2, Vz2, P2): every value,
 * faces outside @inn copied. 8 words per cell instead of the 12 of the two launches. The output
 * arrays must not overlap each other or the inputs (PS_ERR_ARG). fp64_mode: PS_FP64_IEEE
 * (bit-identical to ps_acoustic3d_v + ps_acoustic3d_p; FP32 arrays take only this) or
 * PS_FP64_SPLIT (FP64 arrays, arithmetic on FP32 pairs, ~2^-46 relative rounding per step). */
int ps_acoustic3d_step(ps_array Vx, ps_array Vy, ps_array Vz, ps_array P,
                       ps_array Vx2, ps_array Vy2, ps_array Vz2, ps_array P2,
                       double dt, double rho, double k, double dx, double dy, double dz,
                       int32_t fp64_mode, void* stream, int sync);
/* nt steps of the miniapp's time loop on (Vx, Vy, Vz, P) in place: ps_acoustic3d_step alternating
 * between the caller's arrays and a second set in library scratch (grow-only, one per device and
 * stream, freed by ps_finalize); odd nt ends with a copy back. IEEE FP64 (FP64-pipe bound, where
 * the two kernels are faster) runs ps_acoustic3d_v / _p in place. Asynchronous on `stream`. */
int ps_acoustic3d_run(ps_array Vx, ps_array Vy, ps_array Vz, ps_array P,
                      double dt, double rho, double k, double dx, double dy, double dz,
                      int64_t nt, int32_t fp64_mode, void* stream);

/* ------------------------------------------------------------------------------------ */
/* Stokes2D pseudo-transient solver (miniapps/Stokes2D.jl).                              */
/* ------------------------------------------------------------------------------------ */

/* The arrays of the miniapp (Stokes2D.jl:79-101), nx = size(Pt,1), ny = size(Pt,2):
 * Pt, dtauPt, divV (∇V), txx, tyy, Mus, Rog: (nx, ny); Vx: (nx+1, ny); Vy: (nx, ny+1);
 * txy: (nx-1, ny-1); Rx, dVxdtau, dtauVx: (nx-1, ny-2); Ry, dVydtau, dtauVy: (nx-2, ny-1).
 * All 2-D (n[2] = 1), one dtype. */
typedef struct ps_stokes2d_fields {
    ps_array Pt, dtauPt, divV, Vx, Vy, txx, tyy, txy, Rx, Ry, dVxdtau, dVydtau, dtauVx, dtauVy, Mus, Rog;
} ps_stokes2d_fields;

/* Scalars of the kernels (Stokes2D.jl:73-77): dx, dy, dampX = 1-Vdmp/nx, dampY = 1-Vdmp/ny,
 * Vsc, Ptsc, min_dxy2 = min(dx,dy)^2, max_nxy = max(nx,ny). */
typedef struct ps_stokes2d_params {
    double dx, dy, dampX, dampY, Vsc, Ptsc, min_dxy2;
    int64_t max_nxy;
} ps_stokes2d_params;

typedef struct ps_solve_stats {
    int64_t iters;     /* pseudo-transient iterations executed (all precisions)          */
    int64_t outer;     /* defect-correction outer iterations (1 for the plain FP64 solve) */
    double err;        /* final max(mean|Rx|, mean|Ry|, mean|∇V|), evaluated in FP64      */
    double seconds;    /* wall time of the solve                                          */
    int32_t converged; /* err < tol                                                       */
    int32_t reserved;
} ps_solve_stats;

/* The six `@parallel` calls of the PT loop, one-to-one (Stokes2D.jl:11-55). */
int ps_stokes2d_timesteps(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync);
int ps_stokes2d_compute_P(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync);
int ps_stokes2d_compute_tau(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync);
int ps_stokes2d_compute_dV(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync);
int ps_stokes2d_compute_V(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, void* stream, int sync);
/* `bc_x!(A)`: A[1,:] = A[2,:], A[end,:] = A[end-1,:]; `bc_y!(A)` the same along y (2-D). */
int ps_bc_x2d(ps_array A, void* stream, int sync);
int ps_bc_y2d(ps_array A, void* stream, int sync);

/* n_iter iterations of the PT loop body (compute_P!, compute_τ!, compute_dV!, compute_V!,
 * bc_y!(Vx), bc_x!(Vy); Stokes2D.jl:111-116) with one fused kernel per iteration. Every array,
 * temporaries included, ends bit-identical to the six-call sequence. Synchronises. */
int ps_stokes2d_iterate(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, int64_t n_iter, void* stream);

/* ps_stokes2d_iterate without any device allocation. This entry point has no counterpart in the
 * reference: it exists for callers that cannot let a library allocate device memory, e.g. a host
 * whose device memory is owned by its own pool allocator (a cudaMalloc behind the pool's back can
 * fail or fragment it) or a code path that must not call cudaFree (it synchronises the device).
 * The three ping-pong buffers of the fused iteration come from a file-scope device array of
 * 16 MiB compiled into the library (present on every device that loads it, until exit), so
 * ((nx+1)*ny + nx*(ny+1) + nx*ny) * sizeof(T), each term rounded up to 256 bytes, must not exceed
 * 16 MiB (about 830 x 830 cells in FP64); larger grids return PS_ERR_SHAPE. The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress, with that device current),
 * so make that first call before any stream capture. The address is cached until ps_finalize,
 * which forgets it: a caller that resets the device (cudaDeviceReset) calls ps_finalize first, and
 * the next call looks the address up again. All calls share the one array and it keeps
 * the last call's contents (every element a call reads is written by that call first): calls that
 * overlap on the GPU (concurrent streams, several host threads) race. Allocates nothing; results
 * are bit-identical to ps_stokes2d_iterate. Synchronises. */
int ps_stokes2d_iterate_static(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, int64_t n_iter, void* stream);

/* mean(abs.(Rx)), mean(abs.(Ry)), mean(abs.(∇V)) of the stored arrays (Stokes2D.jl:119). */
int ps_stokes2d_err(const ps_stokes2d_fields* f, double out_mean_abs[3], void* stream);

/* PT solve from the current state until err = max(mean|Rx|, mean|Ry|, mean|∇V|) < tol
 * (the miniapp's `while err > ε` loop, checked every `nout` iterations; nout even).
 *   mode 0: FP64 PT iterations.
 *   mode 1: FP32 PT iterations on the correction (δP, δV) driven by the FP64 residual of the
 *           state (defect correction); the residual, the state update and the convergence check
 *           are FP64.
 * The state arrays must be FP64. dtau arrays are recomputed from Mus with the compute_timesteps!
 * formulas. Returns PS_ERR_NOT_CONVERGED at max_iter, PS_ERR_TIMEOUT after max_seconds (> 0),
 * PS_ERR_NONFINITE on NaN/Inf residuals. Only Pt, Vx, Vy, dVxdtau, dVydtau are updated. */
int ps_stokes2d_solve(const ps_stokes2d_fields* f, const ps_stokes2d_params* p, int32_t mode, double tol,
                      int64_t max_iter, int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream);

/* Stokes2D with an accelerated pseudo-transient (APT) iteration whose pseudo-time steps come from
 * the local viscosity maximum Musτ = @maxloc(Mus) -- the reference's idiom for heterogeneous
 * coefficients (miniapps/HydroMech2D.jl:27). The miniapp's damped iteration (above) diverges at a
 * viscosity contrast of 1e-3; this one keeps its arrays and statements (∇V, P, τ, R, V, the
 * free-slip copies) but relaxes the stresses in pseudo-time (τ is state):
 *   ∇V = @d_xa(Vx)*_dx + @d_ya(Vy)*_dy;  Pt = Pt - kP*∇V
 *   τxx = aτ*τxx + bτ*(@d_xa(Vx)*_dx - ∇V/3);  τyy likewise;  τxy = aτc*τxy + bτc*ε̇xy
 *   Rx, Ry as in Stokes2D.jl:33-34 (times _dx, _dy);  V = V + dτV*R;  bc_y!(Vx), bc_x!(Vy)
 * with dτρ = Vpdt*max_lxy/Re/Musτ, Gdτ = Vpdt^2/dτρ/(r+2), kP = r*Gdτ, aτ = 1/(Gdτ/Mus+1),
 * bτ = 2*Gdτ*aτ (cells); corners: the smallest Gdτ of the four cells, μ = @av(Mus); faces:
 * dτV = the smaller dτρ of the two cells. Arrays: the miniapp's (shapes as ps_stokes2d_fields)
 * plus Must, kP, aT, bT: (nx, ny); aTc, bTc: (nx-1, ny-1); dtVx: (nx-1, ny-2); dtVy: (nx-2, ny-1).
 * No counterpart kernel exists in the reference; its oracle is the C restatement of these
 * statements. */
typedef struct ps_stokes2d_apt_fields {
    ps_array Pt, divV, Vx, Vy, txx, tyy, txy, Rx, Ry, Mus, Rog;
    ps_array Must, kP, aT, bT, aTc, bTc, dtVx, dtVy;
} ps_stokes2d_apt_fields;

/* dx, dy; Vpdt = CFL*min(dx,dy) (CFL = 0.9/sqrt(2)); Re (16π); r (1); max_lxy = max(lx, ly). */
typedef struct ps_stokes2d_apt_params {
    double dx, dy, Vpdt, Re, r, max_lxy;
} ps_stokes2d_apt_params;

/* Musτ and the coefficient arrays from Mus (FP64 arithmetic; FP32 arrays hold the rounded values). */
int ps_stokes2d_apt_coefficients(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, void* stream,
                                 int sync);
/* n_iter APT iterations in place (two kernels each); divV, Rx, Ry hold the last iteration's
 * values. Bit-identical to the oracle's statements. Synchronises. */
int ps_stokes2d_apt_iterate(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, int64_t n_iter,
                            void* stream);
/* FP64 residual of the state (Vx, Vy, Pt) with the stresses at their pseudo-time steady state
 * τ = 2μ(ε̇ - ∇V/3): writes txx, tyy, txy, divV, Rx, Ry and returns mean|Rx|, mean|Ry|, mean|∇V|.
 * FP64 fields only. Synchronises. */
int ps_stokes2d_apt_residual(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, double out_mean_abs[3],
                             void* stream);
/* APT solve from the current state (coefficients recomputed from Mus) until the FP64 residual
 * err = max(mean|Rx|, mean|Ry|, mean|∇V|) < tol, checked every nout iterations.
 *   mode 0: FP64 APT iterations (the stresses are state).
 *   mode 1: FP32 APT sweeps on the correction (δV, δP, δτ) driven by the FP64 residual of the
 *           state (defect correction); residual, update and convergence check in FP64.
 * FP64 fields. On return divV, Rx, Ry hold the FP64 residual of the final state (mode 1 also
 * writes its steady-state stresses into txx, tyy, txy). Returns PS_ERR_NOT_CONVERGED at max_iter,
 * PS_ERR_TIMEOUT after max_seconds (> 0), PS_ERR_NONFINITE on NaN/Inf residuals. */
int ps_stokes2d_apt_solve(const ps_stokes2d_apt_fields* f, const ps_stokes2d_apt_params* p, int32_t mode, double tol,
                          int64_t max_iter, int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream);

/* ------------------------------------------------------------------------------------ */
/* Stokes3D miniapp (miniapps/Stokes3D.jl): the PT kernels of the 3-D analogue.          */
/* ------------------------------------------------------------------------------------ */

/* The miniapp's arrays (Stokes3D.jl:89-110), all of one dtype, (nx, ny, nz) = size(Pt):
 * Pt, dtauPt, divV, Mus, Rog (nx,ny,nz); Vx (nx+1,ny,nz), Vy (nx,ny+1,nz), Vz (nx,ny,nz+1);
 * txx (nx,ny-2,nz-2), tyy (nx-2,ny,nz-2), tzz (nx-2,ny-2,nz); txy (nx-1,ny-1,nz-2),
 * txz (nx-1,ny-2,nz-1), tyz (nx-2,ny-1,nz-1); Rx, dVxdtau, dtauVx (nx-1,ny-2,nz-2);
 * Ry, dVydtau, dtauVy (nx-2,ny-1,nz-2); Rz, dVzdtau, dtauVz (nx-2,ny-2,nz-1). */
typedef struct ps_stokes3d_fields {
    ps_array Pt, dtauPt, divV, Vx, Vy, Vz, txx, tyy, tzz, txy, txz, tyz, Rx, Ry, Rz, dVxdtau, dVydtau, dVzdtau,
        dtauVx, dtauVy, dtauVz, Mus, Rog;
} ps_stokes3d_fields;

/* Scalars of Stokes3D.jl:72-88: dx, dy, dz, dampX = 1-Vdmp/nx, dampY, dampZ, Vsc, Ptsc,
 * min_dxyz2 = min(dx,dy,dz)^2, max_nxyz = max(nx,ny,nz). */
typedef struct ps_stokes3d_params {
    double dx, dy, dz, dampX, dampY, dampZ, Vsc, Ptsc, min_dxyz2;
    int64_t max_nxyz;
} ps_stokes3d_params;

/* The `@parallel` kernels one-to-one (Stokes3D.jl:11-50), bit-identical to the reference
 * (FP64 and FP32 arrays). */
int ps_stokes3d_timesteps(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync);
int ps_stokes3d_compute_P(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync);
int ps_stokes3d_compute_tau(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync);
int ps_stokes3d_compute_dV(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync);
int ps_stokes3d_compute_V(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, void* stream, int sync);
/* `@parallel_indices` free-slip copies bc_x! / bc_y! / bc_z! (Stokes3D.jl:52-68) of a 3-D array. */
int ps_bc_x3d(ps_array A, void* stream, int sync);
int ps_bc_y3d(ps_array A, void* stream, int sync);
int ps_bc_z3d(ps_array A, void* stream, int sync);

/* n_iter iterations of the loop body (Stokes3D.jl:134-143: compute_P!, compute_τ!, compute_dV!,
 * compute_V!, six bc calls) in three launches each, bit-identical to the reference's sequence.
 * Synchronises. */
int ps_stokes3d_iterate(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, int64_t n_iter, void* stream);
/* The same with a choice of schedule. one_launch = 0: three kernels per iteration (compute_P! +
 * compute_τ!, compute_dV! + compute_V!, the six free-slip copies), every array stored each
 * iteration. one_launch = 1: pairs of single-kernel iterations (the state through a second set in
 * library scratch, grow-only, one per device and stream; ∇V, τ and R kept on chip), then the storing
 * kernels for the last one or two iterations; every array ends bit-identical to one_launch = 0. */
int ps_stokes3d_iterate_ex(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, int64_t n_iter,
                           int32_t one_launch, void* stream);

/* mean(abs.(Rx)), mean(abs.(Ry)), mean(abs.(Rz)), mean(abs.(∇V)) of the stored arrays
 * (Stokes3D.jl:145-146), accumulated in FP64. */
int ps_stokes3d_err(const ps_stokes3d_fields* f, double out_mean_abs[4], void* stream);

/* The `while err > ε && iter <= iterMax` loop (Stokes3D.jl:131-149) in FP64: CUDA graphs of nout
 * iterations, the error checked after each. The dtau arrays must have been computed
 * (ps_stokes3d_timesteps). Returns PS_ERR_NOT_CONVERGED at max_iter, PS_ERR_TIMEOUT after
 * max_seconds (> 0), PS_ERR_NONFINITE on NaN/Inf residuals. */
int ps_stokes3d_solve(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, double tol, int64_t max_iter,
                      int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream);
/* The same solve in mixed precision (no counterpart in the reference; the Stokes3D form of
 * ps_stokes2d_solve mode 1): FP32 PT sweeps on a correction with the FP64 residual of the state as
 * source, FP64 residual (the reference's statements), FP64 update and convergence check with the
 * reference's err. Uses library-owned FP32 scratch (26 arrays of the grid's size); stats->outer
 * counts the FP64 corrections, stats->iters the FP32 sweeps. On return Rx, Ry, Rz, divV and the
 * stresses hold the FP64 residual of the returned state. */
int ps_stokes3d_solve_mixed(const ps_stokes3d_fields* f, const ps_stokes3d_params* p, double tol, int64_t max_iter,
                            int64_t nout, double max_seconds, ps_solve_stats* stats, void* stream);

/* ------------------------------------------------------------------------------------ */
/* Run-time compiled kernels: any `@parallel` body of FiniteDifferences macros, or a       */
/* `@parallel_indices` body, beyond the fixed set above (src/parallel.jl:192-277 parses    */
/* them; src/ParallelKernel/parallel.jl:303-315 launches them).                           */
/* ------------------------------------------------------------------------------------ */

/* Compile CUDA C `source` (as generated by ps_gb300/jit.py) with NVRTC for sm_103a, without FMA
 * contraction, and load it on the current device. `entry` is the extern "C" kernel, which takes
 * one argument block by value:
 *   struct { void* a[32]; long long n[32][3]; double s[32]; long long lo[3]; long long cnt[3]; int* err;
 *            long long smem; long long loop; unsigned* ocnt; int ord[10]; }
 * (array pointers and extents, scalars, first thread index and thread counts per dimension, the
 * kernel's error flags -- one device int owned by the handle --, the launch's dynamic shared
 * memory bytes, the indices per thread of a sweep kernel, and the block order of a boundary-first
 * launch: a host-mapped counter, NULL otherwise, and blocks per axis, boundary blocks at the low and
 * high end of each axis and their count).
 * Compile errors return PS_ERR_ARG with the compiler log in ps_last_error(). */
int ps_jit_compile(const char* source, const char* entry, void** kernel);
/* Launch a compiled kernel over count[0] x count[1] x count[2] threads starting at thread index
 * lo (0-based), blocks of 32 x 8 x 1, with the given arrays (one dtype) and scalars. With sync,
 * a set out-of-bounds flag (from this or an earlier asynchronous launch of the same handle) is
 * cleared and returned as PS_ERR_ARG, the counterpart of Julia's BoundsError. */
int ps_jit_launch(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                  const int64_t lo[3], const int64_t count[3], void* stream, int sync);
/* The same with explicit thread-block dimensions and dynamic shared memory bytes (up to 227 KB):
 * `@parallel nblocks nthreads shmem=... kernel!(...)` (src/ParallelKernel/parallel.jl:303-328,
 * 883-898). Kernels that use @sync_threads, warp shuffles or votes need count[d] to be a multiple of
 * threads[d]; a partial block leaves before its first barrier and the launch returns PS_ERR_ARG.
 * loop (NULL: 1, 1, 1) gives the indices per thread along each dimension: a sweep kernel (memopt,
 * generated for it) has loop[d] > 1 in its sweep dimension d (z in 3-D, y in 2-D; src/memopt.jl's
 * loopdim), with threads[d] == 1 there, and each thread covers loop[d] consecutive indices; every
 * other kernel takes 1, 1, 1. */
int ps_jit_launch_ex(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                     const int64_t lo[3], const int64_t count[3], const int32_t threads[3], int64_t shmem,
                     const int32_t loop[3], void* stream, int sync);
/* The memopt z-sweep of a run-time compiled 3-D `@parallel` kernel with its read-only stencil
 * arrays staged plane by plane in shared memory by TMA (src/memopt.jl:190-573 caches the same
 * arrays in registers and shared memory; launched by src/parallel.jl:451-596). The kernel must be
 * the TMA variant ps_gb300/jit.py generates for the definition; its argument block is
 *   struct alignas(64) { CUtensorMap tm[8]; <the ps_jit_compile block> }
 * with tm[i] a 3-D tiled map of arrays[maps[3i]] with box (maps[3i+1], maps[3i+2], 1), zero fill,
 * built here for each launch. The threads start at index 0 (no ranges); loop_z z indices per
 * thread (threads[2] == 1); shmem = the kernel's stage ring. Every staged array must meet TMA's
 * 16-byte rules (base address, x extent x element size and x-y plane size multiples of 16 bytes:
 * PS_ERR_ALIGN otherwise). A bounded wait for a staged plane that gives up stops the kernel and is
 * reported as PS_ERR_TIMEOUT, otherwise as ps_jit_launch_ex. */
int ps_jit_launch_tma(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars, int32_t nscalars,
                      const int64_t count[3], const int32_t threads[3], int64_t shmem, int32_t loop_z,
                      const int32_t* maps, int32_t nmaps, void* stream, int sync);
/* `@hide_communication bw begin @parallel kernel!(...); comm() end` for a run-time compiled
 * `@parallel` kernel over its full grid (count threads from index 0; threads and loop as for
 * ps_jit_launch_ex, at most 256 threads per block; no dynamic shared memory, no barriers, shuffles
 * or votes). One launch on
 * `stream` whose first blocks take the tiles holding the boundary indices t < bw or t >= count - bw
 * (the reference's ranges_outer, src/ParallelKernel/hide_communication.jl:350-394); each such block
 * counts itself in host-mapped memory after its stores, and `comm` runs on this thread as soon as
 * all have, while the inner blocks still run. The kernel must be the boundary-first
 * variant of the definition (ps_gb300/jit.py generates it with the order decode and the count). Returns after the launch completes, with the
 * kernel's flags reported as by a synchronous launch. */
int ps_jit_hide_communication(void* kernel, const ps_array* arrays, int32_t narrays, const double* scalars,
                              int32_t nscalars, const int64_t count[3], const int32_t threads[3], const int32_t loop[3],
                              const int64_t bw[3], ps_comm_fn comm, void* comm_ctx, void* stream);
/* Wait for `stream`, then report (and clear) the error flags left by earlier asynchronous launches
 * of `kernel`, as a synchronous launch does. */
int ps_jit_check(void* kernel, void* stream);
int ps_jit_destroy(void* kernel);

/* ------------------------------------------------------------------------------------ */
/* Learned warm start (no counterpart in the reference): BF16 conv encoder-decoder on the */
/* tcgen05 tensor cores, trained and run by the library's own kernels.                    */
/* ------------------------------------------------------------------------------------ */

enum { PS_NN_RELU = 1, PS_NN_OUT_BF16 = 2, PS_NN_ACCUMULATE = 4 };

/* C[M][N] = A[M][K] * B[N][K]^T for row-major bf16 device matrices A, B (K % 8 == 0, 16-byte
 * aligned), FP32 accumulation in tensor memory; then + bias[n] (bias may be NULL), ReLU
 * (PS_NN_RELU), and C stored as bf16 (PS_NN_OUT_BF16), added into FP32 C with atomics
 * (PS_NN_ACCUMULATE; required for split > 1, K split over `split` CTAs per tile), or stored as
 * FP32. Synchronises. */
int ps_nn_gemm_bf16(const void* A, const void* B, void* C, int64_t M, int64_t N, int64_t K, const float* bias,
                    int32_t flags, int32_t split, void* stream);

/* The warm-start network: a 4-level conv encoder-decoder (3x3 convs, ReLU, 4x4 average pooling,
 * nearest x4 upsampling with skip concatenation; 32, 64, 128, 256 channels; 1x1 output conv),
 * input [B][H][W][2] (log10 viscosity, rho*g; normalised with the net's scales), output
 * [B][H][W][3] (P, Vx, Vy at cells, normalised). Activations and weights bf16, accumulation FP32;
 * FP32 master weights with Adam. H, W multiples of 64; B <= max_batch. All pointers are device
 * memory unless named host. Every call synchronises. */
int ps_nn_create(int64_t H, int64_t W, int32_t max_batch, uint64_t seed, void** net);
int ps_nn_destroy(void* net);
int ps_nn_forward(void* net, const float* x, int32_t B, float* y, void* stream);
/* Gradient of the last forward pass for output gradient dy [B][H][W][3], added to the
 * parameters' gradients (ps_nn_zero_grad clears them). */
int ps_nn_backward(void* net, const float* dy, void* stream);
int ps_nn_zero_grad(void* net, void* stream);
int ps_nn_adam_step(void* net, float lr, float beta1, float beta2, float eps, void* stream);
/* forward + mean squared error against t [B][H][W][3] (per-pixel weights w [B][H][W] or NULL,
 * loss = sum w (y - t)^2 / (3 B H W), written to host *loss) + backward + Adam (0.9, 0.999, 1e-8). */
int ps_nn_train_step(void* net, const float* x, const float* t, const float* w, int32_t B, float lr, double* loss,
                     void* stream);
/* Output of layer 0..14 of the last forward pass, [B][h][w][cout] as host FP32 (hidden layers
 * are stored as bf16; layer 14 is the network output). */
int ps_nn_get_activation(void* net, int32_t layer, float* host);
/* Parameters (host FP32), layer by layer: W [cout][ky][kx][cin] then b [cout]. */
int ps_nn_param_count(void* net, int64_t* count);
int ps_nn_get_params(void* net, float* host);
int ps_nn_set_params(void* net, const float* host);
int ps_nn_get_grads(void* net, float* host);
/* scales: input offsets/scales (log10 mu: [0], [1]; rho*g: [2], [3]), output scales P, Vx, Vy
 * ([4..6]); [7] unused. Stored with the weights. */
int ps_nn_set_scales(void* net, const float scales[8]);
int ps_nn_get_scales(void* net, float scales[8]);
int ps_nn_save(void* net, const char* path);
int ps_nn_load(void* net, const char* path);

/* Warm start of the Stokes2D PT solve: the network's P, Vx, Vy for the viscosity and buoyancy
 * of f, predicted on the network's nvalid x nvalid node grid (the fields resampled bilinearly
 * onto it) and interpolated onto f's staggered arrays; the wall-normal faces (Vx at x walls, Vy
 * at y walls), which the PT iteration keeps fixed, are set to 0, the free-slip copies bc_y!(Vx),
 * bc_x!(Vy) are applied; dVxdtau, dVydtau zeroed. FP64 fields. */
int ps_stokes2d_warm_start(void* net, const ps_stokes2d_fields* f, int32_t nvalid, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PS_GB300_H */
