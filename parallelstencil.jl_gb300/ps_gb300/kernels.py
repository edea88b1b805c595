"""The recognised `@parallel` kernels and the `parallel` / `hide_communication` launchers.

``parallel(kernel, *args, memopt=..., ranges=..., stream=..., sync=True)`` mirrors
``@parallel [ranges] [memopt=...] [stream=...] kernel!(args...)``
(src/parallel.jl:216-276 -> src/ParallelKernel/parallel.jl:303-334): it launches the
libps_b200.so kernel for `kernel` on the device arrays in `args` and, unless ``sync=False``
(``@parallel_async``), synchronises the stream.

Recognised kernels (each is one statement body of the reference, matched by ``from_source``):
  copy3D                   examples/memcopy3D.jl:10-13
  diffusion3D_step         examples/diffusion3D_novis_noperf.jl:10-13           (…/dx^2 form)
  diffusion3D_step_inv     examples/diffusion3D_multigpucpu_hidecomm_novis.jl:12-15 (…*_dx^2)
  diffusion3D_step_flux    test/test_parallel.jl:420-426 (on-the-fly flux form, scalar lam)
  diffusion3D_step_flux_lam  the flux form with a conductivity array (@av_xi(lam) faces)
  acoustic3D_compute_V / _P  miniapps/acoustic3D.jl:11-21
  fd_kernel("@<sel>(R) = @<macro>(A)")  every FiniteDifferences macro (ps_fd_apply)
"""
from __future__ import annotations

import ctypes
import re
from dataclasses import dataclass

from . import _lib
from ._lib import PSLaunch
from .core import ArgumentError, default_memopt, descriptor, require_initialized, stream_handle
from .fd import FdKernel, fd_kernel

PS_DIFF_DIV, PS_DIFF_MUL, PS_DIFF_FLUX, PS_DIFF_FLUX_LAM = 0, 1, 2, 3
FP64_MODES = {"ieee": 0, "split": 1, "split_state": 2, "split_grid": 3}

_lib.register("ps_diffusion3d_run", [ctypes.c_int32] + [_lib.PSArray] * 4 + [ctypes.c_double] * 5 +
              [ctypes.c_int64, ctypes.POINTER(PSLaunch), ctypes.c_void_p])


def _launch_cfg(memopt: bool, loopsize: int, ranges, fp64: str = "ieee"):
    cfg = PSLaunch()
    cfg.memopt = int(bool(memopt))
    cfg.loopsize = int(loopsize or 0)
    if fp64 not in FP64_MODES:
        raise ArgumentError(f"fp64 must be one of {tuple(FP64_MODES)} (obtained {fp64!r})")
    cfg.fp64_mode = FP64_MODES[fp64]
    if ranges is not None:
        lo, hi = ranges_to_box(ranges)
        for d in range(3):
            cfg.range_lo[d], cfg.range_hi[d] = lo[d], hi[d]
    return cfg


def ranges_to_box(ranges):
    """Julia `ranges` (1-based inclusive UnitRanges as (start, stop) pairs, or python ranges
    over 0-based indices) -> 0-based half-open (lo, hi) boxes."""
    lo, hi = [0, 0, 0], [1, 1, 1]
    if len(ranges) > 3:
        raise ArgumentError("ranges must have at most 3 dimensions")
    for d, r in enumerate(ranges):
        if isinstance(r, range):
            if r.step != 1:
                raise ArgumentError("ranges must have step 1")
            lo[d], hi[d] = r.start, r.stop
        else:
            start, stop = r
            lo[d], hi[d] = int(start) - 1, int(stop)
    return lo, hi


@dataclass(frozen=True)
class Kernel:
    name: str
    nargs: int

    def launch(self, args, memopt, loopsize, ranges, stream, sync, fp64="ieee"):  # pragma: no cover - abstract
        raise NotImplementedError


@dataclass(frozen=True)
class Copy3D(Kernel):
    def launch(self, args, memopt, loopsize, ranges, stream, sync, fp64="ieee"):
        T2, T, Ci = args
        cfg = _launch_cfg(memopt, loopsize, ranges, fp64)
        _lib.call("ps_memcopy3d", descriptor(T2), descriptor(T), descriptor(Ci), ctypes.byref(cfg),
                  stream_handle(stream), int(bool(sync)))


@dataclass(frozen=True)
class Diffusion3D(Kernel):
    form: int

    def split_args(self, args):
        T2, T, Ci, lam, dt, hx, hy, hz = args
        if self.form == PS_DIFF_FLUX_LAM:
            return T2, T, Ci, lam, 0.0, dt, hx, hy, hz
        return T2, T, Ci, None, lam, dt, hx, hy, hz

    def launch(self, args, memopt, loopsize, ranges, stream, sync, fp64="ieee"):
        T2, T, Ci, lam_arr, lam, dt, hx, hy, hz = self.split_args(args)
        cfg = _launch_cfg(memopt, loopsize, ranges, fp64)
        _lib.call("ps_diffusion3d_step", self.form, descriptor(T2), descriptor(T), descriptor(Ci),
                  descriptor(lam_arr), float(lam), float(dt), float(hx), float(hy), float(hz), ctypes.byref(cfg),
                  stream_handle(stream), int(bool(sync)))


@dataclass(frozen=True)
class Acoustic3D(Kernel):
    which: str

    def launch(self, args, memopt, loopsize, ranges, stream, sync, fp64="ieee"):
        if ranges is not None:
            raise ArgumentError(f"{self.name}: explicit ranges are not supported")
        if self.which == "V":
            Vx, Vy, Vz, P, dt, rho, dx, dy, dz = args
            _lib.call("ps_acoustic3d_v", descriptor(Vx), descriptor(Vy), descriptor(Vz), descriptor(P), float(dt),
                      float(rho), float(dx), float(dy), float(dz), stream_handle(stream), int(bool(sync)))
        else:
            P, Vx, Vy, Vz, dt, k, dx, dy, dz = args
            _lib.call("ps_acoustic3d_p", descriptor(P), descriptor(Vx), descriptor(Vy), descriptor(Vz), float(dt),
                      float(k), float(dx), float(dy), float(dz), stream_handle(stream), int(bool(sync)))


copy3D = Copy3D("copy3D!", 3)
diffusion3D_step = Diffusion3D("diffusion3D_step!", 8, PS_DIFF_DIV)
diffusion3D_step_inv = Diffusion3D("diffusion3D_step!", 8, PS_DIFF_MUL)
diffusion3D_step_flux = Diffusion3D("diffusion3D_step!", 8, PS_DIFF_FLUX)
diffusion3D_step_flux_lam = Diffusion3D("diffusion3D_step!", 8, PS_DIFF_FLUX_LAM)
acoustic3D_compute_V = Acoustic3D("compute_V!", 9, "V")
acoustic3D_compute_P = Acoustic3D("compute_P!", 9, "P")

# Kernel bodies as written in the reference (whitespace-insensitive) -> kernel.
_SOURCES = {
    "@all(T2) = @all(T) + @all(Ci)": copy3D,
    "@inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)/dx^2 + @d2_yi(T)/dy^2 + @d2_zi(T)/dz^2))": diffusion3D_step,
    "@inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))":
        diffusion3D_step_inv,
    ("@all(qx) = -lam*@d_xi(T)*_dx; @all(qy) = -lam*@d_yi(T)*_dy; @all(qz) = -lam*@d_zi(T)*_dz; "
     "@all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz); "
     "@inn(T2) = @inn(T) + dt*@all(dTdt)"): diffusion3D_step_flux,
    ("@all(qx) = -@av_xi(lam)*@d_xi(T)*_dx; @all(qy) = -@av_yi(lam)*@d_yi(T)*_dy; "
     "@all(qz) = -@av_zi(lam)*@d_zi(T)*_dz; "
     "@all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz); "
     "@inn(T2) = @inn(T) + dt*@all(dTdt)"): diffusion3D_step_flux_lam,
    ("@inn(Vx) = @inn(Vx) - dt/ρ*@d_xi(P)/dx; @inn(Vy) = @inn(Vy) - dt/ρ*@d_yi(P)/dy; "
     "@inn(Vz) = @inn(Vz) - dt/ρ*@d_zi(P)/dz"): acoustic3D_compute_V,
    "@all(P) = @all(P) - dt*k*(@d_xa(Vx)/dx + @d_ya(Vy)/dy + @d_za(Vz)/dz)": acoustic3D_compute_P,
}


def _normalise(src: str) -> str:
    src = re.sub(r"#[^\n]*", "", src)
    parts = [re.sub(r"\s+", "", p) for p in re.split(r"[;\n]", src)]
    return ";".join(p for p in parts if p and p != "return")


_NORMALISED = {_normalise(k): v for k, v in _SOURCES.items()}


def from_source(body: str, ndims: int = 3):
    """Recognise a `@parallel` kernel body (statements separated by ';' or newlines).

    This is the pattern matching the `:GB300` package performs on kernel ASTs: known
    bodies map to their hand-written libps_b200.so kernel; one-statement FD bodies map to
    ps_fd_apply. Anything else raises ArgumentError: other bodies need their full definition
    (argument order) and go through ps_gb300.parallel_kernel, the run-time compiler.
    """
    key = _normalise(body)
    if key in _NORMALISED:
        return _NORMALISED[key]
    if ";" not in key:
        return fd_kernel(body.strip().rstrip(";"), ndims)
    raise ArgumentError("unsupported @parallel kernel body for the GB300 package")


def parallel(kernel, *args, memopt=None, loopsize=0, ranges=None, stream=None, sync=True, fp64="ieee",
             nblocks=None, nthreads=None, shmem=None, grad=None, ad_mode="reverse"):
    """`@parallel [ranges] [nblocks nthreads] [memopt=...] [shmem=...] kernel!(args...)`.

    grad=((A, Ā), (B, B̄), ...) is `@parallel ∇=(A->Ā, B->B̄) [ad_mode=...] kernel!(args...)`
    (src/ParallelKernel/parallel.jl:265-301): the derivative kernel of a run-time compiled kernel
    (ps_gb300.ad), reverse (Enzyme.Reverse) or forward (Enzyme.Forward) mode."""
    require_initialized()
    if grad is not None:
        from .ad import parallel_grad

        if memopt or loopsize or shmem or fp64 != "ieee":
            raise ArgumentError("∇: memopt, loopsize, shmem and fp64 do not apply to derivative kernels")
        parallel_grad(kernel, args, grad, ad_mode=ad_mode, ranges=ranges, stream=stream, sync=sync, nblocks=nblocks,
                      nthreads=nthreads)
        return
    if hasattr(kernel, "jit_launch"):  # run-time compiled kernel (ps_gb300.jit); memopt does not change results
        kernel.jit_launch(args, ranges, stream, sync, nblocks=nblocks, nthreads=nthreads, shmem=shmem, memopt=memopt,
                          loopsize=loopsize, fp64=fp64)
        return
    if nblocks is not None or nthreads is not None or shmem is not None:
        raise ArgumentError("nblocks / nthreads / shmem apply to run-time compiled kernels (parallel_kernel)")
    if isinstance(kernel, FdKernel):
        if ranges is not None or memopt:
            raise ArgumentError("FD operator kernels take no ranges/memopt")
        if fp64 not in ("ieee", "split"):
            raise ArgumentError("fp64 must be 'ieee' or 'split' for FD operator kernels")
        R, A = args
        if fp64 == "split" and descriptor(R).dtype == 0:
            kernel.launch_split(R, A, stream=stream, sync=sync)
        else:
            kernel.launch(R, A, stream=stream, sync=sync)
        return
    if not isinstance(kernel, Kernel):
        raise ArgumentError(f"not a GB300 kernel: {kernel!r}")
    if len(args) != kernel.nargs:
        raise ArgumentError(f"{kernel.name} takes {kernel.nargs} arguments (obtained {len(args)})")
    if memopt is None:
        memopt = default_memopt()
    kernel.launch(args, memopt, loopsize, ranges, stream, sync, fp64)


def run(kernel, T, T2, Ci, lam, dt, hx, hy, hz, nt, *, memopt=True, loopsize=0, fp64="ieee", stream=None,
        sync=True):
    """`for it = 1:nt; @parallel kernel!(T2, T, Ci, lam, dt, h...); T, T2 = T2, T; end` as one call
    (ps_diffusion3d_run); on return T holds the state after nt steps."""
    require_initialized()
    if not isinstance(kernel, Diffusion3D):
        raise ArgumentError("run() is implemented for the diffusion3D kernels")
    _, _, _, lam_arr, lam_s, _, _, _, _ = kernel.split_args((T2, T, Ci, lam, dt, hx, hy, hz))
    cfg = _launch_cfg(memopt, loopsize, None, fp64)
    _lib.call("ps_diffusion3d_run", kernel.form, descriptor(T), descriptor(T2), descriptor(Ci), descriptor(lam_arr),
              float(lam_s), float(dt), float(hx), float(hy), float(hz), int(nt), ctypes.byref(cfg),
              stream_handle(stream))
    if sync:
        from .core import synchronize

        synchronize(stream)


def acoustic3d_step(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, dt, rho, k, dx, dy, dz, *, fp64="ieee", stream=None,
                    sync=True):
    """One step of the acoustic3D time loop (`@parallel compute_V!(...)`, `@parallel compute_P!(...)`,
    miniapps/acoustic3D.jl:55-56) as one kernel (ps_acoustic3d_step): reads (Vx, Vy, Vz, P), writes
    the new state into (Vx2, Vy2, Vz2, P2). fp64 = "ieee" (bit-identical) or "split" (FP32 pairs)."""
    require_initialized()
    if fp64 not in ("ieee", "split"):
        raise ArgumentError(f"fp64 must be 'ieee' or 'split' (obtained {fp64!r})")
    _lib.call("ps_acoustic3d_step", *(descriptor(a) for a in (Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2)), float(dt),
              float(rho), float(k), float(dx), float(dy), float(dz), FP64_MODES[fp64], stream_handle(stream),
              int(bool(sync)))


def acoustic3d_run(Vx, Vy, Vz, P, dt, rho, k, dx, dy, dz, nt, *, fp64="ieee", stream=None, sync=True):
    """`for it = 1:nt; @parallel compute_V!(...); @parallel compute_P!(...); end` in place on
    (Vx, Vy, Vz, P) (ps_acoustic3d_run: one fused kernel per step, a second state set in library
    scratch)."""
    require_initialized()
    if fp64 not in ("ieee", "split"):
        raise ArgumentError(f"fp64 must be 'ieee' or 'split' (obtained {fp64!r})")
    _lib.call("ps_acoustic3d_run", *(descriptor(a) for a in (Vx, Vy, Vz, P)), float(dt), float(rho), float(k),
              float(dx), float(dy), float(dz), int(nt), FP64_MODES[fp64], stream_handle(stream))
    if sync:
        from .core import synchronize

        synchronize(stream)


def parallel_async(kernel, *args, **kw):
    """`@parallel_async kernel!(args...)`: no synchronisation."""
    kw["sync"] = False
    parallel(kernel, *args, **kw)


def hide_communication(boundary_width, kernel, args, comm=None, *, memopt=None, s_boundary=None, s_inner=None,
                       fp64="ieee"):
    """`@hide_communication boundary_width begin @parallel kernel!(args...); comm() end`.

    The six boundary slabs run on a high-priority stream and the inner box on a normal
    stream (src/ParallelKernel/hide_communication.jl:177-258); `comm` runs on the host once
    the boundary slabs are done. The diffusion kernels split inside the library
    (ps_diffusion3d_step_split); run-time compiled kernels split by ranges on two streams.
    """
    require_initialized()
    bw = boundary_width if isinstance(boundary_width, (tuple, list)) else (boundary_width,) * 3
    if len(bw) != 3:
        raise ArgumentError("boundary_width must be an integer or a 3-tuple")
    if hasattr(kernel, "jit_launch"):
        _hide_communication_jit(tuple(int(b) for b in bw), kernel, args, comm, memopt, s_boundary, s_inner, fp64)
        return
    if not isinstance(kernel, Diffusion3D):
        raise ArgumentError("@hide_communication is implemented for the diffusion3D kernels and for run-time "
                            "compiled kernels")
    T2, T, Ci, lam_arr, lam, dt, hx, hy, hz = kernel.split_args(args)
    memopt = default_memopt() if memopt is None else memopt
    sb_def, si_def = _hide_streams()
    if s_boundary is None or s_inner is None:  # the default pair follows the work queued on the current stream
        import torch

        cur = torch.cuda.current_stream()
        for st in (sb_def, si_def):
            st.wait_stream(cur)
    s_boundary = stream_handle(s_boundary if s_boundary is not None else sb_def)
    s_inner = stream_handle(s_inner if s_inner is not None else si_def)
    errors = []

    def _cb(_ctx):
        try:
            if comm is not None:
                comm()
            return 0
        except Exception as e:  # noqa: BLE001 - reported after the call
            errors.append(e)
            return -1

    cb = _lib.COMM_FN(_cb)
    bw_arr = (ctypes.c_int64 * 3)(*[int(b) for b in bw])
    cfg = _launch_cfg(memopt, 0, None, fp64)
    _lib.call("ps_diffusion3d_step_split", kernel.form, descriptor(T2), descriptor(T), descriptor(Ci),
              descriptor(lam_arr), float(lam), float(dt), float(hx), float(hy), float(hz), ctypes.byref(cfg),
              bw_arr, s_boundary, s_inner, cb, None)
    if errors:
        raise errors[0]


_HIDE_STREAMS = {}


def _hide_streams():
    """The default (boundary, inner) stream pair of the current device: a high-priority and a
    normal-priority torch stream, created once (streams outlive the calls that use them)."""
    import torch

    dev = torch.cuda.current_device()
    if dev not in _HIDE_STREAMS:
        _HIDE_STREAMS[dev] = (torch.cuda.Stream(priority=-1), torch.cuda.Stream(priority=0))
    return _HIDE_STREAMS[dev]


def _hide_communication_jit(bw, kernel, args, comm, memopt, s_boundary, s_inner, fp64="ieee"):
    """The boundary/inner split for any run-time compiled kernel: the six boundary boxes of the
    kernel's `@parallel` grid on a high-priority stream, the inner box on a normal one, `comm` on
    the host once the boundary boxes are done, while the inner box runs."""
    import torch

    ms = kernel.grid_extent(args)
    for d in range(3):
        if bw[d] < 0:
            raise ArgumentError("boundary width must be >= 0")
        if not ms[d] > 2 * bw[d]:
            raise ArgumentError("@hide_communication: length(ranges) > 2*boundary_width violated")
        if ms[d] > 1 and bw[d] == 0:
            raise ArgumentError("@hide_communication: boundary_width 0 in a dimension of length > 1")
    # s_boundary / s_inner: torch streams (default: the device's high-priority / normal-priority pair)
    sb_def, si_def = _hide_streams()
    sb = s_boundary if s_boundary is not None else sb_def
    si = s_inner if s_inner is not None else si_def
    cur = torch.cuda.current_stream()
    for s in (sb, si):
        s.wait_stream(cur)
    if kernel.hide_eligible():  # one boundary-first launch on s_inner (after s_boundary's queued work)
        si.wait_stream(sb)
        errors = []

        def _cb(_ctx):
            try:
                if comm is not None:
                    comm()
                return 0
            except Exception as e:  # noqa: BLE001 - reported after the call
                errors.append(e)
                return -1

        try:
            kernel.hide_communication(args, bw, _lib.COMM_FN(_cb), si, memopt=memopt, fp64=fp64)
        finally:
            cur.wait_stream(si)
        if errors:
            raise errors[0]
        return
    lw, hw = widened_widths(bw, ms)
    for lo, hi in get_ranges_outer(lw, ms, hw):
        kernel.jit_launch(args, [range(lo[d], hi[d]) for d in range(3)], sb, False, memopt=memopt, fp64=fp64)
    for lo, hi in get_ranges_inner(lw, ms, hw):
        kernel.jit_launch(args, [range(lo[d], hi[d]) for d in range(3)], si, False, memopt=memopt, fp64=fp64)
    sb.synchronize()
    try:
        if comm is not None:
            comm()
    finally:
        si.synchronize()
        cur.wait_stream(sb)
        cur.wait_stream(si)
    kernel.check(si)


def widened_widths(bw, ms, blocks=(32, 8)):
    """Lower and upper boundary widths with the x and y slabs widened to whole thread blocks
    (default 32 x 8) where the grid allows it: a 16-wide x slab would leave half of every warp idle,
    and an inner box starting mid-block would cost one more block column. The boundary boxes then
    hold a superset of the requested boundary (all computed before `comm`)."""
    lw, hw = list(bw), list(bw)
    for d, blk in enumerate(blocks):
        a = -(-bw[d] // blk) * blk  # lower slab [0, a)
        b = ms[d] - (ms[d] - bw[d]) // blk * blk  # upper slab [ms - b, ms) from a block edge
        if bw[d] > 0 and ms[d] > a + b:
            lw[d], hw[d] = a, b
    return lw, hw


def get_ranges_outer(boundary_width, maxsize, upper_width=None):
    """The six boundary boxes of `@hide_communication` (3-D), 0-based half-open
    (src/ParallelKernel/hide_communication.jl:350-381); `upper_width`: the widths at the upper ends
    when they differ from the lower ones."""
    bw, ms = boundary_width, maxsize
    uw = bw if upper_width is None else upper_width
    boxes = [
        ((0, bw[1], bw[2]), (bw[0], ms[1] - uw[1], ms[2] - uw[2])),
        ((0, 0, 0), (ms[0], ms[1], bw[2])),
        ((0, 0, ms[2] - uw[2]), (ms[0], ms[1], ms[2])),
        ((ms[0] - uw[0], bw[1], bw[2]), (ms[0], ms[1] - uw[1], ms[2] - uw[2])),
        ((0, 0, bw[2]), (ms[0], bw[1], ms[2] - uw[2])),
        ((0, ms[1] - uw[1], bw[2]), (ms[0], ms[1], ms[2] - uw[2])),
    ]
    return [b for b in boxes if all(h > l for l, h in zip(*b))]


def get_ranges_inner(boundary_width, maxsize, upper_width=None):
    bw, ms = boundary_width, maxsize
    uw = bw if upper_width is None else upper_width
    return [((bw[0], bw[1], bw[2]), (ms[0] - uw[0], ms[1] - uw[1], ms[2] - uw[2]))]
