"""Adjoint of the 3-D diffusion step and the checkpointed misfit gradient (libps_b200.so).

This replaces the reference's Enzyme-generated reverse kernels (`@parallel ∇=(T->T̄, lam->lam̄)
diffusion3D_step!(...)`, src/ParallelKernel/parallel.jl:265-301) for the flux-form diffusion step
with a conductivity array:

    adjoint_step(lamT, lamT2, T, Ci, lam, glam, dt, _dx, _dy, _dz)   # one reverse step
    misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt, checkpoint_every)  # dL/dlam of 0.5||T_nt - T_obs||^2

``diffusion_step_rrule`` packages the forward step with its pullback, the shape a ChainRules
`rrule` has on the Julia side.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import PSArray, PSLaunch
from .core import descriptor, empty_like, require_initialized, stream_handle, zeros_like
from .kernels import _launch_cfg, diffusion3D_step_flux_lam, parallel


class PSAdjointStats(ctypes.Structure):
    _fields_ = [("loss", ctypes.c_double), ("checkpoints", ctypes.c_int64), ("recomputed_steps", ctypes.c_int64),
                ("seconds", ctypes.c_double)]


_D = ctypes.c_double
_lib.register("ps_diffusion3d_adjoint_step", [PSArray] * 6 + [_D] * 4 + [ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_diffusion3d_adjoint_step_ex", [PSArray] * 6 + [_D] * 4 + [ctypes.c_int32, ctypes.c_void_p,
                                                                            ctypes.c_int])
_lib.register("ps_diffusion3d_misfit_gradient",
              [PSArray] * 4 + [_D] * 4 + [ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(PSLaunch), PSArray, PSArray,
                                          ctypes.POINTER(PSAdjointStats), ctypes.c_void_p])


def adjoint_step(lamT, lamT2, T, Ci, lam, glam, dt, hx, hy, hz, stream=None, sync=True, fp64="ieee"):
    """lamT = (∂T2/∂T)^T lamT2 (inner cells), glam += (∂T2/∂lam)^T lamT2 for T2 = step(T, lam);
    fp64="split" evaluates it on FP32 pairs (FP64 arrays)."""
    require_initialized()
    cfg = _launch_cfg(False, 0, None, fp64)
    _lib.call("ps_diffusion3d_adjoint_step_ex", descriptor(lamT), descriptor(lamT2), descriptor(T), descriptor(Ci),
              descriptor(lam), descriptor(glam), float(dt), float(hx), float(hy), float(hz), int(cfg.fp64_mode),
              stream_handle(stream), int(bool(sync)))


def misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt, checkpoint_every=20, memopt=True, fp64="ieee", stream=None,
                    return_final=False):
    """(loss, dL/dlam[, T_nt], stats) for L = 0.5 ||T_nt - T_obs||^2."""
    require_initialized()
    g = zeros_like(T0)
    Tf = empty_like(T0) if return_final else None
    st = PSAdjointStats()
    cfg = _launch_cfg(memopt, 0, None, fp64)
    _lib.call("ps_diffusion3d_misfit_gradient", descriptor(T0), descriptor(T_obs), descriptor(Ci), descriptor(lam),
              float(dt), float(h[0]), float(h[1]), float(h[2]), int(nt), int(checkpoint_every), ctypes.byref(cfg),
              descriptor(g), descriptor(Tf) if Tf is not None else PSArray(None, (ctypes.c_int64 * 3)(1, 1, 1), 0, 0),
              ctypes.byref(st), stream_handle(stream))
    if return_final:
        return st.loss, g, Tf, st
    return st.loss, g, st


def diffusion_step_rrule(T, Ci, lam, dt, hx, hy, hz, memopt=True, fp64="ieee"):
    """Forward step T2 = step(T, lam) and its pullback λ2 -> (λT, λlam)."""
    T2 = empty_like(T)
    T2.copy_(T)
    parallel(diffusion3D_step_flux_lam, T2, T, Ci, lam, dt, hx, hy, hz, memopt=memopt, fp64=fp64)

    def pullback(lamT2):
        lamT = empty_like(T)
        glam = zeros_like(T)
        adjoint_step(lamT, lamT2, T, Ci, lam, glam, dt, hx, hy, hz)
        return lamT, glam

    return T2, pullback
