"""Pseudo-transient viscous Stokes 3-D (miniapps/Stokes3D.jl) on libps_b200.so.

``Stokes3D`` holds the miniapp's arrays (Stokes3D.jl:89-110) as device arrays in Julia layout and
exposes the `@parallel` kernels one-to-one (``compute_timesteps``, ``compute_P``, ``compute_tau``,
``compute_dV``, ``compute_V``, ``bc``), ``step_reference_sequence()`` (the loop body as the
miniapp writes it, ten launches), ``iterate(n)`` (the loop body in three launches per
iteration), ``err()`` (Stokes3D.jl:145-146) and ``solve(tol)`` (the `while err > ε` loop in FP64).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import PSArray
from .core import ArgumentError, descriptor, from_host, require_initialized, stream_handle, to_host, zeros
from .stokes import PSSolveStats

FIELDS = ("Pt", "dtauPt", "divV", "Vx", "Vy", "Vz", "txx", "tyy", "tzz", "txy", "txz", "tyz", "Rx", "Ry", "Rz",
          "dVxdtau", "dVydtau", "dVzdtau", "dtauVx", "dtauVy", "dtauVz", "Mus", "Rog")
# extents relative to (nx, ny, nz) = size(Pt)
SHAPES = {"Pt": (0, 0, 0), "dtauPt": (0, 0, 0), "divV": (0, 0, 0), "Vx": (1, 0, 0), "Vy": (0, 1, 0),
          "Vz": (0, 0, 1), "txx": (0, -2, -2), "tyy": (-2, 0, -2), "tzz": (-2, -2, 0), "txy": (-1, -1, -2),
          "txz": (-1, -2, -1), "tyz": (-2, -1, -1), "Rx": (-1, -2, -2), "Ry": (-2, -1, -2), "Rz": (-2, -2, -1),
          "dVxdtau": (-1, -2, -2), "dVydtau": (-2, -1, -2), "dVzdtau": (-2, -2, -1), "dtauVx": (-1, -2, -2),
          "dtauVy": (-2, -1, -2), "dtauVz": (-2, -2, -1), "Mus": (0, 0, 0), "Rog": (0, 0, 0)}


class PSStokes3DFields(ctypes.Structure):
    _fields_ = [(n, PSArray) for n in FIELDS]


class PSStokes3DParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("dx", "dy", "dz", "dampX", "dampY", "dampZ", "Vsc", "Ptsc",
                                               "min_dxyz2")] + [("max_nxyz", ctypes.c_int64)]


_F = ctypes.POINTER(PSStokes3DFields)
_PP = ctypes.POINTER(PSStokes3DParams)
for _name in ("ps_stokes3d_timesteps", "ps_stokes3d_compute_P", "ps_stokes3d_compute_tau", "ps_stokes3d_compute_dV",
              "ps_stokes3d_compute_V"):
    _lib.register(_name, [_F, _PP, ctypes.c_void_p, ctypes.c_int])
for _name in ("ps_bc_x3d", "ps_bc_y3d", "ps_bc_z3d"):
    _lib.register(_name, [PSArray, ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_stokes3d_iterate", [_F, _PP, ctypes.c_int64, ctypes.c_void_p])
_lib.register("ps_stokes3d_iterate_ex", [_F, _PP, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p])
_lib.register("ps_stokes3d_err", [_F, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p])
_lib.register("ps_stokes3d_solve", [_F, _PP, ctypes.c_double, ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                    ctypes.POINTER(PSSolveStats), ctypes.c_void_p])
_lib.register("ps_stokes3d_solve_mixed", [_F, _PP, ctypes.c_double, ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                    ctypes.POINTER(PSSolveStats), ctypes.c_void_p])


@dataclass
class Stokes3DParams:
    """Numerics of Stokes3D.jl:72-88 (defaults: the miniapp's)."""

    nx: int
    ny: int
    nz: int
    lx: float = 10.0
    ly: float = 10.0
    lz: float = 10.0
    Vdmp: float = 4.0
    Vsc: float = 1.0
    Ptsc: float = 1.0 / 4.0

    @property
    def h(self):
        return self.lx / (self.nx - 1), self.ly / (self.ny - 1), self.lz / (self.nz - 1)

    def c_struct(self) -> PSStokes3DParams:
        dx, dy, dz = self.h
        return PSStokes3DParams(dx, dy, dz, 1.0 - self.Vdmp / self.nx, 1.0 - self.Vdmp / self.ny,
                                1.0 - self.Vdmp / self.nz, self.Vsc, self.Ptsc, min(dx, dy, dz) ** 2,
                                max(self.nx, self.ny, self.nz))


def inclusion_setup(nx, ny, nz, lx=10.0, ly=10.0, lz=10.0, mus0=1.0, musi=0.1, rhogi=1.0, radius=None,
                    dtype=np.float64):
    """Mus, Rog of Stokes3D.jl:111-117: a spherical inclusion at the centre (Radc <= r^2, r = 1 on the
    miniapp's 10^3 box; `radius=None` keeps that ratio)."""
    dx, dy, dz = lx / (nx - 1), ly / (ny - 1), lz / (nz - 1)
    r2 = (lx / 10.0) ** 2 if radius is None else radius ** 2
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    radc = (ix * dx - 0.5 * lx) ** 2 + (iy * dy - 0.5 * ly) ** 2 + (iz * dz - 0.5 * lz) ** 2
    Mus = mus0 * np.ones((nx, ny, nz))
    Rog = np.zeros((nx, ny, nz))
    Mus[radc <= r2] = musi
    Rog[radc <= r2] = rhogi
    return np.asfortranarray(Mus.astype(dtype)), np.asfortranarray(Rog.astype(dtype))


class Stokes3D:
    """Device arrays of the Stokes3D miniapp and the GB300 kernels acting on them."""

    BC_SEQUENCE = (("x", "Vy"), ("x", "Vz"), ("y", "Vx"), ("y", "Vz"), ("z", "Vx"), ("z", "Vy"))

    def __init__(self, params: Stokes3DParams, Mus: np.ndarray, Rog: np.ndarray, dtype=np.float64):
        require_initialized()
        n = (params.nx, params.ny, params.nz)
        self.params, self.dtype = params, dtype
        self.arrays = {k: zeros(*(m + o for m, o in zip(n, off)), dtype=dtype) for k, off in SHAPES.items()
                       if k not in ("Mus", "Rog")}
        self.arrays["Mus"] = from_host(np.asarray(Mus, dtype=dtype))
        self.arrays["Rog"] = from_host(np.asarray(Rog, dtype=dtype))
        self._fields = PSStokes3DFields(*[descriptor(self.arrays[k]) for k in FIELDS])
        self._p = params.c_struct()

    def __getitem__(self, name):
        return self.arrays[name]

    def host(self, name) -> np.ndarray:
        return to_host(self.arrays[name])

    def _k(self, entry, stream=None, sync=True):
        _lib.call(entry, ctypes.byref(self._fields), ctypes.byref(self._p), stream_handle(stream), int(bool(sync)))

    def compute_timesteps(self, **kw):
        self._k("ps_stokes3d_timesteps", **kw)

    def compute_P(self, **kw):
        self._k("ps_stokes3d_compute_P", **kw)

    def compute_tau(self, **kw):
        self._k("ps_stokes3d_compute_tau", **kw)

    def compute_dV(self, **kw):
        self._k("ps_stokes3d_compute_dV", **kw)

    def compute_V(self, **kw):
        self._k("ps_stokes3d_compute_V", **kw)

    def bc(self, which, name, stream=None, sync=True):
        _lib.call(f"ps_bc_{which}3d", descriptor(self.arrays[name]), stream_handle(stream), int(bool(sync)))

    def step_reference_sequence(self):
        """One loop body as the miniapp writes it (Stokes3D.jl:134-143), ten launches."""
        self.compute_P()
        self.compute_tau()
        self.compute_dV()
        self.compute_V()
        for which, name in self.BC_SEQUENCE:
            self.bc(which, name)

    def iterate(self, n_iter: int, stream=None, one_launch=False):
        """n_iter iterations of the miniapp's loop body (ps_stokes3d_iterate_ex); one_launch: pairs of
        single-kernel iterations, ending with the storing kernels (bit-identical results)."""
        _lib.call("ps_stokes3d_iterate_ex", ctypes.byref(self._fields), ctypes.byref(self._p), int(n_iter),
                  int(bool(one_launch)), stream_handle(stream))

    def err(self, stream=None):
        out = (ctypes.c_double * 4)()
        _lib.call("ps_stokes3d_err", ctypes.byref(self._fields), out, stream_handle(stream))
        return max(out), tuple(out)

    def solve(self, tol=1e-6, max_iter=100_000, nout=500, max_seconds=0.0, stream=None, mode=0):
        """PT solve to err < tol; mode 0: FP64 (the reference's iteration), mode 1: FP32 sweeps on
        FP64 defect corrections (ps_stokes3d_solve_mixed). Returns PSSolveStats; raises PSError if
        it does not converge."""
        if mode not in (0, 1):
            raise ArgumentError("mode must be 0 (FP64) or 1 (FP32 + FP64 defect correction)")
        st = PSSolveStats()
        fn = _lib.load().ps_stokes3d_solve if mode == 0 else _lib.load().ps_stokes3d_solve_mixed
        rc = fn(ctypes.byref(self._fields), ctypes.byref(self._p), float(tol), int(max_iter), int(nout),
                float(max_seconds), ctypes.byref(st), stream_handle(stream))
        if rc != 0:
            err = _lib.PSError(rc, _lib.last_error())
            err.stats = st
            raise err
        return st
