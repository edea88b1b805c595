"""Pseudo-transient viscous Stokes 2-D (miniapps/Stokes2D.jl) on libps_b200.so.

``Stokes2D`` holds the miniapp's arrays (Stokes2D.jl:79-101) as device arrays in Julia layout
and exposes
  - the six `@parallel` kernels one-to-one (``compute_timesteps``, ``compute_P``, ``compute_tau``,
    ``compute_dV``, ``compute_V``, ``bc_x``/``bc_y``),
  - ``iterate(n)``: n iterations of the loop body with one fused kernel per iteration,
  - ``err()``: max(mean|Rx|, mean|Ry|, mean|∇V|) (Stokes2D.jl:119-120),
  - ``solve(tol, mode)``: the `while err > ε` loop in FP64 (mode 0) or with FP32 PT sweeps on the
    defect-correction update and an FP64 residual / update / convergence check (mode 1).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import PSArray
from .core import descriptor, from_host, require_initialized, stream_handle, to_host, zeros

FIELDS = ("Pt", "dtauPt", "divV", "Vx", "Vy", "txx", "tyy", "txy", "Rx", "Ry", "dVxdtau", "dVydtau", "dtauVx",
          "dtauVy", "Mus", "Rog")


class PSStokes2DFields(ctypes.Structure):
    _fields_ = [(n, PSArray) for n in FIELDS]


class PSStokes2DParams(ctypes.Structure):
    _fields_ = [("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dampX", ctypes.c_double),
                ("dampY", ctypes.c_double), ("Vsc", ctypes.c_double), ("Ptsc", ctypes.c_double),
                ("min_dxy2", ctypes.c_double), ("max_nxy", ctypes.c_int64)]


class PSSolveStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int64), ("outer", ctypes.c_int64), ("err", ctypes.c_double),
                ("seconds", ctypes.c_double), ("converged", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_F = ctypes.POINTER(PSStokes2DFields)
_PP = ctypes.POINTER(PSStokes2DParams)
for _name in ("ps_stokes2d_timesteps", "ps_stokes2d_compute_P", "ps_stokes2d_compute_tau", "ps_stokes2d_compute_dV",
              "ps_stokes2d_compute_V"):
    _lib.register(_name, [_F, _PP, ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_bc_x2d", [PSArray, ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_bc_y2d", [PSArray, ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_stokes2d_iterate", [_F, _PP, ctypes.c_int64, ctypes.c_void_p])
_lib.register("ps_stokes2d_iterate_static", [_F, _PP, ctypes.c_int64, ctypes.c_void_p])
_lib.register("ps_stokes2d_err", [_F, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p])
_lib.register("ps_stokes2d_solve", [_F, _PP, ctypes.c_int32, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                                    ctypes.c_double, ctypes.POINTER(PSSolveStats), ctypes.c_void_p])

MODE_FP64, MODE_MIXED = 0, 1


@dataclass
class Stokes2DParams:
    """Numerics of Stokes2D.jl:60-77 (defaults: the miniapp's)."""

    nx: int
    ny: int
    lx: float = 10.0
    ly: float = 10.0
    Vdmp: float = 4.0
    Vsc: float = 1.0
    Ptsc: float = 1.0 / 4.0

    @property
    def dx(self):
        return self.lx / (self.nx - 1)

    @property
    def dy(self):
        return self.ly / (self.ny - 1)

    def c_struct(self) -> PSStokes2DParams:
        return PSStokes2DParams(self.dx, self.dy, 1.0 - self.Vdmp / self.nx, 1.0 - self.Vdmp / self.ny, self.Vsc,
                                self.Ptsc, min(self.dx, self.dy) ** 2, max(self.nx, self.ny))


@dataclass
class Stokes2DAPTParams:
    """Numerics of the accelerated pseudo-transient iteration (pseudo-time steps from the local
    viscosity maximum): Vpdτ = CFL * min(dx, dy), dτρ = Vpdτ * max(lx, ly) / Re / Musτ,
    Gdτ = Vpdτ^2 / dτρ / (r + 2). Re = 16π converged fastest on a circular inclusion of viscosity
    ratio 1e-3 (127^2 and 255^2: 16400 and 28600 iterations to 1e-8; 5π, the constant-viscosity
    choice, needed about twice as many)."""

    nx: int
    ny: int
    lx: float = 10.0
    ly: float = 10.0
    Re: float = 16.0 * np.pi
    r: float = 1.0
    CFL: float = 0.9 / np.sqrt(2.0)

    @property
    def dx(self):
        return self.lx / (self.nx - 1)

    @property
    def dy(self):
        return self.ly / (self.ny - 1)

    @property
    def Vpdt(self):
        return min(self.dx, self.dy) * self.CFL

    @property
    def max_lxy(self):
        return max(self.lx, self.ly)


def inclusion_setup(nx, ny, lx=10.0, ly=10.0, mus0=1.0, musi=0.1, rhogi=1.0, radius=None, dtype=np.float64):
    """Mus, Rog of Stokes2D.jl:94-99: a circular inclusion at the centre (Radc < r^2).

    The miniapp uses r = 1 on a 10 x 10 box; `radius=None` keeps that ratio (r = lx / 10)."""
    dx, dy = lx / (nx - 1), ly / (ny - 1)
    r2 = (lx / 10.0) ** 2 if radius is None else radius ** 2
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    radc = (ix * dx - 0.5 * lx) ** 2 + (iy * dy - 0.5 * ly) ** 2
    Mus = mus0 * np.ones((nx, ny))
    Rog = np.zeros((nx, ny))
    Mus[radc < r2] = musi
    Rog[radc < r2] = rhogi
    return np.asfortranarray(Mus.astype(dtype)), np.asfortranarray(Rog.astype(dtype))


class Stokes2D:
    """Device arrays of the Stokes2D miniapp and the GB300 kernels acting on them."""

    def __init__(self, params: Stokes2DParams, Mus: np.ndarray, Rog: np.ndarray, dtype=np.float64):
        require_initialized()
        nx, ny = params.nx, params.ny
        self.params, self.dtype = params, dtype
        shapes = {"Pt": (nx, ny), "dtauPt": (nx, ny), "divV": (nx, ny), "Vx": (nx + 1, ny), "Vy": (nx, ny + 1),
                  "txx": (nx, ny), "tyy": (nx, ny), "txy": (nx - 1, ny - 1), "Rx": (nx - 1, ny - 2),
                  "Ry": (nx - 2, ny - 1), "dVxdtau": (nx - 1, ny - 2), "dVydtau": (nx - 2, ny - 1),
                  "dtauVx": (nx - 1, ny - 2), "dtauVy": (nx - 2, ny - 1)}
        self.arrays = {k: zeros(*v, dtype=dtype) for k, v in shapes.items()}
        self.arrays["Mus"] = from_host(np.asarray(Mus, dtype=dtype))
        self.arrays["Rog"] = from_host(np.asarray(Rog, dtype=dtype))
        self._fields = PSStokes2DFields(*[descriptor(self.arrays[n]) for n in FIELDS])
        self._p = params.c_struct()

    def __getitem__(self, name):
        return self.arrays[name]

    def host(self, name) -> np.ndarray:
        return to_host(self.arrays[name])

    def _k(self, entry, stream=None, sync=True):
        _lib.call(entry, ctypes.byref(self._fields), ctypes.byref(self._p), stream_handle(stream), int(bool(sync)))

    # one-to-one `@parallel` kernels
    def compute_timesteps(self, **kw):
        self._k("ps_stokes2d_timesteps", **kw)

    def compute_P(self, **kw):
        self._k("ps_stokes2d_compute_P", **kw)

    def compute_tau(self, **kw):
        self._k("ps_stokes2d_compute_tau", **kw)

    def compute_dV(self, **kw):
        self._k("ps_stokes2d_compute_dV", **kw)

    def compute_V(self, **kw):
        self._k("ps_stokes2d_compute_V", **kw)

    def bc_x(self, name, stream=None, sync=True):
        _lib.call("ps_bc_x2d", descriptor(self.arrays[name]), stream_handle(stream), int(bool(sync)))

    def bc_y(self, name, stream=None, sync=True):
        _lib.call("ps_bc_y2d", descriptor(self.arrays[name]), stream_handle(stream), int(bool(sync)))

    def step_reference_sequence(self):
        """One loop body as the miniapp writes it (Stokes2D.jl:111-116), six launches."""
        self.compute_P()
        self.compute_tau()
        self.compute_dV()
        self.compute_V()
        self.bc_y("Vx")
        self.bc_x("Vy")

    def iterate(self, n_iter: int, stream=None):
        _lib.call("ps_stokes2d_iterate", ctypes.byref(self._fields), ctypes.byref(self._p), int(n_iter),
                  stream_handle(stream))

    def err(self, stream=None):
        out = (ctypes.c_double * 3)()
        _lib.call("ps_stokes2d_err", ctypes.byref(self._fields), out, stream_handle(stream))
        return max(out), tuple(out)

    def solve(self, tol=1e-8, mode=MODE_FP64, max_iter=10_000_000, nout=200, max_seconds=0.0, stream=None):
        """PT solve to err < tol; returns PSSolveStats. Raises PSError if it does not converge."""
        st = PSSolveStats()
        rc = _lib.load().ps_stokes2d_solve(ctypes.byref(self._fields), ctypes.byref(self._p), int(mode), float(tol),
                                           int(max_iter), int(nout), float(max_seconds), ctypes.byref(st),
                                           stream_handle(stream))
        if rc != 0:
            err = _lib.PSError(rc, _lib.last_error())
            err.stats = st
            raise err
        return st


APT_FIELDS = ("Pt", "divV", "Vx", "Vy", "txx", "tyy", "txy", "Rx", "Ry", "Mus", "Rog", "Must", "kP", "aT", "bT", "aTc",
              "bTc", "dtVx", "dtVy")


class PSStokes2DAPTFields(ctypes.Structure):
    _fields_ = [(n, PSArray) for n in APT_FIELDS]


class PSStokes2DAPTParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("dx", "dy", "Vpdt", "Re", "r", "max_lxy")]


_FA = ctypes.POINTER(PSStokes2DAPTFields)
_PA = ctypes.POINTER(PSStokes2DAPTParams)
_lib.register("ps_stokes2d_apt_coefficients", [_FA, _PA, ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_stokes2d_apt_iterate", [_FA, _PA, ctypes.c_int64, ctypes.c_void_p])
_lib.register("ps_stokes2d_apt_residual", [_FA, _PA, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p])
_lib.register("ps_stokes2d_apt_solve", [_FA, _PA, ctypes.c_int32, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_double, ctypes.POINTER(PSSolveStats), ctypes.c_void_p])


class Stokes2DAPT:
    """The Stokes2D arrays with the accelerated pseudo-transient iteration whose pseudo-time steps
    come from @maxloc(Mus) (ps_stokes2d_apt_*): the miniapp's arrays plus the coefficient arrays
    Must, kP, aT, bT (cells), aTc, bTc (corners), dtVx, dtVy (faces)."""

    def __init__(self, params: Stokes2DAPTParams, Mus: np.ndarray, Rog: np.ndarray, dtype=np.float64):
        require_initialized()
        nx, ny = params.nx, params.ny
        self.params, self.dtype = params, dtype
        shapes = {"Pt": (nx, ny), "divV": (nx, ny), "Vx": (nx + 1, ny), "Vy": (nx, ny + 1), "txx": (nx, ny),
                  "tyy": (nx, ny), "txy": (nx - 1, ny - 1), "Rx": (nx - 1, ny - 2), "Ry": (nx - 2, ny - 1),
                  "Must": (nx, ny), "kP": (nx, ny), "aT": (nx, ny), "bT": (nx, ny), "aTc": (nx - 1, ny - 1),
                  "bTc": (nx - 1, ny - 1), "dtVx": (nx - 1, ny - 2), "dtVy": (nx - 2, ny - 1)}
        self.arrays = {k: zeros(*v, dtype=dtype) for k, v in shapes.items()}
        self.arrays["Mus"] = from_host(np.asarray(Mus, dtype=dtype))
        self.arrays["Rog"] = from_host(np.asarray(Rog, dtype=dtype))
        self._fields = PSStokes2DAPTFields(*[descriptor(self.arrays[n]) for n in APT_FIELDS])
        p = params
        self._p = PSStokes2DAPTParams(p.dx, p.dy, p.Vpdt, p.Re, p.r, p.max_lxy)

    def __getitem__(self, name):
        return self.arrays[name]

    def host(self, name) -> np.ndarray:
        return to_host(self.arrays[name])

    def coefficients(self, stream=None, sync=True):
        _lib.call("ps_stokes2d_apt_coefficients", ctypes.byref(self._fields), ctypes.byref(self._p),
                  stream_handle(stream), int(bool(sync)))

    def iterate(self, n_iter: int, stream=None):
        _lib.call("ps_stokes2d_apt_iterate", ctypes.byref(self._fields), ctypes.byref(self._p), int(n_iter),
                  stream_handle(stream))

    def residual(self, stream=None):
        """FP64 residual of the state with the stresses at their steady state: (err, (means))."""
        out = (ctypes.c_double * 3)()
        _lib.call("ps_stokes2d_apt_residual", ctypes.byref(self._fields), ctypes.byref(self._p), out,
                  stream_handle(stream))
        return max(out), tuple(out)

    def solve(self, tol=1e-8, mode=MODE_FP64, max_iter=10_000_000, nout=200, max_seconds=0.0, stream=None):
        """APT solve to err < tol (FP64 residual); returns PSSolveStats. Raises PSError otherwise."""
        st = PSSolveStats()
        rc = _lib.load().ps_stokes2d_apt_solve(ctypes.byref(self._fields), ctypes.byref(self._p), int(mode),
                                               float(tol), int(max_iter), int(nout), float(max_seconds),
                                               ctypes.byref(st), stream_handle(stream))
        if rc != 0:
            err = _lib.PSError(rc, _lib.last_error())
            err.stats = st
            raise err
        return st
