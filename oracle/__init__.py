"""CPU oracle of the GB300 stencil library -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper around ``oracle/ps_oracle.c`` (a plain-C + OpenMP restatement of
ParallelStencil.jl's FiniteDifferences macros and the example / miniapp kernels built
from them). Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use it, and only as the checker / the timed CPU reference; the product path
(``ps_gb300``) never imports it.

Arrays are numpy arrays in Julia layout: shape ``(nx, ny, nz)`` (or ``(nx, ny)``,
``(nx,)``), Fortran order, so ``A[ix, iy, iz]`` (0-based) is the reference's
``A[ix+1, iy+1, iz+1]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libps_oracle.so")
_SOURCES = [os.path.join(_HERE, "ps_oracle.c"), os.path.join(_HERE, "ps_oracle_body.h")]

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-O3 -fopenmp -ffp-contract=off) into oracle/_build."""
    os.makedirs(_BUILD, exist_ok=True)
    newest_src = max(os.path.getmtime(s) for s in _SOURCES)
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= newest_src:
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp, os.path.join(_HERE, "ps_oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
    return _lib


_SUFFIX = {np.dtype(np.float64): "_f64", np.dtype(np.float32): "_f32"}


def _real(dtype):
    return ctypes.c_double if np.dtype(dtype) == np.float64 else ctypes.c_float


def _n3(a: np.ndarray):
    s = list(a.shape) + [1] * (3 - a.ndim)
    return (ctypes.c_int64 * 3)(*s)


def _ptr(a: np.ndarray):
    if not a.flags.f_contiguous:
        raise ValueError("oracle arrays must be Fortran-contiguous (Julia layout)")
    return a.ctypes.data_as(ctypes.c_void_p)


def _fn(name: str, dtype):
    return getattr(lib(), name + _SUFFIX[np.dtype(dtype)])


def _check(rc: int, what: str):
    if rc != 0:
        raise ValueError(f"oracle {what} failed with status {rc}")


def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def fd_apply(kind: int, opdims: int, inn: int, ndims: int, lhs_inn: int, R: np.ndarray, A: np.ndarray) -> None:
    """``@<lhs>(R) = @<op>(A)`` in place on R."""
    f = _fn("orc_fd_apply", R.dtype)
    _check(f(kind, opdims, inn, ndims, lhs_inn, _ptr(R), _n3(R), _ptr(A), _n3(A)), "fd_apply")


def _box(n, lo, hi):
    lo = [0, 0, 0] if lo is None else list(lo)
    hi = list(n) if hi is None else list(hi)
    return (ctypes.c_int64 * 3)(*lo), (ctypes.c_int64 * 3)(*hi)


def memcopy3d(T2, T, Ci, lo=None, hi=None) -> None:
    n = _n3(T)
    l, h = _box(list(n), lo, hi)
    _check(_fn("orc_memcopy3d", T.dtype)(_ptr(T2), _ptr(T), _ptr(Ci), n, l, h), "memcopy3d")


def diffusion3d_step(form, T2, T, Ci, lam_arr, lam, dt, hx, hy, hz, lo=None, hi=None) -> None:
    """One diffusion step; (lo, hi) is the `@parallel` thread box (default: full grid)."""
    R = _real(T.dtype)
    n = _n3(T)
    l, h = _box(list(n), lo, hi)
    lam_p = _ptr(lam_arr) if lam_arr is not None else None
    _check(_fn("orc_diffusion3d_step", T.dtype)(int(form), _ptr(T2), _ptr(T), _ptr(Ci), lam_p, R(lam), R(dt),
                                                R(hx), R(hy), R(hz), n, l, h), "diffusion3d_step")


def acoustic3d_v(Vx, Vy, Vz, P, dt, rho, dx, dy, dz) -> None:
    R = _real(P.dtype)
    _check(_fn("orc_acoustic3d_v", P.dtype)(_ptr(Vx), _ptr(Vy), _ptr(Vz), _ptr(P), _n3(P), R(dt), R(rho), R(dx),
                                            R(dy), R(dz)), "acoustic3d_v")


def diffusion3d_adjoint_step(lamT, lamT2, T, Ci, lam, glam, dt, hx, hy, hz) -> None:
    """One reverse step of the flux-form diffusion step (lamT overwritten, glam accumulated)."""
    R = _real(T.dtype)
    _check(_fn("orc_diffusion3d_adjoint_step", T.dtype)(_ptr(lamT), _ptr(lamT2), _ptr(T), _ptr(Ci), _ptr(lam),
                                                        _ptr(glam), R(dt), R(hx), R(hy), R(hz), _n3(T)),
           "diffusion3d_adjoint_step")


def misfit_forward(T0, Ci, lam, dt, h, nt):
    """nt flux-form diffusion steps from T0 (the oracle's forward; returns all states)."""
    states = [np.asfortranarray(T0.copy())]
    for _ in range(nt):
        T2 = np.asfortranarray(states[-1].copy())
        diffusion3d_step(3, T2, states[-1], Ci, lam, 0.0, dt, *h)
        states.append(T2)
    return states


def misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt):
    """(loss, dL/dlam) of L = 0.5 ||T_nt - T_obs||^2 by the oracle's forward and reverse sweeps."""
    states = misfit_forward(T0, Ci, lam, dt, h, nt)
    r = states[-1] - T_obs
    loss = 0.5 * float(np.sum(r * r))
    lamT = np.asfortranarray(np.zeros_like(T0))
    lamT[1:-1, 1:-1, 1:-1] = r[1:-1, 1:-1, 1:-1]
    glam = np.asfortranarray(np.zeros_like(T0))
    buf = np.asfortranarray(np.zeros_like(T0))
    for n in range(nt - 1, -1, -1):
        diffusion3d_adjoint_step(buf, lamT, states[n], Ci, lam, glam, dt, *h)
        lamT, buf = buf, lamT
    return loss, glam


class Stokes2D:
    """The Stokes2D miniapp's arrays on the host and its kernels (miniapps/Stokes2D.jl:11-55)
    run by the oracle; same field names as ps_gb300.stokes.Stokes2D."""

    def __init__(self, nx, ny, dx, dy, Mus, Rog, Vdmp=4.0, Vsc=1.0, Ptsc=0.25, dtype=np.float64):
        z = lambda *s: np.asfortranarray(np.zeros(s, dtype=dtype))  # noqa: E731
        self.nx, self.ny, self.dtype = nx, ny, np.dtype(dtype)
        self.a = {"Pt": z(nx, ny), "dtauPt": z(nx, ny), "divV": z(nx, ny), "Vx": z(nx + 1, ny), "Vy": z(nx, ny + 1),
                  "txx": z(nx, ny), "tyy": z(nx, ny), "txy": z(nx - 1, ny - 1), "Rx": z(nx - 1, ny - 2),
                  "Ry": z(nx - 2, ny - 1), "dVxdtau": z(nx - 1, ny - 2), "dVydtau": z(nx - 2, ny - 1),
                  "dtauVx": z(nx - 1, ny - 2), "dtauVy": z(nx - 2, ny - 1),
                  "Mus": np.asfortranarray(Mus.astype(dtype)), "Rog": np.asfortranarray(Rog.astype(dtype))}
        self.dx, self.dy = dx, dy
        self.dampX, self.dampY = 1.0 - Vdmp / nx, 1.0 - Vdmp / ny
        self.Vsc, self.Ptsc = Vsc, Ptsc
        self.min_dxy2, self.max_nxy = min(dx, dy) ** 2, max(nx, ny)

    def _f(self, name):
        return _fn(name, self.dtype)

    def __getitem__(self, k):
        return self.a[k]

    def compute_timesteps(self):
        R, a = _real(self.dtype), self.a
        _check(self._f("orc_stokes2d_timesteps")(_ptr(a["dtauVx"]), _ptr(a["dtauVy"]), _ptr(a["dtauPt"]),
                                                 _ptr(a["Mus"]), ctypes.c_int64(self.nx), ctypes.c_int64(self.ny),
                                                 R(self.Vsc), R(self.Ptsc), R(self.min_dxy2),
                                                 ctypes.c_int64(self.max_nxy)), "stokes2d_timesteps")

    def step(self):
        """compute_P!, compute_τ!, compute_dV!, compute_V!, bc_y!(Vx), bc_x!(Vy) (Stokes2D.jl:111-116)."""
        R, a, i64 = _real(self.dtype), self.a, ctypes.c_int64
        nx, ny = i64(self.nx), i64(self.ny)
        _check(self._f("orc_stokes2d_P")(_ptr(a["divV"]), _ptr(a["Pt"]), _ptr(a["Vx"]), _ptr(a["Vy"]),
                                         _ptr(a["dtauPt"]), nx, ny, R(self.dx), R(self.dy)), "P")
        _check(self._f("orc_stokes2d_tau")(_ptr(a["divV"]), _ptr(a["txx"]), _ptr(a["tyy"]), _ptr(a["txy"]),
                                           _ptr(a["Vx"]), _ptr(a["Vy"]), _ptr(a["Mus"]), nx, ny, R(self.dx),
                                           R(self.dy)), "tau")
        _check(self._f("orc_stokes2d_dV")(_ptr(a["Rx"]), _ptr(a["Ry"]), _ptr(a["dVxdtau"]), _ptr(a["dVydtau"]),
                                          _ptr(a["Pt"]), _ptr(a["Rog"]), _ptr(a["txx"]), _ptr(a["tyy"]),
                                          _ptr(a["txy"]), nx, ny, R(self.dampX), R(self.dampY), R(self.dx),
                                          R(self.dy)), "dV")
        _check(self._f("orc_stokes2d_V")(_ptr(a["Vx"]), _ptr(a["Vy"]), _ptr(a["dVxdtau"]), _ptr(a["dVydtau"]),
                                         _ptr(a["dtauVx"]), _ptr(a["dtauVy"]), nx, ny), "V")
        _check(self._f("orc_bc_y2d")(_ptr(a["Vx"]), i64(self.nx + 1), ny), "bc_y")
        _check(self._f("orc_bc_x2d")(_ptr(a["Vy"]), nx, i64(self.ny + 1)), "bc_x")

    def err(self):
        """max(mean|Rx|, mean|Ry|, mean|∇V|) (Stokes2D.jl:119-120)."""
        m = [float(np.mean(np.abs(self.a[k]))) for k in ("Rx", "Ry", "divV")]
        return max(m), tuple(m)


class Stokes2DAPT:
    """The accelerated pseudo-transient Stokes2D iteration (pseudo-time steps from @maxloc(Mus))
    run by the oracle; same field names as ps_gb300.stokes.Stokes2DAPT. Coefficients are computed
    in FP64 from the field's own Mus values and rounded for FP32 fields."""

    SHAPES = {"Pt": (0, 0), "divV": (0, 0), "Vx": (1, 0), "Vy": (0, 1), "txx": (0, 0), "tyy": (0, 0),
              "txy": (-1, -1), "Rx": (-1, -2), "Ry": (-2, -1), "Must": (0, 0), "kP": (0, 0), "aT": (0, 0),
              "bT": (0, 0), "aTc": (-1, -1), "bTc": (-1, -1), "dtVx": (-1, -2), "dtVy": (-2, -1)}
    COEFFS = ("Must", "kP", "aT", "bT", "aTc", "bTc", "dtVx", "dtVy")

    def __init__(self, nx, ny, dx, dy, Mus, Rog, Re, r, Vpdt, max_lxy, dtype=np.float64):
        self.nx, self.ny, self.dtype = nx, ny, np.dtype(dtype)
        self.a = {k: np.asfortranarray(np.zeros((nx + e[0], ny + e[1]), dtype=dtype)) for k, e in self.SHAPES.items()}
        self.a["Mus"] = np.asfortranarray(Mus.astype(dtype))
        self.a["Rog"] = np.asfortranarray(Rog.astype(dtype))
        self._dx, self._dy = 1.0 / dx, 1.0 / dy
        c64 = {k: np.asfortranarray(np.zeros((nx + self.SHAPES[k][0], ny + self.SHAPES[k][1]))) for k in self.COEFFS}
        m64 = np.asfortranarray(self.a["Mus"].astype(np.float64))  # the field's own values, widened
        _check(lib().orc_stokes2d_apt_coeffs(*[_ptr(c64[k]) for k in self.COEFFS], _ptr(m64), ctypes.c_int64(nx),
                                             ctypes.c_int64(ny), ctypes.c_double(Vpdt), ctypes.c_double(Re),
                                             ctypes.c_double(r), ctypes.c_double(max_lxy)), "stokes2d_apt_coeffs")
        for k in self.COEFFS:
            self.a[k][...] = c64[k].astype(dtype)

    def __getitem__(self, k):
        return self.a[k]

    def step(self):
        R, a, i64 = _real(self.dtype), self.a, ctypes.c_int64
        names = ("Vx", "Vy", "Pt", "txx", "tyy", "txy", "divV", "Rx", "Ry", "kP", "aT", "bT", "aTc", "bTc", "dtVx",
                 "dtVy", "Rog")
        _check(_fn("orc_stokes2d_apt_step", self.dtype)(*[_ptr(a[k]) for k in names], i64(self.nx), i64(self.ny),
                                                          R(self._dx), R(self._dy)), "stokes2d_apt_step")

    def err(self):
        """max(mean|Rx|, mean|Ry|, mean|∇V|) of the last iteration (Stokes2D.jl:119-120)."""
        m = [float(np.mean(np.abs(self.a[k]))) for k in ("Rx", "Ry", "divV")]
        return max(m), tuple(m)

    def residual(self):
        """FP64 residual of the current state with the stresses at their steady state: returns
        max(mean|Rx|, mean|Ry|, mean|∇V|) and the arrays (FP64 fields only)."""
        if self.dtype != np.float64:
            raise ValueError("the residual is computed on FP64 fields")
        nx, ny = self.nx, self.ny
        out = {k: np.asfortranarray(np.zeros((nx + e[0], ny + e[1]))) for k, e in
               (("Rx", (-1, -2)), ("Ry", (-2, -1)), ("divV", (0, 0)), ("txx", (0, 0)), ("tyy", (0, 0)),
                ("txy", (-1, -1)))}
        a = self.a
        _check(lib().orc_stokes2d_apt_residual(*[_ptr(out[k]) for k in ("Rx", "Ry", "divV", "txx", "tyy", "txy")],
                                                 _ptr(a["Vx"]), _ptr(a["Vy"]), _ptr(a["Pt"]), _ptr(a["Mus"]),
                                                 _ptr(a["Rog"]), ctypes.c_int64(nx), ctypes.c_int64(ny),
                                                 ctypes.c_double(self._dx), ctypes.c_double(self._dy)),
               "stokes2d_apt_residual")
        m = [float(np.mean(np.abs(out[k]))) for k in ("Rx", "Ry", "divV")]
        return max(m), out


STOKES3D_SHAPES = {  # extents relative to (nx, ny, nz) = size(Pt) (miniapps/Stokes3D.jl:89-110)
    "Pt": (0, 0, 0), "dtauPt": (0, 0, 0), "divV": (0, 0, 0), "Vx": (1, 0, 0), "Vy": (0, 1, 0), "Vz": (0, 0, 1),
    "txx": (0, -2, -2), "tyy": (-2, 0, -2), "tzz": (-2, -2, 0), "txy": (-1, -1, -2), "txz": (-1, -2, -1),
    "tyz": (-2, -1, -1), "Rx": (-1, -2, -2), "Ry": (-2, -1, -2), "Rz": (-2, -2, -1), "dVxdtau": (-1, -2, -2),
    "dVydtau": (-2, -1, -2), "dVzdtau": (-2, -2, -1), "dtauVx": (-1, -2, -2), "dtauVy": (-2, -1, -2),
    "dtauVz": (-2, -2, -1), "Mus": (0, 0, 0), "Rog": (0, 0, 0)}


class Stokes3D:
    """The Stokes3D miniapp's arrays on the host and its kernels (miniapps/Stokes3D.jl:11-68) run by
    the oracle; same field names as ps_gb300.stokes3d.Stokes3D."""

    def __init__(self, nx, ny, nz, dx, dy, dz, Mus, Rog, Vdmp=4.0, Vsc=1.0, Ptsc=0.25, dtype=np.float64):
        n = (nx, ny, nz)
        self.n, self.dtype = n, np.dtype(dtype)
        self.a = {k: np.asfortranarray(np.zeros(tuple(m + o for m, o in zip(n, off)), dtype=dtype))
                  for k, off in STOKES3D_SHAPES.items() if k not in ("Mus", "Rog")}
        self.a["Mus"] = np.asfortranarray(Mus.astype(dtype))
        self.a["Rog"] = np.asfortranarray(Rog.astype(dtype))
        self.dx, self.dy, self.dz = dx, dy, dz
        self.damp = tuple(1.0 - Vdmp / m for m in n)
        self.Vsc, self.Ptsc = Vsc, Ptsc
        self.min_dxyz2, self.max_nxyz = min(dx, dy, dz) ** 2, max(n)

    def _f(self, name):
        return _fn(name, self.dtype)

    def __getitem__(self, k):
        return self.a[k]

    def compute_timesteps(self):
        R, a, i64 = _real(self.dtype), self.a, ctypes.c_int64
        _check(self._f("orc_stokes3d_timesteps")(_ptr(a["dtauVx"]), _ptr(a["dtauVy"]), _ptr(a["dtauVz"]),
                                                 _ptr(a["dtauPt"]), _ptr(a["Mus"]), *map(i64, self.n), R(self.Vsc),
                                                 R(self.Ptsc), R(self.min_dxyz2), i64(self.max_nxyz)), "timesteps")

    def compute_P(self):
        R, a, i64 = _real(self.dtype), self.a, ctypes.c_int64
        _check(self._f("orc_stokes3d_P")(_ptr(a["divV"]), _ptr(a["Pt"]), _ptr(a["Vx"]), _ptr(a["Vy"]), _ptr(a["Vz"]),
                                         _ptr(a["dtauPt"]), *map(i64, self.n), R(self.dx), R(self.dy), R(self.dz)),
               "P")

    def compute_tau(self):
        R, a, i64 = _real(self.dtype), self.a, ctypes.c_int64
        _check(self._f("orc_stokes3d_tau")(*[_ptr(a[k]) for k in ("divV", "txx", "tyy", "tzz", "txy", "txz", "tyz",
                                                                   "Vx", "Vy", "Vz", "Mus")],
                                           *map(i64, self.n), R(self.dx), R(self.dy), R(self.dz)), "tau")

    def compute_dV(self):
        R, a, i64 = _real(self.dtype), self.a, ctypes.c_int64
        _check(self._f("orc_stokes3d_dV")(*[_ptr(a[k]) for k in ("Rx", "Ry", "Rz", "dVxdtau", "dVydtau", "dVzdtau",
                                                                  "Pt", "Rog", "txx", "tyy", "tzz", "txy", "txz",
                                                                  "tyz")],
                                          *map(i64, self.n), *map(R, self.damp), R(self.dx), R(self.dy), R(self.dz)),
               "dV")

    def compute_V(self):
        a, i64 = self.a, ctypes.c_int64
        _check(self._f("orc_stokes3d_V")(*[_ptr(a[k]) for k in ("Vx", "Vy", "Vz", "dVxdtau", "dVydtau", "dVzdtau",
                                                                 "dtauVx", "dtauVy", "dtauVz")],
                                         *map(i64, self.n)), "V")

    def bc(self, which, name):
        A = self.a[name]
        _check(self._f("orc_bc_" + which + "3d")(_ptr(A), *map(ctypes.c_int64, A.shape)), "bc")

    def step(self):
        """One PT iteration as the miniapp's loop body (Stokes3D.jl:134-143)."""
        self.compute_P()
        self.compute_tau()
        self.compute_dV()
        self.compute_V()
        for which, name in (("x", "Vy"), ("x", "Vz"), ("y", "Vx"), ("y", "Vz"), ("z", "Vx"), ("z", "Vy")):
            self.bc(which, name)

    def err(self):
        """max(mean|Rx|, mean|Ry|, mean|Rz|, mean|∇V|) (Stokes3D.jl:145-146)."""
        m = [float(np.mean(np.abs(self.a[k]))) for k in ("Rx", "Ry", "Rz", "divV")]
        return max(m), tuple(m)


def acoustic3d_p(P, Vx, Vy, Vz, dt, k, dx, dy, dz) -> None:
    R = _real(P.dtype)
    _check(_fn("orc_acoustic3d_p", P.dtype)(_ptr(P), _ptr(Vx), _ptr(Vy), _ptr(Vz), _n3(P), R(dt), R(k), R(dx),
                                            R(dy), R(dz)), "acoustic3d_p")
