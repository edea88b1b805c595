"""Generate the known-answer fixtures that pin the oracle and the GPU kernels.

    python tests/golden/make_golden.py        # rewrites tests/golden/golden.npz + golden.json

Every expected array is computed with numpy *broadcasting*, restating the expected-value
expressions of the reference's own tests (which compare each `@parallel` kernel against Julia
broadcasting with exact `==`):
  - every FD macro: test/test_FiniteDifferences1D.jl:51-88, test/test_FiniteDifferences2D.jl:63-129,
    test/test_FiniteDifferences3D.jl:65-185 (sizes (9,), (9,7), (9,7,8); staggered field
    sizes from src/ParallelKernel/FieldAllocators.jl:584-608);
  - masks leaving boundary values untouched: the "apply masks" testsets of the same files;
  - diffusion kernels: test/test_parallel.jl:411-434 (on-the-fly, 32x8x8) and the memopt
    diffusion testsets :521-601, :1018-1036 ((32,8,8) and (33,7,8), unit scalars, inputs
    (ix + (iy-1)nx + (iz-1)nx ny)^3);
  - the Diffusion3D test project (test/test_projects/Diffusion3D/src/backends/diffusion3D.jl:
    8^3, 3 steps), whose kernel is examples/diffusion3D_novis_noperf.jl:10-13.
Julia's `@rand` stream cannot be reproduced, so random inputs use numpy's seeded generator;
they are stored in the fixture next to the expected output. Float32 variants evaluate the same
expressions in float32 (the reference's literal typing casts 0.5 etc. to Float32).
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# Field size templates relative to the grid size (FieldAllocators.jl:584-608, padding=false)
FIELD3 = {
    "A": (-2, -2, -2), "Ax": (-1, -2, -2), "Ay": (-2, -1, -2), "Az": (-2, -2, -1), "Axy": (-1, -1, -2),
    "Axz": (-1, -2, -1), "Ayz": (-2, -1, -1), "Axyz": (-1, -1, -1), "Axyzz": (-1, -1, 0), "Axyyz": (-1, 0, -1),
    "Axxyz": (0, -1, -1), "Axx": (0, -2, -2), "Ayy": (-2, 0, -2), "Azz": (-2, -2, 0), "Axxyy": (0, 0, -2),
    "Axxzz": (0, -2, 0), "Ayyzz": (-2, 0, 0), "Axyyzz": (-1, 0, 0), "Axxyzz": (0, -1, 0), "Axxyyz": (0, 0, -1),
    "Axxyyzz": (0, 0, 0),
}
FIELD2 = {"A": (-2, -2), "Ax": (-1, -2), "Ay": (-2, -1), "Axy": (-1, -1), "Axx": (0, -2), "Ayy": (-2, 0),
          "Axyy": (-1, 0), "Axxy": (0, -1), "Axxyy": (0, 0)}
FIELD1 = {"A": (-2,), "Ax": (-1,), "Axx": (0,)}

I = slice(1, -1)  # 2:end-1
F = slice(1, None)  # 2:end
L = slice(None, -1)  # 1:end-1
A_ = slice(None)  # :
F2 = slice(2, None)  # 3:end
L2 = slice(None, -2)  # 1:end-2


def jl_max(a, b):
    return np.where(np.isnan(a) | np.isnan(b), a - b, np.where(np.signbit(a - b), b, a))


def jl_min(a, b):
    return np.where(np.isnan(a) | np.isnan(b), a - b, np.where(np.signbit(a - b), a, b))


def fd3_cases(f, dt):
    """(statement, input field, expected R = IField) for every 3-D macro."""
    h, q, one = dt(0.5), dt(0.25), dt(1)
    c = []
    c += [("@all(R) = @d_xa(A)", "Ax", f["Ax"][F, :, :] - f["Ax"][L, :, :]),
          ("@all(R) = @d_ya(A)", "Ay", f["Ay"][:, F, :] - f["Ay"][:, L, :]),
          ("@all(R) = @d_za(A)", "Az", f["Az"][:, :, F] - f["Az"][:, :, L]),
          ("@all(R) = @d_xi(A)", "Axyyzz", f["Axyyzz"][F, I, I] - f["Axyyzz"][L, I, I]),
          ("@all(R) = @d_yi(A)", "Axxyzz", f["Axxyzz"][I, F, I] - f["Axxyzz"][I, L, I]),
          ("@all(R) = @d_zi(A)", "Axxyyz", f["Axxyyz"][I, I, F] - f["Axxyyz"][I, I, L])]
    B = f["Axxyyzz"]
    c += [("@all(R) = @d2_xi(A)", "Axxyyzz", (B[F2, I, I] - B[I, I, I]) - (B[I, I, I] - B[L2, I, I])),
          ("@all(R) = @d2_yi(A)", "Axxyyzz", (B[I, F2, I] - B[I, I, I]) - (B[I, I, I] - B[I, L2, I])),
          ("@all(R) = @d2_zi(A)", "Axxyyzz", (B[I, I, F2] - B[I, I, I]) - (B[I, I, I] - B[I, I, L2]))]
    c += [("@all(R) = @all(A)", "A", f["A"].copy()), ("@all(R) = @inn(A)", "Axxyyzz", B[I, I, I]),
          ("@all(R) = @inn_x(A)", "Axx", f["Axx"][I, :, :]), ("@all(R) = @inn_y(A)", "Ayy", f["Ayy"][:, I, :]),
          ("@all(R) = @inn_z(A)", "Azz", f["Azz"][:, :, I]), ("@all(R) = @inn_xy(A)", "Axxyy", f["Axxyy"][I, I, :]),
          ("@all(R) = @inn_xz(A)", "Axxzz", f["Axxzz"][I, :, I]),
          ("@all(R) = @inn_yz(A)", "Ayyzz", f["Ayyzz"][:, I, I])]
    X = f["Axyz"]
    corners8 = [X[L, L, L], X[F, L, L], X[L, F, L], X[F, F, L], X[L, L, F], X[F, L, F], X[L, F, F], X[F, F, F]]
    s = corners8[0]
    for v in corners8[1:]:
        s = s + v
    c.append(("@all(R) = @av(A)", "Axyz", s * dt(0.125)))
    c += [("@all(R) = @av_xa(A)", "Ax", (f["Ax"][F, :, :] + f["Ax"][L, :, :]) * h),
          ("@all(R) = @av_ya(A)", "Ay", (f["Ay"][:, F, :] + f["Ay"][:, L, :]) * h),
          ("@all(R) = @av_za(A)", "Az", (f["Az"][:, :, F] + f["Az"][:, :, L]) * h),
          ("@all(R) = @av_xi(A)", "Axyyzz", (f["Axyyzz"][F, I, I] + f["Axyyzz"][L, I, I]) * h),
          ("@all(R) = @av_yi(A)", "Axxyzz", (f["Axxyzz"][I, F, I] + f["Axxyzz"][I, L, I]) * h),
          ("@all(R) = @av_zi(A)", "Axxyyz", (f["Axxyyz"][I, I, F] + f["Axxyyz"][I, I, L]) * h)]

    def four(Y, a, b, cc, d):
        return ((Y[a] + Y[b]) + Y[cc]) + Y[d]

    Axy, Axz, Ayz = f["Axy"], f["Axz"], f["Ayz"]
    Axyzz, Axyyz, Axxyz = f["Axyzz"], f["Axyyz"], f["Axxyz"]
    quad = {
        "xya": (Axy, "Axy", (L, L, A_), (F, L, A_), (L, F, A_), (F, F, A_)),
        "xza": (Axz, "Axz", (L, A_, L), (F, A_, L), (L, A_, F), (F, A_, F)),
        "yza": (Ayz, "Ayz", (A_, L, L), (A_, F, L), (A_, L, F), (A_, F, F)),
        "xyi": (Axyzz, "Axyzz", (L, L, I), (F, L, I), (L, F, I), (F, F, I)),
        "xzi": (Axyyz, "Axyyz", (L, I, L), (F, I, L), (L, I, F), (F, I, F)),
        "yzi": (Axxyz, "Axxyz", (I, L, L), (I, F, L), (I, L, F), (I, F, F)),
    }
    for k, (Y, nm, a, b, cc, d) in quad.items():
        c.append((f"@all(R) = @av_{k}(A)", nm, four(Y, a, b, cc, d) * q))
    # harmonic averages: k ./ (1 ./a .+ 1 ./b ...), k a power of two (== inv(sum)*k exactly)
    inv = [one / v for v in corners8]
    s = inv[0]
    for v in inv[1:]:
        s = s + v
    c.append(("@all(R) = @harm(A)", "Axyz", dt(8) / s))
    pairs = {"xa": ("Ax", (F, A_, A_), (L, A_, A_)), "ya": ("Ay", (A_, F, A_), (A_, L, A_)),
             "za": ("Az", (A_, A_, F), (A_, A_, L)), "xi": ("Axyyzz", (F, I, I), (L, I, I)),
             "yi": ("Axxyzz", (I, F, I), (I, L, I)), "zi": ("Axxyyz", (I, I, F), (I, I, L))}
    for k, (nm, a, b) in pairs.items():
        Y = f[nm]
        c.append((f"@all(R) = @harm_{k}(A)", nm, dt(2) / (one / Y[b] + one / Y[a])))
    for k, (Y, nm, a, b, cc, d) in quad.items():
        c.append((f"@all(R) = @harm_{k}(A)", nm, dt(4) / (((one / Y[a] + one / Y[b]) + one / Y[cc]) + one / Y[d])))
    mx = jl_max(jl_max(jl_max(jl_max(jl_max(jl_max(B[L2, I, I], B[F2, I, I]), B[I, I, I]), B[I, L2, I]), B[I, F2, I]),
                       B[I, I, L2]), B[I, I, F2])
    mn = jl_min(jl_min(jl_min(jl_min(jl_min(jl_min(B[L2, I, I], B[F2, I, I]), B[I, I, I]), B[I, L2, I]), B[I, F2, I]),
                       B[I, I, L2]), B[I, I, F2])
    c += [("@all(R) = @maxloc(A)", "Axxyyzz", mx), ("@all(R) = @minloc(A)", "Axxyyzz", mn)]
    return c


def fd3_mask_cases(f):
    """`@inn(Rxxyyzz) = ...`: inner values set, boundary values untouched (= 0)."""
    B = f["Axxyyzz"]
    out = []
    for stmt, nm, inner in [("@inn(R) = @all(A)", "A", f["A"]), ("@inn(R) = @inn(A)", "Axxyyzz", B[I, I, I]),
                            ("@inn(R) = @d_xa(A)", "Ax", f["Ax"][F, :, :] - f["Ax"][L, :, :]),
                            ("@inn(R) = @d_yi(A)", "Axxyzz", f["Axxyzz"][I, F, I] - f["Axxyzz"][I, L, I]),
                            ("@inn(R) = @d2_yi(A)", "Axxyyzz",
                             (B[I, F2, I] - B[I, I, I]) - (B[I, I, I] - B[I, L2, I]))]:
        R = np.zeros_like(B)
        R[I, I, I] = inner
        out.append((stmt, nm, R))
    return out


def fd2_cases(f, dt):
    h, q, one = dt(0.5), dt(0.25), dt(1)
    B = f["Axxyy"]
    c = [("@all(R) = @d_xa(A)", "Ax", f["Ax"][F, :] - f["Ax"][L, :]),
         ("@all(R) = @d_ya(A)", "Ay", f["Ay"][:, F] - f["Ay"][:, L]),
         ("@all(R) = @d_xi(A)", "Axyy", f["Axyy"][F, I] - f["Axyy"][L, I]),
         ("@all(R) = @d_yi(A)", "Axxy", f["Axxy"][I, F] - f["Axxy"][I, L]),
         ("@all(R) = @d2_xa(A)", "Axx", (f["Axx"][F2, :] - f["Axx"][I, :]) - (f["Axx"][I, :] - f["Axx"][L2, :])),
         ("@all(R) = @d2_ya(A)", "Ayy", (f["Ayy"][:, F2] - f["Ayy"][:, I]) - (f["Ayy"][:, I] - f["Ayy"][:, L2])),
         ("@all(R) = @d2_xi(A)", "Axxyy", (B[F2, I] - B[I, I]) - (B[I, I] - B[L2, I])),
         ("@all(R) = @d2_yi(A)", "Axxyy", (B[I, F2] - B[I, I]) - (B[I, I] - B[I, L2])),
         ("@all(R) = @all(A)", "A", f["A"].copy()), ("@all(R) = @inn(A)", "Axxyy", B[I, I]),
         ("@all(R) = @inn_x(A)", "Axx", f["Axx"][I, :]), ("@all(R) = @inn_y(A)", "Ayy", f["Ayy"][:, I])]
    Y = f["Axy"]
    c.append(("@all(R) = @av(A)", "Axy", (((Y[L, L] + Y[F, L]) + Y[L, F]) + Y[F, F]) * q))
    c += [("@all(R) = @av_xa(A)", "Ax", (f["Ax"][F, :] + f["Ax"][L, :]) * h),
          ("@all(R) = @av_ya(A)", "Ay", (f["Ay"][:, F] + f["Ay"][:, L]) * h),
          ("@all(R) = @av_xi(A)", "Axyy", (f["Axyy"][F, I] + f["Axyy"][L, I]) * h),
          ("@all(R) = @av_yi(A)", "Axxy", (f["Axxy"][I, F] + f["Axxy"][I, L]) * h)]
    c.append(("@all(R) = @harm(A)", "Axy", dt(4) / (((one / Y[L, L] + one / Y[F, L]) + one / Y[L, F]) + one / Y[F, F])))
    c += [("@all(R) = @harm_xa(A)", "Ax", dt(2) / (one / f["Ax"][L, :] + one / f["Ax"][F, :])),
          ("@all(R) = @harm_ya(A)", "Ay", dt(2) / (one / f["Ay"][:, L] + one / f["Ay"][:, F])),
          ("@all(R) = @harm_xi(A)", "Axyy", dt(2) / (one / f["Axyy"][L, I] + one / f["Axyy"][F, I])),
          ("@all(R) = @harm_yi(A)", "Axxy", dt(2) / (one / f["Axxy"][I, L] + one / f["Axxy"][I, F]))]
    c.append(("@all(R) = @maxloc(A)", "Axxyy",
              jl_max(jl_max(jl_max(jl_max(B[L2, I], B[F2, I]), B[I, I]), B[I, L2]), B[I, F2])))
    c.append(("@all(R) = @minloc(A)", "Axxyy",
              jl_min(jl_min(jl_min(jl_min(B[L2, I], B[F2, I]), B[I, I]), B[I, L2]), B[I, F2])))
    for stmt, nm, inner in [("@inn(R) = @all(A)", "A", f["A"]), ("@inn(R) = @inn(A)", "Axxyy", B[I, I]),
                            ("@inn(R) = @d_xa(A)", "Ax", f["Ax"][F, :] - f["Ax"][L, :]),
                            ("@inn(R) = @d_yi(A)", "Axxy", f["Axxy"][I, F] - f["Axxy"][I, L]),
                            ("@inn(R) = @d2_yi(A)", "Axxyy", (B[I, F2] - B[I, I]) - (B[I, I] - B[I, L2]))]:
        R = np.zeros_like(B)
        R[I, I] = inner
        c.append((stmt, nm, R))
    return c


def fd1_cases(f, dt):
    h, one = dt(0.5), dt(1)
    B, Ax = f["Axx"], f["Ax"]
    c = [("@all(R) = @d(A)", "Ax", Ax[F] - Ax[L]), ("@all(R) = @d2(A)", "Axx", (B[F2] - B[I]) - (B[I] - B[L2])),
         ("@all(R) = @all(A)", "A", f["A"].copy()), ("@all(R) = @inn(A)", "Axx", B[I]),
         ("@all(R) = @av(A)", "Ax", (Ax[L] + Ax[F]) * h), ("@all(R) = @harm(A)", "Ax", dt(2) / (one / Ax[L] + one / Ax[F])),
         ("@all(R) = @maxloc(A)", "Axx", jl_max(jl_max(B[F2], B[I]), B[L2])),
         ("@all(R) = @minloc(A)", "Axx", jl_min(jl_min(B[F2], B[I]), B[L2]))]
    for stmt, nm, inner in [("@inn(R) = @all(A)", "A", f["A"]), ("@inn(R) = @inn(A)", "Axx", B[I]),
                            ("@inn(R) = @d(A)", "Ax", Ax[F] - Ax[L]),
                            ("@inn(R) = @d2(A)", "Axx", (B[F2] - B[I]) - (B[I] - B[L2]))]:
        R = np.zeros_like(B)
        R[I] = inner
        c.append((stmt, nm, R))
    return c


def fields(templates, grid, rng, dt):
    return {k: np.asfortranarray(rng.random(tuple(g + d for g, d in zip(grid, v))).astype(dt))
            for k, v in templates.items()}


def index_cubed(n, dt):
    nx, ny, nz = n
    ix, iy, iz = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    return np.asfortranarray(((ix + (iy - 1) * nx + (iz - 1) * nx * ny).astype(np.float64) ** 3).astype(dt))


def diffusion_ref(T, lam, dt_, _dx, _dy, _dz, Ci):
    """test/test_parallel.jl:427-431 (the expected value of every diffusion testset)."""
    T2 = np.zeros_like(T)
    c = T[I, I, I]
    d2x = (T[F2, I, I] - c) - (c - T[L2, I, I])
    d2y = (T[I, F2, I] - c) - (c - T[I, L2, I])
    d2z = (T[I, I, F2] - c) - (c - T[I, I, L2])
    T2[I, I, I] = c + dt_ * ((lam * Ci[I, I, I]) * ((d2x * (_dx * _dx) + d2y * (_dy * _dy)) + d2z * (_dz * _dz)))
    return T2


def diffusion_project(dt):
    """test/test_projects/Diffusion3D/src/backends/diffusion3D.jl: 8^3, 3 steps, /dx^2 form."""
    lam, cp_min = dt(1.0), dt(1.0)
    lx = ly = lz = 10.0
    nx = ny = nz = 8
    dx, dy, dz = lx / (nx - 1), ly / (ny - 1), lz / (nz - 1)
    ix, iy, iz = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    X, Y, Zc = (ix - 1) * dx, (iy - 1) * dy, (iz - 1) * dz
    Ci = 1.0 / (cp_min + (5 * np.exp(-((X - lx / 1.5)) ** 2 - ((Y - ly / 2)) ** 2 - ((Zc - lz / 1.5)) ** 2)
                          + 5 * np.exp(-((X - lx / 3.0)) ** 2 - ((Y - ly / 2)) ** 2 - ((Zc - lz / 1.5)) ** 2)))
    T = (100 * np.exp(-((X - lx / 2) / 2) ** 2 - ((Y - ly / 2) / 2) ** 2 - ((Zc - lz / 3.0) / 2) ** 2)
         + 50 * np.exp(-((X - lx / 2) / 2) ** 2 - ((Y - ly / 2) / 2) ** 2 - ((Zc - lz / 1.5) / 2) ** 2))
    Ci, T = np.asfortranarray(Ci.astype(dt)), np.asfortranarray(T.astype(dt))
    T0, Ci0 = T.copy(), Ci.copy()
    T2 = T.copy()
    dxs, dys, dzs = dt(dx), dt(dy), dt(dz)
    dt_ = dt(min(dx ** 2, dy ** 2, dz ** 2) * 1.0 / 1.0 / 8.1)
    for _ in range(3):
        c = T[I, I, I]
        d2x = (T[F2, I, I] - c) - (c - T[L2, I, I])
        d2y = (T[I, F2, I] - c) - (c - T[I, L2, I])
        d2z = (T[I, I, F2] - c) - (c - T[I, I, L2])
        s = (d2x / (dxs * dxs) + d2y / (dys * dys)) + d2z / (dzs * dzs)
        T2[I, I, I] = c + dt_ * ((lam * Ci[I, I, I]) * s)
        T, T2 = T2, T
    return dict(T0=T0, Ci=Ci0, T=T, scalars=np.array([lam, dt_, dxs, dys, dzs], dtype=dt))


def stokes2d_numpy(nx, ny, iters, dt):
    """miniapps/Stokes2D.jl:11-55, 93-116 restated with numpy broadcasting (lx = ly = 10,
    μs0 = 1, μsi = 0.1, ρgi = 1, Vdmp = 4, Vsc = 1, Ptsc = 1/4)."""
    lx = ly = 10.0
    dx, dy = lx / (nx - 1), ly / (ny - 1)
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    radc = (ix * dx - 0.5 * lx) ** 2 + (iy * dy - 0.5 * ly) ** 2
    Mus = np.ones((nx, ny))
    Rog = np.zeros((nx, ny))
    Mus[radc < 1.0] = 0.1
    Rog[radc < 1.0] = 1.0
    Mus, Rog = Mus.astype(dt), Rog.astype(dt)
    c = lambda v: dt(v)  # noqa: E731 - literal typing
    dxs, dys = c(dx), c(dy)
    dampX, dampY = c(1.0 - 4.0 / nx), c(1.0 - 4.0 / ny)
    Vsc, Ptsc, min_dxy2, max_nxy = c(1.0), c(0.25), c(min(dx, dy) ** 2), c(max(nx, ny))
    d_xa = lambda A: A[1:, :] - A[:-1, :]  # noqa: E731
    d_ya = lambda A: A[:, 1:] - A[:, :-1]  # noqa: E731
    d_xi = lambda A: A[1:, 1:-1] - A[:-1, 1:-1]  # noqa: E731
    d_yi = lambda A: A[1:-1, 1:] - A[1:-1, :-1]  # noqa: E731
    av = lambda A: (((A[:-1, :-1] + A[1:, :-1]) + A[:-1, 1:]) + A[1:, 1:]) * c(0.25)  # noqa: E731
    av_xi = lambda A: (A[:-1, 1:-1] + A[1:, 1:-1]) * c(0.5)  # noqa: E731
    av_yi = lambda A: (A[1:-1, :-1] + A[1:-1, 1:]) * c(0.5)  # noqa: E731
    dtauVx = ((Vsc * min_dxy2) / av_xi(Mus)) / c(4.1)
    dtauVy = ((Vsc * min_dxy2) / av_yi(Mus)) / c(4.1)
    dtauPt = ((Ptsc * c(4.1)) * Mus) / max_nxy
    Pt = np.zeros((nx, ny), dt)
    Vx, Vy = np.zeros((nx + 1, ny), dt), np.zeros((nx, ny + 1), dt)
    dVxdtau, dVydtau = np.zeros((nx - 1, ny - 2), dt), np.zeros((nx - 2, ny - 1), dt)
    for _ in range(iters):
        divV = d_xa(Vx) / dxs + d_ya(Vy) / dys
        Pt = Pt - dtauPt * divV
        txx = (c(2.0) * Mus) * (d_xa(Vx) / dxs - (c(1.0) / c(3.0)) * divV)
        tyy = (c(2.0) * Mus) * (d_ya(Vy) / dys - (c(1.0) / c(3.0)) * divV)
        txy = (c(2.0) * av(Mus)) * (c(0.5) * (d_yi(Vx) / dys + d_xi(Vy) / dxs))
        Rx = (d_xi(txx) / dxs + d_ya(txy) / dys) - d_xi(Pt) / dxs
        Ry = ((d_yi(tyy) / dys + d_xa(txy) / dxs) - d_yi(Pt) / dys) + av_yi(Rog)
        dVxdtau = dampX * dVxdtau + Rx
        dVydtau = dampY * dVydtau + Ry
        Vx[1:-1, 1:-1] = Vx[1:-1, 1:-1] + dtauVx * dVxdtau
        Vy[1:-1, 1:-1] = Vy[1:-1, 1:-1] + dtauVy * dVydtau
        Vx[:, 0], Vx[:, -1] = Vx[:, 1], Vx[:, -2]
        Vy[0, :], Vy[-1, :] = Vy[1, :], Vy[-2, :]
    out = dict(Mus=Mus, Rog=Rog, Pt=Pt, Vx=Vx, Vy=Vy, divV=divV, txx=txx, tyy=tyy, txy=txy, Rx=Rx, Ry=Ry,
               dVxdtau=dVxdtau, dVydtau=dVydtau, dtauVx=dtauVx, dtauVy=dtauVy, dtauPt=dtauPt)
    return {k: np.asfortranarray(v) for k, v in out.items()}


def stokes3d_numpy(nx, ny, nz, iters, dt):
    """miniapps/Stokes3D.jl:11-68, 116-143 restated with numpy broadcasting (lx = ly = lz = 10,
    μs0 = 1, μsi = 0.1, ρgi = 1, Vdmp = 4, Vsc = 1, Ptsc = 1/4, inclusion Radc <= 1)."""
    lx = 10.0
    dx, dy, dz = lx / (nx - 1), lx / (ny - 1), lx / (nz - 1)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    radc = (ix * dx - 0.5 * lx) ** 2 + (iy * dy - 0.5 * lx) ** 2 + (iz * dz - 0.5 * lx) ** 2
    Mus = np.ones((nx, ny, nz))
    Rog = np.zeros((nx, ny, nz))
    Mus[radc <= 1.0] = 0.1
    Rog[radc <= 1.0] = 1.0
    Mus, Rog = Mus.astype(dt), Rog.astype(dt)
    c = lambda v: dt(v)  # noqa: E731 - literal typing
    dxs, dys, dzs = c(dx), c(dy), c(dz)
    dampX, dampY, dampZ = c(1.0 - 4.0 / nx), c(1.0 - 4.0 / ny), c(1.0 - 4.0 / nz)
    Vsc, Ptsc, min_dxyz2, max_nxyz = c(1.0), c(0.25), c(min(dx, dy, dz) ** 2), c(max(nx, ny, nz))
    d_xa = lambda A: A[1:, :, :] - A[:-1, :, :]  # noqa: E731
    d_ya = lambda A: A[:, 1:, :] - A[:, :-1, :]  # noqa: E731
    d_za = lambda A: A[:, :, 1:] - A[:, :, :-1]  # noqa: E731
    d_xi = lambda A: A[1:, 1:-1, 1:-1] - A[:-1, 1:-1, 1:-1]  # noqa: E731
    d_yi = lambda A: A[1:-1, 1:, 1:-1] - A[1:-1, :-1, 1:-1]  # noqa: E731
    d_zi = lambda A: A[1:-1, 1:-1, 1:] - A[1:-1, 1:-1, :-1]  # noqa: E731
    inn_yz = lambda A: A[:, 1:-1, 1:-1]  # noqa: E731
    inn_xz = lambda A: A[1:-1, :, 1:-1]  # noqa: E731
    inn_xy = lambda A: A[1:-1, 1:-1, :]  # noqa: E731
    av_xi = lambda A: (A[:-1, 1:-1, 1:-1] + A[1:, 1:-1, 1:-1]) * c(0.5)  # noqa: E731
    av_yi = lambda A: (A[1:-1, :-1, 1:-1] + A[1:-1, 1:, 1:-1]) * c(0.5)  # noqa: E731
    av_zi = lambda A: (A[1:-1, 1:-1, :-1] + A[1:-1, 1:-1, 1:]) * c(0.5)  # noqa: E731
    av_xyi = lambda A: (((A[:-1, :-1, 1:-1] + A[1:, :-1, 1:-1]) + A[:-1, 1:, 1:-1]) + A[1:, 1:, 1:-1]) * c(0.25)  # noqa: E731
    av_xzi = lambda A: (((A[:-1, 1:-1, :-1] + A[1:, 1:-1, :-1]) + A[:-1, 1:-1, 1:]) + A[1:, 1:-1, 1:]) * c(0.25)  # noqa: E731
    av_yzi = lambda A: (((A[1:-1, :-1, :-1] + A[1:-1, 1:, :-1]) + A[1:-1, :-1, 1:]) + A[1:-1, 1:, 1:]) * c(0.25)  # noqa: E731
    third = c(1.0) / c(3.0)
    dtauVx = ((Vsc * min_dxyz2) / av_xi(Mus)) / c(6.1)
    dtauVy = ((Vsc * min_dxyz2) / av_yi(Mus)) / c(6.1)
    dtauVz = ((Vsc * min_dxyz2) / av_zi(Mus)) / c(6.1)
    dtauPt = ((Ptsc * c(6.1)) * Mus) / max_nxyz
    Pt = np.zeros((nx, ny, nz), dt)
    Vx, Vy, Vz = np.zeros((nx + 1, ny, nz), dt), np.zeros((nx, ny + 1, nz), dt), np.zeros((nx, ny, nz + 1), dt)
    dVxdtau = np.zeros((nx - 1, ny - 2, nz - 2), dt)
    dVydtau = np.zeros((nx - 2, ny - 1, nz - 2), dt)
    dVzdtau = np.zeros((nx - 2, ny - 2, nz - 1), dt)
    for _ in range(iters):
        divV = (d_xa(Vx) / dxs + d_ya(Vy) / dys) + d_za(Vz) / dzs
        Pt = Pt - dtauPt * divV
        txx = (c(2.0) * inn_yz(Mus)) * (d_xi(Vx) / dxs - third * inn_yz(divV))
        tyy = (c(2.0) * inn_xz(Mus)) * (d_yi(Vy) / dys - third * inn_xz(divV))
        tzz = (c(2.0) * inn_xy(Mus)) * (d_zi(Vz) / dzs - third * inn_xy(divV))
        txy = (c(2.0) * av_xyi(Mus)) * (c(0.5) * (d_yi(Vx) / dys + d_xi(Vy) / dxs))
        txz = (c(2.0) * av_xzi(Mus)) * (c(0.5) * (d_zi(Vx) / dzs + d_xi(Vz) / dxs))
        tyz = (c(2.0) * av_yzi(Mus)) * (c(0.5) * (d_zi(Vy) / dzs + d_yi(Vz) / dys))
        Rx = ((d_xa(txx) / dxs + d_ya(txy) / dys) + d_za(txz) / dzs) - d_xi(Pt) / dxs
        Ry = ((d_ya(tyy) / dys + d_xa(txy) / dxs) + d_za(tyz) / dzs) - d_yi(Pt) / dys
        Rz = (((d_za(tzz) / dzs + d_xa(txz) / dxs) + d_ya(tyz) / dys) - d_zi(Pt) / dzs) + av_zi(Rog)
        dVxdtau = dampX * dVxdtau + Rx
        dVydtau = dampY * dVydtau + Ry
        dVzdtau = dampZ * dVzdtau + Rz
        Vx[1:-1, 1:-1, 1:-1] = Vx[1:-1, 1:-1, 1:-1] + dtauVx * dVxdtau
        Vy[1:-1, 1:-1, 1:-1] = Vy[1:-1, 1:-1, 1:-1] + dtauVy * dVydtau
        Vz[1:-1, 1:-1, 1:-1] = Vz[1:-1, 1:-1, 1:-1] + dtauVz * dVzdtau
        Vy[0, :, :], Vy[-1, :, :] = Vy[1, :, :], Vy[-2, :, :]
        Vz[0, :, :], Vz[-1, :, :] = Vz[1, :, :], Vz[-2, :, :]
        Vx[:, 0, :], Vx[:, -1, :] = Vx[:, 1, :], Vx[:, -2, :]
        Vz[:, 0, :], Vz[:, -1, :] = Vz[:, 1, :], Vz[:, -2, :]
        Vx[:, :, 0], Vx[:, :, -1] = Vx[:, :, 1], Vx[:, :, -2]
        Vy[:, :, 0], Vy[:, :, -1] = Vy[:, :, 1], Vy[:, :, -2]
    out = dict(Mus=Mus, Rog=Rog, Pt=Pt, Vx=Vx, Vy=Vy, Vz=Vz, divV=divV, txx=txx, tyy=tyy, tzz=tzz, txy=txy,
               txz=txz, tyz=tyz, Rx=Rx, Ry=Ry, Rz=Rz, dVxdtau=dVxdtau, dVydtau=dVydtau, dVzdtau=dVzdtau,
               dtauVx=dtauVx, dtauVy=dtauVy, dtauVz=dtauVz, dtauPt=dtauPt)
    return {k: np.asfortranarray(v) for k, v in out.items()}


def main():
    arrays, meta = {}, {"fd": [], "diffusion": [], "stokes2d": [], "stokes3d": []}
    for dtn, dt in (("f64", np.float64), ("f32", np.float32)):
        for nd, (templates, grid, gen) in {3: (FIELD3, (9, 7, 8), None), 2: (FIELD2, (9, 7), None),
                                            1: (FIELD1, (9,), None)}.items():
            rng = np.random.default_rng(1000 + nd)
            f = fields(templates, grid, rng, dt)
            cases = fd3_cases(f, dt) + fd3_mask_cases(f) if nd == 3 else fd2_cases(f, dt) if nd == 2 else fd1_cases(f, dt)
            for i, (stmt, inp, R) in enumerate(cases):
                key = f"fd{nd}_{i:02d}_{dtn}"
                arrays[key + "_A"] = np.asfortranarray(f[inp])
                arrays[key + "_R"] = np.asfortranarray(np.asarray(R, dtype=dt))
                meta["fd"].append({"key": key, "ndims": nd, "statement": stmt, "input": inp, "dtype": dtn})
        for n in ((32, 8, 8), (33, 7, 8)):
            T = index_cubed(n, dt)
            Ci = np.asfortranarray(np.ones(n, dtype=dt))
            one = dt(1)
            key = f"diff_{n[0]}x{n[1]}x{n[2]}_{dtn}"
            arrays[key + "_T"] = T
            arrays[key + "_Ci"] = Ci
            arrays[key + "_T2"] = np.asfortranarray(diffusion_ref(T, one, one, one, one, one, Ci))
            meta["diffusion"].append({"key": key, "n": list(n), "dtype": dtn,
                                      "forms": ["inv", "flux"], "scalars": "lam=dt=_dx=_dy=_dz=1"})
        p = diffusion_project(dt)
        for k, v in p.items():
            arrays[f"project8_{dtn}_{k}"] = v
        nx, ny, iters = 31, 17, 40
        for k, v in stokes2d_numpy(nx, ny, iters, dt).items():
            arrays[f"stokes2d_{dtn}_{k}"] = v
        meta["stokes2d"].append({"prefix": f"stokes2d_{dtn}_", "nx": nx, "ny": ny, "iters": iters, "dtype": dtn})
        n3, iters3 = (15, 13, 11), 30
        for k, v in stokes3d_numpy(*n3, iters3, dt).items():
            arrays[f"stokes3d_{dtn}_{k}"] = v
        meta["stokes3d"].append({"prefix": f"stokes3d_{dtn}_", "n": list(n3), "iters": iters3, "dtype": dtn})
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(meta, fh, indent=1)
    print(f"wrote {len(arrays)} arrays, {len(meta['fd'])} FD cases, {len(meta['diffusion'])} diffusion cases")


if __name__ == "__main__":
    main()
