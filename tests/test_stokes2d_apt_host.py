"""Accelerated pseudo-transient (APT) Stokes2D with pseudo-time steps from @maxloc(Mus), host side:
the C oracle against an independent numpy restatement of the same statements (bit for bit, FP64
and FP32), and the scheme's convergence on the configuration's viscosity contrast of 1e-3, where
the miniapp's damped iteration diverges (checked here too)."""
import numpy as np
import pytest


def numpy_apt(Mus, Rog, dx, dy, Re, r, Vpdt, max_lxy, n_iter, dtype):
    """The scheme restated with numpy broadcasting (same operation order as the statements)."""
    nx, ny = Mus.shape
    M = Mus.astype(dtype).astype(np.float64)  # coefficients in FP64 from the field's own values
    Mt = M.copy()
    Mt[1:-1, 1:-1] = np.maximum(np.maximum(np.maximum(M[:-2, 1:-1], M[2:, 1:-1]), M[1:-1, 1:-1]),
                                np.maximum(M[1:-1, :-2], M[1:-1, 2:]))
    R = ((Vpdt * max_lxy) / Re) / Mt
    G = ((Vpdt * Vpdt) / R) / (r + 2.0)
    kP, aT = r * G, 1.0 / (G / M + 1.0)
    bT = (2.0 * G) * aT
    Gc = np.minimum(np.minimum(G[:-1, :-1], G[1:, :-1]), np.minimum(G[:-1, 1:], G[1:, 1:]))
    mc = (((M[:-1, :-1] + M[1:, :-1]) + M[:-1, 1:]) + M[1:, 1:]) * 0.25
    aTc = 1.0 / (Gc / mc + 1.0)
    bTc = (2.0 * Gc) * aTc
    dtVx = np.minimum(R[:-1, 1:-1], R[1:, 1:-1])
    dtVy = np.minimum(R[1:-1, :-1], R[1:-1, 1:])
    c = {k: v.astype(dtype) for k, v in dict(kP=kP, aT=aT, bT=bT, aTc=aTc, bTc=bTc, dtVx=dtVx, dtVy=dtVy).items()}
    T = dtype
    _dx, _dy, third, h = T(1.0 / dx), T(1.0 / dy), T(1.0 / 3.0), T(0.5)
    Rg = Rog.astype(dtype)
    Vx, Vy = np.zeros((nx + 1, ny), dtype), np.zeros((nx, ny + 1), dtype)
    Pt, txx, tyy, txy = (np.zeros((nx, ny), dtype), np.zeros((nx, ny), dtype), np.zeros((nx, ny), dtype),
                         np.zeros((nx - 1, ny - 1), dtype))
    for _ in range(n_iter):
        dvx, dvy = Vx[1:, :] - Vx[:-1, :], Vy[:, 1:] - Vy[:, :-1]
        d = dvx * _dx + dvy * _dy
        td = d * third
        Pt = Pt - c["kP"] * d
        txx = c["aT"] * txx + c["bT"] * (dvx * _dx - td)
        tyy = c["aT"] * tyy + c["bT"] * (dvy * _dy - td)
        e = h * ((Vx[1:-1, 1:] - Vx[1:-1, :-1]) * _dy + (Vy[1:, 1:-1] - Vy[:-1, 1:-1]) * _dx)
        txy = c["aTc"] * txy + c["bTc"] * e
        Rx = ((txx[1:, 1:-1] - txx[:-1, 1:-1]) * _dx + (txy[:, 1:] - txy[:, :-1]) * _dy) - \
            (Pt[1:, 1:-1] - Pt[:-1, 1:-1]) * _dx
        Ry = (((tyy[1:-1, 1:] - tyy[1:-1, :-1]) * _dy + (txy[1:, :] - txy[:-1, :]) * _dx) -
              (Pt[1:-1, 1:] - Pt[1:-1, :-1]) * _dy) + (Rg[1:-1, :-1] + Rg[1:-1, 1:]) * h
        Vx[1:-1, 1:-1] = Vx[1:-1, 1:-1] + c["dtVx"] * Rx
        Vy[1:-1, 1:-1] = Vy[1:-1, 1:-1] + c["dtVy"] * Ry
        Vx[:, 0], Vx[:, -1] = Vx[:, 1], Vx[:, -2]
        Vy[0, :], Vy[-1, :] = Vy[1, :], Vy[-2, :]
    return dict(Vx=Vx, Vy=Vy, Pt=Pt, txx=txx, tyy=tyy, txy=txy, divV=d, Rx=Rx, Ry=Ry)


def _case(nx, ny, musi):
    from ps_gb300.stokes import Stokes2DAPTParams, inclusion_setup

    Mus, Rog = inclusion_setup(nx, ny, 1.0, 1.0, musi=musi, radius=0.1)
    return Mus, Rog, Stokes2DAPTParams(nx, ny, 1.0, 1.0)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [(31, 31), (40, 23)])
def test_oracle_apt_matches_numpy_restatement(oracle, n, dtype):
    Mus, Rog, p = _case(*n, 1e-3)
    o = oracle.Stokes2DAPT(*n, p.dx, p.dy, Mus, Rog, p.Re, p.r, p.Vpdt, p.max_lxy, dtype=dtype)
    for _ in range(25):
        o.step()
    ref = numpy_apt(Mus, Rog, p.dx, p.dy, p.Re, p.r, p.Vpdt, p.max_lxy, 25, dtype)
    for k, v in ref.items():
        assert np.array_equal(o[k], v), k
    assert np.abs(o["Vy"]).max() > 0


def test_apt_converges_at_contrast_1e3_where_the_miniapp_iteration_diverges(oracle):
    n = 63
    Mus, Rog, p = _case(n, n, 1e-3)
    o = oracle.Stokes2DAPT(n, n, p.dx, p.dy, Mus, Rog, p.Re, p.r, p.Vpdt, p.max_lxy)
    it, err = 0, np.inf
    while it < 40000 and not err < 1e-8:
        for _ in range(500):
            o.step()
        it += 500
        err, _ = o.residual()
    assert err < 1e-8, (it, err)
    m = oracle.Stokes2D(n, n, p.dx, p.dy, Mus, Rog)  # the miniapp's iteration, same setup
    m.compute_timesteps()
    for _ in range(2000):
        m.step()
    assert not np.isfinite(m.err()[0])
