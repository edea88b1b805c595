"""Parity at the benchmark sizes: the 512^3 diffusion workload (FP64 and FP32 fields, the flux form
with a conductivity array) and the 1023^2 Stokes2D PT iteration, against the C oracle on the same
seeded inputs.

Bars: IEEE kernels bit-identical to the oracle; the split-FP32 grid arithmetic of the headline run
within 1e-12 relative max-norm of the oracle after 1, 20, 50 and 100 steps; memcopy3D exactly T + Ci."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 512


@pytest.fixture(scope="module")
def fields512():
    """The headline workload's inputs: T ~ U(0,1), lam = 1 + 0.5 U(0,1), Ci = 1 (seeded)."""
    rng = np.random.default_rng(2)
    T = np.asfortranarray(rng.random((N, N, N)))
    lam = np.asfortranarray(1.0 + 0.5 * np.random.default_rng(3).random((N, N, N)))
    Ci = np.asfortranarray(np.ones((N, N, N)))
    dx = 10.0 / (N - 1)
    sc = (dx * dx / 1.5 / 8.1, 1 / dx, 1 / dx, 1 / dx)
    return T, lam, Ci, sc


def _oracle_steps(oracle, T, Ci, lam, sc, nt):
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(nt):
        oracle.diffusion3d_step(3, b, a, Ci, lam, 0.0, *sc)
        a, b = b, a
    return a


def test_headline_512_ieee_step_is_bit_identical(ps, oracle, fields512):
    T, lam, Ci, sc = fields512
    ref = _oracle_steps(oracle, T, Ci, lam, sc, 1)
    dT, dCi, dlam = ps.from_host(T), ps.from_host(Ci), ps.from_host(lam)
    for memopt in (True, False):
        T2 = ps.from_host(T)
        ps.parallel(ps.kernels.diffusion3D_step_flux_lam, T2, dT, dCi, dlam, *sc, memopt=memopt)
        assert np.array_equal(ps.to_host(T2), ref), memopt
        del T2


def test_headline_512_split_grid_run_within_1e12(ps, oracle, fields512):
    """The benchmark's own run (`ps_diffusion3d_run`, state on the fixed grid) after 1, 20, 50 (the
    workload's step count) and 100 steps, each run from the initial state as one call."""
    T, lam, Ci, sc = fields512
    dCi, dlam = ps.from_host(Ci), ps.from_host(lam)
    ref = T
    done = 0
    for nt in (1, 20, 50, 100):
        ref = _oracle_steps(oracle, ref, Ci, lam, sc, nt - done)
        done = nt
        dT, dT2 = ps.from_host(T), ps.from_host(T)
        ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, dCi, dlam, *sc, nt, fp64="split_grid")
        err = np.abs(ps.to_host(dT) - ref).max() / np.abs(ref).max()
        print(f"split_grid 512^3 after {nt} steps: {err:.3e}")
        assert err <= 1e-12, (nt, err)
        if nt == 100:  # and the IEEE run is the oracle's, bit for bit
            dT.copy_(ps.from_host(T))
            dT2.copy_(dT)
            ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, dCi, dlam, *sc, nt, fp64="ieee")
            assert np.array_equal(ps.to_host(dT), ref)
        del dT, dT2


def test_headline_512_fp32_step_is_bit_identical(ps, oracle, fields512):
    T, lam, Ci, sc = fields512
    T32, lam32, Ci32 = (np.asfortranarray(x.astype(np.float32)) for x in (T, lam, Ci))
    ref = _oracle_steps(oracle, T32, Ci32, lam32, sc, 1)
    T2 = ps.from_host(T32)
    ps.parallel(ps.kernels.diffusion3D_step_flux_lam, T2, ps.from_host(T32), ps.from_host(Ci32), ps.from_host(lam32),
                *sc, memopt=True)
    assert np.array_equal(ps.to_host(T2), ref)


def test_memcopy3d_512(ps, fields512):
    T, lam, Ci, _ = fields512
    T2 = ps.zeros(N, N, N)
    ps.parallel(ps.kernels.copy3D, T2, ps.from_host(T), ps.from_host(lam))
    assert np.array_equal(ps.to_host(T2), T + lam)


@pytest.mark.parametrize("musi", [0.1, 1e-3])
def test_stokes2d_1023_iterations_are_bit_identical(ps, oracle, musi):
    """The Stokes2D benchmark grid (1023^2, unit box, inclusion r = 0.1, rho*g = 1 inside): 200 fused
    PT iterations against 200 oracle loop bodies. Viscosity ratio 0.1 is the benchmark's; at the
    configuration's 1e-3 the reference's iteration diverges, and the GPU diverges identically (the
    same NaN and Inf at the same cells)."""
    from ps_gb300.stokes import Stokes2D, Stokes2DParams, inclusion_setup

    n = 1023
    Mus, Rog = inclusion_setup(n, n, 1.0, 1.0, musi=musi, radius=0.1)
    p = Stokes2DParams(n, n, 1.0, 1.0)
    g = Stokes2D(p, Mus, Rog)
    o = oracle.Stokes2D(n, n, p.dx, p.dy, Mus, Rog)
    g.compute_timesteps()
    o.compute_timesteps()
    g.iterate(200)
    for _ in range(200):
        o.step()
    for k in ("Pt", "Vx", "Vy", "txx", "tyy", "txy", "Rx", "Ry", "dVxdtau", "dVydtau"):
        assert np.array_equal(g.host(k), o[k], equal_nan=True), k
    finite = np.isfinite(g.host("Pt")).all()
    assert finite == (musi == 0.1)
    assert np.nanmax(np.abs(g.host("Vy"))) > 0
