"""Accelerated pseudo-transient Stokes2D (pseudo-time steps from @maxloc(Mus)) on the GPU against the
oracle's restatement of the same statements: coefficients, iterations and the FP64 residual bit
for bit (FP64 and FP32 fields); the FP64 solver's iterates equal the oracle's; the FP64 and
mixed-precision solvers converge at the configuration's viscosity contrast of 1e-3 and agree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ("Vx", "Vy", "Pt", "txx", "tyy", "txy", "divV", "Rx", "Ry")
COEFFS = ("Must", "kP", "aT", "bT", "aTc", "bTc", "dtVx", "dtVy")


def _pair(ps, oracle, nx, ny, musi, dtype=np.float64, lx=1.0):
    from ps_gb300.stokes import Stokes2DAPT, Stokes2DAPTParams, inclusion_setup

    Mus, Rog = inclusion_setup(nx, ny, lx, lx, musi=musi, radius=0.1 * lx)
    p = Stokes2DAPTParams(nx, ny, lx, lx)
    g = Stokes2DAPT(p, Mus, Rog, dtype=dtype)
    o = oracle.Stokes2DAPT(nx, ny, p.dx, p.dy, Mus, Rog, p.Re, p.r, p.Vpdt, p.max_lxy, dtype=dtype)
    g.coefficients()
    return g, o, p


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [(31, 31), (40, 23), (130, 97)])
def test_apt_iterations_are_bit_identical(ps, oracle, n, dtype):
    g, o, _ = _pair(ps, oracle, *n, 1e-3, dtype)
    for k in COEFFS:
        assert np.array_equal(g.host(k), o[k]), k
    g.iterate(37)
    for _ in range(37):
        o.step()
    for k in STATE:
        assert np.array_equal(g.host(k), o[k]), k
    assert np.abs(g.host("Vy")).max() > 0


def test_apt_residual_is_bit_identical(ps, oracle):
    g, o, _ = _pair(ps, oracle, 64, 48, 1e-3)
    g.iterate(50)
    for _ in range(50):
        o.step()
    err, _ = g.residual()
    err_o, arrays = o.residual()
    for k in ("Rx", "Ry", "divV", "txx", "tyy", "txy"):
        assert np.array_equal(g.host(k), arrays[k]), k
    assert abs(err - err_o) <= 1e-12 * err_o


def test_apt_1023_iterations_are_bit_identical(ps, oracle):
    """The configuration's grid (1023^2, unit box, r = 0.1, viscosity ratio 1e-3): 100 iterations."""
    g, o, _ = _pair(ps, oracle, 1023, 1023, 1e-3)
    g.iterate(100)
    for _ in range(100):
        o.step()
    for k in STATE:
        assert np.array_equal(g.host(k), o[k]), k


def test_apt_fp64_solver_converges_on_the_oracle_iterates(ps, oracle):
    """mode 0 at 63^2, ratio 1e-3: converges below 1e-8 on the FP64 residual, and its state equals
    the oracle's after the same number of iterations."""
    from ps_gb300.stokes import MODE_FP64

    g, o, _ = _pair(ps, oracle, 63, 63, 1e-3)
    st = g.solve(tol=1e-8, mode=MODE_FP64, nout=500, max_iter=100_000)
    assert st.converged and st.err < 1e-8 and st.iters % 500 == 0
    for _ in range(st.iters):
        o.step()
    for k in ("Vx", "Vy", "Pt", "txx", "tyy", "txy"):
        assert np.array_equal(g.host(k), o[k]), k
    err_o, _ = o.residual()
    assert err_o < 1e-8


@pytest.mark.parametrize("n", [(63, 63), (127, 95)])
def test_apt_mixed_solver_matches_fp64(ps, oracle, n):
    """mode 1 (FP32 sweeps on the correction, FP64 residual / update / check), ratio 1e-3:
    converges, its state is the FP64 solver's within 1e-5 of the largest value, and the oracle's
    residual of its V and P is below the tolerance."""
    from ps_gb300.stokes import MODE_FP64, MODE_MIXED

    a, o, _ = _pair(ps, oracle, *n, 1e-3)
    b, _, _ = _pair(ps, oracle, *n, 1e-3)
    sa = a.solve(tol=1e-8, mode=MODE_FP64, nout=200, max_iter=400_000)
    sb = b.solve(tol=1e-8, mode=MODE_MIXED, nout=200, max_iter=400_000)
    assert sa.converged and sb.converged and sb.outer >= 1
    for k in ("Vx", "Vy", "Pt"):
        x, y = a.host(k), b.host(k)
        assert np.abs(x - y).max() <= 1e-5 * np.abs(x).max(), (k, np.abs(x - y).max() / np.abs(x).max())
    for k in ("Vx", "Vy", "Pt"):
        o.a[k][...] = b.host(k)
    assert o.residual()[0] < 1e-8


def test_apt_rejects_bad_arguments(ps):
    from ps_gb300.stokes import Stokes2DAPT, Stokes2DAPTParams, inclusion_setup

    Mus, Rog = inclusion_setup(16, 16, 1.0, 1.0)
    g = Stokes2DAPT(Stokes2DAPTParams(16, 16, 1.0, 1.0), Mus, Rog, dtype=np.float32)
    with pytest.raises(ps.PSError):
        g.solve()  # FP64 fields only
    with pytest.raises(ps.PSError):
        g.residual()
    h = Stokes2DAPT(Stokes2DAPTParams(16, 16, 1.0, 1.0, Re=-1.0), Mus, Rog)
    with pytest.raises(ps.PSError):
        h.iterate(1)
