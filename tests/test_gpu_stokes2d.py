"""GPU parity of the Stokes2D PT kernels (miniapps/Stokes2D.jl) and the PT solvers."""
import numpy as np
import pytest

from conftest import DT

pytestmark = pytest.mark.gpu

ALL = ("Pt", "Vx", "Vy", "divV", "txx", "tyy", "txy", "Rx", "Ry", "dVxdtau", "dVydtau")


def _pair(ps, oracle, nx, ny, dtn, lx=10.0, musi=0.1):
    from ps_gb300.stokes import Stokes2D, Stokes2DParams, inclusion_setup

    Mus, Rog = inclusion_setup(nx, ny, lx, lx, musi=musi, dtype=DT[dtn])
    p = Stokes2DParams(nx, ny, lx, lx)
    g = Stokes2D(p, Mus, Rog, dtype=DT[dtn])
    o = oracle.Stokes2D(nx, ny, p.dx, p.dy, Mus, Rog, dtype=DT[dtn])
    g.compute_timesteps()
    o.compute_timesteps()
    return g, o


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_stokes2d_golden(ps, oracle, golden, dtn):
    meta, arr = golden
    case = [c for c in meta["stokes2d"] if c["dtype"] == dtn][0]
    gold = {k[len(case["prefix"]):]: v for k, v in arr.items() if k.startswith(case["prefix"])}
    from ps_gb300.stokes import Stokes2D, Stokes2DParams

    g = Stokes2D(Stokes2DParams(case["nx"], case["ny"]), gold["Mus"], gold["Rog"], dtype=DT[dtn])
    g.compute_timesteps()
    for _ in range(case["iters"]):
        g.step_reference_sequence()
    for k in ALL + ("dtauVx", "dtauVy", "dtauPt"):
        assert np.array_equal(g.host(k), gold[k]), k


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("n", [(31, 17), (33, 9), (64, 40), (127, 127)])
def test_stokes2d_fused_equals_six_kernels(ps, oracle, dtn, n):
    nx, ny = n
    g, o = _pair(ps, oracle, nx, ny, dtn)
    iters = 37
    for _ in range(iters):
        o.step()
    g.iterate(iters)
    for k in ALL:
        assert np.array_equal(g.host(k), o[k]), (k, n, dtn)
    e_gpu, parts = g.err()
    e_orc, oparts = o.err()
    np.testing.assert_allclose(parts, oparts, rtol=1e-12 if dtn == "f64" else 1e-5)


def test_stokes2d_one_to_one_kernels(ps, oracle):
    g, o = _pair(ps, oracle, 45, 29, "f64")
    for _ in range(10):
        o.step()
        g.step_reference_sequence()
    for k in ALL:
        assert np.array_equal(g.host(k), o[k]), k


def test_stokes2d_fp64_solver_iterates_match_oracle(ps, oracle):
    """The graph-launched fused FP64 solver runs the reference's iteration exactly."""
    g, o = _pair(ps, oracle, 63, 63, "f64")
    st = g.solve(tol=1e-4, mode=0, nout=50, max_iter=200_000)
    assert st.converged and st.err < 1e-4
    for _ in range(st.iters):
        o.step()
    for k in ("Pt", "Vx", "Vy", "dVxdtau", "dVydtau"):
        assert np.array_equal(g.host(k), o[k]), k
    assert abs(o.err()[0] - st.err) <= 1e-12 * max(1.0, st.err) + 1e-15


@pytest.mark.parametrize("n", [(63, 63), (127, 95)])
def test_stokes2d_mixed_solver_matches_fp64(ps, oracle, n):
    """FP32 PT sweeps + FP64 defect correction reach the FP64 tolerance and the FP64 solution."""
    nx, ny = n
    a, _ = _pair(ps, oracle, nx, ny, "f64", lx=1.0, musi=0.1)
    b, _ = _pair(ps, oracle, nx, ny, "f64", lx=1.0, musi=0.1)
    tol = 1e-8
    sa = a.solve(tol=tol, mode=0, max_iter=2_000_000)
    sb = b.solve(tol=tol, mode=1, max_iter=2_000_000)
    assert sa.converged and sb.converged and sb.err < tol and sb.outer >= 1
    for k in ("Pt", "Vx", "Vy"):
        ref = a.host(k)
        err = np.abs(b.host(k) - ref).max() / max(np.abs(ref).max(), 1e-30)
        assert err < 1e-5, (k, err)


def test_stokes2d_solver_errors(ps, oracle):
    g, _ = _pair(ps, oracle, 31, 31, "f64")
    with pytest.raises(ps.PSError) as e:
        g.solve(tol=1e-12, mode=0, nout=10, max_iter=20)
    assert e.value.status == -7  # PS_ERR_NOT_CONVERGED
    with pytest.raises(ps.PSError) as e:
        g.solve(tol=1e-8, mode=0, nout=3)
    assert e.value.status == -1
