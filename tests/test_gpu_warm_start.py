"""Learned warm start of the Stokes2D PT solver: what the trained network (the committed weights,
trained on PT solutions generated by the library's own solver) gains over the zero start, and the
invariants of the warm-start state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(seed, n):
    from ps_gb300 import warm_start as W

    return W.random_setup(n, np.random.default_rng(seed))


def test_warm_start_state_invariants(ps):
    from ps_gb300 import nn, warm_start as W
    from ps_gb300.stokes import Stokes2D, Stokes2DParams

    net = W.load_default()
    for n in (255, 300):
        Mus, Rog = _setup(123, n)
        g = Stokes2D(Stokes2DParams(n, n, 1.0, 1.0), Mus, Rog)
        g.compute_timesteps()
        nn.warm_start(net, g)
        P, Vx, Vy = g.host("Pt"), g.host("Vx"), g.host("Vy")
        assert np.isfinite(P).all() and np.isfinite(Vx).all() and np.isfinite(Vy).all()
        assert not np.any(Vx[0]) and not np.any(Vx[-1]) and not np.any(Vy[:, 0]) and not np.any(Vy[:, -1])
        assert np.array_equal(Vx[:, 0], Vx[:, 1]) and np.array_equal(Vx[:, -1], Vx[:, -2])
        assert np.array_equal(Vy[0, :], Vy[1, :]) and np.array_equal(Vy[-1, :], Vy[-2, :])
        assert np.abs(Vy).max() > 0 and not np.any(g.host("dVxdtau"))


def test_mixed_solver_repairs_inconsistent_start(ps):
    """A start state violating the free-slip copies (here: a converged solution with perturbed copy
    rows) must still converge in the mixed-precision solver, as it does in the FP64 one."""
    from ps_gb300.stokes import Stokes2D, Stokes2DParams, inclusion_setup

    n = 127
    Mus, Rog = inclusion_setup(n, n, 1.0, 1.0, musi=0.3)
    g = Stokes2D(Stokes2DParams(n, n, 1.0, 1.0), Mus, Rog)
    g.compute_timesteps()
    g.solve(tol=1e-8, mode=0)
    Vx = g.host("Vx")
    Vx[:, 0] += 1e-3
    g["Vx"].copy_(ps.from_host(np.asfortranarray(Vx)))
    st = g.solve(tol=1e-8, mode=1, max_iter=400_000)
    assert st.converged and st.err < 1e-8


@pytest.mark.parametrize("mode", [0, 1])
def test_warm_start_reduces_pt_iterations(ps, mode):
    """Unseen setups at the training resolution: warm-started solves reach the same 1e-8 residual in
    fewer PT iterations than zero-start solves (FP64 and mixed-precision solvers)."""
    from ps_gb300 import warm_start as W

    net = W.load_default()
    res = W.evaluate(net, 4, n=255, tol=1e-8, mode=mode, seed0=4242)
    assert res["warm_failures"] == 0, res
    assert res["iters_ratio"] < 0.9, res
