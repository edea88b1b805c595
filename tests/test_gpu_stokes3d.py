"""GPU parity of the Stokes3D PT kernels (miniapps/Stokes3D.jl) and the PT solver."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {"f64": np.float64, "f32": np.float32}
STATE = ("Pt", "Vx", "Vy", "Vz", "divV", "txx", "tyy", "tzz", "txy", "txz", "tyz", "Rx", "Ry", "Rz", "dVxdtau",
         "dVydtau", "dVzdtau")


def _pair(ps, oracle, n, dtn, lx=10.0, musi=0.1):
    from ps_gb300.stokes3d import Stokes3D, Stokes3DParams, inclusion_setup

    Mus, Rog = inclusion_setup(*n, lx, lx, lx, musi=musi, dtype=DT[dtn])
    p = Stokes3DParams(*n, lx, lx, lx)
    g = Stokes3D(p, Mus, Rog, dtype=DT[dtn])
    o = oracle.Stokes3D(*n, *p.h, Mus, Rog, dtype=DT[dtn])
    g.compute_timesteps()
    o.compute_timesteps()
    return g, o


def _same(g, o, keys):
    for k in keys:
        assert np.array_equal(g.host(k), o[k]), k


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_stokes3d_golden(ps, golden, dtn):
    """The ten-launch loop body of one-to-one kernels equals the broadcasting restatement."""
    from ps_gb300.stokes3d import Stokes3D, Stokes3DParams

    meta, arr = golden
    case = [c for c in meta["stokes3d"] if c["dtype"] == dtn][0]
    gold = {k[len(case["prefix"]):]: v for k, v in arr.items() if k.startswith(case["prefix"])}
    g = Stokes3D(Stokes3DParams(*case["n"]), gold["Mus"], gold["Rog"], dtype=DT[dtn])
    g.compute_timesteps()
    for k in ("dtauVx", "dtauVy", "dtauVz", "dtauPt"):
        assert np.array_equal(g.host(k), gold[k]), k
    for _ in range(case["iters"]):
        g.step_reference_sequence()
    for k in STATE:
        assert np.array_equal(g.host(k), gold[k]), k


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("n", [(15, 13, 11), (34, 20, 17), (33, 33, 33)])
def test_stokes3d_iterate_matches_oracle(ps, oracle, dtn, n):
    """Three launches per iteration (fused P+τ, fused dV+V, all six copies) == the reference's loop;
    so do pairs of one-launch iterations (s3_fused_k) followed by the storing kernels."""
    g, o = _pair(ps, oracle, n, dtn)
    g.iterate(12)
    g.iterate(13, one_launch=True)
    for _ in range(25):
        o.step()
    _same(g, o, STATE)
    eg, parts_g = g.err()
    eo, parts_o = o.err()
    rtol = 1e-12 if dtn == "f64" else 1e-5
    assert np.allclose(parts_g, parts_o, rtol=rtol, atol=0), (parts_g, parts_o)
    assert eg > 0


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("n,iters", [((61, 29, 100), 5), ((31, 15, 7), 6), ((3, 3, 3), 4)])
def test_stokes3d_one_launch_iterations_random_state(ps, oracle, dtn, n, iters):
    """`iterate` runs pairs of one-launch iterations (s3_fused_k: the state through a second set,
    the stresses and residuals in registers and shared memory) and ends with the storing kernels:
    from a random state, every array equals the oracle's loop bit for bit. The sizes give several
    blocks in x and y, several z sweeps, and the smallest grid."""
    g, o = _pair(ps, oracle, n, dtn)
    rng = np.random.default_rng(8)
    for k in ("Pt", "Vx", "Vy", "Vz", "dVxdtau", "dVydtau", "dVzdtau"):
        v = np.asfortranarray((0.1 * rng.standard_normal(o[k].shape)).astype(DT[dtn]))
        o[k][...] = v
        g[k].copy_(ps.from_host(v))
    g.iterate(iters, one_launch=True)
    for _ in range(iters):
        o.step()
    _same(g, o, STATE)


def test_stokes3d_one_to_one_kernels_random_state(ps, oracle):
    """Each `@parallel` kernel on its own, from a random state (every array read is non-trivial)."""
    n = (19, 14, 12)
    g, o = _pair(ps, oracle, n, "f64")
    rng = np.random.default_rng(5)
    for k in STATE:
        v = np.asfortranarray(rng.standard_normal(o[k].shape))
        o[k][...] = v
        g[k].copy_(ps.from_host(v))
    g.compute_P()
    o.compute_P()
    _same(g, o, ("divV", "Pt"))
    g.compute_tau()
    o.compute_tau()
    _same(g, o, ("txx", "tyy", "tzz", "txy", "txz", "tyz"))
    g.compute_dV()
    o.compute_dV()
    _same(g, o, ("Rx", "Ry", "Rz", "dVxdtau", "dVydtau", "dVzdtau"))
    g.compute_V()
    o.compute_V()
    _same(g, o, ("Vx", "Vy", "Vz"))
    for which, name in g.BC_SEQUENCE:
        g.bc(which, name)
        o.bc(which, name)
        _same(g, o, (name,))


def test_stokes3d_solver(ps, oracle):
    """The graph-launched solver converges and runs exactly the reference's iteration. (The
    miniapp's PT parameters, damping 1 - 4/n and dτPt ~ 1/max(n), diverge on grids below ~40^3 --
    the oracle's iteration grows by ~1.6x per step at 23^3 -- so the solve runs at 63^3.)"""
    n = (63, 63, 63)
    g, _ = _pair(ps, oracle, n, "f64")
    st = g.solve(tol=1e-6, nout=100, max_iter=50_000)
    assert st.converged and st.err < 1e-6 and st.iters % 100 == 0
    assert g.err()[0] < 1e-6
    h, _ = _pair(ps, oracle, n, "f64")
    h.iterate(st.iters)
    for k in ("Pt", "Vx", "Vy", "Vz", "Rx", "Ry", "Rz", "divV"):
        assert np.array_equal(g.host(k), h.host(k)), k


def test_stokes3d_argument_errors(ps):
    from ps_gb300 import PSError
    from ps_gb300.stokes3d import Stokes3D, Stokes3DParams, inclusion_setup

    n = (9, 8, 7)
    Mus, Rog = inclusion_setup(*n)
    g = Stokes3D(Stokes3DParams(*n), Mus, Rog)
    g._fields.Vx.n[0] = 9  # wrong staggered extent
    with pytest.raises(PSError):
        g.compute_P()
    g._fields.Vx.n[0] = 10
    g.compute_P()
    with pytest.raises(PSError):
        g.solve(tol=1e-12, nout=10, max_iter=20)


def test_stokes3d_solver_reports_divergence(ps, oracle):
    """At 23^3 the miniapp's iteration diverges (as the oracle's does): the solver must report
    PS_ERR_NONFINITE, not convergence."""
    from ps_gb300 import PSError

    g, _ = _pair(ps, oracle, (23, 23, 23), "f64")
    with pytest.raises(PSError) as ei:
        g.solve(tol=1e-6, nout=100, max_iter=10_000)
    assert ei.value.status == -11


def test_stokes3d_mixed_solver_matches_fp64(ps, oracle):
    """FP32 sweeps + FP64 defect correction reach the same FP64 residual (the reference's err of the
    returned state) and the same solution as the FP64 solver."""
    n = (63, 63, 63)
    g64, _ = _pair(ps, oracle, n, "f64")
    gmx, _ = _pair(ps, oracle, n, "f64")
    tol = 1e-8
    s64 = g64.solve(tol=tol, nout=100, max_iter=200_000)
    smx = gmx.solve(tol=tol, nout=100, max_iter=200_000, mode=1)
    assert s64.converged and smx.converged and smx.outer >= 2
    e, parts = gmx.err()  # the FP64 residual arrays the solver left for the returned state
    assert e < tol and e == pytest.approx(smx.err, rel=1e-12)
    diffs = {}
    for k in ("Vx", "Vy", "Vz", "Pt"):
        a, b = g64.host(k), gmx.host(k)
        diffs[k] = np.abs(a - b).max() / np.abs(a).max()
    print("stokes3d mixed vs fp64 relative max differences", diffs, s64.iters, smx.iters, smx.outer)
    assert max(diffs.values()) < 1e-3, diffs


def test_stokes3d_mixed_solver_refuses_fp32(ps, oracle):
    from ps_gb300 import PSError

    g, _ = _pair(ps, oracle, (15, 15, 15), "f32")
    with pytest.raises(PSError) as e:
        g.solve(tol=1e-6, mode=1)
    assert e.value.status == -4
