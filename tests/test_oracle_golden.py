"""Pin the CPU oracle against the known-answer fixtures restated from the reference's tests.

Bit-exact: the reference tests compare every kernel to broadcasting with `==`."""
import numpy as np
import pytest

from conftest import DT


def _fd_desc(stmt, nd):
    from ps_gb300.fd import fd_kernel

    k = fd_kernel(stmt, nd)
    d = k.descriptor
    return d.kind, d.opdims, d.inn, d.ndims, k.lhs_inn


def test_oracle_fd_all_macros(oracle, golden):
    meta, arr = golden
    assert len(meta["fd"]) > 150
    for case in meta["fd"]:
        A = arr[case["key"] + "_A"]
        Rexp = arr[case["key"] + "_R"]
        R = np.asfortranarray(np.zeros(Rexp.shape, dtype=DT[case["dtype"]]))
        kind, opdims, inn, nd, lhs_inn = _fd_desc(case["statement"], case["ndims"])
        oracle.fd_apply(kind, opdims, inn, nd, lhs_inn, R, np.asfortranarray(A))
        assert np.array_equal(R, Rexp), (case["key"], case["statement"])


@pytest.mark.parametrize("form", [1, 2])  # _dx^2 form and on-the-fly flux form: same test expectation
def test_oracle_diffusion_known_answers(oracle, golden, form):
    meta, arr = golden
    for case in meta["diffusion"]:
        dt = DT[case["dtype"]]
        T, Ci, T2e = arr[case["key"] + "_T"], arr[case["key"] + "_Ci"], arr[case["key"] + "_T2"]
        T2 = np.asfortranarray(np.zeros_like(T))
        oracle.diffusion3d_step(form, T2, np.asfortranarray(T), np.asfortranarray(Ci), None, 1, 1, 1, 1, 1)
        assert np.array_equal(T2, T2e), case["key"]
        assert T2.dtype == dt


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_oracle_diffusion_project(oracle, golden, dtn):
    _, arr = golden
    p = {k.split("_", 2)[2]: v for k, v in arr.items() if k.startswith(f"project8_{dtn}_")}
    lam, dt_, dx, dy, dz = p["scalars"]
    T = np.asfortranarray(p["T0"].copy())
    T2 = np.asfortranarray(T.copy())
    for _ in range(3):
        oracle.diffusion3d_step(0, T2, T, np.asfortranarray(p["Ci"]), None, lam, dt_, dx, dy, dz)
        T, T2 = T2, T
    assert np.array_equal(T, p["T"])


def test_oracle_masks_keep_boundary(oracle):
    rng = np.random.default_rng(3)
    n = (10, 9, 8)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(rng.random(n))
    T2 = np.asfortranarray(np.full(n, -7.0))
    oracle.diffusion3d_step(3, T2, T, Ci, np.asfortranarray(1 + 0.5 * rng.random(n)), 0, 1e-3, 1, 1, 1)
    inner = np.zeros(n, bool)
    inner[1:-1, 1:-1, 1:-1] = True
    assert np.all(T2[~inner] == -7.0)
    assert np.all(T2[inner] != -7.0)


def test_oracle_flux_lam_equals_scalar_when_constant(oracle):
    """With lam = const, @av_xi(lam) == lam, so the array form equals the scalar flux form."""
    rng = np.random.default_rng(5)
    n = (12, 11, 10)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(rng.random(n))
    lam = np.asfortranarray(np.full(n, 1.25))
    a = np.asfortranarray(np.zeros(n))
    b = np.asfortranarray(np.zeros(n))
    oracle.diffusion3d_step(2, a, T, Ci, None, 1.25, 1e-3, 3.0, 2.0, 1.0)
    oracle.diffusion3d_step(3, b, T, Ci, lam, 0.0, 1e-3, 3.0, 2.0, 1.0)
    assert np.array_equal(a, b)


def test_oracle_ranges_compose(oracle):
    """Running the six `@hide_communication` boundary boxes plus the inner box equals one full call."""
    from ps_gb300.kernels import get_ranges_inner, get_ranges_outer

    rng = np.random.default_rng(9)
    n = (20, 14, 12)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(rng.random(n))
    full = np.asfortranarray(np.zeros(n))
    split = np.asfortranarray(np.zeros(n))
    oracle.diffusion3d_step(1, full, T, Ci, None, 1.0, 1e-3, 2.0, 2.0, 2.0)
    bw = (4, 2, 2)
    for lo, hi in get_ranges_outer(bw, n) + get_ranges_inner(bw, n):
        oracle.diffusion3d_step(1, split, T, Ci, None, 1.0, 1e-3, 2.0, 2.0, 2.0, lo=lo, hi=hi)
    assert np.array_equal(full, split)


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_oracle_stokes2d_vs_broadcasting(oracle, golden, dtn):
    """miniapps/Stokes2D.jl kernels: the oracle's loops equal the broadcasting restatement."""
    meta, arr = golden
    case = [c for c in meta["stokes2d"] if c["dtype"] == dtn][0]
    g = {k[len(case["prefix"]):]: v for k, v in arr.items() if k.startswith(case["prefix"])}
    nx, ny = case["nx"], case["ny"]
    s = oracle.Stokes2D(nx, ny, 10.0 / (nx - 1), 10.0 / (ny - 1), g["Mus"], g["Rog"], dtype=DT[dtn])
    s.compute_timesteps()
    for k in ("dtauVx", "dtauVy", "dtauPt"):
        assert np.array_equal(s[k], g[k]), k
    for _ in range(case["iters"]):
        s.step()
    for k in ("Pt", "Vx", "Vy", "divV", "txx", "tyy", "txy", "Rx", "Ry", "dVxdtau", "dVydtau"):
        assert np.array_equal(s[k], g[k]), k
    assert s.err()[0] > 0


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_oracle_stokes3d_vs_broadcasting(oracle, golden, dtn):
    """miniapps/Stokes3D.jl kernels: the oracle's loops equal the broadcasting restatement."""
    meta, arr = golden
    case = [c for c in meta["stokes3d"] if c["dtype"] == dtn][0]
    g = {k[len(case["prefix"]):]: v for k, v in arr.items() if k.startswith(case["prefix"])}
    nx, ny, nz = case["n"]
    s = oracle.Stokes3D(nx, ny, nz, 10.0 / (nx - 1), 10.0 / (ny - 1), 10.0 / (nz - 1), g["Mus"], g["Rog"],
                        dtype=DT[dtn])
    s.compute_timesteps()
    for k in ("dtauVx", "dtauVy", "dtauVz", "dtauPt"):
        assert np.array_equal(s[k], g[k]), k
    for _ in range(case["iters"]):
        s.step()
    for k in ("Pt", "Vx", "Vy", "Vz", "divV", "txx", "tyy", "tzz", "txy", "txz", "tyz", "Rx", "Ry", "Rz", "dVxdtau",
              "dVydtau", "dVzdtau"):
        assert np.array_equal(s[k], g[k]), k
    assert s.err()[0] > 0


def test_oracle_adjoint_matches_finite_differences(oracle):
    """The oracle's reverse sweep (the restatement the GPU adjoint is checked against) agrees
    with central finite differences of its own forward solver on random directions."""
    rng = np.random.default_rng(4)
    n = (10, 9, 8)
    T0 = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(0.5 + rng.random(n))
    lam = np.asfortranarray(np.exp(0.3 * rng.standard_normal(n)))
    T_obs = np.asfortranarray(T0 + 0.1 * rng.standard_normal(n))
    h = (9.0, 8.0, 7.0)
    dt = (1 / 9.0) ** 2 / lam.max() / 8.1
    nt = 6
    _, g = oracle.misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt)
    for _ in range(4):
        v = np.asfortranarray(rng.standard_normal(n))
        eps = 1e-6
        lp, _ = oracle.misfit_gradient(T0, T_obs, Ci, np.asfortranarray(lam + eps * v), dt, h, nt)
        lm, _ = oracle.misfit_gradient(T0, T_obs, Ci, np.asfortranarray(lam - eps * v), dt, h, nt)
        fd = (lp - lm) / (2 * eps)
        ad = float(np.sum(g * v))
        assert abs(fd - ad) <= 1e-6 * max(1.0, abs(ad)), (fd, ad)
