"""FP64 diffusion with split-FP32 arithmetic (fp64_mode = split): error against the FP64 oracle
must stay <= 1e-12 relative max-norm (the fixed tolerance for FP64 fields)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KERNELS = ["diffusion3D_step", "diffusion3D_step_inv", "diffusion3D_step_flux", "diffusion3D_step_flux_lam"]


def _setup(n, form, seed=0):
    rng = np.random.default_rng(seed)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(0.5 + rng.random(n))
    lam = np.asfortranarray(1 + 0.5 * rng.random(n))
    h = tuple(1.0 / (m - 1) for m in n)
    hs = h if form == 0 else tuple(1 / x for x in h)
    dt = min(h) ** 2 / 1.5 / 8.1 / 1.5
    return T, Ci, lam, hs, dt


def relerr(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def faces_untouched(got, T0):
    """The six boundary faces hold the initial values exactly (the steps write inner cells only)."""
    return all(np.array_equal(np.take(got, i, axis=d), np.take(T0, i, axis=d)) for d in range(3) for i in (0, -1))


@pytest.mark.parametrize("n", [(64, 40, 36), (130, 66, 70), (256, 24, 9), (66, 66, 66)])
@pytest.mark.parametrize("form", [0, 1, 2, 3])
def test_split_one_step_vs_oracle(ps, oracle, n, form):
    T, Ci, lam, hs, dt = _setup(n, form, seed=form)
    ref = np.asfortranarray(T.copy())
    oracle.diffusion3d_step(form, ref, T, Ci, lam if form == 3 else None, 1.3, dt, *hs)
    k = getattr(ps.kernels, KERNELS[form])
    T2 = ps.from_host(T)
    ps.parallel(k, T2, ps.from_host(T), ps.from_host(Ci), ps.from_host(lam) if form == 3 else 1.3, dt, *hs,
                memopt=True, fp64="split")
    got = ps.to_host(T2)
    e = relerr(got, ref)
    assert e <= 1e-13, e
    # boundary cells untouched (T2 started as a copy of T)
    assert np.array_equal(got[0], T[0]) and np.array_equal(got[:, -1], T[:, -1])


def test_split_anisotropic_spacing(ps, oracle):
    n = (64, 48, 40)
    T, Ci, lam, _, dt = _setup(n, 3, seed=7)
    hs = (63.0, 30.0, 17.0)
    dt = (1 / 63.0) ** 2 / 1.5 / 8.1 / 3
    ref = np.asfortranarray(T.copy())
    oracle.diffusion3d_step(3, ref, T, Ci, lam, 0.0, dt, *hs)
    T2 = ps.from_host(T)
    ps.parallel(ps.kernels.diffusion3D_step_flux_lam, T2, ps.from_host(T), ps.from_host(Ci), ps.from_host(lam), dt,
                *hs, memopt=True, fp64="split")
    assert relerr(ps.to_host(T2), ref) <= 1e-13


def test_split_50_steps_within_tolerance(ps, oracle):
    """The cfg-1 workload shape (flux form, lam = 1 + 0.5 U(0,1), Ci = 1), 50 steps, 96^3."""
    n = (96, 96, 96)
    rng = np.random.default_rng(2)
    T = np.asfortranarray(rng.random(n))
    lam = np.asfortranarray(1 + 0.5 * rng.random(n))
    Ci = np.asfortranarray(np.ones(n))
    _dx = n[0] - 1.0
    dt = (1 / _dx) ** 2 / 1.5 / 8.1
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(50):
        oracle.diffusion3d_step(3, b, a, Ci, lam, 0.0, dt, _dx, _dx, _dx)
        a, b = b, a
    dT, dT2, dCi, dl = ps.from_host(T), ps.from_host(T), ps.from_host(Ci), ps.from_host(lam)
    for _ in range(50):
        ps.parallel(ps.kernels.diffusion3D_step_flux_lam, dT2, dT, dCi, dl, dt, _dx, _dx, _dx, memopt=True,
                    fp64="split", sync=False)
        dT, dT2 = dT2, dT
    ps.synchronize()
    e = relerr(ps.to_host(dT), a)
    assert e <= 1e-12, e


def test_split_zeros_and_tiny_values(ps, oracle):
    """Exact zeros stay exact; magnitudes far below 2^-80 are handled (Gaussian tails)."""
    n = (64, 32, 32)
    x = np.linspace(-8, 8, n[0])[:, None, None]
    T = np.asfortranarray(np.broadcast_to(1.7 * np.exp(-x ** 2), n).copy())
    T[:, :, :4] = 0.0
    Ci = np.asfortranarray(np.ones(n))
    _dx = 10.0
    dt = (1 / _dx) ** 2 / 8.1
    ref = np.asfortranarray(T.copy())
    oracle.diffusion3d_step(2, ref, T, Ci, None, 1.0, dt, _dx, _dx, _dx)
    T2 = ps.from_host(T)
    ps.parallel(ps.kernels.diffusion3D_step_flux, T2, ps.from_host(T), ps.from_host(Ci), 1.0, dt, _dx, _dx, _dx,
                memopt=True, fp64="split")
    got = ps.to_host(T2)
    assert relerr(got, ref) <= 1e-13
    assert np.all(got[:, :, :3] == 0.0)


def test_split_out_of_range_is_reported(ps):
    n = (64, 16, 16)
    T = ps.fill(1e300, *n)
    T2 = ps.zeros(*n)
    Ci = ps.ones(*n)
    with pytest.raises(ps.PSError) as e:
        ps.parallel(ps.kernels.diffusion3D_step_inv, T2, T, Ci, 1.0, 1e-3, 1.0, 1.0, 1.0, memopt=True, fp64="split")
    assert e.value.status == -12


def test_split_odd_extent_uses_ieee_path(ps, oracle):
    """nx odd breaks TMA's 16-byte stride rule: the call falls back to the bit-exact IEEE kernels."""
    n = (33, 17, 12)
    T, Ci, lam, hs, dt = _setup(n, 1, seed=3)
    ref = np.asfortranarray(T.copy())
    oracle.diffusion3d_step(1, ref, T, Ci, None, 1.0, dt, *hs)
    T2 = ps.from_host(T)
    ps.parallel(ps.kernels.diffusion3D_step_inv, T2, ps.from_host(T), ps.from_host(Ci), 1.0, dt, *hs, memopt=True,
                fp64="split")
    assert np.array_equal(ps.to_host(T2), ref)


@pytest.mark.parametrize("nt", [7, 8])
@pytest.mark.parametrize("fp64", ["ieee", "split", "split_state"])
@pytest.mark.parametrize("form", [0, 3])
def test_run_driver_vs_oracle_loop(ps, oracle, nt, fp64, form):
    """ps_diffusion3d_run == the examples' time loop (T, T2 swapped each step)."""
    n = (64, 34, 30)
    T, Ci, lam, hs, dt = _setup(n, form, seed=11)
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(nt):
        oracle.diffusion3d_step(form, b, a, Ci, lam if form == 3 else None, 1.3, dt, *hs)
        a, b = b, a
    k = getattr(ps.kernels, KERNELS[form])
    dT, dT2 = ps.from_host(T), ps.from_host(T)
    ps.kernels.run(k, dT, dT2, ps.from_host(Ci), ps.from_host(lam) if form == 3 else 1.3, dt, *hs, nt, fp64=fp64)
    got = ps.to_host(dT)
    if fp64 == "ieee":
        assert np.array_equal(got, a)
    else:
        assert relerr(got, a) <= 1e-12
        assert faces_untouched(got, T)


def test_run_driver_odd_size_falls_back(ps, oracle):
    n = (33, 20, 18)
    T, Ci, lam, hs, dt = _setup(n, 3, seed=12)
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(5):
        oracle.diffusion3d_step(3, b, a, Ci, lam, 0.0, dt, *hs)
        a, b = b, a
    dT, dT2 = ps.from_host(T), ps.from_host(T)
    ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, ps.from_host(Ci), ps.from_host(lam), dt, *hs, 5,
                   fp64="split_state")
    assert np.array_equal(ps.to_host(dT), a)


@pytest.mark.parametrize("n", [(64, 64, 64), (64, 34, 30)])
@pytest.mark.parametrize("form", [0, 1, 2, 3])
@pytest.mark.parametrize("nt", [1, 20, 50, 100])
def test_grid_run_vs_oracle_loop(ps, oracle, n, form, nt):
    """fp64 = split_grid (state on a fixed power-of-two grid): isotropic (cubic) and anisotropic spacing,
    up to the 100 steps of the diffusion examples' time loop."""
    T, Ci, lam, hs, dt = _setup(n, form, seed=20 + form)
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(nt):
        oracle.diffusion3d_step(form, b, a, Ci, lam if form == 3 else None, 1.3, dt, *hs)
        a, b = b, a
    k = getattr(ps.kernels, KERNELS[form])
    dT, dT2 = ps.from_host(T), ps.from_host(T)
    ps.kernels.run(k, dT, dT2, ps.from_host(Ci), ps.from_host(lam) if form == 3 else 1.3, dt, *hs, nt,
                   fp64="split_grid")
    got = ps.to_host(dT)
    e = relerr(got, a)
    assert e <= 1e-12, e
    assert faces_untouched(got, T)


@pytest.mark.parametrize("shift,scale,lscale", [(-0.5, 1e-30, 1e5), (3.0, 7.0e20, 1e-7), (0.0, 1.0, 1.0)])
def test_grid_run_value_ranges(ps, oracle, shift, scale, lscale):
    """Negative values, magnitudes far outside FP32's range relative to 1, scaled conductivities."""
    n = (64, 40, 36)
    T, Ci, lam, hs, dt = _setup(n, 3, seed=31)
    T = np.asfortranarray((T + shift) * scale)
    lam = np.asfortranarray(lam * lscale)
    dt = dt / lscale
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(10):
        oracle.diffusion3d_step(3, b, a, Ci, lam, 0.0, dt, *hs)
        a, b = b, a
    dT, dT2 = ps.from_host(T), ps.from_host(T)
    ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, ps.from_host(Ci), ps.from_host(lam), dt, *hs, 10,
                   fp64="split_grid")
    e = relerr(ps.to_host(dT), a)
    assert e <= 1e-12, e


def test_grid_run_zero_field(ps):
    n = (64, 40, 36)
    _, Ci, lam, hs, dt = _setup(n, 3, seed=32)
    Z = np.zeros(n, order="F")
    dT, dT2 = ps.from_host(Z), ps.from_host(Z)
    ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, ps.from_host(Ci), ps.from_host(lam), dt, *hs, 4,
                   fp64="split_grid")
    assert not np.any(ps.to_host(dT))


def test_grid_run_growth_falls_back_to_split_state(ps):
    """An unstable dt makes max|T| grow past its initial power of two: the grid run is redone with
    value-relative split pairs, so its result is bit-identical to a split_state run."""
    n = (64, 40, 36)
    T, Ci, lam, hs, dt = _setup(n, 3, seed=33)
    dt = dt * 12.0
    out = {}
    for mode in ("split_grid", "split_state"):
        dT, dT2 = ps.from_host(T), ps.from_host(T)
        ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, ps.from_host(Ci), ps.from_host(lam), dt, *hs,
                       6, fp64=mode)
        out[mode] = ps.to_host(dT)
    assert np.abs(out["split_state"]).max() > 1.0  # left the grid of max|T0| < 1
    assert np.array_equal(out["split_grid"], out["split_state"])


def test_grid_run_growth_in_last_step(ps, oracle):
    """Growth past the grid in the last step only: that step writes IEEE doubles directly (summed in
    FP64 where a value left the grid), so no rerun is needed and the result stays within tolerance."""
    n = (64, 40, 36)
    T, Ci, lam, hs, dt = _setup(n, 3, seed=34)
    dt = dt * 12.0
    ref = T.copy(order="F")
    oracle.diffusion3d_step(3, ref, T, Ci, lam, 0.0, dt, *hs)
    assert np.abs(ref).max() > 1.0
    dT, dT2 = ps.from_host(T), ps.from_host(T)
    ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, dT, dT2, ps.from_host(Ci), ps.from_host(lam), dt, *hs, 1,
                   fp64="split_grid")
    e = relerr(ps.to_host(dT), ref)
    assert e <= 1e-12, e
