"""GPU parity of the acoustic3D miniapp kernels (miniapps/acoustic3D.jl:11-21) vs the oracle."""
import numpy as np
import pytest

from conftest import DT

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("n", [(15, 15, 15), (31, 17, 9)])
def test_acoustic3d_steps_vs_oracle(ps, oracle, dtn, n):
    dt = DT[dtn]
    nx, ny, nz = n
    lx = ly = lz = 40.0
    dx, dy, dz = lx / (nx - 1), ly / (ny - 1), lz / (nz - 1)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    P = np.asfortranarray(np.exp(-(ix * dx - 0.5 * lx) ** 2 - (iy * dy - 0.5 * ly) ** 2 - (iz * dz - 0.5 * lz) ** 2)
                          .astype(dt))
    Vx = np.asfortranarray(np.zeros((nx + 1, ny, nz), dt))
    Vy = np.asfortranarray(np.zeros((nx, ny + 1, nz), dt))
    Vz = np.asfortranarray(np.zeros((nx, ny, nz + 1), dt))
    k, rho = 1.0, 1.0
    dts = min(dx, dy, dz) / np.sqrt(k / rho) / 6.1
    dP, dVx, dVy, dVz = (ps.from_host(a) for a in (P, Vx, Vy, Vz))
    for _ in range(20):
        oracle.acoustic3d_v(Vx, Vy, Vz, P, dts, rho, dx, dy, dz)
        oracle.acoustic3d_p(P, Vx, Vy, Vz, dts, k, dx, dy, dz)
        ps.parallel(ps.kernels.acoustic3D_compute_V, dVx, dVy, dVz, dP, dts, rho, dx, dy, dz)
        ps.parallel(ps.kernels.acoustic3D_compute_P, dP, dVx, dVy, dVz, dts, k, dx, dy, dz)
    for a, d in ((P, dP), (Vx, dVx), (Vy, dVy), (Vz, dVz)):
        assert np.array_equal(ps.to_host(d), a)
    assert np.abs(P).max() > 0


def test_acoustic3d_shape_errors(ps):
    P = ps.zeros(8, 8, 8)
    with pytest.raises(ps.PSError) as e:
        ps.parallel(ps.kernels.acoustic3D_compute_V, ps.zeros(8, 8, 8), ps.zeros(8, 9, 8), ps.zeros(8, 8, 9), P,
                    1.0, 1.0, 1.0, 1.0, 1.0)
    assert e.value.status == -3


def _acoustic_setup(n, dt, seed=3):
    """The miniapp's Gaussian P (acoustic3D.jl:39) plus seeded noise on every array, so that faces
    outside @inn hold values a copy must keep."""
    nx, ny, nz = n
    lx = ly = lz = 40.0
    h = (lx / max(nx - 1, 1), ly / max(ny - 1, 1), lz / max(nz - 1, 1))
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    rng = np.random.default_rng(seed)
    P = np.exp(-(ix * h[0] - 0.5 * lx) ** 2 - (iy * h[1] - 0.5 * ly) ** 2 - (iz * h[2] - 0.5 * lz) ** 2)
    P = np.asfortranarray((P + 0.01 * rng.random(n)).astype(dt))
    Vs = [np.asfortranarray((0.01 * rng.standard_normal(s)).astype(dt))
          for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    dts = min(h) / np.sqrt(1.0) / 6.1
    return P, Vs, h, dts


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("n", [(15, 15, 15), (31, 17, 9), (33, 40, 37), (64, 9, 70), (2, 3, 4), (3, 1, 5), (1, 6, 2)])
def test_acoustic3d_fused_step_equals_the_two_kernels(ps, oracle, dtn, n):
    """ps_acoustic3d_step (one kernel, V and P -> V2 and P2) against the oracle's compute_V! then
    compute_P!, bit for bit over 12 steps, every array (faces outside @inn included)."""
    dt = DT[dtn]
    P, (Vx, Vy, Vz), (dx, dy, dz), dts = _acoustic_setup(n, dt)
    k, rho = 1.3, 0.9
    cur = [ps.from_host(a) for a in (Vx, Vy, Vz, P)]
    nxt = [ps.zeros(*a.shape, dtype=dt) for a in (Vx, Vy, Vz, P)]
    for _ in range(12):
        oracle.acoustic3d_v(Vx, Vy, Vz, P, dts, rho, dx, dy, dz)
        oracle.acoustic3d_p(P, Vx, Vy, Vz, dts, k, dx, dy, dz)
        ps.kernels.acoustic3d_step(*cur, *nxt, dts, rho, k, dx, dy, dz)
        cur, nxt = nxt, cur
    for a, d in zip((Vx, Vy, Vz, P), cur):
        assert np.array_equal(ps.to_host(d), a)


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("nt", [7, 8])
def test_acoustic3d_run_in_place(ps, oracle, nt, dtn):
    """ps_acoustic3d_run: FP32 alternates with the library's second set (odd nt copies back), IEEE
    FP64 runs the two kernels in place; both equal the oracle's loop bit for bit."""
    n = (40, 35, 45)
    P, (Vx, Vy, Vz), (dx, dy, dz), dts = _acoustic_setup(n, DT[dtn], seed=5)
    d = [ps.from_host(a) for a in (Vx, Vy, Vz, P)]
    for _ in range(nt):
        oracle.acoustic3d_v(Vx, Vy, Vz, P, dts, 1.0, dx, dy, dz)
        oracle.acoustic3d_p(P, Vx, Vy, Vz, dts, 1.0, dx, dy, dz)
    ps.kernels.acoustic3d_run(*d, dts, 1.0, 1.0, dx, dy, dz, nt)
    for a, x in zip((Vx, Vy, Vz, P), d):
        assert np.array_equal(ps.to_host(x), a)


def test_acoustic3d_split_within_1e12_of_ieee(ps):
    """FP32-pair arithmetic on FP64 arrays against the IEEE run: 200 steps at 64^3 within 1e-12
    (relative max-norm per array); faces outside @inn keep their bits."""
    n = (64, 64, 64)
    P, Vs, (dx, dy, dz), dts = _acoustic_setup(n, np.float64, seed=7)
    out = {}
    for fp64 in ("ieee", "split"):
        d = [ps.from_host(a) for a in (*Vs, P)]
        ps.kernels.acoustic3d_run(*d, dts, 1.0, 1.0, dx, dy, dz, 200, fp64=fp64)
        out[fp64] = [ps.to_host(x) for x in d]
    for a, b in zip(out["ieee"], out["split"]):
        e = np.abs(a - b).max() / np.abs(a).max()
        assert e <= 1e-12, e
    assert not np.array_equal(out["ieee"][3], out["split"][3])  # a different arithmetic really ran
    Vx_i, Vx_s = out["ieee"][0], out["split"][0]
    assert np.array_equal(Vx_i[[0, -1]], Vx_s[[0, -1]])  # faces x = 0, nx are copies


def test_acoustic3d_step_argument_errors(ps):
    d = [ps.zeros(9, 8, 8), ps.zeros(8, 9, 8), ps.zeros(8, 8, 9), ps.zeros(8, 8, 8)]
    e2 = [ps.zeros(9, 8, 8), ps.zeros(8, 9, 8), ps.zeros(8, 8, 9), ps.zeros(8, 8, 8)]
    with pytest.raises(ps.PSError) as e:  # output overlapping an input
        ps.kernels.acoustic3d_step(*d, e2[0], e2[1], e2[2], d[3], 0.1, 1, 1, 1, 1, 1)
    assert e.value.status == -1
    with pytest.raises(ps.PSError) as e:  # wrong Vy2 shape
        ps.kernels.acoustic3d_step(*d, e2[0], ps.zeros(8, 8, 8), e2[2], e2[3], 0.1, 1, 1, 1, 1, 1)
    assert e.value.status == -3
    f = [ps.zeros(9, 8, 8, dtype=np.float32), ps.zeros(8, 9, 8, dtype=np.float32), ps.zeros(8, 8, 9, dtype=np.float32),
         ps.zeros(8, 8, 8, dtype=np.float32)]
    with pytest.raises(ps.PSError) as e:
        ps.kernels.acoustic3d_run(*f, 0.1, 1, 1, 1, 1, 1, 2, fp64="split")
    assert e.value.status == -12


@pytest.mark.parametrize("b", [40.0 / 14, 40.0 / 254, 0.1, 3.0, 1.0 / 3.0, 7.0, -0.37, 1e-5, 1e5, 1e-7, 2.0 ** 20, 1.5])
def test_constant_division_equals_ieee_division(ps, b):
    """The kernels' division by a host-known number (Markstein's method) against the IEEE division
    on the device: FP32 every significand of 12 binades, both signs; FP64 2^25 hashed dividends
    per seed. Divisors outside the method's range (1e-7 in FP32) take the IEEE division."""
    import ctypes

    from ps_gb300 import _lib

    for dtype, n in ((1, 0), (0, 1 << 25)):  # PS_F32, PS_F64
        bad = ctypes.c_int64(-1)
        _lib.call("ps_check_division", float(b), dtype, n, 12345, ctypes.byref(bad), None)
        assert bad.value == 0, (b, dtype, bad.value)
