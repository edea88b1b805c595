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
