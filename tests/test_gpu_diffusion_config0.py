"""The 3-D heat diffusion correctness workload: 128^3 cells on a 10 x 10 x 10 box, a Gaussian
initial temperature T0 = 1.7 exp(-((x-5)^2 + (y-5)^2 + (z-5)^2)) at the cell coordinates
x = (ix-1) dx, dx = lx/(nx-1) (examples/diffusion3D_novis_noperf.jl:19-28), scalar conductivity
lam = 1, Ci = 1/cp = 1 as an array, dt = min(dx, dy, dz)^2 / lam / cp / 8.1, 100 explicit steps of the
on-the-fly flux form (test/test_parallel.jl:420-426: qx = -lam*@d_xi(T)*_dx, ...,
dTdt = @inn(Ci)*(-@d_xa(qx)*_dx - ...), @inn(T2) = @inn(T) + dt*@all(dTdt)), with T and T2 swapped
after every step as the examples' time loop does (examples/diffusion3D_novis_noperf.jl:43-46).

Bars against the oracle (the C restatement of the reference's Threads-backend kernel) after the
full 100 steps: the IEEE kernels bit-identical, step by step through `parallel` (memopt on and off)
and as one `run` call; the multi-step FP64 modes (`split`, `split_state`, and `split_grid`, the
headline arithmetic) within 1e-12 relative max-norm. Boundary values stay the initial ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 128
NT = 100


@pytest.fixture(scope="module")
def case0(oracle):
    lx = 10.0
    dx = lx / (N - 1)
    x = np.arange(N) * dx
    r2 = (x[:, None, None] - lx / 2) ** 2 + (x[None, :, None] - lx / 2) ** 2 + (x[None, None, :] - lx / 2) ** 2
    T0 = np.asfortranarray(1.7 * np.exp(-r2))
    Ci = np.asfortranarray(np.ones((N, N, N)))
    lam, cp = 1.0, 1.0
    dt = min(dx, dx, dx) ** 2 / lam / cp / 8.1
    sc = (lam, dt, 1 / dx, 1 / dx, 1 / dx)
    a, b = T0.copy(order="F"), T0.copy(order="F")
    for _ in range(NT):
        oracle.diffusion3d_step(2, b, a, Ci, None, *sc)
        a, b = b, a
    return T0, Ci, sc, a


def relerr(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_config0_oracle_is_a_diffusing_gaussian(case0):
    T0, _, _, ref = case0
    assert ref.max() < T0.max()  # the peak decays
    assert np.array_equal(ref[0], T0[0]) and np.array_equal(ref[:, :, -1], T0[:, :, -1])  # Dirichlet


@pytest.mark.parametrize("memopt", [True, False])
def test_config0_step_loop_is_bit_identical(ps, case0, memopt):
    T0, Ci, sc, ref = case0
    dT, dT2, dCi = ps.from_host(T0), ps.from_host(T0), ps.from_host(Ci)
    for _ in range(NT):
        ps.parallel(ps.kernels.diffusion3D_step_flux, dT2, dT, dCi, *sc, memopt=memopt, sync=False)
        dT, dT2 = dT2, dT
    ps.synchronize()
    assert np.array_equal(ps.to_host(dT), ref)


@pytest.mark.parametrize("fp64", ["ieee", "split", "split_state", "split_grid"])
def test_config0_run(ps, case0, fp64):
    T0, Ci, sc, ref = case0
    dT, dT2 = ps.from_host(T0), ps.from_host(T0)
    ps.kernels.run(ps.kernels.diffusion3D_step_flux, dT, dT2, ps.from_host(Ci), *sc, NT, fp64=fp64)
    got = ps.to_host(dT)
    if fp64 == "ieee":
        assert np.array_equal(got, ref)
    else:
        e = relerr(got, ref)
        print(f"config 0, {fp64}, {NT} steps: {e:.3e}")
        assert e <= 1e-12, e
        assert np.array_equal(got[0], T0[0]) and np.array_equal(got[-1], T0[-1])
