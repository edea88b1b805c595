"""GPU parity of the hand-written diffusion adjoint and the checkpointed misfit gradient."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(n, seed=4):
    rng = np.random.default_rng(seed)
    x = [np.linspace(0, 10, m) for m in n]
    X, Y, Z = np.meshgrid(*x, indexing="ij")
    T0 = np.asfortranarray(1.7 * np.exp(-((X - 5) ** 2 + (Y - 5) ** 2 + (Z - 5) ** 2) / 4) + 0.1 * rng.random(n))
    Ci = np.asfortranarray(np.ones(n))
    lam = np.asfortranarray(np.exp(0.3 * rng.standard_normal(n)))
    h = tuple((m - 1) / 10.0 for m in n)
    dt = min(1 / hh for hh in h) ** 2 / lam.max() / 8.1
    return T0, Ci, lam, h, dt


def test_adjoint_step_bit_exact(ps, oracle):
    n = (40, 33, 29)
    T0, Ci, lam, h, dt = _problem(n)
    rng = np.random.default_rng(1)
    lamT2 = np.asfortranarray(rng.standard_normal(n))
    glam0 = np.asfortranarray(rng.standard_normal(n))
    ref_l = np.asfortranarray(np.zeros(n))
    ref_g = glam0.copy(order="F")
    oracle.diffusion3d_adjoint_step(ref_l, lamT2, T0, Ci, lam, ref_g, dt, *h)
    dl, dg = ps.zeros(*n), ps.from_host(glam0)
    ps.adjoint.adjoint_step(dl, ps.from_host(lamT2), ps.from_host(T0), ps.from_host(Ci), ps.from_host(lam), dg, dt,
                            *h)
    assert np.array_equal(ps.to_host(dl), ref_l)
    assert np.array_equal(ps.to_host(dg), ref_g)


@pytest.mark.parametrize("fp64", ["ieee", "split"])
def test_misfit_gradient_vs_oracle_32(ps, oracle, fp64):
    """The comparison size of the inverse-conductivity problem (32^3), 24 steps, checkpoint every 5."""
    n = (32, 32, 32)
    T0, Ci, lam, h, dt = _problem(n)
    lam_obs = np.asfortranarray(lam * (1 + 0.05 * np.random.default_rng(9).standard_normal(n)))
    nt = 24
    T_obs = oracle.misfit_forward(T0, Ci, lam_obs, dt, h, nt)[-1]
    loss_ref, g_ref = oracle.misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt)
    loss, g, Tf, st = ps.adjoint.misfit_gradient(ps.from_host(T0), ps.from_host(T_obs), ps.from_host(Ci),
                                                 ps.from_host(lam), dt, h, nt, checkpoint_every=5, fp64=fp64,
                                                 return_final=True)
    assert st.checkpoints == 5 and st.recomputed_steps == nt - 5
    tol = 0 if fp64 == "ieee" else 1e-11
    assert abs(loss - loss_ref) <= max(tol, 1e-13) * loss_ref
    gg = ps.to_host(g)
    assert np.abs(gg - g_ref).max() <= max(tol, 1e-13) * np.abs(g_ref).max()


@pytest.mark.parametrize("n", [(64, 64, 64), (64, 40, 36)])
def test_misfit_gradient_split_grid_vs_ieee(ps, n):
    """The forward and reverse sweeps on fixed power-of-two grids (the adjoint state μ = dt Ci λ
    on its own grid) against the IEEE gradient: loss within 1e-12, gradient within 1e-11 relative
    max-norm. The gradient inherits the forward states' rounding (<= 2^-47 of max|T| per step)
    through λ_nt = T_nt - T_obs, a difference far smaller than T itself; the split-pair path
    has the same bound."""
    T0, Ci, lam, h, dt = _problem(n, seed=11)
    rng = np.random.default_rng(12)
    nt = 40
    dT0, dCi, dlam = ps.from_host(T0), ps.from_host(Ci), ps.from_host(lam)
    lam_obs = ps.from_host(np.asfortranarray(lam * (1 + 0.05 * rng.standard_normal(n))))
    _, _, T_obs, _ = ps.adjoint.misfit_gradient(dT0, dT0, dCi, lam_obs, dt, h, nt, return_final=True)
    out = {}
    for fp64 in ("ieee", "split_grid"):
        loss, g, Tf, st = ps.adjoint.misfit_gradient(dT0, T_obs, dCi, dlam, dt, h, nt, checkpoint_every=8, fp64=fp64,
                                                     return_final=True)
        assert st.checkpoints == 5 and st.recomputed_steps == nt - 5
        out[fp64] = (loss, ps.to_host(g), ps.to_host(Tf))
    (la, ga, Ta), (lb, gb, Tb) = out["ieee"], out["split_grid"]
    assert abs(la - lb) <= 1e-12 * la, (la, lb)
    e = np.abs(ga - gb).max() / np.abs(ga).max()
    print(f"split_grid gradient {n}: {e:.2e} of max|g| against the IEEE gradient")
    assert e <= 1e-11, e
    assert np.abs(Ta - Tb).max() <= 1e-12 * np.abs(Ta).max()
    assert not np.array_equal(ga, gb)  # a different arithmetic really ran


def test_misfit_gradient_split_grid_falls_back(ps):
    """Odd nx (no TMA) and an unstable dt (values leave the grid) both run the split-pair gradient."""
    for n, f in (((33, 20, 18), 1.0), ((64, 40, 36), 12.0)):
        T0, Ci, lam, h, dt = _problem(n, seed=13)
        dt = dt * f
        dT0, dCi, dlam = ps.from_host(T0), ps.from_host(Ci), ps.from_host(lam)
        T_obs = ps.from_host(np.asfortranarray(T0 * 0.9))
        res = {}
        for fp64 in ("split", "split_grid"):
            loss, g, st = ps.adjoint.misfit_gradient(dT0, T_obs, dCi, dlam, dt, h, 6, checkpoint_every=3, fp64=fp64)
            res[fp64] = (loss, ps.to_host(g))
        la, lb = res["split"][0], res["split_grid"][0]  # the loss is an atomic sum: order may differ
        assert la == lb or abs(la - lb) <= 1e-14 * abs(la), (la, lb)
        assert np.array_equal(res["split"][1], res["split_grid"][1], equal_nan=True)


@pytest.mark.parametrize("fp64", ["ieee", "split_grid"])
def test_misfit_gradient_finite_differences(ps, fp64):
    """Central finite differences on 16 random directions (the inverse problem's check)."""
    n = (48, 48, 48)
    T0, Ci, lam, h, dt = _problem(n, seed=5)
    rng = np.random.default_rng(6)
    nt = 20
    dT0, dCi = ps.from_host(T0), ps.from_host(Ci)
    lam_obs = lam * (1 + 0.05 * rng.standard_normal(n))
    _, _, T_obs, _ = ps.adjoint.misfit_gradient(dT0, dT0, dCi, ps.from_host(np.asfortranarray(lam_obs)), dt, h, nt,
                                                return_final=True)
    loss, g, st = ps.adjoint.misfit_gradient(dT0, T_obs, dCi, ps.from_host(lam), dt, h, nt, checkpoint_every=4,
                                             fp64=fp64)
    gh = ps.to_host(g)
    worst = 0.0
    for _ in range(16):
        v = np.asfortranarray(rng.standard_normal(n))
        eps = 1e-6
        lp = ps.adjoint.misfit_gradient(dT0, T_obs, dCi, ps.from_host(np.asfortranarray(lam + eps * v)), dt, h, nt)[0]
        lm = ps.adjoint.misfit_gradient(dT0, T_obs, dCi, ps.from_host(np.asfortranarray(lam - eps * v)), dt, h, nt)[0]
        fd = (lp - lm) / (2 * eps)
        ad = float(np.sum(gh * v))
        worst = max(worst, abs(fd - ad) / max(abs(ad), 1e-30))
    assert worst < 1e-5, worst


def test_adjoint_step_split_close_to_ieee(ps):
    """The reverse step on FP32 pairs (FP64 arrays) against the IEEE one: ≤ 1e-13 relative max-norm."""
    n = (45, 38, 33)
    T0, Ci, lam, h, dt = _problem(n, seed=7)
    rng = np.random.default_rng(2)
    lamT2 = np.asfortranarray(rng.standard_normal(n) * 1e-3)
    glam0 = np.asfortranarray(rng.standard_normal(n) * 1e-2)
    out = {}
    for fp64 in ("ieee", "split"):
        dl, dg = ps.zeros(*n), ps.from_host(glam0)
        ps.adjoint.adjoint_step(dl, ps.from_host(lamT2), ps.from_host(T0), ps.from_host(Ci), ps.from_host(lam), dg, dt,
                                *h, fp64=fp64)
        out[fp64] = (ps.to_host(dl), ps.to_host(dg))
    for a, b in zip(out["ieee"], out["split"]):
        assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()
    assert not np.array_equal(out["ieee"][0], out["split"][0])  # a different arithmetic really ran
