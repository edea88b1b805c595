"""`@parallel ∇` on the GPU: derivative kernels of run-time compiled kernels (ps_gb300.ad) against
the checker (the interpreter on Dual numbers: shadows after = J^T / J shadows before), the
reference's own numerical AD test, and the hand-written adjoint of the diffusion step."""
import numpy as np
import pytest

import ad_kernels as K

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 1e-4}  # relative max-norm; FP32 against the FP64 checker


def _rel(got, ref):
    return float(np.abs(got - ref).max() / max(1e-300, np.abs(ref).max()))


def test_reference_ad_testset(ps):
    """test/ParallelKernel/test_parallel.jl "@parallel ∇ (numerical)": N = 16, a = 6.5, Ā = B̄ = ones
    -> Ā stays 1, B̄ = 1 + a * 100.65; the primal update A += a*B*100.65 happens too."""
    N, a = 16, 6.5
    rng = np.random.default_rng(1)
    A0, B0 = rng.random(N), rng.random(N)
    k = ps.parallel_kernel(K.REF_F, 1)
    A, B = ps.from_host(A0), ps.from_host(B0)
    Ab, Bb = ps.ones(N), ps.ones(N)
    ps.parallel(k, A, B, a, grad=((A, Ab), (B, Bb)))
    assert np.array_equal(ps.to_host(Ab), np.ones(N))
    assert np.array_equal(ps.to_host(Bb), np.full(N, 1.0 + a * 100.65))
    assert np.array_equal(ps.to_host(A), A0 + a * B0 * 100.65)
    assert np.array_equal(ps.to_host(B), B0)


def test_reference_kernel_forward_mode(ps):
    """The reference's AD kernel in forward mode (ad_mode=Enzyme.Forward): tangents of A and B at
    one give the new A's tangent 1 + a*100.65; B's stays 1."""
    N, a = 16, 6.5
    rng = np.random.default_rng(2)
    A0, B0 = rng.random(N), rng.random(N)
    k = ps.parallel_kernel(K.REF_F, 1)
    A, B = ps.from_host(A0), ps.from_host(B0)
    Ad, Bd = ps.ones(N), ps.ones(N)
    ps.parallel(k, A, B, a, grad=((A, Ad), (B, Bd)), ad_mode="forward")
    assert np.array_equal(ps.to_host(Ad), np.full(N, 1.0 + a * 100.65))
    assert np.array_equal(ps.to_host(Bd), np.ones(N))
    assert np.array_equal(ps.to_host(A), A0 + a * B0 * 100.65)


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("mode", ["reverse", "forward"])
@pytest.mark.parametrize("name", sorted(K.KERNELS))
def test_derivative_kernel_vs_checker(ps, name, mode, dtype):
    from oracle import jit_reference as jr

    src, nd, _, dup, _ = K.KERNELS[name]
    argnames, args64 = K.arrays(name, np.float64)
    pos = [argnames.index(d) for d in dup]
    jac = jr.jacobian(src, args64, pos, ndims=nd)
    rng = np.random.default_rng(5)
    sh0 = {p: np.asfortranarray(rng.standard_normal(np.shape(args64[p]))) for p in pos}
    want = (jr.reverse_shadows if mode == "reverse" else jr.forward_shadows)(jac, sh0)
    k = ps.parallel_kernel(src, nd)
    dev = [ps.from_host(a.astype(dtype)) if isinstance(a, np.ndarray) else a for a in args64]
    # the primal kernel alone, for the primal stores of the derivative kernel
    prim = [ps.from_host(a.astype(dtype)) if isinstance(a, np.ndarray) else a for a in args64]
    ps.parallel(k, *prim)
    shd = {p: ps.from_host(sh0[p].astype(dtype)) for p in pos}
    ps.parallel(k, *dev, grad=tuple((dev[p], shd[p]) for p in pos), ad_mode=mode)
    for p in pos:
        got = ps.to_host(shd[p])
        assert _rel(got, want[p]) <= TOL[dtype], (name, mode, argnames[p], _rel(got, want[p]))
    for i, a in enumerate(dev):
        if isinstance(a, (int, float)):
            continue
        assert np.array_equal(ps.to_host(a), ps.to_host(prim[i])), (name, argnames[i])
        if dtype == np.float64 and i in pos:  # the host's libm (sqrt, tanh, pow) may differ in the last bits
            assert _rel(ps.to_host(a), jac[i][0]) <= 1e-14, (name, argnames[i])


def test_reverse_diffusion_step_equals_hand_written_adjoint(ps):
    """The generated reverse kernel of the flux-form step against ps_diffusion3d_adjoint_step (its
    T̄ on inner cells, its lam̄ everywhere), 64 x 48 x 40 FP64."""
    src = K.KERNELS["diffusion_flux_lam"][0]
    n = (64, 48, 40)
    rng = np.random.default_rng(9)
    T0 = np.asfortranarray(rng.random(n))
    lam0 = np.asfortranarray(1 + 0.5 * rng.random(n))
    Ci0 = np.asfortranarray(0.5 + rng.random(n))
    w = np.asfortranarray(rng.standard_normal(n))
    h = (1.3, 0.9, 1.1)
    dt = 0.01
    T, lam, Ci, T2 = ps.from_host(T0), ps.from_host(lam0), ps.from_host(Ci0), ps.from_host(T0)
    T2b, Tb, lamb = ps.from_host(w), ps.zeros(*n), ps.zeros(*n)
    k = ps.parallel_kernel(src, 3)
    ps.parallel(k, T2, T, Ci, lam, dt, *h, grad=((T2, T2b), (T, Tb), (lam, lamb)))
    lT, gl = ps.zeros(*n), ps.zeros(*n)
    ps.adjoint.adjoint_step(lT, ps.from_host(w), ps.from_host(T0), ps.from_host(Ci0), ps.from_host(lam0), gl, dt, *h)
    inner = (slice(1, -1),) * 3
    assert _rel(ps.to_host(Tb)[inner], ps.to_host(lT)[inner]) <= 1e-12
    assert _rel(ps.to_host(lamb), ps.to_host(gl)) <= 1e-12
    # T2's shadow is consumed on the cells the step writes and kept elsewhere
    t2b = ps.to_host(T2b)
    assert np.all(t2b[inner] == 0)
    edge = np.ones(n, bool)
    edge[inner] = False
    assert np.array_equal(t2b[edge], w[edge])


def test_derivative_refusals_launch_nothing(ps):
    from ps_gb300.core import ArgumentError

    A, B = ps.rand(16, seed=1), ps.rand(16, seed=2)
    Ab = ps.zeros(16)
    before = ps.to_host(A)
    race = ps.parallel_kernel("@parallel_indices (ix) function r!(A, B)\n    A[ix] = A[ix+1] + B[ix]\n    return\nend", 1)
    with pytest.raises(ArgumentError, match="race"):
        ps.parallel(race, A, B, grad=((A, Ab),))
    k = ps.parallel_kernel(K.REF_F, 1)
    with pytest.raises(ArgumentError, match="shape"):
        ps.parallel(k, A, B, 1.0, grad=((A, ps.zeros(15)),))
    with pytest.raises(ArgumentError, match="not an array argument"):
        ps.parallel(k, A, B, 1.0, grad=((ps.zeros(16), Ab),))
    with pytest.raises(ArgumentError, match="run-time compiled"):
        ps.parallel(ps.kernels.copy3D, A, B, A, grad=((A, Ab),))
    assert np.array_equal(ps.to_host(A), before) and np.all(ps.to_host(Ab) == 0)


def test_misfit_gradient_32_through_generated_reverse_kernels(ps):
    """Config 4's gradient check at 32^3 with Enzyme's semantics: dL/dlam of L = 0.5||T_nt - T_obs||^2
    over 200 flux-lam steps, built by chaining the generated reverse kernel of the step (`@parallel
    ∇=(T2->λ, T->T̄, lam->lam̄)`) backwards through the stored states, against the hand-written
    checkpointed adjoint (ps_diffusion3d_misfit_gradient). lam = exp(0.3 g), g a Gaussian random
    field (sigma 8 cells); T_obs from lam (1 + 0.05 h)."""
    import torch

    n, nt = 32, 200
    src = K.KERNELS["diffusion_flux_lam"][0]
    k = ps.parallel_kernel(src, 3)

    def grf(seed):
        gen = torch.Generator(device="cuda").manual_seed(seed)
        w = torch.randn((n, n, n), generator=gen, device="cuda", dtype=torch.float64)
        f = torch.fft.fftfreq(n, device="cuda", dtype=torch.float64)
        kx, ky, kz = torch.meshgrid(f, f, f, indexing="ij")
        g = torch.fft.ifftn(torch.fft.fftn(w) * torch.exp(-2 * (torch.pi * 8.0) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))).real
        return (g - g.mean()) / g.std()

    def dev(t):
        A = ps.empty(n, n, n)
        A.copy_(t)
        return A

    x = torch.linspace(0, 10, n, device="cuda", dtype=torch.float64)
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    T0 = dev(1.7 * torch.exp(-((X - 5) ** 2 + (Y - 5) ** 2 + (Z - 5) ** 2)))
    lam = dev(torch.exp(0.3 * grf(4)))
    lam_obs = dev(torch.exp(0.3 * grf(4)) * (1 + 0.05 * grf(5)))
    Ci = ps.ones(n, n, n)
    h = ((n - 1) / 10.0,) * 3
    dt = (10.0 / (n - 1)) ** 2 / float(lam_obs.max()) / 8.1
    _, _, T_obs, _ = ps.adjoint.misfit_gradient(T0, T0, Ci, lam_obs, dt, h, nt, return_final=True)
    loss_h, g_h, _ = ps.adjoint.misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt, checkpoint_every=20)
    # forward: every state kept (the time loop of the examples, T2 starting as a copy of T)
    states = [T0.clone()]
    T2 = T0.clone()
    for _ in range(nt):
        T2.copy_(states[-1])
        ps.parallel(k, T2, states[-1], Ci, lam, dt, *h)
        states.append(T2.clone())
    assert abs(0.5 * float(((states[-1] - T_obs) ** 2).sum()) - loss_h) <= 1e-12 * loss_h
    # reverse: λ_nt = T_nt - T_obs; per step T̄ = J^T λ on all cells, the boundary (copied through the
    # loop) keeps its λ in T2's shadow
    lamb = states[-1].clone()
    lamb.sub_(T_obs)
    glam, Tb, scratch = ps.zeros(n, n, n), ps.zeros(n, n, n), ps.empty(n, n, n)
    for s in range(nt - 1, -1, -1):
        Tb.zero_()
        scratch.copy_(states[s])
        ps.parallel(k, scratch, states[s], Ci, lam, dt, *h, grad=((scratch, lamb), (states[s], Tb), (lam, glam)))
        lamb.add_(Tb)
    assert _rel(ps.to_host(glam), ps.to_host(g_h)) <= 1e-10
