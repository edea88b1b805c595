"""GPU parity: FD operators, memcopy3D and diffusion3D kernels of libps_b200.so vs the oracle and
the known-answer fixtures. FP64 and FP32 results must be bit-identical to the oracle (the
library is built without FMA contraction, like Julia)."""
import numpy as np
import pytest

from conftest import DT

pytestmark = pytest.mark.gpu


def _dev(ps, a):
    return ps.from_host(np.asfortranarray(a))


def test_fd_every_macro_known_answers(ps, golden):
    meta, arr = golden
    for case in meta["fd"]:
        A = arr[case["key"] + "_A"]
        Rexp = arr[case["key"] + "_R"]
        R = ps.zeros(*Rexp.shape, dtype=DT[case["dtype"]])
        k = ps.fd_kernel(case["statement"], case["ndims"])
        ps.parallel(k, R, _dev(ps, A))
        assert np.array_equal(ps.to_host(R), Rexp), (case["key"], case["statement"])


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_fd_z_sweeps_match_the_oracle(ps, oracle, dtn):
    """3-D macros run as z sweeps with a register window of the planes they read; on a grid wide
    enough for 64 z per thread (600 x 600 x 67: one full sweep and a ragged one) every 3-D macro
    is bit-identical to the oracle, with `@all` and `@inn` left-hand sides."""
    from ps_gb300.fd import LHS, MACROS

    n = (600, 600, 67)
    A = np.asfortranarray(np.random.default_rng(11).standard_normal(n).astype(DT[dtn]) + 3.0)
    dA = _dev(ps, A)
    done = 0
    for op, (kind, opd, inn) in sorted(MACROS[3].items()):
        for lhs in ("all", "inn"):
            li = LHS[3][lhs]
            shape = tuple(n[k] - ((inn >> k) & 1) - ((opd >> k) & 1) for k in range(3))
            exp = np.asfortranarray(np.full(shape, -7.0, dtype=DT[dtn]))
            oracle.fd_apply(kind, opd, inn, 3, li, exp, A)
            R = _dev(ps, np.full(shape, -7.0, dtype=DT[dtn]))
            ps.parallel(ps.fd_kernel(f"@{lhs}(R) = @{op}(A)"), R, dA)
            assert np.array_equal(ps.to_host(R), exp), (op, lhs)
            del R
            done += 1
    assert done == 2 * len(MACROS[3])


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_fd_2d_y_sweeps_match_the_oracle(ps, oracle, dtn):
    """2-D macros run as the 3-D sweep over (nx, 1, ny) (y as z): every 2-D macro at 700 x 600 is
    bit-identical to the oracle, `@all` and `@inn`."""
    from ps_gb300.fd import LHS, MACROS

    n = (700, 600)
    A = np.asfortranarray(np.random.default_rng(13).standard_normal(n).astype(DT[dtn]) + 3.0)
    dA = _dev(ps, A)
    for op, (kind, opd, inn) in sorted(MACROS[2].items()):
        for lhs in ("all", "inn"):
            shape = tuple(n[k] - ((inn >> k) & 1) - ((opd >> k) & 1) for k in range(2))
            exp = np.asfortranarray(np.full(shape, -7.0, dtype=DT[dtn]))
            oracle.fd_apply(kind, opd, inn, 2, LHS[2][lhs], exp, A)
            R = _dev(ps, np.full(shape, -7.0, dtype=DT[dtn]))
            ps.parallel(ps.fd_kernel(f"@{lhs}(R) = @{op}(A)", 2), R, dA)
            assert np.array_equal(ps.to_host(R), exp), (op, lhs)


def test_fd_split_fp64_close_to_the_oracle(ps, oracle):
    """fp64="split" for FD operator kernels (FP64 arrays, arithmetic on FP32 pairs, the definition
    run-time compiled): every 3-D macro within 1e-12 of the IEEE oracle (relative max-norm); FP32
    arrays keep the hand-written kernel, bit-identical."""
    from ps_gb300.fd import MACROS

    n = (41, 37, 35)
    A = np.asfortranarray(np.random.default_rng(12).random(n) + 0.5)
    dA, dA32 = _dev(ps, A), _dev(ps, A.astype(np.float32))
    for op, (kind, opd, inn) in sorted(MACROS[3].items()):
        shape = tuple(n[k] - ((inn >> k) & 1) - ((opd >> k) & 1) for k in range(3))
        exp = np.asfortranarray(np.full(shape, -7.0))
        oracle.fd_apply(kind, opd, inn, 3, 0, exp, A)
        R = _dev(ps, np.full(shape, -7.0))
        k = ps.fd_kernel(f"@all(R) = @{op}(A)")
        ps.parallel(k, R, dA, fp64="split")
        got = ps.to_host(R)
        err = np.abs(got - exp).max() / np.abs(exp).max()
        assert err <= 1e-12, (op, err)
        exp32 = np.asfortranarray(np.full(shape, -7.0, dtype=np.float32))
        oracle.fd_apply(kind, opd, inn, 3, 0, exp32, np.asfortranarray(A.astype(np.float32)))
        R32 = _dev(ps, np.full(shape, -7.0, dtype=np.float32))
        ps.parallel(k, R32, dA32, fp64="split")
        assert np.array_equal(ps.to_host(R32), exp32), op
    with pytest.raises(ps.ArgumentError):
        ps.parallel(ps.fd_kernel("@all(R) = @av(A)"), R, dA, fp64="split_grid")


def test_fd_out_of_bounds_is_an_error(ps):
    R = ps.zeros(7, 5, 6)
    A = ps.zeros(7, 5, 6)  # @d_xa needs size(A,1) == size(R,1)+1
    with pytest.raises(ps.PSError) as e:
        ps.parallel(ps.fd_kernel("@all(R) = @d_xa(A)"), R, A)
    assert e.value.status == -3


@pytest.mark.parametrize("memopt", [False, True])
@pytest.mark.parametrize("kernel", ["diffusion3D_step_inv", "diffusion3D_step_flux"])
def test_diffusion_known_answers(ps, golden, memopt, kernel):
    """test/test_parallel.jl:411-434 and the memopt diffusion testsets (loopsize=3)."""
    meta, arr = golden
    k = getattr(ps.kernels, kernel)
    for case in meta["diffusion"]:
        dt = DT[case["dtype"]]
        T = _dev(ps, arr[case["key"] + "_T"])
        Ci = _dev(ps, arr[case["key"] + "_Ci"])
        T2 = ps.zeros(*case["n"], dtype=dt)
        ps.parallel(k, T2, T, Ci, 1.0, 1.0, 1.0, 1.0, 1.0, memopt=memopt, loopsize=3 if memopt else 0)
        assert np.array_equal(ps.to_host(T2), arr[case["key"] + "_T2"]), (case["key"], memopt)


@pytest.mark.parametrize("memopt", [False, True])
@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_diffusion_test_project(ps, golden, memopt, dtn):
    """test/test_projects/Diffusion3D: 8^3, 3 steps of examples/diffusion3D_novis_noperf.jl."""
    _, arr = golden
    p = {k.split("_", 2)[2]: v for k, v in arr.items() if k.startswith(f"project8_{dtn}_")}
    lam, dt_, dx, dy, dz = (float(v) for v in p["scalars"])
    T, T2, Ci = _dev(ps, p["T0"]), _dev(ps, p["T0"]), _dev(ps, p["Ci"])
    for _ in range(3):
        ps.parallel(ps.kernels.diffusion3D_step, T2, T, Ci, lam, dt_, dx, dy, dz, memopt=memopt)
        T, T2 = T2, T
    assert np.array_equal(ps.to_host(T), p["T"])


SIZES = [(9, 7, 8), (33, 7, 9), (31, 33, 17), (64, 32, 20), (130, 66, 70), (256, 24, 9)]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("form", [0, 1, 2, 3])
@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_diffusion_vs_oracle(ps, oracle, n, form, dtn):
    dt = DT[dtn]
    rng = np.random.default_rng(hash((n, form, dtn)) % 2**32)
    T = np.asfortranarray(rng.random(n).astype(dt))
    Ci = np.asfortranarray(rng.random(n).astype(dt))
    lam = np.asfortranarray((1 + 0.5 * rng.random(n)).astype(dt))
    h = (1 / (n[0] - 1), 1 / (n[1] - 1), 1 / (n[2] - 1))
    hs = h if form == 0 else tuple(1 / x for x in h)
    dts = min(h) ** 2 / 1.5 / 8.1
    ref = np.asfortranarray(np.full(n, -1, dtype=dt))
    oracle.diffusion3d_step(form, ref, T, Ci, lam if form == 3 else None, 1.3, dts, *hs)
    k = [ps.kernels.diffusion3D_step, ps.kernels.diffusion3D_step_inv, ps.kernels.diffusion3D_step_flux,
         ps.kernels.diffusion3D_step_flux_lam][form]
    dT, dCi, dlam = _dev(ps, T), _dev(ps, Ci), _dev(ps, lam)
    for memopt, loopsize in [(False, 0), (True, 0), (True, 3), (True, 5)]:
        T2 = ps.fill(-1, *n, dtype=dt)
        ps.parallel(k, T2, dT, dCi, dlam if form == 3 else 1.3, dts, *hs, memopt=memopt, loopsize=loopsize)
        got = ps.to_host(T2)
        assert np.array_equal(got, ref), (n, form, dtn, memopt, loopsize, np.abs(got - ref).max())


@pytest.mark.parametrize("memopt", [False, True])
def test_diffusion_explicit_ranges(ps, oracle, memopt):
    n = (40, 36, 30)
    rng = np.random.default_rng(11)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(rng.random(n))
    lo, hi = (3, 5, 2), (27, 30, 20)
    ref = np.asfortranarray(np.zeros(n))
    oracle.diffusion3d_step(1, ref, T, Ci, None, 1.0, 1e-4, 3.0, 3.0, 3.0, lo=lo, hi=hi)
    T2 = ps.zeros(*n)
    ranges = [range(a, b) for a, b in zip(lo, hi)]
    ps.parallel(ps.kernels.diffusion3D_step_inv, T2, _dev(ps, T), _dev(ps, Ci), 1.0, 1e-4, 3.0, 3.0, 3.0,
                memopt=memopt, ranges=ranges)
    assert np.array_equal(ps.to_host(T2), ref)


@pytest.mark.parametrize("n", [(128, 64, 48), (200, 40, 24)])
@pytest.mark.parametrize("memopt", [False, True])
@pytest.mark.parametrize("form", [1, 3])
def test_hide_communication_split_equals_full(ps, oracle, memopt, form, n):
    """src/ParallelKernel/test_hide_communication.jl: split computation == serial computation;
    the communication callback runs once, after the boundary slabs. At 200 cells in x the x slabs
    are widened to whole 64-cell sweep tiles (63 + 73 threads), at 128 they are not."""
    rng = np.random.default_rng(21)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(rng.random(n))
    lam = np.asfortranarray(1 + 0.5 * rng.random(n))
    ref = np.asfortranarray(np.zeros(n))
    oracle.diffusion3d_step(form, ref, T, Ci, lam if form == 3 else None, 1.0, 1e-4, 5.0, 5.0, 5.0)
    k = ps.kernels.diffusion3D_step_inv if form == 1 else ps.kernels.diffusion3D_step_flux_lam
    T2 = ps.zeros(*n)
    calls = []
    ps.hide_communication((16, 2, 2), k, (T2, _dev(ps, T), _dev(ps, Ci), _dev(ps, lam) if form == 3 else 1.0, 1e-4,
                                          5.0, 5.0, 5.0), comm=lambda: calls.append(1), memopt=memopt)
    assert calls == [1]
    assert np.array_equal(ps.to_host(T2), ref)


@pytest.mark.parametrize("form", [1, 3])
def test_hide_communication_split_fp64_equals_one_launch(ps, form):
    """fp64="split": the boundary slabs and the inner box give the one launch's values bit for bit
    (each cell's arithmetic does not depend on the box it is computed in)."""
    n = (200, 40, 24)
    rng = np.random.default_rng(22)
    T, Ci, lam = rng.random(n), rng.random(n), 1 + 0.5 * rng.random(n)
    k = ps.kernels.diffusion3D_step_inv if form == 1 else ps.kernels.diffusion3D_step_flux_lam
    args = lambda T2: (T2, _dev(ps, T), _dev(ps, Ci), _dev(ps, lam) if form == 3 else 1.0, 1e-4, 5.0, 5.0, 5.0)  # noqa: E731
    A, B = ps.zeros(*n), ps.zeros(*n)
    ps.parallel(k, *args(A), memopt=True, fp64="split")
    ps.hide_communication((16, 2, 2), k, args(B), comm=lambda: None, memopt=True, fp64="split")
    assert np.array_equal(ps.to_host(A), ps.to_host(B))


@pytest.mark.parametrize("memopt,fp64", [(True, "ieee"), (True, "split"), (False, "ieee")])
def test_hide_communication_boundary_is_done_when_comm_runs(ps, oracle, memopt, fp64):
    """What `comm` sees: a full copy of T2 taken inside the callback holds the final values on the
    boundary cells. memopt (one boundary-first launch, each boundary tile counted in host-mapped
    memory): cells 1 .. bw and n-1-bw .. n-2 of every axis; the separate slab launches: the
    reference's ranges, cells 1 .. bw and n-bw+1 .. n-2 (src/ParallelKernel/hide_communication.jl:350-394)."""
    n, bw = (256, 96, 80), (16, 2, 2)
    rng = np.random.default_rng(23)
    T, Ci, lam = (np.asfortranarray(a) for a in (rng.random(n), rng.random(n), 1 + 0.5 * rng.random(n)))
    ref = np.asfortranarray(np.zeros(n))
    oracle.diffusion3d_step(3, ref, T, Ci, lam, 1.0, 1e-4, 5.0, 5.0, 5.0)
    T2 = ps.zeros(*n)
    snaps = []
    ps.hide_communication(bw, ps.kernels.diffusion3D_step_flux_lam, (T2, _dev(ps, T), _dev(ps, Ci), _dev(ps, lam),
                                                                     1e-4, 5.0, 5.0, 5.0),
                          comm=lambda: snaps.append(ps.to_host(T2)), memopt=memopt, fp64=fp64)
    final = ps.to_host(T2)
    if fp64 == "ieee":
        assert np.array_equal(final, ref)
    snap = snaps[0]
    inner = [np.arange(1, m - 1) for m in n]
    for d in range(3):
        hi0 = n[d] - 1 - bw[d] if memopt else n[d] - bw[d] + 1
        for cells in (np.arange(1, bw[d] + 1), np.arange(hi0, n[d] - 1)):
            if cells.size == 0:
                continue
            idx = list(inner)
            idx[d] = cells
            sel = np.ix_(*idx)
            assert np.array_equal(snap[sel], final[sel]), (d, cells[0])


def test_hide_communication_invalid_width(ps):
    T = ps.zeros(16, 16, 16)
    with pytest.raises(ps.PSError):
        ps.hide_communication((8, 2, 2), ps.kernels.diffusion3D_step_inv, (ps.zeros(16, 16, 16), T, T, 1.0, 1.0, 1.0,
                                                                           1.0, 1.0))


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("n", [(512, 16, 9), (33, 7, 9), (5, 3, 2)])
def test_memcopy3d(ps, oracle, dtn, n):
    dt = DT[dtn]
    rng = np.random.default_rng(1)
    T = np.asfortranarray(rng.random(n).astype(dt))
    Ci = np.asfortranarray(rng.random(n).astype(dt))
    ref = np.asfortranarray(np.zeros(n, dtype=dt))
    oracle.memcopy3d(ref, T, Ci)
    T2 = ps.zeros(*n, dtype=dt)
    ps.parallel(ps.kernels.copy3D, T2, _dev(ps, T), _dev(ps, Ci))
    assert np.array_equal(ps.to_host(T2), ref)
    # example values: T .= 1.7; Ci .= 1/2.0 (examples/memcopy3D.jl:25-27)
    T = ps.fill(1.7, *n, dtype=dt)
    Ci = ps.fill(0.5, *n, dtype=dt)
    ps.parallel(ps.kernels.copy3D, T2, T, Ci, memopt=True)
    assert np.all(ps.to_host(T2) == dt(1.7) + dt(0.5))


def test_fp32_error_vs_fp64_oracle(ps, oracle):
    """FP32 fields: error of 50 steps of the lam-array flux form against the FP64 oracle."""
    n = (48, 40, 36)
    rng = np.random.default_rng(2)
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(np.ones(n))
    lam = np.asfortranarray(1 + 0.5 * rng.random(n))
    _dx = n[0] - 1.0
    dts = (1 / _dx) ** 2 / 1.5 / 8.1
    a, b = T.copy(order="F"), T.copy(order="F")
    for _ in range(50):
        oracle.diffusion3d_step(3, b, a, Ci, lam, 0, dts, _dx, _dx, _dx)
        a, b = b, a
    T32, T2_32 = _dev(ps, T.astype(np.float32)), _dev(ps, T.astype(np.float32))
    Ci32, lam32 = _dev(ps, Ci.astype(np.float32)), _dev(ps, lam.astype(np.float32))
    for _ in range(50):
        ps.parallel(ps.kernels.diffusion3D_step_flux_lam, T2_32, T32, Ci32, lam32, dts, _dx, _dx, _dx, memopt=True)
        T32, T2_32 = T2_32, T32
    err = np.abs(ps.to_host(T32).astype(np.float64) - a).max() / np.abs(a).max()
    assert err < 1e-5, err
