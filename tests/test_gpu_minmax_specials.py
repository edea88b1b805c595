"""Special values in the FD kernels whose arithmetic takes shortcuts: Julia's max and min in
`@maxloc` / `@minloc` (a NaN operand makes the result NaN, -0.0 orders below 0.0, infinities and
subnormals compare as values) and the harmonic means' shared reciprocals. Fields drawn from
NaN, +-0.0, +-Inf, +-subnormal and a few normal numbers; the hand-written FD kernels and the
run-time compiled ones (one point per thread and as a sweep, FP32 3-D sweeps staged by TMA) against
the oracle, FP64 and FP32, 2-D and 3-D: the same NaN positions and the same bits elsewhere (the
sign of every zero included). NaN payloads are not compared: the GPU's FP32 arithmetic gives the
canonical NaN."""
import numpy as np
import pytest

from conftest import DT

pytestmark = pytest.mark.gpu


def _field(shape, dt, seed):
    tiny = 1e-310 if dt == np.float64 else 1e-40  # subnormal in either type
    vals = np.array([np.nan, -0.0, 0.0, np.inf, -np.inf, tiny, -tiny, 1.0, -1.0, 2.5, -0.0, 0.0], dtype=dt)
    return np.asfortranarray(vals[np.random.default_rng(seed).integers(0, len(vals), size=shape)])


def _same(got, exp, what):
    ng, ne = np.isnan(got), np.isnan(exp)
    assert np.array_equal(ng, ne), what
    ui = np.uint64 if got.dtype == np.float64 else np.uint32
    assert np.array_equal(got[~ng].view(ui), exp[~ne].view(ui)), what


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("op", ["maxloc", "minloc"])
def test_maxloc_minloc_on_special_values(ps, oracle, dtn, nd, op):
    from ps_gb300.fd import LHS, MACROS

    dt = DT[dtn]
    n = (72, 45, 19) if nd == 3 else (152, 90)  # 72 / 152 columns: rows of 16-byte multiples (TMA)
    A = _field(n, dt, 3 + nd)
    dA = ps.from_host(A)
    kind, opd, inn = MACROS[nd][op]
    src = "@parallel function f!(R, A)\n    @{lhs}(R) = @{op}(A)\n    return\nend"
    for lhs in ("all", "inn"):
        shape = tuple(n[k] - ((inn >> k) & 1) - ((opd >> k) & 1) for k in range(nd))
        exp = np.asfortranarray(np.full(shape, -7.0, dtype=dt))
        oracle.fd_apply(kind, opd, inn, nd, LHS[nd][lhs], exp, A)
        assert np.isnan(exp).any() and (np.signbit(exp) & (exp == 0)).any() and ((exp == 0) & ~np.signbit(exp)).any()
        R = ps.from_host(np.full(shape, -7.0, dtype=dt))
        ps.parallel(ps.fd_kernel(f"@{lhs}(R) = @{op}(A)", nd), R, dA)
        _same(ps.to_host(R), exp, (op, lhs, "fd"))
        k = ps.parallel_kernel(src.format(lhs=lhs, op=op), nd)
        for memopt in (False, True):
            R = ps.from_host(np.full(shape, -7.0, dtype=dt))
            ps.parallel(k, R, dA, memopt=memopt)
            _same(ps.to_host(R), exp, (op, lhs, "run-time compiled", memopt))


@pytest.mark.parametrize("dtn", ["f64", "f32"])
@pytest.mark.parametrize("nd", [2, 3])
def test_harmonic_means_on_special_values(ps, oracle, dtn, nd):
    """Every @harm macro on the same special values (1/+-0 = +-Inf, 1/Inf = 0, subnormals whose
    reciprocals overflow, NaN): the kernels invert each corner once and reuse the reciprocal across
    z steps and, in FP64, across lanes; the results equal the oracle's per-corner divisions."""
    from ps_gb300.fd import LHS, MACROS

    dt = DT[dtn]
    n = (72, 45, 19) if nd == 3 else (152, 90)
    A = _field(n, dt, 11 + nd)
    dA = ps.from_host(A)
    ops = sorted(op for op in MACROS[nd] if op.startswith("harm"))
    assert len(ops) >= 3
    for op in ops:
        kind, opd, inn = MACROS[nd][op]
        shape = tuple(n[k] - ((inn >> k) & 1) - ((opd >> k) & 1) for k in range(nd))
        exp = np.asfortranarray(np.full(shape, -7.0, dtype=dt))
        oracle.fd_apply(kind, opd, inn, nd, LHS[nd]["all"], exp, A)
        R = ps.from_host(np.full(shape, -7.0, dtype=dt))
        ps.parallel(ps.fd_kernel(f"@all(R) = @{op}(A)", nd), R, dA)
        _same(ps.to_host(R), exp, (op, "fd"))
