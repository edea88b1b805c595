"""The TMA variant of run-time compiled 3-D sweeps (ps_jit_launch_tma): read-only stencil arrays
staged plane by plane in shared memory. Its results must equal the plain launch's (one point per
thread) and the register sweep's bit for bit, on extents that are not multiples of the tile, with
short and long sweeps; arrays that break TMA's 16-byte rules fall back to the register sweep."""
import numpy as np
import pytest

import jit_kernels as K

pytestmark = pytest.mark.gpu


def _dev(ps, a):
    return ps.from_host(np.asfortranarray(a))


def _case(ps, name, n, dt, rng):
    import bench

    src = bench.JIT_FLUX_LAM.format(opt="") if name == "FLUX_LAM" else getattr(K, name)
    r = lambda *sh: _dev(ps, rng.standard_normal(sh).astype(dt))  # noqa: E731
    p = lambda *sh: _dev(ps, (rng.random(sh) + 0.5).astype(dt))  # noqa: E731
    if name == "BLEND3D":
        ins, outs, sc = [r(*n), r(*n), p(*n)], [(n[0] - 2, n[1] - 2, n[2] - 2)], (0.3,)
    elif name == "TWO3D":
        ins, outs, sc = [r(*n)], [(n[0] - 2, n[1] - 2, n[2] - 1), n], (0.7,)
    elif name == "FACES3D":
        ins, outs, sc = [r(*n), r(*n)], [n], (0.25,)
    elif name == "FLUX_LAM":
        ins, outs, sc = [r(*n), p(*n), p(*n)], [n], (1e-3, 9.0, 11.0, 13.0)
    else:
        ins, outs, sc = [r(*n), p(*n)], [n], (0.7, 1e-3, 9.0, 11.0, 13.0)
    return src, ins, outs, sc


def _run(ps, k, name, ins, outs, sc, dt, **kw):
    o = [ps.zeros(*sh, dtype=dt) for sh in outs]
    if name == "TWO3D":
        args = [o[0], o[1], ins[0], *sc]
    else:
        args = [*o, *ins, *sc]
    ps.parallel(k, *args, **kw)
    return [ps.to_host(x) for x in o]


def _used_tma(k):
    return k.tma_launches > 0


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", ["HEAT_FLUX", "HEAT_LAP", "BLEND3D", "TWO3D", "FACES3D", "FLUX_LAM"])
def test_tma_sweep_is_bit_identical(ps, name, dt):
    rng = np.random.default_rng(41)
    for n, loops in (((40, 33, 29), (0, 3, 64)), ((128, 96, 70), (0, 16))):
        src, ins, outs, sc = _case(ps, name, n, dt, rng)
        k = ps.parallel_kernel(src)
        ref = _run(ps, k, name, ins, outs, sc, dt, memopt=False)
        for ls in loops:
            k.tma = "always"  # FP64 too (by default FP64 kernels keep the register sweep)
            got = _run(ps, k, name, ins, outs, sc, dt, memopt=True, loopsize=ls)
            for a, b in zip(got, ref):
                assert np.array_equal(a, b), (name, n, ls)
        assert _used_tma(k), name
        k.tma = False
        got = _run(ps, k, name, ins, outs, sc, dt, memopt=True)
        k.tma = True
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (name, n, "register sweep")
        before = k.tma_launches
        _run(ps, k, name, ins, outs, sc, dt, memopt=True)
        assert (k.tma_launches > before) == (dt == np.float32), "default: TMA for FP32 arrays only"


def test_tma_sweep_split_fp64_matches_the_register_sweep(ps):
    """fp64="split" (FP32-pair arithmetic on FP64 arrays): the staged sweep gives the register
    sweep's bits."""
    rng = np.random.default_rng(43)
    src, ins, outs, sc = _case(ps, "FLUX_LAM", (64, 40, 33), np.float64, rng)
    k = ps.parallel_kernel(src)
    k.tma = "always"
    got = _run(ps, k, "FLUX_LAM", ins, outs, sc, np.float64, memopt=True, fp64="split")
    assert _used_tma(k)
    k.tma = False
    ref = _run(ps, k, "FLUX_LAM", ins, outs, sc, np.float64, memopt=True, fp64="split")
    k.tma = True
    assert np.array_equal(got[0], ref[0])


def test_tma_sweep_out_of_bounds_reads_still_reported(ps):
    """A statement whose stencil reaches past an input array is reported (BoundsError), as by the
    register sweep: staging reads zeros there, the bounds check does not depend on it."""
    from ps_gb300 import PSError

    src = "@parallel function oob!(R, A)\n    @inn(R) = @d2_zi(A)\n    return\nend"
    k = ps.parallel_kernel(src)
    R, A = ps.zeros(40, 12, 12, dtype=np.float32), ps.rand(40, 12, 10, dtype=np.float32, seed=3)
    with pytest.raises(PSError, match="BoundsError"):
        ps.parallel(k, R, A, memopt=True)


def test_tma_sweep_falls_back_for_unaligned_arrays(ps):
    """An x extent whose row is not a multiple of 16 bytes (FP64 nx = 37) cannot be staged: the
    register sweep runs, with the same results."""
    rng = np.random.default_rng(47)
    src, ins, outs, sc = _case(ps, "HEAT_LAP", (37, 20, 19), np.float64, rng)
    k = ps.parallel_kernel(src + "\n")  # a fresh kernel object (the cache is keyed by source)
    k.tma = "always"
    got = _run(ps, k, "HEAT_LAP", ins, outs, sc, np.float64, memopt=True)
    ref = _run(ps, k, "HEAT_LAP", ins, outs, sc, np.float64, memopt=False)
    assert not _used_tma(k)
    assert np.array_equal(got[0], ref[0])
