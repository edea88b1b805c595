"""GPU parity of run-time compiled kernels (ps_gb300.parallel_kernel: translated to CUDA C and
compiled by NVRTC for sm_103a inside libps_b200.so) against the known-answer fixtures, the
library's hand-written kernels and the CPU interpreter oracle/jit_reference.py.

Bit-exact for + - * / comparisons, max/min and Bool*x in FP64 and FP32 (no FMA contraction on
either side). Kernels that call the math library (exp; pow with a non-literal exponent) are
compared with a tolerance of 4e-15 (FP64) / 2e-6 (FP32) relative to each value plus the same
fraction of the largest value: the device's and the host's libm agree to a few ulp, not bit for bit."""
import ctypes

import numpy as np
import pytest

import jit_kernels as K
from conftest import DT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jr():
    from oracle import jit_reference

    return jit_reference


def _dev(ps, a):
    return ps.from_host(np.asfortranarray(a))


def _fd_src(stmt):
    return f"@parallel function fd_case!(R, A)\n    {stmt}\n    return\nend"


def test_jit_every_fd_macro_fixture(ps, golden):
    meta, arr = golden
    for case in meta["fd"]:
        Rexp = arr[case["key"] + "_R"]
        R = ps.zeros(*Rexp.shape, dtype=DT[case["dtype"]])
        k = ps.parallel_kernel(_fd_src(case["statement"]), ndims=case["ndims"])
        ps.parallel(k, R, _dev(ps, arr[case["key"] + "_A"]))
        assert np.array_equal(ps.to_host(R), Rexp), (case["key"], case["statement"])


@pytest.mark.parametrize("src", [K.HEAT_FLUX, K.HEAT_LAP], ids=["flux_on_the_fly", "second_differences"])
def test_jit_diffusion_fixtures(ps, golden, src):
    meta, arr = golden
    k = ps.parallel_kernel(src)
    for case in meta["diffusion"]:
        T, Ci, T2e = (arr[case["key"] + s] for s in ("_T", "_Ci", "_T2"))
        T2 = ps.zeros(*T.shape, dtype=T.dtype.type)
        k(T2, _dev(ps, T), _dev(ps, Ci), 1.0, 1.0, 1.0, 1.0, 1.0)
        assert np.array_equal(ps.to_host(T2), T2e), case["key"]


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_jit_diffusion_project(ps, golden, dtn):
    _, arr = golden
    p = {k.split("_", 2)[2]: v for k, v in arr.items() if k.startswith(f"project8_{dtn}_")}
    lam, dt_, dx, dy, dz = (float(v) for v in p["scalars"])
    T, T2, Ci = _dev(ps, p["T0"]), _dev(ps, p["T0"]), _dev(ps, p["Ci"])
    k = ps.parallel_kernel(K.HEAT_DIV)
    for _ in range(3):
        ps.parallel(k, T2, T, Ci, lam, dt_, dx, dy, dz)
        T, T2 = T2, T
    assert np.array_equal(ps.to_host(T), p["T"])


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("src,fixed", [(K.HEAT_FLUX, "diffusion3D_step_flux"), (K.HEAT_LAP, "diffusion3D_step_inv"),
                                       (K.HEAT_DIV, "diffusion3D_step")])
def test_jit_equals_hand_written_diffusion(ps, src, fixed, dt):
    """The compiled body and the library's hand-written kernel for the same body agree bit for bit."""
    rng = np.random.default_rng(21)
    n = (37, 33, 29)
    T, Ci = _dev(ps, rng.random(n).astype(dt)), _dev(ps, (rng.random(n) + 0.5).astype(dt))
    sc = (0.7, 1e-3, 9.0, 11.0, 13.0)
    A, B = ps.zeros(*n, dtype=dt), ps.zeros(*n, dtype=dt)
    ps.parallel(ps.parallel_kernel(src), A, T, Ci, *sc)
    for memopt in (False, True):
        ps.fill_(B, 0.0)
        ps.parallel(getattr(ps.kernels, fixed), B, T, Ci, *sc, memopt=memopt)
        assert np.array_equal(ps.to_host(A), ps.to_host(B)), (fixed, memopt)


@pytest.mark.parametrize("opt", ["", "inbounds=true "])
def test_jit_equals_hand_written_flux_lam(ps, opt):
    """The flux form with a conductivity array (face averages @av_xi(lam)) against the library kernel."""
    import bench

    rng = np.random.default_rng(8)
    n = (35, 30, 27)
    T, Ci, lam = (_dev(ps, rng.random(n) + c) for c in (0.0, 0.5, 1.0))
    A, B = ps.zeros(*n), ps.zeros(*n)
    sc = (1e-3, 9.0, 11.0, 13.0)
    ps.parallel(ps.parallel_kernel(bench.JIT_FLUX_LAM.format(opt=opt)), A, T, Ci, lam, *sc)
    ps.parallel(ps.kernels.diffusion3D_step_flux_lam, B, T, Ci, lam, *sc, memopt=True)
    assert np.array_equal(ps.to_host(A), ps.to_host(B))


def _pos(rng, shape, dt):
    return (rng.random(shape) + 0.5).astype(dt)


def _cases(dt, nx=21, ny=17):
    rng = np.random.default_rng(7)
    r = lambda *s: rng.standard_normal(s).astype(dt)  # noqa: E731
    n3 = 12
    return {
        "STRESS2D": ([r(nx, ny), r(nx, ny), r(nx - 1, ny - 1), r(nx, ny), r(nx + 1, ny), r(nx, ny + 1),
                      _pos(rng, (nx, ny), dt), 3.0, 5.0], None),
        "MOMENTUM2D": ([r(nx - 1, ny - 2), r(nx - 2, ny - 1), r(nx - 1, ny - 2), r(nx - 2, ny - 1), r(nx, ny),
                        r(nx, ny), r(nx, ny), r(nx - 1, ny - 1), r(nx, ny), 3.0, 5.0, 9.81, 0.9], None),
        "VELOCITY2D": ([r(nx + 1, ny), r(nx, ny + 1), r(nx - 1, ny - 2), r(nx - 2, ny - 1), _pos(rng, (nx, ny), dt),
                        r(nx - 2, ny - 2), 0.05], None),
        "UPWIND2D": ([r(nx, ny), r(nx, ny), r(nx, ny), r(nx, ny), 0.01, 3.0, 5.0], None),
        "AUGASSIGN": ([r(40), r(40), 0.3], None),
        "LOCAL_FN": ([np.zeros((6, 5, 4), dt)], None),
        "QUALIFIED2D": ([r(nx, ny), r(nx, ny)], None),
        "SPLAT_COPY": ([r(nx, ny), r(nx, ny), 1.5], None),
        "HEAT2D_FD": ([r(nx, ny), r(nx, ny), _pos(rng, (nx, ny), dt), 0.7, 1e-3, 9.0, 11.0], None),
        "WALLS2D": ([r(nx, ny)], [(1, ny)]),
        "BLEND3D": ([r(n3 - 2, n3 - 2, n3 - 2), r(n3, n3, n3), r(n3, n3, n3), _pos(rng, (n3, n3, n3), dt), 0.3],
                    None),
        "FACES3D": ([r(n3, n3 - 1, n3 + 1), r(n3, n3 - 1, n3 + 1), r(n3, n3 - 1, n3 + 1), 0.25], None),
        "ROD1D": ([r(29), r(29), 0.2], None),
        "LINEAR_INDEX": ([np.zeros((4, 5, 6), dt)], None),
        "D2Z3D": ([r(9, 7, 8), r(9, 7, 8)], None),
        "COMPACTION": ([_pos(rng, (nx, ny), dt), r(nx, ny), r(nx, ny), 0.8, 3.0, 0.1], None),
        "BRANCHES2D": ([r(nx, ny), r(nx, ny), 3, 0.5], None),
        "EARLY_RETURN": ([r(40), r(40), 25], None),
    }


_NDIMS = {"ROD1D": 1, "EARLY_RETURN": 1, "AUGASSIGN": 1}
_TOL = {"COMPACTION", "BRANCHES2D"}  # exp / pow


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", sorted(_cases(np.float64)))
def test_jit_kernels_vs_interpreter(ps, jr, name, dt):
    args, ranges = _cases(dt)[name]
    src = getattr(K, name)
    host = [a.copy() if isinstance(a, np.ndarray) else a for a in args]
    jr.run(src, host, ndims=_NDIMS.get(name), ranges=ranges)
    dev = [_dev(ps, a) if isinstance(a, np.ndarray) else a for a in args]
    ps.parallel(ps.parallel_kernel(src, ndims=_NDIMS.get(name)), *dev, ranges=ranges)
    for i, (h, d) in enumerate(zip(host, dev)):
        if not isinstance(h, np.ndarray):
            continue
        got = ps.to_host(d)
        assert got.dtype == dt
        if name in _TOL:
            rtol = 4e-15 if dt == np.float64 else 2e-6
            # absolute part: a few ulp of the largest value (results formed by cancellation)
            np.testing.assert_allclose(got, h, rtol=rtol, atol=rtol * np.abs(h).max(), err_msg=f"{name} arg {i}")
        else:
            assert np.array_equal(got, h), (name, i, np.abs(got - h).max())
    assert any(isinstance(h, np.ndarray) and not np.array_equal(h, a) for h, a in zip(host, args))  # work was done


def test_jit_ranges_select_a_box(ps, jr):
    A = np.zeros((6, 5, 4))
    jr.run(K.LINEAR_INDEX, [A], ranges=[(2, 4), (1, 3), (2, 2)])
    D = ps.zeros(6, 5, 4)
    ps.parallel(ps.parallel_kernel(K.LINEAR_INDEX), D, ranges=[(2, 4), (1, 3), (2, 2)])
    assert np.array_equal(ps.to_host(D), A)
    assert np.count_nonzero(A) == 9


def test_jit_bounds_error_then_recovery(ps):
    from ps_gb300._lib import PSError

    n = 50
    a = np.arange(n, dtype=np.float64)
    A, B = _dev(ps, a), ps.zeros(n)
    k = ps.parallel_kernel(K.SHIFT_OOB)
    with pytest.raises(PSError, match="BoundsError") as e:
        ps.parallel(k, B, A)
    assert e.value.status == -1
    ps.fill_(B, 0.0)
    ps.parallel(k, B, A, ranges=[(1, n - 1)])  # the flag was cleared; a safe range passes
    assert np.array_equal(ps.to_host(B)[:n - 1], a[1:])
    C = ps.zeros(n)
    ps.parallel(ps.parallel_kernel(K.SHIFT_INBOUNDS), C, A, ranges=[(1, n - 1)])
    assert np.array_equal(ps.to_host(C), ps.to_host(B))


def test_jit_async_on_a_stream(ps):
    import torch

    rng = np.random.default_rng(3)
    T = rng.random((40, 30, 20))
    Ci = rng.random((40, 30, 20)) + 0.5
    k = ps.parallel_kernel(K.HEAT_LAP)
    s = torch.cuda.Stream()
    Td, Cd = _dev(ps, T), _dev(ps, Ci)
    A, B = ps.zeros(40, 30, 20), ps.zeros(40, 30, 20)
    ps.synchronize()
    for _ in range(4):  # ping-pong, queued without synchronisation
        ps.parallel_async(k, A, Td, Cd, 1.0, 0.01, 2.0, 2.0, 2.0, stream=s)
        ps.parallel_async(k, B, A, Cd, 1.0, 0.01, 2.0, 2.0, 2.0, stream=s)
        Td, A, B = B, Td, A
    ps.synchronize(s)
    R = _dev(ps, T)
    X, Y = ps.zeros(40, 30, 20), ps.zeros(40, 30, 20)
    for _ in range(4):
        ps.parallel(k, X, R, Cd, 1.0, 0.01, 2.0, 2.0, 2.0)
        ps.parallel(k, Y, X, Cd, 1.0, 0.01, 2.0, 2.0, 2.0)
        R, X, Y = Y, R, X
    assert np.array_equal(ps.to_host(Td), ps.to_host(R))


def test_jit_c_abi_direct(ps):
    """ps_jit_compile / ps_jit_launch with hand-written CUDA C (no translator), and the compile
    error path through ps_last_error."""
    from ps_gb300 import _lib
    from ps_gb300._lib import PSArray
    from ps_gb300.core import descriptor, stream_handle

    src = b"""
struct ps_jit_args { void* a[32]; long long n[32][3]; double s[32]; long long lo[3]; long long cnt[3]; int* err;
                     long long smem; long long loop; };
extern "C" __global__ void twice(const ps_jit_args g) {
    long long i = g.lo[0] + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (threadIdx.y == 0 && i < g.lo[0] + g.cnt[0]) ((double*)g.a[0])[i] = g.s[0] * ((const double*)g.a[1])[i];
}"""
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ps_jit_compile(src, b"twice", ctypes.byref(h)) == 0
    x = np.arange(100, dtype=np.float64)
    X, Y = _dev(ps, x), ps.zeros(100)
    arrs = (PSArray * 2)(descriptor(Y), descriptor(X))
    sc = (ctypes.c_double * 1)(2.5)
    rc = lib.ps_jit_launch(h, arrs, 2, sc, 1, (ctypes.c_int64 * 3)(0, 0, 0), (ctypes.c_int64 * 3)(100, 1, 1),
                           stream_handle(None), 1)
    assert rc == 0
    assert np.array_equal(ps.to_host(Y), 2.5 * x)
    assert lib.ps_jit_destroy(h) == 0
    bad = ctypes.c_void_p()
    assert lib.ps_jit_compile(b"extern \"C\" __global__ void k() { undeclared = 1; }", b"k", ctypes.byref(bad)) == -1
    assert "undeclared" in _lib.last_error()
    assert not bad.value


# ---------------------------------------------------------------- kernel language on the GPU
@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_jit_shared_memory_tile(ps, jr, dt):
    rng = np.random.default_rng(4)
    nx, ny = 256, 64
    T, Ci = rng.random((nx, ny)).astype(dt), (rng.random((nx, ny)) + 0.5).astype(dt)
    sc = (1.0, 1e-3, 7.0, 9.0)
    host = np.zeros((nx, ny), dt)
    jr.run(K.HEAT2D_PLAIN, [host, T, Ci, *sc])
    A, B = ps.zeros(nx, ny, dtype=dt), ps.zeros(nx, ny, dtype=dt)
    Td, Cd = _dev(ps, T), _dev(ps, Ci)
    shmem = 34 * 10 * np.dtype(dt).itemsize
    ps.parallel(ps.parallel_kernel(K.HEAT2D_TILE), A, Td, Cd, *sc, nthreads=(32, 8), shmem=shmem)
    ps.parallel(ps.parallel_kernel(K.HEAT2D_PLAIN), B, Td, Cd, *sc)
    assert np.array_equal(ps.to_host(A), host) and np.array_equal(ps.to_host(B), host)
    # the interpreter runs the tile kernel block by block with real barriers (small case)
    Ts, Cs = T[:64, :16].copy(), Ci[:64, :16].copy()
    hs = np.zeros((64, 16), dt)
    jr.run(K.HEAT2D_TILE, [hs, Ts, Cs, *sc], nthreads=(32, 8), shmem=shmem)
    S = ps.zeros(64, 16, dtype=dt)
    ps.parallel(ps.parallel_kernel(K.HEAT2D_TILE), S, _dev(ps, Ts), _dev(ps, Cs), *sc, nthreads=(32, 8), shmem=shmem)
    assert np.array_equal(ps.to_host(S), hs)


def test_jit_shared_memory_larger_than_48k(ps):
    """Dynamic shared memory above the 48 KB default (the launch opts the function in)."""
    rng = np.random.default_rng(9)
    nx, ny = 256, 64
    T, Ci = rng.random((nx, ny)), rng.random((nx, ny)) + 0.5
    A, B = ps.zeros(nx, ny), ps.zeros(nx, ny)
    sc = (1.0, 1e-3, 7.0, 9.0)
    ps.parallel(ps.parallel_kernel(K.HEAT2D_TILE), A, _dev(ps, T), _dev(ps, Ci), *sc, nthreads=(32, 8),
                shmem=100 * 1024)
    ps.parallel(ps.parallel_kernel(K.HEAT2D_PLAIN), B, _dev(ps, T), _dev(ps, Ci), *sc)
    assert np.array_equal(ps.to_host(A), ps.to_host(B))


def test_jit_int_expression_converted_once(ps):
    """`A[ix, iy] = ix + (iy - 1) * size(A, 1)` into FP32 beyond 2^24: the Int value rounded once to
    Float32, as Julia converts it (real arithmetic on the parts would round the product and the sum)."""
    n = (5003, 4001)
    A = ps.zeros(*n, dtype=np.float32)
    ps.parallel(ps.parallel_kernel(K.INT_EXPR2D), A)
    i, j = np.meshgrid(np.arange(1, n[0] + 1, dtype=np.int64), np.arange(1, n[1] + 1, dtype=np.int64), indexing="ij")
    assert np.array_equal(ps.to_host(A), (i + (j - 1) * n[0]).astype(np.float32))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_jit_shared_memory_offset_and_splat_3d(ps, jr, dt):
    """A @sharedMem view at a byte offset (2 blockDim.x elements, sizeof(eltype(A))) reversing
    each block's rows in x, and the (I...) kernel on 3-D arrays; both against the interpreter."""
    rng = np.random.default_rng(8)
    A = rng.random((64, 16)).astype(dt)
    nt = (16, 4)
    shmem = (16 * 4 + 2 * 16) * np.dtype(dt).itemsize
    host = np.zeros((64, 16), dt)
    jr.run(K.SMEM_OFFSET, [host, A], nthreads=nt, shmem=shmem)
    exp = A.reshape(4, 16, 16)[:, ::-1, :].reshape(64, 16)  # x reversed within each 16-wide block
    assert np.array_equal(host, exp)
    B = ps.zeros(64, 16, dtype=dt)
    ps.parallel(ps.parallel_kernel(K.SMEM_OFFSET), B, _dev(ps, A), nthreads=nt, shmem=shmem)
    assert np.array_equal(ps.to_host(B), exp)
    X = rng.random((9, 7, 5)).astype(dt)
    Y = ps.zeros(9, 7, 5, dtype=dt)
    ps.parallel(ps.parallel_kernel(K.SPLAT_COPY), Y, _dev(ps, X), 1.5)
    hy = np.zeros((9, 7, 5), dt)
    jr.run(K.SPLAT_COPY, [hy, X, 1.5])
    assert np.array_equal(ps.to_host(Y), hy) and np.array_equal(hy, (dt(1.5) * X).astype(dt))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_jit_warp_shuffles_and_votes(ps, jr, dt):
    rng = np.random.default_rng(6)
    n = 1024
    a = rng.standard_normal(n).astype(dt)
    S = np.zeros(n // 32, dt)
    jr.run(K.WARP_SUMS, [S, a], nthreads=(64,))
    Sd = ps.zeros(n // 32, dtype=dt)
    ps.parallel(ps.parallel_kernel(K.WARP_SUMS), Sd, _dev(ps, a), nthreads=(64,))
    assert np.array_equal(ps.to_host(Sd), S)
    B, C, D = (np.zeros(n, dt) for _ in range(3))
    jr.run(K.WARP_OPS, [B, C, D, a, 1.5], nthreads=(64,))
    Bd, Cd, Dd = (ps.zeros(n, dtype=dt) for _ in range(3))
    ps.parallel(ps.parallel_kernel(K.WARP_OPS), Bd, Cd, Dd, _dev(ps, a), 1.5, nthreads=(64,))
    for h, d in ((B, Bd), (C, Cd), (D, Dd)):
        assert np.array_equal(ps.to_host(d), h)


def test_jit_loops_locals_and_block_ids(ps, jr):
    rng = np.random.default_rng(2)
    A = rng.random((37, 9))
    B = np.zeros_like(A)
    jr.run(K.BOX_X, [B, A, 3])
    Bd = ps.zeros(37, 9)
    ps.parallel(ps.parallel_kernel(K.BOX_X), Bd, _dev(ps, A), 3)
    assert np.array_equal(ps.to_host(Bd), B)
    X = np.zeros((16, 8, 4))
    jr.run(K.BLOCK_IDS, [X], nthreads=(8, 4, 2))
    Xd = ps.zeros(16, 8, 4)
    ps.parallel(ps.parallel_kernel(K.BLOCK_IDS), Xd, nthreads=(8, 4, 2))
    assert np.array_equal(ps.to_host(Xd), X)
    Y = ps.zeros(16, 8, 4)  # nblocks .* nthreads threads from index 1
    ps.parallel(ps.parallel_kernel(K.BLOCK_IDS), Y, nblocks=(2, 2, 2), nthreads=(8, 4, 2))
    assert np.array_equal(ps.to_host(Y), X)


def test_jit_partial_blocks_with_barriers_are_refused(ps):
    """A partial block of a kernel with barriers / shuffles never runs: the Python call refuses it,
    and the kernel itself leaves block-uniformly before its first shuffle and reports it."""
    from ps_gb300 import _lib
    from ps_gb300._lib import PSArray
    from ps_gb300.core import ArgumentError, descriptor, stream_handle

    a = np.arange(100, dtype=np.float64)
    A, S = _dev(ps, a), ps.zeros(4)
    k = ps.parallel_kernel(K.WARP_SUMS)
    with pytest.raises(ArgumentError, match="multiple of the thread block"):
        ps.parallel(k, S, A, nthreads=(64,))
    h = k._handle(1, "double")  # the handle the refused call compiled
    arrs = (PSArray * 2)(descriptor(S), descriptor(A))
    rc = _lib.load().ps_jit_launch_ex(h, arrs, 2, (ctypes.c_double * 1)(0.0), 0, (ctypes.c_int64 * 3)(0, 0, 0),
                                      (ctypes.c_int64 * 3)(100, 1, 1), (ctypes.c_int32 * 3)(64, 1, 1), 0, None,
                                      stream_handle(None), 1)
    assert rc == -1 and "multiple of the thread block" in _lib.last_error()
    ps.parallel(k, S, A, ranges=[(1, 64)], nthreads=(64,))  # a full block afterwards runs normally
    assert np.allclose(ps.to_host(S)[:2], a[:64].reshape(2, 32).sum(axis=1))


# ---------------------------------------------------------------- memopt: z sweeps
@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", ["HEAT_FLUX", "HEAT_LAP", "BLEND3D", "TWO3D", "FLUX_LAM"])
def test_jit_memopt_z_sweep_is_bit_identical(ps, name, dt):
    """memopt=true (z sweeps of 1, 3, 16 and 64 indices per thread, registers carried along z) gives
    exactly the plain launch's result, on odd extents, with and without ranges."""
    import bench

    rng = np.random.default_rng(31)
    n = (37, 33, 29)
    src = bench.JIT_FLUX_LAM.format(opt="") if name == "FLUX_LAM" else getattr(K, name)
    r = lambda *sh: _dev(ps, rng.standard_normal(sh).astype(dt))  # noqa: E731
    p = lambda *sh: _dev(ps, (rng.random(sh) + 0.5).astype(dt))  # noqa: E731
    if name == "BLEND3D":
        ins, outs, sc = [r(*n), r(*n), p(*n)], [(n[0] - 2, n[1] - 2, n[2] - 2)], (0.3,)
    elif name == "TWO3D":
        ins, outs, sc = [r(*n)], [(n[0] - 2, n[1] - 2, n[2] - 1), n], (0.7,)
    elif name == "FLUX_LAM":
        ins, outs, sc = [r(*n), p(*n), p(*n)], [n], (1e-3, 9.0, 11.0, 13.0)
    else:
        ins, outs, sc = [r(*n), p(*n)], [n], (0.7, 1e-3, 9.0, 11.0, 13.0)
    k = ps.parallel_kernel(src)

    def launch(memopt, loopsize=0, ranges=None):
        o = [ps.zeros(*sh, dtype=dt) for sh in outs]
        if name == "TWO3D":
            args = [o[0], o[1], ins[0], *sc]
        else:
            args = [*o, *ins, *sc]
        ps.parallel(k, *args, memopt=memopt, loopsize=loopsize, ranges=ranges)
        return [ps.to_host(x) for x in o]

    ref = launch(False)
    for ls in (1, 3, 16, 64):
        got = launch(True, ls)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (name, ls)
    box = [(2, 30), (3, 25), (4, 27)]
    ref_box, got_box = launch(False, ranges=box), launch(True, 5, ranges=box)
    for a, b in zip(got_box, ref_box):
        assert np.array_equal(a, b), (name, "ranges")


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("name", ["STRESS2D", "MOMENTUM2D", "VELOCITY2D", "COMPACTION", "HEAT2D_FD"])
def test_jit_memopt_y_sweep_is_bit_identical(ps, name, dt):
    """2-D `@parallel` kernels with memopt=true (y sweeps of 1, 3, 16 and 64 indices per thread and the
    default, read-only registers carried along y; src/memopt.jl's loopdim 2) give exactly the plain
    launch's result, over several blocks in x and y, with explicit nthreads and with ranges."""
    args, _ = _cases(dt, nx=300, ny=133)[name]
    k = ps.parallel_kernel(getattr(K, name))

    def launch(memopt, loopsize=0, ranges=None, nthreads=None):
        dev = [_dev(ps, a) if isinstance(a, np.ndarray) else a for a in args]
        ps.parallel(k, *dev, memopt=memopt, loopsize=loopsize, ranges=ranges, nthreads=nthreads)
        return [ps.to_host(d) for d in dev if not isinstance(d, float)]

    ref = launch(False)
    for ls in (0, 1, 3, 16, 64):
        for a, b in zip(launch(True, ls), ref):
            assert np.array_equal(a, b), (name, ls)
    assert (2, "double" if dt == np.float64 else "float", True, False) in k._handles
    for a, b in zip(launch(True, 5, nthreads=(64, 4)), ref):  # the sweep dimension's threads become 1
        assert np.array_equal(a, b), (name, "nthreads")
    box = [(2, 250), (3, 120)]
    for a, b in zip(launch(True, 7, ranges=box), launch(False, ranges=box)):
        assert np.array_equal(a, b), (name, "ranges")


def test_jit_memopt_from_the_definition(ps):
    """`@parallel memopt=true loopsize=3 function ...` selects the z sweep by itself."""
    src = K.HEAT_LAP.replace("@parallel function", "@parallel memopt=true loopsize=3 function")
    k = ps.parallel_kernel(src)
    assert k.kd.options == {"memopt": "true", "loopsize": "3"}
    rng = np.random.default_rng(2)
    T, Ci = _dev(ps, rng.random((40, 21, 19))), _dev(ps, rng.random((40, 21, 19)) + 0.5)
    A, B = ps.zeros(40, 21, 19), ps.zeros(40, 21, 19)
    ps.parallel(k, A, T, Ci, 0.7, 1e-3, 9.0, 11.0, 13.0)
    ps.parallel(ps.kernels.diffusion3D_step_inv, B, T, Ci, 0.7, 1e-3, 9.0, 11.0, 13.0, memopt=False)
    assert np.array_equal(ps.to_host(A), ps.to_host(B))
    # (ndims, type, z sweep, split arithmetic[, "tma": the variant with staged stencil arrays])
    assert any(key[:4] == (3, "double", True, False) for key in k._handles)


@pytest.mark.parametrize("name", ["HEAT_FLUX", "TWO3D"])
@pytest.mark.parametrize("n", [(64, 40, 36), (100, 40, 36)])
def test_jit_hide_communication_equals_one_launch(ps, name, n):
    """@hide_communication with a run-time compiled kernel: the six boundary boxes and the inner box
    on two streams give the one-launch result; comm runs once, after the boundary boxes. At 100
    in x the x slabs are widened to whole 32-thread blocks, at 64 they are not."""
    rng = np.random.default_rng(17)
    k = ps.parallel_kernel(getattr(K, name))
    if name == "HEAT_FLUX":
        T, Ci = _dev(ps, rng.random(n)), _dev(ps, rng.random(n) + 0.5)
        mk = lambda: [ps.zeros(*n)]  # noqa: E731
        rest = [T, Ci, 0.7, 1e-3, 9.0, 11.0, 13.0]
    else:
        B = _dev(ps, rng.standard_normal(n))
        mk = lambda: [ps.zeros(n[0] - 2, n[1] - 2, n[2] - 1), ps.zeros(*n)]  # noqa: E731
        rest = [B, 0.7]
    ref, out = mk(), mk()
    ps.parallel(k, *ref, *rest)
    calls = []
    ps.hide_communication((16, 4, 2), k, (*out, *rest), comm=lambda: calls.append(1))
    assert calls == [1]
    for a, b in zip(ref, out):
        assert np.array_equal(ps.to_host(a), ps.to_host(b))
    with pytest.raises(ps.ArgumentError, match="boundary_width"):
        ps.hide_communication((n[0] // 2, 4, 2), k, (*out, *rest))
    # split FP64 arithmetic through the boxes: the one split launch's values
    ref2, out2 = mk(), mk()
    ps.parallel(k, *ref2, *rest, fp64="split")
    ps.hide_communication((16, 4, 2), k, (*out2, *rest), comm=None, fp64="split")
    for a, b in zip(ref2, out2):
        assert np.array_equal(ps.to_host(a), ps.to_host(b))
    assert not np.array_equal(ps.to_host(ref2[-1]), ps.to_host(ref[-1]))


@pytest.mark.parametrize("fp64", ["ieee", "split"])
def test_jit_hide_communication_boundary_is_done_when_comm_runs(ps, fp64):
    """The boundary-first launch of a run-time compiled kernel: a full copy of T2 taken inside the
    callback holds the final values on the boundary cells of the reference's ranges (thread indices
    t < bw or t >= n - bw, i.e. @inn cells 1 .. bw and n-bw+1 .. n-2)."""
    n, bw = (256, 96, 80), (16, 2, 2)
    rng = np.random.default_rng(19)
    k = ps.parallel_kernel(K.HEAT_FLUX)
    assert k.hide_eligible()
    T, Ci = _dev(ps, rng.random(n)), _dev(ps, rng.random(n) + 0.5)
    rest = [T, Ci, 0.7, 1e-3, 9.0, 11.0, 13.0]
    ref, out = ps.zeros(*n), ps.zeros(*n)
    ps.parallel(k, ref, *rest, fp64=fp64)
    snaps = []
    ps.hide_communication(bw, k, (out, *rest), comm=lambda: snaps.append(ps.to_host(out)), fp64=fp64)
    final = ps.to_host(out)
    assert np.array_equal(final, ps.to_host(ref))
    inner = [np.arange(1, m - 1) for m in n]
    for d in range(3):
        for cells in (np.arange(1, bw[d] + 1), np.arange(n[d] - bw[d] + 1, n[d] - 1)):
            if cells.size == 0:
                continue
            idx = list(inner)
            idx[d] = cells
            sel = np.ix_(*idx)
            assert np.array_equal(snaps[0][sel], final[sel]), (d, cells[0])


# ---------------------------------------------------------------- split FP64 arithmetic
@pytest.mark.parametrize("name", sorted(_cases(np.float64)))
def test_jit_split_fp64_close_to_ieee(ps, name):
    """fp64="split" (FP64 arrays, arithmetic on FP32 pairs) against the IEEE run of the same kernel:
    within 1e-12 of the largest output magnitude (each operation is exact to ~2^-46 of its
    operands; the kernels here chain up to ~60 operations, some with cancellation)."""
    args, ranges = _cases(np.float64)[name]
    src = getattr(K, name)
    k = ps.parallel_kernel(src, ndims=_NDIMS.get(name))
    out = {}
    for fp64 in ("ieee", "split"):
        dev = [_dev(ps, a) if isinstance(a, np.ndarray) else a for a in args]
        ps.parallel(k, *dev, ranges=ranges, fp64=fp64)
        out[fp64] = [ps.to_host(d) for d in dev if not isinstance(d, (int, float))]
    worst = 0.0
    for a, b in zip(out["ieee"], out["split"]):
        scale = max(np.abs(a).max(), 1e-300)
        worst = max(worst, np.abs(a - b).max() / scale)
    assert worst <= 1e-12, (name, worst)


def test_jit_split_fp64_diffusion_run(ps):
    """The headline body in split FP64 arithmetic: 1 step within 1e-13 and 20 steps within 1e-12 of the
    IEEE run (relative max-norm), and really a different arithmetic."""
    import bench

    rng = np.random.default_rng(12)
    n = (64, 48, 40)
    T0, Ci, lam = rng.random(n), rng.random(n) + 0.5, rng.random(n) + 1.0
    k = ps.parallel_kernel(bench.JIT_FLUX_LAM.format(opt=""))
    sc = (1e-4, 20.0, 20.0, 20.0)
    res = {}
    for fp64 in ("ieee", "split"):
        A, B = _dev(ps, T0), _dev(ps, T0)
        dCi, dlam = _dev(ps, Ci), _dev(ps, lam)
        for it in range(20):
            ps.parallel(k, B, A, dCi, dlam, *sc, fp64=fp64)
            A, B = B, A
            if it == 0:
                res[(fp64, 1)] = ps.to_host(A)
        res[(fp64, 20)] = ps.to_host(A)
    for nt, tol in ((1, 1e-13), (20, 1e-12)):
        a, b = res[("ieee", nt)], res[("split", nt)]
        err = np.abs(a - b).max() / np.abs(a).max()
        assert err <= tol, (nt, err)
    assert not np.array_equal(res[("ieee", 1)], res[("split", 1)])


def test_jit_split_fp64_range_flag(ps):
    """A value beyond the pairs' range (|x| >= 2^128) is reported, not silently wrong."""
    from ps_gb300._lib import PSError

    k = ps.parallel_kernel("@parallel function sc!(B, A, s)\n    @all(B) = s*@all(A)\n    return\nend")
    A = _dev(ps, np.full((8, 8, 8), 1e40))
    B = ps.zeros(8, 8, 8)
    with pytest.raises(PSError, match="split FP64") as e:
        ps.parallel(k, B, A, 2.0, fp64="split")
    assert e.value.status == -12
    ps.parallel(k, B, A, 2.0)  # IEEE: fine, and the flag was cleared
    assert np.all(ps.to_host(B) == 2e40)
