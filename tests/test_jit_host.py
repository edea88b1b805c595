"""Run-time compiled kernels, host side (no GPU): the CPU interpreter that checks them is pinned
against the known-answer fixtures, and the translator's parsing, argument rules, error messages and
generated CUDA C are checked without launching anything."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import jit_kernels as K
from conftest import DT

# the reference's source tree (ParallelStencil.jl) named by PS_REFERENCE_DIR: the tests that translate
# its miniapps and examples are skipped when it is unset
REFERENCE = os.environ.get("PS_REFERENCE_DIR", "")


@pytest.fixture(scope="module")
def jr():
    from oracle import jit_reference

    return jit_reference


@pytest.fixture(scope="module")
def jit():
    from ps_gb300 import jit

    return jit


def _fd_src(stmt):
    return f"@parallel function fd_case!(R, A)\n    {stmt}\n    return\nend"


# ---------------------------------------------------------------- the interpreter, pinned
def test_interpreter_matches_every_fd_macro_fixture(jr, golden):
    meta, arr = golden
    assert len(meta["fd"]) > 150
    for case in meta["fd"]:
        Rexp = arr[case["key"] + "_R"]
        R = np.zeros(Rexp.shape, dtype=Rexp.dtype)
        jr.run(_fd_src(case["statement"]), [R, arr[case["key"] + "_A"].copy()], ndims=case["ndims"])
        assert np.array_equal(R, Rexp), (case["key"], case["statement"])


@pytest.mark.parametrize("src", [K.HEAT_FLUX, K.HEAT_LAP], ids=["flux_on_the_fly", "second_differences"])
def test_interpreter_matches_diffusion_fixtures(jr, golden, src):
    meta, arr = golden
    for case in meta["diffusion"]:
        T, Ci, T2e = (arr[case["key"] + s] for s in ("_T", "_Ci", "_T2"))
        T2 = np.zeros_like(T)
        jr.run(src, [T2, T.copy(), Ci.copy(), 1.0, 1.0, 1.0, 1.0, 1.0])
        assert np.array_equal(T2, T2e), case["key"]
        assert T2.dtype == DT[case["dtype"]]


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_interpreter_matches_diffusion_project(jr, golden, dtn):
    _, arr = golden
    p = {k.split("_", 2)[2]: v for k, v in arr.items() if k.startswith(f"project8_{dtn}_")}
    lam, dt_, dx, dy, dz = (float(v) for v in p["scalars"])
    T, T2 = p["T0"].copy(), p["T0"].copy()
    for _ in range(3):
        jr.run(K.HEAT_DIV, [T2, T, p["Ci"].copy(), lam, dt_, dx, dy, dz])
        T, T2 = T2, T
    assert np.array_equal(T, p["T"])


def test_interpreter_explicit_indices_against_broadcasting(jr):
    """Upwind advection and wall copies restated with numpy slicing."""
    rng = np.random.default_rng(11)
    nx, ny = 13, 9
    T, u, w = rng.random((nx, ny)), rng.standard_normal((nx, ny)), rng.standard_normal((nx, ny))
    Tn = np.full((nx, ny), -1.0)
    dt, rdx, rdy = 0.1, 3.0, 2.5
    jr.run(K.UPWIND2D, [Tn, T, u, w, dt, rdx, rdy])
    c = (slice(1, -1), slice(1, -1))
    Tc, uc, wc = T[c], u[c], w[c]
    exp = Tc - dt * (np.where(uc > 0, uc, np.copysign(0.0, uc)) * (Tc - T[:-2, 1:-1]) * rdx
                     + np.where(uc < 0, uc, np.copysign(0.0, uc)) * (T[2:, 1:-1] - Tc) * rdx
                     + np.where(wc > 0, wc, np.copysign(0.0, wc)) * (Tc - T[1:-1, :-2]) * rdy
                     + np.where(wc < 0, wc, np.copysign(0.0, wc)) * (T[1:-1, 2:] - Tc) * rdy)
    assert np.array_equal(Tn[c], exp)
    assert np.all(Tn[0] == -1.0) and np.all(Tn[:, -1] == -1.0)
    W = rng.random((nx, ny))
    W0 = W.copy()
    jr.run(K.WALLS2D, [W], ranges=[(1, ny)])
    assert np.array_equal(W[0], W0[1]) and np.array_equal(W[-1], W0[-2]) and np.array_equal(W[1:-1], W0[1:-1])


def test_interpreter_julia_number_rules(jr):
    """max/min propagate NaN and order signed zeros; Bool * x keeps the sign of zero; x^2 is x*x."""
    A = np.array([[np.nan, -0.0, 0.0, 2.0]]).T.copy()
    B = np.zeros_like(A)
    src = """@parallel_indices (i, j) function rules!(B, A)
        B[i, j] = max(A[i, j], 0.0) + (A[i, j] > 1)*(-0.0) + min(-0.0, 0.0)^2
        return
    end"""
    jr.run(src, [B, A])
    assert np.isnan(B[0, 0])
    assert B[1, 0] == 0.0 and not np.signbit(B[1, 0])
    assert B[3, 0] == 2.0


def test_interpreter_bounds_error(jr):
    A, B = np.arange(6.0), np.zeros(6)
    with pytest.raises(IndexError, match="BoundsError"):
        jr.run(K.SHIFT_OOB, [B, A])
    B[:] = 0
    jr.run(K.SHIFT_OOB, [B, A], ranges=[(1, 5)])
    assert np.array_equal(B[:5], A[1:])


def test_interpreter_linear_index_and_elseif(jr):
    A = np.zeros((4, 5, 6))
    jr.run(K.LINEAR_INDEX, [A])
    ix, iy, iz = np.meshgrid(np.arange(1, 5), np.arange(1, 6), np.arange(1, 7), indexing="ij")
    assert np.array_equal(A, ix + (iy - 1) * 4 + (iz - 1) * 20)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((7, 6))
    Y = np.zeros_like(X)
    jr.run(K.BRANCHES2D, [Y, X, 3, 0.5])
    i, j = np.meshgrid(np.arange(1, 8), np.arange(1, 7), indexing="ij")
    exp = np.where(X > 0.5, np.maximum(X, 0.5) - (np.abs(X) * np.abs(X)) * np.abs(X),
                   np.where(X < -0.5, np.minimum(X, -0.5) + (i > j),
                            np.sqrt(np.abs(X)) * ((j == 1) | (i == 7))))
    assert np.allclose(Y, exp, rtol=1e-15, atol=0)


# ---------------------------------------------------------------- the translator
def test_translator_argument_kinds(jit):
    kd = jit.parse(K.HEAT_LAP)  # untyped arguments follow their use
    assert kd.arrays == ["Tnew", "Told", "Cinv"] and kd.scalars == ["_u03bb_", "_u0394_t", "rdx", "rdy", "rdz"]
    kd = jit.parse(K.BRANCHES2D)
    assert kd.arrays == ["B", "A"] and kd.scalars == ["c", "t"] and kd.int_scalars == {"c"}
    assert kd.kind == "parallel_indices" and kd.index_names == ["ix", "iy"] and kd.options == {"inbounds": "false"}
    kd = jit.parse(K.D2Z3D)
    assert kd.options == {"memopt": "true", "loopsize": "3"}
    kd = jit.parse("@parallel memopt=true loopsize=3 optvars=(A, B) optranges=(A=(0:0, 0:0, 0:0), B=(0:0,0:0,0:0)) "
                   "function f!(A2, A, B)\n    @all(A2) = @all(A) + @all(B)\n    return\nend")
    assert kd.options == {"memopt": "true", "loopsize": "3", "optvars": "(A, B)",
                          "optranges": "(A=(0:0, 0:0, 0:0), B=(0:0,0:0,0:0))"}
    with pytest.raises(jit.ArgumentError):
        jit.parse("@parallel optvars=(A, B function f!(A)\n    @all(A) = 1.0\n    return\nend")
    kd = jit.parse("@parallel function f!(A::Data.Array, B::Data.Array, c::T) where T <: Integer\n"
                   "    @all(A) = @all(B)^c\n    return\nend")
    assert kd.arrays == ["A", "B"] and kd.scalars == ["c"]


@pytest.mark.parametrize("src,msg", [
    ("@parallel function f!(A, B)\n @inn(t) = @all(B)\n @all(A) = @all(t)\n return\nend", "use '@all' instead"),
    ("@parallel function f!(A, B)\n @all(t) = @all(t) + @all(B)\n @all(A) = @all(t)\n return\nend", "auto-dependency"),
    ("@parallel function f!(A, B)\n @all(t) = @all(A)\n @all(A) = @all(t) + @all(B)\n return\nend", "not read-only"),
    ("@parallel function f!(A, B)\n @all(A) = @d_qa(B)\n return\nend", "unknown macro"),
    ("@parallel padding=true function f!(A, B)\n @all(A) = @all(B)\n return\nend", "padding"),
    ("@parallel fancy=1 function f!(A, B)\n @all(A) = @all(B)\n return\nend", "unsupported keyword"),
    ("@parallel function f!(A, s::Data.Number)\n @all(A) = @all(s)\n return\nend", "used as an array"),
    ("@parallel_indices (i, j, k, l) function f!(A)\n A[i] = 1.0\n return\nend", "1-3 index"),
])
def test_translator_rejects(jit, src, msg):
    from ps_gb300.core import ArgumentError

    with pytest.raises(ArgumentError, match=re.escape(msg)):
        jit.generate(jit.parse(src), 3 if "d_qa" not in src else 2, "double")


def test_translator_generated_structure(jit):
    src = jit.generate(jit.parse(K.HEAT_FLUX), 3, "double")
    assert "extern \"C\" __global__ void ps_jit_entry(const ps_jit_args g)" in src
    assert "fx" not in src.split("ps_jit_entry")[1]  # the on-the-fly arrays are inlined
    body = src.split("ps_jit_entry")[1]
    assert body.count("__ldg(") == 8  # the 8 distinct stencil points, each read once (read-only arrays)
    assert "tx + 2 < n1_0" in body and "atomicOr(g.err, 1)" in body  # one bounds check per statement
    assert "tx < n0_0 - 2 && ty < n0_1 - 2 && tz < n0_2 - 2" in src  # @within("@inn", Tnew)
    src = jit.generate(jit.parse(K.SHIFT_INBOUNDS), 1, "float")
    assert "typedef float R;" in src and "jl_ld(a" not in src and "jl_ldg(a" not in src and "jl_st(a" not in src
    src = jit.generate(jit.parse(K.BRANCHES2D), 2, "double")
    assert "const long long s0 = (long long)g.s[0];" in src and "pow(" in src


def _nvcc():
    return shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)


@pytest.mark.skipif(_nvcc() is None, reason="nvcc not available")
def test_generated_sources_compile_for_sm103a(jit, tmp_path):
    """Every test kernel, FP64 and FP32, compiles as CUDA C for sm_103a (the same options NVRTC gets)."""
    srcs = [(n, getattr(K, n)) for n in dir(K) if n.isupper()]
    nd = {"ROD1D": 1, "SHIFT_OOB": 1, "SHIFT_INBOUNDS": 1, "WALLS2D": 2, "WARP_SUMS": 1, "WARP_OPS": 1,
          "EARLY_RETURN": 1, "BOX_X": 2}
    procs = []
    for name, src in srcs:
        ndims = nd.get(name, 2 if "2D" in name else 3)
        for real in ("double", "float"):
            f = tmp_path / f"{name}_{real}.cu"
            f.write_text(jit.generate(jit.parse(src), ndims, real))
            procs.append((f, subprocess.Popen([_nvcc(), "-arch=sm_103a", "-std=c++17", "--fmad=false", "-c", str(f),
                                               "-o", str(f) + ".o"], stdout=subprocess.PIPE,
                                              stderr=subprocess.STDOUT, text=True)))
            if real == "double" and ndims in (2, 3) and src.lstrip().startswith("@parallel function"):
                fz = tmp_path / f"{name}_sweep.cu"  # the memopt variant (sweep along z in 3-D, y in 2-D)
                fz.write_text(jit.generate(jit.parse(src), ndims, "double", zloop=True))
                procs.append((fz, subprocess.Popen([_nvcc(), "-arch=sm_103a", "-std=c++17", "--fmad=false", "-c",
                                                    str(fz), "-o", str(fz) + ".o"], stdout=subprocess.PIPE,
                                                   stderr=subprocess.STDOUT, text=True)))
            if len(procs) % 8 == 0:
                for _, p in procs[-8:]:
                    p.wait()
    for f, p in procs:
        out = p.communicate()[0]
        assert p.returncode == 0, (f.name, out[-2000:])


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "miniapps")), reason="PS_REFERENCE_DIR unset")
def test_reference_miniapp_kernels_translate(jit):
    """Every @parallel / @parallel_indices definition of the reference's miniapps translates."""
    n = 0
    for fn in sorted(os.listdir(os.path.join(REFERENCE, "miniapps"))):
        if not fn.endswith(".jl"):
            continue
        with open(os.path.join(REFERENCE, "miniapps", fn), encoding="utf-8") as fh:
            text = fh.read()
        ndims = 3 if "3D" in fn else 2
        for d in re.findall(r"^(@parallel(?:_indices)?[^\n]*function.*?^end)", text, re.S | re.M):
            assert "ps_jit_entry" in jit.generate(jit.parse(d), ndims, "double"), (fn, d[:60])
            n += 1
    assert n >= 40


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "examples")), reason="PS_REFERENCE_DIR unset")
def test_reference_example_kernels_translate(jit):
    """Every top-level @parallel / @parallel_indices definition of the reference's examples and test
    projects translates, except those over CellArrays and NamedTuples of arrays (not built)."""
    n = 0
    roots = [os.path.join(REFERENCE, "examples"), os.path.join(REFERENCE, "test", "test_projects")]
    for root in roots:
        for dirpath, _, files in os.walk(root):
            for fn in sorted(files):
                if not fn.endswith(".jl") or "CellArray" in fn or "NamedArrayTuple" in fn:
                    continue
                with open(os.path.join(dirpath, fn), encoding="utf-8") as fh:
                    text = fh.read()
                ndims = 2 if "2D" in fn else 1 if "1D" in fn else 3
                for d in re.findall(r"^(@parallel(?:_indices)?[^\n]*function.*?^end)", text, re.S | re.M):
                    kd = jit.parse(d)
                    for nd in ((2, 3) if kd.splat else (ndims,)):
                        assert "ps_jit_entry" in jit.generate(kd, nd, "double"), (fn, d[:60])
                    n += 1
    assert n >= 15


# ---------------------------------------------------------------- kernel language in the interpreter
def test_interpreter_shared_memory_tile_equals_plain(jr):
    rng = np.random.default_rng(4)
    nx, ny = 64, 16
    T, Ci = rng.random((nx, ny)), rng.random((nx, ny)) + 0.5
    A, B = np.zeros((nx, ny)), np.zeros((nx, ny))
    sc = (1.0, 1e-3, 7.0, 9.0)
    jr.run(K.HEAT2D_TILE, [A, T, Ci, *sc], nthreads=(32, 8), shmem=34 * 10 * 8)
    jr.run(K.HEAT2D_PLAIN, [B, T, Ci, *sc])
    assert np.array_equal(A, B) and np.count_nonzero(A) == (nx - 2) * (ny - 2)


def test_interpreter_warp_shuffles_and_votes(jr):
    rng = np.random.default_rng(6)
    n = 128
    a = rng.standard_normal(n)
    S = np.zeros(n // 32)
    jr.run(K.WARP_SUMS, [S, a], nthreads=(64,))
    assert np.allclose(S, a.reshape(-1, 32).sum(axis=1), rtol=1e-14)
    B, C, D = np.zeros(n), np.zeros(n), np.zeros(n)
    jr.run(K.WARP_OPS, [B, C, D, a, 1.5], nthreads=(64,))
    w = a.reshape(-1, 32)
    lane = np.arange(32)
    first = np.repeat(w[:, :1], 32, axis=1)
    up = np.where(lane >= 1, np.roll(w, 1, axis=1), w)
    down = np.where(lane % 16 + 2 < 16, np.roll(w, -2, axis=1), w)
    anyhi = (w > 1.5).any(axis=1, keepdims=True)
    allhi = (w > -1.5).all(axis=1, keepdims=True)
    bal = ((w > 0) * (1 << lane)).sum(axis=1, keepdims=True) % 1024
    assert np.array_equal(B.reshape(-1, 32), first + np.where(anyhi, up, np.copysign(0.0, up)) - down)
    assert np.array_equal(C.reshape(-1, 32), allhi * 1.0 + bal + 0 * w)
    assert np.array_equal(D.reshape(-1, 32), np.broadcast_to(lane + 1 + 3200.0, w.shape))
    with pytest.raises(ValueError, match="multiple of the thread block"):
        jr.run(K.WARP_SUMS, [S, a], ranges=[(1, 100)], nthreads=(64,))


def test_interpreter_loops_and_block_ids(jr):
    rng = np.random.default_rng(2)
    A = rng.random((11, 5))
    B = np.zeros_like(A)
    jr.run(K.BOX_X, [B, A, 2])
    exp = np.array([[A[max(0, i - 2):min(11, i + 3), j].sum() / (min(11, i + 3) - max(0, i - 2))
                     for j in range(5)] for i in range(11)])
    assert np.allclose(B, exp, rtol=1e-15)
    X = np.zeros((16, 8, 4))
    jr.run(K.BLOCK_IDS, [X], nthreads=(8, 4, 2))
    i, j, k = np.meshgrid(np.arange(16), np.arange(8), np.arange(4), indexing="ij")
    exp = (i // 8 + 1) + 10 * (j // 4 + 1) + 100 * (k // 2 + 1) + 1000 * ((i % 8 + 1) + (j % 4 + 1) * 8) + 0.5 * 2
    assert np.array_equal(X, exp)


def test_translator_y_sweep_of_2d_kernels(jit):
    """memopt for 2-D `@parallel` kernels sweeps y (loopdim 2): blockIdx.y covers g.loop consecutive y
    indices and the two T points one row further along y come from the previous row's registers."""
    src = jit.generate(jit.parse(K.HEAT2D_FD), 2, "double", zloop=True)
    body = src.split("ps_jit_entry")[1]
    assert "const long long uy = blockIdx.y * g.loop + it_;" in body
    assert "threadIdx.y" not in body
    carried = re.findall(r"const R (L\d+) = pr(\d) \? P\d_\d+ : (.*?);", body)
    assert len(carried) == 2 and all("a1[" in ld for _, _, ld in carried)  # T (argument 1) only
    plain = jit.generate(jit.parse(K.HEAT2D_FD), 2, "double")
    assert "g.loop" not in plain.split("ps_jit_entry")[1]


def test_translator_z_sweep_carries_only_read_only_points(jit):
    src = jit.generate(jit.parse(K.TWO3D), 3, "double", zloop=True)
    body = src.split("ps_jit_entry")[1]
    assert "for (long long it_ = 0; it_ < g.loop; ++it_)" in body
    carried = re.findall(r"const R (L\d+) = pr(\d) \? P\d_\d+ : (.*?);", body)
    assert carried and all("a2[" in ld for _, _, ld in carried)  # only B (argument 2) is read-only
    assert "a0[" not in "".join(ld for _, _, ld in carried)  # A is written by the first statement


def test_kernel_language_keeps_one_point_per_thread(jit):
    """A `@parallel` kernel that uses the kernel language (@threadIdx, @sharedMem, barriers, shuffles)
    is not turned into a sweep: what those see must stay the launch's own thread layout."""
    src = ("@parallel function kl!(A, B)\n    @all(A) = @all(B) * @threadIdx().x\n    @sync_threads()\n"
           "    return\nend")
    kd = jit.parse(src)
    assert jit.uses_kernel_language(kd)
    assert "g.loop" not in jit.generate(kd, 3, "double", zloop=True).split("ps_jit_entry")[1]
    assert not jit.uses_kernel_language(jit.parse(K.HEAT_FLUX))


def test_interpreter_language_additions(jr):
    """Compound assignment, module-qualified macros, (I...) index tuples, local functions and Int
    expressions, on the interpreter against numpy."""
    rng = np.random.default_rng(3)
    A, B = rng.random(12), rng.random(12)
    A0 = A.copy()
    jr.run(K.AUGASSIGN, [A, B, 0.3])
    assert np.array_equal(A, (((A0 + 0.3 * B * 100.65) - 1.5) * 2) / 3)
    Bq = np.asfortranarray(rng.random((7, 6)))
    A2 = np.zeros((7, 6), order="F")
    jr.run(K.QUALIFIED2D, [A2, Bq])
    exp = np.zeros((7, 6))
    exp[1:-1, 1:-1] = (Bq[1:-1, 2:] - Bq[1:-1, 1:-1]) - (Bq[1:-1, 1:-1] - Bq[1:-1, :-2])
    assert np.array_equal(A2, exp)
    for shape in ((7, 5), (4, 3, 5)):
        X = np.asfortranarray(rng.random(shape))
        Y = np.zeros(shape, order="F")
        jr.run(K.SPLAT_COPY, [Y, X, 1.5])
        assert np.array_equal(Y, 1.5 * X)
    L = np.zeros((6, 5, 4), order="F")
    jr.run(K.LOCAL_FN, [L])
    assert np.array_equal(L, np.arange(1, 121, dtype=float).reshape((6, 5, 4), order="F"))
    F = np.zeros((9, 7), dtype=np.float32, order="F")
    jr.run(K.INT_EXPR2D, [F])
    assert np.array_equal(F, np.arange(1, 64, dtype=np.float32).reshape((9, 7), order="F"))


def test_translator_language_additions(jit):
    """The same kernels translate; local functions leave no call behind, `I...` indexes with the
    thread's own indices, Int expressions stay Int until the store."""
    for name, nd in (("AUGASSIGN", 1), ("QUALIFIED2D", 2), ("SPLAT_COPY", 2), ("SPLAT_COPY", 3), ("LOCAL_FN", 3),
                     ("INT_EXPR2D", 2)):
        src = jit.generate(jit.parse(getattr(K, name)), nd, "float")
        assert "ps_jit_entry" in src
    body = jit.generate(jit.parse(K.LOCAL_FN), 3, "double").split("ps_jit_entry")[1]
    assert "compute_indices" not in body
    body = jit.generate(jit.parse(K.INT_EXPR2D), 2, "float").split("ps_jit_entry")[1]
    assert "- 1LL" in body and "(R)1.0" not in body
    assert jit.parse(K.SPLAT_COPY).splat == "I"


@pytest.mark.parametrize("dtn", ["f64", "f32"])
def test_interpreter_and_c_oracle_agree(jr, oracle, dtn):
    """The two independent CPU restatements -- the C oracle's FD kernels and the interpreter of kernel
    definitions -- agree bit for bit on random fields for every 2-D and 3-D macro, `@all` and `@inn`
    left-hand sides (the golden fixtures pin each at one size; this crosses them at others)."""
    from ps_gb300.fd import LHS, MACROS

    dt = DT[dtn]
    for nd, n in ((3, (9, 8, 7)), (2, (11, 6))):
        A = np.asfortranarray(np.random.default_rng(nd).standard_normal(n).astype(dt) + 2.0)
        for op, (kind, opd, inn) in sorted(MACROS[nd].items()):
            for lhs in ("all", "inn"):
                shape = tuple(n[k] - ((inn >> k) & 1) - ((opd >> k) & 1) for k in range(nd))
                c = np.asfortranarray(np.full(shape, -7.0, dtype=dt))
                oracle.fd_apply(kind, opd, inn, nd, LHS[nd][lhs], c, A)
                p = np.asfortranarray(np.full(shape, -7.0, dtype=dt))
                jr.run(f"@parallel function f!(R, A)\n    @{lhs}(R) = @{op}(A)\n    return\nend", [p, A], ndims=nd)
                assert np.array_equal(c, p, equal_nan=True), (nd, op, lhs)


# ---------------------------------------------------------------- the TMA variant of 3-D sweeps
_TMA_KERNELS = ["HEAT_FLUX", "HEAT_LAP", "HEAT_DIV", "BLEND3D", "FACES3D", "TWO3D", "COMPACTION"]


def _tma_info(jit, name, real, split=False):
    src, _, layout = jit._generate_info(jit.parse(getattr(K, name)), 3, real, True, split, False, True)
    return src, layout


@pytest.mark.parametrize("real", ["double", "float"])
@pytest.mark.parametrize("name", _TMA_KERNELS)
def test_tma_layout_covers_every_staged_read(jit, name, real):
    """Checked on the CPU before any launch: each staged array's TMA box starts on a 16-byte
    boundary in x (the tile origin is a multiple of 32 elements), every (thread, offset) read of the
    generated kernel falls inside its array's box, planes lie inside the ring's span, and the
    stages and mbarriers fit the shared memory the launch gives."""
    src, L = _tma_info(jit, name, real)
    assert L is not None, name
    es = 8 if real == "double" else 4
    g = jit._Gen(jit.parse(getattr(K, name)), 3, True, False, False, tma=True)
    g.source(real)
    ty = jit._Gen.TMA_TY
    ends = sorted(a["off"] for a in L["arrays"]) + [L["stage"]]
    for a in L["arrays"]:
        assert (a["xs"] * es) % 16 == 0 and (32 * L["xc"] * es) % 16 == 0 and (a["bx"] * es) % 16 == 0
        assert a["bx"] <= 256 and a["by"] <= 256 and a["off"] % 128 == 0
        nxt = min(e for e in ends if e > a["off"])
        assert a["off"] + a["bx"] * a["by"] * es <= nxt
        for o in g.staged[a["name"]]:
            assert 0 <= o[2] - L["zl"] < L["span"]
            for lx in (0, 32 * L["xc"] - 1):
                for ly in (0, ty - 1):
                    assert 0 <= lx + o[0] - a["xs"] < a["bx"], (a, o)
                    assert 0 <= ly + o[1] - a["ys"] < a["by"], (a, o)
    assert L["stages"] >= L["span"] + 2 and L["stage"] % 128 == 0
    assert L["smem"] == L["stages"] * L["stage"] + 8 * L["stages"] and L["smem"] <= 227 * 1024
    assert L["tx_bytes"] == sum(a["bx"] * a["by"] * es for a in L["arrays"]) < 2 ** 20
    assert "__TMA[" not in src and "ps_jit_targs" in src and "cp.async.bulk.tensor.3d" in src


@pytest.mark.skipif(_nvcc() is None, reason="nvcc not available")
def test_tma_sources_compile_for_sm103a(jit, tmp_path):
    procs = []
    for name in _TMA_KERNELS:
        for real, split in (("double", False), ("float", False), ("double", True)):
            src, L = _tma_info(jit, name, real, split)
            f = tmp_path / f"{name}_{real}_{split}.cu"
            f.write_text(src)
            procs.append((f, subprocess.Popen([_nvcc(), "-arch=sm_103a", "-std=c++17", "--fmad=false", "-c", str(f),
                                               "-o", str(f) + ".o"], stdout=subprocess.PIPE,
                                              stderr=subprocess.STDOUT, text=True)))
            if len(procs) % 8 == 0:
                for _, p in procs[-8:]:
                    p.wait()
    for f, p in procs:
        out = p.communicate()[0]
        assert p.returncode == 0, (f.name, out[-2000:])


def test_tma_variant_falls_back_where_it_cannot_apply(jit):
    """A kernel without read-only stencil arrays has nothing to stage: the plain sweep is generated."""
    src = "@parallel function cp!(A, B)\n    @all(A) = @all(A) * 2.0\n    return\nend"
    s, _, layout = jit._generate_info(jit.parse(src), 3, "double", True, False, False, True)
    assert layout is None and "cp.async.bulk.tensor" not in s
