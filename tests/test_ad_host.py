"""`@parallel ∇` on the host (no GPU): the derivative checker (the interpreter run on Dual numbers)
against the reference's own numerical AD test and against itself (the transpose identity), and the
derivative-kernel generator's sources (compiled for sm_103a) and refusals."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import ad_kernels as K


@pytest.fixture(scope="module")
def jr():
    from oracle import jit_reference

    return jit_reference


@pytest.fixture(scope="module")
def jit():
    from ps_gb300 import jit

    return jit


@pytest.fixture(scope="module")
def ad():
    from ps_gb300 import ad

    return ad


def test_checker_reproduces_the_reference_ad_testset(jr):
    """test/ParallelKernel/test_parallel.jl "ad numerical": A[ix] += a*B[ix]*100.65 with a = 6.5 and
    both shadows starting at ones; Enzyme's reverse mode leaves Ā = 1 and B̄ = 1 + a*100.65."""
    N, a = 16, 6.5
    rng = np.random.default_rng(3)
    A, B = rng.random(N), rng.random(N)
    jac = jr.jacobian(K.REF_F, [A, B, a], [0, 1])
    sh = jr.reverse_shadows(jac, {0: np.ones(N), 1: np.ones(N)})
    assert np.array_equal(sh[0], np.ones(N))
    assert np.array_equal(sh[1], np.full(N, 1.0 + a * 100.65))
    assert np.array_equal(jac[0][0], A + a * B * 100.65)  # the primal update happened


def test_checker_forward_mode_on_the_reference_kernel(jr):
    """Forward mode (Enzyme.Forward) of the same kernel: with both tangents at one, the written
    element's tangent becomes 1 + a*100.65 and B's stays 1."""
    N, a = 16, 6.5
    rng = np.random.default_rng(4)
    A, B = rng.random(N), rng.random(N)
    jac = jr.jacobian(K.REF_F, [A, B, a], [0, 1])
    sh = jr.forward_shadows(jac, {0: np.ones(N), 1: np.ones(N)})
    assert np.array_equal(sh[0], np.full(N, 1.0 + a * 100.65))
    assert np.array_equal(sh[1], np.ones(N))


@pytest.mark.parametrize("name", sorted(K.KERNELS))
def test_checker_primal_equals_plain_run_and_transpose_identity(jr, name):
    """On Duals the interpreter gives the plain run's values bit for bit, and its reverse and
    forward products are transposes of each other: <w, J v> = <J^T w, v>."""
    src, nd, _, dup, _ = K.KERNELS[name]
    argnames, args = K.arrays(name)
    pos = [argnames.index(d) for d in dup]
    plain = [a.copy(order="F") if isinstance(a, np.ndarray) else a for a in args]
    jr.run(src, plain, ndims=nd)
    jac = jr.jacobian(src, args, pos, ndims=nd)
    for p in pos:
        assert np.array_equal(jac[p][0], plain[p]), (name, argnames[p])
    rng = np.random.default_rng(7)
    v = {p: rng.standard_normal(np.shape(args[p])) for p in pos}
    w = {p: rng.standard_normal(np.shape(args[p])) for p in pos}
    Jv, JTw = jr.forward_shadows(jac, v), jr.reverse_shadows(jac, w)
    lhs = sum(float(np.sum(w[p] * Jv[p])) for p in pos)
    rhs = sum(float(np.sum(JTw[p] * v[p])) for p in pos)
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs)), (name, lhs, rhs)


def test_checker_derivatives_match_central_differences(jr):
    """One directional derivative of a nonlinear kernel against central differences of plain runs."""
    name = "indices_branches"
    src, nd, _, dup, _ = K.KERNELS[name]
    argnames, args = K.arrays(name)
    pos = [argnames.index(d) for d in dup]
    jac = jr.jacobian(src, args, pos, ndims=nd)
    rng = np.random.default_rng(11)
    v = {p: rng.standard_normal(np.shape(args[p])) for p in pos}
    Jv = jr.forward_shadows(jac, v)
    h = 1e-6
    outs = []
    for sgn in (1.0, -1.0):
        a2 = [a.copy(order="F") if isinstance(a, np.ndarray) else a for a in args]
        for p in pos:
            a2[p] = a2[p] + sgn * h * v[p]
        jr.run(src, a2, ndims=nd)
        outs.append(a2)
    for p in pos:
        fd = (outs[0][p] - outs[1][p]) / (2 * h)
        assert np.abs(fd - Jv[p]).max() <= 1e-6 * max(1.0, np.abs(Jv[p]).max()), argnames[p]


def _nvcc():
    return shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)


@pytest.mark.skipif(_nvcc() is None, reason="nvcc not available")
def test_derivative_sources_compile_for_sm103a(jit, ad, tmp_path):
    """Reverse and forward derivative kernels of every test kernel, FP64 and FP32, compile as CUDA C
    for sm_103a with the options NVRTC gets."""
    cases = [("ref_f", K.REF_F, 1, ("A", "B"))] + [(n, s, nd, dup) for n, (s, nd, _, dup, _) in K.KERNELS.items()]
    procs = []
    for name, src, nd, dup in cases:
        for mode in ad.MODES:
            for real in ("double", "float"):
                f = tmp_path / f"{name}_{mode}_{real}.cu"
                f.write_text(ad.generate(jit.parse(src), nd, real, dup, mode))
                procs.append((f, subprocess.Popen([_nvcc(), "-arch=sm_103a", "-std=c++17", "--fmad=false", "-c",
                                                   str(f), "-o", str(f) + ".o"], stdout=subprocess.PIPE,
                                                  stderr=subprocess.STDOUT, text=True)))
                if len(procs) % 8 == 0:
                    for _, p in procs[-8:]:
                        p.wait()
    for f, p in procs:
        out = p.communicate()[0]
        assert p.returncode == 0, (f.name, out[-2000:])


def test_generated_reverse_structure(jit, ad):
    """The reference's AD kernel: the written shadow is taken (read and zeroed) once, B̄ and Ā are
    their threads' own elements (no atomics); the diffusion step's T̄ gathers from neighbours
    (atomics) while T2̄ is taken at the thread's own inner point."""
    src = ad.generate(jit.parse(K.REF_F), 1, "double", ("A", "B"), "reverse")
    assert src.count("ad_take(") == 2 and "true);" not in src.split("ps_fwd_done_:;")[1]
    dsrc = ad.generate(jit.parse(K.KERNELS["diffusion_flux_lam"][0]), 3, "double", ("T2", "T", "lam"), "reverse")
    rev = dsrc.split("ps_fwd_done_:;")[1]
    assert rev.count("ad_take(d0") == 1
    assert "ad_add(d1" in rev and ", true);" in rev  # T read at seven points: shared shadow updates
    fsrc = ad.generate(jit.parse(K.REF_F), 1, "double", ("A", "B"), "forward")
    assert "ad_st(d0" in fsrc and "ad_take" not in fsrc.split("ps_fwd_done_:;")[1]


@pytest.mark.parametrize("src,dup,msg", [
    ("@parallel_indices (ix) function l!(A, B)\n    for i = 1:3\n        A[ix] = A[ix] + B[ix]\n    end\n    return\nend",
     ("A", "B"), "loops"),
    ("@parallel_indices (ix) function r!(A, B)\n    A[ix] = A[ix+1] + B[ix]\n    return\nend", ("A", "B"), "race"),
    ("@parallel_indices (ix) function k!(A, B)\n    A[ix] = B[ix] * @threadIdx().x\n    return\nend", ("A",),
     "kernel language"),
    ("@parallel_indices (ix) function u!(A, B)\n    A[ix] = B[ix]\n    return\nend", ("C",), "not array arguments"),
])
def test_generator_refusals(jit, ad, src, dup, msg):
    from ps_gb300.core import ArgumentError

    with pytest.raises(ArgumentError, match=msg):
        ad.generate(jit.parse(src), 1, "double", dup, "reverse")
