"""The Julia `:GB300` package (parallelstencil.jl_gb300/julia/ParallelStencilGB300), host side.

Julia is not installed on the machines this repository is built and tested on, so the package is
checked as source: every `ccall` in it names a function of include/ps_gb300.h with the same number
of arguments and matching argument / return types; every struct it passes has the fields of its C
counterpart in order; its kernel templates are the bodies the Python recogniser (ps_gb300.kernels)
accepts, and its FiniteDifferences macro tables equal ps_gb300.fd's."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JLDIR = os.path.join(ROOT, "parallelstencil.jl_gb300", "julia", "ParallelStencilGB300", "src")
HEADER = os.path.join(ROOT, "include", "ps_gb300.h")


def _sources():
    out = {}
    for fn in sorted(os.listdir(JLDIR)):
        if fn.endswith(".jl"):
            with open(os.path.join(JLDIR, fn), encoding="utf-8") as fh:
                out[fn] = fh.read()
    return out


def _balanced(text, i):
    """text[i] == '(' -> index just past the matching ')'."""
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "(":
            depth += 1
        elif text[j] == ")":
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced parentheses")


def _split_top(s, sep=","):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur.strip())
    return parts


def julia_ccalls():
    """[(c_function, return_type, [argument types])] of every ccall in the package."""
    calls = []
    for fn, text in _sources().items():
        for m in re.finditer(r"ccall\(\(", text):
            start = m.start() + len("ccall")
            end = _balanced(text, start)
            inner = text[start + 1:end - 1]
            args = _split_top(inner)
            target, ret, types = args[0], args[1], args[2]
            tname = _split_top(target[1:-1])[0]
            types = _split_top(types[1:-1]) if types.startswith("(") else [types]
            if tname.startswith(":"):
                names = [tname[1:]]
            else:  # $(QuoteNode(c)) inside `for (jl, c) in ((:f!, :ps_x), ...)`: the loop's C names
                loop = text.rfind("for (jl, c) in", 0, m.start())
                assert loop >= 0, (fn, text[m.start():m.start() + 80])
                lend = _balanced(text, text.index("(", text.index(" in ", loop)))
                names = re.findall(r":(ps_\w+)", text[loop:lend])
            for name in names:
                calls.append((name, ret, types, fn))
    return calls


def header_prototypes():
    text = open(HEADER, encoding="utf-8").read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"(int|const char\s*\*)\s*(ps_\w+)\s*\(([^;]*?)\)\s*;", text):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        ps = [] if params.strip() == "void" else [" ".join(p.split()) for p in params.split(",")]
        protos[name] = ("int" if ret == "int" else "const char*", ps)
    return protos


def header_structs():
    text = open(HEADER, encoding="utf-8").read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\}\s*(\w+);", text, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            typ, names = decl.split(" ", 1) if not decl.startswith("ps_array") else ("ps_array", decl[len("ps_array "):])
            for nm in names.split(","):
                fields.append(re.sub(r"\[.*\]", "", nm.strip()).lstrip("*"))
        out[m.group(3)] = fields
    return out


JL_TO_C = {
    "Cint": {"int"}, "Int32": {"int32_t", "int"}, "Int64": {"int64_t"}, "Cdouble": {"double"},
    "Ptr{Cvoid}": {"void*", "const void*", "ps_comm_fn"}, "Cstring": {"const char*"},
    "PSArray": {"ps_array"}, "PSFdOp": {"ps_fd_op"},
    "Ref{PSLaunch}": {"const ps_launch*"}, "Ptr{Cdouble}": {"double*", "const double*", "double[3]"},
    "Ptr{Int64}": {"const int64_t[3]"}, "Ptr{Int32}": {"const int32_t*"}, "Ref{Ptr{Cvoid}}": {"void**"},
    "Ptr{PSArray}": {"const ps_array*"},
    "Ref{NTuple{3,Int64}}": {"const int64_t[3]"}, "Ref{NTuple{3,Int32}}": {"const int32_t[3]"},
    "Ref{Stokes2DFields}": {"const ps_stokes2d_fields*"}, "Ref{Stokes2DParams}": {"const ps_stokes2d_params*"},
    "Ref{Stokes2DAPTFields}": {"const ps_stokes2d_apt_fields*"},
    "Ref{Stokes2DAPTParams}": {"const ps_stokes2d_apt_params*"},
    "Ref{Stokes3DFields}": {"const ps_stokes3d_fields*"}, "Ref{Stokes3DParams}": {"const ps_stokes3d_params*"},
    "Ref{SolveStats}": {"ps_solve_stats*"}, "Ref{AdjointStats}": {"ps_adjoint_stats*"},
}


def c_type(param):
    """`const double* out` -> 'const double*'; `double out_mean_abs[3]` -> 'double[3]'."""
    p = re.sub(r"\s*\*\s*", "* ", param.strip()).strip()
    arr = re.search(r"(\[\d*\])$", p)
    if arr:
        p = p[:arr.start()].strip()
    toks = p.split()
    if len(toks) > 1 and not toks[-1].endswith("*"):
        toks = toks[:-1]  # the parameter's name
    return " ".join(toks).replace("* *", "**") + (arr.group(1) if arr else "")


def test_every_ccall_matches_the_header():
    protos = header_prototypes()
    calls = julia_ccalls()
    assert len(calls) >= 40
    for name, ret, types, fn in calls:
        assert name in protos, f"{fn}: {name} is not declared in include/ps_gb300.h"
        cret, params = protos[name]
        assert {"Cint": "int", "Cstring": "const char*"}[ret] == cret, (name, ret, cret)
        assert len(types) == len(params), (name, types, params)
        for jt, cp in zip(types, params):
            ct = c_type(cp)
            assert ct in JL_TO_C.get(jt, set()), f"{name}: Julia {jt} for C '{cp}' ({ct})"


def test_ccalled_functions_cover_the_kernel_entry_points():
    called = {c[0] for c in julia_ccalls()}
    for name in ("ps_init", "ps_memcopy3d", "ps_diffusion3d_step", "ps_diffusion3d_run", "ps_diffusion3d_step_split",
                 "ps_fd_apply", "ps_acoustic3d_v", "ps_acoustic3d_p", "ps_stokes2d_compute_P", "ps_stokes2d_solve",
                 "ps_stokes2d_apt_solve", "ps_stokes3d_solve_mixed", "ps_diffusion3d_misfit_gradient",
                 "ps_jit_launch_ex"):
        assert name in called, name


def test_struct_layouts_match_the_header():
    structs = header_structs()
    text = "\n".join(_sources().values())
    pairs = {"PSArray": "ps_array", "PSLaunch": "ps_launch", "PSFdOp": "ps_fd_op",
             "Stokes2DFields": "ps_stokes2d_fields", "Stokes2DParams": "ps_stokes2d_params",
             "SolveStats": "ps_solve_stats", "Stokes2DAPTFields": "ps_stokes2d_apt_fields",
             "Stokes2DAPTParams": "ps_stokes2d_apt_params", "Stokes3DFields": "ps_stokes3d_fields",
             "Stokes3DParams": "ps_stokes3d_params", "AdjointStats": "ps_adjoint_stats"}
    for jl, c in pairs.items():
        m = re.search(r"\nstruct %s\n(.*?)\nend" % jl, text, flags=re.S)
        assert m, jl
        fields = re.findall(r"(\w+)::", m.group(1))
        assert fields == structs[c], (jl, fields, structs[c])


def test_templates_are_the_python_recognisers_bodies():
    from ps_gb300 import kernels

    text = _sources()["recognise.jl"]
    block = text[text.index("const TEMPLATE_SOURCES"):text.index("const INDICES_TEMPLATE_SOURCES")]
    bodies = re.findall(r'"function \w+!\([^)]*\)\s*(.*?)\s*end"', block, flags=re.S)
    assert len(bodies) == 12
    known = [b for b in bodies if kernels._normalise(b) in kernels._NORMALISED]
    assert len(known) == 7  # copy3D, four diffusion forms, acoustic3D V and P
    rest = [b for b in bodies if b not in known]
    assert all("τ" in b or "Mus" in b or "Vx" in b for b in rest)  # the Stokes2D kernels


def test_fd_tables_equal_the_python_tables():
    from ps_gb300 import fd

    text = _sources()["recognise.jl"]
    for nd in (1, 2, 3):
        py = fd.MACROS[nd]
        for name in py:
            assert f'"{name}"' in text or f'pre * "_{name.split("_", 1)[-1]}"' in text or name in ("av", "harm"), name
    # the left-hand selections
    for nd, tab in fd.LHS.items():
        for name in tab:
            assert f'"{name}" =>' in text, (nd, name)


@pytest.mark.parametrize("fn", ["ParallelStencilGB300.jl", "LibPS.jl", "recognise.jl"])
def test_sources_say_they_were_not_run_here_or_are_bindings(fn):
    text = _sources()[fn]
    assert "module" in text or "function" in text
    if fn == "ParallelStencilGB300.jl":
        assert "no Julia toolchain" in text


def test_chainrules_extension_matches_the_package():
    """The ChainRules extension (ext/) is declared in Project.toml, defines an rrule for each
    differentiable entry point of the package, and calls only LibPS functions that exist."""
    pkg = os.path.dirname(JLDIR)
    with open(os.path.join(pkg, "Project.toml"), encoding="utf-8") as fh:
        proj = fh.read()
    assert re.search(r"\[weakdeps\]\s*\nChainRulesCore\s*=", proj)
    assert 'ParallelStencilGB300ChainRulesCoreExt = "ChainRulesCore"' in proj
    with open(os.path.join(pkg, "ext", "ParallelStencilGB300ChainRulesCoreExt.jl"), encoding="utf-8") as fh:
        ext = fh.read()
    src = _sources()
    main, lib = src["ParallelStencilGB300.jl"], src["LibPS.jl"]
    for f in ("diffusion3d_step", "diffusion3d_misfit"):
        assert f"rrule(::typeof(ParallelStencilGB300.{f})" in ext
        assert re.search(rf"^function {f}\(", main, re.M) and f in main.split("export", 3)[-1]
    for f in set(re.findall(r"LibPS\.(\w+!?)", ext)):
        assert re.search(rf"^(function )?{re.escape(f)}\(|^const .*\b{re.escape(f)}\b", lib, re.M), f
