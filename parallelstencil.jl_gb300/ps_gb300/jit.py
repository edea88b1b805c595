"""Run-time compiled ``@parallel`` / ``@parallel_indices`` kernels (any body, not only the fixed set).

``parallel_kernel(src)`` takes a kernel written as in ParallelStencil.jl, e.g. (miniapps/
ThermalConvection2D.jl:28-34)::

    @parallel function compute_1!(Pt::Data.Array, τxx::Data.Array, ..., β::Data.Number, dx::Data.Number, dy::Data.Number)
        @all(Pt)   = @all(Pt) - dτ_iter/β*@all(∇V)
        @all(τxx)  = 2.0*@all(Eta)*(@d_xa(Vx)/dx  - 1.0/3.0*@all(∇V))
        ...
        return
    end

and generates CUDA C with the rules the reference applies when it parses such a body
(src/parallel.jl:192-277, 654-680, 789-859; src/ParallelKernel/parallel.jl:400-418, 477-485, 795-798):

- thread grid = the largest extent of the array arguments per dimension (or ``ranges``);
- each ``@sel(A) = expr`` statement is masked by ``@within("@sel", A)`` and writes A at the thread
  index shifted by the selection's inner offsets; the FiniteDifferences macros expand to the
  reference's index patterns and operation orders (left-to-right sums, ``*0.5``, ``1.0/(..)*2.0``,
  Julia's NaN-propagating ``max``/``min``);
- a left-hand array that is not an argument is an on-the-fly temporary: its expression is inlined,
  at the shifted index, wherever a later statement uses it;
- floating literals take the array number type, ``x^2`` / ``x^3`` are products as Julia's literal
  powers, ``Bool * x`` keeps Julia's signed zero, no FMA contraction (``--fmad=false``).

``@parallel_indices (ix, iy[, iz]) function f!(...)`` bodies use explicit 1-based indexing,
``size(A, d)``, comparisons, ``if``/``elseif``/``else``, ``for``/``while`` loops, compound
assignments and one-line local functions; the index names (or an index tuple ``(I...)`` used as
``A[I...]``) map to the grid dimensions; Int subexpressions stay Int until a real value is needed.
The kernel language (``@threadIdx`` ... ``@sharedMem``, ``@sync_threads``, shuffles, votes) is
translated for ``nblocks`` / ``nthreads`` / ``shmem`` launches.

memopt (the default for 2-D and 3-D ``@parallel`` kernels without kernel-language calls) sweeps
the last dimension with read-only neighbours carried in registers; ``fp64="split"`` evaluates FP64
kernels on FP32 pairs. The CUDA C is compiled by the library (``ps_jit_compile``, NVRTC for
sm_103a) and cached per source, rank, number type, sweep and arithmetic.
"""
from __future__ import annotations

import ast
import copy
import ctypes
import io
import numbers
import re
import tokenize
from dataclasses import dataclass, field

from . import _lib
from ._lib import PSArray
from .core import ArgumentError, descriptor, require_initialized, stream_handle
from .fd import AV, DIFF, DIFF2, HARM, LHS, MACROS, MAXLOC, MINLOC, SEL
from .kernels import ranges_to_box

_lib.register("ps_jit_compile", [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)])
_lib.register("ps_jit_launch", [ctypes.c_void_p, ctypes.POINTER(PSArray), ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_jit_launch_ex", [ctypes.c_void_p, ctypes.POINTER(PSArray), ctypes.c_int32,
                                   ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                   ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32), ctypes.c_int64,
                                   ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_jit_hide_communication", [ctypes.c_void_p, ctypes.POINTER(PSArray), ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_double), ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32),
                                            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64),
                                            _lib.COMM_FN, ctypes.c_void_p, ctypes.c_void_p])
_lib.register("ps_jit_launch_tma", [ctypes.c_void_p, ctypes.POINTER(PSArray), ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                    ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, ctypes.c_int32,
                                    ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_void_p, ctypes.c_int])
_lib.register("ps_jit_check", [ctypes.c_void_p, ctypes.c_void_p])
_lib.register("ps_jit_destroy", [ctypes.c_void_p])

MAX_ARRAYS = MAX_SCALARS = 32
TMA_RING_BYTES = 64 * 1024  # shared memory for the plane ring of a TMA sweep (sets the planes in flight)
RESIDENT_THREADS = 152 * 2048  # threads a GB300 holds at once (152 SMs x 2048)
# kernel-language macros (src/ParallelKernel/kernel_language.jl): a kernel that uses any of them
# keeps one point per thread (a sweep would change what @threadIdx, @sharedMem and barriers see)
_KERNEL_LANGUAGE = {"__m_" + m for m in ("threadIdx", "blockIdx", "blockDim", "gridDim", "sharedMem", "sync_threads",
                                         "warpsize", "laneid", "active_mask", "shfl_sync", "shfl_up_sync",
                                         "shfl_down_sync", "shfl_xor_sync", "vote_any_sync", "vote_all_sync",
                                         "vote_ballot_sync")}


def uses_kernel_language(kd) -> bool:
    return any(isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in _KERNEL_LANGUAGE
               for n in ast.walk(ast.Module(body=kd.body, type_ignores=[])))


_COLLECTIVE = {"__m_shfl_sync", "__m_shfl_up_sync", "__m_shfl_down_sync", "__m_shfl_xor_sync", "__m_vote_any_sync",
               "__m_vote_all_sync", "__m_vote_ballot_sync"}
_MATH = {"exp", "log", "sqrt", "sin", "cos", "tan", "tanh", "sinh", "cosh", "atan", "asin", "acos", "log10",
         "exp2", "cbrt"}


# ---- reading Julia source ----------------------------------------------------------------
def _ident(name: str) -> str:
    """Julia identifier (Unicode allowed) -> Python identifier."""
    return "".join(c if (c.isascii() and (c.isalnum() or c == "_")) else f"_u{ord(c):04x}_" for c in name)


def _sanitize(text: str) -> str:
    text = re.sub(r"#.*", "", text).replace("$", "")  # `$ix` interpolations name the index itself
    for a, b in (("≤", "<="), ("≥", ">="), ("≠", "!="), ("÷", "//"), ("∈", " in ")):
        text = text.replace(a, b)
    out = []
    for c in text:
        out.append(c if c.isascii() else f"_u{ord(c):04x}_")
    text = "".join(out)
    text = re.sub(r"\b(\w+)\.\.\.", r"__splat_\1", text)  # A[I...]
    # module-qualified macros (FiniteDifferences2D.@inn) are the macros themselves
    text = re.sub(r"\b(?:ParallelStencil\.)?(?:FiniteDifferences[123]D\.)?(?=@)", "", text)
    text = re.sub(r"@(\w+)\s*\(", r"__m_\1(", text)
    text = text.replace("^", "**").replace("&&", " and ").replace("||", " or ")
    text = re.sub(r"!(?!=)", " not ", text)
    text = re.sub(r"\btrue\b", "True", text)
    return re.sub(r"\bfalse\b", "False", text)


def _split_range(text: str) -> list:
    """`a:b` / `a:s:b` (top-level colons) -> [a, b] / [a, s, b]."""
    parts, d, cur = [], 0, ""
    for c in text:
        d += c in "([{"
        d -= c in ")]}"
        if c == ":" and d == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += c
    parts.append(cur.strip())
    if len(parts) not in (2, 3) or not all(parts):
        raise ArgumentError(f"for loops run over a range a:b or a:s:b (obtained {text})")
    return parts


def _to_python(body: str) -> str:
    """Julia statement / if-block structure -> indented Python source (the expressions are Python)."""
    body = "\n".join(line.strip() for line in body.splitlines())  # Julia indentation carries no meaning
    toks = [t for t in tokenize.generate_tokens(io.StringIO(body).readline)
            if t.type not in (tokenize.COMMENT, tokenize.ENCODING)]
    lines, cur, depth, indent = [], [], 0, 0

    def flush():
        nonlocal cur
        s = tokenize.untokenize([(t.type, t.string) for t in cur]).strip() if cur else ""
        # a left-hand selection `@all(A) = ...` becomes the assignable `__lhs_all[A] = ...`
        s = re.sub(r"^__m_(\w+)\s*\(\s*(\w+)\s*\)\s*=(?!=)", r"__lhs_\1[\2] =", s)
        if s == "return" and indent == 0:
            pass  # the closing `return` of the function body
        elif s:
            lines.append("    " * indent + s)
        cur = []

    i = 0
    while i < len(toks):
        t = toks[i]
        if t.type == tokenize.OP and t.string in "([{":
            depth += 1
        elif t.type == tokenize.OP and t.string in ")]}":
            depth -= 1
        if depth == 0 and (t.type in (tokenize.NEWLINE, tokenize.NL, tokenize.ENDMARKER)
                           or (t.type == tokenize.OP and t.string == ";")):
            if not (cur and cur[-1].type == tokenize.OP and cur[-1].string in "+-*/=,<>"):
                flush()
            i += 1
            continue
        if depth == 0 and t.type == tokenize.NAME and t.string == "else" and not cur:
            if lines and lines[-1].rstrip().endswith(":"):
                lines.append("    " * indent + "pass")
            lines.append("    " * (indent - 1) + "else:")
            i += 1
            continue
        if depth == 0 and t.type == tokenize.NAME and t.string in ("if", "elseif") and not cur:
            kw = "if"
            if t.string == "elseif":  # closes the previous branch at the same level
                if lines and lines[-1].rstrip().endswith(":"):
                    lines.append("    " * indent + "pass")
                indent -= 1
                kw = "elif"
            j, cond = i + 1, []
            if toks[j].string == "(":  # the parenthesised condition of a one-line `if (...) stmt end`
                d = 0
                while True:
                    d += toks[j].string == "("
                    d -= toks[j].string == ")"
                    cond.append(toks[j])
                    j += 1
                    if d == 0:
                        break
                nxt = toks[j]
                if (nxt.type == tokenize.OP and nxt.string not in ";([") or nxt.string in ("and", "or"):
                    while toks[j].type not in (tokenize.NEWLINE, tokenize.NL) and toks[j].string != ";":
                        cond.append(toks[j])  # `if (a) && (b)`: the condition goes on
                        j += 1
            else:
                while toks[j].type not in (tokenize.NEWLINE, tokenize.NL) and toks[j].string != ";":
                    cond.append(toks[j])
                    j += 1
            lines.append("    " * indent + kw + " " + tokenize.untokenize([(c.type, c.string) for c in cond]).strip() + ":")
            indent += 1
            i = j
            continue
        if depth == 0 and t.type == tokenize.NAME and t.string in ("for", "while") and not cur:
            j, hdr = i + 1, []
            while toks[j].type not in (tokenize.NEWLINE, tokenize.NL, tokenize.ENDMARKER) and toks[j].string != ";":
                hdr.append(toks[j])
                j += 1
            text = tokenize.untokenize([(c.type, c.string) for c in hdr]).strip()
            if t.string == "while":
                lines.append("    " * indent + "while " + text + ":")
            else:  # for v = a:b / a:s:b (also `in`, `∈`)
                m = re.match(r"(\w+)\s*(?:=|\bin\b)\s*(.+)$", text)
                if not m:
                    raise ArgumentError(f"unsupported for-loop header: {text}")
                parts = _split_range(m.group(2))
                lines.append("    " * indent + f"for {m.group(1)} in __range({', '.join(parts)}):")
            indent += 1
            i = j
            continue
        if depth == 0 and t.type == tokenize.NAME and t.string == "end":
            flush()
            if lines and lines[-1].rstrip().endswith(":"):
                lines.append("    " * indent + "pass")
            indent -= 1
            i += 1
            continue
        if t.type in (tokenize.INDENT, tokenize.DEDENT):
            i += 1
            continue
        cur.append(t)
        i += 1
    flush()
    return "\n".join(lines) + "\n"


@dataclass
class KernelDef:
    name: str
    kind: str                  # "parallel" | "parallel_indices"
    index_names: list          # parallel_indices: ["ix", "iy", ...]
    arrays: list               # argument names (Python identifiers) of the arrays, in order
    scalars: list
    args: list                 # all argument names in order, ("array" | "scalar", name)
    body: list                 # Python AST statements
    source: str = ""
    int_scalars: set = field(default_factory=set)  # scalars declared `::Integer` / `::Int*`
    options: dict = field(default_factory=dict)    # keyword options before `function`
    splat: str = ""            # `@parallel_indices (I...)`: the index tuple's name (indices of any rank)


# keyword options of `@parallel` / `@parallel_indices` definitions (src/parallel.jl:151-175,
# src/ParallelKernel/parallel.jl:160-172); the memopt family changes how the reference schedules the
# kernel, not its results, and is accepted without effect here
# optvars / optranges / optimize_halo_read tune src/memopt.jl's caching; the sweep here carries every
# read-only point and reads halos directly, so they are accepted and change nothing
_OPTIONS = {"ndims", "N", "inbounds", "padding", "memopt", "loopsize", "loopdim", "optvars", "optranges",
            "optimize_halo_read"}


def _array_uses(tree) -> set:
    """Names the body uses as arrays: FD macro operands, indexed names, `size(A, d)` operands and
    left-hand selections."""
    used = set()
    for n in ast.walk(tree):
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.args and isinstance(n.args[0], ast.Name):
            if n.func.id.startswith("__m_") or n.func.id in ("size", "eltype"):
                used.add(n.args[0].id)
        elif isinstance(n, ast.Subscript) and isinstance(n.value, ast.Name):
            if n.value.id.startswith("__lhs_"):
                if isinstance(n.slice, ast.Name):
                    used.add(n.slice.id)
            else:
                used.add(n.value.id)
    return used


_LOCAL_FN = re.compile(r"^[ \t]*(?!__m_)(\w+)[ \t]*\(([\w \t,]*)\)[ \t]*=(?!=)[ \t]*(?:return[ \t]+)?(.+)$", re.M)


def _local_functions(text: str):
    """One-line local function definitions in a kernel body (`f(a, b) = [return] expr`): removed
    from the statements and returned as name -> (parameters, expression), for inlining at each call."""
    fns = {}

    def take(m):
        params = [p.strip() for p in m.group(2).split(",") if p.strip()]
        try:
            expr = ast.parse(m.group(3).strip(), mode="eval").body
        except SyntaxError as e:
            raise ArgumentError(f"cannot parse the local function {m.group(1)}: {e}") from None
        fns[m.group(1)] = (params, expr)
        return ""
    return _LOCAL_FN.sub(take, text), fns


class _Inline(ast.NodeTransformer):
    """Calls of local functions replaced by their expression, parameters bound to the arguments."""

    def __init__(self, fns):
        self.fns = fns

    def visit_Call(self, n):
        self.generic_visit(n)
        if isinstance(n.func, ast.Name) and n.func.id in self.fns:
            params, expr = self.fns[n.func.id]
            if len(params) != len(n.args):
                raise ArgumentError(f"local function {n.func.id} takes {len(params)} arguments")
            bind = dict(zip(params, n.args))

            class _Bind(ast.NodeTransformer):
                def visit_Name(self, m):
                    return copy.deepcopy(bind[m.id]) if m.id in bind else m
            return self.visit(_Bind().visit(copy.deepcopy(expr)))
        return n


class _AugAssign(ast.NodeTransformer):
    """`a op= b` is `a = a op b` (Julia lowers it so)."""

    def visit_AugAssign(self, n):
        load = copy.deepcopy(n.target)
        for x in ast.walk(load):
            if hasattr(x, "ctx"):
                x.ctx = ast.Load()
        load.ctx = ast.Load()
        return ast.copy_location(ast.Assign(targets=[n.target], value=ast.BinOp(left=load, op=n.op, right=n.value)), n)


def _split_commas(text: str):
    """Items separated by commas outside brackets (`A::Data.Array{T,N}, B` is two arguments)."""
    items, cur, depth = [], "", 0
    for ch in text:
        depth += ch in "([{"
        depth -= ch in ")]}"
        if ch == "," and depth == 0:
            items.append(cur)
            cur = ""
        else:
            cur += ch
    return items + [cur]


def _split_options(head: str):
    """`key=value` items separated by blanks outside parentheses (values such as
    `optvars=(A, B)` or `optranges=(A=(-1:1, 0:0, 0:0),)` contain blanks)."""
    items, cur, depth = [], "", 0
    for ch in head:
        depth += ch in "([{"
        depth -= ch in ")]}"
        if ch.isspace() and depth == 0:
            if cur:
                items.append(cur)
            cur = ""
        else:
            cur += ch
    if depth != 0:
        raise ArgumentError(f"unbalanced parentheses in the kernel definition's options: {head}")
    return items + ([cur] if cur else [])


def parse(src: str) -> KernelDef:
    """Parse a Julia `@parallel` / `@parallel_indices` function definition."""
    m = re.search(r"@parallel(_indices)?\b(.*?)\bfunction\s+([^\s(]+)\s*\(", src, re.S)
    if not m:
        raise ArgumentError("expected `@parallel function name!(args...)` or `@parallel_indices (ix,...) function ...`")
    kind = "parallel_indices" if m.group(1) else "parallel"
    head, idx, options, splat = m.group(2).strip(), [], {}, ""
    if kind == "parallel_indices":
        mi = re.match(r"\(([^)]*)\)|([^\s=]+)(?=\s|$)", head)
        if not mi:
            raise ArgumentError("@parallel_indices: argument 'indices' must be a tuple of indices or a single index "
                                "(e.g. (ix, iy, iz) or (ix, iy) or ix ).")
        names = [s.strip() for s in (mi.group(1) if mi.group(1) is not None else mi.group(2)).split(",") if s.strip()]
        head = head[mi.end():].strip()
        ms = re.fullmatch(r"(\w+)\.\.\.", names[0]) if len(names) == 1 else None
        if ms:  # (I...): as many indices as the arrays have dimensions, used as A[I...]
            splat = _ident(ms.group(1))
        else:
            idx = [_ident(s) for s in names]
            if not 1 <= len(idx) <= 3:
                raise ArgumentError("@parallel_indices needs 1-3 index names")
    for opt in _split_options(head):
        k, eq, v = opt.partition("=")
        if not eq or k not in _OPTIONS:
            raise ArgumentError(f"unsupported keyword argument in the kernel definition: {opt}")
        options[k] = v
    if options.get("padding", "false") != "false":
        raise ArgumentError("padding=true is not supported by run-time compiled kernels")
    if "ndims" in options:  # one rank, or a tuple of ranks the definition serves (ndims=(2,3))
        nds = options["ndims"].strip("()").split(",")
        if not all(x.strip().isdigit() and 1 <= int(x) <= 3 for x in nds if x.strip()):
            raise ArgumentError("ndims must be 1, 2 or 3 (or a tuple of them)")
    if options.get("inbounds", "false") not in ("true", "false"):
        raise ArgumentError("inbounds must be true or false")
    # argument list: balanced parentheses after the name
    i, d = m.end() - 1, 0
    for j in range(i, len(src)):
        d += src[j] == "("
        d -= src[j] == ")"
        if d == 0:
            break
    arglist, rest = src[i + 1:j], src[j + 1:]
    rest = re.sub(r"^\s*where\s*(\{[^}]*\}|[^\n]*)", "", rest)  # `where T <: ...` clauses
    rest = rest.rstrip()
    if not rest.endswith("end"):
        raise ArgumentError("kernel definition must end with `end`")
    text, local_fns = _local_functions(_sanitize(rest[:-3]))
    body = _to_python(text)
    try:
        tree = ast.fix_missing_locations(_Inline(local_fns).visit(_AugAssign().visit(ast.parse(body))))
    except SyntaxError as e:
        raise ArgumentError(f"cannot parse the kernel body: {e}") from None
    used = _array_uses(tree)
    args, arrays, scalars, ints = [], [], [], set()
    for a in [s.strip() for s in _split_commas(arglist) if s.strip()]:
        nm, _, ty = a.partition("::")
        nm, ty = _ident(nm.strip()), ty.strip()
        # number and array types decide; untyped arguments and type parameters follow their use in the body
        if re.match(r"(Data\.Number|Real|AbstractFloat|Float\d*|Integer|U?Int\d*|Number)$", ty):
            is_array = False
        elif "Array" in ty or "Field" in ty:
            is_array = True
        else:
            is_array = nm in used
        args.append(("array" if is_array else "scalar", nm))
        (arrays if is_array else scalars).append(nm)
        if not is_array and re.match(r"(Integer|U?Int\d*)$", ty):
            ints.add(nm)
    if len(arrays) > MAX_ARRAYS or len(scalars) > MAX_SCALARS:
        raise ArgumentError(f"at most {MAX_ARRAYS} arrays and {MAX_SCALARS} scalars")
    for n in used - set(arrays):
        if n in scalars:
            raise ArgumentError(f"scalar argument {n} is used as an array")
    return KernelDef(m.group(3), kind, idx, arrays, scalars, args, tree.body, src, ints, options, splat)


# ---- code generation -----------------------------------------------------------------------
def _lit(v):
    return f"((R){float(v)!r})"


class _Gen:
    def __init__(self, kd: KernelDef, ndims: int, zloop: bool = False, split: bool = False, ordered: bool = False,
                 tma: bool = False):
        self.kd, self.nd = kd, ndims
        # the boundary-first variant (ps_jit_hide_communication): its block index comes from the
        # launch's tile order, and every warp counts itself in host-mapped memory at the end
        self.ordered = bool(ordered)
        self.exit = "goto ps_done_;" if self.ordered else "return;"
        # FP64 arrays with the arithmetic on FP32 pairs (R = jd, storage E = double); see _JD below
        self.split = bool(split)
        # memopt: each thread sweeps g.loop consecutive indices of the last dimension (z in 3-D, y in
        # 2-D) and carries read-only stencil points it already holds to the next index
        # (src/memopt.jl's register queues for loopdim 3 and 2, in plain code)
        self.zloop = bool(zloop) and kd.kind == "parallel" and ndims in (2, 3) and not uses_kernel_language(kd)
        self.sweep = ndims - 1 if self.zloop else None
        self.persist = []  # registers that live across the z sweep
        self.nstmt = 0
        self.macros = MACROS[ndims]
        self.sels = LHS[ndims]
        self.aidx = {n: i for i, n in enumerate(kd.arrays)}
        self.sidx = {n: i for i, n in enumerate(kd.scalars)}
        self.temps = {}  # temporary name -> (lhs inn mask, expression)
        self.checked = kd.options.get("inbounds", "false") != "true"
        self.locals = {}   # local variable -> "int" | "real" | "shared"
        self.shared = {}   # @sharedMem array -> index
        self.kernel_language = False
        self.uses_collectives = False  # @sync_threads, shuffles, votes
        self.table = None  # per-statement loads of an FD statement: (array, offsets) -> register
        # the TMA variant of a 3-D sweep: read-only stencil arrays staged plane by plane in shared
        # memory (ps_jit_launch_tma); staged: array -> offsets read; layout: set by source()
        self.tma = bool(tma) and self.zloop and ndims == 3 and not self.ordered
        self.staged = {}
        self.layout = None
        written = set()
        for n in ast.walk(ast.Module(body=kd.body, type_ignores=[])):
            if isinstance(n, ast.Assign):
                for t in n.targets:
                    if isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name):
                        written.add(t.slice.id if t.value.id.startswith("__lhs_") and isinstance(t.slice, ast.Name)
                                    else t.value.id)
        self.read_only = set(kd.arrays) - written  # read through the non-coherent cache (__ldg)

    # element of array `name` at 0-based integer index expressions (strings) per dimension
    def at(self, name, ix):
        k = self.aidx[name]
        ix = list(ix) + ["0"] * (3 - len(ix))
        return f"a{k}[({ix[0]}) + n{k}_0 * (({ix[1]}) + n{k}_1 * ({ix[2]}))]"

    # value of array-or-temporary `name` at thread index + integer offset vector `o`
    def val(self, name, o):
        if name in self.temps:
            li, e = self.temps[name]
            return self.expr(e, tuple(o[d] - ((li >> d) & 1) for d in range(3)))
        if name not in self.aidx:
            raise ArgumentError(f"unknown array {name}")
        t = ("tx", "ty", "tz")
        if self.table is not None:  # FD statement: one register per distinct (array, offset)
            key = (name, tuple(o[d] if d < self.nd else 0 for d in range(3)))
            if key not in self.table:
                self.table[key] = f"L{len(self.table)}"
            return self.table[key]
        return self.load(name, [f"{t[d]}+{o[d]}" if o[d] else t[d] for d in range(self.nd)])

    def wrap(self, ld):
        """A value read from an FP64 array as the arithmetic type (an FP32 pair in split mode; a value
        outside the pairs' range sets big_, reported with the next store)."""
        return f"jd_in({ld}, big_)" if self.split else ld

    def fd_loads(self, p):
        """Declarations of the statement's registered loads, and the bounds condition that covers
        them all (per array: the stencil's largest offset in each dimension)."""
        decl, box = [], {}
        t3 = ("tx", "ty", "tz")
        for (name, o), var in self.table.items():
            k = self.aidx[name]
            idx = [f"{t3[d]}+{o[d]}" if d < self.nd else "0" for d in range(3)]
            ref = f"a{k}[({idx[0]}) + n{k}_0 * (({idx[1]}) + n{k}_1 * ({idx[2]}))]"
            decl.append(f"{p}    const R {var} = " + self.wrap(f"__ldg(&{ref})" if name in self.read_only else ref) + ";")
            lo, hi = box.setdefault(k, ([0] * 3, [0] * 3))
            for d in range(self.nd):
                lo[d], hi[d] = min(lo[d], o[d]), max(hi[d], o[d])
        cond = []
        for k, (lo, hi) in box.items():
            for d in range(self.nd):
                if lo[d] < 0:
                    cond.append(f"{t3[d]} + {lo[d]} >= 0")
                cond.append(f"{t3[d]} + {hi[d]} < n{k}_{d}")
        return decl, " && ".join(cond)

    def zloop_statement(self, p, cond, box, decl, store):
        """An FD statement inside the sweep: a read-only point whose neighbour one index further along
        the sweep was loaded at the previous index comes from that register (read-only values do not
        change; the register is used only when the statement ran at the previous index)."""
        sd = self.sweep

        def along(o, s):
            o = list(o)
            o[sd] += s
            return tuple(o)

        j = self.nstmt
        self.nstmt += 1
        t3 = ("tx", "ty", "tz")
        keys = self.table
        loads, ups = [], []
        for (name, o), var in keys.items():
            k = self.aidx[name]
            idx = [f"{t3[d]}+{o[d]}" for d in range(3)]
            ref = f"a{k}[({idx[0]}) + n{k}_0 * (({idx[1]}) + n{k}_1 * ({idx[2]}))]"
            ro = name in self.read_only
            ld = self.wrap(f"__ldg(&{ref})" if ro else ref)
            nxt = (name, along(o, 1))
            if ro and self.tma:  # from the staged plane (placeholder resolved once the layout is known)
                self.staged.setdefault(name, set()).add(tuple(o))
                loads.append(f"{p}    const R {var} = " + self.wrap(f"__TMA[{k},{o[0]},{o[1]},{o[2]}]__") + ";")
                continue
            if ro and nxt in keys:
                loads.append(f"{p}    const R {var} = pr{j} ? P{j}_{keys[nxt][1:]} : {ld};")
            else:
                loads.append(f"{p}    const R {var} = {ld};")
            if ro and (name, along(o, -1)) in keys:
                self.persist.append(f"    R P{j}_{var[1:]} = 0;")
                ups.append(f"{p}    P{j}_{var[1:]} = {var};")
        self.persist.append(f"    bool pr{j} = false;")
        inner = loads + [store] + ups + [f"{p}    pr{j} = true;"]
        if not self.checked or not box:
            return [f"{p}if ({cond}) {{"] + inner + [f"{p}}} else pr{j} = false;"]
        return [f"{p}if ({cond}) {{", f"{p}  if (!({box})) {{ atomicOr(g.err, 1); pr{j} = false; }} else {{"] + \
            inner + [f"{p}  }}", f"{p}}} else pr{j} = false;"]

    def macro(self, mname, name, off):
        if mname not in self.macros:
            raise ArgumentError(f"unknown macro @{mname} for {self.nd}-D")
        kind, opd, inn = self.macros[mname]
        b = [off[d] + ((inn >> d) & 1) for d in range(3)]

        def shift(d, s):
            o = list(b)
            o[d] += s
            return self.val(name, o)

        dims = [d for d in range(3) if (opd >> d) & 1]
        if kind == SEL:
            return self.val(name, b)
        if kind == DIFF:
            return f"({shift(dims[0], 1)} - {self.val(name, b)})"
        if kind == DIFF2:
            c = self.val(name, b)
            return f"(({shift(dims[0], 1)} - {c}) - ({c} - {shift(dims[0], -1)}))"
        if kind in (AV, HARM):
            terms = []
            for c in range(1 << len(dims)):
                o = list(b)
                for j, d in enumerate(dims):
                    o[d] += (c >> j) & 1
                v = self.val(name, o)
                terms.append(f"((R)1.0 / {v})" if kind == HARM else v)
            s = terms[0]
            for t in terms[1:]:
                s = f"({s} + {t})"
            k = float(1 << len(dims))
            return f"({s} * {_lit(1.0 / k)})" if kind == AV else f"(((R)1.0 / {s}) * {_lit(k)})"
        if kind in (MAXLOC, MINLOC):
            f = "jl_max" if kind == MAXLOC else "jl_min"
            m = f"{f}({f}({shift(0, -1)}, {shift(0, 1)}), {self.val(name, b)})"
            for d in range(1, self.nd):
                m = f"{f}({m}, {f}({shift(d, -1)}, {shift(d, 1)}))"
            return m
        raise ArgumentError(f"macro @{mname} not supported")

    def is_bool(self, e):
        return self.etype(e) == "bool"

    # ---- types: "int" (Julia Int), "real" (the number type R), "bool"
    def etype(self, e):
        T = self.etype
        if isinstance(e, ast.Constant):
            return "bool" if isinstance(e.value, bool) else "int" if isinstance(e.value, int) else "real"
        if isinstance(e, ast.Name):
            if e.id in self.kd.index_names or (self.kd.kind == "parallel" and e.id in ("ix", "iy", "iz")):
                return "int"
            if e.id in self.sidx:
                return "int" if e.id in self.kd.int_scalars else "real"
            if e.id in self.locals:
                return self.locals[e.id]
            return "real"
        if isinstance(e, ast.UnaryOp):
            return "bool" if isinstance(e.op, ast.Not) else T(e.operand)
        if isinstance(e, (ast.Compare, ast.BoolOp)):
            return "bool"
        if isinstance(e, ast.BinOp):
            a, b = T(e.left), T(e.right)
            if isinstance(e.op, ast.Div):
                return "real"
            if isinstance(e.op, ast.Mult) and "bool" in (a, b):
                return b if a == "bool" else a
            return "int" if a in ("int", "bool") and b in ("int", "bool") else "real"
        if isinstance(e, ast.Attribute):
            return "int"
        if isinstance(e, ast.Call) and isinstance(e.func, ast.Name):
            f = e.func.id
            if f in ("size", "__m_warpsize", "__m_laneid", "__m_active_mask", "__m_vote_ballot_sync", "length",
                     "sizeof"):
                return "int"
            if f in ("__m_vote_any_sync", "__m_vote_all_sync"):
                return "bool"
            if f in ("__m_shfl_sync", "__m_shfl_up_sync", "__m_shfl_down_sync", "__m_shfl_xor_sync"):
                return T(e.args[1])
            if f in ("max", "min", "abs"):
                return "int" if all(T(a) == "int" for a in e.args) else "real"
            if f == "ifelse":
                return "int" if T(e.args[1]) == T(e.args[2]) == "int" else "real"
            return "real"
        return "real"

    def expr(self, e, off=(0, 0, 0), ctx="real"):
        E = lambda x, c=ctx: self.expr(x, off, c)  # noqa: E731
        if ctx == "auto":
            ctx = "int" if self.etype(e) in ("int", "bool") else "real"
        if isinstance(e, ast.Constant):
            if isinstance(e.value, bool):
                return "true" if e.value else "false"
            if isinstance(e.value, int) and ctx != "real":
                return f"{e.value}LL"
            return _lit(e.value)
        if isinstance(e, ast.Name):
            if e.id in self.kd.index_names:
                return f"((long long)t{'xyz'[self.kd.index_names.index(e.id)]} + 1)"
            if e.id in self.sidx:
                return f"s{self.sidx[e.id]}"
            if e.id in self.locals and self.locals[e.id] != "shared":
                return f"v_{e.id}"
            if self.kd.kind == "parallel" and e.id in ("ix", "iy", "iz")[:self.nd]:  # ParallelStencil.INDICES
                return f"((long long)t{e.id[1]} + 1)"
            raise ArgumentError(f"unknown name {e.id} in an expression")
        if isinstance(e, ast.UnaryOp):
            if isinstance(e.op, ast.USub):
                return f"(-{E(e.operand)})"
            if isinstance(e.op, ast.UAdd):
                return E(e.operand)
            if isinstance(e.op, ast.Not):
                return f"(!{E(e.operand, 'auto')})"
        if isinstance(e, ast.BinOp):
            if isinstance(e.op, ast.Pow):
                if isinstance(e.right, ast.Constant) and e.right.value in (2, 3) and not isinstance(e.right.value, bool):
                    x = E(e.left)
                    return f"({x} * {x})" if e.right.value == 2 else f"(({x} * {x}) * {x})"
                return f"pow({E(e.left, 'real')}, (R)({E(e.right, 'real')}))"
            if isinstance(e.op, ast.Mult) and (self.is_bool(e.left) or self.is_bool(e.right)):
                b, x = (e.left, e.right) if self.is_bool(e.left) else (e.right, e.left)
                if self.etype(x) == "int":
                    return f"((long long)({E(b, 'auto')}) * {E(x, 'int')})"
                return f"jl_bmul({E(b, 'auto')}, {E(x, 'real')})"
            if isinstance(e.op, (ast.FloorDiv, ast.Mod)):  # Julia ÷ and % (truncating)
                if self.etype(e) == "int":
                    return f"({E(e.left, 'int')} {'/' if isinstance(e.op, ast.FloorDiv) else '%'} {E(e.right, 'int')})"
                if isinstance(e.op, ast.Mod):
                    return f"fmod({E(e.left, 'real')}, {E(e.right, 'real')})"
                return f"trunc({E(e.left, 'real')} / {E(e.right, 'real')})"
            ops = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.Div: "/"}
            if type(e.op) not in ops:
                raise ArgumentError("unsupported operator")
            if self.etype(e) == "int" and not isinstance(e.op, ast.Div):
                # Julia: Int op Int is an Int, converted once where a real value is wanted
                v = f"({E(e.left, 'int')} {ops[type(e.op)]} {E(e.right, 'int')})"
                return f"((R){v})" if ctx == "real" else v
            return f"({E(e.left, 'real')} {ops[type(e.op)]} {E(e.right, 'real')})"
        if isinstance(e, ast.Compare):
            parts, left = [], e.left
            for op, right in zip(e.ops, e.comparators):
                sym = {ast.Lt: "<", ast.LtE: "<=", ast.Gt: ">", ast.GtE: ">=", ast.Eq: "==", ast.NotEq: "!="}[type(op)]
                c = "int" if self.etype(left) in ("int", "bool") and self.etype(right) in ("int", "bool") else "real"
                parts.append(f"({self.expr(left, off, c)} {sym} {self.expr(right, off, c)})")
                left = right
            return "(" + " && ".join(parts) + ")"
        if isinstance(e, ast.BoolOp):
            sym = " && " if isinstance(e.op, ast.And) else " || "
            return "(" + sym.join(self.expr(v, off, "auto") for v in e.values) + ")"
        if isinstance(e, ast.Attribute):  # @threadIdx().x etc. (1-based indices, like CUDA.jl)
            v = e.value
            if isinstance(v, ast.Call) and isinstance(v.func, ast.Name) and e.attr in ("x", "y", "z"):
                f = v.func.id
                base = {"__m_threadIdx": "threadIdx", "__m_blockIdx": "blockIdx", "__m_blockDim": "blockDim",
                        "__m_gridDim": "gridDim"}.get(f)
                if base:
                    self.kernel_language = True
                    plus = " + 1" if f in ("__m_threadIdx", "__m_blockIdx") else ""
                    return f"((long long){base}.{e.attr}{plus})"
            raise ArgumentError("unsupported attribute access")
        if isinstance(e, ast.Call) and isinstance(e.func, ast.Name):
            f = e.func.id
            if f in _COLLECTIVE:
                return self.collective(f, e.args, off)
            if f == "__m_warpsize":
                return "32LL"
            if f == "__m_laneid":
                self.kernel_language = True
                return "((long long)jl_laneid() + 1)"
            if f == "__m_active_mask":
                self.kernel_language = True
                return "((long long)__activemask())"
            if f.startswith("__m_"):
                if len(e.args) != 1 or not isinstance(e.args[0], ast.Name):
                    raise ArgumentError(f"@{f[4:]} takes one array")
                return self.macro(f[4:], e.args[0].id, off)
            if f == "size":
                a, d = e.args
                if a.id in self.shared:
                    return f"sm{self.shared[a.id]}_n{int(d.value) - 1}"
                return f"n{self.aidx[a.id]}_{int(d.value) - 1}"
            if f == "sizeof":  # sizeof(eltype(A)): bytes per element of the kernel's number type
                return "((long long)sizeof(E))"
            if f == "length" and e.args[0].id in self.aidx:
                k = self.aidx[e.args[0].id]
                return f"(n{k}_0 * n{k}_1 * n{k}_2)"
            if f in ("max", "min"):
                if self.etype(e) == "int":
                    r = E(e.args[0], "int")
                    for x in e.args[1:]:
                        r = f"{f}({r}, {E(x, 'int')})"
                    return r
                r = E(e.args[0], "real")
                for x in e.args[1:]:
                    r = f"jl_{f}({r}, {E(x, 'real')})"
                return r
            if f == "abs":
                return f"llabs({E(e.args[0], 'int')})" if self.etype(e) == "int" else f"fabs({E(e.args[0], 'real')})"
            if f == "inv":
                return f"((R)1.0 / {E(e.args[0], 'real')})"
            if f in ("one", "zero"):  # one(eltype(A)) etc.: the number type's 1 / 0
                return "((R)1)" if f == "one" else "((R)0)"
            if f == "ifelse":
                c, a, b = e.args
                t = "int" if self.etype(e) == "int" else "real"
                return f"({E(c, 'auto')} ? {E(a, t)} : {E(b, t)})"
            if f in _MATH:
                return f"{f}({E(e.args[0], 'real')})"
            raise ArgumentError(f"unsupported function {f}")
        if isinstance(e, ast.Subscript):
            return self.load(*self.subscript(e, off))
        raise ArgumentError(f"unsupported expression {ast.dump(e)[:80]}")

    def collective(self, f, args, off):
        """Warp shuffles and votes (src/ParallelKernel/kernel_language.jl:123-193): lanes are 1-based."""
        self.kernel_language = self.uses_collectives = True
        E = lambda x, c: self.expr(x, off, c)  # noqa: E731
        mask = f"(unsigned)({E(args[0], 'int')})"
        if f.startswith("__m_vote"):
            if len(args) != 2:
                raise ArgumentError(f"@{f[4:]}(mask, predicate)")
            fn = {"__m_vote_any_sync": "__any_sync", "__m_vote_all_sync": "__all_sync",
                  "__m_vote_ballot_sync": "__ballot_sync"}[f]
            r = f"{fn}({mask}, {E(args[1], 'auto')})"
            return f"((long long){r})" if fn == "__ballot_sync" else f"({r} != 0)"
        if len(args) not in (3, 4):
            raise ArgumentError(f"@{f[4:]}(mask, val, lane_or_delta[, width])")
        t = "long long" if self.etype(args[1]) == "int" else "E"
        val = f"({t})({E(args[1], 'int' if t == 'long long' else 'real')})"
        if t == "E":  # a real value is shuffled as the storage type (the pair's double in split mode)
            val = f"({t})((R)({E(args[1], 'real')}))"
        arg = f"(int)({E(args[2], 'int')})"
        if f == "__m_shfl_sync":
            arg = f"({arg} - 1)"
        width = f", (int)({E(args[3], 'int')})" if len(args) == 4 else ""
        fn = {"__m_shfl_sync": "__shfl_sync", "__m_shfl_up_sync": "__shfl_up_sync",
              "__m_shfl_down_sync": "__shfl_down_sync", "__m_shfl_xor_sync": "__shfl_xor_sync"}[f]
        r = f"{fn}({mask}, {val}, {arg}{width})"
        return f"((R)({r}))" if t == "E" else r

    def subscript(self, e, off=(0, 0, 0)):
        """`A[i, j, ...]` (1-based, Julia's `end` = size(A, d)) -> (A, 0-based index expressions)."""
        if not isinstance(e.value, ast.Name) or (e.value.id not in self.aidx and e.value.id not in self.shared):
            raise ArgumentError("indexing applies to array arguments and @sharedMem arrays")
        sl = e.slice.elts if isinstance(e.slice, ast.Tuple) else [e.slice]
        if len(sl) == 1 and isinstance(sl[0], ast.Name) and sl[0].id.startswith("__splat_"):
            if not self.kd.splat or sl[0].id != "__splat_" + self.kd.splat:
                raise ArgumentError(f"{sl[0].id[8:]}... is not the kernel's index tuple")
            return e.value.id, ["tx", "ty", "tz"][:self.nd]  # A[I...]: the thread's own point
        if len(sl) > 3:
            raise ArgumentError("at most 3 indices")

        def last(node, d):
            class _End(ast.NodeTransformer):
                def visit_Name(self, n):
                    if n.id == "end":
                        return ast.Call(ast.Name("size", ast.Load()), [ast.Name(e.value.id, ast.Load()),
                                                                       ast.Constant(d + 1)], [])
                    return n
            return _End().visit(node)

        return e.value.id, [f"({self.expr(last(x, d), off, 'int')}) - 1" for d, x in enumerate(sl)]

    def smem_ref(self, name, ix):
        j = self.shared[name]
        ix = list(ix) + ["0"] * (3 - len(ix))
        return f"sm{j}, sm{j}_n0, sm{j}_n1, sm{j}_n2, {ix[0]}, {ix[1]}, {ix[2]}, sm{j}_cap"

    # read of an element; unless `inbounds=true`, an index outside the array sets the error flag and
    # reads 0 (Julia's bounds check raises a BoundsError there)
    def load(self, name, ix):
        if name in self.shared:  # @sharedMem arrays are always bounds-checked (extents and the launch's shmem)
            return self.wrap(f"jl_lds({self.smem_ref(name, ix)}, g.err)")
        ro = name in self.read_only
        if not self.checked:
            return self.wrap(f"__ldg(&{self.at(name, ix)})" if ro else self.at(name, ix))
        k = self.aidx[name]
        ix = list(ix) + ["0"] * (3 - len(ix))
        return self.wrap(f"jl_ld{'g' if ro else ''}(a{k}, n{k}_0, n{k}_1, n{k}_2, {ix[0]}, {ix[1]}, {ix[2]}, g.err)")

    # ---- local variables of @parallel_indices bodies (Julia function scope: declared at the top)
    def infer_locals(self, stmts):
        for s in stmts:
            if isinstance(s, ast.Assign) and len(s.targets) == 1 and isinstance(s.targets[0], ast.Name):
                n = s.targets[0].id
                if n in self.aidx or n in self.sidx or n in self.kd.index_names:
                    raise ArgumentError(f"cannot assign to argument or index {n}")
                v = s.value
                if isinstance(v, ast.Call) and isinstance(v.func, ast.Name) and v.func.id == "__m_sharedMem":
                    if n in self.locals:
                        raise ArgumentError(f"@sharedMem array {n} is assigned twice")
                    self.locals[n] = "shared"
                    self.shared[n] = len(self.shared)
                    continue
                t = self.etype(v)
                t = "int" if t == "bool" else t
                if n in self.locals and self.locals[n] != t:
                    if self.locals[n] == "shared":
                        raise ArgumentError(f"@sharedMem array {n} is assigned twice")
                    self.locals[n] = "real"  # Int and Float assignments: keep the wider type
                else:
                    self.locals.setdefault(n, t)
            elif isinstance(s, ast.For):
                self.locals.setdefault(s.target.id, "int")
                self.infer_locals(s.body)
            elif isinstance(s, (ast.If, ast.While)):
                self.infer_locals(s.body)
                self.infer_locals(s.orelse)

    def shared_decl(self, name, call, p):
        """`A = @sharedMem(T, dims[, offset])`: a view of the launch's dynamic shared memory."""
        j = self.shared[name]
        args = call.args
        if len(args) not in (2, 3):
            raise ArgumentError("@sharedMem(T, dims[, offset])")
        ty = args[0]
        ok = (isinstance(ty, ast.Call) and isinstance(ty.func, ast.Name) and ty.func.id == "eltype") or \
            (isinstance(ty, ast.Attribute) and ty.attr == "Number") or \
            (isinstance(ty, ast.Name) and ty.id in ("Float64", "Float32"))
        if not ok:
            raise ArgumentError("@sharedMem element type must be the kernel's number type (eltype(A), Data.Number)")
        dims = args[1].elts if isinstance(args[1], ast.Tuple) else [args[1]]
        if not 1 <= len(dims) <= 3:
            raise ArgumentError("@sharedMem dims: 1 to 3 extents")
        ext = [f"({self.expr(d, ctx='int')})" for d in dims] + ["1LL"] * (3 - len(dims))
        offs = f"({self.expr(args[2], ctx='int')})" if len(args) == 3 else "0LL"
        self.kernel_language = True
        return [f"{p}sm{j}_off = {offs}; sm{j} = (E*)(ps_smem + (sm{j}_off > 0 ? sm{j}_off : 0));",
                f"{p}sm{j}_n0 = {ext[0]}; sm{j}_n1 = {ext[1]}; sm{j}_n2 = {ext[2]};",
                f"{p}sm{j}_cap = (g.smem - sm{j}_off) / (long long)sizeof(E);"]

    def stmt(self, s, ind):
        p = "    " * ind
        if isinstance(s, ast.If):
            out = [f"{p}if ({self.expr(s.test, ctx='auto')}) {{"]
            for b in s.body:
                out += self.stmt(b, ind + 1)
            if s.orelse:
                out.append(f"{p}}} else {{")
                for b in s.orelse:
                    out += self.stmt(b, ind + 1)
            return out + [f"{p}}}"]
        if isinstance(s, ast.For):
            it = s.iter
            if not (isinstance(it, ast.Call) and isinstance(it.func, ast.Name) and it.func.id == "__range"):
                raise ArgumentError("for loops run over a range a:b or a:s:b")
            v = f"v_{s.target.id}"
            a, b = self.expr(it.args[0], ctx="int"), self.expr(it.args[-1], ctx="int")
            step = self.expr(it.args[1], ctx="int") if len(it.args) == 3 else "1LL"
            out = [f"{p}{{ const long long st_ = {step}, hi_ = {b};",
                   f"{p}for ({v} = {a}; st_ > 0 ? {v} <= hi_ : {v} >= hi_; {v} += st_) {{"]
            for x in s.body:
                out += self.stmt(x, ind + 1)
            return out + [f"{p}}} }}"]
        if isinstance(s, ast.While):
            out = [f"{p}while ({self.expr(s.test, ctx='auto')}) {{"]
            for x in s.body:
                out += self.stmt(x, ind + 1)
            return out + [f"{p}}}"]
        if isinstance(s, ast.Pass):
            return []
        if isinstance(s, ast.Return):  # an early `return` inside a branch: this thread is done
            if s.value is not None:
                raise ArgumentError("kernels return nothing")
            return [f"{p}{self.exit}"]
        if isinstance(s, ast.Expr) and isinstance(s.value, ast.Call) and isinstance(s.value.func, ast.Name):
            f = s.value.func.id
            if f == "__m_sync_threads":
                self.kernel_language = self.uses_collectives = True
                return [f"{p}__syncthreads();"]
            raise ArgumentError(f"unsupported statement {f}")
        if not isinstance(s, ast.Assign) or len(s.targets) != 1:
            raise ArgumentError("kernel statements are assignments, if-blocks, loops or @sync_threads()")
        t = s.targets[0]
        if isinstance(t, ast.Name):  # local variable
            if self.locals.get(t.id) == "shared":
                return self.shared_decl(t.id, s.value, p)
            c = "int" if self.locals[t.id] == "int" else "real"
            cast = "long long" if c == "int" else "R"
            return [f"{p}v_{t.id} = ({cast})({self.expr(s.value, ctx=c)});"]
        if isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name) and t.value.id.startswith("__lhs_"):
            sel, name = t.value.id[6:], t.slice.id
            if sel not in self.sels:
                raise ArgumentError(f"@{sel} cannot be a left-hand side")
            li = self.sels[sel]
            if name in self.temps:  # on-the-fly temporary: inlined where it is used
                return []
            k = self.aidx[name]
            t3 = ("tx", "ty", "tz")
            cond = " && ".join(f"{t3[d]} < n{k}_{d} - {2 * ((li >> d) & 1)}" for d in range(self.nd))
            idx = [f"{t3[d]}+{(li >> d) & 1}" for d in range(self.nd)]
            self.table = {}
            rhs = self.expr(s.value)
            decl, box = self.fd_loads(p)
            store = f"{p}    {self.at(name, idx)} = (E)({rhs});" + (" if (big_) atomicOr(g.err, 4);" if self.split else "")
            if self.zloop:
                out = self.zloop_statement(p, cond, box, decl, store)
                self.table = None
                return out
            self.table = None
            if not self.checked or not box:
                return [f"{p}if ({cond}) {{"] + decl + [store, f"{p}}}"]
            # Julia's bounds check, once per statement: the whole stencil inside every array it reads
            return [f"{p}if ({cond}) {{", f"{p}  if (!({box})) {{ atomicOr(g.err, 1); }} else {{"] + decl + \
                [store, f"{p}  }}", f"{p}}}"]
        if isinstance(t, ast.Subscript):  # @parallel_indices: A[i, j] = expr
            name, ix = self.subscript(t)
            val = self.expr(s.value, ctx="real")
            chk = " if (big_) atomicOr(g.err, 4);" if self.split else ""
            if name in self.shared:
                return [f"{p}jl_sts({self.smem_ref(name, ix)}, g.err, (E)((R)({val})));{chk}"]
            if not self.checked:
                return [f"{p}{self.at(name, ix)} = (E)((R)({val}));{chk}"]
            k = self.aidx[name]
            ix = list(ix) + ["0"] * (3 - len(ix))
            return [f"{p}jl_st(a{k}, n{k}_0, n{k}_1, n{k}_2, {ix[0]}, {ix[1]}, {ix[2]}, g.err, (E)((R)({val})));{chk}"]
        raise ArgumentError("unsupported left-hand side")

    def collect_temps(self):
        """On-the-fly arrays: left-hand arrays that are not arguments (src/parallel.jl:789-819)."""
        writes = {s.targets[0].slice.id for s in self.kd.body if _is_sel_assign(s)} & set(self.aidx)
        for s in self.kd.body:
            if not _is_sel_assign(s) or s.targets[0].slice.id in self.aidx:
                continue
            sel, name = s.targets[0].value.id[6:], s.targets[0].slice.id
            names = {n.id for n in ast.walk(s.value) if isinstance(n, ast.Name)}
            if sel != "all":
                raise ArgumentError("unsupported kernel statements in @parallel kernel definition: partial assignments "
                                    "are not possible for arrays that are not stored in global memory (arrays that "
                                    "are not among the arguments of the kernel); use '@all' instead.")
            if name in names:
                raise ArgumentError("unsupported kernel statements in @parallel kernel definition: auto-dependency is "
                                    "not possible for arrays that are not stored in global memory (arrays that are "
                                    "not among the arguments of the kernel).")
            if names & writes:
                raise ArgumentError(f"unsupported kernel statements in @parallel kernel definition: the assignment of "
                                    f"{name} should be done on the fly as it is not among the arguments of the kernel; "
                                    f"however, this is not possible because it depends on at least one variable that "
                                    f"is not read-only within the scope of the kernel (any of: {sorted(writes)}).")
            self.temps[name] = (self.sels[sel], s.value)

    # ---- the TMA variant of a 3-D sweep (ps_jit_launch_tma)
    TMA_TY = 8  # thread rows per block (blocks of 32 x 8 threads)

    def tma_layout(self, real):
        """Stage layout: per staged array (in argument order) its box (x from the tile origin rounded
        down to 16 bytes, y from the lowest offset) and its bytes in a stage; all arrays share the z
        planes ZL..ZH relative to the thread's index. Raises _NoTma where the variant cannot apply."""
        es = 4 if real == "float" else 8
        al = 16 // es
        xc = 4 if es == 4 else 2  # x cells per thread: a block covers 32 * xc columns
        names = [n for n in self.kd.arrays if n in self.staged]
        if not names or len(names) > 8:
            raise _NoTma()
        zl = min(o[2] for n in names for o in self.staged[n])
        zh = max(o[2] for n in names for o in self.staged[n])
        arrays, off = [], 0
        for n in names:
            offs = self.staged[n]
            xl, xh = min(o[0] for o in offs), max(o[0] for o in offs)
            yl, yh = min(o[1] for o in offs), max(o[1] for o in offs)
            xs = (xl // al) * al
            bx = -(-(32 * xc + xh - xs) // al) * al
            by = self.TMA_TY + yh - yl
            if bx > 256 or by > 256:
                raise _NoTma()
            nbytes = bx * by * es
            arrays.append({"name": n, "k": self.aidx[n], "xs": xs, "ys": yl, "bx": bx, "by": by, "off": off})
            off += -(-nbytes // 128) * 128
        span = zh - zl + 1
        # planes in flight ahead of the step: as many as fit a ring of TMA_RING_BYTES (2 to 8)
        ahead = max(2, min(8, TMA_RING_BYTES // off - span))
        stages = span + ahead
        smem = stages * off + 8 * stages
        if smem > 200 * 1024:
            raise _NoTma()
        return {"arrays": arrays, "zl": zl, "span": span, "stages": stages, "stage": off, "smem": smem, "xc": xc,
                "tx_bytes": sum(a["bx"] * a["by"] * es for a in arrays)}

    def tma_resolve(self, body):
        """Staged loads from the ring: the plane of index tz + oz sits in the stage of sweep step it_
        + (oz - ZL)."""
        L = self.layout
        by_k = {a["k"]: a for a in L["arrays"]}

        def sub(m):
            k, ox, oy, oz = (int(x) for x in m.groups())
            a = by_k[k]
            return (f"((const E*)(jt_p{oz - L['zl']} + {a['off']}))[(threadIdx.y + {oy - a['ys']}) * {a['bx']} + "
                    f"(jt_lx + {ox - a['xs']})]")
        pat = re.compile(r"__TMA\[(\d+),(-?\d+),(-?\d+),(-?\d+)\]__")
        head = ["    if (!jt_to) {", "    #pragma unroll",
                f"    for (int jt_xc = 0; jt_xc < {L['xc']}; ++jt_xc) {{",
                "    const int jt_lx = (int)threadIdx.x + 32 * jt_xc;  // this cell's column in the block's tile",
                "    const long long tx = (long long)jt_x0 + jt_lx;"]
        return head + [pat.sub(sub, line) for line in body] + ["    }", "    }"]

    def tma_loop(self):
        """Guard, loop head and loop tail of the TMA sweep: thread 0 keeps a ring of `stages` planes
        in flight (one mbarrier per stage, bounded waits), every thread waits for the planes of its
        step, and after a block barrier the stage of the plane no longer needed is refilled. The
        ring's bookkeeping is 32-bit: stage of the step's first plane, one phase bit per stage."""
        L = self.layout
        S, SP = L["stages"], L["span"]
        issue = [f"        jt_expect(jt_bar + s_, {L['tx_bytes']}u);"]
        for i, a in enumerate(L["arrays"]):
            issue.append(f"        jt_tma3(ps_smem + s_ * {L['stage']} + {a['off']}, &t_.tm[{i}], jt_bar + s_, "
                         f"jt_x0 + ({a['xs']}), jt_y0 + ({a['ys']}), jt_z0 + ({L['zl']}) + q_);")
        guard = ""  # no ranges: the statements' masks already exclude threads past the arrays

        def stage(c):  # stage of plane it_ + c (c < S)
            return f"(jt_s + {c} >= {S} ? jt_s + {c - S} : jt_s + {c})" if c else "jt_s"
        planes = "\n".join(f"    unsigned char* const jt_p{c} = ps_smem + {stage(c)} * {L['stage']};" for c in range(SP))
        zpre = "\n" + "\n".join(self.persist) + f"""
    unsigned long long* const jt_bar = reinterpret_cast<unsigned long long*>(ps_smem + {S} * {L['stage']});
    const int jt_tid = threadIdx.y * 32 + threadIdx.x;
    const int jt_x0 = (int)blockIdx.x * {32 * L['xc']}, jt_y0 = (int)blockIdx.y * {self.TMA_TY};
    const int jt_z0 = (int)(blockIdx.z * g.loop);
    const int jt_nk = (int)min(g.loop, g.cnt[2] - (long long)jt_z0), jt_nq = jt_nk + {SP - 1};
    int jt_issued = 0;
    auto jt_issue = [&](int q_, int s_) {{
{chr(10).join(issue)}
    }};
    if (jt_tid == 0) {{
        for (int s_ = 0; s_ < {S}; ++s_) jt_bar_init(jt_bar + s_);
        jt_fence_init();
{chr(10).join(f"        jt_prefetch(&t_.tm[{i}]);" for i in range(len(L["arrays"])))}
    }}
    __syncthreads();
    if (jt_tid == 0)
        for (; jt_issued < jt_nq && jt_issued < {S}; ++jt_issued) jt_issue(jt_issued, jt_issued);
    bool jt_to = false;  // a wait for a staged plane gave up
    unsigned jt_ph = 0;  // bit s: parity of the next wait on stage s
    for (int c_ = 0; c_ < {SP - 1}; ++c_) {{  // the first step's planes but its last
        if (!jt_to) jt_to = !jt_wait(jt_bar + c_, 0u);
        jt_ph ^= 1u << c_;
    }}
    int jt_s = 0;  // stage of plane it_
    int jt_w = {SP - 1};  // stage of the plane this step waits for: it_ + {SP - 1}
    for (int it_ = 0; it_ < jt_nk; ++it_) {{
    const long long uz = (long long)jt_z0 + it_;
    const long long tz = uz;
    if (!jt_to) jt_to = !jt_wait(jt_bar + jt_w, (jt_ph >> jt_w) & 1u);
    jt_ph ^= 1u << jt_w;
{planes}"""
        zpost = f"""    if (__syncthreads_or(jt_to)) {{
        if (jt_tid == 0) {{
            atomicOr(g.err, 8);
            for (int q_ = it_; q_ < jt_issued; ++q_) jt_wait(jt_bar + q_ % {S}, (unsigned)((q_ / {S}) & 1));
        }}
        break;
    }}
    if (jt_tid == 0 && jt_issued < jt_nq) {{ jt_issue(jt_issued, jt_s); ++jt_issued; }}
    jt_s = jt_s + 1 == {S} ? 0 : jt_s + 1;
    jt_w = jt_w + 1 == {S} ? 0 : jt_w + 1;
    }}"""
        return guard, zpre, zpost

    def body_lines(self):
        """The kernel body's statements as CUDA C lines (one thread's work)."""
        out = []
        for s in self.kd.body:
            out += self.stmt(s, 1)
        return out

    def extra_decl(self):
        """Further declarations at the top of the kernel (none here; the derivative kernels add theirs)."""
        return []

    def types(self, real):
        if self.split:
            if real != "double":
                raise ArgumentError("fp64='split' applies to FP64 arrays")
            return "typedef double E;" + _JD + "typedef jd R;"
        return f"typedef {real} R;\ntypedef R E;"

    def source(self, real):
        kd = self.kd
        self.collect_temps()
        self.infer_locals(kd.body)
        body = self.body_lines()
        if self.tma:
            self.layout = self.tma_layout(real)
            body = self.tma_resolve(body)
        decl = ["    bool big_ = false;"] if self.split else []
        for name, k in self.aidx.items():
            decl.append(f"    E* const a{k} = (E*)g.a[{k}];")
            decl.append(f"    const long long n{k}_0 = g.n[{k}][0], n{k}_1 = g.n[{k}][1], n{k}_2 = g.n[{k}][2];")
        for name, k in self.sidx.items():
            if name in kd.int_scalars:
                decl.append(f"    const long long s{k} = (long long)g.s[{k}];")
            else:
                decl.append(f"    const R s{k} = {self.wrap(f'g.s[{k}]') if self.split else f'(R)g.s[{k}]'};")
        for name, t in self.locals.items():
            if t == "shared":
                j = self.shared[name]
                decl.append(f"    E* sm{j} = nullptr; long long sm{j}_off = 0, sm{j}_n0 = 0, sm{j}_n1 = 1, "
                            f"sm{j}_n2 = 1, sm{j}_cap = 0;")
            else:
                decl.append(f"    {'long long' if t == 'int' else 'R'} v_{name} = 0;")
        decl += self.extra_decl()
        bi = "bi" if self.ordered else "blockIdx"
        if self.uses_collectives:
            # barriers, shuffles and votes need every thread of a block: a block that reaches past the
            # ranges leaves as a whole before any of them (block-uniform) and reports it (flag 2)
            guard = f"""    if (({bi}.x + 1LL) * blockDim.x > g.cnt[0] || ({bi}.y + 1LL) * blockDim.y > g.cnt[1] ||
        ({bi}.z + 1LL) * blockDim.z > g.cnt[2]) {{
        if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomicOr(g.err, 2);
        {self.exit}
    }}"""
        else:
            guard = f"    if (ux >= g.cnt[0] || uy >= g.cnt[1] || uz >= g.cnt[2]) {self.exit}"
        zpre, zpost = "", ""
        u, t, c = ("ux", "uy", "uz"), ("tx", "ty", "tz"), "xyz"
        grid = [d for d in range(3) if d != self.sweep]
        udecl = ", ".join(f"{u[d]} = {bi}.{c[d]} * (long long)blockDim.{c[d]} + threadIdx.{c[d]}" for d in grid)
        if self.zloop:  # blockDim of the sweep dimension is 1; each block covers g.loop consecutive indices
            sd = self.sweep
            guard = "    if (" + " || ".join(f"{u[d]} >= g.cnt[{d}]" for d in grid) + f") {self.exit}"
            zpre = "\n" + "\n".join(self.persist) + f"""
    for (long long it_ = 0; it_ < g.loop; ++it_) {{
    const long long {u[sd]} = {bi}.{c[sd]} * g.loop + it_;
    if ({u[sd]} >= g.cnt[{sd}]) break;
    const long long {t[sd]} = g.lo[{sd}] + {u[sd]};"""
            zpost = "    }"
        if self.tma:
            guard, zpre, zpost = self.tma_loop()
        pos = "const long long " + ", ".join(f"{t[d]} = g.lo[{d}] + {u[d]}" for d in grid)
        # the boundary-first variant: the body in a block that a finished thread jumps past, then the count
        head = "    const uint3 bi = jl_block(g);\n    {\n" if self.ordered else ""
        # the ordered block index and the count raise register use (56 -> 72 for the diffusion step in
        # split FP64, 4 -> 3 blocks per SM); its launches use blocks of <= 256 threads
        bounds = "__launch_bounds__(256, 4) " if self.ordered else ""
        tail = "    }\nps_done_:\n    jl_block_done(g);\n" if self.ordered else ""
        sweep = f", {c[self.sweep]} sweep" if self.zloop else ""
        return f"""// {kd.kind} {kd.name} ({self.nd}-D, {real}{sweep}) -- generated by ps_gb300.jit
{self.types(real)}
struct ps_jit_args {{ void* a[{MAX_ARRAYS}]; long long n[{MAX_ARRAYS}][3]; double s[{MAX_SCALARS}]; long long lo[3]; long long cnt[3]; int* err; long long smem; long long loop; unsigned* ocnt; int ord[10]; }};
{_TMA_HELPERS if self.tma else ""}{_BLOCK_ORDER if self.ordered else ""}
__device__ __forceinline__ bool jl_in(long long n0, long long n1, long long n2, long long i, long long j, long long k) {{
    return (unsigned long long)i < (unsigned long long)n0 && (unsigned long long)j < (unsigned long long)n1 && (unsigned long long)k < (unsigned long long)n2; }}
__device__ __forceinline__ E jl_ld(const E* a, long long n0, long long n1, long long n2, long long i, long long j, long long k, int* err) {{
    if (jl_in(n0, n1, n2, i, j, k)) return a[i + n0 * (j + n1 * k)];
    atomicOr(err, 1); return (E)0; }}
__device__ __forceinline__ E jl_ldg(const E* a, long long n0, long long n1, long long n2, long long i, long long j, long long k, int* err) {{
    if (jl_in(n0, n1, n2, i, j, k)) return __ldg(&a[i + n0 * (j + n1 * k)]);
    atomicOr(err, 1); return (E)0; }}
__device__ __forceinline__ void jl_st(E* a, long long n0, long long n1, long long n2, long long i, long long j, long long k, int* err, E v) {{
    if (jl_in(n0, n1, n2, i, j, k)) a[i + n0 * (j + n1 * k)] = v; else atomicOr(err, 1); }}
__device__ __forceinline__ E jl_lds(const E* a, long long n0, long long n1, long long n2, long long i, long long j, long long k, long long cap, int* err) {{
    const long long l = i + n0 * (j + n1 * k);
    if (a && jl_in(n0, n1, n2, i, j, k) && l < cap) return a[l];
    atomicOr(err, 1); return (E)0; }}
__device__ __forceinline__ void jl_sts(E* a, long long n0, long long n1, long long n2, long long i, long long j, long long k, long long cap, int* err, E v) {{
    const long long l = i + n0 * (j + n1 * k);
    if (a && jl_in(n0, n1, n2, i, j, k) && l < cap) a[l] = v; else atomicOr(err, 1); }}
__device__ __forceinline__ unsigned jl_laneid() {{ unsigned l; asm volatile("mov.u32 %0, %%laneid;" : "=r"(l)); return l; }}
template <typename T> struct jl_f64 {{ static constexpr bool v = false; }};
template <> struct jl_f64<double> {{ static constexpr bool v = true; }};
template <typename T> struct jl_f32 {{ static constexpr bool v = false; }};
template <> struct jl_f32<float> {{ static constexpr bool v = true; }};
__device__ __forceinline__ long long jl_key(long long b) {{ return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL); }}
__device__ __forceinline__ bool jl_nanb(long long b) {{ return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL; }}
// Julia's max / min (NaN-propagating, -0.0 < 0.0); doubles compare as integer keys (the FP64 pipe is slow)
// and a NaN operand is returned itself; floats use max.NaN / min.NaN (the same bits as the subtraction
// form, whose NaN is the canonical one)
template <typename T>
__device__ __forceinline__ T jl_maxt(T x, T y) {{
    if constexpr (jl_f64<T>::v) {{
        const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
        const T r = jl_key(bx) >= jl_key(by) ? x : y;
        return jl_nanb(bx) ? x : jl_nanb(by) ? y : r;
    }} else if constexpr (jl_f32<T>::v) {{
        float d; asm("max.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(x), "f"(y)); return d;
    }} else {{ T d = x - y; T r = signbit(d) ? y : x; return (isnan(x) || isnan(y)) ? d : r; }}
}}
template <typename T>
__device__ __forceinline__ T jl_mint(T x, T y) {{
    if constexpr (jl_f64<T>::v) {{
        const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
        const T r = jl_key(bx) < jl_key(by) ? x : y;
        return jl_nanb(bx) ? x : jl_nanb(by) ? y : r;
    }} else if constexpr (jl_f32<T>::v) {{
        float d; asm("min.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(x), "f"(y)); return d;
    }} else {{ T d = x - y; T r = signbit(d) ? x : y; return (isnan(x) || isnan(y)) ? d : r; }}
}}
__device__ __forceinline__ R jl_max(R x, R y) {{ return jl_maxt<R>(x, y); }}
__device__ __forceinline__ R jl_min(R x, R y) {{ return jl_mint<R>(x, y); }}
__device__ __forceinline__ R jl_bmul(bool b, R x) {{ return b ? x : copysign((R)0, x); }}
extern "C" __global__ void {bounds}ps_jit_entry({'const __grid_constant__ ps_jit_targs t_' if self.tma else 'const ps_jit_args g'}) {{
    extern __shared__ __align__({128 if self.tma else 16}) unsigned char ps_smem[];
{'    const ps_jit_args& g = t_.g;' + chr(10) if self.tma else ''}{head}    const long long {udecl};
{guard}
    {pos};
    (void)ps_smem;
{chr(10).join(decl)}{zpre}
{chr(10).join(body)}
{zpost}
{tail}}}
"""


class _NoTma(Exception):
    """The TMA variant does not apply to this kernel (no staged stencil arrays, more than eight, or
    boxes or a ring too large); the plain sweep is generated instead."""


# TMA staging of the 3-D sweep variant: the argument block with the tensor maps in front (the
# layout ps_jit_launch_tma fills), mbarrier set-up, a bounded wait (a wait that gives up makes the
# block stop and report flag 8) and the 3-D tile load into shared memory.
_TMA_HELPERS = r"""
struct alignas(64) ps_jit_targs { alignas(64) unsigned long long tm[8][16]; ps_jit_args g; };
__device__ __forceinline__ unsigned jt_s32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void jt_bar_init(unsigned long long* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(jt_s32(b)) : "memory"); }
__device__ __forceinline__ void jt_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void jt_prefetch(const void* m) {
    asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<unsigned long long>(m)) : "memory"); }
__device__ __forceinline__ void jt_expect(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(jt_s32(b)), "r"(bytes) : "memory"); }
__device__ __forceinline__ bool jt_wait(unsigned long long* b, unsigned parity) {
    for (int i = 0; i < (1 << 22); ++i) {
        unsigned ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(jt_s32(b)), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void jt_tma3(void* dst, const void* map, unsigned long long* b, int x, int y, int z) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
                 :: "r"(jt_s32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(jt_s32(b)), "r"(x), "r"(y), "r"(z)
                 : "memory"); }
"""


# Block order of the boundary-first variant (ps_jit_hide_communication): the 1-D grid's first
# ord[9] blocks take the tiles holding boundary indices -- whole layers at both ends of z, then
# whole rows at both ends of y, then column ends of x -- the rest the inner block; each boundary
# block counts itself in host-mapped memory once its stores are done (one system-scope fence and
# atomic per block: per-warp fences measured 22 % slower).
_BLOCK_ORDER = r"""
__device__ __forceinline__ uint3 jl_block(const ps_jit_args& g) {
    const int TX = g.ord[0], TY = g.ord[1], TZ = g.ord[2], bx0 = g.ord[3], bx1 = g.ord[4], by0 = g.ord[5],
              by1 = g.ord[6], bz0 = g.ord[7], bz1 = g.ord[8], nb = g.ord[9];
    int i = (int)blockIdx.x;
    const int IX = TX - bx0 - bx1, IY = TY - by0 - by1;
    if (i >= nb) { i -= nb; return make_uint3(bx0 + i % IX, by0 + (i / IX) % IY, bz0 + i / (IX * IY)); }
    const int layer = TX * TY, nzfull = (bz0 + bz1) * layer;
    if (i < nzfull) { const int l = i / layer, r = i % layer; return make_uint3(r % TX, r / TX, l < bz0 ? l : TZ - bz1 + (l - bz0)); }
    i -= nzfull;
    const int frame = layer - IX * IY, z = bz0 + i / frame;
    int r = i % frame;
    const int nyfull = (by0 + by1) * TX;
    if (r < nyfull) { const int row = r / TX; return make_uint3(r % TX, row < by0 ? row : TY - by1 + (row - by0), z); }
    r -= nyfull;
    const int ex = bx0 + bx1, c = r % ex;
    return make_uint3(c < bx0 ? c : TX - bx1 + (c - bx0), by0 + r / ex, z);
}
__device__ __forceinline__ void jl_block_done(const ps_jit_args& g) {
    if ((int)blockIdx.x >= g.ord[9]) return;
    __syncthreads();  // every thread of the block is past its stores (the variant has no early exit)
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) { __threadfence_system(); atomicAdd_system(g.ocnt, 1u); }
}
"""


# Split FP64 arithmetic for generated kernels: FP64 values as FP32 pairs (h + l, 47-bit
# significands rounded to nearest; |x| < 2^128, magnitudes below 2^-126 flush to 0), split from
# doubles with integer operations, sums by exact two-sums, products with FMA error terms, division
# by one correction step, comparisons and math functions through FP64; results are written back as
# FP64. Each operation is exact to ~2^-46 of its operands' magnitude.
_JD = r"""
__device__ __forceinline__ double jd_f64(float f) {  // exact float -> double with integer operations
    const unsigned b = __float_as_uint(f);
    unsigned hi = (((b >> 3) & 0x0FFFFFFFu) + 0x38000000u) | (b & 0x80000000u);
    hi = (b & 0x7F800000u) ? hi : (b & 0x80000000u);
    return __hiloint2double((int)hi, (int)(b << 29));
}
__device__ __forceinline__ void jd_split2(double x, float& h, float& l, bool& big) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned t = hw & 0x7FFFFFFFu, sgn = hw & 0x80000000u;
    const unsigned fb = __funnelshift_l(lw, hw, 3) ^ 0x40000000u;
    h = __uint_as_float((fb & 0x7FFFFFFFu) | sgn);
    // the next 23 bits, rounded to nearest at the 47th (an unbiased split)
    const unsigned mi = ((lw >> 6) & 0x7FFFFFu) + ((lw >> 5) & 1u);
    const float m = __uint_as_float(mi | 0x4B000000u) - 8388608.0f;
    const unsigned sb = (((hw << 3) & 0xFF800000u) - 0xD7000000u) | sgn;
    l = m * __uint_as_float(sb);
    h = t < 0x38100000u ? 0.0f : h;
    l = t < 0x3AF00000u ? 0.0f : l;
    big |= t >= 0x47F00000u;
}
struct jd {
    float h, l;
    __device__ __forceinline__ jd() : h(0.0f), l(0.0f) {}
    __device__ __forceinline__ jd(float h_, float l_) : h(h_), l(l_) {}
    __device__ __forceinline__ jd(double x) { bool b = false; jd_split2(x, h, l, b); }
    __device__ __forceinline__ jd(long long v) : jd((double)v) {}
    __device__ __forceinline__ jd(int v) : jd((double)v) {}
    __device__ __forceinline__ explicit operator double() const { return jd_f64(h) + jd_f64(l); }
};
__device__ __forceinline__ jd jd_in(double x, bool& big) { jd r; jd_split2(x, r.h, r.l, big); return r; }
__device__ __forceinline__ jd jd_fast2(float s, float e) { const float h = s + e; return jd(h, e - (h - s)); }
__device__ __forceinline__ jd operator+(jd a, jd b) {
    const float s = a.h + b.h, bb = s - a.h, e = (a.h - (s - bb)) + (b.h - bb);
    return jd_fast2(s, e + (a.l + b.l));
}
__device__ __forceinline__ jd operator-(jd a) { return jd(-a.h, -a.l); }
__device__ __forceinline__ jd operator-(jd a, jd b) { return a + (-b); }
__device__ __forceinline__ jd operator*(jd a, jd b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return jd_fast2(p, e);
}
__device__ __forceinline__ jd operator/(jd a, jd b) {
    const float q1 = a.h / b.h;
    const jd r = a - jd(q1, 0.0f) * b;
    return jd_fast2(q1, r.h / b.h);
}
__device__ __forceinline__ bool operator<(jd a, jd b) { return (double)a < (double)b; }
__device__ __forceinline__ bool operator>(jd a, jd b) { return (double)a > (double)b; }
__device__ __forceinline__ bool operator<=(jd a, jd b) { return (double)a <= (double)b; }
__device__ __forceinline__ bool operator>=(jd a, jd b) { return (double)a >= (double)b; }
__device__ __forceinline__ bool operator==(jd a, jd b) { return (double)a == (double)b; }
__device__ __forceinline__ bool operator!=(jd a, jd b) { return (double)a != (double)b; }
__device__ __forceinline__ bool signbit(jd a) { return signbit(a.h); }
__device__ __forceinline__ bool isnan(jd a) { return isnan(a.h) || isnan(a.l); }
__device__ __forceinline__ jd fabs(jd a) { return signbit(a.h) ? -a : a; }
__device__ __forceinline__ jd copysign(jd a, jd b) { const jd m = fabs(a); return signbit(b.h) ? -m : m; }
#define JD_F1(f) __device__ __forceinline__ jd f(jd a) { return jd(::f((double)a)); }
JD_F1(exp) JD_F1(log) JD_F1(sqrt) JD_F1(sin) JD_F1(cos) JD_F1(tan) JD_F1(tanh) JD_F1(sinh) JD_F1(cosh)
JD_F1(atan) JD_F1(asin) JD_F1(acos) JD_F1(log10) JD_F1(exp2) JD_F1(cbrt) JD_F1(trunc)
__device__ __forceinline__ jd pow(jd a, jd b) { return jd(::pow((double)a, (double)b)); }
__device__ __forceinline__ jd fmod(jd a, jd b) { return jd(::fmod((double)a, (double)b)); }
"""


def _is_sel_assign(s):
    t = s.targets[0] if isinstance(s, ast.Assign) and len(s.targets) == 1 else None
    return isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name) and t.value.id.startswith("__lhs_") \
        and isinstance(t.slice, ast.Name)


def generate(kd: KernelDef, ndims: int, dtype: str, zloop: bool = False) -> str:
    """CUDA C of kernel `kd` for `ndims`-D arrays of `dtype` ("double" or "float"); zloop: the memopt
    variant (2-D and 3-D `@parallel` kernels), each thread sweeping consecutive indices of the last
    dimension."""
    return _Gen(kd, ndims, zloop).source(dtype)


def _generate_info(kd: KernelDef, ndims: int, dtype: str, zloop: bool = False, split: bool = False,
                   ordered: bool = False, tma: bool = False):
    """(source, uses collectives, TMA layout or None); tma asks for the TMA variant of a 3-D sweep,
    which falls back to the plain sweep where it does not apply."""
    if tma:
        g = _Gen(kd, ndims, zloop, split, ordered, tma=True)
        if g.tma:
            try:
                src = g.source(dtype)
                return src, g.uses_collectives, g.layout
            except _NoTma:
                pass
    g = _Gen(kd, ndims, zloop, split, ordered)
    src = g.source(dtype)
    return src, g.uses_collectives, None


# ---- kernels -----------------------------------------------------------------------------------
def array_ndims(descs):
    """Rank of a kernel's arrays (the largest; 2-D arrays have n[2] = 1, 1-D arrays n[1] = n[2] = 1)."""
    return max((3 if d.n[2] > 1 else 2 if d.n[1] > 1 else 1) for d in descs) if descs else 1


class JitKernel:
    """A run-time compiled kernel; call it like `@parallel`: ``ps.parallel(k, *args)`` or ``k(*args)``.
    ndims selects the FiniteDifferences{1,2,3}D macros (the reference's `@init_parallel_stencil`
    ndims); None takes the rank of the array arguments."""

    def __init__(self, src: str, ndims=None):
        self.ndims = ndims
        # 3-D sweeps of FP32 arrays stage their stencil arrays by TMA where the launch allows it
        # ("always": FP64 too -- slower there: the FP64 kernels are bound by arithmetic, not loads)
        self.tma = True
        self.tma_launches = 0  # launches that took the TMA variant
        self.kd = parse(src)
        self._kernel_language = uses_kernel_language(self.kd)
        self.name, self.nargs = self.kd.name, len(self.kd.args)
        self._handles = {}
        self._collective = {}
        self._layouts = {}  # TMA stage layout of each TMA-variant handle (None: the plain sweep was generated)

    def source(self, ndims, dtype="double"):
        return generate(self.kd, ndims, dtype)

    def _handle(self, ndims, dtype, zloop=False, split=False, ordered=False, tma=False):
        key = (ndims, dtype, bool(zloop), bool(split)) + (("ordered",) if ordered else ()) + (("tma",) if tma else ())
        if key not in self._handles:
            src, self._collective[key], self._layouts[key] = _generate_info(self.kd, ndims, dtype, zloop, split,
                                                                            ordered, tma)
            h = ctypes.c_void_p()
            _lib.call("ps_jit_compile", src.encode(), b"ps_jit_entry", ctypes.byref(h))
            self._handles[key] = h
        return self._handles[key]

    def __call__(self, *args, ranges=None, stream=None, sync=True, nblocks=None, nthreads=None, shmem=None,
                 memopt=None, loopsize=0, fp64="ieee"):
        self.jit_launch(args, ranges, stream, sync, nblocks=nblocks, nthreads=nthreads, shmem=shmem, memopt=memopt,
                        loopsize=loopsize, fp64=fp64)

    def jit_launch(self, args, ranges=None, stream=None, sync=True, nblocks=None, nthreads=None, shmem=None,
                   memopt=None, loopsize=0, fp64="ieee"):
        """Launch over `ranges` (default: the largest array extents; with `nblocks`, nblocks .* nthreads
        threads) in blocks of `nthreads` (default (32, 8, 1)) with `shmem` bytes of dynamic shared
        memory (src/ParallelKernel/parallel.jl:303-328). memopt (default: the definition's
        `memopt=`, else true) runs 2-D and 3-D `@parallel` kernels as sweeps along the last
        dimension (src/memopt.jl, loopdim 2 and 3) of `loopsize` indices per thread -- by default
        64, as src/parallel.jl:532-543 for compute capability >= 9, halved (down to 2) while the
        launch would have fewer threads than the GPU holds at once -- with the same results.
        fp64="split" evaluates the arithmetic of FP64 kernels on FP32 pairs (each operation within
        ~2^-46 of its operands' magnitude; GB300 issues FP32 at 64x the FP64 rate)."""
        h, A, nA, S, nS, lo, cnt, threads, shmem, loop, layout = self._config(args, ranges, nblocks, nthreads, shmem,
                                                                             memopt, loopsize, fp64, allow_tma=True)
        if layout is not None:  # the 3-D sweep with its stencil arrays staged by TMA
            maps = [x for a in layout["arrays"] for x in (a["k"], a["bx"], a["by"])]
            cnt_t = [-(-cnt[0] // layout["xc"]), cnt[1], cnt[2]]  # threads in x: each covers xc columns
            _lib.call("ps_jit_launch_tma", h, A, nA, S, nS, (ctypes.c_int64 * 3)(*cnt_t),
                      (ctypes.c_int32 * 3)(32, _Gen.TMA_TY, 1), int(layout["smem"]), int(loop[2]),
                      (ctypes.c_int32 * len(maps))(*maps), len(layout["arrays"]), stream_handle(stream),
                      int(bool(sync)))
            self.tma_launches += 1
            return
        _lib.call("ps_jit_launch_ex", h, A, nA, S, nS, (ctypes.c_int64 * 3)(*lo), (ctypes.c_int64 * 3)(*cnt),
                  (ctypes.c_int32 * 3)(*threads), int(shmem or 0), (ctypes.c_int32 * 3)(*loop), stream_handle(stream),
                  int(bool(sync)))

    def hide_eligible(self):
        """A `@parallel` kernel without kernel-language calls (block / thread indices, shared memory,
        barriers, shuffles, votes): its blocks can run in any order, so ps_jit_hide_communication
        may launch the boundary tiles first."""
        return self.kd.kind == "parallel" and not self._kernel_language

    def hide_communication(self, args, bw, comm_fn, stream=None, memopt=None, loopsize=0, fp64="ieee"):
        """One boundary-first launch over the kernel's full grid (ps_jit_hide_communication); comm_fn
        (a ps_comm_fn) runs once the boundary tiles are done."""
        h, A, nA, S, nS, lo, cnt, threads, shmem, loop, _ = self._config(args, None, None, None, None, memopt,
                                                                        loopsize, fp64, ordered=True)
        _lib.call("ps_jit_hide_communication", h, A, nA, S, nS, (ctypes.c_int64 * 3)(*cnt),
                  (ctypes.c_int32 * 3)(*threads), (ctypes.c_int32 * 3)(*loop), (ctypes.c_int64 * 3)(*bw), comm_fn,
                  None, stream_handle(stream))

    def _config(self, args, ranges, nblocks, nthreads, shmem, memopt, loopsize, fp64, ordered=False, allow_tma=False):
        """Handle, argument arrays, launch geometry and TMA stage layout (None: no staging) of one
        launch (see jit_launch); allow_tma picks the TMA variant of a 3-D sweep where it applies."""
        require_initialized()
        if len(args) != self.nargs:
            raise ArgumentError(f"{self.name} takes {self.nargs} arguments (obtained {len(args)})")
        arrs, scal = [], []
        for (kind, name), a in zip(self.kd.args, args):
            if kind == "scalar" and not isinstance(a, numbers.Real):
                raise ArgumentError(f"{self.name}: argument {name} is a scalar (obtained {type(a).__name__})")
            (arrs if kind == "array" else scal).append(a)
        descs = [descriptor(a) for a in arrs]
        dt = {0: "double", 1: "float"}.get(descs[0].dtype) if descs else "double"
        if dt is None or any(d.dtype != descs[0].dtype for d in descs):
            raise ArgumentError("the array arguments must share one FP64 or FP32 type")
        ndims = self.ndims or array_ndims(descs)
        lo, cnt = [0, 0, 0], self._extent(descs, ndims)
        threads = [1, 1, 1]
        if nthreads is not None:
            nthreads = tuple(int(x) for x in (nthreads if isinstance(nthreads, (tuple, list)) else (nthreads,)))
            if not 1 <= len(nthreads) <= 3:
                raise ArgumentError("nthreads: 1 to 3 dimensions")
            threads[:len(nthreads)] = nthreads
        else:
            threads = [32, 8, 1]
        if nblocks is not None:
            if nthreads is None:
                raise ArgumentError("nblocks needs nthreads")
            nb = tuple(int(x) for x in (nblocks if isinstance(nblocks, (tuple, list)) else (nblocks,)))
            nb = nb + (1,) * (3 - len(nb))
            if ranges is None:
                lo, cnt = [0, 0, 0], [nb[d] * threads[d] for d in range(3)]
        if ranges is not None:  # Julia ranges: 1-based (start, stop) pairs, or python ranges over 0-based indices
            lo, hi = ranges_to_box(ranges)
            if min(lo) < 0:
                raise ArgumentError("ranges must start at index 1 or above")
            cnt = [max(0, hi[d] - lo[d]) for d in range(3)]
        # the sweep is the default schedule of 2-D and 3-D @parallel kernels (bit-identical results,
        # faster: a one-point-per-thread kernel keeps too few loads in flight); memopt=false keeps one
        # point per thread, as the definition or the call may ask
        want = memopt if memopt is not None else self.kd.options.get("memopt", "true") == "true"
        zl = bool(want) and self.kd.kind == "parallel" and ndims in (2, 3) and not self._kernel_language
        loop = [1, 1, 1]
        if zl:
            sd = ndims - 1
            if nthreads is None and ndims == 2:
                threads = [128, 1, 1]
            threads[sd] = 1
            ls = int(loopsize or int(self.kd.options.get("loopsize", "0") or 0))
            if ls < 0:
                raise ArgumentError("loopsize must be positive")
            if not ls:
                ls = 64  # the reference's default for compute capability >= 9
                cols = cnt[0] * cnt[1] * cnt[2] // max(1, cnt[sd])
                while ls > 2 and cols * -(-cnt[sd] // ls) < RESIDENT_THREADS:
                    ls //= 2
            loop[sd] = ls
        if fp64 not in ("ieee", "split", "split_state", "split_grid"):
            raise ArgumentError("fp64 must be 'ieee' or 'split'")
        sp = fp64 != "ieee" and dt == "double"
        A = (PSArray * max(1, len(descs)))(*descs)
        S = (ctypes.c_double * max(1, len(scal)))(*[float(x) for x in scal])
        if allow_tma and self.tma and (dt == "float" or self.tma == "always") and zl and ndims == 3 and \
                not ordered and ranges is None and nblocks is None and nthreads is None and not shmem:
            # the 3-D sweep with its stencil arrays staged by TMA, where every staged array meets TMA's
            # 16-byte rules (base address, x extent and x-y plane in bytes); else the plain sweep
            es = 8 if dt == "double" else 4
            ht = self._handle(ndims, dt, zl, sp, False, tma=True)
            layout = self._layouts[(ndims, dt, zl, sp, "tma")]
            if layout is not None and all(not ((d.ptr or 0) % 16 or (d.n[0] * es) % 16 or (d.n[0] * d.n[1] * es) % 16)
                                          for d in (descs[a["k"]] for a in layout["arrays"])):
                return ht, A, len(descs), S, len(scal), lo, cnt, threads, shmem, loop, layout
        h = self._handle(ndims, dt, zl, sp, ordered)
        if self._collective[(ndims, dt, zl, sp) + (("ordered",) if ordered else ())] and \
                any(cnt[d] % threads[d] for d in range(3)):
            raise ArgumentError("a kernel with @sync_threads, shuffles or votes needs ranges that are a multiple of "
                                f"the thread block (ranges {cnt}, nthreads {threads})")
        return h, A, len(descs), S, len(scal), lo, cnt, threads, shmem, loop, None

    @staticmethod
    def _extent(descs, ndims):
        """The `@parallel` grid: the largest extent of the array arguments per dimension
        (src/ParallelKernel/parallel.jl:785-798), 1 beyond ndims."""
        return [max(int(x.n[d]) for x in descs) if descs and d < ndims else 1 for d in range(3)]

    def grid_extent(self, args):
        descs = [descriptor(a) for (kind, _), a in zip(self.kd.args, args) if kind == "array"]
        return self._extent(descs, self.ndims or array_ndims(descs))

    def check(self, stream=None):
        """Wait for `stream` and raise what earlier asynchronous launches of this kernel flagged."""
        for h in self._handles.values():
            _lib.call("ps_jit_check", h, stream_handle(stream))

    def __del__(self):
        try:
            for h in self._handles.values():
                _lib.load().ps_jit_destroy(h)
        except Exception:
            pass


_CACHE = {}


def parallel_kernel(src: str, ndims=None) -> JitKernel:
    """The `@parallel` / `@parallel_indices` function `src` as a run-time compiled kernel (cached)."""
    if (src, ndims) not in _CACHE:
        _CACHE[(src, ndims)] = JitKernel(src, ndims)
    return _CACHE[(src, ndims)]
