"""Test oracle for the run-time compiled kernels (test infrastructure; only the tests use it, as the
checker): a CPU interpreter of `@parallel` / `@parallel_indices` kernel definitions.

It is written independently of the product's translator (ps_gb300/jit.py): its own tokenizer and
precedence parser for the Julia subset, FiniteDifferences macros decoded from their names, and a
plain per-thread evaluation loop. It follows
- src/FiniteDifferences.jl: index patterns and operation orders of the macros (left-to-right sums,
  `*0.5` / `*0.25` / `*0.125` averages, `1.0/(sum of 1.0/A)*k` harmonic averages, nested
  `max`/`min` for @maxloc/@minloc) and the `@within` masks of left-hand selections;
- src/parallel.jl:789-859: a left-hand array that is not an argument is computed on the fly, its
  expression evaluated at the index where it is read (only `@all` is allowed for it);
- src/ParallelKernel/parallel.jl:584-598: literals take the kernel's number type;
- Julia's arithmetic: `x^2` and `x^3` as products (Base.literal_pow), `Bool * x` as
  `ifelse(b, x, copysign(0, x))`, NaN-propagating `max`/`min` with max(-0.0, 0.0) == 0.0, 1-based
  indices with bounds checks (an index outside the array raises IndexError, Julia's BoundsError).

Arithmetic is IEEE double through Python floats, or IEEE single through numpy.float32 scalars, one
operation at a time with no contraction, so FP64/FP32 results of +, -, *, / and comparisons are the
exact values a conforming machine produces. Math functions (exp, sqrt of a non-square, pow with a
non-literal exponent) come from the host's libm and may differ from the device's in the last bits.

Arrays are numpy arrays indexed A[ix-1, iy-1, iz-1] (x first, as Julia's column-major arrays).
"""
from __future__ import annotations

import math
import re
import threading

import numpy as np

__all__ = ["parse", "run", "OracleKernel", "Dual", "jacobian", "reverse_shadows", "forward_shadows"]

# ---------------------------------------------------------------- tokens
_TOKEN = re.compile(r"""
    (?P<nl>\n) | (?P<ws>[ \t\r]+) | (?P<com>\#[^\n]*) |
    (?P<hex>0x[0-9a-fA-F]+) |
    (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?(?:f0)?) |
    (?P<mac>@[A-Za-z_][A-Za-z0-9_]*) |
    (?P<uop>÷|∈) |
    (?P<id>(?:[A-Za-z_]|[^\x00-\x7f])(?:[A-Za-z0-9_!]|[^\x00-\x7f])*) |
    (?P<op>==|!=|<=|>=|&&|\|\||::|\+=|-=|\*=|/=|[-+*/^<>=!(),;\[\]?:.{}$%])
""", re.X)


def _tokens(text):
    text = text.replace("≤", "<=").replace("≥", ">=").replace("≠", "!=")
    # module-qualified macros (FiniteDifferences2D.@inn) are the macros themselves
    text = re.sub(r"\b(?:ParallelStencil\.)?(?:FiniteDifferences[123]D\.)?(?=@)", "", text)
    out, depth = [], 0
    for m in _TOKEN.finditer(text):
        kind, val = m.lastgroup, m.group()
        if kind in ("ws", "com") or val == "$":
            continue
        if kind == "hex":
            kind, val = "num", str(int(val, 16))
        if kind == "uop":
            kind = "op"
        if kind == "id" and val.endswith("!") and m.end() < len(text) and text[m.end()] == "=":
            # `a!=b`: the identifier does not own the `!`
            val = val[:-1]
            out.append(("id", val))
            out.append(("op", "!"))
            continue
        if kind == "op" and val in "([{":
            depth += 1
        elif kind == "op" and val in ")]}":
            depth -= 1
        if kind == "nl":
            if depth > 0:
                continue
            if out and out[-1] == ("nl", "\n"):
                continue
        if kind == "op" and val == ";" and depth == 0:
            kind, val = "nl", "\n"
        out.append((kind, val))
    out.append(("eof", ""))
    return out


class _P:
    """Recursive-descent parser of statements and expressions (Julia precedence)."""

    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def expect(self, val):
        tok = self.next()
        if tok[1] != val:
            raise SyntaxError(f"expected {val!r}, got {tok[1]!r}")
        return tok

    def skip_nl(self):
        while self.peek()[0] == "nl":
            self.i += 1

    # statements
    def block(self, stops):
        out = []
        while True:
            self.skip_nl()
            tok = self.peek()
            if tok[0] == "eof" or (tok[0] == "id" and tok[1] in stops):
                return out
            s = self.statement()
            if s is not None:
                out.append(s)

    def statement(self):
        tok = self.peek()
        if tok == ("id", "return"):
            self.next()
            if self.peek()[0] not in ("nl", "eof") and self.peek()[1] not in ("end", "else", "elseif"):
                self.expr()
            return ("return",)
        if tok == ("id", "if"):
            return self.if_stmt()
        if tok == ("id", "for"):
            self.next()
            var = self.next()[1]
            if self.next()[1] not in ("=", "in", "∈"):
                raise SyntaxError("for v = a:b")
            parts = [self.expr()]
            while self.peek()[1] == ":":
                self.next()
                parts.append(self.expr())
            body = self.block(("end",))
            self.expect("end")
            return ("for", var, parts, body)
        if tok == ("id", "while"):
            self.next()
            cond = self.expr()
            body = self.block(("end",))
            self.expect("end")
            return ("while", cond, body)
        lhs = self.expr()
        if self.peek()[1] in ("+=", "-=", "*=", "/="):  # a op= b is a = a op b
            op = self.next()[1][0]
            self.skip_nl()
            return ("assign", lhs, ("bin", op, lhs, self.expr()))
        if self.peek()[1] != "=" and lhs[0] == "mcall":
            return ("do", lhs)  # @sync_threads()
        if self.peek()[1] != "=":
            raise SyntaxError("kernel statements are assignments, if-blocks, loops or @sync_threads()")
        self.next()
        self.skip_nl()
        return ("assign", lhs, self.expr())

    def if_stmt(self):
        self.next()  # if / elseif
        cond = self.expr()
        body = self.block(("elseif", "else", "end"))
        tok = self.next()
        if tok[1] == "end":
            return ("if", cond, body, [])
        if tok[1] == "else":
            other = self.block(("end",))
            self.expect("end")
            return ("if", cond, body, other)
        self.i -= 1  # elseif: parse as a nested if owning the final `end`
        return ("if", cond, body, [self.if_stmt()])

    # expressions, lowest precedence first
    def expr(self):
        c = self.or_()
        if self.peek()[1] == "?":
            self.next()
            a = self.expr()
            self.expect(":")
            return ("ifelse", c, a, self.expr())
        return c

    def or_(self):
        a = self.and_()
        while self.peek()[1] == "||":
            self.next()
            self.skip_nl()
            a = ("or", a, self.and_())
        return a

    def and_(self):
        a = self.cmp()
        while self.peek()[1] == "&&":
            self.next()
            self.skip_nl()
            a = ("and", a, self.cmp())
        return a

    def cmp(self):
        first = self.arith()
        ops, rest = [], []
        while self.peek()[1] in ("<", "<=", ">", ">=", "==", "!="):
            ops.append(self.next()[1])
            self.skip_nl()
            rest.append(self.arith())
        return ("cmp", ops, [first] + rest) if ops else first

    def arith(self):
        a = self.term()
        while self.peek()[1] in ("+", "-"):
            op = self.next()[1]
            self.skip_nl()
            a = ("bin", op, a, self.term())
        return a

    def term(self):
        a = self.unary()
        while self.peek()[1] in ("*", "/", "÷", "%"):
            op = self.next()[1]
            self.skip_nl()
            a = ("bin", op, a, self.unary())
        return a

    def unary(self):
        if self.peek()[1] in ("-", "+", "!"):
            op = self.next()[1]
            x = self.unary()
            return ("not", x) if op == "!" else (("neg", x) if op == "-" else x)
        return self.power()

    def power(self):
        base = self.postfix()
        if self.peek()[1] == "^":
            self.next()
            return ("pow", base, self.unary())  # right-associative, binds tighter than unary minus on its left
        return base

    def postfix(self):
        tok = self.next()
        if tok[0] == "num":
            v = tok[1]
            if v.endswith("f0") or "." in v or "e" in v.lower():
                return ("num", float(v.replace("f0", "")), True)
            return ("num", int(v), False)
        if tok[0] == "mac":
            self.expect("(")
            args = []
            while self.peek()[1] != ")":
                args.append(self.expr())
                if self.peek()[1] == ",":
                    self.next()
            self.expect(")")
            if len(args) == 1 and args[0][0] == "name" and tok[1][1:] not in _KL:
                return ("macro", tok[1][1:], args[0][1])  # FiniteDifferences macro on an array
            node = ("mcall", tok[1][1:], args)
            if self.peek()[1] == ".":  # @threadIdx().x
                self.next()
                node = ("attr", node, self.next()[1])
            return node
        if tok[1] == "(":
            e = self.expr()
            if self.peek()[1] == ",":  # a tuple (dims of @sharedMem)
                items = [e]
                while self.peek()[1] == ",":
                    self.next()
                    if self.peek()[1] == ")":
                        break
                    items.append(self.expr())
                self.expect(")")
                return ("tuple", items)
            self.expect(")")
            return e
        if tok[0] == "id":
            if self.peek()[1] == "(":
                self.next()
                args = []
                while self.peek()[1] != ")":
                    args.append(self.expr())
                    if self.peek()[1] == ",":
                        self.next()
                self.expect(")")
                return ("call", tok[1], args)
            if self.peek()[1] == "[":
                self.next()
                idx = []
                while self.peek()[1] != "]":
                    idx.append(self.expr())
                    if self.peek()[1] == ",":
                        self.next()
                self.expect("]")
                return ("index", tok[1], idx)
            if tok[1] in ("true", "false"):
                return ("bool", tok[1] == "true")
            return ("name", tok[1])
        raise SyntaxError(f"unexpected token {tok[1]!r}")


# kernel-language macros (src/ParallelKernel/kernel_language.jl)
_KL = {"threadIdx", "blockIdx", "blockDim", "gridDim", "sync_threads", "sharedMem", "warpsize", "laneid",
       "active_mask", "shfl_sync", "shfl_up_sync", "shfl_down_sync", "shfl_xor_sync", "vote_any_sync",
       "vote_all_sync", "vote_ballot_sync"}
_COLL = {"sync_threads", "shfl_sync", "shfl_up_sync", "shfl_down_sync", "shfl_xor_sync", "vote_any_sync",
         "vote_all_sync", "vote_ballot_sync"}


class OracleKernel:
    def __init__(self, name, kind, indices, argnames, body, ndims_opt):
        self.name, self.kind, self.indices = name, kind, indices
        self.argnames, self.body, self.ndims_opt = argnames, body, ndims_opt


def parse(src: str) -> OracleKernel:
    """Read a `@parallel` / `@parallel_indices` function definition."""
    m = re.search(r"@parallel(_indices)?\b(.*?)\bfunction\s+([^\s(]+)\s*\(", src, re.S)
    if not m:
        raise SyntaxError("not a kernel definition")
    kind = "parallel_indices" if m.group(1) else "parallel"
    head, indices = m.group(2).strip(), []
    if kind == "parallel_indices":
        mi = re.match(r"\(([^)]*)\)|(\S+)", head)
        indices = [s.strip() for s in (mi.group(1) if mi.group(1) is not None else mi.group(2)).split(",") if s.strip()]
        head = head[mi.end():]
    # key=value options; values may hold blanks inside parentheses (optvars=(A, B))
    opts = dict(o.split("=", 1) for o in re.findall(r"\w+=(?:\((?:[^()]|\([^()]*\))*\)|\S+)", head))
    depth, j = 0, m.end() - 1
    for j in range(m.end() - 1, len(src)):
        depth += src[j] == "("
        depth -= src[j] == ")"
        if depth == 0:
            break
    # arguments: commas outside brackets separate them (A::Data.Array{T,N} is one)
    argnames = [a.split("::")[0].strip() for a in re.split(r",(?![^{(\[]*[})\]])", src[m.end():j]) if a.strip()]
    rest = src[j + 1:].strip()
    rest = re.sub(r"^where\s*(\{[^}]*\}|[^\n]*)", "", rest).strip()
    assert rest.endswith("end")
    body_text = rest[:-3]
    if len(indices) == 1 and re.fullmatch(r"\w+\.\.\.", indices[0]):
        # (I...): the index tuple; A[I...] indexes A at the thread's own point
        indices = ["..."]
        body_text = re.sub(r"\b\w+\.\.\.", " __splat__ ", body_text)
    # one-line local functions `f(a, b) = [return] expr`: inlined at their calls
    fns = {}
    for fm in re.finditer(r"^[ \t]*(\w+)[ \t]*\(([\w \t,]*)\)[ \t]*=(?!=)[ \t]*(?:return[ \t]+)?(.+)$", body_text, re.M):
        fns[fm.group(1)] = ([a.strip() for a in fm.group(2).split(",") if a.strip()], _P(_tokens(fm.group(3))).expr())
    body_text = re.sub(r"^[ \t]*\w+[ \t]*\([\w \t,]*\)[ \t]*=(?!=)[^\n]*$", "", body_text, flags=re.M)
    p = _P(_tokens(body_text))
    body = _inline(p.block(()), fns) if fns else p.block(())
    nd = opts.get("ndims", "").strip("()")
    return OracleKernel(m.group(3), kind, indices, argnames, body, int(nd) if nd.isdigit() else None)


def _inline(node, fns):
    """Replace calls of local functions by their expression with the parameters bound."""
    if isinstance(node, list):
        return [_inline(x, fns) for x in node]
    if not isinstance(node, tuple):
        return node
    node = tuple(_inline(x, fns) for x in node)
    if len(node) == 3 and node[0] == "call" and node[1] in fns:
        params, expr = fns[node[1]]
        bind = dict(zip(params, node[2]))

        def sub(x):
            if isinstance(x, list):
                return [sub(y) for y in x]
            if not isinstance(x, tuple):
                return x
            if x[0] == "name" and x[1] in bind:
                return bind[x[1]]
            if x[0] == "index" and x[1] in bind and bind[x[1]][0] == "name":
                return ("index", bind[x[1]][1], sub(x[2]))
            return tuple(sub(y) for y in x)
        return _inline(sub(expr), fns)
    return node


# ---------------------------------------------------------------- FiniteDifferences macros by name
_AX = "xyz"


def _decode(name, nd):
    """Macro name -> (kind, operated dims, dims selected inner). kind: sel | d | d2 | av | harm | maxloc | minloc."""
    if name in ("maxloc", "minloc"):
        return name, [], list(range(nd))
    if name == "all":
        return "sel", [], []
    if name == "inn":
        return "sel", [], list(range(nd))
    if name.startswith("inn_"):
        return "sel", [], [_AX.index(c) for c in name[4:]]
    m = re.fullmatch(r"(d2|d|av|harm)(?:_([xyz]+)([ai]))?", name)
    if not m:
        raise KeyError(name)
    kind, dims, mode = m.group(1), m.group(2), m.group(3)
    if dims is None:  # 1-D @d/@d2 along x; @av/@harm (any nd) over all dimensions
        ops = [0] if kind in ("d", "d2") else list(range(nd))
        inner = []
    else:
        ops = [_AX.index(c) for c in dims]
        inner = [d for d in range(nd) if d not in ops] if mode == "i" else []
    if any(d >= nd for d in ops):
        raise KeyError(name)
    if kind in ("d", "d2") and len(ops) != 1:
        raise KeyError(name)
    return kind, ops, inner


# ---------------------------------------------------------------- evaluation
def _jl_max(x, y):
    if x != x or y != y:
        return x + y  # NaN
    if x == y:
        return y if math.copysign(1.0, float(x)) < 0 else x  # max(-0.0, 0.0) == 0.0
    return x if x > y else y


def _jl_min(x, y):
    if x != x or y != y:
        return x + y
    if x == y:
        return x if math.copysign(1.0, float(x)) < 0 else y
    return x if x < y else y


_FUN = {"exp": (math.exp, np.exp), "log": (math.log, np.log), "sqrt": (math.sqrt, np.sqrt),
        "sin": (math.sin, np.sin), "cos": (math.cos, np.cos), "tan": (math.tan, np.tan),
        "tanh": (math.tanh, np.tanh), "sinh": (math.sinh, np.sinh), "cosh": (math.cosh, np.cosh),
        "atan": (math.atan, np.arctan), "asin": (math.asin, np.arcsin), "acos": (math.acos, np.arccos),
        "log10": (math.log10, np.log10), "exp2": (lambda v: 2.0 ** v, np.exp2), "cbrt": (np.cbrt, np.cbrt)}


class _Return(Exception):
    """`return` inside a kernel: the thread is done."""


class _Block:
    """One thread block: indices, dynamic shared memory (zero-filled bytes) and, for kernels with
    barriers, shuffles or votes, the synchronisation of its threads (each thread a Python thread)."""

    def __init__(self, bidx, bdim, gdim, shmem, threaded):
        self.bidx, self.bdim, self.gdim = bidx, bdim, gdim
        self.buf = bytearray(int(shmem))
        self.views = {}
        nthr = bdim[0] * bdim[1] * bdim[2]
        self.bar = threading.Barrier(nthr, timeout=60) if threaded else None
        nw = (nthr + 31) // 32
        self.warp_bars = [threading.Barrier(min(32, nthr - 32 * w), timeout=60) for w in range(nw)] if threaded else []
        self.slots = [[None] * 32 for _ in range(nw)]

    def shared(self, R, dims, offset):
        key = (tuple(dims), offset)
        if key not in self.views:
            dt = np.dtype(np.float32 if R is np.float32 else np.float64)
            need = offset + int(np.prod(dims)) * dt.itemsize
            if offset < 0 or need > len(self.buf):
                raise IndexError(f"BoundsError: @sharedMem{tuple(dims)} at offset {offset} exceeds shmem "
                                 f"{len(self.buf)}")
            self.views[key] = np.ndarray(tuple(dims), dtype=dt, buffer=self.buf, offset=offset, order="F")
        return self.views[key]

    def exchange(self, warp, lane, val):
        """Every lane of the warp deposits its value; all lanes see all values."""
        self.slots[warp][lane] = val
        self.warp_bars[warp].wait()
        snap = list(self.slots[warp])
        self.warp_bars[warp].wait()
        return snap


class _Thread:
    def __init__(self, k, arrays, scalars, temps, R, nd, blk=None, tid=(0, 0, 0)):
        self.k, self.A, self.S, self.temps, self.R, self.nd = k, arrays, scalars, temps, R, nd
        self.blk, self.tid, self.loc = blk, tid, {}
        if blk is not None:
            lin = tid[0] + blk.bdim[0] * (tid[1] + blk.bdim[1] * tid[2])
            self.warp, self.lane = divmod(lin, 32)

    def real(self, v):
        return self.R(v) if isinstance(v, (int, bool, float)) and not isinstance(v, self.R) else v

    def array(self, name):
        if name in self.loc and isinstance(self.loc[name], np.ndarray):
            return self.loc[name]
        return self.A[name]

    def load(self, name, idx, depth=0):
        """Array `name` at 1-based index tuple idx."""
        if name in self.temps:  # on-the-fly: its expression at this index
            return self.ev(self.temps[name], tuple(idx) + (1,) * (3 - len(idx)), depth + 1)
        a = self.array(name)
        idx = list(idx) + [1] * (a.ndim - len(idx))
        if len(idx) > a.ndim and any(i != 1 for i in idx[a.ndim:]):
            raise IndexError(f"BoundsError: {name}{tuple(idx)}")
        for d in range(a.ndim):
            if not 1 <= idx[d] <= a.shape[d]:
                raise IndexError(f"BoundsError: {name}{tuple(idx)} outside {a.shape}")
        return a[tuple(i - 1 for i in idx[:a.ndim])]

    def macro(self, mname, name, I, depth):
        kind, ops, inner = _decode(mname, self.nd)
        base = [I[d] + (1 if d in inner else 0) for d in range(self.nd)]

        def at(shift):
            return self.load(name, [base[d] + shift.get(d, 0) for d in range(self.nd)], depth)

        if kind == "sel":
            return at({})
        if kind == "d":
            return at({ops[0]: 1}) - at({})
        if kind == "d2":
            d = ops[0]
            c = [I[e] + (1 if (e in inner or e == d) else 0) for e in range(self.nd)]
            g = lambda s: self.load(name, [c[e] + (s if e == d else 0) for e in range(self.nd)], depth)  # noqa: E731
            return (g(1) - g(0)) - (g(0) - g(-1))
        if kind in ("av", "harm"):
            terms = []
            for corner in range(1 << len(ops)):  # first operated dimension varies fastest
                v = at({d: (corner >> j) & 1 for j, d in enumerate(ops)})
                terms.append(self.R(1.0) / v if kind == "harm" else v)
            s = terms[0]
            for t in terms[1:]:
                s = s + t
            w = self.R(float(1 << len(ops)))
            return s * (self.R(1.0) / w) if kind == "av" else (self.R(1.0) / s) * w
        if kind in ("maxloc", "minloc"):
            f = _jl_max if kind == "maxloc" else _jl_min
            m = f(f(at({0: -1}), at({0: 1})), at({}))
            for d in range(1, self.nd):
                m = f(m, f(at({d: -1}), at({d: 1})))
            return m
        raise KeyError(mname)

    def kernel_language(self, name, args, I, depth):
        """src/ParallelKernel/kernel_language.jl: 1-based thread/block indices, warps of 32 lanes."""
        E = lambda x: self.ev(x, I, depth)  # noqa: E731
        b = self.blk
        if name == "sharedMem":
            dims = E(args[1])
            dims = list(dims) if isinstance(dims, list) else [dims]
            off = int(E(args[2])) if len(args) > 2 else 0
            return b.shared(self.R, [int(x) for x in dims], off)
        if name == "warpsize":
            return 32
        if name == "laneid":
            return self.lane + 1
        if name == "active_mask":
            return 0xFFFFFFFF
        if name.startswith("vote"):
            pred = bool(E(args[1]))
            snap = b.exchange(self.warp, self.lane, pred)
            mask = int(E(args[0]))
            lanes = [i for i in range(32) if (mask >> i) & 1 and snap[i] is not None]
            if name == "vote_any_sync":
                return any(snap[i] for i in lanes)
            if name == "vote_all_sync":
                return all(snap[i] for i in lanes)
            return sum(1 << i for i in lanes if snap[i])
        if name.startswith("shfl"):
            val = E(args[1])
            x = int(E(args[2]))
            w = int(E(args[3])) if len(args) > 3 else 32
            snap = b.exchange(self.warp, self.lane, val)
            lane, base = self.lane, self.lane - self.lane % w
            if name == "shfl_sync":
                src = base + (x - 1) % w
            elif name == "shfl_up_sync":
                src = lane - x if lane % w >= x else lane
            elif name == "shfl_down_sync":
                src = lane + x if lane % w + x < w else lane
            else:  # xor: a partner outside the lane's partition returns the lane's own value
                src = lane ^ x
                src = src if src // w == lane // w else lane
            v = snap[src] if src < 32 and snap[src] is not None else val
            return v
        raise NameError(name)

    def ev(self, e, I, depth=0):
        if depth > 64:
            raise RecursionError("on-the-fly arrays nested too deeply")
        R, op = self.R, e[0]
        E = lambda x: self.ev(x, I, depth)  # noqa: E731
        if op == "num":
            return R(e[1]) if e[2] else e[1]
        if op == "bool":
            return e[1]
        if op == "tuple":
            return [E(x) for x in e[1]]
        if op == "name":
            n = e[1]
            if n in self.loc:
                return self.loc[n]
            if n in self.S:
                return self.S[n]
            if self.k.kind == "parallel_indices" and n in self.k.indices:
                return I[self.k.indices.index(n)]
            if self.k.kind == "parallel" and n in ("ix", "iy", "iz")[:self.nd]:
                return I["xyz".index(n[1])]
            raise NameError(n)
        if op == "neg":
            return -E(e[1])
        if op == "not":
            return not E(e[1])
        if op == "bin":
            a, b = E(e[2]), E(e[3])
            sym = e[1]
            if sym == "*" and (isinstance(a, bool) or isinstance(b, bool)):
                flag, x = (a, b) if isinstance(a, bool) else (b, a)
                if isinstance(x, int) and not isinstance(x, bool):
                    return x if flag else 0
                x = self.real(x)
                return x if flag else R(math.copysign(0.0, float(x)))
            if isinstance(a, int) and isinstance(b, int) and sym != "/":
                if sym in ("÷", "%"):  # truncating, like Julia's div and rem
                    q = abs(a) // abs(b) * (1 if (a >= 0) == (b >= 0) else -1)
                    return q if sym == "÷" else a - b * q
                return a + b if sym == "+" else a - b if sym == "-" else a * b
            a, b = self.real(a), self.real(b)
            if sym == "%":
                return R(math.fmod(float(a), float(b)))
            if sym == "÷":
                return R(math.trunc(a / b))
            return a + b if sym == "+" else a - b if sym == "-" else a * b if sym == "*" else a / b
        if op == "pow":
            x, n = E(e[1]), e[2]
            if n[0] == "num" and not n[2] and n[1] in (2, 3):
                x = self.real(x) if not isinstance(x, int) else x
                return x * x if n[1] == 2 else (x * x) * x
            x, p = self.real(x), self.real(E(n))
            if isinstance(x, Dual) or isinstance(p, Dual):
                return Dual.lift(x) ** p
            return R(float(x) ** float(p))
        if op == "cmp":
            vals = [E(v) for v in e[2]]
            for (sym, a, b) in zip(e[1], vals, vals[1:]):
                ok = {"<": a < b, "<=": a <= b, ">": a > b, ">=": a >= b, "==": a == b, "!=": a != b}[sym]
                if not ok:
                    return False
            return True
        if op == "and":
            return bool(E(e[1])) and bool(E(e[2]))
        if op == "or":
            return bool(E(e[1])) or bool(E(e[2]))
        if op == "ifelse":
            return E(e[2]) if E(e[1]) else E(e[3])
        if op == "macro":
            return self.macro(e[1], e[2], I, depth)
        if op == "mcall":
            return self.kernel_language(e[1], e[2], I, depth)
        if op == "attr":
            name, field = e[1][1], e[2]
            d = "xyz".index(field)
            b = self.blk
            return {"threadIdx": self.tid[d] + 1, "blockIdx": b.bidx[d] + 1, "blockDim": b.bdim[d],
                    "gridDim": b.gdim[d]}[name]
        if op == "index":
            shape = self.array(e[1]).shape + (1, 1)
            if len(e[2]) == 1 and e[2][0] == ("name", "__splat__"):
                return self.load(e[1], list(I[:self.array(e[1]).ndim]), depth)
            idx = [int(self.ev(_subst_end(x, shape[d]), I, depth)) for d, x in enumerate(e[2])]
            return self.load(e[1], idx, depth)
        if op == "call":
            f, args = e[1], e[2]
            if f == "size":
                a = self.array(args[0][1])
                d = E(args[1])
                return a.shape[d - 1] if d <= a.ndim else 1
            if f == "eltype":
                return R
            if f == "sizeof":  # sizeof(eltype(A))
                return 8 if R is float else 4
            if f in ("max", "min"):
                vals = [E(x) for x in args]
                if all(isinstance(v, int) and not isinstance(v, bool) for v in vals):
                    return max(vals) if f == "max" else min(vals)
                g = _jl_max if f == "max" else _jl_min
                r = self.real(vals[0])
                for x in vals[1:]:
                    r = g(r, self.real(x))
                return r
            if f == "abs":
                v = E(args[0])
                return abs(v) if isinstance(v, int) else abs(self.real(v))
            if f == "inv":
                return R(1.0) / self.real(E(args[0]))
            if f in ("one", "zero"):
                return R(1.0 if f == "one" else 0.0)
            if f == "ifelse":
                return E(args[1]) if E(args[0]) else E(args[2])
            if f in _FUN:
                v = self.real(E(args[0]))
                if isinstance(v, Dual):
                    return v.apply(f)
                fn = _FUN[f][0 if R is float else 1]
                return R(fn(v))
            raise NameError(f)
        raise ValueError(op)

    def run(self, stmts, I):
        for s in stmts:
            if s[0] == "return":
                raise _Return()
            if s[0] == "if":
                self.run(s[2] if self.ev(s[1], I) else s[3], I)
                continue
            if s[0] == "for":
                _, var, parts, body = s
                a, b = int(self.ev(parts[0], I)), int(self.ev(parts[-1], I))
                st = int(self.ev(parts[1], I)) if len(parts) == 3 else 1
                v = a
                while (v <= b) if st > 0 else (v >= b):
                    self.loc[var] = v
                    self.run(body, I)
                    v += st
                continue
            if s[0] == "while":
                while self.ev(s[1], I):
                    self.run(s[2], I)
                continue
            if s[0] == "do":
                if s[1][1] != "sync_threads":
                    raise SyntaxError(f"unsupported statement @{s[1][1]}")
                self.blk.bar.wait()
                continue
            _, lhs, rhs = s
            if lhs[0] == "name":  # local variable (a @sharedMem array or a number)
                v = self.ev(rhs, I)
                self.loc[lhs[1]] = v if isinstance(v, (np.ndarray, int)) and not isinstance(v, bool) \
                    else self.real(v)
            elif lhs[0] == "macro":
                sel, name = lhs[1], lhs[2]
                if name in self.temps:
                    continue
                kind, _, inner = _decode(sel, self.nd)
                a = self.A[name]
                # @within: the thread index lies inside the selection of A
                if any(I[d] > (a.shape[d] if d < a.ndim else 1) - (2 if d in inner else 0) for d in range(self.nd)):
                    continue
                v = self.real(self.ev(rhs, I))
                idx = tuple(I[d] - 1 + (1 if d in inner else 0) for d in range(a.ndim))
                a[idx] = v
            elif lhs[0] == "index":
                a = self.array(lhs[1])
                shape = a.shape + (1, 1)
                if len(lhs[2]) == 1 and lhs[2][0] == ("name", "__splat__"):
                    idx = list(I[:a.ndim])
                else:
                    idx = [int(self.ev(_subst_end(x, shape[d]), I)) for d, x in enumerate(lhs[2])]
                v = self.real(self.ev(rhs, I))
                for d in range(a.ndim):
                    if not 1 <= idx[d] <= a.shape[d]:
                        raise IndexError(f"BoundsError: {lhs[1]}{tuple(idx)} outside {a.shape}")
                a[tuple(i - 1 for i in idx[:a.ndim])] = v
            else:
                raise SyntaxError("unsupported left-hand side")


def _subst_end(e, n):
    if e == ("name", "end"):
        return ("num", n, False)
    if isinstance(e, tuple):
        return tuple(_subst_end(x, n) if isinstance(x, tuple) else
                     ([_subst_end(y, n) for y in x] if isinstance(x, list) else x) for x in e)
    return e


def _uses(node, names):
    if isinstance(node, tuple):
        if node and node[0] == "mcall" and node[1] in names:
            return True
        return any(_uses(x, names) for x in node)
    if isinstance(node, list):
        return any(_uses(x, names) for x in node)
    return False


def run(src, args, ndims=None, ranges=None, nthreads=None, nblocks=None, shmem=0):
    """Run kernel `src` on numpy arrays / scalars `args` (arrays are modified in place, like the
    device kernel). ranges: 1-based inclusive (start, stop) per dimension (dimensions not given
    have one index); default 1..max extent, or nblocks .* nthreads. nthreads (default (32, 8, 1))
    and shmem only matter for kernels that use the kernel language."""
    k = parse(src)
    if len(args) != len(k.argnames):
        raise TypeError("argument count")
    arrays = {n: a for n, a in zip(k.argnames, args) if isinstance(a, np.ndarray)}
    dts = {a.dtype for a in arrays.values() if a.dtype != object}  # object arrays hold Duals (jacobian)
    assert len(dts) <= 1
    R = np.float32 if dts == {np.dtype(np.float32)} else float
    scalars = {}
    for n, v in zip(k.argnames, args):
        if not isinstance(v, np.ndarray):
            scalars[n] = int(v) if isinstance(v, (int, np.integer)) and not isinstance(v, bool) else R(v)
    nd = ndims or k.ndims_opt or max(a.ndim for a in arrays.values())
    temps = {}
    for s in k.body:
        if s[0] == "assign" and s[1][0] == "macro" and s[1][2] not in arrays:
            if s[1][1] != "all":
                raise ValueError("on-the-fly arrays take @all")
            temps[s[1][2]] = s[2]
    bdim = list(nthreads) + [1] * (3 - len(nthreads)) if nthreads else [32, 8, 1]
    ext = [max((a.shape[d] if d < a.ndim else 1) for a in arrays.values()) for d in range(3)]
    lo, cnt = [1, 1, 1], [ext[0] if nd >= 1 else 1, ext[1] if nd >= 2 else 1, ext[2] if nd >= 3 else 1]
    if nblocks is not None:
        nb = list(nblocks) + [1] * (3 - len(nblocks))
        cnt = [nb[d] * bdim[d] for d in range(3)]
    if ranges is not None:
        lo, cnt = [1, 1, 1], [1, 1, 1]
        for d, r in enumerate(ranges):
            lo[d], cnt[d] = r[0], r[1] - r[0] + 1
    threaded = _uses(k.body, _COLL) or any(s[0] == "do" for s in _walk_stmts(k.body))
    if threaded and any(cnt[d] % bdim[d] for d in range(3)):
        raise ValueError("a kernel with @sync_threads, shuffles or votes needs ranges that are a multiple of the "
                         "thread block")
    gdim = [-(-cnt[d] // bdim[d]) for d in range(3)]
    for bz in range(gdim[2]):
        for by in range(gdim[1]):
            for bx in range(gdim[0]):
                blk = _Block((bx, by, bz), bdim, gdim, shmem, threaded)
                members = []
                for tz in range(bdim[2]):
                    for ty in range(bdim[1]):
                        for tx in range(bdim[0]):
                            u = (bx * bdim[0] + tx, by * bdim[1] + ty, bz * bdim[2] + tz)
                            if any(u[d] >= cnt[d] for d in range(3)):
                                continue
                            I = tuple(lo[d] + u[d] for d in range(3))
                            members.append((_Thread(k, arrays, scalars, temps, R, nd, blk, (tx, ty, tz)), I))
                if not threaded:
                    for t, I in members:
                        try:
                            t.run(k.body, I)
                        except _Return:
                            pass
                    continue
                errors = []

                def work(t, I):
                    try:
                        t.run(k.body, I)
                    except _Return:
                        pass
                    except BaseException as ex:  # a failing thread releases the others
                        errors.append(ex)
                        blk.bar.abort()
                        for wb in blk.warp_bars:
                            wb.abort()

                ths = [threading.Thread(target=work, args=m) for m in members]
                for th in ths:
                    th.start()
                for th in ths:
                    th.join()
                if errors:
                    real = [x for x in errors if not isinstance(x, threading.BrokenBarrierError)]
                    raise (real or errors)[0]


def _walk_stmts(stmts):
    for s in stmts:
        yield s
        if s[0] == "if" and len(s) == 4:
            yield from _walk_stmts(s[2])
            yield from _walk_stmts(s[3])
        elif s[0] == "for":
            yield from _walk_stmts(s[3])
        elif s[0] == "while":
            yield from _walk_stmts(s[2])


# ---------------------------------------------------------------- derivatives (the `@parallel ∇` checker)
def _comb(d1, a, d2, b):
    r = {k: a * v for k, v in d1.items()}
    for k, v in d2.items():
        r[k] = r.get(k, 0.0) + b * v
    return r


_DFUN = {"exp": lambda x, y: y, "log": lambda x, y: 1.0 / x, "sqrt": lambda x, y: 0.5 / y,
         "sin": lambda x, y: math.cos(x), "cos": lambda x, y: -math.sin(x), "tan": lambda x, y: 1.0 + y * y,
         "tanh": lambda x, y: 1.0 - y * y, "sinh": lambda x, y: math.cosh(x), "cosh": lambda x, y: math.sinh(x),
         "atan": lambda x, y: 1.0 / (1.0 + x * x), "asin": lambda x, y: 1.0 / math.sqrt(1.0 - x * x),
         "acos": lambda x, y: -1.0 / math.sqrt(1.0 - x * x), "log10": lambda x, y: 1.0 / (x * math.log(10.0)),
         "exp2": lambda x, y: y * math.log(2.0), "cbrt": lambda x, y: 1.0 / (3.0 * y * y)}


class Dual:
    """A double value with its first derivatives with respect to chosen inputs (a sparse map
    input -> derivative). The value follows IEEE double arithmetic exactly as the interpreter's
    plain floats do; the derivatives follow the chain rule of each operation. Comparisons look at
    the value, so branches, max / min and ifelse select like the plain run."""

    __slots__ = ("v", "d")
    __hash__ = None

    def __init__(self, v, d=None):
        self.v, self.d = float(v), d if d is not None else {}

    @staticmethod
    def lift(x):
        return x if isinstance(x, Dual) else Dual(float(x))

    def __float__(self):
        return self.v

    def __add__(self, o):
        o = Dual.lift(o)
        return Dual(self.v + o.v, _comb(self.d, 1.0, o.d, 1.0))

    def __radd__(self, o):
        return Dual.lift(o) + self

    def __sub__(self, o):
        o = Dual.lift(o)
        return Dual(self.v - o.v, _comb(self.d, 1.0, o.d, -1.0))

    def __rsub__(self, o):
        return Dual.lift(o) - self

    def __mul__(self, o):
        o = Dual.lift(o)
        return Dual(self.v * o.v, _comb(self.d, o.v, o.d, self.v))

    def __rmul__(self, o):
        return Dual.lift(o) * self

    def __truediv__(self, o):
        o = Dual.lift(o)
        q = self.v / o.v
        return Dual(q, _comb(self.d, 1.0 / o.v, o.d, -q / o.v))

    def __rtruediv__(self, o):
        return Dual.lift(o) / self

    def __neg__(self):
        return Dual(-self.v, {k: -v for k, v in self.d.items()})

    def __abs__(self):
        return -self if math.copysign(1.0, self.v) < 0 else self

    def __pow__(self, p):
        p = Dual.lift(p)
        v = self.v ** p.v
        d = {k: p.v * self.v ** (p.v - 1.0) * x for k, x in self.d.items()}
        if p.d:
            d = _comb(d, 1.0, p.d, v * math.log(self.v))
        return Dual(v, d)

    def apply(self, f):
        y = float(_FUN[f][0](self.v))
        g = _DFUN[f](self.v, y)
        return Dual(y, {k: g * x for k, x in self.d.items()})

    def _o(self, o):
        return o.v if isinstance(o, Dual) else o

    def __lt__(self, o):
        return self.v < self._o(o)

    def __le__(self, o):
        return self.v <= self._o(o)

    def __gt__(self, o):
        return self.v > self._o(o)

    def __ge__(self, o):
        return self.v >= self._o(o)

    def __eq__(self, o):
        return self.v == self._o(o)

    def __ne__(self, o):
        return self.v != self._o(o)


def jacobian(src, args, dup, **kw):
    """The Jacobian of kernel `src`'s state map over the arrays at argument positions `dup` (FP64):
    each of their elements starts as a Dual seeded with itself, the kernel runs in the interpreter
    (other arrays and scalars as given, so values stored into them lose their derivatives, like
    constants), and every element of a duplicated array afterwards is its output -- an element the
    kernel did not write keeps its own seed (identity row). Returns {position: (values, rows)} with
    rows an object array of derivative maps {(position, flat index): value}, flat indices in
    column-major order. `kw` goes to run() (ndims, ranges, ...)."""
    seeded = list(args)
    for p in dup:
        a = np.asarray(args[p], dtype=np.float64)
        o = np.empty(a.shape, dtype=object, order="F")
        for idx in np.ndindex(a.shape):
            o[idx] = Dual(a[idx], {(p, int(np.ravel_multi_index(idx, a.shape, order="F"))): 1.0})
        seeded[p] = o
    run(src, seeded, **kw)
    out = {}
    for p in dup:
        o = seeded[p]
        vals = np.empty(o.shape, order="F")
        rows = np.empty(o.shape, dtype=object, order="F")
        for idx in np.ndindex(o.shape):
            x = o[idx]
            vals[idx] = float(x)
            rows[idx] = x.d if isinstance(x, Dual) else {}
        out[p] = (vals, rows)
    return out


def reverse_shadows(jac, shadows):
    """Reverse mode: shadows after = J^T shadows before (`shadows`: {position: array}); the shadow of
    an element the kernel overwrote starts from zero, and every input element gathers the adjoints
    of the outputs it reached."""
    new = {p: np.zeros(np.shape(s), order="F") for p, s in shadows.items()}
    flat = {p: np.asarray(s, dtype=np.float64).ravel(order="F") for p, s in shadows.items()}
    acc = {p: np.zeros(f.size) for p, f in flat.items()}
    for p, (_, rows) in jac.items():
        rf = rows.ravel(order="F")
        for e in range(rf.size):
            w = flat[p][e]
            if w == 0.0:
                continue
            for (q, j), c in rf[e].items():
                acc[q][j] += c * w
    for p in new:
        new[p] = acc[p].reshape(np.shape(shadows[p]), order="F")
    return new


def forward_shadows(jac, shadows):
    """Forward mode: shadows after = J shadows before."""
    flat = {p: np.asarray(s, dtype=np.float64).ravel(order="F") for p, s in shadows.items()}
    new = {}
    for p, (_, rows) in jac.items():
        rf = rows.ravel(order="F")
        out = np.zeros(rf.size)
        for e in range(rf.size):
            out[e] = sum(c * flat[q][j] for (q, j), c in rf[e].items())
        new[p] = out.reshape(rows.shape, order="F")
    return new
