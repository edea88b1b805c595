"""Derivatives of run-time compiled kernels: ``@parallel ∇=(A->Ā, B->B̄) f!(A, B, a)``.

The reference differentiates a kernel with Enzyme: `@parallel ∇=(A->Ā, B->B̄) f!(A, B, a)` expands
to `@parallel configcall=f!(A, B, a) AD.autodiff_deferred!(Enzyme.Reverse, f!,
DuplicatedNoNeed(A, Ā), DuplicatedNoNeed(B, B̄), Const(a))` (src/ParallelKernel/parallel.jl:265-301)
and every thread runs `Enzyme.autodiff_deferred(mode, f!, Const, args...)` on its own point
(src/ParallelKernel/EnzymeExt/autodiff_gpu.jl:35-40). Here the derivative kernel is generated from
the definition's source, like the kernel itself (ps_gb300.jit), and compiled for sm_103a:

- reverse mode (``ad_mode="reverse"``, Enzyme.Reverse): each thread runs its statements -- the
  primal stores happen, as in Enzyme's combined reverse mode -- keeping every intermediate value in
  registers, then walks them backwards: the shadow of a written element is read and zeroed (the
  element's old value no longer reaches the result) and the adjoint of every value read from a
  duplicated array is added to that array's shadow. A shadow element that other threads may also
  update takes an atomic addition (as Enzyme's gradient accumulation on the GPU does); a shadow
  that only its own thread touches is updated in place. Over the kernel's state map M -> F(M) of
  the duplicated arrays: shadow <- J_F(M)^T shadow.
- forward mode (``ad_mode="forward"``, Enzyme.Forward): the tangent of every value is carried
  beside it, and the shadow of a written element receives the tangent of its new value:
  shadow <- J_F(M) shadow (elements not written keep theirs).

Scalars are constants (Enzyme.Const), and so are the arrays not named in ∇. Supported bodies:
`@parallel` kernels (FiniteDifferences macros, on-the-fly arrays, masks of the left-hand
selections) and `@parallel_indices` kernels with explicit indexing, local variables and
if / elseif / else blocks (an early `return` included); arithmetic + - * /, literal and general
powers, max / min / abs / ifelse / inv and the kernel language's math functions. Loops and
kernel-language calls (shared memory, barriers, shuffles) are refused, and so is a duplicated
array that is written and also accessed at another index (its threads would race).
"""
from __future__ import annotations

import ast
import ctypes
import numbers
import re

from . import _lib
from ._lib import PSArray
from .core import ArgumentError, descriptor, require_initialized, stream_handle
from .fd import AV, DIFF, DIFF2, HARM, MAXLOC, MINLOC, SEL
from .jit import _MATH, JitKernel, _Gen, _lit, array_ndims, uses_kernel_language
from .kernels import ranges_to_box

MODES = ("reverse", "forward")
_ONE = "((R)1.0)"
_LITERAL = re.compile(r"^\(\(R\)[-+0-9.eE]+\)$")  # a number literal of the kernel's type
_SCALAR = re.compile(r"^s[0-9]+$")                  # a scalar argument


class _X:
    """A real value of the derivative kernel: an SSA register with an adjoint / tangent (`var`), or a
    value without derivative (a literal, a scalar argument, or a register holding a constant)."""

    __slots__ = ("code", "var")

    def __init__(self, code, var=False):
        self.code, self.var = code, var


# Shadow-memory helpers of the generated kernels (bounds-checked like the primal accesses: an index
# outside the array was already reported by the primal load, and its shadow is left alone).
_HELPERS = r"""
__device__ __forceinline__ bool ad_in(long long n0, long long n1, long long n2, long long i, long long j, long long k) {
    return (unsigned long long)i < (unsigned long long)n0 && (unsigned long long)j < (unsigned long long)n1 && (unsigned long long)k < (unsigned long long)n2; }
__device__ __forceinline__ E ad_ld(const E* d, long long n0, long long n1, long long n2, long long i, long long j, long long k) {
    return ad_in(n0, n1, n2, i, j, k) ? d[i + n0 * (j + n1 * k)] : (E)0; }
__device__ __forceinline__ void ad_st(E* d, long long n0, long long n1, long long n2, long long i, long long j, long long k, E v) {
    if (ad_in(n0, n1, n2, i, j, k)) d[i + n0 * (j + n1 * k)] = v; }
__device__ __forceinline__ E ad_take(E* d, long long n0, long long n1, long long n2, long long i, long long j, long long k) {
    if (!ad_in(n0, n1, n2, i, j, k)) return (E)0;
    const long long l = i + n0 * (j + n1 * k); const E g = d[l]; d[l] = (E)0; return g; }
__device__ __forceinline__ void ad_add(E* d, long long n0, long long n1, long long n2, long long i, long long j, long long k, E v, bool shared) {
    if (!ad_in(n0, n1, n2, i, j, k)) return;
    const long long l = i + n0 * (j + n1 * k);
    if (shared) atomicAdd(&d[l], v); else d[l] += v; }
"""


class _AdGen(_Gen):
    """Source of the derivative kernel of one definition (one point per thread)."""

    def __init__(self, kd, ndims, dup, mode):
        if mode not in MODES:
            raise ArgumentError(f"ad_mode must be one of {MODES}")
        if uses_kernel_language(kd):
            raise ArgumentError(f"{kd.name}: kernels that use the kernel language (@sharedMem, barriers, shuffles, "
                                "votes, thread indices) cannot be differentiated here")
        super().__init__(kd, ndims)
        unknown = [n for n in dup if n not in kd.arrays]
        if unknown:
            raise ArgumentError(f"∇: {unknown} are not array arguments of {kd.name}")
        self.dup = [n for n in kd.arrays if n in dup]
        self.didx = {n: len(kd.arrays) + i for i, n in enumerate(self.dup)}
        self.mode = mode
        self.nv = 0
        self.vars = []       # (register, C type) declared at the top of the kernel
        self.dvars = []      # registers with an adjoint (b...) or tangent (t...)
        self.tape = []       # (executed flag, nodes, store) per statement, in execution order
        self.nodes = None
        self.cur = {}        # real local variable -> its current value
        self.cache = None    # loads of one `@parallel` statement: (array, offsets) -> value
        self.keys = {}       # array -> access keys (offsets / index expressions) of all its accesses
        self.written = set()
        self.fw = []
        self.ind = "    "

    # ---- registers and nodes
    def _new(self, ctype):
        name = {"R": "v", "long long": "i", "bool": "f"}[ctype] + str(self.nv)
        self.nv += 1
        self.vars.append((name, ctype))
        return name

    def emit(self, line):
        self.fw.append(self.ind + line)

    def const(self, code):
        """A value without derivative; anything but a literal or a scalar is kept in a register
        (the reverse sweep must see the value of the forward sweep)."""
        if _LITERAL.match(code) or _SCALAR.match(code):
            return _X(code)
        c = self._new("R")
        self.emit(f"{c} = {code};")
        return _X(c)

    def node(self, op, code, ins, aux=None):
        if op != "load" and not any(x.var for x in ins):
            return self.const(code)
        v = self._new("R")
        self.dvars.append(v)
        self.emit(f"{v} = {code};")
        out = _X(v, True)
        self.nodes.append((op, out, ins, aux))
        if self.mode == "forward":
            self.emit(f"t{v} = {self.tangent(op, out, ins, aux)};")
        return out

    def bin(self, op, sym, a, b):
        return self.node(op, f"({a.code} {sym} {b.code})", [a, b])

    def flag(self, code):
        f = self._new("bool")
        self.emit(f"{f} = {code};")
        return f

    # ---- loads
    def key(self, name, key):
        self.keys.setdefault(name, set()).add(key)

    def leaf(self, name, idx, key=None):
        if name in self.shared or name not in self.aidx:
            raise ArgumentError(f"∇: {name} is not an array argument")
        self.key(name, key or ("i", tuple(idx)))
        ivs = []
        for x in idx:
            iv = self._new("long long")
            self.emit(f"{iv} = {x};")
            ivs.append(iv)
        code = self.load(name, ivs)
        if name in self.dup:
            return self.node("load", code, [], aux=(name, ivs))
        return self.const(code)

    def lval(self, name, o):
        if name in self.temps:  # on-the-fly array: its expression at the shifted index
            li, e = self.temps[name]
            return self.lo(e, tuple(o[d] - ((li >> d) & 1) for d in range(3)))
        if name not in self.aidx:
            raise ArgumentError(f"unknown array {name}")
        o3 = tuple(o[d] if d < self.nd else 0 for d in range(3))
        if self.cache is not None and (name, o3) in self.cache:
            return self.cache[(name, o3)]
        t = ("tx", "ty", "tz")
        idx = [f"{t[d]}+{o3[d]}" if o3[d] else t[d] for d in range(self.nd)]
        x = self.leaf(name, idx, ("o", o3[:self.nd]))
        if self.cache is not None:
            self.cache[(name, o3)] = x
        return x

    def lmacro(self, mname, name, off):
        """A FiniteDifferences macro as value nodes, in the operation order of the forward kernel."""
        if mname not in self.macros:
            raise ArgumentError(f"unknown macro @{mname} for {self.nd}-D")
        kind, opd, inn = self.macros[mname]
        b = [off[d] + ((inn >> d) & 1) for d in range(3)]

        def shift(d, s):
            o = list(b)
            o[d] += s
            return self.lval(name, o)

        dims = [d for d in range(3) if (opd >> d) & 1]
        if kind == SEL:
            return self.lval(name, b)
        if kind == DIFF:
            return self.bin("sub", "-", shift(dims[0], 1), self.lval(name, b))
        if kind == DIFF2:
            c = self.lval(name, b)
            return self.bin("sub", "-", self.bin("sub", "-", shift(dims[0], 1), c),
                            self.bin("sub", "-", c, shift(dims[0], -1)))
        if kind in (AV, HARM):
            terms = []
            for c in range(1 << len(dims)):
                o = list(b)
                for j, d in enumerate(dims):
                    o[d] += (c >> j) & 1
                v = self.lval(name, o)
                terms.append(self.bin("div", "/", _X(_ONE), v) if kind == HARM else v)
            s = terms[0]
            for t in terms[1:]:
                s = self.bin("add", "+", s, t)
            k = float(1 << len(dims))
            if kind == AV:
                return self.bin("mul", "*", s, _X(_lit(1.0 / k)))
            return self.bin("mul", "*", self.bin("div", "/", _X(_ONE), s), _X(_lit(k)))
        if kind in (MAXLOC, MINLOC):
            op, f = ("max", "jl_max") if kind == MAXLOC else ("min", "jl_min")

            def m(x, y):
                return self.node(op, f"{f}({x.code}, {y.code})", [x, y])
            r = m(m(shift(0, -1), shift(0, 1)), self.lval(name, b))
            for d in range(1, self.nd):
                r = m(r, m(shift(d, -1), shift(d, 1)))
            return r
        raise ArgumentError(f"macro @{mname} not supported")

    # ---- real expressions as value nodes
    def lo(self, e, off=(0, 0, 0)):
        t = self.etype(e)
        if t == "int":
            return self.const(self.expr(e, off, "real"))
        if t == "bool":
            return self.const(f"((R)({self.expr(e, off, 'auto')}))")
        if isinstance(e, ast.Constant):
            return _X(_lit(e.value))
        if isinstance(e, ast.Name):
            if e.id in self.sidx:
                return _X(f"s{self.sidx[e.id]}")
            if e.id in self.cur:
                return self.cur[e.id]
            if e.id in self.locals:
                raise ArgumentError(f"∇: local {e.id} is read before it is assigned")
            raise ArgumentError(f"unknown name {e.id} in an expression")
        if isinstance(e, ast.UnaryOp):
            if isinstance(e.op, ast.USub):
                a = self.lo(e.operand, off)
                return self.node("neg", f"(-{a.code})", [a])
            if isinstance(e.op, ast.UAdd):
                return self.lo(e.operand, off)
        if isinstance(e, ast.BinOp):
            if isinstance(e.op, ast.Pow):
                if isinstance(e.right, ast.Constant) and e.right.value in (2, 3) and not isinstance(e.right.value, bool):
                    x = self.lo(e.left, off)
                    sq = self.bin("mul", "*", x, x)
                    return sq if e.right.value == 2 else self.bin("mul", "*", sq, x)
                a, b = self.lo(e.left, off), self.lo(e.right, off)
                return self.node("pow", f"pow({a.code}, (R)({b.code}))", [a, b])
            if isinstance(e.op, ast.Mult) and (self.is_bool(e.left) or self.is_bool(e.right)):
                bl, x = (e.left, e.right) if self.is_bool(e.left) else (e.right, e.left)
                f = self.flag(self.expr(bl, off, "auto"))
                xv = self.lo(x, off)
                return self.node("bmul", f"jl_bmul({f}, {xv.code})", [xv], f)
            if isinstance(e.op, ast.Mod):
                a, b = self.lo(e.left, off), self.lo(e.right, off)
                return self.node("fmod", f"fmod({a.code}, {b.code})", [a, b])
            if isinstance(e.op, ast.FloorDiv):  # a step function: no derivative
                a, b = self.lo(e.left, off), self.lo(e.right, off)
                return self.const(f"trunc({a.code} / {b.code})")
            ops = {ast.Add: ("add", "+"), ast.Sub: ("sub", "-"), ast.Mult: ("mul", "*"), ast.Div: ("div", "/")}
            if type(e.op) not in ops:
                raise ArgumentError("unsupported operator")
            op, sym = ops[type(e.op)]
            return self.bin(op, sym, self.lo(e.left, off), self.lo(e.right, off))
        if isinstance(e, ast.Call) and isinstance(e.func, ast.Name):
            f = e.func.id
            if f.startswith("__m_"):
                if len(e.args) != 1 or not isinstance(e.args[0], ast.Name):
                    raise ArgumentError(f"@{f[4:]} takes one array")
                return self.lmacro(f[4:], e.args[0].id, off)
            if f in ("max", "min"):
                r = self.lo(e.args[0], off)
                for x in e.args[1:]:
                    xv = self.lo(x, off)
                    r = self.node(f, f"jl_{f}({r.code}, {xv.code})", [r, xv])
                return r
            if f == "abs":
                a = self.lo(e.args[0], off)
                return self.node("abs", f"fabs({a.code})", [a])
            if f == "inv":
                a = self.lo(e.args[0], off)
                return self.bin("div", "/", _X(_ONE), a)
            if f in ("one", "zero"):
                return _X("((R)1)" if f == "one" else "((R)0)")
            if f == "ifelse":
                c = self.flag(self.expr(e.args[0], off, "auto"))
                a, b = self.lo(e.args[1], off), self.lo(e.args[2], off)
                return self.node("select", f"({c} ? {a.code} : {b.code})", [a, b], c)
            if f in _MATH:
                a = self.lo(e.args[0], off)
                return self.node(f, f"{f}({a.code})", [a])
            raise ArgumentError(f"∇: unsupported function {f}")
        if isinstance(e, ast.Subscript):
            name, ix = self.subscript(e, off)
            return self.leaf(name, ix)
        raise ArgumentError(f"∇: unsupported expression {ast.dump(e)[:80]}")

    # ---- statements (forward sweep; the reverse sweep is built from the tape)
    def stmt(self, s, ind):
        saved = self.fw, self.ind
        self.fw, self.ind = [], "    " * ind
        try:
            self._stmt(s, ind)
            return self.fw
        finally:
            self.fw, self.ind = saved

    def begin(self):
        f = self.flag("true")
        self.nodes = []
        return f

    def end(self, f, store=None):
        self.tape.append((f, self.nodes, store))
        self.nodes = None

    def store(self, name, idx, rhs):
        """Primal store of rhs at idx (0-based index registers or expressions) and, in forward mode,
        of its tangent into the shadow."""
        k = self.aidx[name]
        i3 = list(idx) + ["0"] * (3 - len(idx))
        if self.checked:
            self.emit(f"jl_st(a{k}, n{k}_0, n{k}_1, n{k}_2, {i3[0]}, {i3[1]}, {i3[2]}, g.err, (E)({rhs.code}));")
        else:
            self.emit(f"{self.at(name, idx)} = (E)({rhs.code});")
        if self.mode == "forward" and name in self.dup:
            t = f"t{rhs.code}" if rhs.var else "(R)0"
            self.emit(f"ad_st(d{k}, n{k}_0, n{k}_1, n{k}_2, {i3[0]}, {i3[1]}, {i3[2]}, (E)({t}));")
        self.written.add(name)
        return (name, i3, rhs)

    def _stmt(self, s, ind):
        if isinstance(s, ast.If):
            c = self.flag(f"({self.expr(s.test, ctx='auto')})")
            before = dict(self.cur)
            self.emit(f"if ({c}) {{")
            for b in s.body:
                self.fw += self.stmt(b, ind + 1)
            then = self.cur
            self.cur = dict(before)
            if s.orelse:
                self.emit("} else {")
                for b in s.orelse:
                    self.fw += self.stmt(b, ind + 1)
            self.emit("}")
            other = self.cur
            self.cur = dict(before)
            for name in sorted(set(then) | set(other)):
                a, b = then.get(name, _X("((R)0)")), other.get(name, _X("((R)0)"))
                if a is b:
                    self.cur[name] = a
                    continue
                f = self.begin()
                v = self.node("select", f"({c} ? {a.code} : {b.code})", [a, b], c)
                self.emit(f"v_{name} = {v.code};")
                self.end(f)
                self.cur[name] = v
            return
        if isinstance(s, (ast.For, ast.While)):
            raise ArgumentError("∇: kernels with loops cannot be differentiated here")
        if isinstance(s, ast.Pass):
            return
        if isinstance(s, ast.Return):
            if s.value is not None:
                raise ArgumentError("kernels return nothing")
            self.emit("goto ps_fwd_done_;")
            return
        if not isinstance(s, ast.Assign) or len(s.targets) != 1:
            raise ArgumentError("∇: kernel statements are assignments and if-blocks")
        t = s.targets[0]
        if isinstance(t, ast.Name):  # local variable
            if self.locals.get(t.id) == "int":
                self.emit(f"v_{t.id} = (long long)({self.expr(s.value, ctx='int')});")
                return
            f = self.begin()
            v = self.lo(s.value)
            self.emit(f"v_{t.id} = {v.code};")
            self.end(f)
            self.cur[t.id] = v
            return
        if isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name) and t.value.id.startswith("__lhs_"):
            sel, name = t.value.id[6:], t.slice.id
            if sel not in self.sels:
                raise ArgumentError(f"@{sel} cannot be a left-hand side")
            if name in self.temps:
                return
            li = self.sels[sel]
            k = self.aidx[name]
            t3 = ("tx", "ty", "tz")
            cond = " && ".join(f"{t3[d]} < n{k}_{d} - {2 * ((li >> d) & 1)}" for d in range(self.nd))
            self.emit(f"if ({cond}) {{")
            saved = self.ind
            self.ind += "    "
            f = self.begin()
            self.cache = {}
            rhs = self.lo(s.value)
            self.cache = None
            o = tuple((li >> d) & 1 for d in range(self.nd))
            self.key(name, ("o", o))
            idx = [f"{t3[d]}+{o[d]}" if o[d] else t3[d] for d in range(self.nd)]
            st = self.store(name, idx, rhs)
            self.end(f, st)
            self.ind = saved
            self.emit("}")
            return
        if isinstance(t, ast.Subscript):  # @parallel_indices: A[i, j] = expr
            name, ix = self.subscript(t)
            if name in self.shared:
                raise ArgumentError("∇: @sharedMem arrays cannot be differentiated")
            f = self.begin()
            rhs = self.lo(s.value)
            self.key(name, ("i", tuple(ix)))
            ivs = []
            for x in ix:
                iv = self._new("long long")
                self.emit(f"{iv} = {x};")
                ivs.append(iv)
            st = self.store(name, ivs, rhs)
            self.end(f, st)
            return
        raise ArgumentError("unsupported left-hand side")

    # ---- derivative rules
    def tangent(self, op, out, ins, aux):
        a = ins[0] if ins else None
        b = ins[1] if len(ins) > 1 else None
        A, B, O = (a.code if a else ""), (b.code if b else ""), out.code

        def T(x):
            return f"t{x.code}" if x.var else "(R)0"
        if op == "load":
            name, ivs = aux
            k = self.aidx[name]
            i3 = list(ivs) + ["0"] * (3 - len(ivs))
            return f"(R)ad_ld(d{k}, n{k}_0, n{k}_1, n{k}_2, {i3[0]}, {i3[1]}, {i3[2]})"
        if op == "add":
            return f"({T(a)} + {T(b)})"
        if op == "sub":
            return f"({T(a)} - {T(b)})"
        if op == "neg":
            return f"(-{T(a)})"
        if op == "mul":
            return f"({T(a)} * {B} + {A} * {T(b)})"
        if op == "div":
            return f"(({T(a)} - {O} * {T(b)}) / {B})"
        if op == "select":
            return f"({aux} ? {T(a)} : {T(b)})"
        if op == "bmul":
            return f"({aux} ? {T(a)} : (R)0)"
        if op in ("max", "min"):
            sel = f"!signbit({A} - {B})" if op == "max" else f"signbit({A} - {B})"
            return f"(({sel}) ? {T(a)} : {T(b)})"
        if op == "abs":
            return f"(signbit({A}) ? -{T(a)} : {T(a)})"
        if op == "pow":
            s = f"{T(a)} * {B} * pow({A}, {B} - (R)1)"
            return f"({s} + {T(b)} * {O} * log({A}))" if b.var else f"({s})"
        if op == "fmod":
            return f"({T(a)} - {T(b)} * trunc({A} / {B}))"
        return f"({T(a)} * {self.dfun(op, A, O)})"

    def dfun(self, op, A, O):
        """d op(A) / dA, with O = op(A)."""
        return {"exp": O, "exp2": f"{O} * (R)0.6931471805599453", "log": f"((R)1 / {A})",
                "log10": f"((R)1 / ({A} * (R)2.302585092994046))", "sqrt": f"((R)1 / ({O} + {O}))",
                "cbrt": f"((R)1 / ((R)3 * {O} * {O}))", "sin": f"cos({A})", "cos": f"(-sin({A}))",
                "tan": f"((R)1 + {O} * {O})", "tanh": f"((R)1 - {O} * {O})", "sinh": f"cosh({A})",
                "cosh": f"sinh({A})", "atan": f"((R)1 / ((R)1 + {A} * {A}))",
                "asin": f"((R)1 / sqrt((R)1 - {A} * {A}))", "acos": f"(-(R)1 / sqrt((R)1 - {A} * {A}))"}[op]

    def adjoint(self, op, out, ins, aux):
        a = ins[0] if ins else None
        b = ins[1] if len(ins) > 1 else None
        A, B, O, bo = (a.code if a else ""), (b.code if b else ""), out.code, f"b{out.code}"
        lines = []

        def acc(x, expr):
            if x is not None and x.var:
                lines.append(f"b{x.code} += {expr};")
        if op == "load":
            name, ivs = aux
            k = self.aidx[name]
            i3 = list(ivs) + ["0"] * (3 - len(ivs))
            lines.append(f"ad_add(d{k}, n{k}_0, n{k}_1, n{k}_2, {i3[0]}, {i3[1]}, {i3[2]}, (E){bo}, "
                         f"{'true' if self.is_shared(name) else 'false'});")
        elif op == "add":
            acc(a, bo)
            acc(b, bo)
        elif op == "sub":
            acc(a, bo)
            acc(b, f"-{bo}")
        elif op == "neg":
            acc(a, f"-{bo}")
        elif op == "mul":
            acc(a, f"{bo} * {B}")
            acc(b, f"{bo} * {A}")
        elif op == "div":
            acc(a, f"{bo} / {B}")
            acc(b, f"-({bo} * {O}) / {B}")
        elif op == "select":
            acc(a, f"({aux} ? {bo} : (R)0)")
            acc(b, f"({aux} ? (R)0 : {bo})")
        elif op == "bmul":
            acc(a, f"({aux} ? {bo} : (R)0)")
        elif op in ("max", "min"):
            sel = f"!signbit({A} - {B})" if op == "max" else f"signbit({A} - {B})"
            acc(a, f"(({sel}) ? {bo} : (R)0)")
            acc(b, f"(({sel}) ? (R)0 : {bo})")
        elif op == "abs":
            acc(a, f"(signbit({A}) ? -{bo} : {bo})")
        elif op == "pow":
            acc(a, f"{bo} * {B} * pow({A}, {B} - (R)1)")
            acc(b, f"{bo} * {O} * log({A})")
        elif op == "fmod":
            acc(a, bo)
            acc(b, f"-{bo} * trunc({A} / {B})")
        else:
            acc(a, f"{bo} * {self.dfun(op, A, O)}")
        return lines

    def is_shared(self, name):
        """Whether other threads may touch the shadow elements this thread touches: unless every
        access of the array in the kernel goes to one index of the thread's own (the same offsets /
        the same index expressions of the thread indices alone)."""
        ks = self.keys.get(name, set())
        if len(ks) != 1:
            return True
        (kind, k), = ks
        return kind == "i" and any("v_" in x for x in k)

    def check_races(self):
        for name in self.dup:
            if name in self.written and self.is_shared(name):
                raise ArgumentError(f"∇: {name} is written and also accessed at another index in {self.kd.name} "
                                    "(its threads would race)")

    def reverse_lines(self):
        out = []
        for f, nodes, store in reversed(self.tape):
            blk = []
            if store is not None:
                name, i3, rhs = store
                if name not in self.dup:  # a constant array: nothing flows back from its elements
                    continue
                k = self.aidx[name]
                g = f"ad_take(d{k}, n{k}_0, n{k}_1, n{k}_2, {i3[0]}, {i3[1]}, {i3[2]})"
                blk.append(f"b{rhs.code} += (R){g};" if rhs.var else f"(void){g};")
            for op, o, ins, aux in reversed(nodes):
                blk += self.adjoint(op, o, ins, aux)
            if blk:
                out += [f"    if ({f}) {{"] + ["        " + x for x in blk] + ["    }"]
        return out

    # ---- hooks of the kernel template
    def body_lines(self):
        fw = []
        for s in self.kd.body:
            fw += self.stmt(s, 1)
        self.check_races()
        out = fw + ["    if (0) goto ps_fwd_done_;", "ps_fwd_done_:;"]
        if self.mode == "reverse":
            out += self.reverse_lines()
        return out

    def extra_decl(self):
        decl = []
        for name in self.dup:
            decl.append(f"    E* const d{self.aidx[name]} = (E*)g.a[{self.didx[name]}];")
        init = {"R": "0", "long long": "0", "bool": "false"}
        for v, ctype in self.vars:
            decl.append(f"    {ctype} {v} = {init[ctype]};")
        p = "b" if self.mode == "reverse" else "t"
        for v in self.dvars:
            decl.append(f"    R {p}{v} = 0;")
        return decl

    def types(self, real):
        return super().types(real) + "\n" + _HELPERS


def generate(kd, ndims, dtype, dup, mode="reverse"):
    """CUDA C of the derivative kernel of `kd` (arrays `dup` duplicated; their shadows follow the
    primal arrays in the argument list)."""
    return _AdGen(kd, ndims, set(dup), mode).source(dtype)


def _pairs(kernel: JitKernel, args, grad):
    """`grad` = ((primal, shadow), ...), as ∇=(A->Ā, B->B̄): primals matched to the call's array
    arguments by identity. Returns the duplicated argument names and their shadows in order."""
    names = {}
    for (kind, name), a in zip(kernel.kd.args, args):
        if kind == "array":
            names.setdefault(id(a), name)
    dup = {}
    for pair in grad:
        if len(pair) != 2:
            raise ArgumentError("∇ pairs are (primal, shadow)")
        p, s = pair
        if id(p) not in names:
            raise ArgumentError("∇: a primal is not an array argument of the kernel call")
        n = names[id(p)]
        if n in dup:
            raise ArgumentError(f"∇: {n} appears twice")
        dup[n] = s
    return dup


def parallel_grad(kernel: JitKernel, args, grad, ad_mode="reverse", ranges=None, stream=None, sync=True,
                  nblocks=None, nthreads=None):
    """`@parallel ∇=(A->Ā, ...) [ad_mode=...] kernel!(args...)` for a run-time compiled kernel:
    launches the derivative kernel over the kernel's own grid (or `ranges` / nblocks .* nthreads),
    one point per thread. Shadows are arrays of the primals' shapes and number type."""
    require_initialized()
    if not isinstance(kernel, JitKernel):
        raise ArgumentError("∇ applies to run-time compiled kernels (ps_gb300.parallel_kernel)")
    if ad_mode not in MODES:
        raise ArgumentError(f"ad_mode must be one of {MODES}")
    if len(args) != kernel.nargs:
        raise ArgumentError(f"{kernel.name} takes {kernel.nargs} arguments (obtained {len(args)})")
    dup = _pairs(kernel, args, grad)
    arrs, scal, by_name = [], [], {}
    for (kind, name), a in zip(kernel.kd.args, args):
        if kind == "scalar":
            if not isinstance(a, numbers.Real):
                raise ArgumentError(f"{kernel.name}: argument {name} is a scalar (obtained {type(a).__name__})")
            scal.append(a)
        else:
            arrs.append(a)
            by_name[name] = a
    descs = [descriptor(a) for a in arrs]
    order = [n for n in kernel.kd.arrays if n in dup]
    sdescs = [descriptor(dup[n]) for n in order]
    for n, sd in zip(order, sdescs):
        pd = descriptor(by_name[n])
        if tuple(sd.n) != tuple(pd.n) or sd.dtype != pd.dtype:
            raise ArgumentError(f"∇: the shadow of {n} must have its shape and number type")
    dt = {0: "double", 1: "float"}.get(descs[0].dtype) if descs else "double"
    if dt is None or any(d.dtype != descs[0].dtype for d in descs):
        raise ArgumentError("the array arguments must share one FP64 or FP32 type")
    if len(descs) + len(sdescs) > 32:
        raise ArgumentError("∇: at most 32 arrays and shadows")
    ndims = kernel.ndims or array_ndims(descs)
    lo, cnt = [0, 0, 0], JitKernel._extent(descs, ndims)
    threads = [32, 8, 1]
    if nthreads is not None:
        nt = tuple(int(x) for x in (nthreads if isinstance(nthreads, (tuple, list)) else (nthreads,)))
        threads = list(nt) + [1] * (3 - len(nt))
    if nblocks is not None:
        if nthreads is None:
            raise ArgumentError("nblocks needs nthreads")
        nb = tuple(int(x) for x in (nblocks if isinstance(nblocks, (tuple, list)) else (nblocks,)))
        nb = nb + (1,) * (3 - len(nb))
        cnt = [nb[d] * threads[d] for d in range(3)]
    if ranges is not None:
        lo, hi = ranges_to_box(ranges)
        if min(lo) < 0:
            raise ArgumentError("ranges must start at index 1 or above")
        cnt = [max(0, hi[d] - lo[d]) for d in range(3)]
    key = ("ad", ad_mode, tuple(order), ndims, dt)
    if key not in kernel._handles:
        src = generate(kernel.kd, ndims, dt, order, ad_mode)
        h = ctypes.c_void_p()
        _lib.call("ps_jit_compile", src.encode(), b"ps_jit_entry", ctypes.byref(h))
        kernel._handles[key] = h
    h = kernel._handles[key]
    alld = descs + sdescs
    A = (PSArray * len(alld))(*alld)
    S = (ctypes.c_double * max(1, len(scal)))(*[float(x) for x in scal])
    _lib.call("ps_jit_launch_ex", h, A, len(alld), S, len(scal), (ctypes.c_int64 * 3)(*lo),
              (ctypes.c_int64 * 3)(*cnt), (ctypes.c_int32 * 3)(*threads), 0, (ctypes.c_int32 * 3)(1, 1, 1),
              stream_handle(stream), int(bool(sync)))
