"""FiniteDifferences{1,2,3}D macros as ps_fd_op descriptors, and one-statement FD kernels.

Each macro of src/FiniteDifferences.jl is a descriptor ``(kind, opdims, inn)``:
  kind    SEL / DIFF / DIFF2 / AV / HARM / MAXLOC / MINLOC
  opdims  bit mask (x=1, y=2, z=4) of the dimensions it differences / averages over
  inn     bit mask of the dimensions whose base index is the inner index ``ixi = ix+1``
e.g. ``@d_xi`` (src/FiniteDifferences.jl:331) reads ``A[ix+1,iyi,izi] - A[ix,iyi,izi]``, so it is
``(DIFF, x, y|z)``. ``fd_kernel("@inn(R) = @d2_yi(A)")`` builds the one-statement ``@parallel``
kernel that ``ps_fd_apply`` runs.
"""
from __future__ import annotations

import re
from dataclasses import dataclass

from . import _lib
from .core import ArgumentError, descriptor, stream_handle

SEL, DIFF, DIFF2, AV, HARM, MAXLOC, MINLOC = range(7)
X, Y, Z = 1, 2, 4


def _table3():
    XYZ = X | Y | Z
    t = {
        "d_xa": (DIFF, X, 0), "d_ya": (DIFF, Y, 0), "d_za": (DIFF, Z, 0),
        "d_xi": (DIFF, X, Y | Z), "d_yi": (DIFF, Y, X | Z), "d_zi": (DIFF, Z, X | Y),
        "d2_xi": (DIFF2, X, XYZ), "d2_yi": (DIFF2, Y, XYZ), "d2_zi": (DIFF2, Z, XYZ),
        "all": (SEL, 0, 0), "inn": (SEL, 0, XYZ), "inn_x": (SEL, 0, X), "inn_y": (SEL, 0, Y), "inn_z": (SEL, 0, Z),
        "inn_xy": (SEL, 0, X | Y), "inn_xz": (SEL, 0, X | Z), "inn_yz": (SEL, 0, Y | Z),
        "maxloc": (MAXLOC, XYZ, XYZ), "minloc": (MINLOC, XYZ, XYZ),
    }
    for kind, pre in ((AV, "av"), (HARM, "harm")):
        t[pre] = (kind, XYZ, 0)
        t[pre + "_xa"], t[pre + "_ya"], t[pre + "_za"] = (kind, X, 0), (kind, Y, 0), (kind, Z, 0)
        t[pre + "_xi"], t[pre + "_yi"], t[pre + "_zi"] = (kind, X, Y | Z), (kind, Y, X | Z), (kind, Z, X | Y)
        t[pre + "_xya"], t[pre + "_xza"], t[pre + "_yza"] = (kind, X | Y, 0), (kind, X | Z, 0), (kind, Y | Z, 0)
        t[pre + "_xyi"], t[pre + "_xzi"], t[pre + "_yzi"] = (kind, X | Y, Z), (kind, X | Z, Y), (kind, Y | Z, X)
    return t


def _table2():
    XY = X | Y
    t = {
        "d_xa": (DIFF, X, 0), "d_ya": (DIFF, Y, 0), "d_xi": (DIFF, X, Y), "d_yi": (DIFF, Y, X),
        "d2_xa": (DIFF2, X, X), "d2_ya": (DIFF2, Y, Y), "d2_xi": (DIFF2, X, XY), "d2_yi": (DIFF2, Y, XY),
        "all": (SEL, 0, 0), "inn": (SEL, 0, XY), "inn_x": (SEL, 0, X), "inn_y": (SEL, 0, Y),
        "maxloc": (MAXLOC, XY, XY), "minloc": (MINLOC, XY, XY),
    }
    for kind, pre in ((AV, "av"), (HARM, "harm")):
        t[pre] = (kind, XY, 0)
        t[pre + "_xa"], t[pre + "_ya"] = (kind, X, 0), (kind, Y, 0)
        t[pre + "_xi"], t[pre + "_yi"] = (kind, X, Y), (kind, Y, X)
    return t


def _table1():
    return {"d": (DIFF, X, 0), "d2": (DIFF2, X, X), "all": (SEL, 0, 0), "inn": (SEL, 0, X), "av": (AV, X, 0),
            "harm": (HARM, X, 0), "maxloc": (MAXLOC, X, X), "minloc": (MINLOC, X, X)}


MACROS = {1: _table1(), 2: _table2(), 3: _table3()}

# Left-hand selections accepted by `@within` (src/FiniteDifferences.jl:397-408): name -> inn mask.
LHS = {
    1: {"all": 0, "inn": X},
    2: {"all": 0, "inn": X | Y, "inn_x": X, "inn_y": Y},
    3: {"all": 0, "inn": X | Y | Z, "inn_x": X, "inn_y": Y, "inn_z": Z, "inn_xy": X | Y, "inn_xz": X | Z,
        "inn_yz": Y | Z},
}

_STMT = re.compile(r"^\s*@(\w+)\(\s*(\w+)\s*\)\s*=\s*@(\w+)\(\s*(\w+)\s*\)\s*;?\s*$")


@dataclass(frozen=True)
class FdKernel:
    """`@parallel f!(R, A) = (@<lhs>(R) = @<op>(A); return)` for one FD macro."""

    ndims: int
    lhs: str
    op: str

    @property
    def descriptor(self) -> _lib.PSFdOp:
        kind, opdims, inn = MACROS[self.ndims][self.op]
        return _lib.PSFdOp(kind, opdims, inn, self.ndims)

    @property
    def lhs_inn(self) -> int:
        return LHS[self.ndims][self.lhs]

    def launch(self, R, A, stream=None, sync=True) -> None:
        _lib.call("ps_fd_apply", self.descriptor, self.lhs_inn, descriptor(R), descriptor(A), stream_handle(stream),
                  int(bool(sync)))

    @property
    def source(self) -> str:
        """The kernel as a `@parallel` definition."""
        return f"@parallel function fd!(R, A)\n    @{self.lhs}(R) = @{self.op}(A)\n    return\nend"

    def launch_split(self, R, A, stream=None, sync=True) -> None:
        """FP64 arrays, arithmetic on FP32 pairs: the definition run-time compiled with fp64="split"
        (each operation within ~2^-46 of its operands' magnitude)."""
        from .jit import parallel_kernel

        parallel_kernel(self.source, self.ndims).jit_launch((R, A), None, stream, sync, fp64="split")


def fd_kernel(statement: str, ndims: int = 3) -> FdKernel:
    """Parse a one-statement FD kernel body such as ``"@all(R) = @d_xa(A)"``."""
    m = _STMT.match(statement)
    if not m:
        raise ArgumentError("unsupported kernel statement: expected '@<sel>(R) = @<macro>(A)'")
    lhs, rname, op, aname = m.groups()
    if ndims not in MACROS:
        raise ArgumentError(f"ndims must be 1, 2 or 3 (obtained {ndims})")
    if lhs not in LHS[ndims]:
        raise ArgumentError(f"unsupported left-hand macro @{lhs} for {ndims}-D")
    if op not in MACROS[ndims]:
        raise ArgumentError(f"unknown macro @{op} in FiniteDifferences{ndims}D")
    if rname == aname:
        raise ArgumentError("the output array must differ from the input array")
    return FdKernel(ndims, lhs, op)
