"""ctypes binding of libps_b200.so (the C ABI declared in include/ps_gb300.h).

The library must have been built (``parallelstencil.jl_gb300/build.py``); loading fails loudly
otherwise -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("PS_B200_LIB", os.path.join(_PKG_ROOT, "lib", "libps_b200.so"))

PS_OK = 0
STATUS_NAMES = {
    0: "PS_OK", -1: "PS_ERR_ARG", -2: "PS_ERR_NULL", -3: "PS_ERR_SHAPE", -4: "PS_ERR_DTYPE", -5: "PS_ERR_ALIGN",
    -6: "PS_ERR_CUDA", -7: "PS_ERR_NOT_CONVERGED", -8: "PS_ERR_TIMEOUT", -9: "PS_ERR_NOT_INIT",
    -10: "PS_ERR_NOMEM", -11: "PS_ERR_NONFINITE", -12: "PS_ERR_UNSUPPORTED",
}
PS_F64, PS_F32, PS_BF16 = 0, 1, 2


class PSError(RuntimeError):
    """A libps_b200 call returned a non-zero status (the reference raises a typed exception)."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class PSArray(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("n", ctypes.c_int64 * 3), ("dtype", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class PSLaunch(ctypes.Structure):
    _fields_ = [("memopt", ctypes.c_int32), ("loopsize", ctypes.c_int32), ("range_lo", ctypes.c_int64 * 3),
                ("range_hi", ctypes.c_int64 * 3), ("fp64_mode", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class PSFdOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("opdims", ctypes.c_int32), ("inn", ctypes.c_int32),
                ("ndims", ctypes.c_int32)]


COMM_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p)

_A = PSArray
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64

# name -> argtypes (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    "ps_init": [_I],
    "ps_finalize": [],
    "ps_last_error": [],
    "ps_abi_version": [],
    "ps_device_count": [ctypes.POINTER(_I)],
    "ps_check_division": [_D, _I32, _I64, ctypes.c_uint64, ctypes.POINTER(_I64), _P],
    "ps_alloc": [ctypes.POINTER(_A), _I32, _I64, _I64, _I64],
    "ps_free": [ctypes.POINTER(_A)],
    "ps_fill": [_A, _D, _P],
    "ps_copy_h2d": [_A, _P, _P],
    "ps_copy_d2h": [_P, _A, _P],
    "ps_copy_h2d_async": [_A, _P, _P],
    "ps_copy_d2h_async": [_P, _A, _P],
    "ps_copy_d2d_async": [_A, _A, _P],
    "ps_stream_create": [_I, ctypes.POINTER(_P)],
    "ps_stream_destroy": [_P],
    "ps_synchronize": [_P],
    "ps_fd_apply": [PSFdOp, _I32, _A, _A, _P, _I],
    "ps_memcopy3d": [_A, _A, _A, ctypes.POINTER(PSLaunch), _P, _I],
    "ps_diffusion3d_step": [_I32, _A, _A, _A, _A, _D, _D, _D, _D, _D, ctypes.POINTER(PSLaunch), _P, _I],
    "ps_diffusion3d_step_split": [_I32, _A, _A, _A, _A, _D, _D, _D, _D, _D, ctypes.POINTER(PSLaunch),
                                  ctypes.POINTER(_I64), _P, _P,
                                  COMM_FN, _P],
    "ps_acoustic3d_v": [_A, _A, _A, _A, _D, _D, _D, _D, _D, _P, _I],
    "ps_acoustic3d_p": [_A, _A, _A, _A, _D, _D, _D, _D, _D, _P, _I],
    "ps_acoustic3d_step": [_A] * 8 + [_D] * 6 + [_I32, _P, _I],
    "ps_acoustic3d_run": [_A] * 4 + [_D] * 6 + [_I64, _I32, _P],
}
_RESTYPES = {"ps_last_error": ctypes.c_char_p}

_lib = None


def load() -> ctypes.CDLL:
    """Load libps_b200.so and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libps_b200.so not built ({LIB_PATH}); run parallelstencil.jl_gb300/build.py")
    lib = ctypes.CDLL(LIB_PATH)
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = _RESTYPES.get(name, ctypes.c_int)
    _lib = lib
    return lib


def register(name: str, argtypes, restype=ctypes.c_int) -> None:
    """Declare an additional entry point (used by submodules that extend the ABI)."""
    SIGNATURES[name] = argtypes
    if restype is not ctypes.c_int:
        _RESTYPES[name] = restype
    if _lib is not None:
        fn = getattr(_lib, name)
        fn.argtypes = argtypes
        fn.restype = restype


def last_error() -> str:
    msg = load().ps_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    if rc != PS_OK:
        raise PSError(rc, last_error())


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
