"""Initialisation, `Data` types, allocators and device-array plumbing.

Python mirror of the reference's user-facing setup (names and argument meaning kept):
  - ``init_parallel_stencil(package, numbertype, ndims; memopt)``  <- ``@init_parallel_stencil``
    (src/init_parallel_stencil.jl:20-51); the package is ``GB300``.
  - ``Data.Number`` / ``Data.Array``  <- the Data module (src/ParallelKernel/Data.jl:246-280).
  - ``zeros/ones/rand/fill/fill_``  <- ``@zeros/@ones/@rand/@fill/@fill!``
    (src/ParallelKernel/allocators.jl:279-375; on CUDA ``@rand`` draws on the host and copies,
    CUDAExt/allocators.jl:5 -- the same is done here with a seeded numpy generator).

Device arrays are torch CUDA tensors in Julia (column-major) layout: shape ``(nx, ny, nz)`` with
strides ``(1, nx, nx*ny)``, so ``A[ix, iy, iz]`` (0-based) is the reference's
``A[ix+1, iy+1, iz+1]``. torch only provides the memory and streams; every kernel is a
libps_b200.so entry point.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import PSArray, PSError

GB300 = "GB300"
SUPPORTED_PACKAGES = (GB300,)
SUPPORTED_NDIMS = (1, 2, 3)
_NUMBERTYPES = {"Float64": np.float64, "Float32": np.float32, np.float64: np.float64, np.float32: np.float32,
                "float64": np.float64, "float32": np.float32}


class ArgumentError(ValueError):
    """Invalid argument (the reference's `ArgumentError`)."""


class NotInitializedError(RuntimeError):
    """`init_parallel_stencil` was not called (src/ParallelKernel/Exceptions.jl)."""


class _State:
    initialized = False
    package = None
    numbertype = None
    ndims = None
    memopt = False
    device = 0


_state = _State()


def _torch():
    import torch

    return torch


def _torch_dtype(numbertype):
    torch = _torch()
    return torch.float64 if np.dtype(numbertype) == np.float64 else torch.float32


class Data:
    """`Data.Number` and `Data.Array` of the initialised module."""

    Number = None

    @staticmethod
    def Array(host) -> "torch.Tensor":  # noqa: F821
        """`Data.Array(host_array)`: copy a host array (Julia layout) to the device."""
        return from_host(np.asarray(host, dtype=Data.Number))


def init_parallel_stencil(package=GB300, numbertype="Float64", ndims=3, *, memopt=False, inbounds=False,
                          padding=False, device=0) -> None:
    """Initialise the GB300 backend: select and initialise the device and set `Data`."""
    if _state.initialized:
        if (package, _NUMBERTYPES.get(numbertype), ndims, memopt) != (_state.package, _state.numbertype, _state.ndims,
                                                                       _state.memopt):
            raise ArgumentError("ParallelStencil has already been initialized with different arguments; "
                                "call reset_parallel_stencil() first")
        return
    if package not in SUPPORTED_PACKAGES:
        raise ArgumentError(f"unsupported package type (obtained: {package}); supported: {SUPPORTED_PACKAGES}")
    if numbertype not in _NUMBERTYPES:
        raise ArgumentError(f"unsupported numbertype {numbertype!r} (Float64 or Float32)")
    if ndims not in SUPPORTED_NDIMS:
        raise ArgumentError(f"ndims must be one of {SUPPORTED_NDIMS} (obtained: {ndims})")
    if not isinstance(memopt, bool):
        raise ArgumentError("memopt must be of type Bool")
    if padding:
        raise ArgumentError("padding=true is not supported by the GB300 package")
    _lib.call("ps_init", int(device))
    _torch().cuda.set_device(device)
    _state.package, _state.numbertype, _state.ndims, _state.memopt = package, _NUMBERTYPES[numbertype], ndims, memopt
    _state.device = device
    _state.initialized = True
    Data.Number = _state.numbertype


def is_initialized() -> bool:
    return _state.initialized


def reset_parallel_stencil() -> None:
    _state.initialized = False
    _state.package = _state.numbertype = _state.ndims = None
    _state.memopt = False
    Data.Number = None


def require_initialized() -> None:
    if not _state.initialized:
        raise NotInitializedError("init_parallel_stencil has not been called")


def default_memopt() -> bool:
    return _state.memopt


# ---------------------------------------------------------------------------------------
# Device arrays
# ---------------------------------------------------------------------------------------
def _size3(size):
    size = tuple(int(s) for s in size)
    if not 1 <= len(size) <= 3 or any(s < 1 for s in size):
        raise ArgumentError(f"invalid array size {size}")
    return size


def empty(*size, dtype=None):
    """Uninitialised device array of Julia layout (column-major)."""
    require_initialized()
    torch = _torch()
    if len(size) == 1 and isinstance(size[0], (tuple, list)):
        size = tuple(size[0])
    size = _size3(size)
    strides, acc = [], 1
    for s in size:
        strides.append(acc)
        acc *= s
    dt = _torch_dtype(dtype or _state.numbertype)
    return torch.empty_strided(size, tuple(strides), dtype=dt, device=f"cuda:{_state.device}")


def empty_like(A):
    """Uninitialised device array with the size, layout and element type of A."""
    torch = _torch()
    return torch.empty_strided(tuple(A.shape), tuple(A.stride()), dtype=A.dtype, device=A.device)


def zeros_like(A):
    Z = empty_like(A)
    fill_(Z, 0.0)
    return Z


def zeros(*size, dtype=None):
    """`@zeros(size...)`."""
    A = empty(*size, dtype=dtype)
    fill_(A, 0.0)
    return A


def ones(*size, dtype=None):
    """`@ones(size...)`."""
    A = empty(*size, dtype=dtype)
    fill_(A, 1.0)
    return A


def fill(value, *size, dtype=None):
    """`@fill(value, size...)`."""
    A = empty(*size, dtype=dtype)
    fill_(A, value)
    return A


def fill_(A, value) -> None:
    """`@fill!(A, value)`."""
    _lib.call("ps_fill", descriptor(A), float(value), None)


def rand(*size, dtype=None, seed=0):
    """`@rand(size...)`: uniform(0,1) drawn on the host with a seeded generator, then copied."""
    if len(size) == 1 and isinstance(size[0], (tuple, list)):
        size = tuple(size[0])
    dt = dtype or _state.numbertype
    host = np.random.default_rng(seed).random(size, dtype=np.float64).astype(dt)
    return from_host(np.asfortranarray(host))


def from_host(a: np.ndarray):
    """Copy a host numpy array (Julia layout) into a new device array."""
    require_initialized()
    a = np.asfortranarray(a)
    if a.dtype not in (np.float64, np.float32):
        raise ArgumentError(f"unsupported element type {a.dtype}")
    A = empty(*a.shape, dtype=a.dtype.type)
    torch = _torch()
    A.copy_(torch.from_numpy(a))
    return A


def to_host(A) -> np.ndarray:
    """`Array(A)`: copy a device array to a host numpy array (Julia layout)."""
    t = A.detach().cpu()
    return np.asfortranarray(t.numpy())


def dtype_code(dtype) -> int:
    torch = _torch()
    if dtype in (torch.float64, np.float64):
        return _lib.PS_F64
    if dtype in (torch.float32, np.float32):
        return _lib.PS_F32
    raise ArgumentError(f"unsupported element type {dtype}")


def is_column_major(shape, strides) -> bool:
    acc = 1
    for s, st in zip(shape, strides):
        if s != 1 and st != acc:
            return False
        acc *= s
    return True


def descriptor(A) -> PSArray:
    """ps_array descriptor of a device array (dense, column-major, float64/float32)."""
    if A is None:
        return PSArray(None, (ctypes.c_int64 * 3)(1, 1, 1), _lib.PS_F64, 0)
    if not getattr(A, "is_cuda", False):
        raise ArgumentError("kernel arguments must be device arrays (Data.Array)")
    shape = tuple(A.shape)
    if not 1 <= len(shape) <= 3:
        raise ArgumentError(f"arrays must have 1 to 3 dimensions (obtained {len(shape)})")
    if not is_column_major(shape, A.stride()):
        raise ArgumentError("arrays must be dense and column-major (Julia layout); use ps_gb300.zeros/Data.Array")
    n = list(shape) + [1] * (3 - len(shape))
    return PSArray(A.data_ptr(), (ctypes.c_int64 * 3)(*n), dtype_code(A.dtype), 0)


def stream_handle(stream=None):
    """Raw cudaStream_t of a torch stream (default: the current stream)."""
    if stream is None:
        return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


def synchronize(stream=None) -> None:
    """`@synchronize()` / `@synchronize(stream)`."""
    _lib.call("ps_synchronize", stream_handle(stream))


__all__ = ["GB300", "Data", "init_parallel_stencil", "is_initialized", "reset_parallel_stencil", "zeros", "ones",
           "rand", "fill", "fill_", "empty", "from_host", "to_host", "descriptor", "synchronize", "PSError",
           "ArgumentError", "NotInitializedError"]
