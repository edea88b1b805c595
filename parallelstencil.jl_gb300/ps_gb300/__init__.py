"""ps_gb300 -- Python host interface of the GB300 stencil library (libps_b200.so).

Mirrors the user-facing interface of ParallelStencil.jl for its finite-difference hot path:

    import ps_gb300 as ps
    ps.init_parallel_stencil(ps.GB300, "Float64", 3)          # @init_parallel_stencil(GB300, Float64, 3)
    T, T2, Ci = ps.zeros(nx, ny, nz), ps.zeros(nx, ny, nz), ps.ones(nx, ny, nz)
    ps.parallel(ps.kernels.diffusion3D_step, T2, T, Ci, lam, dt, dx, dy, dz)   # @parallel diffusion3D_step!(...)

Every kernel runs in libps_b200.so (hand-written sm_103a CUDA); there is no CPU or library
fallback, and a missing library raises at import of the kernels.
"""
from . import _lib, ad, adjoint, core, fd, jit, kernels, nn, stokes, stokes3d
from ._lib import PSError
from .core import (GB300, ArgumentError, Data, NotInitializedError, descriptor, empty, fill, fill_, from_host,
                   init_parallel_stencil, is_initialized, ones, rand, reset_parallel_stencil, synchronize, to_host,
                   zeros)
from .fd import fd_kernel
from .jit import parallel_kernel
from .kernels import from_source, hide_communication, parallel, parallel_async

__all__ = [
    "GB300", "ArgumentError", "Data", "NotInitializedError", "PSError", "descriptor", "empty", "fill", "fill_",
    "from_host", "init_parallel_stencil", "is_initialized", "ones", "rand", "reset_parallel_stencil", "synchronize",
    "to_host", "zeros", "fd_kernel", "from_source", "hide_communication", "parallel", "parallel_async", "kernels",
    "fd", "core", "stokes", "stokes3d", "jit", "parallel_kernel", "ad",
]
