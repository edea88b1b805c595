"""ps_stokes2d_iterate_static: the Stokes2D PT iteration for callers that cannot let the library
allocate device memory (their device memory belongs to their own pool allocator, or they must not
call cudaFree, which synchronises the device). Its ping-pong buffers come from a fixed 16 MiB device
array inside the library instead of cudaMalloc.

Checked through the C ABI against ps_stokes2d_iterate (same fused kernel, so the results must be
bit-identical) on two calls in a row: the shared static array keeps the first call's contents, and
the second call must not depend on them. This file is collected last on purpose, so that a run
stopping at its first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("Pt", "Vx", "Vy", "divV", "txx", "tyy", "txy", "Rx", "Ry", "dVxdtau", "dVydtau")


def _pair(ps, nx, ny, dtype=np.float64):
    from ps_gb300.stokes import Stokes2D, Stokes2DParams, inclusion_setup

    Mus, Rog = inclusion_setup(nx, ny, 1.0, 1.0, musi=0.1, dtype=dtype)
    a = Stokes2D(Stokes2DParams(nx, ny, 1.0, 1.0), Mus, Rog, dtype=dtype)
    b = Stokes2D(Stokes2DParams(nx, ny, 1.0, 1.0), Mus, Rog, dtype=dtype)
    a.compute_timesteps()
    b.compute_timesteps()
    return a, b


def _static(ps, s, n_iter):
    from ps_gb300 import _lib
    from ps_gb300.core import stream_handle

    return _lib.load().ps_stokes2d_iterate_static(ctypes.byref(s._fields), ctypes.byref(s._p), int(n_iter),
                                                   stream_handle(None))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [(63, 47), (130, 97)])
def test_static_scratch_iteration_matches_allocating_entry_point(ps, n, dtype):
    ref, new = _pair(ps, *n, dtype=dtype)
    for n_iter in (7, 6):  # two calls in a row; odd then even iteration counts
        ref.iterate(n_iter)
        assert _static(ps, new, n_iter) == 0
        for k in FIELDS:
            assert np.array_equal(new.host(k), ref.host(k)), (n, n_iter, k)
    assert np.abs(new.host("Vy")).max() > 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_static_scratch_larger_grid_then_smaller(ps, dtype):
    """The buffer offsets inside the shared array depend on the grid: a call on a smaller grid after
    one on a larger grid (the array still holding the larger call's fields) gives the allocating
    entry point's result as well."""
    for n in ((130, 97), (63, 47)):
        ref, new = _pair(ps, *n, dtype=dtype)
        for n_iter in (5, 4):
            ref.iterate(n_iter)
            assert _static(ps, new, n_iter) == 0
            for k in FIELDS:
                assert np.array_equal(new.host(k), ref.host(k)), (n, n_iter, k)


def test_static_scratch_rejects_grids_beyond_its_size(ps):
    from ps_gb300 import _lib

    ref, new = _pair(ps, 1023, 1023)  # needs ~25 MB of scratch in FP64; the array holds 16 MiB
    before = new.host("Pt")
    rc = _static(ps, new, 2)
    assert rc == -3  # PS_ERR_SHAPE
    assert "static buffer" in _lib.last_error()
    assert np.array_equal(new.host("Pt"), before)
