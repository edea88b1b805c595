"""Edge cases of the kernels' inputs: empty arrays, the smallest grids (no or one inner cell),
ranges of zero length, and a mix of staggered extents. Empty arrays are refused with a status
(never a launch); grids without inner cells leave every value untouched."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(ps, a):
    return ps.from_host(np.asfortranarray(a))


def test_empty_arrays_are_refused_cleanly(ps):
    """An extent of 0 is refused by the allocator (ArgumentError) and by every entry point
    (PS_ERR_SHAPE), before anything is launched."""
    import ctypes

    from ps_gb300 import _lib
    from ps_gb300._lib import PSArray
    from ps_gb300.core import descriptor, stream_handle

    with pytest.raises(ps.ArgumentError):
        ps.zeros(0, 4, 4)
    A = ps.zeros(4, 4, 4)
    E = descriptor(A)
    E.n[0] = 0
    lib, s = _lib.load(), stream_handle(None)
    assert lib.ps_memcopy3d(E, E, E, None, s, 1) == -3
    assert lib.ps_fill(E, 1.0, s) == -3
    k = ps.parallel_kernel("@parallel function f!(R, A)\n @all(R) = @all(A)\n return\nend")
    h = k._handle(3, "double")
    arrs = (PSArray * 2)(E, descriptor(A))
    assert lib.ps_jit_launch(h, arrs, 2, (ctypes.c_double * 1)(0.0), 0, (ctypes.c_int64 * 3)(0, 0, 0),
                             (ctypes.c_int64 * 3)(4, 4, 4), s, 1) == -3
    assert "extent" in _lib.last_error()
    ps.parallel(ps.kernels.copy3D, A, A, A)  # nothing was launched; the context is fine


@pytest.mark.parametrize("n", [(1, 1, 1), (2, 2, 2), (3, 3, 3), (3, 4, 5), (5, 3, 3), (64, 3, 3), (3, 3, 70)])
@pytest.mark.parametrize("memopt", [False, True])
def test_smallest_grids_match_the_oracle(ps, oracle, n, memopt):
    rng = np.random.default_rng(sum(n))
    T = np.asfortranarray(rng.random(n))
    Ci = np.asfortranarray(rng.random(n) + 0.5)
    lam = np.asfortranarray(rng.random(n) + 1.0)
    sc = (1e-3, 2.0, 3.0, 4.0)
    for form, kern in ((3, ps.kernels.diffusion3D_step_flux_lam), (2, ps.kernels.diffusion3D_step_flux),
                       (0, ps.kernels.diffusion3D_step)):
        ref = T.copy(order="F")
        args = (lam, 0.0) if form == 3 else (None, 0.7)
        oracle.diffusion3d_step(form, ref, T, Ci, *args, *sc)
        T2 = _dev(ps, T)
        lam_arg = _dev(ps, lam) if form == 3 else 0.7
        ps.parallel(kern, T2, _dev(ps, T), _dev(ps, Ci), lam_arg, *sc, memopt=memopt)
        got = ps.to_host(T2)
        assert np.array_equal(got, ref), (form, n)
        if min(n) < 3:
            assert np.array_equal(got, T)  # no inner cell: nothing is written


def test_zero_length_ranges_do_nothing(ps):
    src = "@parallel_indices (i, j) function one!(A)\n A[i, j] = 1.0\n return\nend"
    A = ps.zeros(8, 8)
    ps.parallel(ps.parallel_kernel(src), A, ranges=[(3, 2), (1, 8)])
    assert not ps.to_host(A).any()
    ps.parallel(ps.parallel_kernel(src), A, ranges=[(3, 3), (1, 8)])
    assert ps.to_host(A).sum() == 8


def test_staggered_extents_share_one_grid(ps, oracle):
    """@all(R) = @d_xa(A) with R one shorter in x than A: the grid spans the larger extent and the
    mask keeps R's last x plane (and everything past it) untouched."""
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.random((9, 7, 8)))
    R0 = np.asfortranarray(np.full((8, 7, 8), -3.0))
    k = ps.fd_kernel("@inn_yz(R) = @d_xi(A)")
    R = _dev(ps, R0)
    ps.parallel(k, R, _dev(ps, A))
    exp = R0.copy(order="F")
    exp[:, 1:-1, 1:-1] = A[1:, 1:-1, 1:-1] - A[:-1, 1:-1, 1:-1]
    assert np.array_equal(ps.to_host(R), exp)
