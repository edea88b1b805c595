"""The memopt kernels of the reference's test suite (test/test_parallel.jl:437-800: copies, second
differences along y and z, the diffusion step in explicit-index, FD-macro and on-the-fly forms,
shifted higher-order stencils over one and three arrays, staggered second arrays), run-time
compiled and launched with memopt=true, against the expected arrays those tests build with
broadcasting -- restated here with numpy slices in the same operation order. Inputs are the tests'
`(ix + (iy-1) nx + (iz-1) nx ny)^3` fields (times 1, 2, 3), so every value is an integer below
2^53 and the bar is exact equality, as in the reference. Grid sizes: the tests' (32, 8, 8) and
the ragged (33, 7, 8) and (31, 7, 9) their comments list. The 2-D testset (:1084-1195: y second
differences in index and FD-macro form, a mixed x/y stencil over two arrays, optranges, loopsize
and optimize_halo_read) runs the same way at (32, 8), (33, 7) and (300, 131)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(32, 8, 8), (33, 7, 8), (31, 7, 9), (36, 7, 8)]  # (36, 7, 8): ragged, with 16-byte FP64 rows

# FP64 kernels run the register sweep by default; "always" runs them staged by TMA where the rows
# allow it ((32, 8, 8) and (36, 7, 8)), so the reference's memopt kernels check both schedules
STAGED = {"tma": True}


@pytest.fixture(autouse=True, params=[True, "always"], ids=["sweep", "tma"])
def _schedule(request):
    STAGED["tma"] = request.param
    yield
    STAGED["tma"] = True


def cube(shape, scale=1.0):
    n = int(np.prod(shape))
    return np.asfortranarray(scale * np.arange(1, n + 1, dtype=np.float64).reshape(shape, order="F") ** 3)


def _run(ps, src, arrays, scalars=()):
    dev = [ps.from_host(np.asfortranarray(a)) for a in arrays]
    k = ps.parallel_kernel(src)
    k.tma = STAGED["tma"]
    ps.parallel(k, *dev, *scalars, memopt=True)
    k.tma = True
    return [ps.to_host(d) for d in dev]


COPY_IDX = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 optvars=A optranges=(A=(0:0,0:0,0:0),) function copy_memopt!(A2, A)
    A2[ix,iy,iz] = A[ix,iy,iz]
    return
end"""

COPY_FD = """@parallel memopt=true loopsize=3 optvars=A optranges=(A=(0:0,0:0,0:0),) function copy_memopt!(A2, A)
    @all(A2) = @all(A)
    return
end"""

COPY2_FD = """@parallel memopt=true loopsize=3 optvars=(A, B) optranges=(A=(0:0,0:0,0:0), B=(0:0,0:0,0:0)) function copy_memopt!(A2, A, B)
    @all(A2) = @all(A) + @all(B)
    return
end"""

D2Z_IDX = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 function d2_memopt!(A2, A)
    if (iz>1 && iz<size(A2,3))
        A2[ix,iy,iz] = A[ix,iy,iz+1] - 2*A[ix,iy,iz] + A[ix,iy,iz-1]
    end
    return
end"""

D2Y_IDX = """@parallel_indices (ix,iy,iz) memopt=true function d2_memopt!(A2, A)
    if (iy>1 && iy<size(A2,2))
        A2[ix,iy,iz] = A[ix,iy+1,iz] - 2*A[ix,iy,iz] + A[ix,iy-1,iz]
    end
    return
end"""

D2ZI_FD = """@parallel memopt=true loopsize=3 function d2_memopt!(A2, A)
    @inn(A2) = @d2_zi(A)
    return
end"""

D2YI_FD = """@parallel memopt=true loopsize=3 function d2_memopt!(A2, A)
    @inn(A2) = @d2_yi(A)
    return
end"""

DIFF_IDX = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    if (1<ix<size(T2,1) && 1<iy<size(T2,2) && 1<iz<size(T2,3))
        T2[ix,iy,iz] = T[ix,iy,iz] + dt*(Ci[ix,iy,iz]*(
                        - ((-lam*(T[ix+1,iy,iz] - T[ix,iy,iz])*_dx) - (-lam*(T[ix,iy,iz] - T[ix-1,iy,iz])*_dx))*_dx
                        - ((-lam*(T[ix,iy+1,iz] - T[ix,iy,iz])*_dy) - (-lam*(T[ix,iy,iz] - T[ix,iy-1,iz])*_dy))*_dy
                        - ((-lam*(T[ix,iy,iz+1] - T[ix,iy,iz])*_dz) - (-lam*(T[ix,iy,iz] - T[ix,iy,iz-1])*_dz))*_dz)
                        );
    end
    return
end"""

DIFF_FD = """@parallel memopt=true loopsize=3 function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))
    return
end"""

DIFF_OTF = """@parallel memopt=true loopsize=3 function diffusion3D_step!(T2, T, Ci, lam::Data.Number, dt, _dx, _dy, _dz)
    @all(qx)   = -lam*@d_xi(T)*_dx
    @all(qy)   = -lam*@d_yi(T)*_dy
    @all(qz)   = -lam*@d_zi(T)*_dz
    @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz)
    @inn(T2)   = @inn(T) + dt*@all(dTdt)
    return
end"""

HIGHER = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 function higher_order_memopt!(A2, A)
    if (ix-4>1 && ix-1<size(A2,1) && iy+2>1 && iy+2<=size(A2,2) && iz-2>=1 && iz+3<=size(A2,3))
        A2[ix-1,iy+2,iz] = A[ix-1,iy+2,iz+3] - 2*A[ix-3,iy+2,iz] + A[ix-4,iy+2,iz-2]
    end
    return
end"""

HIGHER3 = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 function higher_order_memopt!(A2, B2, C2, A, B, C)
    if (ix-4>1 && ix-1<size(A2,1) && iy+2>1 && iy+2<=size(A2,2) && iz-2>=1 && iz+3<=size(A2,3))
        A2[ix-1,iy+2,iz] = A[ix-1,iy+2,iz+3] - 2*A[ix-3,iy+2,iz] + A[ix-4,iy+2,iz-2]
    end
    if (ix-4>1 && ix-1<size(B2,1) && iy+2>1 && iy+2<=size(B2,2) && iz+1>=1 && iz+2<=size(B2,3))
        B2[ix-1,iy+2,iz+1] = B[ix-1,iy+2,iz+2] - 2*B[ix-3,iy+2,iz+1] + B[ix-4,iy+2,iz+1]
    end
    if (ix-4>1 && ix-1<size(C2,1) && iy+2>1 && iy+2<=size(C2,2) && iz-1>=1 && iz<=size(C2,3))
        C2[ix-1,iy+2,iz-1] = C[ix-1,iy+2,iz] - 2*C[ix-3,iy+2,iz-1] + C[ix-4,iy+2,iz-1]
    end
    return
end"""

TWO_Z = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 function d2_memopt!(A2, A, B)
    if (iz>1 && iz<size(A2,3))
        A2[ix,iy,iz] = A[ix,iy,iz+1] - 2*A[ix,iy,iz] + A[ix,iy,iz-1] + B[ix,iy,iz] - B[ix,iy,iz-1]
    end
    return
end"""

TWO_Y = """@parallel_indices (ix,iy,iz) memopt=true loopsize=3 function d2_memopt!(A2, A, B)
    if (iy>1 && iy<size(A2,2))
        A2[ix,iy,iz] = A[ix,iy+1,iz] - 2*A[ix,iy,iz] + A[ix,iy-1,iz] + B[ix,iy+1,iz] - 2*B[ix,iy,iz] + B[ix,iy-1,iz]
    end
    return
end"""

TWO_X = """@parallel_indices (ix,iy,iz) memopt=true function d2_memopt!(A2, A, B)
    if (ix>1 && ix<size(A2,1))
        A2[ix,iy,iz] = A[ix+1,iy,iz] - 2*A[ix,iy,iz] + A[ix-1,iy,iz] + B[ix,iy,iz] - B[ix-1,iy,iz]
    end
    return
end"""

MOD_Z = """@parallel memopt=true loopsize=3 function diffusion3D_step_modified!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    @inn(T2) = @inn(T) + dt*(lam*@d_zi(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))
    return
end"""

MOD_X = """@parallel memopt=true loopsize=3 function diffusion3D_step_modified!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    @inn(T2) = @inn(T) + dt*(lam*@d_xi(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))
    return
end"""

MOD3 = """@parallel memopt=true loopsize=3 function diffusion3D_step_modified!(T2, T, Ci, B, lam, dt, _dx, _dy, _dz)
    @inn(T2) = @inn(T) + dt*(lam*@d_xi(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2)) + @d2_yi(B)
    return
end"""

I = slice(1, -1)  # Julia 2:end-1


def _lap(T):
    """The three second differences of the inner points, as @d2_xi, @d2_yi, @d2_zi."""
    c = T[I, I, I]
    return ((T[2:, I, I] - c) - (c - T[:-2, I, I]), (T[I, 2:, I] - c) - (c - T[I, :-2, I]),
            (T[I, I, 2:] - c) - (c - T[I, I, :-2]))


@pytest.mark.parametrize("n", SIZES)
def test_memopt_copies(ps, n):
    A = cube(n)
    for src in (COPY_IDX, COPY_FD):
        A2, _ = _run(ps, src, [np.zeros(n), A])
        assert np.array_equal(A2, A)
    B = cube(n, 2.0)
    A2, _, _ = _run(ps, COPY2_FD, [np.zeros(n), A, B])
    assert np.array_equal(A2, A + B)


@pytest.mark.parametrize("n", SIZES)
def test_memopt_second_differences(ps, n):
    A = cube(n)
    for src, axis in ((D2Z_IDX, 2), (D2Y_IDX, 1)):
        A2, _ = _run(ps, src, [np.zeros(n), A])
        ref = np.zeros(n)
        sl = [slice(None)] * 3
        hi, mid, lo = list(sl), list(sl), list(sl)
        hi[axis], mid[axis], lo[axis] = slice(2, None), I, slice(None, -2)
        ref[tuple(mid)] = A[tuple(hi)] - 2 * A[tuple(mid)] + A[tuple(lo)]
        assert np.array_equal(A2, ref), src
    for src, k in ((D2ZI_FD, 2), (D2YI_FD, 1)):
        A2, _ = _run(ps, src, [np.zeros(n), A])
        ref = np.zeros(n)
        ref[I, I, I] = _lap(A)[k]
        assert np.array_equal(A2, ref), src


@pytest.mark.parametrize("n", SIZES)
def test_memopt_diffusion_forms(ps, n):
    T, Ci = cube(n), np.asfortranarray(np.ones(n))
    one = (1.0, 1.0, 1.0, 1.0, 1.0)  # lam, dt, _dx, _dy, _dz
    c = T[I, I, I]
    d2x, d2y, d2z = _lap(T)
    # explicit indices: - ((-lam*(T+ - T)*_dx) - (-lam*(T - T-)*_dx))*_dx - ... (all scalars 1)
    fx = -((-(T[2:, I, I] - c)) - (-(c - T[:-2, I, I])))
    fy = ((-(T[I, 2:, I] - c)) - (-(c - T[I, :-2, I])))
    fz = ((-(T[I, I, 2:] - c)) - (-(c - T[I, I, :-2])))
    ref = np.zeros(n)
    ref[I, I, I] = c + (Ci[I, I, I] * (fx - fy - fz))
    T2, *_ = _run(ps, DIFF_IDX, [np.zeros(n), T, Ci], one)
    assert np.array_equal(T2, ref)
    ref = np.zeros(n)
    ref[I, I, I] = c + (Ci[I, I, I] * ((d2x + d2y) + d2z))
    T2, *_ = _run(ps, DIFF_FD, [np.zeros(n), T, Ci], one)
    assert np.array_equal(T2, ref)
    # on the fly: q = -lam*d(T)*_d, dTdt = Ci*(-d(qx)*_dx - d(qy)*_dy - d(qz)*_dz)
    qx, qy, qz = -(T[1:, I, I] - T[:-1, I, I]), -(T[I, 1:, I] - T[I, :-1, I]), -(T[I, I, 1:] - T[I, I, :-1])
    ref = np.zeros(n)
    ref[I, I, I] = c + Ci[I, I, I] * ((-(qx[1:] - qx[:-1]) - (qy[:, 1:] - qy[:, :-1])) - (qz[:, :, 1:] - qz[:, :, :-1]))
    T2, *_ = _run(ps, DIFF_OTF, [np.zeros(n), T, Ci], one)
    assert np.array_equal(T2, ref)


@pytest.mark.parametrize("n", SIZES)
def test_memopt_shifted_higher_order(ps, n):
    A, B, C = cube(n), cube(n, 2.0), cube(n, 3.0)
    A2, _ = _run(ps, HIGHER, [np.zeros(n), A])
    ref = np.zeros(n)
    ref[4:-1, 2:, 2:-3] = A[4:-1, 2:, 5:] - 2 * A[2:-3, 2:, 2:-3] + A[1:-4, 2:, :-5]
    assert np.array_equal(A2, ref)
    A2, B2, C2, *_ = _run(ps, HIGHER3, [np.zeros(n), np.zeros(n), np.zeros(n), A, B, C])
    ra, rb, rc = np.zeros(n), np.zeros(n), np.zeros(n)
    ra[4:-1, 2:, 2:-3] = A[4:-1, 2:, 5:] - 2 * A[2:-3, 2:, 2:-3] + A[1:-4, 2:, :-5]
    rb[4:-1, 2:, 1:-1] = B[4:-1, 2:, 2:] - 2 * B[2:-3, 2:, 1:-1] + B[1:-4, 2:, 1:-1]
    rc[4:-1, 2:, :-1] = C[4:-1, 2:, 1:] - 2 * C[2:-3, 2:, :-1] + C[1:-4, 2:, :-1]
    assert np.array_equal(A2, ra) and np.array_equal(B2, rb) and np.array_equal(C2, rc)


@pytest.mark.parametrize("n", SIZES)
def test_memopt_two_and_three_arrays(ps, n):
    A = cube(n)
    nx, ny, nz = n
    # @XXYYZField: (nx, ny, nz-1); @XYYZZField: (nx-1, ny, nz) (padding=false)
    Bz, Bx, By = cube((nx, ny, nz - 1), 2.0), cube((nx - 1, ny, nz), 2.0), cube(n, 2.0)
    A2, *_ = _run(ps, TWO_Z, [np.zeros(n), A, Bz])
    ref = np.zeros(n)
    ref[:, :, I] = A[:, :, 2:] - 2 * A[:, :, I] + A[:, :, :-2] + Bz[:, :, 1:] - Bz[:, :, :-1]
    assert np.array_equal(A2, ref)
    A2, *_ = _run(ps, TWO_Y, [np.zeros(n), A, By])
    ref = np.zeros(n)
    ref[:, I, :] = (((A[:, 2:] - 2 * A[:, I]) + A[:, :-2] + By[:, 2:]) - 2 * By[:, I]) + By[:, :-2]
    assert np.array_equal(A2, ref)
    A2, *_ = _run(ps, TWO_X, [np.zeros(n), A, Bx])
    ref = np.zeros(n)
    ref[I] = A[2:] - 2 * A[I] + A[:-2] + Bx[1:] - Bx[:-1]
    assert np.array_equal(A2, ref)
    T, c = A, A[I, I, I]
    lap = _lap(T)
    s = (lap[0] + lap[1]) + lap[2]
    for src, Ci, dC in ((MOD_Z, Bz, lambda C: C[I, I, 1:] - C[I, I, :-1]), (MOD_X, Bx, lambda C: C[1:, I, I] - C[:-1, I, I])):
        T2, *_ = _run(ps, src, [np.zeros(n), T, Ci], (1.0,) * 5)
        ref = np.zeros(n)
        ref[I, I, I] = c + (dC(Ci) * s)
        assert np.array_equal(T2, ref), src
    B3 = cube(n, 3.0)
    T2, *_ = _run(ps, MOD3, [np.zeros(n), T, Bx, B3], (1.0,) * 5)
    ref = np.zeros(n)
    ref[I, I, I] = c + ((Bx[1:, I, I] - Bx[:-1, I, I]) * s) + _lap(B3)[1]
    assert np.array_equal(T2, ref)


# ---------------------------------------------------------------- 2-D (test/test_parallel.jl:1084-1195)
D2Y_2D_IDX = """@parallel_indices (ix, iy) ndims=2 memopt=true loopdim=2 function d2_memopt_indices!(A2, A)
    if (1 < iy < size(A2, 2))
        A2[ix, iy] = A[ix, iy + 1] - 2 * A[ix, iy] + A[ix, iy - 1]
    end
    return
end"""

D2YI_2D_FD = """@parallel ndims=2 memopt=true optvars=B loopdim=2 function d2_memopt_kernel!(A2, B)
    @inn(A2) = @d2_yi(B)
    return
end"""

MIXED_2D = """@parallel_indices (ix, iy) ndims=2 memopt=true loopdim=2 optvars=A function mixed_memopt_indices!(A2, A, B)
    if (1 < ix < size(A2, 1) && 1 < iy < size(A2, 2))
        A2[ix, iy] = (A[ix, iy + 1] - 2 * A[ix, iy] + A[ix, iy - 1]) + (B[ix + 1, iy] - 2 * B[ix, iy] + B[ix - 1, iy])
    end
    return
end"""

RANGED_2D = """@parallel_indices (ix, iy) ndims=2 memopt=true loopdim=2 optvars=A optranges=(A=(0:0, -1:1, 0:0),) function ranged_memopt_indices!(A2, A)
    if (1 < iy < size(A2, 2))
        A2[ix, iy] = A[ix, iy + 1] - 2 * A[ix, iy] + A[ix, iy - 1]
    end
    return
end"""

LOOP4_2D = """@parallel_indices (ix, iy) ndims=2 memopt=true loopdim=2 loopsize=4 function loopsize_memopt_indices!(A2, A)
    if (1 < iy < size(A2, 2))
        A2[ix, iy] = A[ix, iy + 1] - 2 * A[ix, iy] + A[ix, iy - 1]
    end
    return
end"""

HALO_2D = """@parallel_indices (ix, iy) ndims=2 memopt=true loopdim=2 optvars=A optranges=(A=(0:0, -1:1, 0:0),) optimize_halo_read=false function halo_read_memopt_indices!(A2, A)
    if (1 < iy < size(A2, 2))
        A2[ix, iy] = A[ix, iy + 1] - 2 * A[ix, iy] + A[ix, iy - 1]
    end
    return
end"""


def cube2(shape):
    n = int(np.prod(shape))
    return np.asfortranarray(np.arange(1, n + 1, dtype=np.float64).reshape(shape, order="F") ** 3)


@pytest.mark.parametrize("n", [(32, 8), (33, 7), (300, 131)])
def test_memopt_2d_cases(ps, n):
    """The 2-D memopt kernels (y sweeps for the `@parallel` one), exact against the tests' broadcast
    expectations, at the tests' (32, 8), a ragged size and one with several blocks per dimension."""
    A = cube2(n)
    ref = np.zeros(n)
    ref[:, 1:-1] = A[:, 2:] - 2 * A[:, 1:-1] + A[:, :-2]
    for src in (D2Y_2D_IDX, RANGED_2D, LOOP4_2D, HALO_2D):
        A2, _ = _run(ps, src, [np.zeros(n), A])
        assert np.array_equal(A2, ref), src[:60]
    A2, _ = _run(ps, D2YI_2D_FD, [np.zeros(n), A])
    r2 = np.zeros(n)
    r2[1:-1, 1:-1] = A[1:-1, 2:] - 2 * A[1:-1, 1:-1] + A[1:-1, :-2]
    # @d2_yi is (B[y+1] - B) - (B - B[y-1]); the expectation's `B+ - 2B + B-` is the same integer
    assert np.array_equal(A2, r2)
    i, j = np.meshgrid(np.arange(1, n[0] + 1), np.arange(1, n[1] + 1), indexing="ij")
    B = np.asfortranarray((2 * i - j).astype(np.float64))
    A2, _, _ = _run(ps, MIXED_2D, [np.zeros(n), A, B])
    r3 = np.zeros(n)
    r3[1:-1, 1:-1] = (A[1:-1, 2:] - 2 * A[1:-1, 1:-1] + A[1:-1, :-2]) + (B[2:, 1:-1] - 2 * B[1:-1, 1:-1] + B[:-2, 1:-1])
    assert np.array_equal(A2, r3)
