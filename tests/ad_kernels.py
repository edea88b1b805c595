"""Kernels differentiated by the `@parallel ∇` tests (host and GPU): name -> (source, ndims, sizes,
differentiated arguments, scalar arguments). Array arguments get seeded random values."""
import numpy as np

# the reference's own numerical AD test (test/ParallelKernel/test_parallel.jl, testset "ad numerical")
REF_F = """@parallel_indices (ix) function f!(A, B, a)
    A[ix] += a * B[ix] * 100.65
    return
end"""

KERNELS = {
    # the flux form with a conductivity array: on-the-fly fluxes, @inn output
    "diffusion_flux_lam": ("""@parallel function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    @all(qx)   = -@av_xi(lam)*@d_xi(T)*_dx
    @all(qy)   = -@av_yi(lam)*@d_yi(T)*_dy
    @all(qz)   = -@av_zi(lam)*@d_zi(T)*_dz
    @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz)
    @inn(T2)   = @inn(T) + dt*@all(dTdt)
    return
end""", 3, (9, 7, 6), ("T2", "T", "lam"), {"dt": 0.01, "_dx": 1.3, "_dy": 0.9, "_dz": 1.1}),
    # selections, @maxloc (NaN-propagating max), @harm, @d2 and a literal power
    "maxloc_harm": ("""@parallel function m!(R, A, B)
    @inn(R) = @maxloc(A) * @harm(B) + @d2_yi(A)^2
    return
end""", 3, (7, 8, 6), ("R", "A", "B"), {}),
    # two statements, the second reads what the first wrote (at the same point); a staggered array
    "two_statements_2d": ("""@parallel function s!(P, V, M, c)
    @all(P) = @all(P) - c*@av_xa(M)*@all(P)
    @all(V) = @all(V)*@all(P) + exp(@d_xa(M)) - inv(@all(M) + 2.0)
    return
end""", 2, {"*": (11, 9), "M": (12, 9)}, ("P", "V", "M"), {"c": 0.3}),
    # explicit indices, locals, if / elseif / else, an early return, math functions
    "indices_branches": ("""@parallel_indices (ix, iy) function g!(A, B, C, c)
    x = B[ix, iy] * c
    if ix > 1 && ix < size(A, 1)
        x = x + sqrt(B[ix-1, iy]) - max(C[ix+1, iy], B[ix, iy])
    elseif iy > 5
        return
    else
        x = ifelse(C[ix, iy] > 0.5, x, -x) * tanh(C[ix, iy])
    end
    A[ix, iy] = x^3 / (1.0 + abs(C[ix, iy] - 0.5)) + B[ix, iy]^c
    return
end""", 2, (10, 8), ("A", "B", "C"), {"c": 1.7}),
    # an in-place update with a neighbour read of another array (atomic shadow updates) in 3-D
    "inplace_neighbours": ("""@parallel_indices (ix, iy, iz) function h!(A, B)
    if ix < size(A, 1) && iy > 1
        A[ix, iy, iz] = A[ix, iy, iz] * B[ix+1, iy-1, iz] + log(B[ix, iy, iz] + 1.0) * B[ix+1, iy, iz]
    end
    return
end""", 3, (8, 6, 5), ("A", "B"), {}),
}


def arrays(name, dtype=np.float64, seed=0):
    """Seeded arguments of kernel `name`: arrays (positive, away from branch points) and scalars in
    argument order, with the names of the array arguments."""
    src, nd, n, dup, scal = KERNELS[name]
    head = src.split("(", 1)[1] if src.startswith("@parallel function") else src.split("function", 1)[1].split("(", 1)[1]
    argnames = [a.strip() for a in head.split(")", 1)[0].split(",")]
    rng = np.random.default_rng(seed)
    out, anames = [], []
    for a in argnames:
        if a in scal:
            out.append(scal[a])
        else:
            shape = n if isinstance(n, tuple) else n.get(a, n["*"])
            out.append(np.asfortranarray((0.5 + rng.random(shape)).astype(dtype)))
            anames.append(a)
    return argnames, out
