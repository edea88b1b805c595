"""Kernel definitions (in ParallelStencil.jl's kernel language) shared by the run-time compilation
tests. They are written for these tests: each one exercises a group of features the translator
has to get right, with array sizes chosen so that every read of a thread inside its statement's
`@within` mask is inside its array."""

# 3-D heat step with on-the-fly fluxes (test/test_parallel.jl:411-434 tests this form)
HEAT_FLUX = """@parallel function heat_flux_step!(Tnew, Told, Cinv, λ::Data.Number, Δt::Data.Number, rdx, rdy, rdz)
    @all(fx)   = -λ*@d_xi(Told)*rdx           # on-the-fly arrays (not arguments)
    @all(fy)   = -λ*@d_yi(Told)*rdy
    @all(fz)   = -λ*@d_zi(Told)*rdz
    @all(rate) = @inn(Cinv)*(-@d_xa(fx)*rdx - @d_ya(fy)*rdy - @d_za(fz)*rdz)
    @inn(Tnew) = @inn(Told) + Δt*@all(rate)
    return
end"""

# 3-D heat step, second differences (test/test_parallel.jl:521-563 tests this form)
HEAT_LAP = """@parallel function heat_step!(Tnew, Told, Cinv, λ, Δt, rdx, rdy, rdz)
    @inn(Tnew) = @inn(Told) + Δt*(λ*@inn(Cinv)*(@d2_xi(Told)*rdx^2 + @d2_yi(Told)*rdy^2 + @d2_zi(Told)*rdz^2))
    return
end"""

# the same with divisions (examples/diffusion3D_novis_noperf.jl:10-13 is this form)
HEAT_DIV = """@parallel function heat_div_step!(Tnew, Told, Cinv, lam, dt, dx, dy, dz)
    @inn(Tnew) = @inn(Told) + dt*(lam*@inn(Cinv)*(@d2_xi(Told)/dx^2 + @d2_yi(Told)/dy^2 + @d2_zi(Told)/dz^2))
    return
end"""

# 2-D staggered viscous stresses: @av, face differences, temporaries read by the same thread
STRESS2D = """@parallel function stress2d!(Sxx, Syy, Sxy, divV, Vx, Vy, Eta, rdx::Data.Number, rdy::Data.Number)
    @all(divV) = @d_xa(Vx)*rdx + @d_ya(Vy)*rdy
    @all(Sxx)  = 2.0*@all(Eta)*(@d_xa(Vx)*rdx - 1.0/3.0*@all(divV))
    @all(Syy)  = 2.0*@all(Eta)*(@d_ya(Vy)*rdy - 1.0/3.0*@all(divV))
    @all(Sxy)  = 2.0*@av(Eta)*(0.5*(@d_yi(Vx)*rdy + @d_xi(Vy)*rdx))
    return
end"""

# 2-D momentum residuals with @av_yi and damped rates
MOMENTUM2D = """@parallel function momentum2d!(Rx, Ry, dVx, dVy, P, Sxx, Syy, Sxy, Rho, rdx, rdy, g, damp)
    @all(Rx)  = @d_xi(Sxx)*rdx + @d_ya(Sxy)*rdy - @d_xi(P)*rdx
    @all(Ry)  = @d_yi(Syy)*rdy + @d_xa(Sxy)*rdx - @d_yi(P)*rdy - g*@av_yi(Rho)
    @all(dVx) = damp*@all(dVx) + @all(Rx)
    @all(dVy) = damp*@all(dVy) + @all(Ry)
    return
end"""

# 2-D velocity update on inner points with harmonic means and a local maximum
VELOCITY2D = """@parallel function velocity2d!(Vx, Vy, dVx, dVy, Eta, Emax, h)
    @all(Emax) = @maxloc(Eta)
    @inn(Vx)   = @inn(Vx) + h/@harm_xi(Eta)*@all(dVx)
    @inn(Vy)   = @inn(Vy) + h/@harm_yi(Eta)*@all(dVy)
    return
end"""

# 2-D heat diffusion with FiniteDifferences2D macros (the y sweep of memopt 2-D)
HEAT2D_FD = """@parallel function heat2d_fd!(T2, T, Ci, lam, dt, _dx, _dy)
    @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx*_dx + @d2_yi(T)*_dy*_dy))
    return
end"""

# compound assignments on array elements (Julia lowers `a op= b` to `a = a op b`)
AUGASSIGN = """@parallel_indices (ix) function augassign!(A, B, a)
    A[ix] += a * B[ix] * 100.65
    A[ix] -= 1.5
    A[ix] *= 2
    A[ix] /= 3
    return
end"""

# module-qualified FD macros and the memopt options of a 2-D y sweep
QUALIFIED2D = """@parallel ndims=2 memopt=true optvars=B loopdim=2 loopsize=3 function qualified2d!(A2, B)
    FiniteDifferences2D.@inn(A2) = FiniteDifferences2D.@d2_yi(B)
    return
end"""

# an index tuple of any rank: (I...) with A[I...], for 2-D and 3-D arrays (ndims=(2,3))
SPLAT_COPY = """@parallel_indices (I...) ndims=(2,3) N=ndims function splat_copy!(B::Data.Array{T,N}, A::Data.Array{T,N}, c::T) where {T}
    B[I...] = c * A[I...]
    return
end"""

# a @sharedMem view at a byte offset given with sizeof(eltype(A))
SMEM_OFFSET = """@parallel_indices (ix,iy) function smem_offset!(B, A)
    tx  = @threadIdx().x
    ty  = @threadIdx().y
    A_l = @sharedMem(eltype(A), (@blockDim().x, @blockDim().y), 2*@blockDim().x*sizeof(eltype(A)))
    A_l[tx,ty] = A[ix,iy]
    @sync_threads()
    B[ix,iy] = A_l[@blockDim().x+1-tx,ty]
    return
end"""

# a one-line local function, inlined at its call (test/ParallelKernel/test_parallel.jl)
LOCAL_FN = """@parallel_indices (ix,iy,iz) function write_indices!(A)
    compute_indices(A) = return ix + (iy-1)*size(A,1) + (iz-1)*size(A,1)*size(A,2)
    A[ix,iy,iz] = compute_indices(A)
    return
end"""

# an Int expression stored into a real array: computed as Int, converted once (as Julia does)
INT_EXPR2D = """@parallel_indices (ix, iy) function int_expr2d!(A)
    A[ix, iy] = ix + (iy - 1) * size(A, 1)
    return
end"""

# 2-D first-order upwind advection: explicit indices, chained comparisons, Bool * x
UPWIND2D = """@parallel_indices (i, j) function upwind2d!(Tn, T, u, w, dt, rdx, rdy)
    if (1 < i < size(T, 1) && 1 < j < size(T, 2))
        Tn[i, j] = T[i, j] - dt*((u[i, j] > 0)*u[i, j]*(T[i, j] - T[i-1, j])*rdx +
                                 (u[i, j] < 0)*u[i, j]*(T[i+1, j] - T[i, j])*rdx +
                                 (w[i, j] > 0)*w[i, j]*(T[i, j] - T[i, j-1])*rdy +
                                 (w[i, j] < 0)*w[i, j]*(T[i, j+1] - T[i, j])*rdy)
    end
    return
end"""

# 2-D insulated side walls: `end` inside indices, one index over the second dimension's range
WALLS2D = """@parallel_indices (j) function walls2d!(T)
    T[1, j]   = T[2, j]
    T[end, j] = T[end-1, j]
    return
end"""

# power-law permeability and exponential compaction (math library calls)
COMPACTION = """@parallel function compaction!(Phi, K, Pe, phi0::Data.Number, n::Data.Number, lam::Data.Number)
    @all(K)   = (@all(Phi)/phi0)^n
    @all(Phi) = @all(Phi)*exp(-lam*@all(Pe))
    return
end"""

# 3-D mixed operators: corner averages, harmonic and local maximum, second differences
BLEND3D = """@parallel function blend3d!(Out, Q, B, D, s::Data.Number)
    @all(Out) = @av_xyi(B) - s*@harm_zi(D) + @maxloc(B)*@d2_yi(D) + @av(Q)*@d_za(B)
    return
end"""

# 3-D partial inner selection on the left-hand side
FACES3D = """@parallel function faces3d!(W, B, D, s)
    @inn_yz(W) = @inn_yz(B) + s*@av_za(D)
    return
end"""

# 1-D rod
ROD1D = """@parallel function rod1d!(U2, U, k)
    @inn(U2) = @inn(U) + k*@d2(U)
    return
end"""

# thread indices inside a @parallel body (test/test_parallel.jl:402-410 uses ParallelStencil.INDICES)
LINEAR_INDEX = """@parallel function linear_index!(A)
    @all(A) = $ix + ($iy-1)*size(A,1) + ($iz-1)*size(A,1)*size(A,2)
    return
end"""

# elseif / else chains, ifelse, max/min, abs, integer scalar exponent
BRANCHES2D = """@parallel_indices (ix, iy) inbounds=false function branches2d!(B, A, c::Integer, t)
    if A[ix, iy] > t
        B[ix, iy] = max(A[ix, iy], t) - abs(A[ix, iy])^c
    elseif A[ix, iy] < -t
        B[ix, iy] = min(A[ix, iy], -t) + ifelse(ix > iy, one(t), zero(t))
    else
        B[ix, iy] = sqrt(abs(A[ix, iy]))*(iy == 1 || ix == size(A, 1))
    end
    return
end"""

# 3-D explicit-index second difference along z (test/test_parallel.jl:466-479 tests this form)
D2Z3D = """@parallel_indices (ix, iy, iz) memopt=true loopsize=3 function d2z3d!(A2, A)
    if (iz > 1 && iz < size(A2, 3))
        A2[ix, iy, iz] = A[ix, iy, iz+1] - 2*A[ix, iy, iz] + A[ix, iy, iz-1]
    end
    return
end"""

# reads one element past the end for the last thread (Julia raises a BoundsError)
SHIFT_OOB = """@parallel_indices (i) function shift!(B, A)
    B[i] = A[i+1]
    return
end"""

# the same kernel compiled without bounds checks is only ever launched over safe ranges
SHIFT_INBOUNDS = """@parallel_indices (i) inbounds=true function shift_inb!(B, A)
    B[i] = A[i+1]
    return
end"""

# ---- kernel language (src/ParallelKernel/kernel_language.jl): blocks, shared memory, warps

# 2-D heat step staged through a shared-memory tile with a one-cell halo, the pattern of
# examples/diffusion2D_shmem_novis.jl (here with the barrier outside any branch)
HEAT2D_TILE = """@parallel_indices (ix, iy) function heat2d_tile!(T2, T, Ci, lam, dt, rdx, rdy)
    tx = @threadIdx().x + 1
    ty = @threadIdx().y + 1
    Tl = @sharedMem(eltype(T), (@blockDim().x + 2, @blockDim().y + 2))
    Tl[tx, ty] = T[ix, iy]
    if (ix > 1 && @threadIdx().x == 1) Tl[tx-1, ty] = T[ix-1, iy] end
    if (ix < size(T, 1) && @threadIdx().x == @blockDim().x) Tl[tx+1, ty] = T[ix+1, iy] end
    if (iy > 1 && @threadIdx().y == 1) Tl[tx, ty-1] = T[ix, iy-1] end
    if (iy < size(T, 2) && @threadIdx().y == @blockDim().y) Tl[tx, ty+1] = T[ix, iy+1] end
    @sync_threads()
    if (1 < ix < size(T2, 1) && 1 < iy < size(T2, 2))
        T2[ix, iy] = Tl[tx, ty] + dt*Ci[ix, iy]*lam*((Tl[tx+1, ty] - 2.0*Tl[tx, ty] + Tl[tx-1, ty])*rdx*rdx +
                                                    (Tl[tx, ty+1] - 2.0*Tl[tx, ty] + Tl[tx, ty-1])*rdy*rdy)
    end
    return
end"""

# the same step without shared memory (the reference value for the tile kernel)
HEAT2D_PLAIN = """@parallel_indices (ix, iy) function heat2d_plain!(T2, T, Ci, lam, dt, rdx, rdy)
    if (1 < ix < size(T2, 1) && 1 < iy < size(T2, 2))
        T2[ix, iy] = T[ix, iy] + dt*Ci[ix, iy]*lam*((T[ix+1, iy] - 2.0*T[ix, iy] + T[ix-1, iy])*rdx*rdx +
                                                   (T[ix, iy+1] - 2.0*T[ix, iy] + T[ix, iy-1])*rdy*rdy)
    end
    return
end"""

# butterfly sum of each warp's 32 values (every lane ends with the same sum)
WARP_SUMS = """@parallel_indices (i) function warp_sums!(S, A)
    v = A[i]
    o = 16
    while o >= 1
        v = v + @shfl_xor_sync(0xffffffff, v, o)
        o = o ÷ 2
    end
    if @laneid() == 1
        S[(i - 1) ÷ 32 + 1] = v
    end
    return
end"""

# broadcasts, shifts within 16-lane partitions, votes and ballots
WARP_OPS = """@parallel_indices (i) function warp_ops!(B, C, D, A, t)
    v = A[i]
    first = @shfl_sync(0xffffffff, v, 1)
    up = @shfl_up_sync(0xffffffff, v, 1)
    down = @shfl_down_sync(0xffffffff, v, 2, 16)
    anyhi = @vote_any_sync(0xffffffff, v > t)
    allhi = @vote_all_sync(0xffffffff, v > -t)
    bal = @vote_ballot_sync(0xffffffff, v > 0)
    B[i] = first + up*anyhi - down
    C[i] = allhi*1.0 + (bal % 1024)
    D[i] = @laneid() + 100*@warpsize()
    return
end"""

# loops and local variables: a box filter along x of half-width w
BOX_X = """@parallel_indices (ix, iy) function box_x!(B, A, w::Integer)
    s = 0.0
    c = 0
    for k = max(1, ix - w):min(size(A, 1), ix + w)
        s = s + A[k, iy]
        c = c + 1
    end
    B[ix, iy] = s / c
    return
end"""

# block and thread coordinates of a 3-D launch
BLOCK_IDS = """@parallel_indices (ix, iy, iz) function block_ids!(A)
    A[ix, iy, iz] = @blockIdx().x + 10*@blockIdx().y + 100*@blockIdx().z +
                    1000*(@threadIdx().x + @threadIdx().y*@blockDim().x) + 0.5*@gridDim().z
    return
end"""

# an early `return` inside a branch ends the thread
EARLY_RETURN = """@parallel_indices (i) function clip_tail!(B, A, m::Integer)
    if i > m
        return
    end
    B[i] = 2.0*A[i]
    return
end"""

# two statements along z: the second reads (at its own index) what the first wrote, which the z
# sweep must never carry in a register
TWO3D = """@parallel function two3d!(A, C, B, s)
    @all(A) = @d_za(B)*s + @av_zi(B)
    @inn(C) = @inn(C) + @all(A)*@d2_zi(B)
    return
end"""
