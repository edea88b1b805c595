"""
    ParallelStencilGB300

The `:GB300` package of ParallelStencil.jl: `@parallel` kernels of the reference's examples and
miniapps (diffusion3D in its three statement forms and with a conductivity array, memcopy3D,
acoustic3D, the Stokes2D kernels and free-slip copies) and every one-statement FiniteDifferences
kernel run as the hand-written sm_103a kernels of libps_b200.so, called through its C ABI
(`include/ps_gb300.h`). There is no CUDA.jl kernel generation, no multi-backend dispatch and no
CPU fallback on that path: a definition the package does not recognise is an error at definition
time.

Usage -- the examples' call sites stay as they are; only the package changes:

    using ParallelStencilGB300                      # instead of `using ParallelStencil`
    using ParallelStencil.FiniteDifferences3D
    @init_parallel_stencil(GB300, Float64, 3)
    @parallel function diffusion3D_step!(T2, T, Ci, lam, dt, dx, dy, dz) ... end
    @parallel diffusion3D_step!(T2, T, Ci, lam, dt, dx, dy, dz)

`@init_parallel_stencil(GB300, T, N)` initialises ParallelStencil with CUDA.jl device arrays
(`Data.Array{N}` = `CuArray{T,N}`: libps_b200.so works on them in place), `ps_init` on the task's
device, and registers `:GB300` in `ParallelStencil.ParallelKernel.SUPPORTED_PACKAGES`
(src/ParallelKernel/shared.jl:24). Allocators (`@zeros`, `@ones`, `@rand`, `@fill`) are
ParallelStencil's. `@parallel`, `@parallel_async`, `@parallel_indices` and `@hide_communication`
are this package's: a definition is matched against the library's kernels (`recognise`), a call
lowers to the matching `ccall`.

Not run on the machines this package was written on: they have no Julia toolchain. The `ccall`
signatures are checked against `include/ps_gb300.h` by the repository's host tests, and the same
kernels are exercised through the Python mirror of this interface (`ps_gb300`).
"""
module ParallelStencilGB300

using CUDA
using MacroTools: MacroTools, isexpr
using ParallelStencil

include("LibPS.jl")
using .LibPS

"""A `@parallel` definition recognised as one of libps_b200.so's kernels."""
struct GB300Kernel
    name::Symbol
    kind::Symbol
    form::Int
    fd::LibPS.PSFdOp
    lhs_inn::Int32
    nargs::Int
end
(k::GB300Kernel)(args...) = throw(ArgumentError("$(k.name) is a GB300 kernel: launch it with @parallel $(k.name)(...)"))

include("recognise.jl")

const GB300 = :GB300
const NDIMS = Dict{Module,Int}()

export @init_parallel_stencil, @parallel, @parallel_async, @parallel_indices, @hide_communication, GB300
export @zeros, @ones, @rand, @fill, @synchronize, ParallelStencil
export diffusion3d_step, diffusion3d_misfit

macro zeros(args...) esc(:(ParallelStencil.@zeros($(args...)))) end
macro ones(args...) esc(:(ParallelStencil.@ones($(args...)))) end
macro rand(args...) esc(:(ParallelStencil.@rand($(args...)))) end
macro fill(args...) esc(:(ParallelStencil.@fill($(args...)))) end
macro synchronize(args...) :(LibPS.synchronize($(map(esc, args)...))) end

function __init__()
    build_templates!()
    pk = ParallelStencil.ParallelKernel
    GB300 in pk.SUPPORTED_PACKAGES || push!(pk.SUPPORTED_PACKAGES, GB300)
end

"""
    @init_parallel_stencil(GB300, numbertype, ndims)

ParallelStencil's initialisation with CUDA.jl arrays, then `ps_init` on the current device.
"""
macro init_parallel_stencil(package, numbertype, ndims, kwargs...)
    package === :GB300 || throw(ArgumentError("ParallelStencilGB300 initialises the GB300 package (obtained $package)"))
    NDIMS[__module__] = ndims
    quote
        ParallelStencil.@init_parallel_stencil(CUDA, $numbertype, $ndims, $(kwargs...))
        ParallelStencilGB300.LibPS.init(CUDA.deviceid(CUDA.device()))
    end |> esc
end

ndims_of(m::Module) = get(NDIMS, m, 3)

# split `@parallel [ranges] [kw=val ...] call` into (positional, keywords, call)
function split_call(args)
    pos, kw = Any[], Dict{Symbol,Any}()
    for a in args[1:end-1]
        isexpr(a, :(=)) ? (kw[a.args[1]] = a.args[2]) : push!(pos, a)
    end
    return pos, kw, args[end]
end

"""
    @parallel function k!(args...) ... end       # definition: recognised at expansion time
    @parallel [ranges] [memopt=...] [stream=...] k!(args...)   # call: the matching ccall

src/parallel.jl:192-277 (definitions and calls); `ranges` as in
src/ParallelKernel/parallel.jl:303-315 (1-based UnitRanges).
"""
macro parallel(args...)
    parallel_gateway(__module__, args; async = false)
end
macro parallel_async(args...)
    parallel_gateway(__module__, args; async = true)
end

function parallel_gateway(caller::Module, args; async::Bool)
    pos, kw, last = split_call(args)
    if isexpr(last, :function) || (isexpr(last, :(=)) && isexpr(last.args[1], :call))
        nd = get(kw, :ndims, ndims_of(caller))
        k = recognise(last, nd)
        return esc(:(const $(k.name) = $k))
    end
    isexpr(last, :call) || throw(ArgumentError("@parallel: expected a kernel definition or a kernel call"))
    ranges = isempty(pos) ? nothing : pos[1]
    memopt = get(kw, :memopt, false)
    stream = get(kw, :stream, :(CUDA.stream()))
    kernel, cargs = last.args[1], last.args[2:end]
    return esc(:(ParallelStencilGB300.launch($kernel, $(cargs...); ranges = $ranges, memopt = $memopt,
                                             stream = $stream, sync = $(!async))))
end

"""
    @parallel_indices (ix, iy) function k!(A) ... end

The free-slip copies of the Stokes miniapps (bc_x!, bc_y!) are recognised; any other
`@parallel_indices` body goes through the run-time compiled path.
"""
macro parallel_indices(indices, def)
    k = recognise(def, ndims_of(__module__); indices = Tuple(isexpr(indices, :tuple) ? indices.args : (indices,)))
    esc(:(const $(k.name) = $k))
end

# ---- lowering of calls ------------------------------------------------------------------------
function launch(k::GB300Kernel, args...; ranges = nothing, memopt = false, stream = CUDA.stream(), sync = true)
    length(args) == k.nargs || throw(ArgumentError("$(k.name): expected $(k.nargs) arguments, obtained $(length(args))"))
    cfg = LibPS.launch_cfg(; memopt = Bool(memopt), ranges = ranges)
    if k.kind === :copy3D
        LibPS.memcopy3d!(args..., cfg; stream, sync)
    elseif k.kind === :diffusion
        LibPS.diffusion3d_step!(k.form, args..., cfg; stream, sync)
    elseif k.kind === :acoustic_V
        ranges === nothing || throw(ArgumentError("$(k.name): explicit ranges are not supported"))
        LibPS.acoustic3d_v!(args...; stream, sync)
    elseif k.kind === :acoustic_P
        ranges === nothing || throw(ArgumentError("$(k.name): explicit ranges are not supported"))
        LibPS.acoustic3d_p!(args...; stream, sync)
    elseif k.kind === :fd
        ranges === nothing || throw(ArgumentError("$(k.name): explicit ranges are not supported"))
        LibPS.fd_apply!(k.fd, k.lhs_inn, args[1], args[2]; stream, sync)
    elseif k.kind === :bc_x2d
        LibPS.bc_x2d!(args[1]; stream, sync)
    elseif k.kind === :bc_y2d
        LibPS.bc_y2d!(args[1]; stream, sync)
    elseif k.kind in (:s2_timesteps, :s2_P, :s2_tau, :s2_dV, :s2_V)
        ranges === nothing || throw(ArgumentError("$(k.name): explicit ranges are not supported"))
        stokes2d_call(k.kind, args; stream, sync)
    else
        throw(ArgumentError("$(k.name): unknown GB300 kernel kind $(k.kind)"))
    end
    return nothing
end

# The Stokes2D entry points take the miniapp's whole field set; a kernel call supplies the arrays
# it uses and the others are stand-ins of the right shape (never read or written by that kernel).
const STANDINS = Dict{Tuple{DataType,Int,Int},NamedTuple}()

function stokes2d_standins(::Type{T}, nx, ny) where {T}
    get!(STANDINS, (T, nx, ny)) do
        z(s...) = CUDA.zeros(T, s...)
        (Pt = z(nx, ny), dtauPt = z(nx, ny), divV = z(nx, ny), Vx = z(nx + 1, ny), Vy = z(nx, ny + 1), txx = z(nx, ny),
         tyy = z(nx, ny), txy = z(nx - 1, ny - 1), Rx = z(nx - 1, ny - 2), Ry = z(nx - 2, ny - 1),
         dVxdtau = z(nx - 1, ny - 2), dVydtau = z(nx - 2, ny - 1), dtauVx = z(nx - 1, ny - 2),
         dtauVy = z(nx - 2, ny - 1), Mus = z(nx, ny), Rog = z(nx, ny))
    end
end

function stokes2d_call(kind::Symbol, a; stream, sync)
    if kind === :s2_timesteps     # (dτVx, dτVy, dτPt, Mus, Vsc, Ptsc, min_dxy2, max_nxy)
        T, (nx, ny) = eltype(a[4]), size(a[4])
        given = (dtauVx = a[1], dtauVy = a[2], dtauPt = a[3], Mus = a[4])
        p = LibPS.Stokes2DParams(1.0, 1.0, 0.0, 0.0, a[5], a[6], a[7], Int64(a[8]))
        LibPS.stokes2d_timesteps!(fields2d(T, nx, ny, given), p; stream, sync)
    elseif kind === :s2_P         # (∇V, Pt, Vx, Vy, dτPt, dx, dy)
        T, (nx, ny) = eltype(a[2]), size(a[2])
        given = (divV = a[1], Pt = a[2], Vx = a[3], Vy = a[4], dtauPt = a[5])
        LibPS.stokes2d_compute_P!(fields2d(T, nx, ny, given), params2d(a[6], a[7]); stream, sync)
    elseif kind === :s2_tau       # (∇V, τxx, τyy, τxy, Vx, Vy, Mus, dx, dy)
        T, (nx, ny) = eltype(a[2]), size(a[2])
        given = (divV = a[1], txx = a[2], tyy = a[3], txy = a[4], Vx = a[5], Vy = a[6], Mus = a[7])
        LibPS.stokes2d_compute_tau!(fields2d(T, nx, ny, given), params2d(a[8], a[9]); stream, sync)
    elseif kind === :s2_dV        # (Rx, Ry, dVxdτ, dVydτ, Pt, Rog, τxx, τyy, τxy, dampX, dampY, dx, dy)
        T, (nx, ny) = eltype(a[5]), size(a[5])
        given = (Rx = a[1], Ry = a[2], dVxdtau = a[3], dVydtau = a[4], Pt = a[5], Rog = a[6], txx = a[7], tyy = a[8],
                 txy = a[9])
        p = LibPS.Stokes2DParams(a[12], a[13], a[10], a[11], 0.0, 0.0, 0.0, 0)
        LibPS.stokes2d_compute_dV!(fields2d(T, nx, ny, given), p; stream, sync)
    else                          # (Vx, Vy, dVxdτ, dVydτ, dτVx, dτVy)
        T, nx, ny = eltype(a[1]), size(a[1], 1) - 1, size(a[1], 2)
        given = (Vx = a[1], Vy = a[2], dVxdtau = a[3], dVydtau = a[4], dtauVx = a[5], dtauVy = a[6])
        LibPS.stokes2d_compute_V!(fields2d(T, nx, ny, given), params2d(1.0, 1.0); stream, sync)
    end
end

params2d(dx, dy) = LibPS.Stokes2DParams(dx, dy, 0.0, 0.0, 0.0, 0.0, 0.0, 0)
fields2d(::Type{T}, nx, ny, given::NamedTuple) where {T} =
    LibPS.Stokes2DFields(merge(stokes2d_standins(T, nx, ny), given))

"""
    @hide_communication boundary_width begin
        @parallel diffusion3D_step!(T2, T, Ci, lam, dt, dx, dy, dz)
        update_halo!(T2)            # any statements: run once the boundary slabs are done
    end

src/ParallelKernel/hide_communication.jl:177-258: the six boundary slabs run on a high-priority
stream, the statements after the kernel call run as the communication callback, the inner box
runs on a second stream; both are synchronised on return (`ps_diffusion3d_step_split`).
"""
macro hide_communication(bw, block)
    stmts = filter(s -> !(s isa LineNumberNode), isexpr(block, :block) ? block.args : Any[block])
    first_stmt = stmts[1]
    (isexpr(first_stmt, :macrocall) && first_stmt.args[1] === Symbol("@parallel")) ||
        throw(ArgumentError("@hide_communication: the block must start with a @parallel diffusion kernel call"))
    call = first_stmt.args[end]
    kw = Dict{Symbol,Any}(a.args[1] => a.args[2] for a in first_stmt.args[3:end-1] if isexpr(a, :(=)))
    memopt = get(kw, :memopt, true)
    comm = :(() -> begin $(stmts[2:end]...); nothing end)
    esc(:(ParallelStencilGB300.hide_communication($bw, $(call.args[1]), $comm, $(call.args[2:end]...);
                                                  memopt = $memopt)))
end

function hide_communication(bw, k::GB300Kernel, comm, args...; memopt = true)
    k.kind === :diffusion || throw(ArgumentError("@hide_communication: $(k.name) is not a diffusion kernel"))
    cfg = LibPS.launch_cfg(; memopt = Bool(memopt))
    LibPS.diffusion3d_step_split!(k.form, args..., cfg, bw, comm)
    return nothing
end

# ---- whole solves and runs that have no single `@parallel` call in the reference ---------------
"""
    diffusion3d_run!(k, T, T2, Ci, lam, dt, dx, dy, dz, nt; fp64_mode = LibPS.PS_FP64_SPLIT_GRID)

The examples' time loop `for it = 1:nt; @parallel k(T2, T, ...); T, T2 = T2, T; end` as one call
(examples/diffusion3D_novis_noperf.jl:43-46); on return T holds the state after nt steps.
"""
diffusion3d_run!(k::GB300Kernel, T, T2, Ci, lam, dt, dx, dy, dz, nt; fp64_mode = LibPS.PS_FP64_SPLIT_GRID,
                 stream = CUDA.stream()) =
    LibPS.diffusion3d_run!(k.form, T, T2, Ci, lam, dt, dx, dy, dz, nt,
                           LibPS.launch_cfg(; memopt = true, fp64_mode = fp64_mode); stream)

"""
    diffusion3d_step(T, Ci, lam, dt, _dx, _dy, _dz) -> T2

One step of the flux form with a conductivity array (PS_DIFF_FLUX_LAM) into a new array: inner
cells updated, boundary cells copied from T (Dirichlet data). Differentiable in the inner cells of
T and in lam: the ChainRules extension gives its `rrule` (pullback: the hand-written adjoint step;
boundary cells get a zero cotangent).
"""
function diffusion3d_step(T, Ci, lam, dt, _dx, _dy, _dz; memopt = true)
    T2 = copy(T)
    LibPS.diffusion3d_step!(3, T2, T, Ci, lam, dt, _dx, _dy, _dz, LibPS.launch_cfg(; memopt = Bool(memopt)))
    return T2
end

"""
    diffusion3d_misfit(T0, T_obs, Ci, lam, dt, _dx, _dy, _dz, nt; checkpoint_every = 20) -> L

L = 0.5 ||T_nt - T_obs||^2 after nt flux-lam steps from T0. Differentiable in lam: the ChainRules
extension's `rrule` returns dL/dlam from the checkpointed adjoint (ps_diffusion3d_misfit_gradient).
"""
function diffusion3d_misfit(T0, T_obs, Ci, lam, dt, _dx, _dy, _dz, nt; checkpoint_every = 20,
                            fp64_mode = LibPS.PS_FP64_IEEE)
    g = similar(lam)
    cfg = LibPS.launch_cfg(; memopt = true, fp64_mode = fp64_mode)
    return LibPS.misfit_gradient!(g, T0, T_obs, Ci, lam, dt, _dx, _dy, _dz, nt, checkpoint_every, cfg).loss
end

end # module ParallelStencilGB300
