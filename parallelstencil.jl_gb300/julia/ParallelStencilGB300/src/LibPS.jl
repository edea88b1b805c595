# LibPS -- `ccall` bindings of libps_b200.so (include/ps_gb300.h). Every struct below has the
# layout of its C counterpart; every wrapper throws with the library's message on a non-zero
# status. Arrays are CUDA.jl device arrays (dense, column-major, caller-owned), passed as
# ps_array descriptors; the stream is the task's CUDA.jl stream unless one is given.
module LibPS

using CUDA

const lib = get(ENV, "PS_GB300_LIB", normpath(joinpath(@__DIR__, "..", "..", "..", "lib", "libps_b200.so")))

# ---- descriptors (ps_array, ps_launch, ps_fd_op) ----------------------------------------
struct PSArray
    ptr::Ptr{Cvoid}
    n::NTuple{3,Int64}
    dtype::Int32
    reserved::Int32
end

struct PSLaunch
    memopt::Int32
    loopsize::Int32
    range_lo::NTuple{3,Int64}
    range_hi::NTuple{3,Int64}
    fp64_mode::Int32
    reserved::Int32
end

struct PSFdOp
    kind::Int32
    opdims::Int32
    inn::Int32
    ndims::Int32
end

const PS_F64, PS_F32 = Int32(0), Int32(1)
const PS_FP64_IEEE, PS_FP64_SPLIT, PS_FP64_SPLIT_STATE, PS_FP64_SPLIT_GRID = Int32(0), Int32(1), Int32(2), Int32(3)
const NULL_ARRAY = PSArray(C_NULL, (1, 1, 1), PS_F64, Int32(0))

dtype(::Type{Float64}) = PS_F64
dtype(::Type{Float32}) = PS_F32
dtype(::Type{T}) where {T} = throw(ArgumentError("the GB300 package supports Float64 and Float32 arrays (obtained $T)"))

desc(A::CuArray{T,N}) where {T,N} =
    PSArray(Ptr{Cvoid}(UInt(pointer(A))), ntuple(d -> d <= N ? Int64(size(A, d)) : Int64(1), 3), dtype(T), Int32(0))
desc(::Nothing) = NULL_ARRAY

stream_ptr(s = CUDA.stream()) = Ptr{Cvoid}(UInt(s.handle))

# `ranges` of a call (1-based UnitRanges, as `@parallel ranges kernel!(...)` takes them) as the
# 0-based half-open boxes of ps_launch; `nothing` = the full grid.
function launch_cfg(; memopt::Bool = false, loopsize::Integer = 0, ranges = nothing, fp64_mode::Integer = 0)
    lo, hi = (0, 0, 0), (0, 0, 0)
    if ranges !== nothing
        r = ranges isa Tuple ? ranges : (ranges,)
        lo = ntuple(d -> d <= length(r) ? Int64(first(r[d]) - 1) : Int64(0), 3)
        hi = ntuple(d -> d <= length(r) ? Int64(last(r[d])) : Int64(1), 3)
    end
    PSLaunch(Int32(memopt), Int32(loopsize), lo, hi, Int32(fp64_mode), Int32(0))
end

last_error() = unsafe_string(ccall((:ps_last_error, lib), Cstring, ()))
check(rc::Integer) = rc == 0 ? nothing : throw(ErrorException("libps_b200 (status $rc): " * last_error()))

# ---- lifetime, streams -------------------------------------------------------------------
init(device::Integer = 0) = check(ccall((:ps_init, lib), Cint, (Cint,), device))
finalize() = check(ccall((:ps_finalize, lib), Cint, ()))
abi_version() = ccall((:ps_abi_version, lib), Cint, ())
synchronize(s = CUDA.stream()) = check(ccall((:ps_synchronize, lib), Cint, (Ptr{Cvoid},), stream_ptr(s)))

function stream_create(priority::Integer)
    s = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:ps_stream_create, lib), Cint, (Cint, Ref{Ptr{Cvoid}}), priority, s))
    return s[]
end
stream_destroy(s::Ptr{Cvoid}) = check(ccall((:ps_stream_destroy, lib), Cint, (Ptr{Cvoid},), s))

# ---- FD macro kernels, memcopy, diffusion ------------------------------------------------
fd_apply!(op::PSFdOp, lhs_inn::Integer, R, A; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_fd_apply, lib), Cint, (PSFdOp, Int32, PSArray, PSArray, Ptr{Cvoid}, Cint),
                op, Int32(lhs_inn), desc(R), desc(A), stream_ptr(stream), Cint(sync)))

memcopy3d!(T2, T, Ci, cfg::PSLaunch; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_memcopy3d, lib), Cint, (PSArray, PSArray, PSArray, Ref{PSLaunch}, Ptr{Cvoid}, Cint),
                desc(T2), desc(T), desc(Ci), cfg, stream_ptr(stream), Cint(sync)))

# form: 0 = `…/dx^2`, 1 = `…*_dx^2`, 2 = on-the-fly flux (scalar lam), 3 = flux with a conductivity array
function diffusion3d_step!(form::Integer, T2, T, Ci, lam, dt, hx, hy, hz, cfg::PSLaunch; stream = CUDA.stream(),
                           sync = true)
    lam_arr, lam_s = lam isa CuArray ? (desc(lam), 0.0) : (NULL_ARRAY, Float64(lam))
    check(ccall((:ps_diffusion3d_step, lib), Cint,
                (Int32, PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble,
                 Ref{PSLaunch}, Ptr{Cvoid}, Cint),
                Int32(form), desc(T2), desc(T), desc(Ci), lam_arr, lam_s, dt, hx, hy, hz, cfg, stream_ptr(stream),
                Cint(sync)))
end

function diffusion3d_run!(form::Integer, T, T2, Ci, lam, dt, hx, hy, hz, nt::Integer, cfg::PSLaunch;
                          stream = CUDA.stream())
    lam_arr, lam_s = lam isa CuArray ? (desc(lam), 0.0) : (NULL_ARRAY, Float64(lam))
    check(ccall((:ps_diffusion3d_run, lib), Cint,
                (Int32, PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Int64,
                 Ref{PSLaunch}, Ptr{Cvoid}),
                Int32(form), desc(T), desc(T2), desc(Ci), lam_arr, lam_s, dt, hx, hy, hz, Int64(nt), cfg,
                stream_ptr(stream)))
end

# `@hide_communication bw begin @parallel step!(...); comm() end`: comm runs once the boundary
# slabs are done, while the inner box computes
const COMM = Ref{Any}(nothing)
comm_trampoline(::Ptr{Cvoid})::Cint = (COMM[](); Cint(0))
function diffusion3d_step_split!(form::Integer, T2, T, Ci, lam, dt, hx, hy, hz, cfg::PSLaunch, bw, comm)
    COMM[] = comm
    cb = comm === nothing ? C_NULL : @cfunction(comm_trampoline, Cint, (Ptr{Cvoid},))
    sb, si = stream_create(1), stream_create(0)
    lam_arr, lam_s = lam isa CuArray ? (desc(lam), 0.0) : (NULL_ARRAY, Float64(lam))
    try
        check(ccall((:ps_diffusion3d_step_split, lib), Cint,
                    (Int32, PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble,
                     Ref{PSLaunch}, Ptr{Int64}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                    Int32(form), desc(T2), desc(T), desc(Ci), lam_arr, lam_s, dt, hx, hy, hz, cfg,
                    collect(Int64.(bw)), sb, si, cb, C_NULL))
    finally
        stream_destroy(sb)
        stream_destroy(si)
    end
end

# ---- adjoint of the diffusion step (`@parallel ∇=(...)`) ---------------------------------
adjoint_step!(lamT, lamT2, T, Ci, lam, glam, dt, hx, hy, hz; fp64_mode = 0, stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_diffusion3d_adjoint_step_ex, lib), Cint,
                (PSArray, PSArray, PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Int32,
                 Ptr{Cvoid}, Cint),
                desc(lamT), desc(lamT2), desc(T), desc(Ci), desc(lam), desc(glam), dt, hx, hy, hz, Int32(fp64_mode),
                stream_ptr(stream), Cint(sync)))

struct AdjointStats
    loss::Cdouble
    checkpoints::Int64
    recomputed_steps::Int64
    seconds::Cdouble
end

function misfit_gradient!(dL_dlam, T0, T_obs, Ci, lam, dt, hx, hy, hz, nt, checkpoint_every, cfg::PSLaunch;
                          T_final = nothing, stream = CUDA.stream())
    st = Ref(AdjointStats(0.0, 0, 0, 0.0))
    check(ccall((:ps_diffusion3d_misfit_gradient, lib), Cint,
                (PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Int64, Int64, Ref{PSLaunch},
                 PSArray, PSArray, Ref{AdjointStats}, Ptr{Cvoid}),
                desc(T0), desc(T_obs), desc(Ci), desc(lam), dt, hx, hy, hz, Int64(nt), Int64(checkpoint_every), cfg,
                desc(dL_dlam), desc(T_final), st, stream_ptr(stream)))
    return st[]
end

# ---- acoustic3D ----------------------------------------------------------------------------
acoustic3d_v!(Vx, Vy, Vz, P, dt, rho, dx, dy, dz; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_acoustic3d_v, lib), Cint,
                (PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cvoid}, Cint),
                desc(Vx), desc(Vy), desc(Vz), desc(P), dt, rho, dx, dy, dz, stream_ptr(stream), Cint(sync)))
acoustic3d_p!(P, Vx, Vy, Vz, dt, k, dx, dy, dz; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_acoustic3d_p, lib), Cint,
                (PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Ptr{Cvoid}, Cint),
                desc(P), desc(Vx), desc(Vy), desc(Vz), dt, k, dx, dy, dz, stream_ptr(stream), Cint(sync)))
# both statements in one kernel, old state -> new state (fp64_mode 0 IEEE, 1 FP32 pairs on FP64 arrays)
acoustic3d_step!(Vx, Vy, Vz, P, Vx2, Vy2, Vz2, P2, dt, rho, k, dx, dy, dz; fp64_mode = 0, stream = CUDA.stream(),
                 sync = true) =
    check(ccall((:ps_acoustic3d_step, lib), Cint,
                (PSArray, PSArray, PSArray, PSArray, PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble,
                 Cdouble, Cdouble, Cdouble, Int32, Ptr{Cvoid}, Cint),
                desc(Vx), desc(Vy), desc(Vz), desc(P), desc(Vx2), desc(Vy2), desc(Vz2), desc(P2), dt, rho, k, dx, dy,
                dz, Int32(fp64_mode), stream_ptr(stream), Cint(sync)))
# the miniapp's time loop in place (acoustic3D.jl:55-56)
acoustic3d_run!(Vx, Vy, Vz, P, dt, rho, k, dx, dy, dz, nt; fp64_mode = 0, stream = CUDA.stream()) =
    check(ccall((:ps_acoustic3d_run, lib), Cint,
                (PSArray, PSArray, PSArray, PSArray, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble, Int64, Int32,
                 Ptr{Cvoid}),
                desc(Vx), desc(Vy), desc(Vz), desc(P), dt, rho, k, dx, dy, dz, Int64(nt), Int32(fp64_mode),
                stream_ptr(stream)))

# ---- Stokes2D (miniapps/Stokes2D.jl) -------------------------------------------------------
struct Stokes2DFields
    Pt::PSArray; dtauPt::PSArray; divV::PSArray; Vx::PSArray; Vy::PSArray; txx::PSArray; tyy::PSArray
    txy::PSArray; Rx::PSArray; Ry::PSArray; dVxdtau::PSArray; dVydtau::PSArray; dtauVx::PSArray
    dtauVy::PSArray; Mus::PSArray; Rog::PSArray
end
Stokes2DFields(a::NamedTuple) = Stokes2DFields((desc(getfield(a, k)) for k in fieldnames(Stokes2DFields))...)

struct Stokes2DParams
    dx::Cdouble; dy::Cdouble; dampX::Cdouble; dampY::Cdouble; Vsc::Cdouble; Ptsc::Cdouble; min_dxy2::Cdouble
    max_nxy::Int64
end

struct SolveStats
    iters::Int64
    outer::Int64
    err::Cdouble
    seconds::Cdouble
    converged::Int32
    reserved::Int32
end

for (jl, c) in ((:stokes2d_timesteps!, :ps_stokes2d_timesteps), (:stokes2d_compute_P!, :ps_stokes2d_compute_P),
                (:stokes2d_compute_tau!, :ps_stokes2d_compute_tau), (:stokes2d_compute_dV!, :ps_stokes2d_compute_dV),
                (:stokes2d_compute_V!, :ps_stokes2d_compute_V))
    @eval $jl(f::Stokes2DFields, p::Stokes2DParams; stream = CUDA.stream(), sync = true) =
        check(ccall(($(QuoteNode(c)), lib), Cint, (Ref{Stokes2DFields}, Ref{Stokes2DParams}, Ptr{Cvoid}, Cint),
                    f, p, stream_ptr(stream), Cint(sync)))
end
bc_x2d!(A; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_bc_x2d, lib), Cint, (PSArray, Ptr{Cvoid}, Cint), desc(A), stream_ptr(stream), Cint(sync)))
bc_y2d!(A; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_bc_y2d, lib), Cint, (PSArray, Ptr{Cvoid}, Cint), desc(A), stream_ptr(stream), Cint(sync)))
stokes2d_iterate!(f::Stokes2DFields, p::Stokes2DParams, n_iter; stream = CUDA.stream()) =
    check(ccall((:ps_stokes2d_iterate, lib), Cint, (Ref{Stokes2DFields}, Ref{Stokes2DParams}, Int64, Ptr{Cvoid}),
                f, p, Int64(n_iter), stream_ptr(stream)))
function stokes2d_err(f::Stokes2DFields; stream = CUDA.stream())
    out = zeros(Cdouble, 3)
    check(ccall((:ps_stokes2d_err, lib), Cint, (Ref{Stokes2DFields}, Ptr{Cdouble}, Ptr{Cvoid}), f, out,
                stream_ptr(stream)))
    return maximum(out)
end
function stokes2d_solve!(f::Stokes2DFields, p::Stokes2DParams, mode, tol, max_iter, nout; max_seconds = 0.0,
                         stream = CUDA.stream())
    st = Ref(SolveStats(0, 0, 0.0, 0.0, 0, 0))
    check(ccall((:ps_stokes2d_solve, lib), Cint,
                (Ref{Stokes2DFields}, Ref{Stokes2DParams}, Int32, Cdouble, Int64, Int64, Cdouble, Ref{SolveStats},
                 Ptr{Cvoid}),
                f, p, Int32(mode), tol, Int64(max_iter), Int64(nout), max_seconds, st, stream_ptr(stream)))
    return st[]
end

# Stokes2D with the accelerated pseudo-transient iteration (pseudo-time steps from @maxloc(Mus))
struct Stokes2DAPTFields
    Pt::PSArray; divV::PSArray; Vx::PSArray; Vy::PSArray; txx::PSArray; tyy::PSArray; txy::PSArray; Rx::PSArray
    Ry::PSArray; Mus::PSArray; Rog::PSArray; Must::PSArray; kP::PSArray; aT::PSArray; bT::PSArray; aTc::PSArray
    bTc::PSArray; dtVx::PSArray; dtVy::PSArray
end
Stokes2DAPTFields(a::NamedTuple) = Stokes2DAPTFields((desc(getfield(a, k)) for k in fieldnames(Stokes2DAPTFields))...)

struct Stokes2DAPTParams
    dx::Cdouble; dy::Cdouble; Vpdt::Cdouble; Re::Cdouble; r::Cdouble; max_lxy::Cdouble
end

stokes2d_apt_coefficients!(f::Stokes2DAPTFields, p::Stokes2DAPTParams; stream = CUDA.stream(), sync = true) =
    check(ccall((:ps_stokes2d_apt_coefficients, lib), Cint,
                (Ref{Stokes2DAPTFields}, Ref{Stokes2DAPTParams}, Ptr{Cvoid}, Cint), f, p, stream_ptr(stream),
                Cint(sync)))
stokes2d_apt_iterate!(f::Stokes2DAPTFields, p::Stokes2DAPTParams, n_iter; stream = CUDA.stream()) =
    check(ccall((:ps_stokes2d_apt_iterate, lib), Cint,
                (Ref{Stokes2DAPTFields}, Ref{Stokes2DAPTParams}, Int64, Ptr{Cvoid}), f, p, Int64(n_iter),
                stream_ptr(stream)))
function stokes2d_apt_residual!(f::Stokes2DAPTFields, p::Stokes2DAPTParams; stream = CUDA.stream())
    out = zeros(Cdouble, 3)
    check(ccall((:ps_stokes2d_apt_residual, lib), Cint,
                (Ref{Stokes2DAPTFields}, Ref{Stokes2DAPTParams}, Ptr{Cdouble}, Ptr{Cvoid}), f, p, out,
                stream_ptr(stream)))
    return maximum(out)
end
function stokes2d_apt_solve!(f::Stokes2DAPTFields, p::Stokes2DAPTParams, mode, tol, max_iter, nout;
                             max_seconds = 0.0, stream = CUDA.stream())
    st = Ref(SolveStats(0, 0, 0.0, 0.0, 0, 0))
    check(ccall((:ps_stokes2d_apt_solve, lib), Cint,
                (Ref{Stokes2DAPTFields}, Ref{Stokes2DAPTParams}, Int32, Cdouble, Int64, Int64, Cdouble,
                 Ref{SolveStats}, Ptr{Cvoid}),
                f, p, Int32(mode), tol, Int64(max_iter), Int64(nout), max_seconds, st, stream_ptr(stream)))
    return st[]
end

# ---- Stokes3D (miniapps/Stokes3D.jl) -------------------------------------------------------
struct Stokes3DFields
    Pt::PSArray; dtauPt::PSArray; divV::PSArray; Vx::PSArray; Vy::PSArray; Vz::PSArray; txx::PSArray
    tyy::PSArray; tzz::PSArray; txy::PSArray; txz::PSArray; tyz::PSArray; Rx::PSArray; Ry::PSArray; Rz::PSArray
    dVxdtau::PSArray; dVydtau::PSArray; dVzdtau::PSArray; dtauVx::PSArray; dtauVy::PSArray; dtauVz::PSArray
    Mus::PSArray; Rog::PSArray
end
Stokes3DFields(a::NamedTuple) = Stokes3DFields((desc(getfield(a, k)) for k in fieldnames(Stokes3DFields))...)

struct Stokes3DParams
    dx::Cdouble; dy::Cdouble; dz::Cdouble; dampX::Cdouble; dampY::Cdouble; dampZ::Cdouble; Vsc::Cdouble
    Ptsc::Cdouble; min_dxyz2::Cdouble; max_nxyz::Int64
end

for (jl, c) in ((:stokes3d_timesteps!, :ps_stokes3d_timesteps), (:stokes3d_compute_P!, :ps_stokes3d_compute_P),
                (:stokes3d_compute_tau!, :ps_stokes3d_compute_tau), (:stokes3d_compute_dV!, :ps_stokes3d_compute_dV),
                (:stokes3d_compute_V!, :ps_stokes3d_compute_V))
    @eval $jl(f::Stokes3DFields, p::Stokes3DParams; stream = CUDA.stream(), sync = true) =
        check(ccall(($(QuoteNode(c)), lib), Cint, (Ref{Stokes3DFields}, Ref{Stokes3DParams}, Ptr{Cvoid}, Cint),
                    f, p, stream_ptr(stream), Cint(sync)))
end
for (jl, c) in ((:bc_x3d!, :ps_bc_x3d), (:bc_y3d!, :ps_bc_y3d), (:bc_z3d!, :ps_bc_z3d))
    @eval $jl(A; stream = CUDA.stream(), sync = true) =
        check(ccall(($(QuoteNode(c)), lib), Cint, (PSArray, Ptr{Cvoid}, Cint), desc(A), stream_ptr(stream),
                    Cint(sync)))
end
stokes3d_iterate!(f::Stokes3DFields, p::Stokes3DParams, n_iter; one_launch = false, stream = CUDA.stream()) =
    check(ccall((:ps_stokes3d_iterate_ex, lib), Cint,
                (Ref{Stokes3DFields}, Ref{Stokes3DParams}, Int64, Int32, Ptr{Cvoid}),
                f, p, Int64(n_iter), Int32(one_launch), stream_ptr(stream)))
function stokes3d_solve!(f::Stokes3DFields, p::Stokes3DParams, tol, max_iter, nout; mixed = false,
                         max_seconds = 0.0, stream = CUDA.stream())
    st = Ref(SolveStats(0, 0, 0.0, 0.0, 0, 0))
    if mixed
        check(ccall((:ps_stokes3d_solve_mixed, lib), Cint,
                    (Ref{Stokes3DFields}, Ref{Stokes3DParams}, Cdouble, Int64, Int64, Cdouble, Ref{SolveStats},
                     Ptr{Cvoid}),
                    f, p, tol, Int64(max_iter), Int64(nout), max_seconds, st, stream_ptr(stream)))
    else
        check(ccall((:ps_stokes3d_solve, lib), Cint,
                    (Ref{Stokes3DFields}, Ref{Stokes3DParams}, Cdouble, Int64, Int64, Cdouble, Ref{SolveStats},
                     Ptr{Cvoid}),
                    f, p, tol, Int64(max_iter), Int64(nout), max_seconds, st, stream_ptr(stream)))
    end
    return st[]
end

# ---- run-time compiled kernels (any other @parallel / @parallel_indices body) -------------
function jit_compile(source::AbstractString, entry::AbstractString)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:ps_jit_compile, lib), Cint, (Cstring, Cstring, Ref{Ptr{Cvoid}}), source, entry, h))
    return h[]
end
function jit_launch!(h::Ptr{Cvoid}, arrays::Vector{PSArray}, scalars::Vector{Float64}, lo::NTuple{3,Int64},
                     count::NTuple{3,Int64}, threads::NTuple{3,Int32}, shmem::Integer, loop::NTuple{3,Int32};
                     stream = CUDA.stream(), sync = true)
    check(ccall((:ps_jit_launch_ex, lib), Cint,
                (Ptr{Cvoid}, Ptr{PSArray}, Int32, Ptr{Cdouble}, Int32, Ref{NTuple{3,Int64}}, Ref{NTuple{3,Int64}},
                 Ref{NTuple{3,Int32}}, Int64, Ref{NTuple{3,Int32}}, Ptr{Cvoid}, Cint),
                h, arrays, Int32(length(arrays)), scalars, Int32(length(scalars)), lo, count, threads, Int64(shmem),
                loop, stream_ptr(stream), Cint(sync)))
end
# the TMA variant of an FP32 3-D sweep: maps = (array index, box x, box y) per staged array
function jit_launch_tma!(h::Ptr{Cvoid}, arrays::Vector{PSArray}, scalars::Vector{Float64},
                         count::NTuple{3,Int64}, threads::NTuple{3,Int32}, shmem::Integer, loop_z::Integer,
                         maps::Vector{Int32}; stream = CUDA.stream(), sync = true)
    check(ccall((:ps_jit_launch_tma, lib), Cint,
                (Ptr{Cvoid}, Ptr{PSArray}, Int32, Ptr{Cdouble}, Int32, Ref{NTuple{3,Int64}}, Ref{NTuple{3,Int32}},
                 Int64, Int32, Ptr{Int32}, Int32, Ptr{Cvoid}, Cint),
                h, arrays, Int32(length(arrays)), scalars, Int32(length(scalars)), count, threads, Int64(shmem),
                Int32(loop_z), maps, Int32(length(maps) ÷ 3), stream_ptr(stream), Cint(sync)))
end
jit_check(h::Ptr{Cvoid}; stream = CUDA.stream()) =
    check(ccall((:ps_jit_check, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h, stream_ptr(stream)))
jit_destroy(h::Ptr{Cvoid}) = check(ccall((:ps_jit_destroy, lib), Cint, (Ptr{Cvoid},), h))

end # module LibPS
