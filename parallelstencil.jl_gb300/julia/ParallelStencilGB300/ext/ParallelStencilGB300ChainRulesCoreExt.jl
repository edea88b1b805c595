"""
    ParallelStencilGB300ChainRulesCoreExt

ChainRules `rrule`s for the differentiable entry points of ParallelStencilGB300 (loaded when
ChainRulesCore is): the flux-form diffusion step with a conductivity array and the checkpointed
misfit loss of its time loop. Their pullbacks run the hand-written adjoint kernels of
libps_b200.so (`ps_diffusion3d_adjoint_step`, `ps_diffusion3d_misfit_gradient`), in place of the
Enzyme reverse pass that `@parallel ∇=(T->T̄, lam->lam̄) diffusion3D_step!(...)` runs in the
reference (src/ParallelKernel/parallel.jl:265-301). Not run on the machines this package was
written on (no Julia toolchain there); the same kernels are tested through the Python mirror
(`ps_gb300.adjoint`).
"""
module ParallelStencilGB300ChainRulesCoreExt

using ChainRulesCore
using CUDA
using ParallelStencilGB300
using ParallelStencilGB300: LibPS

# T2 = step(T, lam): inner cells updated, boundary cells copied from T (the examples' Dirichlet
# values). Pullback: λ2 -> (λT, glam) with λT = (∂T2/∂T)^T λ2 on inner cells and zero on boundary
# cells (Dirichlet data, constants of the time loop), glam = (∂T2/∂lam)^T λ2.
function ChainRulesCore.rrule(::typeof(ParallelStencilGB300.diffusion3d_step), T::CuArray{Float64,3},
                              Ci::CuArray{Float64,3}, lam::CuArray{Float64,3}, dt::Real, _dx::Real, _dy::Real,
                              _dz::Real)
    T2 = ParallelStencilGB300.diffusion3d_step(T, Ci, lam, dt, _dx, _dy, _dz)
    function diffusion3d_step_pullback(ΔT2)
        λ2 = CuArray{Float64,3}(unthunk(ΔT2))
        λT, glam = similar(T), CUDA.zeros(Float64, size(T))
        LibPS.adjoint_step!(λT, λ2, T, Ci, lam, glam, dt, _dx, _dy, _dz)
        return (NoTangent(), λT, NoTangent(), glam, NoTangent(), NoTangent(), NoTangent(), NoTangent())
    end
    return T2, diffusion3d_step_pullback
end

# L(lam) = 0.5 ||T_nt - T_obs||^2 after nt steps from T0; the gradient comes from the checkpointed
# adjoint (one forward state every `checkpoint_every` steps, segments recomputed in the reverse sweep).
function ChainRulesCore.rrule(::typeof(ParallelStencilGB300.diffusion3d_misfit), T0::CuArray{Float64,3},
                              T_obs::CuArray{Float64,3}, Ci::CuArray{Float64,3}, lam::CuArray{Float64,3}, dt::Real,
                              _dx::Real, _dy::Real, _dz::Real, nt::Integer; checkpoint_every::Integer = 20,
                              fp64_mode::Integer = LibPS.PS_FP64_IEEE)
    g = similar(lam)
    cfg = LibPS.launch_cfg(; memopt = true, fp64_mode = fp64_mode)
    st = LibPS.misfit_gradient!(g, T0, T_obs, Ci, lam, dt, _dx, _dy, _dz, nt, checkpoint_every, cfg)
    function diffusion3d_misfit_pullback(ΔL)
        return (NoTangent(), NoTangent(), NoTangent(), NoTangent(), unthunk(ΔL) .* g, NoTangent(), NoTangent(),
                NoTangent(), NoTangent(), NoTangent())
    end
    return st.loss, diffusion3d_misfit_pullback
end

end # module
