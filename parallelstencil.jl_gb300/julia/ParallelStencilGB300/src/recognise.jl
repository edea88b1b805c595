# Recognition of `@parallel` / `@parallel_indices` kernel definitions: a definition is normalised
# (line numbers dropped, argument names replaced by their positions, type annotations and
# module-qualified macro names stripped, `return` dropped) and compared with the normalised
# kernels that libps_b200.so implements by hand. The statements below are the ones of the
# reference's examples and miniapps that these kernels replace (file:line beside each).

using MacroTools: MacroTools, isexpr, postwalk, rmlines, splitarg, splitdef, longdef

macroname(m) = isexpr(m, :.) ? m.args[end].value : m          # FiniteDifferences3D.@inn -> Symbol("@inn")

function strip_macro_lines(ex)
    postwalk(ex) do x
        isexpr(x, :macrocall) ? Expr(:macrocall, macroname(x.args[1]), nothing, x.args[3:end]...) : x
    end
end

is_return(s) = s === nothing || s == :return || (isexpr(s, :return) && (isempty(s.args) || s.args[1] === nothing))

function body_statements(body)
    b = rmlines(body)
    stmts = isexpr(b, :block) ? b.args : Any[b]
    return Any[s for s in stmts if !is_return(s)]
end

"""
    normalise(def) -> (nargs, statements)

The definition's argument count and its statements with argument `i` renamed to `_arg<i>`.
For `@parallel_indices (ix, iy) function ...` the index names are renamed to `_idx<i>`.
"""
function normalise(def::Expr, indices = ())
    d = splitdef(longdef(rmlines(def)))
    args = [splitarg(a)[1] for a in d[:args]]
    ren = Dict{Symbol,Symbol}()
    for (i, a) in enumerate(args)
        ren[a] = Symbol("_arg", i)
    end
    for (i, a) in enumerate(indices)
        ren[a] = Symbol("_idx", i)
    end
    stmts = body_statements(d[:body])
    stmts = [postwalk(x -> (x isa Symbol && haskey(ren, x)) ? ren[x] : x, strip_macro_lines(s)) for s in stmts]
    return length(args), stmts
end

# ---- the hand-written kernels ---------------------------------------------------------------
# kind, argument count and the definition whose statements it replaces
const TEMPLATE_SOURCES = [
    # examples/memcopy3D.jl:10-13
    (:copy3D, 3, 0, "function copy3D!(T2, T, Ci) @all(T2) = @all(T) + @all(Ci) end"),
    # examples/diffusion3D_novis_noperf.jl:10-13
    (:diffusion, 3, 0,
     "function diffusion3D_step!(T2, T, Ci, lam, dt, dx, dy, dz)
          @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)/dx^2 + @d2_yi(T)/dy^2 + @d2_zi(T)/dz^2))
      end"),
    # examples/diffusion3D_multigpucpu_hidecomm_novis.jl:12-15
    (:diffusion, 3, 1,
     "function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
          @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))
      end"),
    # test/test_parallel.jl:420-426 (on-the-fly flux form)
    (:diffusion, 3, 2,
     "function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
          @all(qx)   = -lam*@d_xi(T)*_dx
          @all(qy)   = -lam*@d_yi(T)*_dy
          @all(qz)   = -lam*@d_zi(T)*_dz
          @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz)
          @inn(T2)   = @inn(T) + dt*@all(dTdt)
      end"),
    # the same with a conductivity array (face conductivities @av_xi(lam) ...)
    (:diffusion, 3, 3,
     "function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
          @all(qx)   = -@av_xi(lam)*@d_xi(T)*_dx
          @all(qy)   = -@av_yi(lam)*@d_yi(T)*_dy
          @all(qz)   = -@av_zi(lam)*@d_zi(T)*_dz
          @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz)
          @inn(T2)   = @inn(T) + dt*@all(dTdt)
      end"),
    # miniapps/acoustic3D.jl:11-21
    (:acoustic_V, 3, 0,
     "function compute_V!(Vx, Vy, Vz, P, dt, ρ, dx, dy, dz)
          @inn(Vx) = @inn(Vx) - dt/ρ*@d_xi(P)/dx
          @inn(Vy) = @inn(Vy) - dt/ρ*@d_yi(P)/dy
          @inn(Vz) = @inn(Vz) - dt/ρ*@d_zi(P)/dz
      end"),
    (:acoustic_P, 3, 0,
     "function compute_P!(P, Vx, Vy, Vz, dt, k, dx, dy, dz)
          @all(P) = @all(P) - dt*k*(@d_xa(Vx)/dx + @d_ya(Vy)/dy + @d_za(Vz)/dz)
      end"),
    # miniapps/Stokes2D.jl:11-43
    (:s2_timesteps, 2, 0,
     "function compute_timesteps!(dτVx, dτVy, dτPt, Mus, Vsc, Ptsc, min_dxy2, max_nxy)
          @all(dτVx) = Vsc*min_dxy2/@av_xi(Mus)/4.1
          @all(dτVy) = Vsc*min_dxy2/@av_yi(Mus)/4.1
          @all(dτPt) = Ptsc*4.1*@all(Mus)/max_nxy
      end"),
    (:s2_P, 2, 0,
     "function compute_P!(∇V, Pt, Vx, Vy, dτPt, dx, dy)
          @all(∇V)  = @d_xa(Vx)/dx + @d_ya(Vy)/dy
          @all(Pt)  = @all(Pt) - @all(dτPt)*@all(∇V)
      end"),
    (:s2_tau, 2, 0,
     "function compute_τ!(∇V, τxx, τyy, τxy, Vx, Vy, Mus, dx, dy)
          @all(τxx) = 2.0*@all(Mus)*(@d_xa(Vx)/dx - 1.0/3.0*@all(∇V))
          @all(τyy) = 2.0*@all(Mus)*(@d_ya(Vy)/dy - 1.0/3.0*@all(∇V))
          @all(τxy) = 2.0*@av(Mus)*(0.5*(@d_yi(Vx)/dy + @d_xi(Vy)/dx))
      end"),
    (:s2_dV, 2, 0,
     "function compute_dV!(Rx, Ry, dVxdτ, dVydτ, Pt, Rog, τxx, τyy, τxy, dampX, dampY, dx, dy)
          @all(Rx)    = @d_xi(τxx)/dx + @d_ya(τxy)/dy - @d_xi(Pt)/dx
          @all(Ry)    = @d_yi(τyy)/dy + @d_xa(τxy)/dx - @d_yi(Pt)/dy + @av_yi(Rog)
          @all(dVxdτ) = dampX*@all(dVxdτ) + @all(Rx)
          @all(dVydτ) = dampY*@all(dVydτ) + @all(Ry)
      end"),
    (:s2_V, 2, 0,
     "function compute_V!(Vx, Vy, dVxdτ, dVydτ, dτVx, dτVy)
          @inn(Vx) = @inn(Vx) + @all(dτVx)*@all(dVxdτ)
          @inn(Vy) = @inn(Vy) + @all(dτVy)*@all(dVydτ)
      end"),
]

# miniapps/Stokes2D.jl:45-55: `@parallel_indices (ix,iy)` free-slip copies
const INDICES_TEMPLATE_SOURCES = [
    (:bc_x2d, 2, 0, "(ix, iy)", "function bc_x!(A) A[1, iy] = A[2, iy]; A[end, iy] = A[end-1, iy] end"),
    (:bc_y2d, 2, 0, "(ix, iy)", "function bc_y!(A) A[ix, 1] = A[ix, 2]; A[ix, end] = A[ix, end-1] end"),
]

struct Template
    kind::Symbol
    ndims::Int
    form::Int
    nargs::Int
    stmts::Vector{Any}
end

const TEMPLATES = Template[]
const INDICES_TEMPLATES = Template[]

function build_templates!()
    empty!(TEMPLATES)
    empty!(INDICES_TEMPLATES)
    for (kind, nd, form, src) in TEMPLATE_SOURCES
        n, s = normalise(Meta.parse(src))
        push!(TEMPLATES, Template(kind, nd, form, n, s))
    end
    for (kind, nd, form, idx, src) in INDICES_TEMPLATE_SOURCES
        n, s = normalise(Meta.parse(src), Tuple(Meta.parse(idx).args))
        push!(INDICES_TEMPLATES, Template(kind, nd, form, n, s))
    end
end

# ---- one-statement FD kernels: `@<sel>(R) = @<macro>(A)` (src/FiniteDifferences.jl) -----------
const SEL, DIFF, DIFF2, AV, HARM, MAXLOC, MINLOC = 0, 1, 2, 3, 4, 5, 6
const X, Y, Z = 1, 2, 4

function fd_table(nd::Int)
    t = Dict{String,NTuple{3,Int}}()
    if nd == 3
        XYZ = X | Y | Z
        merge!(t, Dict("d_xa" => (DIFF, X, 0), "d_ya" => (DIFF, Y, 0), "d_za" => (DIFF, Z, 0),
                       "d_xi" => (DIFF, X, Y | Z), "d_yi" => (DIFF, Y, X | Z), "d_zi" => (DIFF, Z, X | Y),
                       "d2_xi" => (DIFF2, X, XYZ), "d2_yi" => (DIFF2, Y, XYZ), "d2_zi" => (DIFF2, Z, XYZ),
                       "all" => (SEL, 0, 0), "inn" => (SEL, 0, XYZ), "inn_x" => (SEL, 0, X), "inn_y" => (SEL, 0, Y),
                       "inn_z" => (SEL, 0, Z), "inn_xy" => (SEL, 0, X | Y), "inn_xz" => (SEL, 0, X | Z),
                       "inn_yz" => (SEL, 0, Y | Z), "maxloc" => (MAXLOC, XYZ, XYZ), "minloc" => (MINLOC, XYZ, XYZ)))
        for (kind, pre) in ((AV, "av"), (HARM, "harm"))
            t[pre] = (kind, XYZ, 0)
            t[pre * "_xa"], t[pre * "_ya"], t[pre * "_za"] = (kind, X, 0), (kind, Y, 0), (kind, Z, 0)
            t[pre * "_xi"], t[pre * "_yi"], t[pre * "_zi"] = (kind, X, Y | Z), (kind, Y, X | Z), (kind, Z, X | Y)
            t[pre * "_xya"], t[pre * "_xza"], t[pre * "_yza"] = (kind, X | Y, 0), (kind, X | Z, 0), (kind, Y | Z, 0)
            t[pre * "_xyi"], t[pre * "_xzi"], t[pre * "_yzi"] = (kind, X | Y, Z), (kind, X | Z, Y), (kind, Y | Z, X)
        end
    elseif nd == 2
        XY = X | Y
        merge!(t, Dict("d_xa" => (DIFF, X, 0), "d_ya" => (DIFF, Y, 0), "d_xi" => (DIFF, X, Y), "d_yi" => (DIFF, Y, X),
                       "d2_xa" => (DIFF2, X, X), "d2_ya" => (DIFF2, Y, Y), "d2_xi" => (DIFF2, X, XY),
                       "d2_yi" => (DIFF2, Y, XY), "all" => (SEL, 0, 0), "inn" => (SEL, 0, XY), "inn_x" => (SEL, 0, X),
                       "inn_y" => (SEL, 0, Y), "maxloc" => (MAXLOC, XY, XY), "minloc" => (MINLOC, XY, XY)))
        for (kind, pre) in ((AV, "av"), (HARM, "harm"))
            t[pre] = (kind, XY, 0)
            t[pre * "_xa"], t[pre * "_ya"] = (kind, X, 0), (kind, Y, 0)
            t[pre * "_xi"], t[pre * "_yi"] = (kind, X, Y), (kind, Y, X)
        end
    else
        merge!(t, Dict("d" => (DIFF, X, 0), "d2" => (DIFF2, X, X), "all" => (SEL, 0, 0), "inn" => (SEL, 0, X),
                       "av" => (AV, X, 0), "harm" => (HARM, X, 0), "maxloc" => (MAXLOC, X, X),
                       "minloc" => (MINLOC, X, X)))
    end
    return t
end

const LHS = Dict(1 => Dict("all" => 0, "inn" => X),
                 2 => Dict("all" => 0, "inn" => X | Y, "inn_x" => X, "inn_y" => Y),
                 3 => Dict("all" => 0, "inn" => X | Y | Z, "inn_x" => X, "inn_y" => Y, "inn_z" => Z,
                           "inn_xy" => X | Y, "inn_xz" => X | Z, "inn_yz" => Y | Z))

"""
    recognise(def, ndims; indices=()) -> GB300Kernel

The libps_b200.so kernel a `@parallel` (or, with `indices`, `@parallel_indices`) definition
lowers to. Throws ArgumentError for any other body: those need the run-time compiled path.
"""
function recognise(def::Expr, ndims::Integer; indices = ())
    name = splitdef(longdef(rmlines(def)))[:name]
    n, stmts = normalise(def, indices)
    pool = isempty(indices) ? TEMPLATES : INDICES_TEMPLATES
    for t in pool
        if t.nargs == n && t.stmts == stmts && (t.ndims == ndims || !isempty(indices))
            return GB300Kernel(Symbol(name), t.kind, t.form, LibPS.PSFdOp(0, 0, 0, 0), Int32(0), n)
        end
    end
    if isempty(indices) && n == 2 && length(stmts) == 1
        s = stmts[1]
        if isexpr(s, :(=)) && isexpr(s.args[1], :macrocall) && isexpr(s.args[2], :macrocall) &&
           s.args[1].args[3:end] == [:_arg1] && s.args[2].args[3:end] == [:_arg2]
            lhs, op = String(s.args[1].args[1])[2:end], String(s.args[2].args[1])[2:end]
            tab = fd_table(Int(ndims))
            if haskey(LHS[ndims], lhs) && haskey(tab, op)
                kind, opdims, inn = tab[op]
                return GB300Kernel(Symbol(name), :fd, 0, LibPS.PSFdOp(kind, opdims, inn, ndims),
                                   Int32(LHS[ndims][lhs]), n)
            end
        end
    end
    throw(ArgumentError("@parallel $(name): the GB300 package implements the kernels of the reference's examples " *
                        "and miniapps and one-statement FiniteDifferences kernels; other bodies go through the " *
                        "run-time compiler (ps_gb300.parallel_kernel and ps_jit_compile / ps_jit_launch_ex)"))
end
