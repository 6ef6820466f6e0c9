"""
    GBDycore

Julia binding of libgbdycore (the GB300 dry dynamical-core IMEX step).  The
functions below have the signatures of the ClimaAtmos hooks they replace
(src/simulation/integrator.jl:189-225), so `args_integrator` can pass them to
`CTS.ClimaODEFunction` unchanged; each is one `ccall` into the C ABI declared in
include/gbdycore.h.  `p.gb` holds the library context (a `GBContext`).

State buffers are CuArrays in ClimaCore's VIJFH layout: `parent(Y.c)` is
(Nv, 4, 4, 4, Nh) with components (ρ, uₕ₁, uₕ₂, ρe_tot) and `parent(Y.f)` is
(Nv + 1, 4, 4, 1, Nh); their device pointers are passed without copies.
"""
module GBDycore

import CUDA
import LinearAlgebra

const libgbdycore = get(ENV, "GBDYCORE_LIB", joinpath(@__DIR__, "..", "gbdycore", "libgbdycore.so"))

const GB_OK = Cint(0)

struct GBConfig
    h_elem::Cint
    z_elem::Cint
    ft_bytes::Cint
    z_stretch::Cint
    z_max::Cdouble
    dz_bottom::Cdouble
    dt::Cdouble
    nu_v::Cdouble
    nu_s::Cdouble
    div_damp::Cdouble
    sponge_zd::Cdouble
    alpha_uh::Cdouble
    alpha_w::Cdouble
    upwinding::Cint
    grav::Cdouble
    omega::Cdouble
    R_d::Cdouble
    cp_d::Cdouble
    cv_d::Cdouble
    T_0::Cdouble
    p_ref::Cdouble
    T_min_ref::Cdouble
    T_surf_ref::Cdouble
    T_min_sgs::Cdouble
    radius::Cdouble
    # Held-Suarez forcing (rad: held_suarez): 0 off, 1 on
    held_suarez::Cint
    hs_day::Cdouble
    hs_sigma_b::Cdouble
    hs_dT_y::Cdouble
    hs_T_equator::Cdouble
    hs_dtheta_z::Cdouble
    hs_T_min::Cdouble
    hs_p_ref_theta::Cdouble
    hs_MSLP::Cdouble
end

struct GBFieldVec
    c::Ptr{Cvoid}
    f::Ptr{Cvoid}
end

mutable struct GBContext
    handle::Ptr{Cvoid}
end

fieldvec(Y) = GBFieldVec(
    reinterpret(Ptr{Cvoid}, pointer(parent(Y.c))),
    reinterpret(Ptr{Cvoid}, pointer(parent(Y.f))),
)

function check(ctx::GBContext, rc::Cint)
    rc == GB_OK && return nothing
    buf = Vector{UInt8}(undef, 512)
    ccall((:gb_last_error, libgbdycore), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), ctx.handle, buf, length(buf))
    error("libgbdycore status $rc: " * unsafe_string(pointer(buf)))
end

function GBContext(cfg::GBConfig)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:gb_ctx_create, libgbdycore), Cint, (Ref{GBConfig}, Ref{Ptr{Cvoid}}), cfg, h)
    rc == GB_OK || error("gb_ctx_create failed with status $rc")
    ctx = GBContext(h[])
    finalizer(c -> ccall((:gb_ctx_destroy, libgbdycore), Cint, (Ptr{Cvoid},), c.handle), ctx)
    # work on CUDA.jl's task-local stream
    stream = CUDA.stream().handle
    check(ctx, ccall((:gb_set_stream, libgbdycore), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx.handle, stream))
    return ctx
end

# ---- hooks (same signatures as the reference's) ----

set_precomputed_quantities!(Y, p, t) =
    check(p.gb, ccall((:gb_set_precomputed_quantities, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble), p.gb.handle, fieldvec(Y), t))

function remaining_tendency!(Yₜ, Yₜ_lim, Y, p, t)
    check(p.gb, ccall((:gb_remaining_tendency, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble), p.gb.handle, fieldvec(Yₜ), fieldvec(Y), t))
    return Yₜ
end

implicit_tendency!(Yₜ, Y, p, t) =
    check(p.gb, ccall((:gb_implicit_tendency, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble), p.gb.handle, fieldvec(Yₜ), fieldvec(Y), t))

"""The Jacobian blocks live in the library context; this struct is the handle CTS carries."""
struct GBJacobian
    p::Any
end
Base.zero(j::GBJacobian) = j

update_jacobian!(jacobian::GBJacobian, Y, p, dtγ, t) =
    check(p.gb, ccall((:gb_update_jacobian, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble, Cdouble), p.gb.handle, fieldvec(Y), dtγ, t))

LinearAlgebra.ldiv!(ΔY, jacobian::GBJacobian, R) =
    check(jacobian.p.gb, ccall((:gb_ldiv, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec), jacobian.p.gb.handle, fieldvec(ΔY), fieldvec(R)))

correct_implicit_advection_tendency!(Yₜ, Y, p, t) =
    check(p.gb, ccall((:gb_correct_implicit_advection_tendency, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble), p.gb.handle, fieldvec(Yₜ), fieldvec(Y), t))

dss!(Y, p, t) =
    check(p.gb, ccall((:gb_dss, libgbdycore), Cint, (Ptr{Cvoid}, GBFieldVec), p.gb.handle, fieldvec(Y)))

"""One or more fused ARS343 steps (graph-captured) in place of CTS's stage loop."""
step!(Y, p, t, dt, nsteps = 1) =
    check(p.gb, ccall((:gb_step, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble, Cdouble, Cint, Cint), p.gb.handle, fieldvec(Y), t, dt, nsteps, 1))

function global_sums(Y, p)
    out = zeros(Cdouble, 2)
    check(p.gb, ccall((:gb_global_sums, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Ptr{Cdouble}), p.gb.handle, fieldvec(Y), out))
    return out
end

"""Sums of squares of the Newton residuals (ρ, ρe_tot, u₃) of the last step; throws if a kernel
flagged a non-finite residual or a device wait that timed out."""
function newton_residual(p)
    out = zeros(Cdouble, 3)
    check(p.gb, ccall((:gb_newton_residual, libgbdycore), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.gb.handle, out))
    return out
end

"""What `solve_atmos!` returns (src/simulation/solve.jl:93-97)."""
struct AtmosSolveResults{S, W}
    sol::S
    ret_code::Symbol
    walltime::W
end

"""
    solve_atmos!(Y, p, t, dt, nsteps; save_state = nothing)

One untimed step, then `nsteps` timed fused steps (src/simulation/solve.jl:119-149).  A library
error ends the run as the reference's catch does: `save_state(Y)` is called when given, and the
results carry `:simulation_crashed`.
"""
function solve_atmos!(Y, p, t, dt, nsteps; save_state = nothing)
    try
        step!(Y, p, t, dt, 1)
        CUDA.synchronize()
        walltime = @elapsed begin
            step!(Y, p, t + dt, dt, nsteps)
            CUDA.synchronize()
        end
        newton_residual(p)
        return AtmosSolveResults(Y, :success, walltime)
    catch err
        isnothing(save_state) || save_state(Y)
        @error "simulation crashed" exception = (err, catch_backtrace())
        return AtmosSolveResults(nothing, :simulation_crashed, nothing)
    end
end

# ---- reverse mode (the pullback halves of ChainRulesCore.rrule(solve!, ...)) ----

"""Advance Y by n fused steps (gb_step with graph replay)."""
solve!(Y, p, dt, n) = step!(Y, p, 0.0, dt, n)

"""Forward half of the trajectory gradient: Y advances n steps, a checkpoint every `every`."""
adjoint_forward!(Y, p, dt, n, every) =
    check(p.gb, ccall((:gb_adjoint_forward, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble, Cdouble, Cint, Cint), p.gb.handle, fieldvec(Y), 0.0, dt, n, every))

"""Pullback of the last adjoint_forward!: Ybar (dJ/dY_n in, dJ/dY_0 out); returns (dJ/dnu, dJ/drate)."""
function adjoint_reverse!(Ybar, p)
    d = zeros(Cdouble, 2)
    peak = Ref{Csize_t}(0)
    check(p.gb, ccall((:gb_adjoint_reverse, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Ptr{Cdouble}, Ref{Csize_t}), p.gb.handle, fieldvec(Ybar), d, peak))
    return d[1], d[2]
end

"""Pullback of one step from Y: Ybar (cotangent of the next state in, of Y out)."""
function step_vjp!(Ybar, Y, p, t, dt)
    d = zeros(Cdouble, 2)
    check(p.gb, ccall((:gb_step_vjp, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble, Cdouble, Ptr{Cdouble}), p.gb.handle, fieldvec(Ybar),
        fieldvec(Y), t, dt, d))
    return d[1], d[2]
end

end # module
