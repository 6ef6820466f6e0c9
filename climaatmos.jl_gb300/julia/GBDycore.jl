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
ClimaCore numbers the elements along a space-filling curve
(src/simulation/grids.jl:74-75) and gives each element its own (ξ¹, ξ²) frame:
`element_layout` reads both from the space's node coordinates
(gb_match_elements), and the context is built in that layout, so the library's
geometry tables, DSS plan and kernels address the state exactly where ClimaCore
keeps it.  `assert_layout` checks the buffers before every context is used.
"""
module GBDycore

import CUDA
import LinearAlgebra
import ChainRulesCore
import ClimaCore: Fields, Spaces, Geometry

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
    # the caller's element layout (gb_match_elements), C_NULL: the library's own order
    elem_map::Ptr{Cint}
    elem_orient::Ptr{Cint}
    # numerics.test_dycore_consistency: NaN-fill the library's scratch before each use
    test_dycore_consistency::Cint
    # terrain-following levels: surface elevation per node (caller's element and node order),
    # C_NULL: flat; warp 0 linear (LinearAdaption), 1 SLEVE (SLEVEAdaption) with eta_h and s
    z_surface::Ptr{Cdouble}
    warp::Cint
    sleve_eta::Cdouble
    sleve_s::Cdouble
    # moist 0M (microphysics_model EquilibriumMicrophysics0M): 1 adds Y.c.ρq_tot as the fifth
    # centre component (the column hooks only); the Thermodynamics.jl constants of the moist
    # thermodynamics and the Newton iterations of the saturation adjustment
    moist::Cint
    R_v::Cdouble
    cp_v::Cdouble
    cp_l::Cdouble
    cp_i::Cdouble
    LH_v0::Cdouble
    LH_s0::Cdouble
    T_triple::Cdouble
    press_triple::Cdouble
    T_freeze::Cdouble
    T_icenuc::Cdouble
    pow_icenuc::Cdouble
    sa_iters::Cint
end

# A copy of cfg with the named fields replaced.
function with_fields(cfg::GBConfig; kw...)
    vals = map(f -> haskey(kw, f) ? kw[f] : getfield(cfg, f), fieldnames(GBConfig))
    return GBConfig(vals...)
end

"""
    terrain(space) -> (z_surface, warp, eta_h, s) or nothing

The surface elevation of a ClimaCore extruded space with hypsography (its grid's
`hypsography.surface`, a field on the horizontal space), as a [Nh][16] array in the space's
element and node order (node n = i + 4 j), and the warp: LinearAdaption -> 0, SLEVEAdaption ->
1 with its eta_h and s.  `nothing` for a flat space.
"""
function terrain(space)
    grid = Spaces.grid(space)
    hasproperty(grid, :hypsography) || return nothing
    hyps = grid.hypsography
    hasproperty(hyps, :surface) || return nothing
    zs = Array(parent(hyps.surface))                        # (Nq, Nq, 1, Nh)
    Nq, _, _, Nh = size(zs)
    out = Array{Cdouble}(undef, Nq, Nq, Nh)                # C order [Nh][16], n = i + 4 j
    for h in 1:Nh, j in 1:Nq, i in 1:Nq
        out[i, j, h] = zs[i, j, 1, h]
    end
    if hasproperty(hyps, :ηₕ)
        return out, Cint(1), Cdouble(hyps.ηₕ), Cdouble(hyps.s)
    end
    return out, Cint(0), 0.7, 10.0
end

struct GBFieldVec
    c::Ptr{Cvoid}
    f::Ptr{Cvoid}
end

mutable struct GBContext
    handle::Ptr{Cvoid}
    cfg::GBConfig
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

"""
    element_layout(cfg, space) -> (elem_map, elem_orient)

The element numbering and per-element frames of a ClimaCore space (any space whose
horizontal space is the cubed sphere of `cfg.h_elem`): the unit vectors of every node, in
the space's own element order and (i, j) order, matched against the library's grid by
gb_match_elements.  Refuses a grid that is not the equiangular cubed sphere at `h_elem` or
an element whose frame is mirrored.
"""
function element_layout(cfg::GBConfig, space)
    hspace = Spaces.horizontal_space(space)
    coords = parent(Fields.coordinate_field(hspace))       # (Nq, Nq, 2, Nh): lat, long in degrees
    coords = Array(coords)
    Nq, _, _, Nh = size(coords)
    Nq == 4 || error("GBDycore: the library is built for Nq = 4, the space has Nq = $Nq")
    Nh == 6 * cfg.h_elem^2 || error("GBDycore: the space has $Nh elements, h_elem = $(cfg.h_elem) needs $(6 * cfg.h_elem^2)")
    xyz = Array{Cdouble}(undef, 3, Nq, Nq, Nh)             # C order [Nh][16][3], node n = i + 4 j
    for h in 1:Nh, j in 1:Nq, i in 1:Nq
        φ, λ = coords[i, j, 1, h], coords[i, j, 2, h]
        xyz[1, i, j, h] = cosd(φ) * cosd(λ)
        xyz[2, i, j, h] = cosd(φ) * sind(λ)
        xyz[3, i, j, h] = sind(φ)
    end
    elem_map = zeros(Cint, Nh)
    elem_orient = zeros(Cint, Nh)
    rc = ccall((:gb_match_elements, libgbdycore), Cint, (Ref{GBConfig}, Ptr{Cdouble}, Ptr{Cint}, Ptr{Cint}),
        cfg, xyz, elem_map, elem_orient)
    rc == GB_OK || error("gb_match_elements: the space's nodes are not the library's cubed sphere (status $rc)")
    return elem_map, elem_orient
end

"""
    assert_layout(ctx, Y)

The buffers handed to the library are what the header says: `Y.c` holds (ρ, uₕ, ρe_tot), and
ρq_tot last in a moist 0M context, with uₕ a 2-component covariant vector, `Y.f` holds u₃ alone,
both CuArrays of the context's float type with ClimaCore's VIJFH parent shapes
(Nv, 4, 4, 4 or 5, Nh) and (Nv + 1, 4, 4, 1, Nh).
"""
function assert_layout(ctx::GBContext, Y)
    cfg = ctx.cfg
    FT = cfg.ft_bytes == 8 ? Float64 : Float32
    Nh, Nv = 6 * cfg.h_elem^2, cfg.z_elem
    names = cfg.moist == 1 ? (:ρ, :uₕ, :ρe_tot, :ρq_tot) : (:ρ, :uₕ, :ρe_tot)
    propertynames(Y.c) == names || error("GBDycore: Y.c must hold $names, it holds $(propertynames(Y.c))")
    propertynames(Y.f) == (:u₃,) || error("GBDycore: Y.f must hold (u₃,), it holds $(propertynames(Y.f))")
    eltype(Y.c.uₕ) <: Geometry.Covariant12Vector || error("GBDycore: uₕ must be a Covariant12Vector field")
    eltype(Y.f.u₃) <: Geometry.Covariant3Vector || error("GBDycore: u₃ must be a Covariant3Vector field")
    pc, pf = parent(Y.c), parent(Y.f)
    pc isa CUDA.CuArray{FT} && pf isa CUDA.CuArray{FT} ||
        error("GBDycore: the state must be CuArrays of $FT (the context's precision)")
    nfc = ctx.cfg.moist == 1 ? 5 : 4   # (ρ, uₕ, ρe_tot[, ρq_tot])
    size(pc) == (Nv, 4, 4, nfc, Nh) || error("GBDycore: parent(Y.c) is $(size(pc)), expected $((Nv, 4, 4, nfc, Nh))")
    size(pf) == (Nv + 1, 4, 4, 1, Nh) || error("GBDycore: parent(Y.f) is $(size(pf)), expected $((Nv + 1, 4, 4, 1, Nh))")
    return nothing
end

"""
    GBContext(cfg; space = nothing)

The library context.  With a ClimaCore `space` the context is built in that space's element
layout (`element_layout`); without one, in the library's panel-major order.
"""
function GBContext(cfg::GBConfig; space = nothing)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    if space === nothing
        rc = ccall((:gb_ctx_create, libgbdycore), Cint, (Ref{GBConfig}, Ref{Ptr{Cvoid}}), cfg, h)
    else
        elem_map, elem_orient = element_layout(cfg, space)
        t = terrain(space)
        zs = t === nothing ? Cdouble[] : t[1]
        rc = GC.@preserve elem_map elem_orient zs begin
            c = with_fields(cfg; elem_map = pointer(elem_map), elem_orient = pointer(elem_orient))
            if t !== nothing
                c = with_fields(c; z_surface = pointer(zs), warp = t[2], sleve_eta = t[3], sleve_s = t[4])
            end
            ccall((:gb_ctx_create, libgbdycore), Cint, (Ref{GBConfig}, Ref{Ptr{Cvoid}}), c, h)
        end
    end
    rc == GB_OK || error("gb_ctx_create failed with status $rc")
    # the library copies the layout and the surface into its tables; the context keeps no pointer
    ctx = GBContext(h[], with_fields(cfg; elem_map = C_NULL, elem_orient = C_NULL, z_surface = C_NULL))
    finalizer(c -> ccall((:gb_ctx_destroy, libgbdycore), Cint, (Ptr{Cvoid},), c.handle), ctx)
    # work on CUDA.jl's task-local stream
    stream = CUDA.stream().handle
    check(ctx, ccall((:gb_set_stream, libgbdycore), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx.handle, stream))
    return ctx
end

# ---- hooks (same signatures as the reference's) ----

"""The device pointers of a FieldVector after `assert_layout` (every hook goes through this)."""
gbvec(ctx::GBContext, Y) = (assert_layout(ctx, Y); fieldvec(Y))

set_precomputed_quantities!(Y, p, t) =
    check(p.gb, ccall((:gb_set_precomputed_quantities, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble), p.gb.handle, gbvec(p.gb, Y), t))

function remaining_tendency!(Yₜ, Yₜ_lim, Y, p, t)
    check(p.gb, ccall((:gb_remaining_tendency, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble), p.gb.handle, gbvec(p.gb, Yₜ), gbvec(p.gb, Y), t))
    return Yₜ
end

implicit_tendency!(Yₜ, Y, p, t) =
    check(p.gb, ccall((:gb_implicit_tendency, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble), p.gb.handle, gbvec(p.gb, Yₜ), gbvec(p.gb, Y), t))

"""The Jacobian blocks live in the library context; this struct is the handle CTS carries."""
struct GBJacobian
    p::Any
end
Base.zero(j::GBJacobian) = j

update_jacobian!(jacobian::GBJacobian, Y, p, dtγ, t) =
    check(p.gb, ccall((:gb_update_jacobian, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble, Cdouble), p.gb.handle, gbvec(p.gb, Y), dtγ, t))

LinearAlgebra.ldiv!(ΔY, jacobian::GBJacobian, R) =
    check(jacobian.p.gb, ccall((:gb_ldiv, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec), jacobian.p.gb.handle, gbvec(jacobian.p.gb, ΔY),
        gbvec(jacobian.p.gb, R)))

correct_implicit_advection_tendency!(Yₜ, Y, p, t) =
    check(p.gb, ccall((:gb_correct_implicit_advection_tendency, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble), p.gb.handle, gbvec(p.gb, Yₜ), gbvec(p.gb, Y), t))

dss!(Y, p, t) =
    check(p.gb, ccall((:gb_dss, libgbdycore), Cint, (Ptr{Cvoid}, GBFieldVec), p.gb.handle, gbvec(p.gb, Y)))

"""One or more fused ARS343 steps (graph-captured) in place of CTS's stage loop."""
step!(Y, p, t, dt, nsteps = 1) =
    check(p.gb, ccall((:gb_step, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble, Cdouble, Cint, Cint), p.gb.handle, gbvec(p.gb, Y), t, dt, nsteps, 1))

function global_sums(Y, p)
    out = zeros(Cdouble, 2)
    check(p.gb, ccall((:gb_global_sums, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Ptr{Cdouble}), p.gb.handle, gbvec(p.gb, Y), out))
    return out
end

"""∫ρ, ∫ρe_tot and ∫ρq_tot (0 for a dry context): the sums check_conservation compares."""
function conservation_sums(Y, p)
    out = zeros(Cdouble, 3)
    check(p.gb, ccall((:gb_conservation_sums, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Ptr{Cdouble}), p.gb.handle, gbvec(p.gb, Y), out))
    return out
end

"""check_conservation (src/simulation/solve.jl:216-265) from the conservation sums of a run's
first and last states, for a surface without a slab ocean."""
function check_conservation(first, last, moist::Bool; energy_surface_change = 0.0,
                            energy_radiation_input = 0.0)
    energy_conservation =
        abs(last[2] - first[2] + energy_surface_change - energy_radiation_input) / first[2]
    mass_conservation = (last[1] - first[1]) / first[1]
    water_conservation = moist ? abs(last[3] - first[3]) / last[3] : 0.0
    return (; energy_conservation, mass_conservation, water_conservation)
end

"""Sums of squares of the Newton residuals (ρ, ρe_tot, u₃) of the last step; throws if a kernel
flagged a non-finite residual or a device wait that timed out."""
function newton_residual(p)
    out = zeros(Cdouble, 3)
    check(p.gb, ccall((:gb_newton_residual, libgbdycore), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.gb.handle, out))
    return out
end

# ---- solve_atmos!(simulation) over the fused step ----

"""
    GBSimulation(Y, p, t_start, t_end, dt; output_dir = nothing, save_state = nothing)

What `solve_atmos!` needs of an `AtmosSimulation` (src/simulation/AtmosSimulations.jl:307)
when the CTS integrator is replaced by the fused step: the state `Y` (its FieldVector, in
the layout of `p.gb`), the cache `p` holding the `GBContext` as `p.gb`, the time span and
step, and what a crash writes (`save_state(Y, t, output_dir)`, the counterpart of
`save_state_to_disk_func`, src/callbacks/callbacks.jl:297-321).
"""
mutable struct GBSimulation{Y, P, FT}
    Y::Y
    p::P
    t::FT
    t_end::FT
    dt::FT
    output_dir::Union{Nothing, String}
    save_state::Any
end
GBSimulation(Y, p, t_start, t_end, dt; output_dir = nothing, save_state = nothing) =
    GBSimulation(Y, p, promote(t_start, t_end, dt)..., output_dir, save_state)

"""What `solve_atmos!` returns (src/simulation/solve.jl:86-97)."""
struct AtmosSolveResults{S, RT, WT}
    sol::S
    ret_code::RT
    walltime::WT
end

"""
    solve_atmos!(simulation::GBSimulation)

`solve_atmos!(simulation)` (src/simulation/solve.jl:119-160) on the fused step: one step
outside the timed region, then the steps to `t_end`, timed on the device; SYPD and the wall
time per step are logged as `timed_solve!` logs them (solve.jl:56-82).  A library error
(a non-finite Newton residual, a device wait that ran out, a CUDA error) ends the run as the
reference's `catch` does: the state is saved when `save_state` is given and the results
carry `:simulation_crashed`.
"""
function solve_atmos!(sim::GBSimulation)
    (; Y, p, dt) = sim
    t_start = sim.t
    nsteps = round(Int, (sim.t_end - sim.t) / dt)
    nsteps >= 1 || error("solve_atmos!: t_end is less than one step ahead")
    try
        step!(Y, p, sim.t, dt, 1)
        sim.t += dt
        CUDA.synchronize()
        walltime = CUDA.@elapsed begin
            step!(Y, p, sim.t, dt, nsteps - 1)
        end
        sim.t += (nsteps - 1) * dt
        newton_residual(p)                     # raises on a flagged device failure
        sypd = ((sim.t_end - t_start) / (365 * 24 * 3600)) / (walltime / (24 * 3600))
        @info "solve! walltime = $(round(walltime, digits = 3))"
        @info "sypd: $(round(sypd, digits = 3))"
        @info "wall_time_per_timestep: $(walltime / max(nsteps - 1, 1)) s"
        return AtmosSolveResults(Y, :success, walltime)
    catch err
        isnothing(sim.save_state) || sim.save_state(Y, sim.t, sim.output_dir)
        @error "ClimaAtmos simulation crashed. Stacktrace for failed simulation" exception =
            (err, catch_backtrace())
        return AtmosSolveResults(nothing, :simulation_crashed, nothing)
    end
end

# ---- reverse mode: ChainRulesCore.rrule of the n-step solve ----

"""
    solve(Y0, θ, p, dt, n) -> Y_n

`n` fused steps from a copy of `Y0`.  `θ = (ν = ..., rate = ...)` names the two calibrated
scalars, the hyperdiffusivity ν₄ (ν_scalar follows it through the Prandtl number) and the
Rayleigh sponge rate; they are fixed when the context is made, so `θ` must equal the
context's values, and the rrule below returns the derivative with respect to them.
"""
function solve(Y0, θ::NamedTuple{(:ν, :rate)}, p, dt, n)
    check_params(p.gb, θ)
    Y = copy(Y0)
    step!(Y, p, 0.0, dt, n)
    return Y
end

function check_params(ctx::GBContext, θ)
    c = ctx.cfg
    θ.ν == c.nu_v || error("GBDycore.solve: θ.ν = $(θ.ν) differs from the context's ν = $(c.nu_v)")
    (θ.rate == c.alpha_uh && θ.rate == c.alpha_w) ||
        error("GBDycore.solve: θ.rate = $(θ.rate) differs from the context's sponge rate")
    return nothing
end

"""Forward half of the trajectory gradient: Y advances n steps, a checkpoint every `every`."""
adjoint_forward!(Y, p, dt, n, every) =
    check(p.gb, ccall((:gb_adjoint_forward, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Cdouble, Cdouble, Cint, Cint), p.gb.handle, gbvec(p.gb, Y), 0.0, dt, n, every))

"""Pullback of the last adjoint_forward!: Ybar (dJ/dY_n in, dJ/dY_0 out); returns (dJ/dν, dJ/drate)
and the device bytes the library held at the peak of the pass."""
function adjoint_reverse!(Ybar, p)
    d = zeros(Cdouble, 2)
    peak = Ref{Csize_t}(0)
    check(p.gb, ccall((:gb_adjoint_reverse, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, Ptr{Cdouble}, Ref{Csize_t}), p.gb.handle, gbvec(p.gb, Ybar), d, peak))
    return d[1], d[2], Int(peak[])
end

"""How many trailing checkpoint segments the forward half keeps the stage data of (HBM for
recomputation: the pullback then recomputes only the segments before them)."""
adjoint_record_segments!(p, k::Integer) =
    check(p.gb, ccall((:gb_adjoint_set_record_segments, libgbdycore), Cint, (Ptr{Cvoid}, Cint), p.gb.handle, k))

"""Pullback of one step from Y: Ybar (cotangent of the next state in, of Y out)."""
function step_vjp!(Ybar, Y, p, t, dt)
    d = zeros(Cdouble, 2)
    check(p.gb, ccall((:gb_step_vjp, libgbdycore), Cint,
        (Ptr{Cvoid}, GBFieldVec, GBFieldVec, Cdouble, Cdouble, Ptr{Cdouble}), p.gb.handle, gbvec(p.gb, Ybar),
        gbvec(p.gb, Y), t, dt, d))
    return d[1], d[2]
end

"""
    ChainRulesCore.rrule(::typeof(solve), Y0, θ, p, dt, n; checkpoint_every = 5, record_segments = nothing)

Reverse mode of `solve` (the differentiable step that calibration of ν and the sponge rate
needs): the forward half runs `gb_adjoint_forward` (the n steps, a checkpoint every
`checkpoint_every`, the stage data of the last `record_segments` segments kept), the pullback
`gb_adjoint_reverse` (each other checkpoint segment recomputed with its stage data kept, then reversed with the transposed SE operators, DSS and column
solves).  The cotangent of Y_n comes in as a FieldVector; it returns the cotangents of Y0
and of θ = (ν, rate); `p`, `dt` and `n` get none.
"""
function ChainRulesCore.rrule(::typeof(solve), Y0, θ::NamedTuple{(:ν, :rate)}, p, dt, n; checkpoint_every = 5,
                              record_segments = nothing)
    check_params(p.gb, θ)
    record_segments === nothing || adjoint_record_segments!(p, record_segments)
    Y = copy(Y0)
    adjoint_forward!(Y, p, dt, n, checkpoint_every)
    function solve_pullback(Ȳ)
        Ybar = copy(ChainRulesCore.unthunk(Ȳ))
        dν, drate, _ = adjoint_reverse!(Ybar, p)
        θbar = ChainRulesCore.Tangent{typeof(θ)}(; ν = dν, rate = drate)
        return (ChainRulesCore.NoTangent(), Ybar, θbar, ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(),
            ChainRulesCore.NoTangent())
    end
    return Y, solve_pullback
end

end # module
