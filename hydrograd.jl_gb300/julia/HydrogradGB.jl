# HydrogradGB.jl -- Julia binding of libhydrograd_gb.so (include/hydrograd_gb.h).
#
# Drop-in point: Hydrograd.jl builds its ODE right-hand side as
#   ODEFunction((du, u, p, t) -> swe_2d_rhs(du, u, p, t, swe_extra_params))
# in src/applications/solve_swe_2D.jl:281-307; `ode_function` below returns the
# same ODEFunction backed by the device RHS, and `probe_loss` / `final_loss`
# carry ChainRulesCore rules whose pullbacks come from the device's checkpointed
# discrete adjoint, so Zygote never traces into the RHS.
#
# Every entry point returns an int status (0 = OK); `check` turns a failure
# into a Julia `error` with hg_last_error's message, as the reference's own
# `error` / `@assert` calls report.  Host arrays passed to the library are kept
# alive across each ccall (GC.@preserve where a struct holds raw pointers).
module HydrogradGB

using ChainRulesCore

const lib = get(ENV, "HYDROGRAD_GB_LIB", joinpath(@__DIR__, "..", "build", "libhydrograd_gb.so"))

# ---- structs of the C ABI ---------------------------------------------------

struct MeshDesc                       # hg_mesh_desc
    n_nodes::Int32
    node_x::Ptr{Float64}
    node_y::Ptr{Float64}
    node_z::Ptr{Float64}
    n_cells::Int32
    cell_node_count::Ptr{Int32}
    cell_nodes::Ptr{Int32}
    n_strings::Int32
    string_ids::Ptr{Int32}
    string_offsets::Ptr{Int32}
    string_nodes::Ptr{Int32}
    string_bc::Ptr{Int32}
end

struct Consts                         # hg_consts
    g::Float64
    k_n::Float64
    h_small::Float64
    riemann::Int32
    order::Int32
end

struct FinalObs                       # hg_final_obs
    wse::Ptr{Float64}
    u::Ptr{Float64}
    v::Ptr{Float64}
    zb_wse::Ptr{Float64}
end

const PRECISION = Dict(:fp64 => Int32(0), :fp32c => Int32(1))
const BC = Dict("WALL" => Int32(0), "SYMM" => Int32(1), "INLET-Q" => Int32(2), "EXIT-H" => Int32(3))
riemann_code(s::AbstractString) = Int32(Dict("Roe" => 0, "HLL" => 1, "HLLC" => 2)[s])

# ---- errors -----------------------------------------------------------------

function last_error(ctx::Ptr{Cvoid})
    buf = Vector{UInt8}(undef, 1024)
    ccall((:hg_last_error, lib), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int32), ctx, buf, Int32(length(buf)))
    return unsafe_string(pointer(buf))
end
check(ctx::Ptr{Cvoid}, rc::Integer) = rc == 0 ? nothing : error("hydrograd_gb (status $rc): ", last_error(ctx))

# ---- context ----------------------------------------------------------------

"""A device context (hg_ctx) and the number of cells it holds."""
mutable struct Context
    ptr::Ptr{Cvoid}
    n::Int
    function Context(ptr::Ptr{Cvoid}, n::Integer)
        c = new(ptr, Int(n))
        finalizer(destroy!, c)
        return c
    end
end
Base.unsafe_convert(::Type{Ptr{Cvoid}}, c::Context) = c.ptr

function destroy!(c::Context)
    if c.ptr != C_NULL
        ccall((:hg_destroy, lib), Cint, (Ptr{Cvoid},), c.ptr)
        c.ptr = C_NULL
    end
    return nothing
end

"""
    create(geom, bc_codes; precision=:fp64, g=9.81, k_n=1.0, h_small=1e-3, riemann="Roe")

A context from an SRH-2D geometry as Hydrograd reads it (`srhgeom_obj`,
SRH_2D_SRHGeom.jl:14-46: nodeCoordinates, elementNodesList, elementNodesCount,
nodeStringsDict) and the boundary type of each NodeString id (`bc_codes`:
id => 0 wall, 1 symmetry, 2 inlet-Q, 3 exit-H).  Ids become 0-based.
"""
function create(geom, bc_codes::AbstractDict; precision::Symbol=:fp64, g=9.81, k_n=1.0, h_small=1e-3,
                riemann::AbstractString="Roe", device::Integer=0)
    x = Vector{Float64}(geom.nodeCoordinates[:, 1])
    y = Vector{Float64}(geom.nodeCoordinates[:, 2])
    z = Vector{Float64}(geom.nodeCoordinates[:, 3])
    ncell = size(geom.elementNodesList, 1)
    cn = zeros(Int32, 8, ncell)                      # row-major [n_cells, 8] as C reads it
    for c in 1:ncell, k in 1:min(8, size(geom.elementNodesList, 2))
        cn[k, c] = Int32(geom.elementNodesList[c, k] - 1)
    end
    cnt = Int32.(geom.elementNodesCount)
    ids = sort(collect(keys(geom.nodeStringsDict)))
    ids32 = Int32.(ids)
    nodes = [Int32.(geom.nodeStringsDict[i] .- 1) for i in ids]
    offs = Int32.(cumsum([0; length.(nodes)]))
    flat = reduce(vcat, nodes; init=Int32[])
    bc = Int32[get(bc_codes, i, Int32(-1)) for i in ids]
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve x y z cn cnt ids32 flat offs bc begin
        d = MeshDesc(Int32(length(x)), pointer(x), pointer(y), pointer(z), Int32(ncell), pointer(cnt), pointer(cn),
                     Int32(length(ids32)), pointer(ids32), pointer(offs), pointer(flat), pointer(bc))
        k = Consts(g, k_n, h_small, riemann_code(riemann), Int32(2))   # device order: Hilbert curve
        rc = ccall((:hg_create, lib), Cint, (Ref{MeshDesc}, Ref{Consts}, Int32, Int32, Ref{Ptr{Cvoid}}),
                   d, k, PRECISION[precision], Int32(device), out)
        check(C_NULL, rc)
    end
    return Context(out[], ncell)
end

struct EnsembleDesc                   # hg_ensemble_desc
    n_meshes::Int32
    meshes::Ptr{MeshDesc}
    n_members::Int32
    member_mesh::Ptr{Int32}
end

"""
Many problems in one context (hg_ensemble_create): member m runs on
meshes[member_mesh[m]] (`meshes` are MeshDesc whose arrays the caller keeps
alive for the call; member_mesh 0-based).  Returns the context and the
members' first cell, inlet-Q and exit-H boundary in the concatenation
(hg_ensemble_layout; member m, 1-based, owns cells cells[m]+1 : cells[m+1]).
"""
function ensemble_create(meshes::Vector{MeshDesc}, member_mesh::Vector{Int32}; precision::Symbol=:fp32c, g=9.81,
                         k_n=1.0, h_small=1e-3, device::Integer=0)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve meshes member_mesh begin
        e = EnsembleDesc(Int32(length(meshes)), pointer(meshes), Int32(length(member_mesh)), pointer(member_mesh))
        rc = ccall((:hg_ensemble_create, lib), Cint, (Ref{EnsembleDesc}, Ref{Consts}, Int32, Int32, Ref{Ptr{Cvoid}}),
                   e, Consts(g, k_n, h_small, Int32(0), Int32(2)), PRECISION[precision], Int32(device), out)
        check(C_NULL, rc)
    end
    nm = Ref{Int32}(0)
    check(out[], ccall((:hg_ensemble_layout, lib), Cint, (Ptr{Cvoid}, Ref{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}),
                       out[], nm, C_NULL, C_NULL, C_NULL))
    cells = zeros(Int32, nm[] + 1); inlets = zeros(Int32, nm[] + 1); exits = zeros(Int32, nm[] + 1)
    check(out[], ccall((:hg_ensemble_layout, lib), Cint, (Ptr{Cvoid}, Ref{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}),
                       out[], nm, cells, inlets, exits))
    return Context(out[], Int(cells[end])), cells, inlets, exits
end

# ---- parameters (process_model_parameters_2D.jl: zone n, per-cell zb, inlet Q) ----

set_still_water!(ctx::Context, wstill::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_still_water, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, wstill))

function set_manning_zones!(ctx::Context, matID::AbstractVector{<:Integer}, n::Vector{Float64})
    mat32 = Int32.(matID)                            # 0-based zone of each cell
    check(ctx.ptr, ccall((:hg_set_manning_zones, lib), Cint, (Ptr{Cvoid}, Ptr{Int32}, Int32, Ptr{Float64}),
                         ctx, mat32, Int32(length(n)), n))
end
set_manning_cells!(ctx::Context, n::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_manning_cells, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, n))
set_zb!(ctx::Context, zb::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_zb_cells, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, zb))
set_inlet_q!(ctx::Context, q::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_inlet_q, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32), ctx, q, Int32(length(q))))
set_exit_wse!(ctx::Context, w::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_exit_wse, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32), ctx, w, Int32(length(w))))
set_riemann_solver!(ctx::Context, s::AbstractString) =
    check(ctx.ptr, ccall((:hg_set_riemann_solver, lib), Cint, (Ptr{Cvoid}, Int32), ctx, riemann_code(s)))
set_dt_min!(ctx::Context, dt_min::Real) =
    check(ctx.ptr, ccall((:hg_set_dt_min, lib), Cint, (Ptr{Cvoid}, Float64), ctx, Float64(dt_min)))
# The steps the gradients differentiate: :ssprk2 (default) or :tsit5 (fixed Tsit5 steps).
set_adjoint_integrator!(ctx::Context, integrator::Symbol) =
    check(ctx.ptr, ccall((:hg_set_adjoint_integrator, lib), Cint, (Ptr{Cvoid}, Int32), ctx,
                         Int32(integrator === :tsit5 ? 1 : integrator === :ssprk2 ? 0 : error("integrator"))))
# The step sizes the Tsit5 gradients differentiate (e.g. tsit5_steps of an adaptive solve);
# an empty vector returns to steps of the call's dt.
set_adjoint_steps!(ctx::Context, dts::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_adjoint_steps, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32), ctx,
                         isempty(dts) ? C_NULL : dts, Int32(length(dts))))
# The step sizes the last solve_tsit5! accepted.
function tsit5_steps(ctx::Context)
    cnt = Ref{Int32}(0)
    check(ctx.ptr, ccall((:hg_tsit5_steps, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32, Ref{Int32}), ctx, C_NULL,
                         Int32(0), cnt))
    out = zeros(Float64, cnt[])
    isempty(out) || check(ctx.ptr, ccall((:hg_tsit5_steps, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32, Ref{Int32}),
                                         ctx, out, Int32(length(out)), cnt))
    return out
end
set_hydrograph!(ctx::Context, group::Integer, t::Vector{Float64}, q::Vector{Float64}) =
    check(ctx.ptr, ccall((:hg_set_inlet_hydrograph, lib), Cint, (Ptr{Cvoid}, Int32, Int32, Ptr{Float64}, Ptr{Float64}),
                         ctx, Int32(group), Int32(length(t)), t, q))
set_adjoint_tape!(ctx::Context, nbytes::Integer) =
    check(ctx.ptr, ccall((:hg_set_adjoint_tape, lib), Cint, (Ptr{Cvoid}, Int64), ctx, Int64(nbytes)))

# ---- state-dependent resistance (semi_discretize_swe_2D.jl:141-181,516-533) ----

const RES = Dict("constant" => 0, "power_law" => 1, "sigmoid" => 2, "inverse" => 3, "h_Umag_ks" => 4)
"""Manning's n as a function of the state (process_ManningN_2D.jl:102-213), recomputed in every RHS."""
function set_manning_function!(ctx::Context, fn::AbstractString, p::AbstractDict,
                               ks_cells::Union{Nothing,Vector{Float64}}=nothing)
    prm = Float64[get(p, k, 0.0) for k in ("n_lower", "n_upper", "k", "h_mid")]
    ks = ks_cells === nothing ? Ptr{Float64}(C_NULL) : pointer(ks_cells)
    GC.@preserve ks_cells begin
        check(ctx.ptr, ccall((:hg_set_manning_function, lib), Cint,
                             (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Ptr{Float64}),
                             ctx, Int32(RES[fn]), prm, Int32(length(prm)), ks))
    end
end

struct UdeDesc                        # hg_ude_desc
    kind::Int32
    n_hidden::Int32
    hidden::Ptr{Int32}
    activation::Ptr{Int32}
    params::Ptr{Float64}
    n_params::Int32
    output_bounds::NTuple{2,Float64}
    h_bounds::NTuple{2,Float64}
    u_bounds::NTuple{2,Float64}
    ks_bounds::NTuple{2,Float64}
    ks_cells::Ptr{Float64}
    layernorm_over_batch::Int32
end
const ACT = Dict("relu" => 0, "leakyrelu" => 1, "sigmoid" => 2, "tanh" => 3, "softplus" => 4)
const UDE = Dict("ManningN_h" => 5, "ManningN_h_Umag_ks" => 6, "FlowResistance" => 7)

"""
A UDE closure in the RHS (process_UDE.jl:3-56 network; `cfg` as the reference's
UDE_options hold it; θ = the Lux parameters flattened in Lux's order).
"""
"""dL/d{n_lower, n_upper, k, h_mid} of the state-dependent n function from the last gradient call."""
function resistance_grad(ctx::Context)
    g = zeros(4)
    check(ctx.ptr, ccall((:hg_resistance_grad, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, g))
    return g
end

"""dL/dθ of the UDE network from the last gradient call, θ in set_ude!'s (Lux's flattened) order:
the gradient UDE_training (swe_2D_UDE.jl:119) takes through the solve."""
function ude_grad(ctx::Context, nparams::Integer)
    g = zeros(nparams)
    check(ctx.ptr, ccall((:hg_ude_grad, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64), ctx, g, Int64(nparams)))
    return g
end

function set_ude!(ctx::Context, choice::AbstractString, cfg::AbstractDict, θ::Vector{Float64},
                  ks_cells::Vector{Float64}=Float64[])
    hid = Int32.(cfg["hidden_layers"])
    act = Int32[ACT[a] for a in cfg["activations"]]
    ub = choice == "FlowResistance" ? cfg["velocity_magnitude_bounds"] : get(cfg, "Umag_bounds", [0.0, 1.0])
    two(v) = (Float64(v[1]), Float64(v[2]))
    GC.@preserve hid act θ ks_cells begin
        d = UdeDesc(Int32(UDE[choice]), Int32(length(hid)), pointer(hid), pointer(act), pointer(θ), Int32(length(θ)),
                    two(cfg["output_bounds"]), two(cfg["h_bounds"]), two(ub), two(get(cfg, "ks_bounds", [0.0, 1.0])),
                    isempty(ks_cells) ? Ptr{Float64}(C_NULL) : pointer(ks_cells), Int32(1))
        check(ctx.ptr, ccall((:hg_set_ude, lib), Cint, (Ptr{Cvoid}, Ref{UdeDesc}), ctx, d))
    end
end

"""
The active parameter of swe_2d_rhs (semi_discretize_swe_2D.jl:112-199): which
of zone n, per-cell zb or inlet Q the parameter vector `p` replaces.  Calling
it writes `p` into the context.
"""
struct ActiveParam
    ctx::Context
    name::String                 # "ManningN", "zb", "Q" or "UDE" (the network's weights)
    matID::Vector{Int32}         # 0-based zone of each cell (ManningN)
    ude_choice::String           # UDE: set_ude!'s choice, cfg and ks per cell
    ude_cfg::Dict{String,Any}
    ks::Vector{Float64}
end
ActiveParam(ctx::Context, name::AbstractString, matID::AbstractVector{<:Integer}) =
    ActiveParam(ctx, String(name), Int32.(matID), "", Dict{String,Any}(), Float64[])
ActiveParam(ctx::Context, choice::AbstractString, cfg::AbstractDict, ks::Vector{Float64}=Float64[]) =
    ActiveParam(ctx, "UDE", Int32[], String(choice), Dict{String,Any}(cfg), ks)
function (a::ActiveParam)(p::AbstractVector{<:Real})
    v = Vector{Float64}(p)
    a.name == "ManningN" ? set_manning_zones!(a.ctx, a.matID, v) :
    a.name == "zb" ? set_zb!(a.ctx, v) :
    a.name == "Q" ? set_inlet_q!(a.ctx, v) :
    a.name == "UDE" ? set_ude!(a.ctx, a.ude_choice, a.ude_cfg, v, a.ks) : error("active parameter: ManningN, zb, Q or UDE")
    return nothing
end

# ---- forward ------------------------------------------------------------------

"""dQdt = swe_2d_rhs(Q, p, t) on the device (hg_rhs); Q = [xi; q_x; q_y]."""
function rhs!(ctx::Context, dQ::Vector{Float64}, Q::Vector{Float64}, t::Real)
    check(ctx.ptr, ccall((:hg_rhs, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Float64, Ptr{Float64}),
                         ctx, Q, Float64(t), dQ))
    return dQ
end

"""
The reference's ODEFunction (solve_swe_2D.jl:281-307) on the device: `apply`
writes the parameter vector into the context before each evaluation.
"""
function ode_function(ctx::Context, apply::ActiveParam; in_place::Bool=true, ODEFunction=nothing)
    f_ip = (du, u, p, t) -> (apply(p); rhs!(ctx, du, u, t); nothing)
    f_oop = (u, p, t) -> (apply(p); rhs!(ctx, similar(u), u, t))
    return ODEFunction === nothing ? (in_place ? f_ip : f_oop) : ODEFunction(in_place ? f_ip : f_oop)
end

"""
`solve(prob, Tsit5(); abstol, reltol, saveat)` (swe_2D_forward_simulation.jl:37-39)
on the device (hg_integrate_tsit5); Q is overwritten with the final state and
`saves[:, i]` holds the state at `saveat[i]`.
"""
function solve_tsit5!(ctx::Context, Q::Vector{Float64}, tspan; abstol=1e-6, reltol=1e-3,
                      saveat::Vector{Float64}=Float64[], adaptive::Bool=true, dt::Real=0.0, maxiters::Integer=0)
    saves = zeros(length(Q), length(saveat))
    stats = zeros(Int32, 3)                          # accepted, rejected, RHS evaluations
    check(ctx.ptr, ccall((:hg_integrate_tsit5, lib), Cint,
                         (Ptr{Cvoid}, Ptr{Float64}, Float64, Float64, Float64, Float64, Float64, Int32, Int32, Int32,
                          Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
                         ctx, Q, Float64(tspan[1]), Float64(tspan[2]), Float64(abstol), Float64(reltol), Float64(dt),
                         Int32(adaptive), Int32(maxiters), Int32(length(saveat)), saveat, saves, stats))
    return Q, saves, stats
end

"""
`nsteps` explicit steps from Q (in place): method 0 SSP-RK2, 1 the reference's
Euler loop (custom_ODE_solvers.jl:5-95); dt > 0 fixed, dt <= 0 the CFL step.
Returns the step sizes taken and, every `save_every` steps, the saved states.
"""
function integrate!(ctx::Context, Q::Vector{Float64}, nsteps::Integer; method::Integer=0, dt::Real=-1.0,
                    cfl::Real=0.4, t0::Real=0.0, save_every::Integer=0)
    nsave = save_every > 0 ? nsteps ÷ save_every : 0
    saves = zeros(length(Q), nsave)
    dts = zeros(nsteps)
    check(ctx.ptr, ccall((:hg_integrate, lib), Cint,
                         (Ptr{Cvoid}, Ptr{Float64}, Float64, Int32, Int32, Float64, Float64, Int32, Ptr{Float64},
                          Ptr{Float64}),
                         ctx, Q, Float64(t0), Int32(nsteps), Int32(method), Float64(dt), Float64(cfl),
                         Int32(save_every), saves, dts))
    return Q, dts, saves
end

# ---- gradients ------------------------------------------------------------------

"""
Probe-depth loss mean_{steps, probes} (h - obs)^2 over `nsteps` SSP-RK2 steps of
`dt` and its gradients (hg_loss_and_grad): per-cell n, per-cell zb, inlet Q.
`probes` are 1-based cell ids; `obs` is nprobe x nsteps (column per step).
"""
function loss_and_grad(ctx::Context, Q0::Vector{Float64}, nsteps::Integer, dt::Real,
                       probes::AbstractVector{<:Integer}, obs::AbstractMatrix{<:Real}; ckpt_every::Integer=50)
    n = ctx.n
    p32 = Int32.(probes .- 1)
    o = Matrix{Float64}(obs)                         # column-major nprobe x nsteps = row-major [step][probe]
    size(o) == (length(p32), nsteps) || error("obs must be nprobe x nsteps")
    loss = Ref{Float64}(0.0)
    gn, gzb, gq, Qf = zeros(n), zeros(n), zeros(64), zeros(3n)
    check(ctx.ptr, ccall((:hg_loss_and_grad, lib), Cint,
                         (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32, Ptr{Int32}, Ptr{Float64}, Int32,
                          Ref{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                         ctx, Q0, Int32(nsteps), Float64(dt), Int32(ckpt_every), p32, o, Int32(length(p32)), loss,
                         gn, gzb, gq, Qf))
    return loss[], gn, gzb, gq, Qf
end

"""λᵀ dQ_final/d(n, zb, Q) (hg_final_vjp): one row of swe_2D_sensitivity.jl's Jacobian per call."""
function final_vjp(ctx::Context, Q0::Vector{Float64}, nsteps::Integer, dt::Real, λ::Vector{Float64};
                   ckpt_every::Integer=50)
    n = ctx.n
    gn, gzb, gq, Qf = zeros(n), zeros(n), zeros(64), zeros(3n)
    check(ctx.ptr, ccall((:hg_final_vjp, lib), Cint,
                         (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                          Ptr{Float64}, Ptr{Float64}),
                         ctx, Q0, Int32(nsteps), Float64(dt), Int32(ckpt_every), λ, gn, gzb, gq, Qf))
    return gn, gzb, gq, Qf
end

"""The zone-n Jacobian of the final state (3n x nzones), as ForwardDiff.jacobian in swe_2D_sensitivity.jl:80."""
function zone_jacobian(ctx::Context, Q0::Vector{Float64}, nsteps::Integer, dt::Real,
                       matID::AbstractVector{<:Integer}, nzones::Integer)
    J = zeros(length(Q0), nzones)
    λ = zeros(length(Q0))
    for r in eachindex(Q0)
        λ[r] = 1.0
        gn, _, _, _ = final_vjp(ctx, Q0, nsteps, dt, λ)
        for z in 1:nzones
            J[r, z] = sum(gn[matID .== z - 1])
        end
        λ[r] = 0.0
    end
    return J
end

"""
The final-state inversion loss of compute_loss_inversion (swe_2D_inversion.jl:383-431)
and its gradients (hg_final_loss_and_grad).  `obs` holds WSE_truth, u_truth,
v_truth and zb_cell_truth as the reference's truth JSON does.
"""
function final_loss_and_grad(ctx::Context, Q0::Vector{Float64}, nsteps::Integer, dt::Real, obs::AbstractDict;
                             active_zb::Bool=false, ckpt_every::Integer=50)
    n = ctx.n
    w = Vector{Float64}(obs["WSE_truth"]); u = Vector{Float64}(obs["u_truth"])
    v = Vector{Float64}(obs["v_truth"]); z = Vector{Float64}(obs["zb_cell_truth"])
    parts, gn, gz, gq, Qf = zeros(3), zeros(n), zeros(n), zeros(64), zeros(3n)
    GC.@preserve w u v z begin
        o = FinalObs(pointer(w), pointer(u), pointer(v), active_zb ? Ptr{Float64}(C_NULL) : pointer(z))
        check(ctx.ptr, ccall((:hg_final_loss_and_grad, lib), Cint,
                             (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32, Ref{FinalObs}, Ptr{Float64},
                              Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                             ctx, Q0, Int32(nsteps), Float64(dt), Int32(ckpt_every), o, parts, gn, gz, gq, Qf))
    end
    return parts, (manning=gn, zb=gz, inletq=gq), Qf    # parts = (WSE + uv, WSE, uv)
end

# Gradient of the active parameter from the per-cell gradients.
function param_gradient(a::ActiveParam, gn, gzb, gq, np::Integer)
    a.name == "ManningN" && return [sum(gn[a.matID .== z - 1]) for z in 1:np]
    a.name == "zb" && return gzb
    a.name == "UDE" && return ude_grad(a.ctx, np)
    return gq[1:np]
end

"""The probe loss as a function of the active parameter θ (see loss_and_grad)."""
function probe_loss(apply::ActiveParam, θ::AbstractVector{<:Real}, Q0::Vector{Float64}, nsteps::Integer, dt::Real,
                    probes::AbstractVector{<:Integer}, obs::AbstractMatrix{<:Real})
    apply(θ)
    loss, _, _, _, _ = loss_and_grad(apply.ctx, Q0, nsteps, dt, probes, obs)
    return loss
end

function ChainRulesCore.rrule(::typeof(probe_loss), apply::ActiveParam, θ::AbstractVector{<:Real},
                              Q0::Vector{Float64}, nsteps::Integer, dt::Real, probes::AbstractVector{<:Integer},
                              obs::AbstractMatrix{<:Real})
    apply(θ)
    loss, gn, gzb, gq, _ = loss_and_grad(apply.ctx, Q0, nsteps, dt, probes, obs)
    gθ = param_gradient(apply, gn, gzb, gq, length(θ))
    probe_loss_pullback(ȳ) = (NoTangent(), NoTangent(), ȳ .* gθ, NoTangent(), NoTangent(), NoTangent(), NoTangent(),
                              NoTangent())
    return loss, probe_loss_pullback
end

"""The final-state inversion loss as a function of the active parameter θ."""
function final_loss(apply::ActiveParam, θ::AbstractVector{<:Real}, Q0::Vector{Float64}, nsteps::Integer, dt::Real,
                    obs::AbstractDict)
    apply(θ)
    parts, _, _ = final_loss_and_grad(apply.ctx, Q0, nsteps, dt, obs; active_zb=apply.name == "zb")
    return parts[1]
end

function ChainRulesCore.rrule(::typeof(final_loss), apply::ActiveParam, θ::AbstractVector{<:Real},
                              Q0::Vector{Float64}, nsteps::Integer, dt::Real, obs::AbstractDict)
    apply(θ)
    parts, g, _ = final_loss_and_grad(apply.ctx, Q0, nsteps, dt, obs; active_zb=apply.name == "zb")
    gθ = param_gradient(apply, g.manning, g.zb, g.inletq, length(θ))
    final_loss_pullback(ȳ) = (NoTangent(), NoTangent(), ȳ .* gθ, NoTangent(), NoTangent(), NoTangent(), NoTangent())
    return parts[1], final_loss_pullback
end

end # module
