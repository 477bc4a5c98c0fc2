# HCCGB300.jl — the Julia side of the drop-in: a `TimeStepper` whose functor calls libhcc_gb300.so through
# `ccall`, behind HyperCloudCore's own API (HyperbolicPDE traits, MUSCL, MOOD, tableaus, ParticleGrid).
#
# Usage (mirrors GeneralRKTimeStepper, src/TimeStepping/TimeSteppers.jl:195-229):
#
#   using HyperCloudCore, HCCGB300
#   ts = GB300RKTimeStepper(eq, pg, MUSCL(Float64, 2, 4, 2, NoLimiter(), RusanovFlux(); div_order = 2),
#                           MOOD(EPD1(), MOODu1(1e-4 * prod(pg.meta.dx))), RK3_SSP_Tableau(Float64);
#                           bc_map = Dict(1 => HCCGB300.OUTFLOW, 2 => HCCGB300.OUTFLOW, 3 => HCCGB300.OUTFLOW,
#                                         4 => HCCGB300.OUTFLOW), precision = :fp64)
#   while t < tmax
#       dt = min(0.4 * get_time_step(pg, eq, ts), tmax - t)
#       ts(eq, pg, t, dt)
#       t += dt
#   end
#
# The grid's positions, tags and states are uploaded at construction; `ts(eq, pg, t, dt)` runs the step on the
# GPU and writes `pg.rhos` and `pg.core.particle_orders` back, so every host-side consumer of the reference
# (snapshot writers, diagnostics) keeps working.
module HCCGB300

using HyperCloudCore
using StaticArrays

export GB300RKTimeStepper, hcc_pde_kind

const libhcc = get(ENV, "HCC_GB300_LIB", joinpath(@__DIR__, "..", "libhcc_gb300.so"))

const KEEP, DIRICHLET, OUTFLOW = Int32(0), Int32(1), Int32(2)

# hcc_config (include/hcc.h), field for field
mutable struct HccConfig
    abi_version::Int32; dim::Int32; n_vars::Int32; pde::Int32; precision::Int32; muscl_order::Int32
    div_order::Int32; mood_criterion::Int32; mood_strategy::Int32; tableau::Int32; mood_substeps::Int32
    periodic::NTuple{3, Int32}; bc_by_tag::NTuple{16, Int32}; max_mood_iterations::Int32
    scheme::Int32; limiter::Int32; slot_capacity::Int32; flux::Int32; reset_orders_per_stage::Int32
    reserved_i::NTuple{3, Int32}
    dx::NTuple{3, Float64}; radius::Float64; weight_alpha::Float64
    canvas_min::NTuple{3, Float64}; canvas_max::NTuple{3, Float64}
    domain_min::NTuple{3, Float64}; domain_max::NTuple{3, Float64}
    mood_delta::Float64; velocity::NTuple{48, Float64}; gamma::Float64; bgk_epsilon::Float64
    bgk_macro_velocity::NTuple{3, Float64}; bgk_coefficient::Float64; bgk_interior_factor::Float64
    u2_plateau::Float64
    u2_ratio::Float64
    reserved_d::NTuple{6, Float64}
    HccConfig() = (c = new(); ccall((:hcc_config_defaults, libhcc), Cvoid, (Ref{HccConfig},), c); c)
end

# PDE -> physics module of the library (the trait the kernels are selected by). Euler is a user HyperbolicPDE
# that declares itself with `hcc_pde_kind(::MyEuler) = 1` and `hcc_gamma(::MyEuler) = γ`.
hcc_pde_kind(::HyperbolicPDE) = error("this HyperbolicPDE has no GB300 physics module")
hcc_gamma(eq) = 1.4

_check(st, h, call) = st == 0 || error("$call: " * unsafe_string(ccall((:hcc_last_error, libhcc), Cstring, (Ptr{Cvoid},), h)))

mutable struct GB300RKTimeStepper{D, M} <: TimeStepper
    handle::Ptr{Cvoid}
    N::Int
end

_tableau_id(bt) = error("unknown tableau")
_strategy_id(::EPD0) = Int32(1); _strategy_id(::EPD1) = Int32(2); _strategy_id(::EPD2) = Int32(3)
_strategy_id(::StrictEPD0) = Int32(4)
_strategy_id(::MOODStrategy) = Int32(0)
_flux_id(::RusanovFlux) = Int32(0)
_flux_id(::AlignedRusanovFlux) = Int32(1)
_limiter_id(::NoLimiter) = Int32(0)
_limiter_id(::BarthJespersenLimiter{:soft}) = Int32(1)
_limiter_id(::BarthJespersenLimiter{:hard}) = Int32(2)
_limiter_id(::VenkatakrishnanLimiter{:soft}) = Int32(3)
_limiter_id(::VenkatakrishnanLimiter{:hard}) = Int32(4)
_criterion(c::MOODu1) = (Int32(1), Float64(c.d))
_criterion(c::MOODu2) = (Int32(4), Float64(c.d))
_criterion(::MOODPAD) = (Int32(2), 0.0)
_criterion(::OnlyMOOD) = (Int32(3), 0.0)
_criterion(::NoMOOD) = (Int32(0), 0.0)

# pg.mover (GridMovers.jl:28-63) -> hcc_set_mover; PrescribedMover takes a rigid motion (velocity, omega, center)
struct HccMover
    kind::Int32; full_search_per_stage::Int32; alpha::Float64
    velocity::NTuple{3, Float64}; omega::NTuple{3, Float64}; center::NTuple{3, Float64}
    keep_volumes::Int32; shepard_sweeps::Int32          # volume_estimator: ShepardVolumes(sweeps) or nothing
end
struct RigidMotion
    velocity::NTuple{3, Float64}; omega::NTuple{3, Float64}; center::NTuple{3, Float64}
end
function _set_mover(h, mv; full_search_per_stage::Bool = false, volume_estimator = ShepardVolumes())
    z = (0.0, 0.0, 0.0)
    kv = volume_estimator === nothing ? Int32(1) : Int32(0)
    sw = volume_estimator === nothing ? Int32(1) : Int32(volume_estimator.sweeps)
    m = mv isa LagrangianMover ? HccMover(1, full_search_per_stage, 1.0, z, z, z, kv, sw) :
        mv isa ScaledLagrangianMover ? HccMover(2, full_search_per_stage, Float64(mv.alpha), z, z, z, kv, sw) :
        mv isa PrescribedMover && mv.velocity isa RigidMotion ?
            HccMover(3, full_search_per_stage, 1.0, mv.velocity.velocity, mv.velocity.omega, mv.velocity.center, kv, sw) :
        mv isa NoGridMover ? HccMover(0, 0, 1.0, z, z, z, kv, sw) : error("unsupported mover $(typeof(mv))")
    _check(ccall((:hcc_set_mover, libhcc), Cint, (Ptr{Cvoid}, Ref{HccMover}), h, m), h, "hcc_set_mover")
end

function GB300RKTimeStepper(eq::HyperbolicPDE{D, M, T}, pg::ParticleGrid{D, M, T}, interp::MUSCL, mood::MOOD,
                            tableau_id::Integer; bc_map = Dict{Int, Int32}(), precision::Symbol = :fp64,
                            reset_orders_per_stage::Bool = false, mood_substeps::Bool = true) where {D, M, T}
    cfg = HccConfig()
    cfg.dim, cfg.n_vars, cfg.pde = D, M, hcc_pde_kind(eq)
    cfg.precision = precision === :fp32 ? 1 : 0
    cfg.muscl_order = HyperCloudCore._extract_order(interp)
    cfg.limiter = _limiter_id(interp.limiter)
    cfg.flux = _flux_id(interp.flux)
    cfg.tableau = tableau_id
    cfg.reset_orders_per_stage = Int32(reset_orders_per_stage)
    cfg.mood_substeps = Int32(mood_substeps)
    cfg.mood_strategy = _strategy_id(mood.strategy)
    cfg.mood_criterion, cfg.mood_delta = _criterion(mood.criterion)
    if mood.criterion isa MOODu2
        cfg.u2_plateau, cfg.u2_ratio = Float64(mood.criterion.plateau), Float64(mood.criterion.ratio)
    end
    pad3(v, z) = ntuple(d -> d <= length(v) ? Float64(v[d]) : z, 3)
    cfg.dx = pad3(pg.meta.dx, 1.0); cfg.radius = pg.meta.R
    cfg.weight_alpha = pg.neighbor.weight_func.alpha
    cfg.canvas_min = pad3(pg.domain.canvas_mins, 0.0); cfg.canvas_max = pad3(pg.domain.canvas_maxs, 1.0)
    cfg.domain_min = pad3(pg.geometry.mins, 0.0); cfg.domain_max = pad3(pg.geometry.maxs, 1.0)
    cfg.periodic = ntuple(d -> d <= D ? Int32(pg.domain.is_periodic[d]) : Int32(0), 3)
    cfg.bc_by_tag = ntuple(t -> Int32(get(bc_map, t, KEEP)), 16)
    cfg.gamma = hcc_gamma(eq)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:hcc_create, libhcc), Cint, (Ref{HccConfig}, Int64, Ref{Ptr{Cvoid}}), cfg, 0, h)
    _check(st, h[], "hcc_create")
    N = pg.meta.N
    pos = reinterpret(Float64, pg.core.positions[1:N])
    bnd = UInt8.(pg.core.is_boundary[1:N]); tags = Int32.(pg.core.tags[1:N]); vol = Float64.(pg.core.volumes[1:N])
    _check(ccall((:hcc_upload_cloud, libhcc), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{UInt8}, Ptr{Int32}, Ptr{Float64}),
                 h[], N, pos, bnd, tags, vol), h[], "hcc_upload_cloud")
    _check(ccall((:hcc_build_neighbours, libhcc), Cint, (Ptr{Cvoid},), h[]), h[], "hcc_build_neighbours")
    _check(ccall((:hcc_prepare_geometry, libhcc), Cint, (Ptr{Cvoid},), h[]), h[], "hcc_prepare_geometry")
    _set_mover(h[], pg.mover)
    ts = GB300RKTimeStepper{D, M}(h[], N)
    finalizer(t -> ccall((:hcc_destroy, libhcc), Cint, (Ptr{Cvoid},), t.handle), ts)
    return ts
end

# build_timestepper(context; time_conf) (Builders/timestepper.jl:15-35) for the GB300 stepper: the same context keys
# (:Equation, :Scheme, :MOOD, :Tableau, :Grid) and Time options (reset_orders_per_stage, full_search_per_stage,
# mood_substeps), plus :Precision (:fp64 / :fp32) and :BCMap (tag => HCC_BC_* kind).
function build_gb300_timestepper(context::Dict; time_conf::Dict = Dict{Symbol, Any}())
    pg = context[:Grid]::ParticleGrid
    ts = GB300RKTimeStepper(context[:Equation], pg, context[:Scheme], context[:MOOD], _tableau_id(context[:Tableau]);
                            bc_map = get(context, :BCMap, Dict{Int, Int32}()),
                            precision = get(context, :Precision, :fp64),
                            reset_orders_per_stage = get(time_conf, :reset_orders_per_stage, false)::Bool,
                            mood_substeps = get(time_conf, :mood_substeps, true)::Bool)
    _set_mover(ts.handle, pg.mover; full_search_per_stage = get(time_conf, :full_search_per_stage, false)::Bool)
    return ts
end

# (ts::GeneralRKTimeStepper)(eq, pg, t, dt) (TimeSteppers.jl:531): one step on the GPU, pg.rhos written back.
function (ts::GB300RKTimeStepper{D, M})(eq::HyperbolicPDE, pg::ParticleGrid, t::Real, dt::Real) where {D, M}
    U = reinterpret(Float64, pg.rhos[1:ts.N])
    _check(ccall((:hcc_upload_state, libhcc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ts.handle, U), ts.handle, "hcc_upload_state")
    _check(ccall((:hcc_step, libhcc), Cint, (Ptr{Cvoid}, Cdouble, Cdouble), ts.handle, t, dt), ts.handle, "hcc_step")
    out = Vector{Float64}(undef, ts.N * M)
    _check(ccall((:hcc_download_state, libhcc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ts.handle, out), ts.handle, "hcc_download_state")
    for i in 1:ts.N
        pg.rhos[i] = State{M, Float64}(ntuple(m -> out[(i - 1) * M + m], Val(M)))
    end
    orders = Vector{Int32}(undef, ts.N)
    _check(ccall((:hcc_download_orders, libhcc), Cint, (Ptr{Cvoid}, Ptr{Int32}), ts.handle, orders), ts.handle, "hcc_download_orders")
    pg.core.particle_orders[1:ts.N] .= orders
    return nothing
end

# get_time_step(pg, eq, interp) (ParticleGrids.jl:386) on the GPU stepper's cached weights.
function HyperCloudCore.get_time_step(pg::ParticleGrid, eq::HyperbolicPDE, ts::GB300RKTimeStepper{D, M}) where {D, M}
    U = reinterpret(Float64, pg.rhos[1:ts.N])
    _check(ccall((:hcc_upload_state, libhcc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ts.handle, U), ts.handle, "hcc_upload_state")
    dt = Ref{Float64}(0.0)
    _check(ccall((:hcc_time_step, libhcc), Cint, (Ptr{Cvoid}, Ref{Float64}), ts.handle, dt), ts.handle, "hcc_time_step")
    return dt[]
end

# Launch shapes of the step and the autotuner (hcc_tuning / hcc_autotune): the shapes change no result.
struct HccTuning
    flux_block::Int32
    gather_block::Int32
    list_blocks_per_sm::Int32
    drop_blocks_per_sm::Int32
end

struct HccTuneReport
    best::HccTuning
    default_ms::Float64
    best_ms::Float64
    candidates::Int32
    steps::Int32
end

# Times the candidates over `steps` steps of size dt from the stepper's current state and keeps the fastest.
function autotune!(ts::GB300RKTimeStepper, dt::Real; steps::Integer = 5)
    r = Ref{HccTuneReport}()
    _check(ccall((:hcc_autotune, libhcc), Cint, (Ptr{Cvoid}, Cdouble, Int32, Ref{HccTuneReport}),
                 ts.handle, dt, steps, r), ts.handle, "hcc_autotune")
    return r[]
end

function set_tuning!(ts::GB300RKTimeStepper, t::HccTuning)
    _check(ccall((:hcc_set_tuning, libhcc), Cint, (Ptr{Cvoid}, Ref{HccTuning}), ts.handle, t), ts.handle, "hcc_set_tuning")
    return ts
end

end # module
