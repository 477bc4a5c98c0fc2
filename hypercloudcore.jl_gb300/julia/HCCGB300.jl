# HCCGB300.jl — the Julia side of the drop-in: a `TimeStepper` whose functor calls libhcc_gb300.so through
# `ccall`, behind HyperCloudCore's own API (HyperbolicPDE traits, MUSCL, MOOD, tableaus, ParticleGrid).
#
# Usage (mirrors GeneralRKTimeStepper, src/TimeStepping/TimeSteppers.jl:195-229):
#
#   using HyperCloudCore, HCCGB300
#   ts = GB300RKTimeStepper(eq, pg, MUSCL(Float64, 2, 4, 2, NoLimiter(), RusanovFlux(); div_order = 2),
#                           MOOD(EPD1(), MOODu1(1e-4 * prod(pg.meta.dx))), RK3_SSP_Tableau(Float64);
#                           precision = :fp64)
#   while t < tmax
#       dt = min(0.4 * get_time_step(pg, eq, ts), tmax - t)
#       ts(eq, pg, t, dt)
#       t += dt
#   end
#
# The boundary conditions come from the grid's own map, pg.geometry.bc_map (FixedDirichlet / OutflowBC per tag,
# BoundaryConditions.jl:43-130); the tableau is the tableau object itself (any built-in one of
# ButcherTableaus.jl:125-263); the scheme may be MUSCL (with its div_order, moment_correction and streamed
# settings), WENO, CentralDivergence or UpwindDivergence.
#
# The grid's positions, tags and states are uploaded at construction; `ts(eq, pg, t, dt)` runs the step on the
# GPU and writes `pg.rhos` and `pg.core.particle_orders` back, so every host-side consumer of the reference
# (snapshot writers, diagnostics) keeps working.
module HCCGB300

using HyperCloudCore
using StaticArrays

export GB300RKTimeStepper, hcc_pde_kind

const libhcc = get(ENV, "HCC_GB300_LIB", joinpath(@__DIR__, "..", "libhcc_gb300.so"))

# The enums of include/hcc.h, value for value.
const HCC_BC_KEEP, HCC_BC_DIRICHLET, HCC_BC_OUTFLOW = Int32(0), Int32(1), Int32(2)
const KEEP, DIRICHLET, OUTFLOW = HCC_BC_KEEP, HCC_BC_DIRICHLET, HCC_BC_OUTFLOW
const HCC_TAB_RK1_EULER = Int32(0)
const HCC_TAB_RK2_SSP = Int32(1)
const HCC_TAB_RK2_RALSTON = Int32(2)
const HCC_TAB_RK3_SSP = Int32(3)
const HCC_TAB_RK4_CLASSICAL = Int32(4)
const HCC_TAB_RK4_SSP = Int32(5)
const HCC_TAB_IMEX_EULER = Int32(6)
const HCC_TAB_IMEX_ARS233 = Int32(7)
const HCC_TAB_IMEX_ARS222 = Int32(8)
const HCC_TAB_IMEX_PRSSP3 = Int32(9)
const HCC_TAB_IMEX_SSP2332 = Int32(10)
const HCC_MOOD_NONE, HCC_MOOD_U1, HCC_MOOD_PAD, HCC_MOOD_ONLY, HCC_MOOD_U2 = Int32(0), Int32(1), Int32(2), Int32(3), Int32(4)
const HCC_EPD_NONE, HCC_EPD0, HCC_EPD1, HCC_EPD2, HCC_STRICT_EPD0 = Int32(0), Int32(1), Int32(2), Int32(3), Int32(4)
const HCC_SCHEME_MUSCL, HCC_SCHEME_WENO, HCC_SCHEME_CENTRAL, HCC_SCHEME_UPWIND = Int32(0), Int32(1), Int32(2), Int32(3)
const HCC_UPWIND_TIWARI, HCC_UPWIND_PRAVEEN = Int32(1), Int32(2)
const HCC_LIMITER_NONE, HCC_LIMITER_BJ_SOFT, HCC_LIMITER_BJ_HARD = Int32(0), Int32(1), Int32(2)
const HCC_LIMITER_VK_SOFT, HCC_LIMITER_VK_HARD = Int32(3), Int32(4)
const HCC_FLUX_RUSANOV, HCC_FLUX_ALIGNED = Int32(0), Int32(1)

# hcc_config (include/hcc.h), field for field
mutable struct HccConfig
    abi_version::Int32; dim::Int32; n_vars::Int32; pde::Int32; precision::Int32; muscl_order::Int32
    div_order::Int32; mood_criterion::Int32; mood_strategy::Int32; tableau::Int32; mood_substeps::Int32
    periodic::NTuple{3, Int32}; bc_by_tag::NTuple{16, Int32}; max_mood_iterations::Int32
    scheme::Int32; limiter::Int32; slot_capacity::Int32; flux::Int32; reset_orders_per_stage::Int32
    upwind_algorithm::Int32; moment_correction::Int32; reserved_i::NTuple{1, Int32}
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

# The tableau object (ButcherTableaus.jl:125-263 build IMEXButcherTableau values, not types): matched coefficient
# for coefficient against the built-in tableaus of its element type; an Integer is taken as the hcc_tableau id.
const _BUILTIN_TABLEAUS = ((HyperCloudCore.RK1_Euler_Tableau, HCC_TAB_RK1_EULER),
                           (HyperCloudCore.RK2_SSP_Tableau, HCC_TAB_RK2_SSP),
                           (HyperCloudCore.RK2_Ralston_Tableau, HCC_TAB_RK2_RALSTON),
                           (HyperCloudCore.RK3_SSP_Tableau, HCC_TAB_RK3_SSP),
                           (HyperCloudCore.RK4_Classical_Tableau, HCC_TAB_RK4_CLASSICAL),
                           (HyperCloudCore.RK4_SSP_Tableau, HCC_TAB_RK4_SSP),
                           (HyperCloudCore.IMEX_Euler_Tableau, HCC_TAB_IMEX_EULER),
                           (HyperCloudCore.IMEX_ARS233_Tableau, HCC_TAB_IMEX_ARS233),
                           (HyperCloudCore.IMEX_ARS222_Tableau, HCC_TAB_IMEX_ARS222),
                           (HyperCloudCore.IMEX_PRSSP3_Tableau, HCC_TAB_IMEX_PRSSP3),
                           (HyperCloudCore.IMEX_SSP2332_Tableau, HCC_TAB_IMEX_SSP2332))
_same_tableau(x, y) = all(isapprox(getfield(x, f), getfield(y, f); rtol = 0, atol = 64 * eps(Float64))
                          for f in (:a, :a_t, :c, :c_t, :b, :b_t))
function _tableau_id(bt::HyperCloudCore.IMEXButcherTableau{T}) where {T}
    for (make, id) in _BUILTIN_TABLEAUS
        ref = make(T)
        size(ref.a) == size(bt.a) && _same_tableau(bt, ref) && return id
    end
    error("GB300 stepper: the tableau is none of the built-in tableaus (ButcherTableaus.jl:125-263)")
end
_tableau_id(id::Integer) = Int32(id)

_strategy_id(::EPD0) = HCC_EPD0
_strategy_id(::EPD1) = HCC_EPD1
_strategy_id(::EPD2) = HCC_EPD2
_strategy_id(::StrictEPD0) = HCC_STRICT_EPD0
_strategy_id(::MOODStrategy) = HCC_EPD_NONE
_flux_id(::RusanovFlux) = HCC_FLUX_RUSANOV
_flux_id(::AlignedRusanovFlux) = HCC_FLUX_ALIGNED
_flux_id(f) = error("GB300 stepper: unsupported numerical flux $(typeof(f))")
_limiter_id(::NoLimiter) = HCC_LIMITER_NONE
_limiter_id(::BarthJespersenLimiter{:soft}) = HCC_LIMITER_BJ_SOFT
_limiter_id(::BarthJespersenLimiter{:hard}) = HCC_LIMITER_BJ_HARD
_limiter_id(::VenkatakrishnanLimiter{:soft}) = HCC_LIMITER_VK_SOFT
_limiter_id(::VenkatakrishnanLimiter{:hard}) = HCC_LIMITER_VK_HARD
_limiter_id(l) = error("GB300 stepper: unsupported limiter $(typeof(l))")
_criterion(c::MOODu1) = (HCC_MOOD_U1, Float64(c.d))
_criterion(c::MOODu2) = (HCC_MOOD_U2, Float64(c.d))
_criterion(::MOODPAD) = (HCC_MOOD_PAD, 0.0)
_criterion(::OnlyMOOD) = (HCC_MOOD_ONLY, 0.0)
_criterion(::NoMOOD) = (HCC_MOOD_NONE, 0.0)

# pg.geometry.bc_map (tag => condition functor, Domains.jl:27; applied by apply_boundary_conditions!,
# BoundaryConditions.jl:43-48) -> bc_by_tag. The library implements the two conditions the package ships.
_bc_kind(::FixedDirichlet) = HCC_BC_DIRICHLET
_bc_kind(::OutflowBC) = HCC_BC_OUTFLOW
_bc_kind(bc) = error("GB300 stepper: no device implementation of the boundary condition $(typeof(bc))")
function _bc_by_tag(bc_map)
    kinds = fill(HCC_BC_KEEP, 16)
    for (tag, bc) in bc_map
        1 <= tag <= 16 || error("GB300 stepper: boundary tag $tag outside 1..16")
        kinds[tag] = bc isa Integer ? Int32(bc) : _bc_kind(bc)
    end
    return ntuple(t -> kinds[t], 16)
end

# The divergence interpolator -> (scheme, order, div_order, limiter, flux, upwind algorithm, moment correction).
# MUSCL's `streamed` setting selects between two evaluations of the same divergence (MUSCL.jl:426-458); the library
# always streams, so either value is accepted.
function _scheme!(cfg, interp::MUSCL{D, M, T, B_LEN, MAX_ORDER, DIV_ORDER}) where {D, M, T, B_LEN, MAX_ORDER, DIV_ORDER}
    cfg.scheme = HCC_SCHEME_MUSCL
    cfg.muscl_order = MAX_ORDER
    cfg.div_order = DIV_ORDER
    cfg.limiter = _limiter_id(interp.limiter)
    cfg.flux = _flux_id(interp.flux)
    cfg.moment_correction = Int32(interp.moment isa Val{true})
    return cfg
end
function _scheme!(cfg, ::WENO{D, M, T, MAX_ORDER, DIV_ORDER}) where {D, M, T, MAX_ORDER, DIV_ORDER}
    cfg.scheme, cfg.muscl_order, cfg.div_order = HCC_SCHEME_WENO, MAX_ORDER, DIV_ORDER
    return cfg
end
function _scheme!(cfg, ::CentralDivergence{D, M, T, MAX_ORDER, DIV_ORDER}) where {D, M, T, MAX_ORDER, DIV_ORDER}
    cfg.scheme, cfg.muscl_order, cfg.div_order = HCC_SCHEME_CENTRAL, MAX_ORDER, DIV_ORDER
    return cfg
end
_upwind_alg(::Type{<:TiwariAlgorithm}) = HCC_UPWIND_TIWARI
_upwind_alg(::Type{<:PraveenAlgorithm}) = HCC_UPWIND_PRAVEEN
_upwind_alg(A) = error("GB300 stepper: unsupported upwind algorithm $A")
function _scheme!(cfg, u::UpwindDivergence{D, M, T, MAX_ORDER, DIV_ORDER, B_LEN, INTERPS, ALG}) where
        {D, M, T, MAX_ORDER, DIV_ORDER, B_LEN, INTERPS, ALG}
    cfg.muscl_order, cfg.div_order = MAX_ORDER, DIV_ORDER
    cfg.flux = _flux_id(u.flux)
    if ALG <: ClassicAlgorithm             # UpwindDivergence(:Classic) is the first-order MUSCL scheme
        cfg.scheme = HCC_SCHEME_MUSCL
    else
        cfg.scheme = HCC_SCHEME_UPWIND
        cfg.upwind_algorithm = _upwind_alg(ALG)
    end
    return cfg
end
_scheme!(cfg, interp) = error("GB300 stepper: unsupported divergence interpolator $(typeof(interp))")

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

function GB300RKTimeStepper(eq::HyperbolicPDE{D, M, T}, pg::ParticleGrid{D, M, T}, interp, mood::MOOD,
                            tableau; bc_map = nothing, precision::Symbol = :fp64,
                            reset_orders_per_stage::Bool = false, mood_substeps::Bool = true) where {D, M, T}
    cfg = HccConfig()
    cfg.dim, cfg.n_vars, cfg.pde = D, M, hcc_pde_kind(eq)
    cfg.precision = precision === :fp32 ? 1 : 0
    _scheme!(cfg, interp)
    cfg.tableau = _tableau_id(tableau)
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
    # the grid's own conditions; an explicit bc_map (tag => FixedDirichlet() / OutflowBC() or an hcc_bc_kind) replaces them
    cfg.bc_by_tag = _bc_by_tag(bc_map === nothing ? pg.geometry.bc_map : bc_map)
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
# mood_substeps), plus :Precision (:fp64 / :fp32) and, to override the grid's own map, :BCMap.
function build_gb300_timestepper(context::Dict; time_conf::Dict = Dict{Symbol, Any}())
    pg = context[:Grid]::ParticleGrid
    ts = GB300RKTimeStepper(context[:Equation], pg, context[:Scheme], context[:MOOD], context[:Tableau];
                            bc_map = get(context, :BCMap, nothing),
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
