/*
 * hcc.h — C ABI of the GB300 explicit right-hand-side library (libhcc_gb300.so).
 *
 * The library runs the hot path of the meshless solver HyperCloudCore.jl on one GPU:
 * cell-list neighbour search -> MLS moment/divergence weights -> MUSCL reconstruction ->
 * Rusanov flux -> streamed divergence -> SSP-RK / IMEX stage update with MOOD -> CFL time step.
 *
 * Conventions
 *  - Every call returns an hcc_status; hcc_last_error() gives the message of the last failure
 *    of a context (a static string for a NULL context).
 *  - Pointers are HOST pointers; the caller's buffers are read or written only during the call.
 *  - Particle-indexed host arrays use 0-based particle numbers in the caller's order; the library
 *    keeps that numbering (it is the reference's Morton numbering when the caller reorders first).
 *  - Positions and states are row-major: pos[i*D + d], U[i*M + m].
 *  - One CUDA stream per context. A context is not thread-safe; distinct contexts are independent.
 *  - All device memory is owned by the context and sized at hcc_create / hcc_upload_cloud.
 *
 * Reference interfaces each entry point replaces are cited as file:line of HyperCloudCore.jl.
 */
#ifndef HCC_GB300_H
#define HCC_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HCC_ABI_VERSION 1
#define HCC_MAX_DIM 3
#define HCC_MAX_VARS 16
#define HCC_MAX_TAGS 16

typedef enum {
    HCC_OK = 0,
    HCC_ERR_INVALID = 1,     /* bad argument or configuration (ArgumentError in the reference) */
    HCC_ERR_CAPACITY = 2,    /* particle or neighbour count above the reservation (CapacityError) */
    HCC_ERR_CUDA = 3,        /* a CUDA call failed */
    HCC_ERR_STATE = 4,       /* call out of order (e.g. a step before the neighbour search) */
    HCC_ERR_NONFINITE = 5,   /* non-finite time step or state where one is required */
    HCC_ERR_TIMEOUT = 6,     /* an iteration cap was reached (MOOD fixed point) */
    HCC_ERR_UNSUPPORTED = 7  /* a combination this build does not instantiate */
} hcc_status;

/* Physics modules compiled into the kernels (HyperbolicPDE subtypes of the reference). */
typedef enum {
    HCC_PDE_ADVECTION = 0,   /* diagonal linear advection: F_d(U)_m = c[d][m] U_m (test/PDEs/linear_advection.jl:24-32) */
    HCC_PDE_EULER = 1,       /* compressible Euler, ideal gas, M = D + 2 (not in the reference; PAD = rho>0, p>0, finite) */
    HCC_PDE_BGK = 2          /* discrete-velocity kinetic relaxation: advection with speeds v_k + implicit
                                Maxwellian relaxation (test/kinetic_source.jl:67-104) */
} hcc_pde_kind;

typedef enum {
    HCC_FP64 = 0,            /* plain FP64 path */
    HCC_FP32 = 1             /* FP32 bulk: states, reconstruction, fluxes and updates in FP32, Kahan-compensated
                                divergence; MLS assembly and Cholesky stay FP64 */
} hcc_precision;

typedef enum {               /* MOOD criterion (src/TimeStepping/MOOD.jl) */
    HCC_MOOD_NONE = 0,       /* NoMOOD: MOOD() */
    HCC_MOOD_U1 = 1,         /* MOODu1(delta): relaxed DMP + PAD */
    HCC_MOOD_PAD = 2,        /* MOODPAD(): admissibility only */
    HCC_MOOD_ONLY = 3,       /* OnlyMOOD(): flags everything (testing) */
    HCC_MOOD_U2 = 4          /* MOODu2(delta; plateau, ratio): u1 + plateau test + smooth-extremum override from the
                                curvature terms of a degree-2 reconstruction (MOOD.jl:104-130, :223-271) */
} hcc_mood_criterion;

typedef enum {               /* MOOD strategy (interface orders), MOOD.jl:20-28, :76-87 */
    HCC_EPD_NONE = 0,        /* NoStrategy: own orders (o_i, o_j) */
    HCC_EPD0 = 1,            /* (o_i, o_j) */
    HCC_EPD1 = 2,            /* min(o_i, o_j) on both sides */
    HCC_EPD2 = 3,            /* min over N(i) u N(j) on both sides */
    HCC_STRICT_EPD0 = 4      /* (o_i, o_j) + one-hop forcing: the neighbours of a dropped particle are lowered to its
                                order (MOOD.jl:28-64, :312-320) */
} hcc_mood_strategy;

typedef enum {               /* src/TimeStepping/ButcherTableaus.jl */
    HCC_TAB_RK1_EULER = 0, HCC_TAB_RK2_SSP = 1, HCC_TAB_RK2_RALSTON = 2, HCC_TAB_RK3_SSP = 3,
    HCC_TAB_RK4_CLASSICAL = 4, HCC_TAB_RK4_SSP = 5,
    HCC_TAB_IMEX_EULER = 6, HCC_TAB_IMEX_ARS233 = 7, HCC_TAB_IMEX_ARS222 = 8,
    HCC_TAB_IMEX_PRSSP3 = 9, HCC_TAB_IMEX_SSP2332 = 10
} hcc_tableau;

typedef enum {               /* divergence interpolator (src/Interpolation/) */
    HCC_SCHEME_MUSCL = 0,    /* MUSCL (MUSCL.jl), streamed divergence */
    HCC_SCHEME_WENO = 1,     /* meshless WENO, scalar equations only (WENO.jl) */
    HCC_SCHEME_CENTRAL = 2,  /* CentralDivergence (Central.jl): intercept fit of degree = order of F_j - F_i */
    HCC_SCHEME_UPWIND = 3    /* UpwindDivergence (Upwind.jl), scalar advection, order 1, `upwind_algorithm` below
                                (:Classic is the first-order MUSCL scheme: HCC_SCHEME_MUSCL with muscl_order 1) */
} hcc_scheme;

typedef enum {               /* UpwindDivergence algorithms (Upwind.jl) */
    HCC_UPWIND_TIWARI = 1,   /* per axis: the gradient fit on the upwind side (v_d x_d <= 0), times v_d */
    HCC_UPWIND_PRAVEEN = 2   /* 2-D: edge-normal / tangential upwind coefficients from the local moment matrix */
} hcc_upwind_algorithm;

typedef enum {               /* slope limiters of the MUSCL pre-pass (Limiter.jl) */
    HCC_LIMITER_NONE = 0,    /* NoLimiter */
    HCC_LIMITER_BJ_SOFT = 1, /* BarthJespersenLimiter(:soft): limits the first-degree terms */
    HCC_LIMITER_BJ_HARD = 2, /* BarthJespersenLimiter(:hard): limits every term */
    HCC_LIMITER_VK_SOFT = 3, /* VenkatakrishnanLimiter(:soft) */
    HCC_LIMITER_VK_HARD = 4  /* VenkatakrishnanLimiter(:hard) */
} hcc_limiter;

typedef enum {               /* numerical flux of MUSCL (FluxFunctions.jl) */
    HCC_FLUX_RUSANOV = 0,    /* RusanovFlux: states sorted per axis by the sign of the distance */
    HCC_FLUX_ALIGNED = 1     /* AlignedRusanovFlux: sorted by the sign of the slot's divergence weight where either
                                particle is below the full order (and on every pair of a first-order scheme) */
} hcc_flux;

typedef enum {               /* src/Grid/BoundaryConditions.jl */
    HCC_BC_KEEP = 0,         /* no condition for the tag: the particle keeps its start-of-step state */
    HCC_BC_DIRICHLET = 1,    /* FixedDirichlet */
    HCC_BC_OUTFLOW = 2       /* OutflowBC: nearest resolved donor, <= 5 passes */
} hcc_bc_kind;

/* Plain-old-data configuration. Zero-initialise, then fill. */
typedef struct {
    int32_t abi_version;               /* HCC_ABI_VERSION */
    int32_t dim;                       /* D in {1,2,3} */
    int32_t n_vars;                    /* M */
    int32_t pde;                       /* hcc_pde_kind */
    int32_t precision;                 /* hcc_precision */
    int32_t muscl_order;               /* MUSCL max_order in {1,2,3} (MUSCL.jl:116) */
    int32_t div_order;                 /* MUSCL div_order (0 = adaptive) */
    int32_t mood_criterion;            /* hcc_mood_criterion */
    int32_t mood_strategy;             /* hcc_mood_strategy */
    int32_t tableau;                   /* hcc_tableau */
    int32_t mood_substeps;             /* 1: check the Euler substeps of SSP tableaus (default of the reference) */
    int32_t periodic[HCC_MAX_DIM];     /* per axis */
    int32_t bc_by_tag[HCC_MAX_TAGS];   /* hcc_bc_kind per boundary tag 1..16 (index tag-1) */
    int32_t max_mood_iterations;       /* cap of the MOOD fixed point per checkpoint (0 -> 64) */
    int32_t scheme;                    /* hcc_scheme */
    int32_t limiter;                   /* hcc_limiter (MUSCL only) */
    int32_t slot_capacity;             /* neighbours per particle the lists may hold (0: no limit) */
    int32_t flux;                      /* hcc_flux (MUSCL numerical flux) */
    int32_t reset_orders_per_stage;    /* 1: restore the maximum order before each stage's full pass */
    int32_t upwind_algorithm;          /* hcc_upwind_algorithm (HCC_SCHEME_UPWIND) */
    int32_t moment_correction;         /* MUSCL(...; moment_correction = true): first-order schemes only (MUSCL.jl:57) */
    int32_t reserved_i[1];
    double  dx[HCC_MAX_DIM];           /* nominal spacing per axis; h = min(dx) scales the MLS basis */
    double  radius;                    /* support radius R of ExponentialWeightFunction */
    double  weight_alpha;              /* alpha of ExponentialWeightFunction (MLSWeightFunctions.jl:79-82) */
    double  canvas_min[HCC_MAX_DIM];   /* box of the cell list (ghost canvas) */
    double  canvas_max[HCC_MAX_DIM];
    double  domain_min[HCC_MAX_DIM];   /* physical box (periodic wrap length = domain_max - domain_min) */
    double  domain_max[HCC_MAX_DIM];
    double  mood_delta;                /* delta of MOODu1 */
    double  velocity[HCC_MAX_DIM][HCC_MAX_VARS]; /* advection speeds c[d][m]; BGK: kinetic speeds v_k,d */
    double  gamma;                     /* Euler adiabatic index */
    double  bgk_epsilon;               /* BGK relaxation time */
    double  bgk_macro_velocity[HCC_MAX_DIM]; /* BGK macro flux: scalar linear advection with this velocity */
    double  bgk_coefficient;           /* Maxwellian coefficient of the single macro moment (1/NK) */
    double  bgk_interior_factor;       /* RelaxationSourceTerm interior_factor (default D) */
    double  u2_plateau;                /* MOODu2 plateau (default 1e-3; 0 disables the plateau test) */
    double  u2_ratio;                  /* MOODu2 curvature ratio (default 0.5; 0 disables the magnitude test) */
    double  reserved_d[6];
} hcc_config;

typedef struct {
    int64_t n_particles;
    int64_t n_interior;
    int32_t max_neighbours;
    int32_t min_neighbours_interior;
    int64_t total_neighbours;
    int64_t mood_iterations;           /* MOOD recompute passes in the last step */
    int64_t mood_flagged;              /* particles that dropped an order in the last step (mood_flags) */
    int64_t inadmissible;              /* mood_inadmissible(ts) of the last step (TimeSteppers.jl:272) */
    int64_t kernel_launches;           /* kernels launched by the last hcc_step / hcc_time_step */
    int64_t steps;                     /* steps taken by the context */
    int64_t kernel_launches_total;     /* kernels launched since the context was created */
    int64_t graph_steps;               /* steps taken as one captured CUDA graph (hcc_set_step_graphs) */
    int64_t predicted;                 /* particles the troubled-point predictor pre-lowered in the last step */
} hcc_counters;

typedef struct hcc_ctx hcc_ctx;

/* Fills *cfg with the reference's defaults (MUSCL 2, SSP-RK3, EPD1/MOODu1, alpha 1, mood_substeps 1). */
void hcc_config_defaults(hcc_config *cfg);

/* Context = GeneralRKTimeStepper(pde, MUSCL(...; storage), MOOD(...), tableau) (TimeSteppers.jl:195-229)
   + the ParticleGrid metadata (ParticleGrids.jl:221-279). `capacity` reserves particles (MemoryBudget.jl:110). */
hcc_status hcc_create(const hcc_config *cfg, int64_t capacity, hcc_ctx **out);
hcc_status hcc_destroy(hcc_ctx *ctx);
const char *hcc_last_error(const hcc_ctx *ctx);
const char *hcc_status_string(hcc_status s);

/* Device copy of the cloud: device_grid(ArrayType, pg) (DeviceAdapt.jl:73). pos: N*D, is_boundary: N (0/1),
   tags: N, volumes: N (may be NULL -> prod(dx)). */
hcc_status hcc_upload_cloud(hcc_ctx *ctx, int64_t n, const double *pos, const uint8_t *is_boundary,
                            const int32_t *tags, const double *volumes);

/* Neighbour search: (nd::NeighborData)(pg) (NeighborLogic.jl:235-274) with the cell list of
   build_global_bins! (:116-136). Slot-major device layout (_slot_range, :182). */
hcc_status hcc_build_neighbours(hcc_ctx *ctx);

/* Neighbour lists in the reference's row-major order (ranges as counts, NeighborLogic.jl:282):
   counts[N]; then idx/w/dist of total_neighbours slots (dist: total*D). Any output may be NULL. */
hcc_status hcc_download_neighbours(hcc_ctx *ctx, int32_t *counts, int32_t *idx, double *w, double *dist);

/* The lists of n_sel selected particles (the per-particle slot views pg.neighbor.indices[ranges[i]] of
   NeighbourViews.jl:11-43 / NeighborLogic.jl:182), for inspecting a large cloud without downloading every list:
   counts[q] = the full count of particle ids[q]; its first min(count, max_slots) slots in idx[q*max_slots + k],
   w[q*max_slots + k], dist[(q*max_slots + k)*dim + d]; the slots of a row past the count are zero. Any output
   may be NULL. */
hcc_status hcc_download_neighbours_of(hcc_ctx *ctx, int64_t n_sel, const int64_t *ids, int32_t max_slots,
                                      int32_t *counts, int32_t *idx, double *w, double *dist);

/* prepare_geometry!(muscl, pg) (MUSCL.jl:172-187): cached inverse moments, ok flags, per-slot
   divergence weights (update_divergence_weights!, MUSCL.jl:197-223) and the outflow donor map. */
hcc_status hcc_prepare_geometry(hcc_ctx *ctx);

/* Per-slot divergence weights (dweights), row-major like hcc_download_neighbours: total*D. ok_r/ok_d: N each. */
hcc_status hcc_download_geometry(hcc_ctx *ctx, double *dweights, uint8_t *ok_recon, uint8_t *ok_div);

/* pg.rhos (N*M). FP32 contexts convert. */
hcc_status hcc_upload_state(hcc_ctx *ctx, const double *U);
hcc_status hcc_download_state(hcc_ctx *ctx, double *U);
hcc_status hcc_upload_state_f32(hcc_ctx *ctx, const float *U);
hcc_status hcc_download_state_f32(hcc_ctx *ctx, float *U);

/* get_time_step(pg, eq, interp) (ParticleGrids.jl:386-415): CFL number 1, cached slot weights. */
hcc_status hcc_time_step(hcc_ctx *ctx, double *dt_out);

/* One explicit right-hand side K = -2 div + sources at the current state, all particles at full order:
   compute_explicit_rhs!(..., full = true) (TimeSteppers.jl:312-356). K: N*M. */
hcc_status hcc_compute_rhs(hcc_ctx *ctx, double *K);

/* Grid movers (GridMovers.jl): positions become stage variables of the tableau (explicit part), the flux is taken in
   the frame of each particle's grid velocity w (ALEFrame: F - w U, wave speeds shifted), distances, weights and MLS
   caches are refreshed at every stage position with the start-of-step topology (or a full search per stage), and a
   full neighbour search (with periodic re-wrap) follows every step. No counterpart for PrescribedMover's arbitrary
   Julia function: the prescribed field here is w(x) = velocity + omega x (x - center). */
typedef enum {
    HCC_MOVER_NONE = 0,        /* NoGridMover */
    HCC_MOVER_LAGRANGIAN = 1,  /* LagrangianMover: w = fluid_velocity(eq, U) (scalar advection, Euler) */
    HCC_MOVER_SCALED = 2,      /* ScaledLagrangianMover(alpha): w = alpha fluid_velocity(eq, U) */
    HCC_MOVER_PRESCRIBED = 3   /* PrescribedMover: w = velocity + omega x (x - center) (2-D: omega[2] about z) */
} hcc_mover_kind;

typedef struct {
    int32_t kind;                      /* hcc_mover_kind */
    int32_t full_search_per_stage;     /* 1: rebuild the neighbour topology at every stage position */
    double alpha;                      /* ScaledLagrangianMover */
    double velocity[HCC_MAX_DIM];      /* prescribed translation */
    double omega[HCC_MAX_DIM];         /* prescribed angular velocity */
    double center[HCC_MAX_DIM];        /* centre of the prescribed rotation */
    int32_t keep_volumes;              /* 1: volume_estimator = nothing; 0 (default): ShepardVolumes after each step */
    int32_t shepard_sweeps;            /* sweeps of ShepardVolumes (0 -> 1, the reference's default) */
} hcc_mover;

/* Select the grid mover of the context (default HCC_MOVER_NONE); before hcc_step. */
hcc_status hcc_set_mover(hcc_ctx *ctx, const hcc_mover *mover);

/* Current particle positions (N x D row-major, the caller's numbering; moved by hcc_step on moving grids). */
hcc_status hcc_download_positions(hcc_ctx *ctx, double *pos);

/* Checkpoint / resume. hcc_save_snapshot writes the context's particle positions, state (in its precision), orders
   and MOOD flags of the last step and its step count to a binary file; hcc_load_snapshot reads one written by a
   context of the same configuration (dim, n_vars, pde, precision) and particle count, rebuilds the neighbour lists
   and geometry at the saved positions and restores the rest. No counterpart in the reference. */
hcc_status hcc_save_snapshot(hcc_ctx *ctx, const char *path);
hcc_status hcc_load_snapshot(hcc_ctx *ctx, const char *path);

/* One time step: (ts::GeneralRKTimeStepper)(eq, pg, t, dt) (TimeSteppers.jl:531-577). */
hcc_status hcc_step(hcc_ctx *ctx, double t, double dt);

/* Run hcc_step as one captured CUDA graph (default on): each MOOD fixed point is a conditional WHILE node decided
   on the device, with no host wait inside the step. Off: the host drives the fixed points (one counter read per
   drop pass). Both give identical results; steps taken while profiling is on always use the host-driven form.
   No counterpart in the reference (its loop is host-driven, TimeSteppers.jl:454-477). */
hcc_status hcc_set_step_graphs(hcc_ctx *ctx, int enable);

/* pg.core.particle_orders (N) and mood_flags(ts) (TimeSteppers.jl:258) of the last step. */
hcc_status hcc_download_orders(hcc_ctx *ctx, int32_t *orders);
hcc_status hcc_download_mood_flags(hcc_ctx *ctx, uint8_t *flags);

hcc_status hcc_get_counters(hcc_ctx *ctx, hcc_counters *out);

/* update_volumes!(pg, ShepardVolumes(sweeps)) (Volumes.jl:183-240): S_i = w(0) + sum_j w_ij, V_i = 1 / S_i,
   `sweeps` partition-of-unity sweeps V_i <- (w(0)/S_i) V_i + sum_j (w_ij / S_j) V_j, negatives clamped to 0 and
   sum V rescaled to the box volume prod(domain_max - domain_min). Moving grids run it after every step unless the
   mover keeps the volumes. hcc_download_volumes: the current V (N). */
hcc_status hcc_update_volumes(hcc_ctx *ctx, int32_t sweeps);
hcc_status hcc_download_volumes(hcc_ctx *ctx, double *volumes);

/* total_mass(pg) (Volumes.jl:103-107) accumulated in FP64 on the device: out[M]. */
hcc_status hcc_total_mass(hcc_ctx *ctx, double *out);

/* Per-kernel device time of the steps taken while profiling is on (CUDA events around every gather and flux
   launch on the context's stream). No counterpart in the reference (it times whole steps with @elapsed,
   benchmark/step.jl:77). */
typedef struct {
    double gather_ms;            /* full reconstruction passes */
    int64_t gather_launches;
    double flux_ms;              /* full flux passes */
    int64_t flux_launches;
    double recompute_ms;         /* MOOD recompute passes (masked gather + flux) */
    int64_t recompute_launches;
    int64_t steps;
    double predict_ms;           /* troubled-point predictor (feature pass + network), when one is attached */
    int64_t predict_launches;
} hcc_kernel_times;
hcc_status hcc_set_profiling(hcc_ctx *ctx, int enable);
hcc_status hcc_get_kernel_times(hcc_ctx *ctx, hcc_kernel_times *out, int reset);

/* Batched ensemble: many independent clouds of the same configuration (physics, spacing, radius, scheme) advanced
   by one context — one cell list, one set of passes, one captured step graph — with no communication between the
   clouds. No counterpart in the reference (one ParticleGrid per run). The clouds (concatenated; cloud c is
   [offsets[c], offsets[c+1])) come in their own frames; the library packs their bounding boxes side by side
   (shelf packing, tallest first) with gaps of two support radii, so that no particle has a neighbour in another
   cloud, sets the context's canvas to the union and uploads it. shifts[c*dim + d] (may be NULL) receives the
   translation applied to cloud c, canvas[0..2*dim) (may be NULL) the union box (min then max). Non-periodic
   configurations only. Afterwards the context behaves as with hcc_upload_cloud on the union (same particle
   numbering: cloud by cloud); every step uses one dt for all clouds (the minimum CFL step of the union). */
hcc_status hcc_upload_batch(hcc_ctx *ctx, int32_t n_clouds, const int64_t *offsets, const double *pos,
                            const uint8_t *is_boundary, const int32_t *tags, const double *volumes, double *shifts,
                            double *canvas);

/* The packing hcc_upload_batch applies, on the host only (no context, no GPU): shifts[c*dim + d] and the union box
   canvas[0..2*dim) for clouds of `dim`-D positions with support `radius`. HCC_ERR_INVALID for bad arguments,
   HCC_ERR_NONFINITE for a non-finite position. */
hcc_status hcc_batch_layout(int32_t dim, double radius, int32_t n_clouds, const int64_t *offsets, const double *pos,
                            double *shifts, double *canvas);

/* Per-cloud time steps of a batch (the reference advances every ParticleGrid with its own get_time_step,
   ParticleGrids.jl:386-415): dt_out[c] = the CFL step of cloud c (hcc_time_step restricted to its particles; the
   minimum over the batch is what hcc_time_step returns). */
hcc_status hcc_batch_time_steps(hcc_ctx *ctx, double *dt_out);

/* One step of every cloud of a batch, cloud c with its own dts[c] (the candidates, implicit parts and substeps of
   each particle use its cloud's coefficients); otherwise as hcc_step. */
hcc_status hcc_batch_step(hcc_ctx *ctx, double t, const double *dts);

/* total_mass per cloud of the last hcc_upload_batch: out[c*M + m] (FP64 accumulation on the device). */
hcc_status hcc_batch_total_mass(hcc_ctx *ctx, double *out);

/* CFL time step of caller-owned device arrays WITHOUT allocating device memory. No counterpart in the reference.
   For callers that cannot allocate GPU memory when they need a time step: a code that reserves its device memory
   up front and then freezes it, or one that routes all device memory through its own pool and forbids
   cudaMalloc/cudaFree inside its time loop. Same value as hcc_time_step (ParticleGrids.jl:386-450 arithmetic, FP64).
   Inputs are DEVICE pointers in the library's slot-major layout: counts[n], nidx[k*npad + i],
   dweights[(k*dim + d)*npad + i], is_boundary[n], U[i*n_vars + m] (FP64); physics parameters come from cfg
   (pde, dim, n_vars, velocity, gamma). Supported shapes (pde: dim, n_vars): HCC_PDE_EULER: (1, 3), (2, 4), (3, 5);
   HCC_PDE_ADVECTION and HCC_PDE_BGK: (1, 1), (2, 1), (3, 1), (2, 2), (2, 16), (1, 2); any other shape returns
   HCC_ERR_UNSUPPORTED. stream is a cudaStream_t of the CURRENT device (NULL = default stream; a stream of another
   device returns HCC_ERR_INVALID); *dt_out is written on return (the call synchronises the stream). A runtime error
   left pending by an earlier, unrelated CUDA call is consumed on entry; HCC_ERR_CUDA reports this call's own
   launch or copy failure.
   Scratch: a fixed file-scope device array (about 512 KiB on every GPU where the library's no-allocation module is
   loaded, held until the process exits); n above HCC_NOALLOC_MAX_PARTICLES returns HCC_ERR_CAPACITY. All calls
   share it: calls that overlap on the GPU race and must be serialised by the caller.
   First call: under CUDA's lazy module loading (the default) the first call on a device loads the module that holds
   the scratch array and the kernels, and that load can allocate device memory; it also looks up the array's device
   address (a CUDA runtime query). Make one call with n > 0, for each shape used, on each device before the caller's
   memory is frozen and before any stream capture; calls after that allocate nothing. */
#define HCC_NOALLOC_MAX_PARTICLES (65536 * 256)
hcc_status hcc_cfl_time_step_noalloc(const hcc_config *cfg, int64_t n, int64_t npad, const int32_t *counts,
                                     const int32_t *nidx, const double *dweights, const uint8_t *is_boundary,
                                     const double *U, void *stream, double *dt_out);

/* ------------------------------------------------------------------ learned troubled-point predictor
   No counterpart in the reference (its MOOD loop computes every particle at full order first, MOOD.jl:375-405).
   A small MLP (24 -> 64 -> 64 -> 1, GELU with a polynomial normal CDF, BF16 weights and activations on the tensor
   cores, FP32 accumulate)
   reads 24 stencil features of the start-of-step state and pre-lowers the order of the particles it predicts to be
   troubled (one order, as a MOOD drop), before the step's first reconstruction. Full MOOD still runs on every
   particle as the judge; the predictor only saves recompute passes. The network is trained on the device (forward
   and backward kernels, Adam) on (feature, MOOD-flag) pairs the solver itself generates.

   Features, per particle i, from its neighbours j (offsets x_ij) and four quantities q (Euler: density,
   rho E - |m|^2 / 2 (= rho p / (gamma - 1)), |m|^2, total energy E; other systems: components 0..3, the last
   repeated), six per quantity, in FP32:
   range / (|max| + |min|), (2 q_i - max - min) / range, (q_i - mean_j q_j) / range, RMS residual of the
   least-squares linear fit / range, |gradient| h / range, RMS deviation / range; max/min over {i} + N(i); the last
   five are 0 where range <= 1e-6 (|max| + |min|); every feature is clamped to [-8, 8] (NaN -> 0). */
#define HCC_MLP_FEATURES 24
#define HCC_MLP_HIDDEN 64
/* Flat FP32 parameter vector: W1[64][24], b1[64], W2[64][64], b2[64], w3[64], b3 (z1 = W1 x + b1, ...). */
#define HCC_MLP_NPARAMS (64 * 24 + 64 + 64 * 64 + 64 + 64 + 1)

typedef struct hcc_mlp hcc_mlp;

typedef struct {
    int64_t capacity;        /* training rows held on the device */
    double neg_keep;         /* fraction of unflagged interior particles kept by hcc_mlp_collect (flagged: all) */
    uint64_t seed;           /* negative sampling and mini-batch draws */
    double lr, beta1, beta2, adam_eps;   /* Adam */
    double pos_weight;       /* weight of the flagged class in the binary cross-entropy */
    double reserved[4];
} hcc_mlp_config;

hcc_status hcc_mlp_create(const hcc_mlp_config *cfg, hcc_mlp **out);
void hcc_mlp_destroy(hcc_mlp *mlp);
const char *hcc_mlp_last_error(const hcc_mlp *mlp);

/* Parameters (HCC_MLP_NPARAMS FP32, the master copy Adam updates) and the input normalisation
   (mean[24], inv_std[24]: x' = (x - mean) * inv_std). Setting parameters resets Adam. */
hcc_status hcc_mlp_get_params(hcc_mlp *mlp, float *params, float *norm);
hcc_status hcc_mlp_set_params(hcc_mlp *mlp, const float *params, const float *norm);

/* Training set. hcc_mlp_collect appends the features the context computed at the start of its last step (see
   hcc_set_feature_capture) with that step's MOOD flags as labels; hcc_mlp_add_rows appends host rows
   (X[n][24], y[n]). hcc_mlp_rows reports the rows held and how many are flagged. hcc_mlp_clear empties it. */
hcc_status hcc_mlp_collect(hcc_mlp *mlp, hcc_ctx *ctx);
hcc_status hcc_mlp_add_rows(hcc_mlp *mlp, const float *X, const uint8_t *y, int64_t n);
hcc_status hcc_mlp_rows(hcc_mlp *mlp, int64_t *rows, int64_t *flagged);
hcc_status hcc_mlp_clear(hcc_mlp *mlp);

/* Normalisation from the training rows [0, (1 - holdout) rows): mean and 1/std per feature. */
hcc_status hcc_mlp_fit_norm(hcc_mlp *mlp, double holdout);

/* iters Adam steps on mini-batches of `batch` rows drawn from [0, (1 - holdout) rows); *loss_out = mean loss of the
   last mini-batch. */
hcc_status hcc_mlp_train(hcc_mlp *mlp, int64_t iters, int64_t batch, double holdout, double *loss_out);

/* Confusion counts {tp, fp, fn, tn} of the rows [(1 - holdout) rows, rows) at probability threshold thr. */
hcc_status hcc_mlp_evaluate(hcc_mlp *mlp, double thr, double holdout, int64_t *counts);

/* One forward/backward pass on host rows without an update: the mean loss and its gradient (HCC_MLP_NPARAMS). */
hcc_status hcc_mlp_loss_grad(hcc_mlp *mlp, const float *X, const uint8_t *y, int64_t n, float *grad, double *loss);

/* Logits of host rows X[n][24] through the inference kernel. */
hcc_status hcc_mlp_predict_rows(hcc_mlp *mlp, const float *X, int64_t n, float *logits);

/* Attach a predictor to a context (NULL detaches): every hcc_step then pre-lowers the particles whose predicted
   probability exceeds thr. The predictor must outlive the attachment. */
hcc_status hcc_set_predictor(hcc_ctx *ctx, hcc_mlp *mlp, double thr);

/* Keep the start-of-step features of every step (for hcc_mlp_collect / hcc_download_features). */
hcc_status hcc_set_feature_capture(hcc_ctx *ctx, int enable);

/* Features (N x 24) of the current state (the start state of the next step), and the particles the predictor
   pre-lowered in the last step (N, 0/1). */
hcc_status hcc_download_features(hcc_ctx *ctx, float *features);
hcc_status hcc_download_predicted(hcc_ctx *ctx, uint8_t *predicted);

/* Launch shapes of a step. They change no result: every particle is computed by the same code whatever the grid
   (the results are bit-identical across shapes). No counterpart in the reference (KernelAbstractions picks its
   workgroup size at launch). */
typedef struct hcc_tuning {
    int32_t flux_block;          /* threads per block of the full flux pass (and the other schemes' full passes):
                                    32, 64, 96 or 128; default 128 */
    int32_t gather_block;        /* threads per block of the full reconstruction pre-pass: 32..128 step 32; 128 */
    int32_t list_blocks_per_sm;  /* grid of the MOOD worklist (recompute) passes, blocks per SM: 1..32; 8 */
    int32_t drop_blocks_per_sm;  /* grid of the MOOD decision pass, blocks per SM: 1..32; 2 */
} hcc_tuning;

typedef struct hcc_tune_report {
    hcc_tuning best;             /* the shapes kept (applied to the context) */
    double default_ms;           /* ms per step with the shapes in place when the tuner started */
    double best_ms;              /* ms per step with `best` */
    int32_t candidates;          /* configurations timed */
    int32_t steps;               /* timed steps per configuration (after one warm-up step) */
} hcc_tune_report;

hcc_status hcc_get_tuning(hcc_ctx *ctx, hcc_tuning *out);
/* HCC_ERR_INVALID for a value outside the ranges above. Drops the captured step graphs. */
hcc_status hcc_set_tuning(hcc_ctx *ctx, const hcc_tuning *tuning);

/* The project's autotuner: coordinate descent over the four shapes (flux block {128, 96, 64}, gather block
   {128, 64}, worklist blocks per SM {8, 4, 16, 2}, decision blocks per SM {2, 1, 4}), each configuration timed
   with CUDA events over `steps` steps of size dt (the context's own step path: captured graph or host-driven)
   from the current state after one warm-up step; a change is kept when it is at least 1 % faster. The state,
   the step counters and the predictor's rough-tile marks are restored afterwards, so the next hcc_step computes
   what it would have without tuning. Needs an uploaded state; HCC_ERR_STATE on a moving grid (its steps move the
   particles). `report` may be NULL. */
hcc_status hcc_autotune(hcc_ctx *ctx, double dt, int32_t steps, hcc_tune_report *report);

/* The compile-time launch bounds and variant switches the library was built with, e.g. "flux_block=128
   flux_minb=7 flux_minb_wide=4 flux_minb64=3 flux_minb_many=2 fp32_packed=0 tile_flux_pf=8 tile_stage_unroll=4
   flux_kahan_block=4 tile_flux_group=2 tile_gather_group=8" (static string; no GPU
   needed). Tells apart variant builds loaded side by side. */
const char *hcc_build_info(void);

/* Tile staging of the FP32 full passes (no counterpart in the reference; the reference's gather and flux loops read
   neighbours through the slot views, NeighbourViews.jl:11-43). For an FP32 context with MUSCL of order <= 2, the
   degree-1 divergence fit, EPD0/EPD1/StrictEPD0 interface orders and a fixed grid, hcc_prepare_geometry also builds
   tile tables: per tile of 128 consecutive particles the union of their neighbours, which one thread block stages in
   shared memory, and per slot the neighbour's place in it; the full passes then recompute the slot offsets, weights
   and divergence / gradient weights from quantised positions and per-particle FP32 fit rows instead of reading the
   per-slot streams. Results agree with the stream-fed passes to FP32 rounding (both round the same FP64 geometry).
   Enabled by default for 3-D contexts (about 66 neighbours a particle: faster than the stream-fed passes), off by
   default for 1-D and 2-D ones (about 19 neighbours: slower); enable = 1 / 0 chooses either way. */
hcc_status hcc_set_tile_staging(hcc_ctx *ctx, int32_t enable);
/* Whether the full passes of the next step are tile-staged, the union entries over all tiles and the largest union
   (any output may be NULL). */
hcc_status hcc_get_tile_staging(hcc_ctx *ctx, int32_t *active, int64_t *union_entries, int32_t *largest_union);

/* Calibration, no counterpart in the reference: the FP64 FMA rate of the current GPU in TFLOP/s (an FMA counts 2),
   from chains of dependent FMAs on every SM timed with CUDA events on the default stream (allocates 8 bytes). The
   denominator of the FP64 path's roofline (the GPU's FP64 units are a small fraction of its FP32 ones). */
hcc_status hcc_fp64_fma_rate(double *tflops_out);

/* Waits for the context's stream. */
hcc_status hcc_synchronize(hcc_ctx *ctx);

/* The context's CUDA stream (cudaStream_t) so a caller can time or order work on it. */
void *hcc_stream(hcc_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* HCC_GB300_H */
