/*
 * oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement (C++17, OpenMP over particles) of HyperCloudCore.jl's explicit right-hand-side path,
 * used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference legs as the
 * checker. The product (libhcc_gb300.so) never links, loads or calls it.
 *
 * Parity pinning: the reference is Julia and cannot run in this environment. The restatement is pinned to
 * the reference's own known-answer tests (test/unit_core.jl, test/unit_schemes.jl: exact linear divergence,
 * zero-sum divergence weights, neighbour counts vs brute force, interface orders, mask expansion, MOOD
 * termination, SSP coefficients, CFL host formula, streamed vs buffered, cached vs direct), ported in
 * tests/test_oracle_kat.py. No reference-run golden vectors exist.
 *
 * The entry points mirror include/hcc.h with an orc_ prefix and the same argument meaning.
 */
#ifndef HCC_ORACLE_H
#define HCC_ORACLE_H
#include "../include/hcc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

hcc_status orc_create(const hcc_config *cfg, orc_ctx **out);
hcc_status orc_destroy(orc_ctx *ctx);
const char *orc_last_error(const orc_ctx *ctx);
hcc_status orc_set_threads(int n);
hcc_status orc_upload_cloud(orc_ctx *ctx, int64_t n, const double *pos, const uint8_t *is_boundary,
                            const int32_t *tags, const double *volumes);
hcc_status orc_build_neighbours(orc_ctx *ctx);
hcc_status orc_neighbour_total(orc_ctx *ctx, int64_t *total, int32_t *max_nb);
hcc_status orc_download_neighbours(orc_ctx *ctx, int32_t *counts, int32_t *idx, double *w, double *dist);
hcc_status orc_download_positions(orc_ctx *ctx, double *pos);
/* Neighbour counts of every particle (pass 1 of the search only, no lists kept). */
hcc_status orc_neighbour_counts(orc_ctx *ctx, int32_t *counts);
/* The lists of n_sel selected particles in the reference's order: row q holds particle ids[q]'s slots
   idx[q*max_slots + k], w[q*max_slots + k], dist[(q*max_slots + k)*D + d] (zero past the count); counts[q].
   HCC_ERR_CAPACITY when a count exceeds max_slots. The cell list covers the whole cloud; no other list is kept. */
hcc_status orc_neighbours_of(orc_ctx *ctx, int64_t n_sel, const int64_t *ids, int32_t max_slots, int32_t *counts,
                             int32_t *idx, double *w, double *dist);
hcc_status orc_prepare_geometry(orc_ctx *ctx);
hcc_status orc_download_geometry(orc_ctx *ctx, double *dweights, uint8_t *ok_recon, uint8_t *ok_div);
hcc_status orc_upload_state(orc_ctx *ctx, const double *U);
hcc_status orc_download_state(orc_ctx *ctx, double *U);
hcc_status orc_time_step(orc_ctx *ctx, double *dt_out);
hcc_status orc_compute_rhs(orc_ctx *ctx, double *K);
/* The same with given particle orders (starved lowering still applies). */
hcc_status orc_compute_rhs_orders(orc_ctx *ctx, const int32_t *orders, double *K);
hcc_status orc_step(orc_ctx *ctx, double t, double dt);
hcc_status orc_download_orders(orc_ctx *ctx, int32_t *orders);
hcc_status orc_upload_orders(orc_ctx *ctx, const int32_t *orders);
hcc_status orc_download_mood_flags(orc_ctx *ctx, uint8_t *flags);
hcc_status orc_get_counters(orc_ctx *ctx, hcc_counters *out);
hcc_status orc_total_mass(orc_ctx *ctx, double *out);
/* 1: streamed divergence (MUSCL(...; streamed = true), the library's path); 0: buffered fit (reference default). */
hcc_status orc_set_streamed(orc_ctx *ctx, int streamed);

/* Gradients of the last gather pass: N * Br * M. */
hcc_status orc_download_gradients(orc_ctx *ctx, double *g, int32_t *br_out);

/* ---- kernels-level helpers for the known-answer tests (no context) ---- */
/* SSP coefficient of a built-in tableau (ButcherTableaus.jl:86-118). */
double orc_ssp_coefficient(int32_t tableau);
/* basis_count(D, degree) (Interpolators.jl:170-177). */
int32_t orc_basis_count(int32_t D, int32_t degree);
/* _div_idx / _divergence_index (MUSCL.jl:11-32). */
int32_t orc_div_idx(int32_t D, int32_t o);
int32_t orc_divergence_index(int32_t DO, int32_t D, int32_t p_order, int32_t num_nb);
/* Exponent table of the MLS basis (Interpolators.jl:138-155): exps[B*D]; returns B. */
int32_t orc_basis_exponents(int32_t D, int32_t degree, int32_t *exps);
/* MLS divergence Σ_d ∂_d F_d of per-slot flux differences with the intercept fit of degree q
   (Interpolator{D,q,1} functor, Interpolators.jl:290-334). dists: K*D, w: K, dF: K*D*M (d-major per slot).
   out: M. Returns 1 if the factorisation succeeded. */
int32_t orc_mls_divergence(int32_t D, int32_t M, int32_t q, int32_t K, const double *dists, const double *w,
                           const double *dF, double scale, double *out);
/* MLS gradient fit (_mls_solve, Interpolators.jl:372-400): out: B*M coefficients (scaled). Returns ok. */
int32_t orc_mls_solve(int32_t D, int32_t M, int32_t q, int32_t K, const double *dists, const double *w,
                      const double *df, double scale, double *out);
/* _cholesky_moment (Interpolators.jl:46-64) of an explicit B×B matrix: writes U (row-major B×B),
   returns 1 if ok; *plain_ok = 1 if the unregularised factorisation passed the pivot test. */
int32_t orc_cholesky_moment(int32_t B, const double *Nmat, double *U, int32_t *plain_ok);
/* Expand a particle mask by `hops` (MOOD.jl:323-351) on the context's neighbour lists. */
hcc_status orc_expand_mask(orc_ctx *ctx, uint8_t *mask, int32_t hops);
/* Interface orders of an edge (MOOD.jl:76-87) with the context's strategy and current orders. */
hcc_status orc_interface_orders(orc_ctx *ctx, int64_t i, int64_t j, int32_t *oi, int32_t *oj);
/* detect_and_drop! (MOOD.jl:375-405) against explicit prev/cand states; dirty may be NULL (full). */
hcc_status orc_detect_and_drop(orc_ctx *ctx, const double *prev, const double *cand, int32_t full,
                               const uint8_t *dirty, int32_t with_eq, int32_t *changed_any);
/* Stencil features of the learned troubled-point predictor of the current state (N x 24, FP32; definitions in
   include/hcc.h), and the particles the next orc_step pre-lowers by one order (NULL: none). */
hcc_status orc_features(orc_ctx *ctx, float *out);
hcc_status orc_set_prelowered(orc_ctx *ctx, const uint8_t *mask);
/* update_volumes!(pg, ShepardVolumes(sweeps)) (Volumes.jl:183-229) and the current volumes (N). */
hcc_status orc_update_volumes(orc_ctx *ctx, int32_t sweeps);
hcc_status orc_download_volumes(orc_ctx *ctx, double *volumes);
/* Grid mover of the context (GridMovers.jl). */
hcc_status orc_set_mover(orc_ctx *ctx, const hcc_mover *mover);
/* The MOOD criterion of particle p (MOOD.jl:175-271) for hand-set stage states (N*M), gradients (N*Br*M), orders
   and a candidate (M): *flag = 1 if flagged. */
hcc_status orc_criterion_flags(orc_ctx *ctx, int64_t p, const double *prev, const double *grads, const int32_t *orders,
                               const double *cand, int32_t *flag);
/* apply_boundary_conditions! (BoundaryConditions.jl:43-130) on buf (N*M) with rhos = the context state. */
hcc_status orc_apply_bcs(orc_ctx *ctx, double *buf);

#ifdef __cplusplus
}
#endif
#endif
