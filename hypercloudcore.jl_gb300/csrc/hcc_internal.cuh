// hcc_internal.cuh — shared declarations of the GB300 explicit-RHS library (not part of the public ABI).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/hcc.h"

// Launch bounds of the stage kernels (compile-time; a variant build overrides them with -D, and
// hcc_build_info reports the values a library was built with).
#ifndef HCC_FLUX_MINB_MANY
#define HCC_FLUX_MINB_MANY 2     // FP32 flux blocks per SM for systems of 8+ components (16-velocity BGK)
#endif
#ifndef HCC_FLUX_BLOCK
#define HCC_FLUX_BLOCK 128
#endif
#ifndef HCC_FLUX_MINB
#define HCC_FLUX_MINB 7            // FP32, D*M < 12: caps the flux kernel at 72 registers
#endif
#ifndef HCC_FLUX_MINB_WIDE
#define HCC_FLUX_MINB_WIDE 4       // FP32, D*M >= 12 (3-D Euler): 128 registers
#endif
#ifndef HCC_FP32_PACKED
#define HCC_FP32_PACKED 0          // FP32 stage kernels: 1 = packed FP32x2 instructions for component pairs (measured
                                   // slower than scalar instructions in the tile-staged 3-D flux pass)
#endif
#ifndef HCC_TILE_FLUX_PF
#define HCC_TILE_FLUX_PF 8         // tile-staged flux pass: union places of a thread's slots fetched this many slots ahead
#endif
#ifndef HCC_TILE_FLUX_GROUP
#define HCC_TILE_FLUX_GROUP 2      // tile-staged flux pass: union places in groups of this size, the slot body unrolled
                                   // over a group (0: a rotating window of HCC_TILE_FLUX_PF places)
#endif
#ifndef HCC_FLUX_STREAM_GROUP
#define HCC_FLUX_STREAM_GROUP 1    // stream-fed FP32 full flux pass: slots in groups of this size, the body unrolled
#endif
#ifndef HCC_TILE_GATHER_GROUP
#define HCC_TILE_GATHER_GROUP 8    // tile-staged gather pass: union places in groups of this size, the slot body unrolled
#endif
#ifndef HCC_FLUX_KAHAN_BLOCK
#define HCC_FLUX_KAHAN_BLOCK 4     // tile-staged flux pass: slot terms summed plainly per block, blocks compensated
#endif
#ifndef HCC_TILE_STAGE_UNROLL
#define HCC_TILE_STAGE_UNROLL 4    // tile passes: union entries a thread stages per round (halved for wide rows)
#endif
#ifndef HCC_FLUX_MINB64
#define HCC_FLUX_MINB64 3          // FP64: its Euler flux needs ~140 registers without spilling
#endif

#define HCC_MAX_STAGES 5
#define HCC_BLOCK 256

namespace hcc {

// ----------------------------------------------------------------------------------- float helpers
// Base.min / Base.max of Julia for IEEE floats: NaN-propagating, -0 below +0 (Julia Base `min`/`max` on IEEE floats; the reference calls them in `_local_extrema`, src/Interpolation/Limiter.jl, and in the MOOD extrema, src/TimeStepping/MOOD.jl).
template <typename T> __host__ __device__ __forceinline__ bool is_nan(T x) { return x != x; }
template <typename T> __host__ __device__ __forceinline__ T jmin(T x, T y) {
    bool take_y = (y < x) || (signbit(y) && !signbit(x));
    return take_y ? (is_nan(x) ? x : y) : (is_nan(y) ? y : x);
}
template <typename T> __host__ __device__ __forceinline__ T jmax(T x, T y) {
    bool take_y = (y > x) || (!signbit(y) && signbit(x));
    return take_y ? (is_nan(x) ? x : y) : (is_nan(y) ? y : x);
}

// basis_count(D, degree) (src/Interpolation/Interpolators.jl:170-177)
__host__ __device__ __forceinline__ int basis_count(int D, int degree) {
    if (degree <= 0) return 0;
    long n = 1;
    for (int k = 1; k <= degree; ++k) n = (n * (D + k)) / k;
    return int(n - 1);
}
// _div_idx / _divergence_index (src/Interpolation/MUSCL.jl:11-32)
__host__ __device__ __forceinline__ int div_idx(int D, int o) {
    if (o <= 2) return 2;
    return ((o % 2 == 1) && (D < 3 || o <= 3)) ? o + 1 : o;
}
__host__ __device__ __forceinline__ int divergence_index(int DO, int D, int p_order, int num_nb) {
    int idx = (DO == 0) ? div_idx(D, p_order) : div_idx(D, DO);
    int b0 = (DO == 0) ? p_order : DO;
    int base = b0 > 2 ? b0 : 2;
    if (idx > base && 2 * num_nb < 3 * (basis_count(D, idx - 1) + 1)) idx = base;
    while (idx > 2 && num_nb < basis_count(D, idx - 1) + 1) idx -= 1;
    return idx;
}

// Compile-time exponent table of the MLS basis of degree Q in D variables (_generate_exponents,
// Interpolators.jl:138-155): per degree, the tuples in Iterators.product order sorted by (-max(t), reverse(t)), with
// the Taylor prefactors 1/prod(t!).
constexpr int cbasis_count(int D, int q) {
    if (q <= 0) return 0;
    long n = 1;
    for (int k = 1; k <= q; ++k) n = (n * (D + k)) / k;
    return int(n - 1);
}
template <int D, int Q> struct ExpTable {
    static constexpr int B = cbasis_count(D, Q);
    int e[B > 0 ? B : 1][3];
    double pref[B > 0 ? B : 1];
    bool hp[B > 0 ? B : 1];
    constexpr ExpTable() : e{}, pref{}, hp{} {
        int k = 0;
        for (int order = 1; order <= Q; ++order) {
            const int first = k, n = order + 1;
            int total = 1;
            for (int d = 0; d < D; ++d) total *= n;
            for (int lin = 0; lin < total; ++lin) {
                int r = lin, sum = 0, t[3] = {0, 0, 0};
                for (int d = 0; d < D; ++d) { t[d] = r % n; r /= n; sum += t[d]; }
                if (sum != order) continue;
                for (int d = 0; d < 3; ++d) e[k][d] = t[d];
                ++k;
            }
            for (int q = first + 1; q < k; ++q)           // insertion sort of this degree's tuples
                for (int j = q; j > first; --j) {
                    int ma = 0, mb = 0;
                    for (int d = 0; d < D; ++d) { ma = e[j][d] > ma ? e[j][d] : ma; mb = e[j - 1][d] > mb ? e[j - 1][d] : mb; }
                    bool less = false, decided = ma != mb;
                    if (decided) less = ma > mb;
                    for (int d = D - 1; d >= 0 && !decided; --d)
                        if (e[j][d] != e[j - 1][d]) { less = e[j][d] < e[j - 1][d]; decided = true; }
                    if (!less) break;
                    for (int d = 0; d < 3; ++d) { int tmp = e[j][d]; e[j][d] = e[j - 1][d]; e[j - 1][d] = tmp; }
                }
        }
        for (int q = 0; q < B; ++q) {
            int den = 1;
            for (int d = 0; d < D; ++d)
                for (int f = 2; f <= e[q][d]; ++f) den *= f;
            pref[q] = 1.0 / double(den);
            hp[q] = den != 1;
        }
    }
};

// build_basis of degree Q (Interpolators.jl:194-218) from the compile-time table: prefactor first, then the
// factors x_d or x_d^t in axis order (x^2 = x*x, x^3 = x*x*x, Base.literal_pow).
template <int D, int Q, typename T>
__host__ __device__ __forceinline__ void table_basis(const T *x, T *p) {
    constexpr ExpTable<D, Q> tab{};
#pragma unroll
    for (int k = 0; k < ExpTable<D, Q>::B; ++k) {
        bool have = tab.hp[k];
        T v = have ? T(tab.pref[k]) : T(0);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int t = tab.e[k][d];
            if (t == 0) continue;
            const T f = (t == 1) ? x[d] : (t == 2 ? x[d] * x[d] : x[d] * x[d] * x[d]);
            v = have ? v * f : f;
            have = true;
        }
        p[k] = v;
    }
}

// Reconstruction basis of degree 1 or 2 (build_basis, Interpolators.jl:194-218), in the order of
// _generate_exponents: degree-1 terms x, y, z; then x²/2, y²/2, z²/2; then xy, xz, yz.
template <int D, int DEG> struct RBasis { static constexpr int B = (DEG == 1) ? D : (D == 1 ? 2 : (D == 2 ? 5 : 9)); };

template <int D, int DEG, typename T>
__host__ __device__ __forceinline__ void recon_basis(const T *x, T *p) {
    if constexpr (DEG == 1) {
#pragma unroll
        for (int d = 0; d < D; ++d) p[d] = x[d];
    } else {
        if constexpr (D == 1) { p[0] = x[0]; p[1] = T(0.5) * (x[0] * x[0]); }
        if constexpr (D == 2) {
            p[0] = x[0]; p[1] = x[1];
            p[2] = T(0.5) * (x[0] * x[0]); p[3] = T(0.5) * (x[1] * x[1]); p[4] = x[0] * x[1];
        }
        if constexpr (D == 3) {
            p[0] = x[0]; p[1] = x[1]; p[2] = x[2];
            p[3] = T(0.5) * (x[0] * x[0]); p[4] = T(0.5) * (x[1] * x[1]); p[5] = T(0.5) * (x[2] * x[2]);
            p[6] = x[0] * x[1]; p[7] = x[0] * x[2]; p[8] = x[1] * x[2];
        }
    }
}
// build_scale_factors (Interpolators.jl:236-247) for degree 1/2 bases
template <int D, int DEG, typename T>
__host__ __device__ __forceinline__ T recon_scale(int b, T invL) {
    return (b < D) ? invL : invL * invL;
}

// ----------------------------------------------------------------------------------- physics
// Parameters of the compiled-in HyperbolicPDE modules (selected by trait at hcc_create).
template <typename T> struct PhysParams {
    T c[HCC_MAX_DIM][HCC_MAX_VARS];   // advection speeds (BGK: kinetic speeds v_k,d)
    T amax[HCC_MAX_DIM];              // spectral radius per axis
    T gamma, gm1;
    T inv_eps, coeff;                 // BGK
    T a_macro[HCC_MAX_DIM];
    T sinv[HCC_MAX_VARS][HCC_MAX_DIM];
};

// Scheme-wide constants of the stage kernels.
struct SchemeParams {
    int max_order, DO, strategy, criterion;
    int has_source;                   // BGK relaxation source present
    int limiter;                      // hcc_limiter
    int aligned;                      // AlignedRusanovFlux
    int upwind_alg;                   // hcc_upwind_algorithm (HCC_SCHEME_UPWIND)
};

// Device view of the neighbour lists and geometry caches (slot-major, stride = npad).
template <typename T> struct Geometry {
    int64_t n, npad;
    const int32_t *cnt;               // [n]
    const int32_t *nidx;              // [kmax * npad]
    const T *dist;                    // [(k*D + d) * npad + i]
    const T *wt;                      // [k * npad + i]
    const T *dw;                      // [(k*D + d) * npad + i]  divergence weights of the cached fit
    const T *dw1;                     // degree-1 dynamic set (schemes whose full divergence degree is > 1)
    const uint8_t *ok_r, *ok_d, *ok_1;
    const T *inv_r;                   // [i * Br * Br]
    const T *gw;                      // FP32, degree-1 reconstruction: gradient weights of the cached fit,
                                      // [(k*D + b) * npad + i] = invL Σ_c inv_r[b][c] w_k x_k[c] (else nullptr)
    const uint8_t *bnd;
    const T *mw;                      // moment-correction weights e^d_ij [(k*D + d) * npad + i] (or nullptr)
    const T *dwc[3];                  // CentralDivergence: weights of the intercept fit of degree q = 1..3
    const uint8_t *okc[3];
    T invL;
    double invL64;                    // 1/min(dx) in FP64 (the MLS fits of both paths)
    double h64;                       // min(dx)
    // FP32 meshless WENO of Euler: per particle the first-derivative rows of the inverse moment matrices of its
    // central and one-sided stencils, degrees 1 and 2 ([i][degree - 1][stencil][d][b], FP32, nullptr when absent),
    // and the sizes of its one-sided stencils ([i][2 d + side - 1])
    const float *wops;
    const int32_t *wcnt;
    // FP64 meshless WENO of Euler: the Cholesky factors of the same moment matrices (packed upper triangles,
    // [i][degree - 1][stencil][B2 (B2 + 1) / 2]) and their flags ([i][degree - 1][stencil]), nullptr when absent
    const double *wchol;
    const uint8_t *wok;
};

// Tile staging of the FP32 full passes (MUSCL of order <= 2 with the degree-1 divergence fit, fixed grids): the
// particles in tiles of HCC_TILE consecutive (Morton-numbered) particles; per tile the sorted union of its particles
// and of all their neighbours, which one thread block stages in shared memory; per slot the neighbour's place in its
// particle's tile union (16 bits); per union entry the position relative to the tile's first particle as int32
// multiples of the tile's power-of-two quantum (so x_j - x_i is an exact integer difference, rounded once when
// converted to FP32); per particle the FP32 rows of its cached fits: A_d and B_de of the divergence weights
// dw_k[d] = w_k (A_d + sum_e B_de x_e) and G_bc of the gradient weights gw_k[b] = w_k sum_c G_bc x_c, with
// w_k = w(|x_k|^2) the weight function. The slot streams of distances, weights and divergence weights are then
// never read by the full passes: they recompute them from positions that come from shared memory.
#ifndef HCC_TILE
#define HCC_TILE 128
#endif
struct TileView {
    int64_t ntiles;
    const int64_t *ustart;            // [ntiles + 1] union offsets
    const int32_t *uid;               // [utotal] particle numbers, ascending within a tile
    const int4 *upos;                 // [utotal] quantised offsets from the tile's first particle (x, y, z, 0)
    const float *quantum;             // [ntiles] length of one unit of upos (a power of two)
    const uint16_t *lidx;             // [kmax * npad] slot k of particle i: place of its neighbour in the union
    const uint16_t *lself;            // [n] place of the particle itself in its tile's union
    const float *coef;                // [n * cw] A (D), B (D*D), G (D*D), zero-padded to cw floats
    int cw;                           // a multiple of 4
    int umax;                         // largest union of any tile
    float wscale;                     // alpha / R^2 of the weight function
};

// dt-dependent coefficients of one candidate, read by the kernels from device memory so that one captured step
// graph serves every dt: hE[j] = dt a_t (0 = skipped), hI[j] = dt a (0 = skipped), h_sub = dt / C of the Euler
// substep, dt_ii = dt a_ii and its inverse for the implicit part.
template <typename T> struct StageCoeffs {
    double hEd[HCC_MAX_STAGES];       // dt a_t in FP64: the stage positions of a moving grid
    T hE[HCC_MAX_STAGES];
    T hI[HCC_MAX_STAGES];
    T h_sub;
    T dt_ii, inv_dt_ii;
};

// Arguments of the gather (reconstruction) and flux kernels.
template <typename T> struct StageArgs {
    Geometry<T> g;
    PhysParams<T> ph;
    SchemeParams sc;
    int8_t *orders;
    const int8_t *nbmin;              // EPD2: neighbourhood minimum of the orders
    T *grad;                          // [i * Br * M]
    const T *U;                       // stage state Y_s
    double *wflux64;                  // FP64 Euler WENO: per particle F_d(U)_m and lambda_d of the stage state
    T *K;                             // K_E[s]
    int full;                         // 1: every particle; 0: the members of a tile worklist
    // Worklist pass: tiles of 32 consecutive particles (one warp each, coalesced slot-major loads), the tiles to
    // visit, their count (device) and one member bit per particle (a word per tile).
    const int32_t *wtiles;
    const unsigned *wcount;
    uint32_t *wmask;
    int clear_wmask;                  // flux pass over the reach: clear each tile's word once read
    uint32_t *rmask;                  // gather pass over the changed orders: the reach of its members (the member
    int32_t *rtiles;                  // and its neighbours) is marked here, each tile listed once
    unsigned *rcount;
    int list_blocks;                  // grid of a worklist pass (warp-stride over the tiles)
    int flux_block, gather_block;     // block sizes of the full flux / gather passes (multiples of 32, <= 128)
    // epilogue: next candidate (Y_{s+1} or the final state) and the MOOD check of checkpoint s+1
    int form_next;
    const T *Un;                      // start-of-step state (pg.rhos)
    const T *KE[HCC_MAX_STAGES];
    const T *KI[HCC_MAX_STAGES];
    const StageCoeffs<T> *coef;       // device: the dt-dependent coefficients of this candidate (of cloud 0)
    const int32_t *cloud_id;          // batches stepped with one dt per cloud: particle -> cloud (else nullptr) ...
    int coef_stride;                  // ... and the coefficient entries per cloud
    int n_prev;                       // stages entering the candidate (K_E[s] is this kernel's own)
    int self_slot;                    // index of K_E[s] among KE (its value comes from registers)
    T *Ynext;
    T *KInext;
    int implicit_mode;                // 0 none, 1 implicit solve (a_ii != 0), 2 explicit source evaluation
    int check;                        // run the MOOD check of the candidate
    uint32_t *rough_words;            // last stage with a predictor: per tile, the particles whose stencil range of
                                      // the stage state is not flat (the next step's feature pass skips the rest)
    int check_substep;                // 1: W = Y_s + h_sub (K + KI_s), 0: the candidate itself
    const T *KIs;                     // K_I[s] for the substep of implicit-source tableaus
    T delta;
    T u2_plateau, u2_ratio, u2_h;     // MOODu2: plateau and curvature-ratio parameters, h = min(dx)
    const unsigned long long *u2_range;   // MOODu2 global range of the stage state (ordered keys: lo[M], hi[M],
                                          // NaN bits), nullptr when the plateau test is off
    // moving grid (GridMovers.jl): mover kind and parameters, the current positions (SoA FP64), this stage's grid
    // velocities (out), the start-of-step positions, the grid velocities of earlier stages and the next positions
    int mover;
    T mv_alpha;
    double mv_v[3], mv_om[3], mv_c[3];
    const double *pos;
    double *KXout;
    const double *x_n;
    const double *KX[HCC_MAX_STAGES];
    double *Xnext;
    int tile;                         // 1: full passes of this FP32 context are tile-staged (tv is valid)
    TileView tv;
    uint32_t *tmask;                  // MOOD check: failed candidates (a ballot word per tile) ...
    int32_t *ttiles;                  // ... the tiles with a failure ...
    unsigned *tcount;                 // ... and their count
    uint8_t *inadm;
};

// The coefficients of particle i's candidate: its cloud's set when the batch is stepped with one dt per cloud.
template <typename T>
__device__ __forceinline__ const StageCoeffs<T> *coef_of(const StageArgs<T> &a, int64_t i) {
    return a.cloud_id ? a.coef + int64_t(a.cloud_id[i]) * a.coef_stride : a.coef;
}

// Device-side tile worklists of the MOOD fixed point: t = tiles with failed candidates, c = tiles with a dropped
// order (cn: the list being filled by the current decrement, published as c by the decision), d = the reach of the
// changed orders (one or two hops), d1 = its one-hop part; done = blocks finished in the decrement launch; f = tiles
// offered a lower order by StrictEPD0 forcing.
struct ListCounts {
    unsigned t, c, cn, d, d1, done, f, pad1;
};

// Append v to a device list; warp-aggregated: one atomic per group of converged lanes.
__device__ __forceinline__ void list_append(int32_t *list, unsigned *count, int32_t v) {
    const unsigned act = __activemask();
    const int lane = int(threadIdx.x & 31);
    const int leader = __ffs(act) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, unsigned(__popc(act)));
    base = __shfl_sync(act, base, leader);
    list[base + unsigned(__popc(act & ((1u << lane) - 1u)))] = v;
}

// Reach of the changed orders (expand_mask!, MOOD.jl:343-351; _expand_body!, :323-335: a particle is marked if it
// or a neighbour was), pushed from the changed particles: the neighbour relation is symmetric (one radius, exactly
// antisymmetric distances), so marking every neighbour of a changed particle marks the same set as the pull over
// all particles. The first bit set in a tile's word lists the tile (once).
__device__ __forceinline__ void reach_mark(uint32_t *mask, int32_t *tiles, unsigned *count, int32_t j) {
    if (atomicOr(&mask[j >> 5], 1u << (j & 31)) == 0u) list_append(tiles, count, j >> 5);
}

// reach_mark for a whole warp (all 32 lanes call it; j < 0: no mark): lanes whose particles share a tile combine their
// bits first, one atomic per distinct tile word, and the newly listed tiles are appended together.
__device__ __forceinline__ void reach_mark_warp(uint32_t *mask, int32_t *tiles, unsigned *count, int32_t j) {
    const int lane = int(threadIdx.x & 31);
    const int32_t t = j >= 0 ? (j >> 5) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, t);
    const unsigned bits = __reduce_or_sync(grp, j >= 0 ? (1u << (j & 31)) : 0u);
    bool fresh = false;
    if (lane == __ffs(grp) - 1 && t >= 0) fresh = atomicOr(&mask[t], bits) == 0u;
    const unsigned nb = __ballot_sync(0xffffffffu, fresh);
    if (nb) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(count, unsigned(__popc(nb)));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (fresh) tiles[base + unsigned(__popc(nb & ((1u << lane) - 1u)))] = t;
    }
}

// Launchers of one (precision, D, M, pde, reconstruction degree) instantiation.
// Arguments of the geometry pass of the FP32 meshless WENO of Euler (FP64 slot streams in, FP32 operators out).
struct WenoGeomArgs {
    int64_t n, npad;
    const int32_t *cnt;
    const double *dist, *w;
    const uint8_t *bnd;
    double invL64;
    float *ops;                       // FP32 contexts: the operators
    int32_t *wcnt;
    double *chol;                     // FP64 contexts: the packed Cholesky factors and their flags
    uint8_t *ok;
};
// doubles of the packed WENO Cholesky factors of one particle: 2 degrees x (2D + 1) stencils x B2 (B2 + 1) / 2
inline int weno_chol_doubles(int D) { return 2 * (2 * D + 1) * cbasis_count(D, 2) * (cbasis_count(D, 2) + 1) / 2; }
// floats of the WENO operators of one particle: 2 degrees x (2D + 1) stencils x D rows x the degree-2 basis
inline int weno_ops_floats(int D) { return 2 * (2 * D + 1) * D * cbasis_count(D, 2); }

struct StageOps {
    int D, M, pde, rdeg, Br;
    void (*gather)(const void *args, int64_t n, cudaStream_t s);
    void (*flux)(const void *args, int64_t n, cudaStream_t s);
    void (*stage1)(const void *args, int64_t n, cudaStream_t s);   // Y_1 (predictor + implicit part)
    void (*cfl)(const void *args, int64_t n, unsigned long long *dt_bits, cudaStream_t s);
    void (*weno)(const void *args, int64_t n, cudaStream_t s);   // WENO flux pass (scalar advection only)
    void (*central)(const void *args, int64_t n, cudaStream_t s);   // CentralDivergence pass
    void (*upwind)(const void *args, int64_t n, cudaStream_t s);    // UpwindDivergence :Tiwari / :Praveen pass
    void (*weno_geom)(const WenoGeomArgs &g, cudaStream_t s);      // FP32 Euler WENO operators (or nullptr)
};

const StageOps *stage_ops_f64_r1(int D, int M, int pde);
const StageOps *stage_ops_f64_r2(int D, int M, int pde);
const StageOps *stage_ops_f32_r1(int D, int M, int pde);
const StageOps *stage_ops_f32_r2(int D, int M, int pde);

// ----------------------------------------------------------------------------------- search / geometry
struct SearchArgs {
    int64_t n, npad;
    int D;
    double *pos;                      // SoA [d * npad + i]
    int periodic[3];
    double cmin[3], csize[3], Lphys[3], Lwrap[3], invLwrap[3];
    int dims[3];
    int64_t nbins;
    int noff;
    const int64_t *binnb;             // [nbins * noff]
    int32_t *bin_of;                  // [n]
    int32_t *cell_count;              // [nbins + 1]
    int64_t *cell_start;              // [nbins + 2]
    int32_t *cell_cursor;             // [nbins]
    int32_t *cellp;                   // [n]
    int32_t *cnt;                     // [n]
    double R_sq, alpha, invR2;
    // exact FP32 prefilter of the r^2 test (nullptr: FP64 only): an FP32 copy of the positions, the largest
    // |coordinate| (float bits, written by the bin pass), the wrap lengths in FP32 and the largest wrap length
    float *pos32;
    unsigned int *pmax;
    float L32[3], invL32[3];
    double Lmax;
    // output (slot-major)
    int32_t *nidx;
    double *w;
    double *dist;
    int kmax;
};

hcc_status search_bins(SearchArgs &a, cudaStream_t s, std::string &err);
hcc_status search_count(SearchArgs &a, cudaStream_t s, unsigned long long *d_stats, std::string &err);
hcc_status search_write(SearchArgs &a, cudaStream_t s, std::string &err);
hcc_status search_refresh(SearchArgs &a, cudaStream_t s, std::string &err);

struct MlsArgs {
    int64_t n, npad;
    int D, rdeg, Br, ddeg, Bd, max_order, DO;
    int need_dw1;
    const int32_t *cnt, *nidx;
    const double *dist, *w;
    double invL;
    double *inv_r; uint8_t *ok_r;
    double *inv_d; uint8_t *ok_d;
    double *dw; double *dw1; uint8_t *ok_1;
    int weno_cfl_degree;              // > 0: per-slot CFL weights of the assembled Taylor fit (WENO), not MUSCL caches
    int central_qmax;                 // > 0: CentralDivergence weight sets of degree 1..central_qmax
    double *dwc[3];
    uint8_t *okc[3];
    double *mw;                       // != nullptr: moment-correction weights of a first-order scheme (from dw)
    int aligned;                      // AlignedRusanovFlux (the dissipation direction of the moment weights)
};
hcc_status mls_prepare(MlsArgs &a, cudaStream_t s, std::string &err);

// Outflow donor map (BoundaryConditions.jl:82-130 with the state-free part precomputed per geometry).
struct DonorArgs {
    int64_t n, npad;
    int D;
    const int32_t *cnt, *nidx;
    const double *dist;
    const uint8_t *bnd;
    const int32_t *tags;
    int32_t *status, *status_prev, *root;
};
hcc_status donor_map(DonorArgs &a, int tag, cudaStream_t s, std::string &err);

// Small utility kernels (hcc_util.cu).
void launch_cast_f64_to_f32(const double *src, float *dst, int64_t n, cudaStream_t s);
void launch_cast_f32_to_f64(const float *src, double *dst, int64_t n, cudaStream_t s);
void launch_fill_i8(int8_t *p, int8_t v, int64_t n, cudaStream_t s);
void launch_bc_apply(void *Y, const void *rhos, const int32_t *blist, const int32_t *bsrc, int64_t nb, int M,
                     int is_f32, cudaStream_t s);
// Second hop of the reach (EPD2): d1 = the one-hop tiles and their words (copied to words1), then the neighbours
// of their members are marked; the neighbourhood minimum of the orders over the one-hop members.
void launch_reach_hop2(ListCounts *counts, const int32_t *dtiles, int32_t *dtiles_out, uint32_t *dmask,
                       uint32_t *words1, const int32_t *cnt, const int32_t *nidx, int64_t npad, int blocks,
                       cudaStream_t s);
// Neighbourhood minimum of the orders: every particle (tiles == nullptr) or the members of the tiles.
void launch_nbmin(const int8_t *orders, int8_t *nbmin, const int32_t *cnt, const int32_t *nidx, int64_t n,
                  int64_t npad, const int32_t *tiles, const uint32_t *words, const unsigned *count, int blocks,
                  cudaStream_t s);
// MOODu2 global range of a state (_global_range, MOOD.jl:215-221): keys[0, M) = ordered keys of the minima,
// keys[M, 2M) of the maxima, keys[2M] = bit m set if component m holds a NaN. Clears the keys first.
void launch_u2_range(const void *U, int64_t n, int M, int is_f32, unsigned long long *keys, cudaStream_t s);
// Ordered 64-bit key of a double (monotone in the value, -0 below +0) and back.
__host__ __device__ __forceinline__ unsigned long long order_key(double v) {
    unsigned long long b;
    memcpy(&b, &v, sizeof(b));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double order_value(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    memcpy(&v, &b, sizeof(v));
    return v;
}
// StrictEPD0 forcing (forced_order(::Halo{1}), MOOD.jl:54-64; _mood_force!, :312-320): the particles dropped in the
// last decrement (c tiles) offer their order to their interior neighbours, which take it where it is lower and join
// the changed list. forced[] holds 0x7f7f7f7f between calls.
void launch_force(const int32_t *ctiles, uint32_t *cmask, ListCounts *counts, int32_t *ctiles_out, int8_t *orders,
                  const uint8_t *bnd, const int32_t *cnt, const int32_t *nidx, int64_t npad, int32_t *forced,
                  uint32_t *fmask, int32_t *ftiles, int blocks, cudaStream_t s);
void launch_count_inadmissible(const uint8_t *inadm, const uint8_t *bnd, int64_t n, unsigned long long *out,
                               cudaStream_t s);
// Gradient weights of the cached degree-1 fit (FP64 sums, FP32 store): gw[(k*D + b) * npad + i] =
// invL Σ_c inv_r[b][c] w_k (dist_k[c] invL) for particles with ok_r, 0 elsewhere.
void launch_grad_weights(int64_t n, int64_t npad, int D, int kmax, const int32_t *cnt, const double *dist,
                         const double *w, const double *inv_r, const uint8_t *ok_r, double invL, float *gw,
                         cudaStream_t s);
void launch_shepard(const int32_t *cnt, const int32_t *nidx, const double *w, int64_t n, int64_t npad, double w0,
                    int sweeps, double *S, double *V, double *Vt, double *partial, cudaStream_t s);
void launch_scale(double *V, int64_t n, double f, cudaStream_t s);
unsigned shepard_blocks(int64_t n);
void launch_total_mass(const void *U, const double *vol, int64_t n, int M, int is_f32, double *out,
                       cudaStream_t s);
// Statistics of the MOOD fixed points of one step (device; zeroed at the start of the step).
struct MoodStats {
    unsigned long long iterations, flagged, inadmissible, timeout;
    unsigned int iter_in_checkpoint, pad;
    unsigned long long predicted;     // particles the troubled-point predictor pre-lowered
    unsigned long long pred_rows;     // rows that passed the predictor's smoothness gate
    unsigned int tc_error, pad2;      // a tensor-core wait of the predictor gave up
};

// One launch after a flux pass with the MOOD check: boundary conditions of the new candidate (first bc_blocks
// blocks), the MOOD decrement of the failed candidates into the changed list (the other blocks), and — in the last
// block to finish — the decision of the fixed point (publish the changed list, reset the other lists, update the
// statistics, and set the WHILE condition of a step graph when has_handle).
struct DropArgs {
    void *Y;
    const void *rhos;
    const int32_t *blist, *bsrc;
    int64_t nb;
    int M, bc_blocks;
    int8_t *orders;
    uint8_t *trig_step;
    const int32_t *ttiles;
    const uint32_t *tmask;
    int32_t *ctiles;
    uint32_t *cmask;
    ListCounts *counts;
    MoodStats *stats;
    cudaGraphConditionalHandle h;
    int has_handle, cap;
};
void launch_drop_decide(const DropArgs &a, int is_f32, int drop_blocks, cudaStream_t s);
void launch_gather_rows(const void *slotmajor, void *rowmajor, const int32_t *cnt, const int64_t *rowstart,
                        int64_t n, int64_t npad, int width, int elem_bytes, cudaStream_t s);
// FP64 FMA rate of the current device in TFLOP/s (2 FLOP per FMA), from a timed kernel on every SM.
double fp64_fma_rate_tflops(int sms, cudaStream_t st, cudaError_t *err);
void launch_gather_rows_of(const void *src, void *dst, const int32_t *cnt, const int64_t *ids, int64_t n_sel,
                           int64_t npad, int width, int max_slots, int elem_bytes, cudaStream_t s);


// Tile tables of a context (hcc_tiles.cu): built from the FP64 geometry after the MLS caches; `ok` = 0 when the
// cloud does not qualify (a union above 65535 entries or beyond the shared-memory budget, a periodic axis shorter than
// 2 (tile extent) + R), in which case the full passes keep the slot streams.
struct TileBuild {
    int64_t n, npad;
    int D, kmax;
    const int32_t *cnt, *nidx;
    const double *pos;                // SoA [d * npad + i]
    int periodic[3];
    double Lwrap[3], invLwrap[3], R;
    const double *inv_r, *inv_d;      // FP64 inverse moments: D x D (reconstruction), (D+1) x (D+1) (divergence)
    const uint8_t *ok_r, *ok_d;
    double invL, wscale;
    int max_union;                    // refuse unions above this many entries
};
struct TileTables {
    int64_t ntiles = 0, utotal = 0;
    int64_t *ustart = nullptr;
    int32_t *uid = nullptr;
    int4 *upos = nullptr;
    float *quantum = nullptr;
    uint16_t *lidx = nullptr, *lself = nullptr;
    float *coef = nullptr;
    int cw = 0, umax = 0;
    float wscale = 0.f;
    int ok = 0;
    void release();
};
hcc_status build_tile_tables(const TileBuild &b, TileTables &t, cudaStream_t s, std::string &err);

// ----------------------------------------------------------------------------------- learned predictor
// Inputs of the stencil features (state in the context's precision, slot-major neighbour lists and offsets).
struct FeatArgs {
    const void *U;
    int f32, D, M, pde;
    int64_t n, npad;
    const int32_t *cnt, *nidx;
    const void *dist;                 // [(k*D + d) * npad + i], element type of U
    const uint8_t *bnd;
    float h, gm1;                     // min(dx); gamma - 1 (Euler)
};
// Device view of the network: BF16 images of W1 [64][24] and W2 [64][64] (row-major), the FP32 master parameters
// (biases and w3 are read from it) and the input normalisation mean[24], inv_std[24].
struct MlpWeights {
    const uint16_t *W1, *W2;
    const float *params, *norm;
};
// Buffers and outputs of the in-step prediction: the compact list of gated rows (normalised BF16 features, four
// 16-byte segments each, and their particle numbers), the mask of predicted particles and the orders they get.
struct PredictOut {
    int8_t *orders;
    int8_t lowered;                   // order of a predicted particle (one below the maximum)
    uint8_t *pred;                    // [n] 0/1
    float *logits;                    // [n] or nullptr
    unsigned long long *count;        // predicted particles (accumulated)
    float thr_logit;
    const uint32_t *rough;            // [tiles] from the last step's final flux pass (nullptr: every particle)
    uint4 *rows;                      // [cap * 4] (nullptr: features only)
    int32_t *row_idx;                 // [cap]
    unsigned long long *nrows;        // rows appended (zeroed before the pass)
    int64_t cap;
};
bool launch_features(const FeatArgs &fa, float *out, cudaStream_t s);
// Pass 1 (features, gate, compaction; raw features into `raw` when not null) and pass 2 (the network).
bool launch_predict(const FeatArgs &fa, const MlpWeights &w, const PredictOut &po, float *raw, int grid,
                    unsigned *err, cudaStream_t s);
MlpWeights mlp_weights(const hcc_mlp *m);
hcc_status mlp_append(hcc_mlp *m, const float *feat, const uint8_t *labels, const uint8_t *bnd, int64_t n,
                      cudaStream_t s);

}  // namespace hcc
