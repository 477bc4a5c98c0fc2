// hcc_util.cu — small device passes of the time stepper: boundary conditions, MOOD decrement / mask dilation /
// neighbourhood orders, conserved totals, conversions and the row-major export of slot-major arrays.
#include <algorithm>

#include "hcc_internal.cuh"

namespace hcc {
namespace {

inline unsigned grid_for(int64_t n, int bs = HCC_BLOCK) { return unsigned((n + bs - 1) / bs); }

__global__ void k_cast_f64_f32(const double *s, float *d, int64_t n) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) d[i] = float(s[i]);
}
__global__ void k_cast_f32_f64(const float *s, double *d, int64_t n) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) d[i] = double(s[i]);
}
__global__ void k_fill_i8(int8_t *p, int8_t v, int64_t n) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// apply_boundary_conditions! with the precomputed donor map: Dirichlet / no condition -> start-of-step state,
// outflow -> the state of the resolved interior donor (BoundaryConditions.jl:43-130).
template <typename T>
__global__ void k_bc(T *Y, const T *rhos, const int32_t *blist, const int32_t *bsrc, int64_t nb, int M) {
    int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= nb) return;
    int64_t b = blist[q];
    int32_t src = bsrc[q];
    for (int m = 0; m < M; ++m) Y[b * M + m] = (src >= 0) ? Y[int64_t(src) * M + m] : rhos[b * M + m];
}

// After a flux pass with the MOOD check, one launch: the boundary conditions of the new candidate (blocks below
// bc_blocks; apply_boundary_conditions!, BoundaryConditions.jl:43-130), _mood_drop! (MOOD.jl:299-309) over the
// failed candidates — an order above 1 drops by one and the particle joins the changed list — and, in the last
// block to finish, the loop condition of mood_checkpoint! (TimeSteppers.jl:454-477): no changed order ends the loop;
// otherwise the flagged count grows and the loop repeats, unless the checkpoint already ran `cap` recomputes (the
// timeout flag ends it). The decision publishes the changed list and clears the other lists for the next pass.
template <typename T>
__global__ void k_drop_decide(const DropArgs a) {
    if (int(blockIdx.x) < a.bc_blocks) {
        T *Y = static_cast<T *>(a.Y);
        const T *rhos = static_cast<const T *>(a.rhos);
        for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < a.nb;
             q += int64_t(a.bc_blocks) * blockDim.x) {
            const int64_t b = a.blist[q];
            const int32_t src = a.bsrc[q];
            for (int m = 0; m < a.M; ++m) Y[b * a.M + m] = (src >= 0) ? Y[int64_t(src) * a.M + m] : rhos[b * a.M + m];
        }
    } else {
        // one warp per tile of failed candidates; the changed members form the tile's word of the c list
        const unsigned nt = a.counts->t;
        const int lane = int(threadIdx.x & 31);
        const unsigned warp = ((blockIdx.x - unsigned(a.bc_blocks)) * blockDim.x + threadIdx.x) >> 5;
        const unsigned nwarps = ((gridDim.x - unsigned(a.bc_blocks)) * blockDim.x) >> 5;
        for (unsigned q = warp; q < nt; q += nwarps) {
            const int32_t tile = a.ttiles[q];
            const uint32_t word = a.tmask[tile];
            const int64_t i = int64_t(tile) * 32 + lane;
            bool ch = false;
            if ((word >> lane) & 1u) {
                const int8_t o = a.orders[i];
                if (o > 1) {
                    a.orders[i] = int8_t(o - 1);
                    a.trig_step[i] = 1;
                    ch = true;
                }
            }
            const unsigned b = __ballot_sync(0xffffffffu, ch);
            if (lane == 0 && b) {
                a.cmask[tile] = b;
                a.ctiles[atomicAdd(&a.counts->cn, 1u)] = tile;
            }
        }
    }
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&a.counts->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    ListCounts *ct = a.counts;
    MoodStats *st = a.stats;
    const unsigned changed = atomicAdd(&ct->cn, 0u);
    ct->c = changed;
    ct->cn = 0;
    ct->t = 0;
    ct->d = 0;
    ct->f = 0;
    ct->done = 0;
    unsigned go = 0;
    if (changed == 0) {
        st->iter_in_checkpoint = 0;
    } else {
        st->flagged += changed;
        if (st->iter_in_checkpoint >= unsigned(a.cap)) {
            st->timeout = 1;
            st->iter_in_checkpoint = 0;
        } else {
            st->iter_in_checkpoint += 1;
            st->iterations += 1;
            go = 1;
        }
    }
    __threadfence();
    if (a.has_handle) cudaGraphSetConditional(a.h, go);
}

// StrictEPD0 forcing, push half: every member of a c tile (dropped in the last decrement) offers its order to its
// interior neighbours (atomicMin), which are marked in the f tiles.
__global__ void k_force_push(const int32_t *ctiles, const uint32_t *cmask, ListCounts *counts, const int8_t *orders,
                             const uint8_t *bnd, const int32_t *cnt, const int32_t *nidx, int64_t npad, int32_t *forced,
                             uint32_t *fmask, int32_t *ftiles) {
    const unsigned nt = counts->c;
    const int lane = int(threadIdx.x & 31);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = ctiles[q];
        if (!((cmask[tile] >> lane) & 1u)) continue;
        const int64_t p = int64_t(tile) * 32 + lane;
        const int32_t v = orders[p];
        const int c = cnt[p];
        for (int k = 0; k < c; ++k) {
            const int32_t j = nidx[int64_t(k) * npad + p];
            if (bnd[j]) continue;
            atomicMin(&forced[j], v);
            reach_mark(fmask, ftiles, &counts->f, j);
        }
    }
}
// Pull half: a marked particle takes the offered order where it is lower than its own (post-decrement) order and joins
// the changed list; the offers and marks are cleared.
__global__ void k_force_apply(ListCounts *counts, const int32_t *ftiles, uint32_t *fmask, int32_t *forced,
                              int8_t *orders, uint32_t *cmask, int32_t *ctiles) {
    const unsigned nt = counts->f;
    const int lane = int(threadIdx.x & 31);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = ftiles[q];
        const uint32_t word = fmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        bool ch = false;
        if ((word >> lane) & 1u) {
            const int32_t o = forced[i];
            forced[i] = 0x7f7f7f7f;
            if (o < int32_t(orders[i])) {
                orders[i] = int8_t(o);
                ch = true;
            }
        }
        const unsigned b = __ballot_sync(0xffffffffu, ch);
        if (lane == 0) {
            fmask[tile] = 0u;
            if (b && atomicOr(&cmask[tile], b) == 0u) ctiles[atomicAdd(&counts->c, 1u)] = tile;
        }
    }
}

// Second hop of the reach (EPD2): the one-hop tiles d[0, d1) and their words are fixed first (the words are
// copied before the second hop sets more bits in them), then the neighbours of their members are marked.
__global__ void k_reach_fix(ListCounts *counts, const int32_t *dtiles, const uint32_t *dmask, uint32_t *words1) {
    const unsigned n1 = counts->d;
    if (blockIdx.x == 0 && threadIdx.x == 0) counts->d1 = n1;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n1; q += gridDim.x * blockDim.x)
        words1[q] = dmask[dtiles[q]];
}
__global__ void k_reach_hop2(ListCounts *counts, int32_t *dtiles, uint32_t *dmask, const uint32_t *words1,
                             const int32_t *cnt, const int32_t *nidx, int64_t npad) {
    const unsigned n1 = counts->d1;
    const int lane = int(threadIdx.x & 31);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < n1; q += nwarps) {
        const bool mem = (words1[q] >> lane) & 1u;
        const int64_t i = int64_t(dtiles[q]) * 32 + lane;
        const int c = mem ? cnt[i] : 0;
        const int kw = __reduce_max_sync(0xffffffffu, c);
        for (int k = 0; k < kw; ++k)     // slot by slot across the warp, combined atomics
            reach_mark_warp(dmask, dtiles, &counts->d, k < c ? nidx[int64_t(k) * npad + i] : -1);
    }
}

// _nb_min_order (MOOD.jl:66-74) for EPD2, for every particle (list == nullptr) or the listed ones.
__device__ __forceinline__ void nbmin_one(const int8_t *orders, int8_t *nbmin, const int32_t *cnt,
                                          const int32_t *nidx, int64_t npad, int64_t i) {
    int8_t o = orders[i];
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) {
        int8_t oj = orders[nidx[int64_t(k) * npad + i]];
        o = oj < o ? oj : o;
    }
    nbmin[i] = o;
}
__global__ void k_nbmin(const int8_t *orders, int8_t *nbmin, const int32_t *cnt, const int32_t *nidx, int64_t n,
                        int64_t npad) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) nbmin_one(orders, nbmin, cnt, nidx, npad, i);
}
__global__ void k_nbmin_tiles(const int8_t *orders, int8_t *nbmin, const int32_t *cnt, const int32_t *nidx,
                              int64_t npad, const int32_t *tiles, const uint32_t *words, const unsigned *count) {
    const unsigned nt = *count;
    const int lane = int(threadIdx.x & 31);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps)
        if ((words[q] >> lane) & 1u) nbmin_one(orders, nbmin, cnt, nidx, npad, int64_t(tiles[q]) * 32 + lane);
}

// MOODu2 global range: per component, the minimum and maximum ordered keys over every particle (boundary ones
// included, as view(U, 1:N)), NaNs recorded separately (Julia's min/max propagate them).
template <typename T>
__global__ void k_u2_range(const T *U, int64_t n, int M, unsigned long long *keys) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (int m = 0; m < M; ++m) {
        unsigned long long lo = ~0ull, hi = 0ull;
        unsigned nan = 0;
        if (i < n) {
            const double v = double(U[i * M + m]);
            if (v != v) nan = 1;
            else lo = hi = order_key(v);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, o), h2 = __shfl_down_sync(0xffffffffu, hi, o);
            lo = l2 < lo ? l2 : lo;
            hi = h2 > hi ? h2 : hi;
        }
        const unsigned anynan = __any_sync(0xffffffffu, nan);
        if ((threadIdx.x & 31) == 0) {
            if (lo != ~0ull) atomicMin(&keys[m], lo);
            if (hi != 0ull) atomicMax(&keys[M + m], hi);
            if (anynan) atomicOr(&keys[2 * M], 1ull << m);
        }
    }
}

// Interior candidates that are not admissible once a fixed point has converged (_count_inadmissible,
// TimeSteppers.jl:481-490).
__global__ void k_count_inadm(const uint8_t *inadm, const uint8_t *bnd, int64_t n, unsigned long long *out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const unsigned ia = (i < n && !bnd[i] && inadm[i]) ? 1u : 0u;
    const unsigned b = __ballot_sync(0xffffffffu, ia);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, (unsigned long long)__popc(b));
}

// Gradient weights of the cached degree-1 fit: the reconstruction pre-pass (apply_weights, Interpolators.jl:585-602)
// computes g_b = invL Σ_c inv_r[b][c] Σ_k w_k x_k[c] (f_j - f_i); regrouped per slot, g_b = Σ_k gw_k[b] (f_j - f_i).
__global__ void k_grad_weights(int64_t n, int64_t npad, int D, int kmax, const int32_t *cnt, const double *dist,
                               const double *w, const double *inv_r, const uint8_t *ok_r, double invL, float *gw) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = ok_r[i] ? cnt[i] : 0;
    const double *inv = inv_r + i * D * D;
    for (int k = 0; k < kmax; ++k) {
        double x[3] = {0.0, 0.0, 0.0};
        const double wk = k < c ? w[int64_t(k) * npad + i] : 0.0;
        for (int d = 0; d < D; ++d) x[d] = k < c ? dist[(int64_t(k) * D + d) * npad + i] * invL : 0.0;
        for (int b = 0; b < D; ++b) {
            double acc = 0.0;
            for (int q = 0; q < D; ++q) acc += inv[b * D + q] * x[q];
            gw[(int64_t(k) * D + b) * npad + i] = float(invL * (wk * acc));
        }
    }
}

// total_mass (Volumes.jl:103-107) in FP64.
template <typename T>
__global__ void k_total_mass(const T *U, const double *vol, int64_t n, int M, double *out) {
    __shared__ double red[HCC_BLOCK / 32][HCC_MAX_VARS];
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (int m = 0; m < M; ++m) {
        double v = (i < n) ? vol[i] * double(U[i * M + m]) : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][m] = v;
    }
    __syncthreads();
    if (threadIdx.x < M) {
        double s = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
        atomicAdd(&out[threadIdx.x], s);
    }
}

// slot-major [ (k*width + c) * npad + i ] -> row-major [ (rowstart[i] + k) * width + c ]
template <typename E>
__global__ void k_rows(const E *src, E *dst, const int32_t *cnt, const int64_t *rowstart, int64_t n, int64_t npad,
                       int width) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cnt[i];
    int64_t r0 = rowstart[i];
    for (int k = 0; k < c; ++k)
        for (int q = 0; q < width; ++q) dst[(r0 + k) * width + q] = src[(int64_t(k) * width + q) * npad + i];
}

// slot-major [ (k*width + c) * npad + ids[q] ] -> [ (q*max_slots + k) * width + c ] for the selected particles;
// the slots of a row past the particle's count are zero
template <typename E>
__global__ void k_rows_of(const E *src, E *dst, const int32_t *cnt, const int64_t *ids, int64_t n_sel, int64_t npad,
                          int width, int max_slots) {
    const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= n_sel) return;
    const int64_t i = ids[q];
    const int c = cnt[i] < max_slots ? cnt[i] : max_slots;
    for (int k = 0; k < max_slots; ++k)
        for (int e = 0; e < width; ++e)
            dst[(q * max_slots + k) * width + e] = k < c ? src[(int64_t(k) * width + e) * npad + i] : E(0);
}

// Eight independent chains of dependent FP64 FMAs per thread (x <- x a + b, bounded: converges to b / (1 - a)); the
// sum is written only when it equals an impossible value, so the chains stay live without a store per thread.
__global__ void __launch_bounds__(256) k_fp64_fma(double *sink, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = double(threadIdx.x) * 1e-9 + q;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = fma(x[q], a, b);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s = s + x[q];
    if (s == -1.0) sink[0] = s;
}

}  // namespace

double fp64_fma_rate_tflops(int sms, cudaStream_t st, cudaError_t *err) {
    double *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.0f;
    const int iters = 1 << 14, blocks = sms * 8, threads = 256;
    cudaError_t e = cudaMalloc(&sink, sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_fp64_fma<<<blocks, threads, 0, st>>>(sink, iters / 16, 0.999999, 1e-6);   // warm-up
        cudaEventRecord(e0, st);
        k_fp64_fma<<<blocks, threads, 0, st>>>(sink, iters, 0.999999, 1e-6);
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    *err = e;
    if (e != cudaSuccess || ms <= 0.0f) return 0.0;
    const double flops = 2.0 * 8.0 * double(iters) * double(blocks) * double(threads);
    return flops / (double(ms) * 1e-3) / 1e12;
}

void launch_cast_f64_to_f32(const double *src, float *dst, int64_t n, cudaStream_t s) {
    if (n > 0) k_cast_f64_f32<<<grid_for(n), HCC_BLOCK, 0, s>>>(src, dst, n);
}
void launch_cast_f32_to_f64(const float *src, double *dst, int64_t n, cudaStream_t s) {
    if (n > 0) k_cast_f32_f64<<<grid_for(n), HCC_BLOCK, 0, s>>>(src, dst, n);
}
void launch_fill_i8(int8_t *p, int8_t v, int64_t n, cudaStream_t s) {
    if (n > 0) k_fill_i8<<<grid_for(n), HCC_BLOCK, 0, s>>>(p, v, n);
}
void launch_bc_apply(void *Y, const void *rhos, const int32_t *blist, const int32_t *bsrc, int64_t nb, int M,
                     int is_f32, cudaStream_t s) {
    if (nb <= 0) return;
    if (is_f32)
        k_bc<float><<<grid_for(nb), HCC_BLOCK, 0, s>>>(static_cast<float *>(Y), static_cast<const float *>(rhos), blist,
                                                        bsrc, nb, M);
    else
        k_bc<double><<<grid_for(nb), HCC_BLOCK, 0, s>>>(static_cast<double *>(Y), static_cast<const double *>(rhos),
                                                         blist, bsrc, nb, M);
}
void launch_drop_decide(const DropArgs &a, int is_f32, int drop_blocks, cudaStream_t s) {
    const unsigned blocks = unsigned(a.bc_blocks + std::max(1, drop_blocks));
    if (is_f32) k_drop_decide<float><<<blocks, HCC_BLOCK, 0, s>>>(a);
    else k_drop_decide<double><<<blocks, HCC_BLOCK, 0, s>>>(a);
}
void launch_reach_hop2(ListCounts *counts, const int32_t *dtiles, int32_t *dtiles_out, uint32_t *dmask,
                       uint32_t *words1, const int32_t *cnt, const int32_t *nidx, int64_t npad, int blocks,
                       cudaStream_t s) {
    k_reach_fix<<<blocks, HCC_BLOCK, 0, s>>>(counts, dtiles, dmask, words1);
    k_reach_hop2<<<blocks, HCC_BLOCK, 0, s>>>(counts, dtiles_out, dmask, words1, cnt, nidx, npad);
}
void launch_nbmin(const int8_t *orders, int8_t *nbmin, const int32_t *cnt, const int32_t *nidx, int64_t n,
                  int64_t npad, const int32_t *tiles, const uint32_t *words, const unsigned *count, int blocks,
                  cudaStream_t s) {
    if (tiles)
        k_nbmin_tiles<<<blocks, HCC_BLOCK, 0, s>>>(orders, nbmin, cnt, nidx, npad, tiles, words, count);
    else if (n > 0)
        k_nbmin<<<grid_for(n), HCC_BLOCK, 0, s>>>(orders, nbmin, cnt, nidx, n, npad);
}
void launch_u2_range(const void *U, int64_t n, int M, int is_f32, unsigned long long *keys, cudaStream_t s) {
    cudaMemsetAsync(keys, 0xff, size_t(M) * sizeof(unsigned long long), s);
    cudaMemsetAsync(keys + M, 0, size_t(M + 1) * sizeof(unsigned long long), s);
    if (n <= 0) return;
    if (is_f32) k_u2_range<float><<<grid_for(n), HCC_BLOCK, 0, s>>>(static_cast<const float *>(U), n, M, keys);
    else k_u2_range<double><<<grid_for(n), HCC_BLOCK, 0, s>>>(static_cast<const double *>(U), n, M, keys);
}
void launch_force(const int32_t *ctiles, uint32_t *cmask, ListCounts *counts, int32_t *ctiles_out, int8_t *orders,
                  const uint8_t *bnd, const int32_t *cnt, const int32_t *nidx, int64_t npad, int32_t *forced,
                  uint32_t *fmask, int32_t *ftiles, int blocks, cudaStream_t s) {
    k_force_push<<<blocks, HCC_BLOCK, 0, s>>>(ctiles, cmask, counts, orders, bnd, cnt, nidx, npad, forced, fmask, ftiles);
    k_force_apply<<<blocks, HCC_BLOCK, 0, s>>>(counts, ftiles, fmask, forced, orders, cmask, ctiles_out);
}
void launch_count_inadmissible(const uint8_t *inadm, const uint8_t *bnd, int64_t n, unsigned long long *out,
                               cudaStream_t s) {
    if (n > 0) k_count_inadm<<<grid_for(n), HCC_BLOCK, 0, s>>>(inadm, bnd, n, out);
}
void launch_grad_weights(int64_t n, int64_t npad, int D, int kmax, const int32_t *cnt, const double *dist,
                         const double *w, const double *inv_r, const uint8_t *ok_r, double invL, float *gw,
                         cudaStream_t s) {
    if (n > 0) k_grad_weights<<<grid_for(n), HCC_BLOCK, 0, s>>>(n, npad, D, kmax, cnt, dist, w, inv_r, ok_r, invL, gw);
}
// ShepardVolumes (Volumes.jl:183-229): kernel sums and the 1/S start, the partition-of-unity sweeps, and the
// clamped volumes' block partial sums for the renormalisation.
__global__ void k_shepard_sums(const int32_t *cnt, const double *w, int64_t n, int64_t npad, double w0, double *S,
                               double *V) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sm = w0;
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) sm = sm + w[int64_t(k) * npad + i];
    S[i] = sm;
    V[i] = 1.0 / sm;
}
__global__ void k_shepard_sweep(const int32_t *cnt, const int32_t *nidx, const double *w, int64_t n, int64_t npad,
                                double w0, const double *S, const double *V, double *Vt) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = (w0 / S[i]) * V[i];
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) {
        const int64_t j = nidx[int64_t(k) * npad + i];
        acc = acc + (w[int64_t(k) * npad + i] / S[j]) * V[j];
    }
    Vt[i] = acc;
}
__global__ void k_clamp_partials(double *V, int64_t n, double *partial) {
    __shared__ double sh[HCC_BLOCK];
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        v = V[i] > 0.0 ? V[i] : 0.0;
        V[i] = v;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (int(threadIdx.x) < o) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}
__global__ void k_scale(double *V, int64_t n, double f) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) V[i] = V[i] * f;
}

void launch_shepard(const int32_t *cnt, const int32_t *nidx, const double *w, int64_t n, int64_t npad, double w0,
                    int sweeps, double *S, double *V, double *Vt, double *partial, cudaStream_t s) {
    if (n <= 0) return;
    k_shepard_sums<<<grid_for(n), HCC_BLOCK, 0, s>>>(cnt, w, n, npad, w0, S, V);
    for (int q = 0; q < sweeps; ++q) {
        k_shepard_sweep<<<grid_for(n), HCC_BLOCK, 0, s>>>(cnt, nidx, w, n, npad, w0, S, V, Vt);
        cudaMemcpyAsync(V, Vt, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
    k_clamp_partials<<<grid_for(n), HCC_BLOCK, 0, s>>>(V, n, partial);
}
void launch_scale(double *V, int64_t n, double f, cudaStream_t s) {
    if (n > 0) k_scale<<<grid_for(n), HCC_BLOCK, 0, s>>>(V, n, f);
}
unsigned shepard_blocks(int64_t n) { return grid_for(n); }

void launch_total_mass(const void *U, const double *vol, int64_t n, int M, int is_f32, double *out, cudaStream_t s) {
    cudaMemsetAsync(out, 0, sizeof(double) * M, s);
    if (n <= 0) return;
    if (is_f32) k_total_mass<float><<<grid_for(n), HCC_BLOCK, 0, s>>>(static_cast<const float *>(U), vol, n, M, out);
    else k_total_mass<double><<<grid_for(n), HCC_BLOCK, 0, s>>>(static_cast<const double *>(U), vol, n, M, out);
}
void launch_gather_rows(const void *src, void *dst, const int32_t *cnt, const int64_t *rowstart, int64_t n,
                        int64_t npad, int width, int elem_bytes, cudaStream_t s) {
    if (n <= 0) return;
    if (elem_bytes == 8)
        k_rows<unsigned long long><<<grid_for(n), HCC_BLOCK, 0, s>>>(
            static_cast<const unsigned long long *>(src), static_cast<unsigned long long *>(dst), cnt, rowstart, n, npad, width);
    else if (elem_bytes == 4)
        k_rows<unsigned int><<<grid_for(n), HCC_BLOCK, 0, s>>>(
            static_cast<const unsigned int *>(src), static_cast<unsigned int *>(dst), cnt, rowstart, n, npad, width);
}

void launch_gather_rows_of(const void *src, void *dst, const int32_t *cnt, const int64_t *ids, int64_t n_sel,
                           int64_t npad, int width, int max_slots, int elem_bytes, cudaStream_t s) {
    if (n_sel <= 0) return;
    if (elem_bytes == 8)
        k_rows_of<unsigned long long><<<grid_for(n_sel), HCC_BLOCK, 0, s>>>(
            static_cast<const unsigned long long *>(src), static_cast<unsigned long long *>(dst), cnt, ids, n_sel, npad,
            width, max_slots);
    else if (elem_bytes == 4)
        k_rows_of<unsigned int><<<grid_for(n_sel), HCC_BLOCK, 0, s>>>(
            static_cast<const unsigned int *>(src), static_cast<unsigned int *>(dst), cnt, ids, n_sel, npad, width,
            max_slots);
}

}  // namespace hcc
