// hcc_util.cu — small device passes of the time stepper: boundary conditions, MOOD decrement / mask dilation /
// neighbourhood orders, conserved totals, conversions and the row-major export of slot-major arrays.
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

// _mood_drop! (MOOD.jl:299-309) + the change count; also counts the interior candidates that are not admissible
// (_count_inadmissible, TimeSteppers.jl:481-490). counters: [0] changed, [1] inadmissible.
__global__ void k_mood_drop(int8_t *orders, uint8_t *triggered, uint8_t *changed, uint8_t *trig_step,
                            const uint8_t *inadm, const uint8_t *bnd, int64_t n, unsigned long long *counters) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned ch = 0, ia = 0;
    if (i < n) {
        uint8_t c = 0;
        if (triggered[i]) {
            if (orders[i] > 1) {
                orders[i] = int8_t(orders[i] - 1);
                c = 1;
                trig_step[i] = 1;
            }
            triggered[i] = 0;
        }
        changed[i] = c;
        ch = c;
        ia = (!bnd[i] && inadm[i]) ? 1u : 0u;
    }
    unsigned bc = __ballot_sync(0xffffffffu, ch), bi = __ballot_sync(0xffffffffu, ia);
    if ((threadIdx.x & 31) == 0) {
        if (bc) atomicAdd(&counters[0], (unsigned long long)__popc(bc));
        if (bi) atomicAdd(&counters[1], (unsigned long long)__popc(bi));
    }
}

// One hop of expand_mask! (_expand_body!, MOOD.jl:323-335: a particle is marked if it or a neighbour was), as a
// push from the marked particles: the neighbour relation is symmetric (one radius, exactly antisymmetric
// distances), so marking every neighbour of a marked particle marks the same set as the pull over all particles,
// while only the few marked particles read their lists. dst must be cleared before.
__global__ void k_expand(const uint8_t *src, uint8_t *dst, const int32_t *cnt, const int32_t *nidx, int64_t n,
                         int64_t npad) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !src[i]) return;
    dst[i] = 1;
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) dst[nidx[int64_t(k) * npad + i]] = 1;
}

// _nb_min_order (MOOD.jl:66-74) for EPD2.
__global__ void k_nbmin(const int8_t *orders, int8_t *nbmin, const int32_t *cnt, const int32_t *nidx, int64_t n,
                        int64_t npad) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int8_t o = orders[i];
    int c = cnt[i];
    for (int k = 0; k < c; ++k) {
        int8_t oj = orders[nidx[int64_t(k) * npad + i]];
        o = oj < o ? oj : o;
    }
    nbmin[i] = o;
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

// Decision of one MOOD fixed-point iteration inside a step graph, after a drop pass (the loop condition of
// mood_checkpoint!, TimeSteppers.jl:461-476): no changed order ends the loop and adds the inadmissible count;
// otherwise the flagged count grows and the loop repeats, unless the checkpoint already ran `cap` recomputes
// (the timeout flag ends it). One thread.
__global__ void k_mood_decide(const unsigned long long *counters, MoodStats *st, cudaGraphConditionalHandle h,
                              int cap) {
    const unsigned long long changed = counters[0];
    unsigned go = 0;
    if (changed == 0) {
        st->inadmissible += counters[1];
        st->iter_in_checkpoint = 0;
    } else {
        st->flagged += changed;
        if (st->iter_in_checkpoint >= unsigned(cap)) {
            st->timeout = 1;
            st->iter_in_checkpoint = 0;
        } else {
            st->iter_in_checkpoint += 1;
            st->iterations += 1;
            go = 1;
        }
    }
    cudaGraphSetConditional(h, go);
}

}  // namespace

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
void launch_mood_drop(int8_t *orders, uint8_t *triggered, uint8_t *changed, uint8_t *trig_step, const uint8_t *inadm,
                      const uint8_t *bnd, int64_t n, unsigned long long *counters, cudaStream_t s) {
    cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), s);
    if (n > 0) k_mood_drop<<<grid_for(n), HCC_BLOCK, 0, s>>>(orders, triggered, changed, trig_step, inadm, bnd, n, counters);
}
void launch_mood_decide(const unsigned long long *counters, MoodStats *stats, cudaGraphConditionalHandle h, int cap,
                        cudaStream_t s) {
    k_mood_decide<<<1, 1, 0, s>>>(counters, stats, h, cap);
}
void launch_expand(const uint8_t *src, uint8_t *dst, const int32_t *cnt, const int32_t *nidx, int64_t n, int64_t npad,
                   cudaStream_t s) {
    if (n <= 0) return;
    cudaMemsetAsync(dst, 0, size_t(n), s);
    k_expand<<<grid_for(n), HCC_BLOCK, 0, s>>>(src, dst, cnt, nidx, n, npad);
}
void launch_nbmin(const int8_t *orders, int8_t *nbmin, const int32_t *cnt, const int32_t *nidx, int64_t n, int64_t npad,
                  cudaStream_t s) {
    if (n > 0) k_nbmin<<<grid_for(n), HCC_BLOCK, 0, s>>>(orders, nbmin, cnt, nidx, n, npad);
}
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

}  // namespace hcc
