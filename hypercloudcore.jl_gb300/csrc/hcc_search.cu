// hcc_search.cu — cell-list neighbour search on the device (compiled with -fmad=false: the FP64 distances,
// r² tests and weights must match the reference's rounding, src/Grid/NeighborLogic.jl).
//
// Pipeline: bin + histogram (atomics) -> exclusive scan of the bin counts -> scatter (atomic cursor) ->
// per-bin sort by descending particle index (the only order the reference's lists depend on) -> count pass ->
// capacity check on the host -> write pass into slot-major arrays (slot k of particle i at k*npad + i).
#include "hcc_internal.cuh"

namespace hcc {
namespace {

__device__ __forceinline__ double jmod(double x, double y) {
    double r = fmod(x, y);
    if (r == 0.0) return copysign(r, y);
    if ((r > 0) != (y > 0)) return r + y;
    return r;
}

// _wrap_position! (NeighborLogic.jl:279-286) + get_flat_bin_index (:86-102) + _bin_count! (:139-144)
__global__ void k_bin(SearchArgs a) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int64_t lin = 0, stride = 1;
    for (int d = 0; d < a.D; ++d) {
        double p = a.pos[d * a.npad + i];
        if (a.periodic[d]) {
            p = a.cmin[d] + jmod(p - a.cmin[d], a.Lphys[d]);
            a.pos[d * a.npad + i] = p;
        }
        double f = floor((p - a.cmin[d]) / a.csize[d]);
        int64_t id = int64_t(f) + 1;
        id = id < 1 ? 1 : (id > a.dims[d] ? a.dims[d] : id);
        lin += (id - 1) * stride;
        stride *= a.dims[d];
    }
    a.bin_of[i] = int32_t(lin);
    atomicAdd(&a.cell_count[lin], 1);
}

// Exclusive scan of the bin counts into cell_start (one block; the bin count is at most a few 10^6).
__global__ void k_scan_bins(const int32_t *count, int64_t *start, int64_t nbins, int64_t n) {
    __shared__ int64_t warp_sums[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t base = 0; base < nbins; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        int64_t v = (i < nbins) ? count[i] : 0;
        int64_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int64_t s = (lane < int(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int64_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        int64_t incl = x + (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
        if (i < nbins) start[i] = incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        start[nbins] = n;        // dummy bin: empty
        start[nbins + 1] = n;
    }
}

// _bin_scatter! (NeighborLogic.jl:146-151)
__global__ void k_scatter(SearchArgs a) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int32_t b = a.bin_of[i];
    int32_t k = atomicAdd(&a.cell_cursor[b], 1);
    a.cellp[a.cell_start[b] + k] = int32_t(i);
}

// _bin_sort! (NeighborLogic.jl:153-167): insertion sort of each bin, descending index.
__global__ void k_binsort(SearchArgs a) {
    int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= a.nbins) return;
    int64_t lo = a.cell_start[b], hi = a.cell_start[b + 1] - 1;
    for (int64_t s = lo + 1; s <= hi; ++s) {
        int32_t v = a.cellp[s];
        int64_t t = s - 1;
        while (t >= lo && a.cellp[t] < v) {
            a.cellp[t + 1] = a.cellp[t];
            --t;
        }
        a.cellp[t + 1] = v;
    }
}

// get_distance (ParticleGrids.jl:209-219) and sum(abs2, dist)
template <int D>
__device__ __forceinline__ double pair_distance(const SearchArgs &a, int64_t i, int64_t j, double *dist) {
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        double dx = a.pos[d * a.npad + j] - a.pos[d * a.npad + i];
        dist[d] = dx - a.Lwrap[d] * rint(dx * a.invLwrap[d]);
        s = (d == 0) ? dist[d] * dist[d] : s + dist[d] * dist[d];
    }
    return s;
}

// FP32 copy of the positions and the largest |coordinate| over the cloud (non-negative floats order like their
// bits), for the prefilter of the count and write passes.
__global__ void k_prep32(SearchArgs a) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    float m = 0.0f;
    if (i < a.n) {
        for (int d = 0; d < a.D; ++d) {
            const float f = float(a.pos[d * a.npad + i]);
            a.pos32[d * a.npad + i] = f;
            m = fmaxf(m, fabsf(f));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(a.pmax, __float_as_uint(m));
}

// Exact FP32 prefilter of the test r^2 <= R^2. With u = 2^-24, P the largest |coordinate| and L the largest wrap
// length, each FP32 axis offset (positions rounded to FP32, the same wrap integer as the FP64 path) lies within
// Delta = 16 u (P + L) of the FP64 one, and the FP32 sum of squares s within rho s (s >= R^2) or rho R^2 (s < R^2) of
// the FP64 r^2, rho = 2 (2 sqrt(D) Delta / R + 3 D Delta^2 / R^2 + D u) (a factor 2 of margin). So s < R^2 (1 - rho)
// proves the pair inside and s > R^2 / (1 - rho) outside; the band between, a wrap quotient within 0.01 of a half
// integer (where the FP32 and FP64 wrap integers may differ), a NaN or rho >= 0.05 leave the decision to FP64.
// The lists, their order, weights and distances are therefore those of the FP64 test, bit for bit.
template <int D> struct Prefilter {
    bool on;
    float lo, hi, pi[3];
    __device__ __forceinline__ Prefilter(const SearchArgs &a, int64_t i) : on(false), lo(0.0f), hi(0.0f) {
        pi[0] = pi[1] = pi[2] = 0.0f;
        if (!a.pos32) return;
        const double u = 5.9604644775390625e-08;
        const double P = double(__uint_as_float(*a.pmax));
        const double delta = 16.0 * u * (P + a.Lmax);
        const double R = sqrt(a.R_sq);
        const double rho = 2.0 * (2.0 * sqrt(double(D)) * delta / R + 3.0 * D * delta * delta / a.R_sq + D * u);
        if (!(rho < 0.05)) return;
        on = true;
        lo = __double2float_rd(a.R_sq * (1.0 - rho));
        hi = __double2float_ru(a.R_sq / (1.0 - rho));
#pragma unroll
        for (int d = 0; d < D; ++d) pi[d] = a.pos32[d * a.npad + i];
    }
    // +1: inside, -1: outside, 0: undecided (the FP64 test decides)
    __device__ __forceinline__ int decide(const SearchArgs &a, int64_t j) const {
        float s = 0.0f;
        bool amb = false;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const float dx = __fsub_rn(a.pos32[d * a.npad + j], pi[d]);
            const float q = __fmul_rn(dx, a.invL32[d]);
            const float r = rintf(q);
            amb = amb || fabsf(__fsub_rn(fabsf(__fsub_rn(q, r)), 0.5f)) < 0.01f;
            const float dd = __fsub_rn(dx, __fmul_rn(a.L32[d], r));
            s = (d == 0) ? __fmul_rn(dd, dd) : __fadd_rn(s, __fmul_rn(dd, dd));
        }
        if (amb) return 0;
        return s < lo ? 1 : (s > hi ? -1 : 0);
    }
};

// _count_neighbours! (NeighborLogic.jl:288-301); stats: [0] max count, [1] total, [2] min interior count
template <int D>
__global__ void k_count(SearchArgs a, unsigned long long *stats) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int32_t c = 0;
    if (i < a.n) {
        const int64_t *win = a.binnb + int64_t(a.bin_of[i]) * a.noff;
        const Prefilter<D> pf(a, i);
        double dist[3];
        for (int w = 0; w < a.noff; ++w) {
            int64_t b = win[w];
            for (int64_t s = a.cell_start[b]; s < a.cell_start[b + 1]; ++s) {
                int32_t j = a.cellp[s];
                if (j == i) continue;
                const int dec = pf.on ? pf.decide(a, j) : 0;
                if (dec > 0 || (dec == 0 && pair_distance<D>(a, i, j, dist) <= a.R_sq)) ++c;
            }
        }
        a.cnt[i] = c;
    }
    // warp-aggregated statistics
    unsigned long long mx = (i < a.n) ? (unsigned long long)c : 0ull;
    unsigned long long sm = mx;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long om = __shfl_down_sync(0xffffffffu, mx, o);
        unsigned long long os = __shfl_down_sync(0xffffffffu, sm, o);
        mx = om > mx ? om : mx;
        sm += os;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&stats[0], mx);
        atomicAdd(&stats[1], sm);
    }
}

// ExponentialWeightFunction (MLSWeightFunctions.jl:68-82)
__device__ __forceinline__ double exp_weight(double d2, double alpha, double invR2) {
    double arg = (-alpha) * d2 * invR2;
    double y = -arg;
    double den = 1.0 + y * (1.0 + y * (0.5 + y * (0.16666666666666666 + y * 0.041666666666666664)));
    return 1.0 / den;
}

// _write_neighbours! (NeighborLogic.jl:309-329) into the slot-major layout. With the FP32 prefilter in two phases:
// the candidates in window order, decided in FP32 (FP64 only in the undecided band), give the slot indices; then
// every lane computes the FP64 distances and weights of its own slots with the warp converged (a warp instruction
// costs the FP64 unit the same with one lane or 32, and about one candidate in six is accepted). The values and
// their order are those of the one-phase FP64 loop.
template <int D>
__global__ void k_write(SearchArgs a) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int64_t *win = a.binnb + int64_t(a.bin_of[i]) * a.noff;
    const Prefilter<D> pf(a, i);
    double dist[3];
    int k = 0;
    if (pf.on) {
        for (int w = 0; w < a.noff; ++w) {
            int64_t b = win[w];
            for (int64_t s = a.cell_start[b]; s < a.cell_start[b + 1]; ++s) {
                int32_t j = a.cellp[s];
                if (j == i) continue;
                const int dec = pf.decide(a, j);
                if (dec > 0 || (dec == 0 && pair_distance<D>(a, i, j, dist) <= a.R_sq)) {
                    if (k < a.kmax) a.nidx[int64_t(k) * a.npad + i] = j;
                    ++k;
                }
            }
        }
        const int nk = k < a.kmax ? k : a.kmax;
        for (int q = 0; q < nk; ++q) {
            const int64_t slot = int64_t(q) * a.npad + i;
            const double d2 = pair_distance<D>(a, i, a.nidx[slot], dist);
            a.w[slot] = exp_weight(d2, a.alpha, a.invR2);
#pragma unroll
            for (int d = 0; d < D; ++d) a.dist[(int64_t(q) * D + d) * a.npad + i] = dist[d];
        }
        return;
    }
    for (int w = 0; w < a.noff; ++w) {
        int64_t b = win[w];
        for (int64_t s = a.cell_start[b]; s < a.cell_start[b + 1]; ++s) {
            int32_t j = a.cellp[s];
            if (j == i) continue;
            double d2 = pair_distance<D>(a, i, j, dist);
            if (d2 <= a.R_sq) {
                if (k < a.kmax) {
                    int64_t slot = int64_t(k) * a.npad + i;
                    a.nidx[slot] = j;
                    a.w[slot] = exp_weight(d2, a.alpha, a.invR2);
#pragma unroll
                    for (int d = 0; d < D; ++d) a.dist[(int64_t(k) * D + d) * a.npad + i] = dist[d];
                }
                ++k;
            }
        }
    }
}

// refresh_geometry! (GridMovers.jl:95-121): distances and weights of the existing slots at the current positions
// (start-of-step topology), weight 0 for pairs that drifted beyond R
template <int D>
__global__ void k_refresh(SearchArgs a) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int c = a.cnt[i];
    double dist[3];
    for (int k = 0; k < c; ++k) {
        const int64_t slot = int64_t(k) * a.npad + i;
        const double d2 = pair_distance<D>(a, i, a.nidx[slot], dist);
#pragma unroll
        for (int d = 0; d < D; ++d) a.dist[(int64_t(k) * D + d) * a.npad + i] = dist[d];
        a.w[slot] = d2 <= a.R_sq ? exp_weight(d2, a.alpha, a.invR2) : 0.0;
    }
}

inline unsigned grid_for(int64_t n) { return unsigned((n + HCC_BLOCK - 1) / HCC_BLOCK); }

hcc_status check_launch(std::string &err, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return HCC_ERR_CUDA;
    }
    return HCC_OK;
}

}  // namespace

hcc_status search_bins(SearchArgs &a, cudaStream_t s, std::string &err) {
    if (a.n == 0) return HCC_OK;
    cudaMemsetAsync(a.cell_count, 0, sizeof(int32_t) * (a.nbins + 1), s);
    cudaMemsetAsync(a.cell_cursor, 0, sizeof(int32_t) * a.nbins, s);
    k_bin<<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a);
    if (a.pos32) {
        cudaMemsetAsync(a.pmax, 0, sizeof(unsigned int), s);
        k_prep32<<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a);
    }
    k_scan_bins<<<1, 1024, 0, s>>>(a.cell_count, a.cell_start, a.nbins, a.n);
    k_scatter<<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a);
    k_binsort<<<grid_for(a.nbins), HCC_BLOCK, 0, s>>>(a);
    return check_launch(err, "neighbour search (cell list)");
}

hcc_status search_count(SearchArgs &a, cudaStream_t s, unsigned long long *d_stats, std::string &err) {
    if (a.n == 0) return HCC_OK;
    cudaMemsetAsync(d_stats, 0, sizeof(unsigned long long) * 2, s);
    switch (a.D) {
    case 1: k_count<1><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a, d_stats); break;
    case 2: k_count<2><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a, d_stats); break;
    default: k_count<3><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a, d_stats); break;
    }
    return check_launch(err, "neighbour search (count)");
}

hcc_status search_refresh(SearchArgs &a, cudaStream_t s, std::string &err) {
    if (a.n == 0) return HCC_OK;
    switch (a.D) {
    case 1: k_refresh<1><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a); break;
    case 2: k_refresh<2><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a); break;
    default: k_refresh<3><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a); break;
    }
    return check_launch(err, "geometry refresh");
}

hcc_status search_write(SearchArgs &a, cudaStream_t s, std::string &err) {
    if (a.n == 0) return HCC_OK;
    switch (a.D) {
    case 1: k_write<1><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a); break;
    case 2: k_write<2><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a); break;
    default: k_write<3><<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a); break;
    }
    return check_launch(err, "neighbour search (write)");
}

}  // namespace hcc
