// hcc_tiles.cu — the tile tables of the FP32 full passes (see TileView in hcc_internal.cuh).
//
// Built once per geometry, after the neighbour search and the FP64 MLS caches:
//   1. per tile (one block): the ids of its particles and of all their neighbours, bitonic-sorted in shared memory,
//      duplicates and padding dropped -> a per-tile list and its length;
//   2. on the host: the exclusive scan of the lengths (union offsets) and the largest union;
//   3. per tile (one block): the lists compacted into one array, and every entry's position relative to the
//      tile's first particle (the minimum-image offset on periodic axes) as int32 multiples of a power-of-two
//      quantum chosen from the tile's extent (|offset| <= 2^29 quanta, so differences stay within int32);
//   4. per particle: each slot's place in the tile's union (binary search) and the particle's own place;
//   5. per particle: the FP32 rows of the cached fits from the FP64 inverse moments.
#include "hcc_internal.cuh"
#include <algorithm>
#include <climits>
#include <vector>

namespace hcc {
namespace {

constexpr int kSortThreads = 1024;

template <typename P> void tfree(P *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Step 1: the sorted, duplicate-free union of tile t into tmp[t * cap ...), its length into ucount[t].
// Shared memory: cap2 ints (a power of two >= cap = HCC_TILE (kmax + 1)) and kSortThreads scan words.
__global__ void __launch_bounds__(kSortThreads) k_tile_union(int64_t n, int64_t npad, int kmax, const int32_t *cnt,
                                                             const int32_t *nidx, int cap, int cap2, int32_t *tmp,
                                                             int32_t *ucount) {
    extern __shared__ int32_t sh[];
    int32_t *keys = sh;
    int32_t *scan = sh + cap2;
    const int64_t t = blockIdx.x;
    const int64_t i0 = t * HCC_TILE;
    for (int q = threadIdx.x; q < cap2; q += blockDim.x) {
        int32_t v = INT_MAX;
        if (q < cap) {
            const int p = q % HCC_TILE, k = q / HCC_TILE;
            const int64_t i = i0 + p;
            if (i < n) {
                if (k == 0) v = int32_t(i);
                else if (k - 1 < cnt[i]) v = nidx[int64_t(k - 1) * npad + i];
            }
        }
        keys[q] = v;
    }
    __syncthreads();
    // bitonic sort, ascending
    for (int size = 2; size <= cap2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int q = threadIdx.x; q < cap2 / 2; q += blockDim.x) {
                const int lo = 2 * stride * (q / stride) + (q % stride);
                const int hi = lo + stride;
                const bool up = ((lo & size) == 0);
                const int32_t a = keys[lo], b = keys[hi];
                if ((a > b) == up) { keys[lo] = b; keys[hi] = a; }
            }
            __syncthreads();
        }
    }
    // unique: each thread takes a contiguous chunk, counts its first occurrences, block exclusive scan, writes
    const int per = cap2 / kSortThreads;
    const int c0 = threadIdx.x * per;
    int mine = 0;
    for (int q = c0; q < c0 + per; ++q) {
        const int32_t v = keys[q];
        mine += (v != INT_MAX && (q == 0 || keys[q - 1] != v)) ? 1 : 0;
    }
    scan[threadIdx.x] = mine;
    __syncthreads();
    for (int off = 1; off < kSortThreads; off <<= 1) {     // Hillis-Steele inclusive scan
        const int v = threadIdx.x >= off ? scan[threadIdx.x - off] : 0;
        __syncthreads();
        scan[threadIdx.x] += v;
        __syncthreads();
    }
    int pos = scan[threadIdx.x] - mine;
    int32_t *out = tmp + t * int64_t(cap);
    for (int q = c0; q < c0 + per; ++q) {
        const int32_t v = keys[q];
        if (v != INT_MAX && (q == 0 || keys[q - 1] != v)) out[pos++] = v;
    }
    if (threadIdx.x == kSortThreads - 1) ucount[t] = scan[threadIdx.x];
}

__device__ __forceinline__ double wrap_offset(double dx, int per, double L, double invL) {
    return per ? dx - L * nearbyint(dx * invL) : dx;
}

struct UnionArgs {
    int64_t n, npad;
    int D, cap;
    const int32_t *tmp;
    const int64_t *ustart;
    const double *pos;
    int periodic[3];
    double Lwrap[3], invLwrap[3], R;
    int32_t *uid;
    int4 *upos;
    float *quantum;
    int *fail;                        // set when a periodic axis is too short for consistent offsets
};

// Step 3: compaction and quantised offsets of tile t (one block).
__global__ void __launch_bounds__(256) k_tile_positions(const UnionArgs a) {
    __shared__ double red[256 / 32][3];
    __shared__ double s_q;
    const int64_t t = blockIdx.x;
    const int64_t u0 = a.ustart[t];
    const int nu = int(a.ustart[t + 1] - u0);
    const int64_t iref = t * HCC_TILE;
    double xr[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < a.D; ++d) xr[d] = a.pos[int64_t(d) * a.npad + iref];
    double ext[3] = {0.0, 0.0, 0.0};
    for (int e = threadIdx.x; e < nu; e += blockDim.x) {
        const int32_t j = a.tmp[t * int64_t(a.cap) + e];
        a.uid[u0 + e] = j;
        for (int d = 0; d < a.D; ++d) {
            const double o = wrap_offset(a.pos[int64_t(d) * a.npad + j] - xr[d], a.periodic[d], a.Lwrap[d],
                                         a.invLwrap[d]);
            ext[d] = fmax(ext[d], fabs(o));
        }
    }
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) ext[d] = fmax(ext[d], __shfl_down_sync(0xffffffffu, ext[d], o));
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; ++d) red[threadIdx.x >> 5][d] = ext[d];
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int d = 0; d < a.D; ++d) {
            double ed = 0.0;
            for (int w = 0; w < int(blockDim.x >> 5); ++w) ed = fmax(ed, red[w][d]);
            // minimum-image offsets of the union stay consistent while 2 ext < L - R on a periodic axis
            if (a.periodic[d] && !(2.0 * ed < a.Lwrap[d] - a.R)) atomicExch(a.fail, 1);
            m = fmax(m, ed);
        }
        int ex = 0;
        if (m > 0.0) frexp(m, &ex);                // m < 2^ex
        s_q = ldexp(1.0, ex - 29);                 // |offset| / quantum < 2^29
        a.quantum[t] = float(s_q);
    }
    __syncthreads();
    const double inv_q = 1.0 / s_q;                // exact: a power of two
    for (int e = threadIdx.x; e < nu; e += blockDim.x) {
        const int32_t j = a.uid[u0 + e];
        int q[3] = {0, 0, 0};
        for (int d = 0; d < a.D; ++d) {
            const double o = wrap_offset(a.pos[int64_t(d) * a.npad + j] - xr[d], a.periodic[d], a.Lwrap[d],
                                         a.invLwrap[d]);
            q[d] = int(llrint(o * inv_q));
        }
        a.upos[u0 + e] = make_int4(q[0], q[1], q[2], 0);
    }
}

__device__ __forceinline__ int find_in(const int32_t *u, int nu, int32_t v) {
    int lo = 0, hi = nu - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (u[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Step 4: the union place of every slot and of the particle itself.
__global__ void k_tile_lidx(int64_t n, int64_t npad, const int32_t *cnt, const int32_t *nidx, const int64_t *ustart,
                            const int32_t *uid, uint16_t *lidx, uint16_t *lself) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t t = i / HCC_TILE;
    const int32_t *u = uid + ustart[t];
    const int nu = int(ustart[t + 1] - ustart[t]);
    lself[i] = uint16_t(find_in(u, nu, int32_t(i)));
    const int c = cnt[i];
    for (int k = 0; k < c; ++k) lidx[int64_t(k) * npad + i] = uint16_t(find_in(u, nu, nidx[int64_t(k) * npad + i]));
}

// Step 5: FP32 rows of the cached fits.
__global__ void k_tile_coef(int64_t n, int D, const double *inv_r, const double *inv_d, const uint8_t *ok_r,
                            const uint8_t *ok_d, double invL, int cw, float *coef) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float *c = coef + i * cw;
    for (int q = 0; q < cw; ++q) c[q] = 0.0f;
    const int Bd = D + 1;
    const double il2 = invL * invL;
    if (ok_d[i]) {
        const double *v = inv_d + i * Bd * Bd;
        for (int d = 0; d < D; ++d) {
            c[d] = float(v[(1 + d) * Bd] * invL);
            for (int e = 0; e < D; ++e) c[D + d * D + e] = float(v[(1 + d) * Bd + 1 + e] * il2);
        }
    }
    if (ok_r[i]) {
        const double *v = inv_r + i * D * D;
        for (int b = 0; b < D; ++b)
            for (int e = 0; e < D; ++e) c[D + D * D + b * D + e] = float(v[b * D + e] * il2);
    }
}

}  // namespace

void TileTables::release() {
    tfree(ustart); tfree(uid); tfree(upos); tfree(quantum); tfree(lidx); tfree(lself); tfree(coef);
    ntiles = utotal = 0;
    umax = 0;
    ok = 0;
}

hcc_status build_tile_tables(const TileBuild &b, TileTables &t, cudaStream_t s, std::string &err) {
    t.release();
    if (b.n <= 0) return HCC_OK;
    auto cu = [&](cudaError_t e, const char *what) -> hcc_status {
        if (e == cudaSuccess) return HCC_OK;
        err = std::string("tile tables: ") + what + ": " + cudaGetErrorString(e);
        return HCC_ERR_CUDA;
    };
    const int64_t ntiles = (b.n + HCC_TILE - 1) / HCC_TILE;
    const int cap = HCC_TILE * (b.kmax + 1);
    int cap2 = kSortThreads;
    while (cap2 < cap) cap2 <<= 1;
    const size_t sort_smem = size_t(cap2 + kSortThreads) * sizeof(int32_t);
    if (sort_smem > 160 * 1024) return HCC_OK;            // stencils too wide to sort a tile in shared memory
    hcc_status st;
    int32_t *tmp = nullptr, *ucount = nullptr;
    int *fail = nullptr;
    if ((st = cu(cudaMalloc(&tmp, size_t(ntiles) * cap * sizeof(int32_t)), "union buffer")) != HCC_OK) return st;
    if ((st = cu(cudaMalloc(&ucount, size_t(ntiles) * sizeof(int32_t)), "union counts")) != HCC_OK) {
        cudaFree(tmp);
        return st;
    }
    auto done = [&](hcc_status r) {
        tfree(tmp); tfree(ucount); tfree(fail);
        if (r != HCC_OK) t.release();
        return r;
    };
    if ((st = cu(cudaFuncSetAttribute(k_tile_union, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sort_smem)),
                 "sort shared memory")) != HCC_OK)
        return done(st);
    k_tile_union<<<unsigned(ntiles), kSortThreads, sort_smem, s>>>(b.n, b.npad, b.kmax, b.cnt, b.nidx, cap, cap2, tmp,
                                                                   ucount);
    if ((st = cu(cudaGetLastError(), "union sort")) != HCC_OK) return done(st);
    std::vector<int32_t> h_count(ntiles);
    if ((st = cu(cudaMemcpyAsync(h_count.data(), ucount, size_t(ntiles) * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
                 "union counts")) != HCC_OK)
        return done(st);
    if ((st = cu(cudaStreamSynchronize(s), "union sort")) != HCC_OK) return done(st);
    std::vector<int64_t> h_start(ntiles + 1, 0);
    int umax = 0;
    for (int64_t q = 0; q < ntiles; ++q) {
        h_start[q + 1] = h_start[q] + h_count[q];
        umax = std::max(umax, h_count[q]);
    }
    if (umax > 65535 || umax > b.max_union) return done(HCC_OK);   // not eligible: the caller keeps the slot streams
    t.ntiles = ntiles;
    t.utotal = h_start[ntiles];
    t.umax = umax;
    t.cw = ((b.D + 2 * b.D * b.D) + 3) / 4 * 4;
    t.wscale = float(b.wscale);
    if ((st = cu(cudaMalloc(&t.ustart, size_t(ntiles + 1) * sizeof(int64_t)), "union offsets")) != HCC_OK ||
        (st = cu(cudaMalloc(&t.uid, size_t(std::max<int64_t>(t.utotal, 1)) * sizeof(int32_t)), "union ids")) != HCC_OK ||
        (st = cu(cudaMalloc(&t.upos, size_t(std::max<int64_t>(t.utotal, 1)) * sizeof(int4)), "union positions")) != HCC_OK ||
        (st = cu(cudaMalloc(&t.quantum, size_t(ntiles) * sizeof(float)), "tile quanta")) != HCC_OK ||
        (st = cu(cudaMalloc(&t.lidx, size_t(std::max(b.kmax, 1)) * size_t(b.npad) * sizeof(uint16_t)), "slot places")) != HCC_OK ||
        (st = cu(cudaMalloc(&t.lself, size_t(b.n) * sizeof(uint16_t)), "own places")) != HCC_OK ||
        (st = cu(cudaMalloc(&t.coef, size_t(b.n) * t.cw * sizeof(float)), "fit rows")) != HCC_OK ||
        (st = cu(cudaMalloc(&fail, sizeof(int)), "flag")) != HCC_OK)
        return done(st);
    if ((st = cu(cudaMemcpyAsync(t.ustart, h_start.data(), size_t(ntiles + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                                 s), "union offsets")) != HCC_OK ||
        (st = cu(cudaMemsetAsync(fail, 0, sizeof(int), s), "flag")) != HCC_OK)
        return done(st);
    UnionArgs ua{};
    ua.n = b.n; ua.npad = b.npad; ua.D = b.D; ua.cap = cap; ua.tmp = tmp; ua.ustart = t.ustart; ua.pos = b.pos;
    for (int d = 0; d < 3; ++d) {
        ua.periodic[d] = b.periodic[d];
        ua.Lwrap[d] = b.Lwrap[d];
        ua.invLwrap[d] = b.invLwrap[d];
    }
    ua.R = b.R;
    ua.uid = t.uid; ua.upos = t.upos; ua.quantum = t.quantum; ua.fail = fail;
    k_tile_positions<<<unsigned(ntiles), 256, 0, s>>>(ua);
    const unsigned g = unsigned((b.n + 255) / 256);
    k_tile_lidx<<<g, 256, 0, s>>>(b.n, b.npad, b.cnt, b.nidx, t.ustart, t.uid, t.lidx, t.lself);
    k_tile_coef<<<g, 256, 0, s>>>(b.n, b.D, b.inv_r, b.inv_d, b.ok_r, b.ok_d, b.invL, t.cw, t.coef);
    if ((st = cu(cudaGetLastError(), "tile tables")) != HCC_OK) return done(st);
    int h_fail = 0;
    if ((st = cu(cudaMemcpyAsync(&h_fail, fail, sizeof(int), cudaMemcpyDeviceToHost, s), "flag")) != HCC_OK ||
        (st = cu(cudaStreamSynchronize(s), "tile tables")) != HCC_OK)
        return done(st);
    if (h_fail) {                                             // periodic axis too short: not eligible
        t.release();
        return done(HCC_OK);
    }
    t.ok = 1;
    return done(HCC_OK);
}

}  // namespace hcc
