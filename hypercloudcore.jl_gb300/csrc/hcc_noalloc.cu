// hcc_noalloc.cu — hcc_cfl_time_step_noalloc: the CFL time step of caller-owned device arrays, computed without
// allocating any device memory.
//
// Some callers cannot allocate GPU memory at the moment they need a time step: a host code whose device memory
// is reserved up front and then frozen (the reference's reserve!/CapacityError budget, src/MemoryBudget.jl:110,
// src/Growable.jl:39-47, has the same contract), or an application that hands all of its device memory to its
// own pool allocator and forbids cudaMalloc/cudaFree in its time loop. For them this entry point takes the
// neighbour lists, divergence weights and states as device pointers they own and keeps its only scratch — one
// partial minimum per thread block — in a file-scope __device__ array of fixed size.
//
// Scratch rules:
//  * g_cfl_scratch holds 65536 partial minima plus one result word (about 512 KiB of device memory per GPU on
//    which this file's module is loaded; the module stays loaded until the process exits).
//  * n above HCC_NOALLOC_MAX_PARTICLES (= max blocks x block size) is rejected with HCC_ERR_CAPACITY.
//  * Every call shares the array and leaves its contents behind. A call writes every word it reads before reading
//    it (each block writes its partial, then the final kernel reads exactly those partials and writes the result
//    word), so no word has to start at zero and nothing is cleared. Calls that overlap on the GPU (two streams,
//    or two host threads on one device) race on the array and must be serialised by the caller.
//  * Host code never uses g_cfl_scratch's name as an address: the device address comes from
//    cudaGetSymbolAddress, once per device, with that device current, on the first call made on that device.
//  * First call per device: with CUDA's lazy module loading (the default), that call is what loads this file's
//    module (the scratch array and the kernels), and loading can allocate device memory. A caller that freezes its
//    device memory must therefore make one call with n > 0 for each physics shape it will use on each device
//    before it freezes the memory (and before any stream capture); later calls allocate nothing.
//  * The stream must belong to the current device (checked: HCC_ERR_INVALID otherwise).
#include "hcc_stage_impl.cuh"
#include <algorithm>
#include <cstring>
#include <mutex>

namespace hcc {
namespace {

constexpr int kNoallocBlock = 256;
constexpr int kNoallocMaxBlocks = HCC_NOALLOC_MAX_PARTICLES / kNoallocBlock;

__device__ __align__(256) unsigned long long g_cfl_scratch[kNoallocMaxBlocks + 1];

struct NoallocArgs {
    PhysParams<double> ph;
    int64_t n, npad;
    const int32_t *cnt, *nidx;
    const double *dw;
    const uint8_t *bnd;
    const double *U;
    unsigned long long *scratch;
};

// Phase 1: per-particle dt_i exactly as k_cfl (ParticleGrids.jl:439-450), one minimum per block into scratch.
template <int D, int M, int PDE>
__global__ void __launch_bounds__(kNoallocBlock) k_cfl_partials(const NoallocArgs a) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double dti = INFINITY;
    if (i < a.n && !a.bnd[i]) {
        const int cnt = a.cnt[i];
        if (cnt > 0) {
            double Li[D];
            speeds<double, D, M, PDE>(a.ph, a.U + i * M, Li);
            double sum_c = 0.0;
            for (int k = 0; k < cnt; ++k) {
                const int32_t j = a.nidx[int64_t(k) * a.npad + i];
                double Lj[D];
                speeds<double, D, M, PDE>(a.ph, a.U + int64_t(j) * M, Lj);
                double dot = 0.0;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    double pr = fabs(a.dw[(int64_t(k) * D + d) * a.npad + i]) * jmax(Li[d], Lj[d]);
                    dot = (d == 0) ? pr : dot + pr;
                }
                sum_c = sum_c + dot;
            }
            if (sum_c > floatmin_of<double>()) dti = (1.0 / double(D)) / sum_c;
        }
    }
    __shared__ unsigned long long red[kNoallocBlock / 32];
    unsigned long long b = __double_as_longlong(dti);   // positive doubles order like their bits
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long ob = __shfl_down_sync(0xffffffffu, b, o);
        b = ob < b ? ob : b;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long v = (threadIdx.x < kNoallocBlock / 32) ? red[threadIdx.x] : 0x7ff0000000000000ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long ov = __shfl_down_sync(0xffffffffu, v, o);
            v = ov < v ? ov : v;
        }
        if (threadIdx.x == 0) a.scratch[blockIdx.x] = v;
    }
}

// Phase 2: one block reduces the `blocks` partial minima into the result word scratch[kNoallocMaxBlocks].
__global__ void __launch_bounds__(1024) k_cfl_final(unsigned long long *scratch, int blocks) {
    __shared__ unsigned long long red[32];
    unsigned long long v = 0x7ff0000000000000ull;   // +Inf
    for (int q = threadIdx.x; q < blocks; q += blockDim.x) {
        unsigned long long x = scratch[q];
        v = x < v ? x : v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long ov = __shfl_down_sync(0xffffffffu, v, o);
        v = ov < v ? ov : v;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long w = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0x7ff0000000000000ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long ow = __shfl_down_sync(0xffffffffu, w, o);
            w = ow < w ? ow : w;
        }
        if (threadIdx.x == 0) scratch[kNoallocMaxBlocks] = w;
    }
}

// Device address of g_cfl_scratch, looked up once per device with that device current.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned long long *g_scratch_ptr[kMaxDevices] = {};

hcc_status scratch_address(unsigned long long **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return HCC_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return HCC_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_cfl_scratch);
        if (e != cudaSuccess || !p) return HCC_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<unsigned long long *>(p);
    }
    *out = g_scratch_ptr[dev];
    return HCC_OK;
}

template <int D, int M, int PDE>
void launch_partials(const NoallocArgs &a, int blocks, cudaStream_t s) {
    k_cfl_partials<D, M, PDE><<<blocks, kNoallocBlock, 0, s>>>(a);
}

bool launch_for(int D, int M, int pde, const NoallocArgs &a, int blocks, cudaStream_t s) {
    if (pde == HCC_PDE_EULER) {
        if (D == 1 && M == 3) { launch_partials<1, 3, HCC_PDE_EULER>(a, blocks, s); return true; }
        if (D == 2 && M == 4) { launch_partials<2, 4, HCC_PDE_EULER>(a, blocks, s); return true; }
        if (D == 3 && M == 5) { launch_partials<3, 5, HCC_PDE_EULER>(a, blocks, s); return true; }
        return false;
    }
    // advection and the kinetic model have state-independent speeds: one instantiation per (D, M)
    if (D == 1 && M == 1) { launch_partials<1, 1, HCC_PDE_ADVECTION>(a, blocks, s); return true; }
    if (D == 2 && M == 1) { launch_partials<2, 1, HCC_PDE_ADVECTION>(a, blocks, s); return true; }
    if (D == 3 && M == 1) { launch_partials<3, 1, HCC_PDE_ADVECTION>(a, blocks, s); return true; }
    if (D == 2 && M == 2) { launch_partials<2, 2, HCC_PDE_ADVECTION>(a, blocks, s); return true; }
    if (D == 2 && M == 16) { launch_partials<2, 16, HCC_PDE_ADVECTION>(a, blocks, s); return true; }
    if (D == 1 && M == 2) { launch_partials<1, 2, HCC_PDE_ADVECTION>(a, blocks, s); return true; }
    return false;
}

}  // namespace
}  // namespace hcc

extern "C" hcc_status hcc_cfl_time_step_noalloc(const hcc_config *cfg, int64_t n, int64_t npad,
                                                const int32_t *counts, const int32_t *nidx, const double *dweights,
                                                const uint8_t *is_boundary, const double *U, void *stream,
                                                double *dt_out) {
    using namespace hcc;
    if (!cfg || !dt_out || n < 0 || npad < n) return HCC_ERR_INVALID;
    if (n > 0 && (!counts || !nidx || !dweights || !is_boundary || !U)) return HCC_ERR_INVALID;
    if (cfg->dim < 1 || cfg->dim > 3 || cfg->n_vars < 1 || cfg->n_vars > HCC_MAX_VARS) return HCC_ERR_INVALID;
    if (n > int64_t(HCC_NOALLOC_MAX_PARTICLES)) return HCC_ERR_CAPACITY;   // n beyond the fixed scratch
    if (n == 0) { *dt_out = INFINITY; return HCC_OK; }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // an error left pending by an earlier, unrelated runtime call is consumed here, so that the launch check below
    // reports this call's own launches only
    (void)cudaGetLastError();
    if (s) {
        int cur = 0, sdev = 0;
        if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(s, &sdev) != cudaSuccess) return HCC_ERR_CUDA;
        if (sdev != cur) return HCC_ERR_INVALID;          // the scratch address below is the current device's
    }
    unsigned long long *scratch = nullptr;
    hcc_status st = scratch_address(&scratch);
    if (st != HCC_OK) return st;
    NoallocArgs a{};
    // physics parameters (the spectral radius per axis for advection and the kinetic model, gamma for Euler)
    for (int d = 0; d < cfg->dim; ++d) {
        double am = 0.0;
        for (int m = 0; m < cfg->n_vars; ++m) am = std::max(am, std::fabs(cfg->velocity[d][m]));
        a.ph.amax[d] = am;
    }
    a.ph.gamma = cfg->gamma;
    a.ph.gm1 = cfg->gamma - 1.0;
    a.n = n; a.npad = npad; a.cnt = counts; a.nidx = nidx; a.dw = dweights; a.bnd = is_boundary; a.U = U;
    a.scratch = scratch;
    const int blocks = int((n + kNoallocBlock - 1) / kNoallocBlock);
    const int pde = cfg->pde == HCC_PDE_BGK ? HCC_PDE_ADVECTION : cfg->pde;
    if (cfg->pde == HCC_PDE_EULER && cfg->n_vars != cfg->dim + 2) return HCC_ERR_INVALID;
    if (!launch_for(cfg->dim, cfg->n_vars, pde, a, blocks, s)) return HCC_ERR_UNSUPPORTED;
    k_cfl_final<<<1, 1024, 0, s>>>(scratch, blocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return HCC_ERR_CUDA;
    unsigned long long bits = 0;
    e = cudaMemcpyAsync(&bits, scratch + kNoallocMaxBlocks, sizeof(bits), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return HCC_ERR_CUDA;
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    *dt_out = v;
    return HCC_OK;
}
