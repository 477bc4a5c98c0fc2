// hcc_stage_impl.cuh — the per-stage kernels, templated on the arithmetic type T (double: plain FP64 path,
// float: FP32 bulk path), the dimension D, the number of state components M, the physics module PDE and the
// reconstruction degree RDEG. Included once per precision by hcc_stage_f64.cu / hcc_stage_f32.cu.
//
// Thread per particle over slot-major neighbour arrays: the 32 threads of a warp read slot k of 32 consecutive
// particles from consecutive addresses; neighbour states, gradients and orders are gathered through L1/L2
// (the Morton numbering keeps a warp's stencils overlapping).
#pragma once
#include <algorithm>

#include "hcc_internal.cuh"

// Launch shape of the flux pass (threads per block, minimum resident blocks per SM for the register budget): the
// HCC_FLUX_* constants of hcc_internal.cuh.

namespace hcc {

// ----------------------------------------------------------------------------------- physics (device)
template <typename T> struct Accum;    // FP32: Kahan-compensated sums; FP64: plain sums
template <> struct Accum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s = s + x; }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct Accum<float> {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s; }
};

// FP32 component vectors in pairs: the packed FP32x2 instructions of sm_100+ (per component identical to the scalar
// operations; a - b as fma(b, -1, a) is the same rounding of the same exact value). HCC_FP32_PACKED=0 builds the
// same arithmetic from scalar instructions (identical results; which form runs faster is measured).
#if HCC_FP32_PACKED
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
#else
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) {
    return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
#endif
__device__ __forceinline__ float2 p_bc(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 p_ld(const float *x, int q) { return make_float2(x[2 * q], x[2 * q + 1]); }
__device__ __forceinline__ void p_st(float *x, int q, float2 v) { x[2 * q] = v.x; x[2 * q + 1] = v.y; }

// Per-component sums of the flux pass: FP64 plain; FP32 Kahan-compensated, in pairs (scalar tail for odd M).
template <typename T, int M> struct AccumV {
    T s[M];
    __device__ __forceinline__ AccumV() {
#pragma unroll
        for (int m = 0; m < M; ++m) s[m] = T(0);
    }
    __device__ __forceinline__ void add(const T *t) {
#pragma unroll
        for (int m = 0; m < M; ++m) s[m] = s[m] + t[m];
    }
};
template <int M> struct AccumV<float, M> {
    float s[M], c[M];
    __device__ __forceinline__ AccumV() {
#pragma unroll
        for (int m = 0; m < M; ++m) { s[m] = 0.0f; c[m] = 0.0f; }
    }
    __device__ __forceinline__ void add(const float *t) {
#pragma unroll
        for (int q = 0; q < M / 2; ++q) {
            const float2 y = p_sub(p_ld(t, q), p_ld(c, q));
            const float2 u = p_add(p_ld(s, q), y);
            p_st(c, q, p_sub(p_sub(u, p_ld(s, q)), y));
            p_st(s, q, u);
        }
        if constexpr (M & 1) {
            const float y = t[M - 1] - c[M - 1];
            const float u = s[M - 1] + y;
            c[M - 1] = (u - s[M - 1]) - y;
            s[M - 1] = u;
        }
    }
};

// Compensated sums of the tile-staged flux pass in blocks: NB slot terms summed plainly, then the block's sum added
// with compensation (NB = 1: every term compensated, as AccumV). `flush` adds a partial block; `sum` then holds
// the compensated sums.
template <int M, int NB> struct BlockAccum {
    AccumV<float, M> sum;
    float p[M];
    int n;
    __device__ __forceinline__ BlockAccum() : n(0) {
#pragma unroll
        for (int m = 0; m < M; ++m) p[m] = 0.0f;
    }
    __device__ __forceinline__ void add(const float *t) {
        if constexpr (NB == 1) {
            sum.add(t);
        } else {
#pragma unroll
            for (int m = 0; m < M; ++m) p[m] = p[m] + t[m];
            if (++n == NB) flush();
        }
    }
    __device__ __forceinline__ void flush() {
        if constexpr (NB > 1) {
            if (n > 0) {
                sum.add(p);
#pragma unroll
                for (int m = 0; m < M; ++m) p[m] = 0.0f;
                n = 0;
            }
        }
    }
};

template <typename T> __device__ __forceinline__ T floatmin_of();
template <> __device__ __forceinline__ double floatmin_of<double>() { return 2.2250738585072014e-308; }
template <> __device__ __forceinline__ float floatmin_of<float>() { return 1.17549435e-38f; }

// Arithmetic kernels of the two paths. FP64 (plain path): IEEE division and square root — the oracle's exact
// sequence. FP32 (bulk path, compiled with denormals flushed to zero): the fast reciprocal and reciprocal square
// root of the special-function unit (≤ 2 ulp; sqrt(x) = x rsqrt(x), 0 at 0, NaN below); its results are compared
// with the FP64 oracle to tolerance. Both keep Julia's NaN-propagating min/max:
// a reconstruction with negative pressure has a NaN sound speed, and the NaN must reach the candidate so that the
// admissibility check flags it (fmaxf would drop it and keep the high order).
template <typename T> __device__ __forceinline__ T recip(T x) { return T(1) / x; }
template <> __device__ __forceinline__ float recip<float>(float x) { return __fdividef(1.0f, x); }
template <typename T> __device__ __forceinline__ T root(T x) { return sqrt(x); }
template <> __device__ __forceinline__ float root<float>(float x) { return x == 0.0f ? 0.0f : x * rsqrtf(x); }
template <typename T> __device__ __forceinline__ T vmin(T x, T y) { return jmin(x, y); }
template <typename T> __device__ __forceinline__ T vmax(T x, T y) { return jmax(x, y); }
// FP32: the NaN-propagating forms of the min/max instructions (one instruction each)
template <> __device__ __forceinline__ float vmin<float>(float x, float y) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
    return r;
}
template <> __device__ __forceinline__ float vmax<float>(float x, float y) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
    return r;
}

// Load N contiguous elements with 16-byte vectors where the layout guarantees the alignment (particle-major
// arrays of 4 floats / 2 doubles per vector from a 256-byte-aligned base).
template <typename T, int N>
__device__ __forceinline__ void load_vec(const T *__restrict__ p, T *out) {
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
        for (int q = 0; q < N / 4; ++q) {
            float4 v = reinterpret_cast<const float4 *>(p)[q];
            out[4 * q] = v.x; out[4 * q + 1] = v.y; out[4 * q + 2] = v.z; out[4 * q + 3] = v.w;
        }
    } else if constexpr (sizeof(T) == 8 && N % 2 == 0) {
#pragma unroll
        for (int q = 0; q < N / 2; ++q) {
            double2 v = reinterpret_cast<const double2 *>(p)[q];
            out[2 * q] = v.x; out[2 * q + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int q = 0; q < N; ++q) out[q] = p[q];
    }
}

// Store N contiguous elements with 16-byte vectors under the same alignment guarantee.
template <typename T, int N>
__device__ __forceinline__ void store_vec(T *__restrict__ p, const T *v) {
    if constexpr (sizeof(T) == 4 && N % 4 == 0) {
#pragma unroll
        for (int q = 0; q < N / 4; ++q)
            reinterpret_cast<float4 *>(p)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else if constexpr (sizeof(T) == 8 && N % 2 == 0) {
#pragma unroll
        for (int q = 0; q < N / 2; ++q) reinterpret_cast<double2 *>(p)[q] = make_double2(v[2 * q], v[2 * q + 1]);
    } else {
#pragma unroll
        for (int q = 0; q < N; ++q) p[q] = v[q];
    }
}

// Euler primitives: inv_rho = 1/rho, u_d = m_d inv_rho, p = (gamma-1)(E - 0.5 (rho |u|^2)), c = sqrt(gamma p inv_rho).
template <typename T, int D>
__device__ __forceinline__ void euler_prim(const PhysParams<T> &ph, const T *U, T &inv_rho, T *u, T &p) {
    T rho = U[0];
    inv_rho = recip(rho);
    T q2 = T(0);
#pragma unroll
    for (int d = 0; d < D; ++d) {
        u[d] = U[1 + d] * inv_rho;
        q2 = (d == 0) ? u[d] * u[d] : q2 + u[d] * u[d];
    }
    p = ph.gm1 * (U[D + 1] - T(0.5) * (rho * q2));
}

// flux(eq, U) (API.jl:23) for the compiled-in modules; lam[d] = max_eigenvalue(eq, U, d) (API.jl:38).
// On a moving grid (w != nullptr) the flux and speeds of ALEFrame(eq, w) (GridMovers.jl:77-83): F_d - w_d U and
// max_eigenvalue(eq, U, d, w_d) (API.jl:51-58): |u_d - w_d| + c (Euler), |c_d - w_d| (scalar advection,
// test/PDEs/linear_advection.jl:35), else max_eigenvalue + |w_d|.
template <typename T, int D, int M, int PDE>
__device__ __forceinline__ void flux_and_speed(const PhysParams<T> &ph, const T *U, T (*F)[M], T *lam,
                                               const T *w = nullptr) {
    if constexpr (PDE == HCC_PDE_EULER) {
        T inv_rho, u[D], p;
        euler_prim<T, D>(ph, U, inv_rho, u, p);
        T c = root(ph.gamma * p * inv_rho);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            F[d][0] = U[1 + d];
#pragma unroll
            for (int e = 0; e < D; ++e) {
                T v = U[1 + e] * u[d];
                F[d][1 + e] = (e == d) ? v + p : v;
            }
            F[d][D + 1] = (U[D + 1] + p) * u[d];
            lam[d] = fabs(w ? u[d] - w[d] : u[d]) + c;
        }
    } else {
#pragma unroll
        for (int d = 0; d < D; ++d) {
#pragma unroll
            for (int m = 0; m < M; ++m) F[d][m] = ph.c[d][m] * U[m];
            lam[d] = !w ? ph.amax[d]
                        : ((PDE == HCC_PDE_ADVECTION && M == 1) ? fabs(ph.c[d][0] - w[d]) : ph.amax[d] + fabs(w[d]));
        }
    }
    if (w) {
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
            for (int m = 0; m < M; ++m) F[d][m] = F[d][m] - w[d] * U[m];
    }
}

// FP32 Euler on a fixed grid, the flux contracted with a weight vector w: Fw(U) = sum_d w_d F_d(U) =
// (m.w, (u.w) m + p w, (E + p)(u.w)), and the axis speeds |u_d| + c of flux_and_speed. One contracted flux
// replaces the D axis fluxes and their contraction in the flux pass (the Rusanov flux is linear in the F_d).
template <int D>
__device__ __forceinline__ void euler_projected(const PhysParams<float> &ph, const float *U, const float *w,
                                                float *Fn, float *lam) {
    float inv_rho, u[D], p;
    euler_prim<float, D>(ph, U, inv_rho, u, p);
    const float c = root(ph.gamma * p * inv_rho);
    float un = u[0] * w[0], mw = U[1] * w[0];
#pragma unroll
    for (int d = 1; d < D; ++d) { un = un + u[d] * w[d]; mw = mw + U[1 + d] * w[d]; }
    Fn[0] = mw;
#pragma unroll
    for (int e = 0; e < D; ++e) Fn[1 + e] = un * U[1 + e] + p * w[e];
    Fn[D + 1] = (U[D + 1] + p) * un;
#pragma unroll
    for (int d = 0; d < D; ++d) lam[d] = fabsf(u[d]) + c;
}

// Whether the flux pass takes the contracted Euler form (FP32, fixed grid, no moment correction).
template <typename T, int PDE, bool ALE, bool MOM> constexpr bool projected_flux() {
    return sizeof(T) == 4 && PDE == HCC_PDE_EULER && !ALE && !MOM;
}

// The own flux a flux pass keeps for particle i: F(f_i) per axis (FP64), doubled (FP32, the scaled Rusanov form),
// or for the contracted Euler form the constants 2 Fw(f_i) is formed from in every slot, in the first row:
// (2u, 2p, E + p).
template <typename T, int D, int M, int PDE, bool ALE, bool MOM>
__device__ __forceinline__ void own_flux(const PhysParams<T> &ph, const T *fi, T (*Fi)[M], const T *wp) {
    if constexpr (projected_flux<T, PDE, ALE, MOM>()) {
        T inv_rho, u[D], p;
        euler_prim<T, D>(ph, fi, inv_rho, u, p);
#pragma unroll
        for (int d = 0; d < D; ++d) Fi[0][d] = T(2) * u[d];
        Fi[0][D] = T(2) * p;
        Fi[0][D + 1] = fi[D + 1] + p;
    } else {
        T lam[D];
        flux_and_speed<T, D, M, PDE>(ph, fi, Fi, lam, wp);
        if constexpr (sizeof(T) == 4) {
#pragma unroll
            for (int d = 0; d < D; ++d)
#pragma unroll
                for (int m = 0; m < M; ++m) Fi[d][m] = T(2) * Fi[d][m];
        }
    }
}

// grid_velocity (GridMovers.jl:60-63) of particle i: fluid velocity (Euler m_d / rho, scalar advection c_d), scaled,
// or the prescribed field velocity + omega x (x - center) at its current position
template <typename T, int D, int M, int PDE>
__device__ __forceinline__ void grid_velocity(const StageArgs<T> &a, int64_t i, const T *U, T *w) {
    if (a.mover == HCC_MOVER_PRESCRIBED) {
        double r[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = a.pos[int64_t(d) * a.g.npad + i] - a.mv_c[d];
        if constexpr (D == 1) {
            w[0] = T(a.mv_v[0]);
        } else if constexpr (D == 2) {
            w[0] = T(a.mv_v[0] - a.mv_om[2] * r[1]);
            w[1] = T(a.mv_v[1] + a.mv_om[2] * r[0]);
        } else {
            w[0] = T(a.mv_v[0] + (a.mv_om[1] * r[2] - a.mv_om[2] * r[1]));
            w[1] = T(a.mv_v[1] + (a.mv_om[2] * r[0] - a.mv_om[0] * r[2]));
            w[2] = T(a.mv_v[2] + (a.mv_om[0] * r[1] - a.mv_om[1] * r[0]));
        }
        return;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if constexpr (PDE == HCC_PDE_EULER) w[d] = U[1 + d] / U[0];
        else w[d] = a.ph.c[d][0];
        if (a.mover == HCC_MOVER_SCALED) w[d] = a.mv_alpha * w[d];
    }
}

template <typename T, int D, int M, int PDE>
__device__ __forceinline__ void speeds(const PhysParams<T> &ph, const T *U, T *lam) {
    if constexpr (PDE == HCC_PDE_EULER) {
        T inv_rho, u[D], p;
        euler_prim<T, D>(ph, U, inv_rho, u, p);
        T c = root(ph.gamma * p * inv_rho);
#pragma unroll
        for (int d = 0; d < D; ++d) lam[d] = fabs(u[d]) + c;
    } else {
#pragma unroll
        for (int d = 0; d < D; ++d) lam[d] = ph.amax[d];
    }
}

// is_admissible (API.jl:48): finite; Euler also rho > 0 and p > 0.
template <typename T, int D, int M, int PDE>
__device__ __forceinline__ bool admissible(const PhysParams<T> &ph, const T *U) {
    bool ok = true;
#pragma unroll
    for (int m = 0; m < M; ++m) ok = ok && isfinite(U[m]);
    if constexpr (PDE == HCC_PDE_EULER) {
        if (!ok) return false;
        T inv_rho, u[D], p;
        euler_prim<T, D>(ph, U, inv_rho, u, p);
        return U[0] > T(0) && p > T(0);
    }
    return ok;
}

// BGK Maxwellian of the single macro moment (evaluate_source / implicit_solve, test/kinetic_source.jl:67-104).
template <typename T, int D, int M>
__device__ __forceinline__ void maxwellian(const PhysParams<T> &ph, const T *U, T *Mk) {
    T u = U[0];
#pragma unroll
    for (int k = 1; k < M; ++k) u = u + U[k];
    T F[D];
#pragma unroll
    for (int d = 0; d < D; ++d) F[d] = ph.a_macro[d] * u;
#pragma unroll
    for (int k = 0; k < M; ++k) {
        T fd = F[0] * ph.sinv[k][0];
#pragma unroll
        for (int d = 1; d < D; ++d) fd = fd + F[d] * ph.sinv[k][d];
        Mk[k] = ph.coeff * (u + fd);
    }
}

// Implicit part of a stage (TimeSteppers.jl:427-444): mode 1 solves U_out - dt a_ii S(U_out) = U_in and sets
// K_I = (U_out - U_in) / (dt a_ii); mode 2 evaluates K_I = S(Y) explicitly.
template <typename T, int D, int M, int PDE>
__device__ __forceinline__ void implicit_part(const StageArgs<T> &a, int64_t i, T *Y, T *KIout) {
    if constexpr (PDE == HCC_PDE_BGK) {
        T Mk[M];
        maxwellian<T, D, M>(a.ph, Y, Mk);
        if (a.implicit_mode == 1) {
            const StageCoeffs<T> *cf = coef_of(a, i);
            T dto = cf->dt_ii * a.ph.inv_eps;
            T denom = T(1) / (T(1) + dto);
            const T inv_dt_ii = cf->inv_dt_ii;
#pragma unroll
            for (int k = 0; k < M; ++k) {
                T out = (Y[k] + dto * Mk[k]) * denom;
                KIout[k] = (out - Y[k]) * inv_dt_ii;
                Y[k] = out;
            }
        } else {
#pragma unroll
            for (int k = 0; k < M; ++k) KIout[k] = (Mk[k] - Y[k]) * a.ph.inv_eps;
        }
    } else {
#pragma unroll
        for (int k = 0; k < M; ++k) KIout[k] = T(0);
    }
}

// ----------------------------------------------------------------------------------- slope limiters
// limiter_phi (Limiter.jl:35-46): Barth-Jespersen min(1, r); Venkatakrishnan (r² + 2r)/(r² + r + 2), for r > 1 in
// s = 1/r.
template <typename T>
__device__ __forceinline__ T limiter_phi(int lim, T r) {
    if (lim == HCC_LIMITER_BJ_SOFT || lim == HCC_LIMITER_BJ_HARD) return vmin(T(1), r);
    const T rp = vmax(T(0), r);
    const T sv = T(1) / vmax(T(1), rp);
    const T small = (rp * rp + T(2) * rp) / (rp * rp + rp + T(2));
    const T large = (T(1) + T(2) * sv) / (T(1) + sv + T(2) * (sv * sv));
    return rp > T(1) ? large : small;
}

template <typename T> __device__ __forceinline__ T eps16();
template <> __device__ __forceinline__ double eps16<double>() { return 16.0 * 2.220446049250313e-16; }
template <> __device__ __forceinline__ float eps16<float>() { return 16.0f * 1.1920929e-7f; }

// _limit_slopes for BJ / VK (Limiter.jl:120-143): local extrema over {i} ∪ N(i) (_local_extrema, :61-69), the
// bounding coefficient over the interface reconstructions (_bounding_phi / _update_phi, :76-100), then the
// gradient terms (hard: every term; soft: the first-degree ones) scaled by it.
template <typename T, int D, int M, int RDEG>
__device__ __forceinline__ void limit_slopes(const StageArgs<T> &a, int64_t i, int cnt, const T *fi,
                                             T (*out)[M]) {
    constexpr int BR = RBasis<D, RDEG>::B;
    const int64_t np = a.g.npad;
    T umax[M], umin[M], phi[M];
#pragma unroll
    for (int m = 0; m < M; ++m) { umax[m] = fi[m]; umin[m] = fi[m]; phi[m] = T(1); }
    for (int k = 0; k < cnt; ++k) {
        const int32_t j = a.g.nidx[int64_t(k) * np + i];
        T fj[M];
        load_vec<T, M>(a.U + int64_t(j) * M, fj);
#pragma unroll
        for (int m = 0; m < M; ++m) { umax[m] = vmax(umax[m], fj[m]); umin[m] = vmin(umin[m], fj[m]); }
    }
    const T tol16 = eps16<T>();
    for (int k = 0; k < cnt; ++k) {
        T hx[D], p[BR];
#pragma unroll
        for (int d = 0; d < D; ++d) hx[d] = T(0.5) * a.g.dist[(int64_t(k) * D + d) * np + i];
        recon_basis<D, RDEG, T>(hx, p);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            T recon = out[0][m] * p[0];
#pragma unroll
            for (int b = 1; b < BR; ++b) recon = recon + out[b][m] * p[b];
            const T bound = recon > T(0) ? umax[m] : umin[m];
            const T tol = tol16 * vmax(fabs(fi[m]), fabs(bound));
            if (fabs(recon) > tol) phi[m] = vmin(phi[m], limiter_phi<T>(a.sc.limiter, (bound - fi[m]) / recon));
        }
    }
    const bool hard = a.sc.limiter == HCC_LIMITER_BJ_HARD || a.sc.limiter == HCC_LIMITER_VK_HARD;
#pragma unroll
    for (int b = 0; b < BR; ++b)
        if (hard || b < D) {
#pragma unroll
            for (int m = 0; m < M; ++m) out[b][m] = out[b][m] * phi[m];
        }
}

// ----------------------------------------------------------------------------------- gather pass
// update_content! of MUSCL (MUSCL.jl:351-384) with NoLimiter: starved-order lowering, cached full-order fit
// (apply_weights, Interpolators.jl:585-602), dynamic lower-degree fit, or zero (order 1).
template <typename T, int D, int M, int PDE, int RDEG>
__device__ __forceinline__ void gather_one(const StageArgs<T> &a, const int64_t i) {
    constexpr int BR = RBasis<D, RDEG>::B;
    if (a.g.bnd[i]) return;
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    int p = a.orders[i];
    const int p0 = p;
    while (p > 1 && cnt < basis_count(D, p - 1)) --p;
    if (p < p0) a.orders[i] = int8_t(p);
    T *g = a.grad + i * (BR * M);
    T fi[M];
#pragma unroll
    for (int m = 0; m < M; ++m) fi[m] = a.U[i * M + m];
    T out[BR][M];
#pragma unroll
    for (int b = 0; b < BR; ++b)
#pragma unroll
        for (int m = 0; m < M; ++m) out[b][m] = T(0);
    const T invL = a.g.invL;
    bool done = false;
    if constexpr (sizeof(T) == 4 && RDEG == 1) {
        // FP32, degree 1: the cached fit as one weight vector per slot (nidx + D floats per slot)
        if (p == a.sc.max_order && p > 1 && a.g.ok_r[i] && a.g.gw) {
            // slots in groups of G: the group's indices, weights and neighbour states are all in flight together
            constexpr int G = 4;
            int k = 0;
            for (; k + G <= cnt; k += G) {
                int32_t j[G];
                T gk[G][D], df[G][M];
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    j[q] = a.g.nidx[int64_t(k + q) * np + i];
#pragma unroll
                    for (int d = 0; d < D; ++d) gk[q][d] = a.g.gw[(int64_t(k + q) * D + d) * np + i];
                }
#pragma unroll
                for (int q = 0; q < G; ++q) load_vec<T, M>(a.U + int64_t(j[q]) * M, df[q]);
#pragma unroll
                for (int q = 0; q < G; ++q)
#pragma unroll
                    for (int m = 0; m < M; ++m) {
                        const T dm = df[q][m] - fi[m];
#pragma unroll
                        for (int b = 0; b < BR; ++b) out[b][m] = out[b][m] + gk[q][b] * dm;
                    }
            }
            for (; k < cnt; ++k) {
                const int32_t j = a.g.nidx[int64_t(k) * np + i];
                T gk[D], df[M];
#pragma unroll
                for (int d = 0; d < D; ++d) gk[d] = a.g.gw[(int64_t(k) * D + d) * np + i];
                load_vec<T, M>(a.U + int64_t(j) * M, df);
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const T dm = df[m] - fi[m];
#pragma unroll
                    for (int b = 0; b < BR; ++b) out[b][m] = out[b][m] + gk[b] * dm;
                }
            }
            done = true;
        }
    }
    if (done) {
    } else if (p == a.sc.max_order && p > 1 && a.g.ok_r[i]) {
        T bs[BR][M];
#pragma unroll
        for (int b = 0; b < BR; ++b)
#pragma unroll
            for (int m = 0; m < M; ++m) bs[b][m] = T(0);
        int32_t jn = cnt > 0 ? a.g.nidx[i] : 0;
        T dn[D], wn = cnt > 0 ? a.g.wt[i] : T(0);
#pragma unroll
        for (int d = 0; d < D; ++d) dn[d] = cnt > 0 ? a.g.dist[int64_t(d) * np + i] : T(0);
        for (int k = 0; k < cnt; ++k) {
            const int32_t j = jn;
            T x[D], pb[BR];
#pragma unroll
            for (int d = 0; d < D; ++d) x[d] = dn[d] * invL;
            const T w = wn;
            if (k + 1 < cnt) {
                const int64_t s1 = int64_t(k + 1) * np + i;
                jn = a.g.nidx[s1];
                wn = a.g.wt[s1];
#pragma unroll
                for (int d = 0; d < D; ++d) dn[d] = a.g.dist[(int64_t(k + 1) * D + d) * np + i];
            }
            recon_basis<D, RDEG, T>(x, pb);
            T df[M];
            load_vec<T, M>(a.U + int64_t(j) * M, df);
#pragma unroll
            for (int m = 0; m < M; ++m) df[m] = df[m] - fi[m];
#pragma unroll
            for (int b = 0; b < BR; ++b)
#pragma unroll
                for (int m = 0; m < M; ++m) bs[b][m] = bs[b][m] + w * (pb[b] * df[m]);
        }
        const T *inv = a.g.inv_r + i * (BR * BR);
        T invm[BR][BR];
#pragma unroll
        for (int b = 0; b < BR; ++b)
#pragma unroll
            for (int c = 0; c < BR; ++c) invm[b][c] = inv[b * BR + c];
#pragma unroll
        for (int b = 0; b < BR; ++b) {
            const T sc = recon_scale<D, RDEG, T>(b, invL);
#pragma unroll
            for (int m = 0; m < M; ++m) {
                T acc = invm[b][0] * bs[0][m];
#pragma unroll
                for (int c = 1; c < BR; ++c) acc = acc + invm[b][c] * bs[c][m];
                out[b][m] = acc * sc;
            }
        }
    } else if (p > 1 && p - 1 < RDEG) {
        // Interpolator{D, 1, 1} (_mls_solve, Interpolators.jl:372-400): moment matrix and Cholesky in FP64
        constexpr int B1 = D;
        double N[B1 * B1];
        T bs[B1][M];
#pragma unroll
        for (int q = 0; q < B1 * B1; ++q) N[q] = 0.0;
#pragma unroll
        for (int b = 0; b < B1; ++b)
#pragma unroll
            for (int m = 0; m < M; ++m) bs[b][m] = T(0);
        const double invLd = double(invL);
        for (int k = 0; k < cnt; ++k) {
            const int64_t s = int64_t(k) * np + i;
            const int32_t j = a.g.nidx[s];
            double xd[D];
            T xt[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                T dk = a.g.dist[(int64_t(k) * D + d) * np + i];
                xd[d] = double(dk) * invLd;
                xt[d] = dk * invL;
            }
            const T w = a.g.wt[s];
            const double wd = double(w);
#pragma unroll
            for (int r = 0; r < B1; ++r)
#pragma unroll
                for (int c = 0; c < B1; ++c) N[r * B1 + c] = N[r * B1 + c] + wd * (xd[r] * xd[c]);
#pragma unroll
            for (int b = 0; b < B1; ++b)
#pragma unroll
                for (int m = 0; m < M; ++m) bs[b][m] = bs[b][m] + w * (xt[b] * (a.U[int64_t(j) * M + m] - fi[m]));
        }
        // _cholesky_moment
        double U[B1 * B1];
        bool ok = true;
        for (int attempt = 0; attempt < 2; ++attempt) {
            ok = true;
            for (int r = 0; r < B1 * B1; ++r) U[r] = 0.0;
            for (int r = 0; r < B1 && ok; ++r)
                for (int c = r; c < B1; ++c) {
                    double sm = N[r * B1 + c];
                    for (int q = 0; q < r; ++q) sm = sm - U[q * B1 + r] * U[q * B1 + c];
                    if (r == c) {
                        if (!(sm > 0.0)) { ok = false; break; }
                        U[r * B1 + r] = sqrt(sm);
                    } else U[r * B1 + c] = sm / U[r * B1 + r];
                }
            if (attempt == 0 && ok) {
                for (int q = 0; q < B1; ++q) {
                    double u = U[q * B1 + q];
                    if (!(u * u > 10.0 * 2.220446049250313e-16 * N[q * B1 + q])) { ok = false; break; }
                }
                if (ok) break;
            }
            if (attempt == 0) {
                double tr = 0.0;
                for (int q = 0; q < B1; ++q) tr = tr + N[q * B1 + q];
                double er = 1.4901161193847656e-08 * tr / double(B1);
                for (int q = 0; q < B1; ++q) N[q * B1 + q] = N[q * B1 + q] + er;
            }
        }
        if (ok) {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                double y[B1], x[B1];
                for (int r = 0; r < B1; ++r) {
                    double t = double(bs[r][m]);
                    for (int q = 0; q < r; ++q) t = t - U[q * B1 + r] * y[q];
                    y[r] = t / U[r * B1 + r];
                }
                for (int r = B1 - 1; r >= 0; --r) {
                    double t = y[r];
                    for (int q = r + 1; q < B1; ++q) t = t - U[r * B1 + q] * x[q];
                    x[r] = t / U[r * B1 + r];
                }
#pragma unroll
                for (int b = 0; b < B1; ++b) out[b][m] = T(x[b] * invLd);
            }
        }
    }
    if (a.sc.limiter != HCC_LIMITER_NONE && p > 1) limit_slopes<T, D, M, RDEG>(a, i, cnt, fi, out);
    store_vec<T, BR * M>(g, &out[0][0]);
}

// FP32 degree-1 worklist pass of the reconstruction with four warps per tile: warp 0 lowers starved orders and picks
// the path; on the cached gradient-weight path warp w sums the slots k = w, w + 4, ... and marks their neighbours'
// reach, warp 0 adds the four partial sums in a fixed order, applies the limiter and stores the gradients; any
// other particle is reconstructed whole by warp 0.
template <typename T, int D, int M, int PDE, int RDEG>
__global__ void __launch_bounds__(128) k_gather_tiles(const StageArgs<T> a) {
    constexpr int BR = RBasis<D, RDEG>::B;
    __shared__ T parts[4][32][BR * M];
    __shared__ int path[32];
    const int lane = int(threadIdx.x & 31), w = int(threadIdx.x >> 5);
    const unsigned nt = *a.wcount;
    const int64_t np = a.g.npad;
    for (unsigned q = blockIdx.x; q < nt; q += gridDim.x) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool live = ((word >> lane) & 1u) && !a.g.bnd[i];
        const int cnt = live ? a.g.cnt[i] : 0;
        if (w == 0) {
            int gp = 0;
            if (live) {
                int p = a.orders[i];
                const int p0 = p;
                while (p > 1 && cnt < basis_count(D, p - 1)) --p;
                if (p < p0) a.orders[i] = int8_t(p);
                gp = (p == a.sc.max_order && p > 1 && a.g.ok_r[i] && a.g.gw) ? 1 : 0;
            }
            path[lane] = gp;
        }
        __syncthreads();
        const int gp = path[lane];
        {
            // warp-uniform slot loop over every live member (the reach marks, combined across the warp); the
            // cached-fit members also accumulate their gradients here
            const int myc = (live && gp) ? cnt : 0;
            const int myr = (live && a.rmask) ? cnt : myc;
            const int kw = __reduce_max_sync(0xffffffffu, myr);
            T fi[M], out[BR * M];
            if (myc > 0) load_vec<T, M>(a.U + i * M, fi);
#pragma unroll
            for (int b = 0; b < BR * M; ++b) out[b] = T(0);
            for (int k = w; k < kw; k += 4) {
                const int32_t j = k < myr ? a.g.nidx[int64_t(k) * np + i] : -1;
                if (k < myc) {
                    T gk[D], df[M];
#pragma unroll
                    for (int d = 0; d < D; ++d) gk[d] = a.g.gw[(int64_t(k) * D + d) * np + i];
                    load_vec<T, M>(a.U + int64_t(j) * M, df);
#pragma unroll
                    for (int m = 0; m < M; ++m) {
                        const T dm = df[m] - fi[m];
#pragma unroll
                        for (int b = 0; b < BR; ++b) out[b * M + m] = out[b * M + m] + gk[b] * dm;
                    }
                }
                if (a.rmask) reach_mark_warp(a.rmask, a.rtiles, a.rcount, j);
            }
            if (myc > 0 || (live && gp))
#pragma unroll
                for (int b = 0; b < BR * M; ++b) parts[w][lane][b] = out[b];
        }
        __syncthreads();
        if (w == 0 && a.rmask) reach_mark_warp(a.rmask, a.rtiles, a.rcount, live ? int32_t(i) : -1);
        if (w == 0 && live) {
            if (gp) {
                T fi[M], out[BR][M];
                load_vec<T, M>(a.U + i * M, fi);
#pragma unroll
                for (int b = 0; b < BR; ++b)
#pragma unroll
                    for (int m = 0; m < M; ++m)
                        out[b][m] = ((parts[0][lane][b * M + m] + parts[1][lane][b * M + m]) + parts[2][lane][b * M + m]) +
                                    parts[3][lane][b * M + m];
                if (a.sc.limiter != HCC_LIMITER_NONE) limit_slopes<T, D, M, RDEG>(a, i, cnt, fi, out);
                store_vec<T, BR * M>(a.grad + i * (BR * M), &out[0][0]);
            } else {
                gather_one<T, D, M, PDE, RDEG>(a, i);
            }
        }
        if (threadIdx.x == 0 && a.clear_wmask) a.wmask[tile] = 0u;   // every lane read the word before the barrier
        __syncthreads();
    }
}

// A full pass (one thread per particle) or a worklist pass over tiles (one warp per tile, the members of its word)
// that also marks the one-hop reach of each member in rmask / rtiles.
template <typename T, int D, int M, int PDE, int RDEG>
__global__ void __launch_bounds__(128) k_gather(const StageArgs<T> a) {
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if (i < a.g.n) gather_one<T, D, M, PDE, RDEG>(a, i);
        return;
    }
    const unsigned nt = *a.wcount;
    const int64_t np = a.g.npad;
    const int lane = int(threadIdx.x & 31);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        __syncwarp();
        if (a.clear_wmask && lane == 0) a.wmask[tile] = 0u;     // the changed list is consumed here
        const bool mem = (word >> lane) & 1u;
        const int32_t i = tile * 32 + lane;
        if (mem) gather_one<T, D, M, PDE, RDEG>(a, i);
        if (a.rmask) {
            // the reach (members and their neighbours), slot by slot across the warp with combined atomics
            reach_mark_warp(a.rmask, a.rtiles, a.rcount, mem ? i : -1);
            const int c = mem ? a.g.cnt[i] : 0;
            const int kw = __reduce_max_sync(0xffffffffu, c);
            for (int k = 0; k < kw; ++k)
                reach_mark_warp(a.rmask, a.rtiles, a.rcount, k < c ? a.g.nidx[int64_t(k) * np + i] : -1);
        }
    }
}

// Epilogue of a flux pass for particle i: K_E[s] stored, the next candidate formed (_stage_predictor!,
// TimeSteppers.jl:400-421, and the implicit part), the Euler substep (:511-518) and the MOOD check of the next
// checkpoint (_mood_flag!, MOOD.jl:289-295) against the extrema mn/mx of {i} ∪ N(i) of the stage state.
// MOODu2 override (_u2_fails, MOOD.jl:241-271), for the DMP-violating components of a particle of order >= 3: per
// axis the curvature terms (reconstruction terms D + d) over {i} ∪ N(i) keep one sign, and over the neighbours within
// 1.5h comparable magnitudes, or are negligible; otherwise the candidate is flagged. A rare path (DMP violators only).
template <typename T, int D, int M, int RDEG>
__device__ __noinline__ bool u2_curvature_fails(const StageArgs<T> &a, int64_t i, const bool *viol) {
    constexpr int BR = RBasis<D, RDEG>::B;
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    const T h = a.u2_h, h2 = h * h, r15 = T(1.5) * h, near_sq = r15 * r15, dl = a.delta;
    for (int d = 0; d < D; ++d) {
        const int b = D + d;
        T mini[M], maxi[M], minA[M], maxA[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const T ci = a.grad[(i * BR + b) * M + m];
            mini[m] = maxi[m] = ci;
            minA[m] = maxA[m] = fabs(ci);
        }
        for (int k = 0; k < cnt; ++k) {
            const int64_t j = a.g.nidx[int64_t(k) * np + i];
            T r2 = T(0);
#pragma unroll
            for (int e = 0; e < D; ++e) {
                const T x = a.g.dist[(int64_t(k) * D + e) * np + i];
                r2 = (e == 0) ? x * x : r2 + x * x;
            }
            const bool near = r2 <= near_sq;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const T cj = a.grad[(j * BR + b) * M + m];
                mini[m] = vmin(mini[m], cj);
                maxi[m] = vmax(maxi[m], cj);
                if (near) { minA[m] = vmin(minA[m], fabs(cj)); maxA[m] = vmax(maxA[m], fabs(cj)); }
            }
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
            if (!viol[m]) continue;
            if (vmax(fabs(mini[m]), fabs(maxi[m])) * h2 < dl) continue;    // negligible curvature
            const bool same_sign = (mini[m] * h2) * (maxi[m] * h2) > -(dl * dl);
            const bool comparable = a.u2_ratio <= T(0) || minA[m] >= a.u2_ratio * maxA[m];
            if (!(same_sign && comparable)) return true;
        }
    }
    return false;
}

template <typename T, int D, int M, int PDE, int RDEG = 0>
__device__ __forceinline__ bool stage_epilogue(const StageArgs<T> &a, int64_t i, const T *fi, const T *Kv,
                                               const T *mn, const T *mx) {
    store_vec<T, M>(a.K + i * M, Kv);
    if (!a.form_next) return false;
    // _stage_predictor! for the next candidate
    T Y[M];
    load_vec<T, M>(a.Un + i * M, Y);
    const StageCoeffs<T> *cf = coef_of(a, i);
    for (int j = 0; j < a.n_prev; ++j) {
        const T hE = cf->hE[j], hI = cf->hI[j];
        if (hE != T(0)) {
            const T h = hE;
            if (j == a.self_slot) {
#pragma unroll
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + h * Kv[m];
            } else {
                T kv[M];
                load_vec<T, M>(a.KE[j] + i * M, kv);
#pragma unroll
                for (int m = 0; m < M; ++m) Y[m] = Y[m] + h * kv[m];
            }
        }
        if (hI != T(0)) {
            const T h = hI;
            T kv[M];
            load_vec<T, M>(a.KI[j] + i * M, kv);
#pragma unroll
            for (int m = 0; m < M; ++m) Y[m] = Y[m] + h * kv[m];
        }
    }
    if (a.implicit_mode) {
        T KIo[M];
        implicit_part<T, D, M, PDE>(a, i, Y, KIo);
        store_vec<T, M>(a.KInext + i * M, KIo);
    }
    store_vec<T, M>(a.Ynext + i * M, Y);
    if (a.Xnext) {
        // moving grid: the next stage positions X = x_n + Σ_j dt ã_j K_X[j] (_stage_predictor!, :403-421)
        const int64_t np = a.g.npad;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            double X = a.x_n[int64_t(d) * np + i];
            for (int j = 0; j < a.n_prev; ++j) {
                const double h = cf->hEd[j];
                if (h != 0.0) {
                    const double kx = (j == a.self_slot) ? a.KXout[int64_t(d) * np + i] : a.KX[j][int64_t(d) * np + i];
                    X = X + h * kx;
                }
            }
            a.Xnext[int64_t(d) * np + i] = X;
        }
    }
    if (!a.check) return false;
    T cand[M];
    if (a.check_substep) {
        if (a.KIs) {
#pragma unroll
            for (int m = 0; m < M; ++m) cand[m] = fi[m] + cf->h_sub * (Kv[m] + a.KIs[i * M + m]);
        } else {
#pragma unroll
            for (int m = 0; m < M; ++m) cand[m] = fi[m] + cf->h_sub * Kv[m];
        }
    } else {
#pragma unroll
        for (int m = 0; m < M; ++m) cand[m] = Y[m];
    }
    const bool adm = admissible<T, D, M, PDE>(a.ph, cand);
    bool flag = !adm;
    if (a.sc.criterion == HCC_MOOD_ONLY) flag = true;
    else if (a.sc.criterion == HCC_MOOD_U1 && !flag) {
        const T dl = a.delta, d3 = dl * dl * dl;
        if constexpr (sizeof(T) == 8) {
#pragma unroll
            for (int m = 0; m < M; ++m)
                if (fabs(mx[m] - mn[m]) >= d3 && (cand[m] < mn[m] - dl || cand[m] > mx[m] + dl)) flag = true;
        } else {
            // FP32: the bounds are padded by 16 unit round-offs of their magnitude on top of delta, so the round-off
            // of the FP32 update (a few units on a flat state) is not read as a new extremum.
            constexpr T kPad = T(16) * T(1.1920928955078125e-7);
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const T pad = dl + kPad * vmax(fabs(mn[m]), fabs(mx[m]));
                if (fabs(mx[m] - mn[m]) >= d3 && (cand[m] < mn[m] - pad || cand[m] > mx[m] + pad)) flag = true;
            }
        }
    }
    else if (a.sc.criterion == HCC_MOOD_U2 && !flag) {
        // DMP violators that are not a plateau (the u1 test, plus max - min < plateau x global range)
        const T dl = a.delta, d3 = dl * dl * dl;
        bool viol[M], any = false;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            T pad = dl;
            if constexpr (sizeof(T) == 4) pad = dl + T(16) * T(1.1920928955078125e-7) * vmax(fabs(mn[m]), fabs(mx[m]));
            bool v = fabs(mx[m] - mn[m]) >= d3 && (cand[m] < mn[m] - pad || cand[m] > mx[m] + pad);
            if (v && a.u2_range) {
                const unsigned long long nanbits = a.u2_range[2 * M];
                const T range = ((nanbits >> m) & 1ull) ? T(NAN)
                                                        : T(order_value(a.u2_range[M + m])) - T(order_value(a.u2_range[m]));
                v = !(mx[m] - mn[m] < a.u2_plateau * range);
            }
            viol[m] = v;
            any = any || v;
        }
        if (any) {
            if constexpr (RDEG >= 2) {
                flag = (a.sc.max_order < 3 || a.orders[i] < 3) ? true : u2_curvature_fails<T, D, M, RDEG>(a, i, viol);
            } else {
                flag = true;
            }
        }
    }
    a.inadm[i] = !adm;
    return flag;
}

// ----------------------------------------------------------------------------------- flux pass
// Number of reconstruction terms an interface of order o keeps (mask_basis, Interpolators.jl:265-284):
// basis_count(D, o - 1) for 2 <= o <= RDEG + 1, else 0 — compile-time values, no integer division per slot.
template <int D, int RDEG>
__device__ __forceinline__ int interface_terms(int o) {
    constexpr int b1 = cbasis_count(D, 1), b2 = cbasis_count(D, 2);
    return (o == 2) ? b1 : ((o == 3 && RDEG >= 2) ? b2 : 0);
}

// Resident blocks per SM the flux kernel is compiled for: as many as its registers allow without spilling
// (FP32 2-D scalar/Euler: 72 registers; wider states and FP64 need more).
template <typename T, int D, int M> constexpr int flux_min_blocks() {
    if (sizeof(T) == 8) return M >= 8 ? 1 : (D * M >= 12 ? 2 : HCC_FLUX_MINB64);
    return M >= 8 ? HCC_FLUX_MINB_MANY : (D * M >= 12 ? HCC_FLUX_MINB_WIDE : HCC_FLUX_MINB);
}

// The MUSCL functor (MUSCL.jl:390-508) in its streamed form: per slot, EPD interface reconstruction, physical
// fluxes, Rusanov (FluxFunctions.jl:66-76) with sort_flux (Utils.jl:95-102), the flux difference ΔF and its
// contraction with the divergence weights; K_E = -2 Σ c·ΔF (TimeSteppers.jl:354). Fused epilogue: the next
// candidate (_stage_predictor!, :400-421, and the implicit part), the Euler substep (:511-518) and the MOOD
// check of the next checkpoint (_mood_flag!, MOOD.jl:289-295; the extrema come from this loop's neighbour reads).
// Partial sums of a particle's slots handled by one warp of a split tile (FP32 worklist passes).
template <typename T, int M> struct FluxPart {
    T s[M], c[M], mn[M], mx[M];
};

// One slot k of the flux pass of particle i (the MUSCL functor's slot body, MUSCL.jl:463-508): interface orders oi,
// oj and the sort orientation `below` are the caller's; the interface reconstructions, the physical fluxes, the
// Rusanov flux of the pair sorted by the signs of the axis offsets (sort_flux, Utils.jl:95-102; FluxFunctions.jl:66-76)
// and its flux difference contracted with the slot's divergence weights wk go into acc.
template <typename T, int D, int M, int PDE, int RDEG, bool ALE, bool MOM, class Acc>
__device__ __forceinline__ void flux_slot(const StageArgs<T> &a, const T *fi, const T (*gi)[M], const T (*Fi)[M],
                                          const T *wp, const T *fj, const T *gj, const int oi, const int oj,
                                          const bool below, const T *dk, const T *wk, Acc &acc,
                                          const int64_t i, const int k) {
    constexpr int BR = RBasis<D, RDEG>::B;
    constexpr bool kFast = sizeof(T) == 4;   // FP32: scaled Rusanov form
    const int64_t np = a.g.npad;
    (void)np; (void)i; (void)k; (void)wp;
    T pi[BR], pj[BR];
    if constexpr (kFast && RDEG == 1) {
        // degree 1: an interface of order 2 keeps the linear terms, order 1 none (the midpoint offsets
        // ±dk/2 scaled by 0 or ±1/2)
        const T si = oi >= 2 ? T(0.5) : T(0), sj = oj >= 2 ? T(-0.5) : T(0);
#pragma unroll
        for (int d = 0; d < D; ++d) { pi[d] = si * dk[d]; pj[d] = sj * dk[d]; }
    } else {
        const int keep_i = interface_terms<D, RDEG>(oi);
        const int keep_j = interface_terms<D, RDEG>(oj);
        T hx[D];
#pragma unroll
        for (int d = 0; d < D; ++d) hx[d] = T(0.5) * dk[d];
        recon_basis<D, RDEG, T>(hx, pi);
#pragma unroll
        for (int d = 0; d < D; ++d) hx[d] = T(-0.5) * dk[d];
        recon_basis<D, RDEG, T>(hx, pj);
#pragma unroll
        for (int b = 0; b < BR; ++b) {
            if (b >= keep_i) pi[b] = T(0);
            if (b >= keep_j) pj[b] = T(0);
        }
    }
    if constexpr (kFast && PDE != HCC_PDE_EULER && !ALE) {
        // FP32, linear fluxes F_d(f)_m = c_dm f_m with constant speeds (advection, BGK), fixed grid: the
        // doubled Rusanov difference per component on the fly, without flux arrays (registers:
        // 2 (F_n - F_i)_m = sum_d w_d (c_dm (f_ij + f_ji - 2 f_i) - s_d max(λ_d) (f_ji - f_ij)))
        T sw[D];
#pragma unroll
        for (int d = 0; d < D; ++d)
            sw[d] = (below ? wk[d] : dk[d]) > T(0) ? a.ph.amax[d] : -a.ph.amax[d];
        T t[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            T si = gi[0][m] * pi[0];
            T sj = gj[m] * pj[0];
#pragma unroll
            for (int b = 1; b < BR; ++b) {
                si = si + gi[b][m] * pi[b];
                sj = sj + gj[b * M + m] * pj[b];
            }
            const T fij = fi[m] + si, fji = fj[m] + sj;
            const T sum = (fij + fji) - T(2) * fi[m], jump = fji - fij;
            T tm = wk[0] * (a.ph.c[0][m] * sum - sw[0] * jump);
#pragma unroll
            for (int d = 1; d < D; ++d) tm = tm + wk[d] * (a.ph.c[d][m] * sum - sw[d] * jump);
            t[m] = tm;
            if constexpr (MOM) {
                T se = a.ph.amax[0] * a.g.mw[(int64_t(k) * D) * np + i];
#pragma unroll
                for (int d = 1; d < D; ++d) se = se + a.ph.amax[d] * a.g.mw[(int64_t(k) * D + d) * np + i];
                t[m] = t[m] - se * jump;
            }
        }
        acc.add(t);
        return;
    }
    T fij[M], fji[M];
    if constexpr (kFast) {
#pragma unroll
        for (int q = 0; q < M / 2; ++q) {
            float2 si = p_mul(p_ld(gi[0], q), p_bc(pi[0]));
            float2 sj = p_mul(p_ld(gj, q), p_bc(pj[0]));
#pragma unroll
            for (int b = 1; b < BR; ++b) {
                si = p_fma(p_ld(gi[b], q), p_bc(pi[b]), si);
                sj = p_fma(p_ld(gj + b * M, q), p_bc(pj[b]), sj);
            }
            p_st(fij, q, p_add(p_ld(fi, q), si));
            p_st(fji, q, p_add(p_ld(fj, q), sj));
        }
    }
#pragma unroll
    for (int m = kFast ? (M / 2) * 2 : 0; m < M; ++m) {
        T si = gi[0][m] * pi[0];
        T sj = gj[m] * pj[0];
#pragma unroll
        for (int b = 1; b < BR; ++b) {
            si = si + gi[b][m] * pi[b];
            sj = sj + gj[b * M + m] * pj[b];
        }
        fij[m] = fi[m] + si;
        fji[m] = fj[m] + sj;
    }
    if constexpr (projected_flux<T, PDE, ALE, MOM>()) {
        // FP32 Euler, fixed grid: the doubled Rusanov difference contracted with the slot's divergence weights,
        //   sum_d w_d [(F_d(f_ij) + F_d(f_ji)) - s_d max(λ_d) (f_ji - f_ij) - 2 F_d(f_i)]
        //     = Fw(f_ij) + Fw(f_ji) - S (f_ji - f_ij) - 2 Fw(f_i),   S = sum_d w_d s_d max(λ_d)
        // with Fw(U) = sum_d w_d F_d(U) (euler_projected) and 2 Fw(f_i) = (rho (2u.w), (2u.w) m + 2p w,
        // (E + p)(2u.w)) from the own constants of own_flux.
        T Fa[M], Fb[M], la[D], lb[D];
        euler_projected<D>(a.ph, fij, wk, Fa, la);
        euler_projected<D>(a.ph, fji, wk, Fb, lb);
        T S = T(0), un2 = T(0);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const T sd = vmax(la[d], lb[d]);
            const T ssd = (below ? wk[d] : dk[d]) > T(0) ? sd : -sd;
            S = (d == 0) ? wk[0] * ssd : S + wk[d] * ssd;
            un2 = (d == 0) ? wk[0] * Fi[0][0] : un2 + wk[d] * Fi[0][d];
        }
        T t[M], own[M];
        own[0] = fi[0] * un2;
#pragma unroll
        for (int e = 0; e < D; ++e) own[1 + e] = un2 * fi[1 + e] + Fi[0][D] * wk[e];
        own[D + 1] = Fi[0][D + 1] * un2;
#pragma unroll
        for (int m = 0; m < M; ++m) t[m] = ((Fa[m] + Fb[m]) - S * (fji[m] - fij[m])) - own[m];
        acc.add(t);
        return;
    }
    T Fij[D][M], Fji[D][M], lij[D], lji[D];
    flux_and_speed<T, D, M, PDE>(a.ph, fij, Fij, lij, wp);
    flux_and_speed<T, D, M, PDE>(a.ph, fji, Fji, lji, wp);
    T t[M];
    if constexpr (kFast) {
        // FP32: 2 (F_n - F_i) = (F_ij + F_ji) - s_d max(λ) (f_ji - f_ij) - 2 F_i with s_d = sign of the
        // axis component (the sort_flux orientation folded into the speed); the factor 2 leaves K = -Σ.
        // (pairs of components with the packed instructions, a scalar tail for odd M)
        T jump[M];
#pragma unroll
        for (int q = 0; q < M / 2; ++q) p_st(jump, q, p_sub(p_ld(fji, q), p_ld(fij, q)));
        if constexpr (M & 1) jump[M - 1] = fji[M - 1] - fij[M - 1];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const T ssd = (below ? wk[d] : dk[d]) > T(0) ? vmax(lij[d], lji[d]) : -vmax(lij[d], lji[d]);
            const float2 nssd = p_bc(-ssd), w2 = p_bc(wk[d]);
#pragma unroll
            for (int q = 0; q < M / 2; ++q) {
                const float2 Fs = p_add(p_ld(Fij[d], q), p_ld(Fji[d], q));
                const float2 dF2 = p_sub(p_fma(nssd, p_ld(jump, q), Fs), p_ld(Fi[d], q));
                p_st(t, q, (d == 0) ? p_mul(w2, dF2) : p_fma(w2, dF2, p_ld(t, q)));
            }
            if constexpr (M & 1) {
                const T dF2 = ((Fij[d][M - 1] + Fji[d][M - 1]) - ssd * jump[M - 1]) - Fi[d][M - 1];
                t[M - 1] = (d == 0) ? wk[0] * dF2 : t[M - 1] + wk[d] * dF2;
            }
        }
    } else {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const bool pos = (below ? wk[d] : dk[d]) > T(0);
            // sort_flux + Rusanov without per-component selects: F_L + F_R is Fij + Fji in either order
            // (IEEE addition commutes) and max(λ_L, λ_R) is symmetric; only f_R - f_L keeps its
            // orientation
            const T sdd = vmax(lij[d], lji[d]);
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const T jump = pos ? (fji[m] - fij[m]) : (fij[m] - fji[m]);
                const T Fn = T(0.5) * ((Fij[d][m] + Fji[d][m]) - sdd * jump);
                const T dF = Fn - Fi[d][m];
                t[m] = (d == 0) ? wk[0] * dF : t[m] + wk[d] * dF;
            }
        }
    }
    acc.add(t);
    if constexpr (MOM) {
        // moment correction of a first-order scheme (MUSCL.jl:501-505): -1/2 sum_d s_d e^d_ij (f_ji - f_ij),
        // the speeds s_d = max(λ_d) of the pair (FP32: the doubled form of the scaled Rusanov flux)
        T se = vmax(lij[0], lji[0]) * a.g.mw[(int64_t(k) * D) * np + i];
#pragma unroll
        for (int d = 1; d < D; ++d) se = se + vmax(lij[d], lji[d]) * a.g.mw[(int64_t(k) * D + d) * np + i];
        const T corr = kFast ? se : T(0.5) * se;
        T t2[M];
#pragma unroll
        for (int m = 0; m < M; ++m) t2[m] = -(corr * (fji[m] - fij[m]));
        acc.add(t2);
    }
}

// The flux pass of particle i over its slots k0, k0 + KSTEP, ... With KSTEP = 1 the whole pass and its epilogue;
// with KSTEP > 1 (FP32) the partial sums and extrema go to `part` for the caller to combine.
template <typename T, int D, int M, int PDE, int RDEG, bool ALE, int KSTEP = 1, bool MOM = false>
__device__ __forceinline__ bool flux_one(const StageArgs<T> &a, const int64_t i, const int k0 = 0,
                                         FluxPart<T, M> *part = nullptr, bool *rough = nullptr) {
    constexpr int BR = RBasis<D, RDEG>::B;
    if (a.g.bnd[i]) {
        if (a.full) {
#pragma unroll
            for (int m = 0; m < M; ++m) a.K[i * M + m] = T(0);
            if (a.mover)
#pragma unroll
                for (int d = 0; d < D; ++d) a.KXout[int64_t(d) * a.g.npad + i] = 0.0;
        }
        return false;
    }
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    const T invL = a.g.invL;
    (void)invL;
    T fi[M], gi[BR][M], Fi[D][M];
    load_vec<T, M>(a.U + i * M, fi);
    load_vec<T, BR * M>(a.grad + i * (BR * M), &gi[0][0]);
    // moving grid: this particle's grid velocity (K_X of the stage) and every flux in its frame
    T wv[D];
    const T *wp = nullptr;
    if constexpr (ALE) {
        grid_velocity<T, D, M, PDE>(a, i, fi, wv);
        wp = wv;
        if (k0 == 0)
#pragma unroll
            for (int d = 0; d < D; ++d) a.KXout[int64_t(d) * a.g.npad + i] = double(wv[d]);
    }
    own_flux<T, D, M, PDE, ALE, MOM>(a.ph, fi, Fi, wp);
    constexpr bool kFast = sizeof(T) == 4;   // FP32: scaled Rusanov form (flux_slot)
    const int oi_own = a.orders[i];
    const int didx = divergence_index(a.sc.DO, D, oi_own, cnt);
    const bool cached = a.g.ok_d[i] && didx == divergence_index(a.sc.DO, D, a.sc.max_order, cnt);
    const T *wsl = cached ? a.g.dw : a.g.dw1;
    const bool wok = cnt > 0 && (cached || (a.g.dw1 != nullptr && didx == 2 && a.g.ok_1[i]));
    const bool need_ext = a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2);
    const int nbmin_i = (a.sc.strategy == HCC_EPD2) ? a.nbmin[i] : 0;
    AccumV<T, M> acc;
    T mn[M], mx[M];
#pragma unroll
    for (int m = 0; m < M; ++m) { mn[m] = fi[m]; mx[m] = fi[m]; }

    // one slot: its neighbour's state, gradient and order, the interface orders, the flux
    auto slot = [&](const int32_t j, const T *dk, const T *wk, const int k) {
        T fj[M];
        load_vec<T, M>(a.U + int64_t(j) * M, fj);
        T gj[BR * M];
        load_vec<T, BR * M>(a.grad + int64_t(j) * (BR * M), gj);
        if (need_ext) {
#pragma unroll
            for (int m = 0; m < M; ++m) { mn[m] = vmin(mn[m], fj[m]); mx[m] = vmax(mx[m], fj[m]); }
        }
        const int oj_own = a.orders[j];
        int oi, oj;
        if (a.sc.strategy == HCC_EPD1) { oi = oj = (oi_own < oj_own ? oi_own : oj_own); }
        else if (a.sc.strategy == HCC_EPD2) { int nj = a.nbmin[j]; oi = oj = (nbmin_i < nj ? nbmin_i : nj); }
        else { oi = oi_own; oj = oj_own; }
        // AlignedRusanovFlux (MUSCL.jl:331-338): where either particle is below the full order (every pair at
        // order 1) the states are sorted by the signs of the slot's divergence weights instead of the distance
        const bool below = a.sc.aligned && (a.sc.max_order == 1 || oi_own < a.sc.max_order ||
                                            oj_own < a.sc.max_order);
        flux_slot<T, D, M, PDE, RDEG, ALE, MOM>(a, fi, gi, Fi, wp, fj, gj, oi, oj, below, dk, wk, acc, i, k);
    };
    // FP32 full passes: the slots in groups of UF, the next group's slot data in flight while this group is
    // computed (the slot body unrolled over the group); otherwise a one-deep software pipeline
    constexpr int UF = (kFast && KSTEP == 1) ? HCC_FLUX_STREAM_GROUP : 1;
    if (UF > 1 && wok && k0 < cnt) {
        int32_t jb[UF];
        T dkb[UF][D], wkb[UF][D];
#pragma unroll
        for (int u = 0; u < UF; ++u) {
            const int ku = k0 + u;
            jb[u] = ku < cnt ? a.g.nidx[int64_t(ku) * np + i] : 0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                dkb[u][d] = ku < cnt ? a.g.dist[(int64_t(ku) * D + d) * np + i] : T(0);
                wkb[u][d] = ku < cnt ? wsl[(int64_t(ku) * D + d) * np + i] : T(0);
            }
        }
        for (int k = k0; k < cnt; k += UF) {
            int32_t jn[UF];
            T dkn[UF][D], wkn[UF][D];
#pragma unroll
            for (int u = 0; u < UF; ++u) {
                const int kn = k + UF + u;
                jn[u] = kn < cnt ? a.g.nidx[int64_t(kn) * np + i] : 0;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    dkn[u][d] = kn < cnt ? a.g.dist[(int64_t(kn) * D + d) * np + i] : T(0);
                    wkn[u][d] = kn < cnt ? wsl[(int64_t(kn) * D + d) * np + i] : T(0);
                }
            }
#pragma unroll
            for (int u = 0; u < UF; ++u) {
                if (k + u >= cnt) break;
                slot(jb[u], dkb[u], wkb[u], k + u);
            }
#pragma unroll
            for (int u = 0; u < UF; ++u) {
                jb[u] = jn[u];
#pragma unroll
                for (int d = 0; d < D; ++d) { dkb[u][d] = dkn[u][d]; wkb[u][d] = wkn[u][d]; }
            }
        }
    } else if (wok && k0 < cnt) {
        // slot data of the next slot are loaded while this one is computed (one-deep software pipeline)
        int32_t jn = a.g.nidx[int64_t(k0) * np + i];
        T dkn[D], wkn[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            dkn[d] = a.g.dist[(int64_t(k0) * D + d) * np + i];
            wkn[d] = wsl[(int64_t(k0) * D + d) * np + i];
        }
        for (int k = k0; k < cnt; k += KSTEP) {
            const int32_t j = jn;
            T dk[D], wk[D];
#pragma unroll
            for (int d = 0; d < D; ++d) { dk[d] = dkn[d]; wk[d] = wkn[d]; }
            if (k + KSTEP < cnt) {
                jn = a.g.nidx[int64_t(k + KSTEP) * np + i];
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    dkn[d] = a.g.dist[(int64_t(k + KSTEP) * D + d) * np + i];
                    wkn[d] = wsl[(int64_t(k + KSTEP) * D + d) * np + i];
                }
            }
            slot(j, dk, wk, k);
        }
    } else if (need_ext) {
        for (int k = k0; k < cnt; k += KSTEP) {
            const int32_t j = a.g.nidx[int64_t(k) * np + i];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                T fj = a.U[int64_t(j) * M + m];
                mn[m] = vmin(mn[m], fj);
                mx[m] = vmax(mx[m], fj);
            }
        }
    }
    if constexpr (KSTEP > 1) {
        static_assert(sizeof(T) == 4, "split tiles are the FP32 path");
#pragma unroll
        for (int m = 0; m < M; ++m) {
            part->s[m] = acc.s[m];
            part->c[m] = acc.c[m];
            part->mn[m] = mn[m];
            part->mx[m] = mx[m];
        }
        return false;
    }
    T Kv[M];
#pragma unroll
    for (int m = 0; m < M; ++m) Kv[m] = kFast ? -acc.s[m] : -(T(2) * acc.s[m]);
    if (rough) {
        // the stencil of the stage state is not flat in some component (without the extrema: assume not flat)
        bool r = !need_ext;
#pragma unroll
        for (int m = 0; m < M; ++m) r = r || (mx[m] - mn[m]) > T(1e-6) * (fabs(mx[m]) + fabs(mn[m]));
        *rough = r;
    }
    return stage_epilogue<T, D, M, PDE, RDEG>(a, i, fi, Kv, mn, mx);
}

// Failed candidates of one tile (a warp's ballot) into the t list.
template <typename T> __device__ __forceinline__ void tile_failures(const StageArgs<T> &a, int64_t tile, bool f) {
    const unsigned b = __ballot_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && b) {
        a.tmask[tile] = b;
        a.ttiles[atomicAdd(a.tcount, 1u)] = int32_t(tile);
    }
}

// A full pass (one thread per particle) or a worklist pass over tiles (one warp per tile, the members of its word;
// the reach marks are cleared once read). Either way each warp reports the failed candidates of its tile.
template <typename T, int D, int M, int PDE, int RDEG, bool ALE, bool MOM = false>
__global__ void __launch_bounds__(HCC_FLUX_BLOCK, flux_min_blocks<T, D, M>()) k_flux(const StageArgs<T> a) {
    const int lane = int(threadIdx.x & 31);
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        bool rough = false;
        const bool f = (i < a.g.n) ? flux_one<T, D, M, PDE, RDEG, ALE, 1, MOM>(a, i, 0, nullptr,
                                                                               a.rough_words ? &rough : nullptr)
                                   : false;
        if (a.check) tile_failures(a, i >> 5, f);
        if (a.rough_words) {
            const unsigned b = __ballot_sync(0xffffffffu, rough);
            if (lane == 0 && (i >> 5) * 32 < a.g.n) a.rough_words[i >> 5] = b;
        }
        return;
    }
    const unsigned nt = *a.wcount;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool f = ((word >> lane) & 1u) ? flux_one<T, D, M, PDE, RDEG, ALE, 1, MOM>(a, i) : false;
        if (a.check) tile_failures(a, tile, f);
        if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
    }
}

// FP32 worklist pass with four warps per tile: warp w takes the slots k = w, w + 4, ... of every member of the tile
// (a quarter of the serial slot chain, the latency that bounds the short worklist passes), warp 0 combines the four
// compensated partial sums (Kahan over the partials, minus their compensations) and the extrema, and runs the
// epilogue. One block per tile, block-stride over the list.
template <typename T, int D, int M, int PDE, int RDEG, bool ALE, bool MOM = false>
__global__ void __launch_bounds__(128) k_flux_tiles(const StageArgs<T> a) {
    __shared__ FluxPart<T, M> parts[4][32];
    const int lane = int(threadIdx.x & 31), w = int(threadIdx.x >> 5);
    const unsigned nt = *a.wcount;
    for (unsigned q = blockIdx.x; q < nt; q += gridDim.x) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool live = ((word >> lane) & 1u) && !a.g.bnd[i];
        if (live) flux_one<T, D, M, PDE, RDEG, ALE, 4, MOM>(a, i, w, &parts[w][lane]);
        __syncthreads();
        if (w == 0) {
            bool f = false;
            if (live) {
                T Kv[M], mn[M], mx[M], fi[M];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    T sm = T(0), cm = T(0), comp = T(0);
                    mn[m] = parts[0][lane].mn[m];
                    mx[m] = parts[0][lane].mx[m];
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        const T y = parts[v][lane].s[m] - cm;
                        const T u = sm + y;
                        cm = (u - sm) - y;
                        sm = u;
                        comp = comp + parts[v][lane].c[m];
                        mn[m] = vmin(mn[m], parts[v][lane].mn[m]);
                        mx[m] = vmax(mx[m], parts[v][lane].mx[m]);
                    }
                    Kv[m] = -(sm - comp);
                }
                load_vec<T, M>(a.U + i * M, fi);
                f = stage_epilogue<T, D, M, PDE, RDEG>(a, i, fi, Kv, mn, mx);
            }
            if (a.check) tile_failures(a, tile, f);
            if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------------------------- tile-staged full passes (FP32)
// Full gather and flux passes of an FP32 context with tile tables (TileView): one block per tile of HCC_TILE
// consecutive particles first copies the tile's neighbour union into shared memory -- positions (and orders), states,
// and for the flux pass the gradients; a thread copies whole entries, and the ascending union ids make a warp's loads
// cover contiguous runs -- then every slot reads its neighbour from shared memory with 16-byte loads. Offsets
// x_j - x_i are exact differences of the quantised union positions, rounded once to FP32; the weight w(|x|^2) and the
// slot's gradient and divergence weights follow from the particle's FP32 fit rows. The arithmetic after that is
// flux_slot / the cached gather of the stream-fed passes. Each thread loads the union place of its next slot while
// it computes the current one.

// Shared-memory layout. Gather pass: one row per union entry, the position (D ints) then the state. Flux pass: an
// int4 array of positions (the order in .w), then one row per entry of the state and the gradient. Rows are whole
// 16-byte groups, an odd number of them, so the rows that the lanes of a warp read spread over the banks.
constexpr int tile_odd_groups(int words) {
    const int g = (words + 3) / 4;
    return (g % 2 == 1) ? g : g + 1;
}
template <int D, int M> constexpr int tile_gather_row() { return 4 * tile_odd_groups(D + M); }
template <int D, int M> constexpr int tile_flux_row() { return 4 * tile_odd_groups(M + D * M); }

// Exponential weight of a squared distance (MLSWeightFunctions.jl:68-82: 1 / the degree-4 Taylor sum of e^y,
// y = alpha r^2 / R^2), FP32.
__device__ __forceinline__ float tile_weight(float r2, float wscale) {
    const float y = r2 * wscale;
    return recip<float>(1.0f + y * (1.0f + y * (0.5f + y * (0.16666667f + y * 0.041666668f))));
}

template <int D>
__device__ __forceinline__ void tile_offset(const int *qj, const int *qi, float qt, float *x) {
#pragma unroll
    for (int d = 0; d < D; ++d) x[d] = float(qj[d] - qi[d]) * qt;
}

// N words of a 16-byte-aligned shared-memory row as whole 16-byte loads.
template <int N>
__device__ __forceinline__ void lds_words(const float *row, float *out) {
    constexpr int G = (N + 3) / 4;
    const float4 *r4 = reinterpret_cast<const float4 *>(row);
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const float4 v = r4[g];
        if (4 * g + 0 < N) out[4 * g + 0] = v.x;
        if (4 * g + 1 < N) out[4 * g + 1] = v.y;
        if (4 * g + 2 < N) out[4 * g + 2] = v.z;
        if (4 * g + 3 < N) out[4 * g + 3] = v.w;
    }
}

// N words into a 16-byte-aligned shared-memory row (the padding of the last group is written as zero).
template <int N>
__device__ __forceinline__ void sts_words(float *row, const float *in) {
    constexpr int G = (N + 3) / 4;
    float4 *r4 = reinterpret_cast<float4 *>(row);
#pragma unroll
    for (int g = 0; g < G; ++g)
        r4[g] = make_float4(in[4 * g], 4 * g + 1 < N ? in[4 * g + 1] : 0.0f, 4 * g + 2 < N ? in[4 * g + 2] : 0.0f,
                            4 * g + 3 < N ? in[4 * g + 3] : 0.0f);
}

// Reconstruction pre-pass, two threads per particle of the tile (slots k = h, h + 2, ... for h = 0, 1): the cached
// degree-1 fit of gather_one with the gradient weights recomputed per slot, the second thread's partial sums added by
// the first through shared memory; every other case (boundary, starved or lowered order, failed fit, limiter) goes
// through gather_one itself.
// Union entries a thread stages per round in the tile passes (all their loads in flight before the first store):
// HCC_TILE_STAGE_UNROLL for rows of up to 12 words, half as many for wider rows (registers).
template <int RW> constexpr int tile_stage_unroll() {
    return RW <= 12 ? HCC_TILE_STAGE_UNROLL : (HCC_TILE_STAGE_UNROLL + 1) / 2;
}

template <int D, int M> constexpr int tile_gather_min_blocks() { return M >= 8 ? 1 : 3; }

template <int D, int M, int PDE>
__global__ void __launch_bounds__(2 * HCC_TILE, tile_gather_min_blocks<D, M>()) k_gather_tile(const StageArgs<float> a) {
    extern __shared__ __align__(16) float sm[];
    constexpr int W = tile_gather_row<D, M>();
    const int64_t t = blockIdx.x;
    {
        const int64_t u0 = a.tv.ustart[t];
        const int nu = int(a.tv.ustart[t + 1] - u0);
        // SU entries per thread and round: their ids first, then every load of the round in flight, then the stores
        constexpr int SU = tile_stage_unroll<D + M>();
        const int nt = int(blockDim.x);
        for (int e0 = threadIdx.x; e0 < nu; e0 += SU * nt) {
            int32_t jj[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) jj[u] = e0 + u * nt < nu ? a.tv.uid[u0 + e0 + u * nt] : 0;
            float v[SU][D + M];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                if (e0 + u * nt >= nu) break;
                const int4 q = a.tv.upos[u0 + e0 + u * nt];
                v[u][0] = __int_as_float(q.x);
                if constexpr (D > 1) v[u][1] = __int_as_float(q.y);
                if constexpr (D > 2) v[u][2] = __int_as_float(q.z);
#pragma unroll
                for (int m = 0; m < M; ++m) v[u][D + m] = a.U[int64_t(jj[u]) * M + m];
            }
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                if (e0 + u * nt >= nu) break;
                sts_words<D + M>(sm + (e0 + u * nt) * W, v[u]);
            }
        }
    }
    float *parts = sm + a.tv.umax * W;           // [HCC_TILE][D * M] partial gradients of the second threads
    __syncthreads();
    const int pl = int(threadIdx.x) % HCC_TILE, h = int(threadIdx.x) / HCC_TILE;
    const int64_t i = t * HCC_TILE + pl;
    int mode = 0;                                 // 1: the cached fit here, 2: gather_one (first thread)
    int cnt = 0;
    if (i < a.g.n && !a.g.bnd[i]) {
        cnt = a.g.cnt[i];
        int q = a.orders[i];
        while (q > 1 && cnt < basis_count(D, q - 1)) --q;
        mode = (q == a.sc.max_order && q > 1 && a.g.ok_r[i] && a.sc.limiter == HCC_LIMITER_NONE) ? 1 : 2;
    }
    float out[D][M];
#pragma unroll
    for (int b = 0; b < D; ++b)
#pragma unroll
        for (int m = 0; m < M; ++m) out[b][m] = 0.0f;
    if (mode == 1) {
        const int64_t np = a.g.npad;
        float own[D + M];
        lds_words<D + M>(sm + int(a.tv.lself[i]) * W, own);
        int qi[D];
#pragma unroll
        for (int d = 0; d < D; ++d) qi[d] = __float_as_int(own[d]);
        float G[D][D];
        const float *cf = a.tv.coef + i * a.tv.cw + D + D * D;
#pragma unroll
        for (int b = 0; b < D; ++b)
#pragma unroll
            for (int c = 0; c < D; ++c) G[b][c] = cf[b * D + c];
        const float qt = a.tv.quantum[t], ws = a.tv.wscale;
        // this thread's slots h, h + 2, ...: their union places in groups of PF, the next group's loads in flight
        // while this group is summed
        constexpr int PF = HCC_TILE_GATHER_GROUP;
        const int mine = cnt > h ? (cnt - h + 1) / 2 : 0;
        const uint16_t *lp = a.tv.lidx + int64_t(h) * np + i;
        const int64_t step = 2 * np;
        int lbuf[PF];
#pragma unroll
        for (int q = 0; q < PF; ++q) lbuf[q] = q < mine ? int(lp[int64_t(q) * step]) : 0;
        for (int k0 = 0; k0 < mine; k0 += PF) {
            int lnext[PF];
#pragma unroll
            for (int q = 0; q < PF; ++q) lnext[q] = k0 + PF + q < mine ? int(lp[int64_t(k0 + PF + q) * step]) : 0;
#pragma unroll
            for (int q = 0; q < PF; ++q) {
                if (k0 + q >= mine) break;
                float r[D + M];
                lds_words<D + M>(sm + lbuf[q] * W, r);
                int qj[D];
#pragma unroll
                for (int d = 0; d < D; ++d) qj[d] = __float_as_int(r[d]);
                float x[D];
                tile_offset<D>(qj, qi, qt, x);
                float r2 = x[0] * x[0];
#pragma unroll
                for (int d = 1; d < D; ++d) r2 = r2 + x[d] * x[d];
                const float w = tile_weight(r2, ws);
                float gk[D];
#pragma unroll
                for (int b = 0; b < D; ++b) {
                    float v = G[b][0] * x[0];
#pragma unroll
                    for (int c = 1; c < D; ++c) v = v + G[b][c] * x[c];
                    gk[b] = w * v;
                }
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float dm = r[D + m] - own[D + m];
#pragma unroll
                    for (int b = 0; b < D; ++b) out[b][m] = out[b][m] + gk[b] * dm;
                }
            }
#pragma unroll
            for (int q = 0; q < PF; ++q) lbuf[q] = lnext[q];
        }
        if (h == 1)
#pragma unroll
            for (int b = 0; b < D; ++b)
#pragma unroll
                for (int m = 0; m < M; ++m) parts[pl * (D * M) + b * M + m] = out[b][m];
    }
    __syncthreads();
    if (h == 1) return;
    if (mode == 2) {
        gather_one<float, D, M, PDE, 1>(a, i);
    } else if (mode == 1) {
#pragma unroll
        for (int b = 0; b < D; ++b)
#pragma unroll
            for (int m = 0; m < M; ++m) out[b][m] = out[b][m] + parts[pl * (D * M) + b * M + m];
        store_vec<float, D * M>(a.grad + i * (D * M), &out[0][0]);
    }
}

// Flux pass, two threads per particle of the tile (slots k = h, h + 2, ... for h = 0, 1); the second writes its
// compensated partial sums and extrema to shared memory, the first combines them and runs the epilogue.
template <int D, int M> constexpr int tile_flux_min_blocks() { return M >= 8 ? 1 : 2; }

template <int D, int M, int PDE>
__global__ void __launch_bounds__(2 * HCC_TILE, tile_flux_min_blocks<D, M>()) k_flux_tile(const StageArgs<float> a) {
    extern __shared__ __align__(16) float sm[];
    constexpr int W = tile_flux_row<D, M>();
    constexpr int RW = M + D * M;                 // used words of a row: the state, then the gradient
    const int64_t t = blockIdx.x;
    const int64_t u0 = a.tv.ustart[t];
    const int nu = int(a.tv.ustart[t + 1] - u0);
    int4 *spos = reinterpret_cast<int4 *>(sm);
    float *srow = sm + 4 * a.tv.umax;
    FluxPart<float, M> *parts = reinterpret_cast<FluxPart<float, M> *>(srow + a.tv.umax * W);
    // the particle's own global loads (count, union place, fit rows, the first union places of its slots) are issued
    // before the staging so that their latency overlaps it; none of them reads shared memory
    const int pl = int(threadIdx.x) % HCC_TILE, h = int(threadIdx.x) / HCC_TILE;
    const int64_t i = t * HCC_TILE + pl;
    const bool live = i < a.g.n && !a.g.bnd[i];
    const int64_t np = a.g.npad;
    // this thread's slots h, h + 2, ...: union places PF slots ahead (a rotating window), or in groups of PF with the
    // next group in flight (HCC_TILE_FLUX_GROUP > 0: the slot body unrolled over the group)
    // (wide states, M >= 8, keep the window: the unrolled group spills their registers)
    constexpr int GROUP = M >= 8 ? 0 : HCC_TILE_FLUX_GROUP;
    constexpr int PF = GROUP > 0 ? GROUP : HCC_TILE_FLUX_PF;
    const int64_t lstep = 2 * np;
    const uint16_t *lp = a.tv.lidx + int64_t(h) * np + i;
    int cnt = 0, li = 0, mine = 0;
    bool wok = false;
    int lb[PF];
    float A[D], B[D][D];
    if (live) {
        cnt = a.g.cnt[i];
        li = int(a.tv.lself[i]);
        wok = cnt > 0 && a.g.ok_d[i];
        const float *cf = a.tv.coef + i * a.tv.cw;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            A[d] = cf[d];
#pragma unroll
            for (int e = 0; e < D; ++e) B[d][e] = cf[D + d * D + e];
        }
        mine = cnt > h ? (cnt - h + 1) / 2 : 0;
#pragma unroll
        for (int q = 0; q < PF; ++q) lb[q] = q < mine ? int(lp[int64_t(q) * lstep]) : 0;
        lp += int64_t(PF) * lstep;
    }
    {
        // SU entries per thread and round: their ids first, then every load of the round in flight, then the stores
        constexpr int SU = tile_stage_unroll<RW>();
        const int nt = int(blockDim.x);
        for (int e0 = threadIdx.x; e0 < nu; e0 += SU * nt) {
            int32_t jj[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) jj[u] = e0 + u * nt < nu ? a.tv.uid[u0 + e0 + u * nt] : 0;
            int4 qq[SU];
            float v[SU][RW];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                if (e0 + u * nt >= nu) break;
                const int64_t j = jj[u];
                qq[u] = a.tv.upos[u0 + e0 + u * nt];
                qq[u].w = a.orders[j];
#pragma unroll
                for (int m = 0; m < M; ++m) v[u][m] = a.U[j * M + m];
#pragma unroll
                for (int c = 0; c < D * M; ++c) v[u][M + c] = a.grad[j * (D * M) + c];
            }
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                if (e0 + u * nt >= nu) break;
                spos[e0 + u * nt] = qq[u];
                sts_words<RW>(srow + (e0 + u * nt) * W, v[u]);
            }
        }
    }
    __syncthreads();
    const bool need_ext = a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2);
    BlockAccum<M, HCC_FLUX_KAHAN_BLOCK> blk;
    AccumV<float, M> &acc = blk.sum;
    float mn[M], mx[M], fi[M];
    float gi[D][M], Fi[D][M];
    if (live) {
        const int4 q4 = spos[li];
        const int qi[3] = {q4.x, q4.y, q4.z};
        const int oi_own = q4.w;
        {
            float own[RW];
            lds_words<RW>(srow + li * W, own);
#pragma unroll
            for (int m = 0; m < M; ++m) { fi[m] = own[m]; mn[m] = fi[m]; mx[m] = fi[m]; }
#pragma unroll
            for (int b = 0; b < D; ++b)
#pragma unroll
                for (int m = 0; m < M; ++m) gi[b][m] = own[M + b * M + m];
        }
        own_flux<float, D, M, PDE, false, false>(a.ph, fi, Fi, nullptr);
        if (wok) {
            const float qt = a.tv.quantum[t], ws = a.tv.wscale;
            auto slot = [&](const int l, const int k) {
                const int4 qj4 = spos[l];
                const int qj[3] = {qj4.x, qj4.y, qj4.z};
                float dk[D], wk[D];
                tile_offset<D>(qj, qi, qt, dk);
                float r2 = dk[0] * dk[0];
#pragma unroll
                for (int d = 1; d < D; ++d) r2 = r2 + dk[d] * dk[d];
                const float w = tile_weight(r2, ws);
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    float v = A[d];
#pragma unroll
                    for (int e = 0; e < D; ++e) v = v + B[d][e] * dk[e];
                    wk[d] = w * v;
                }
                float r[RW];
                lds_words<RW>(srow + l * W, r);
                if (need_ext) {
#pragma unroll
                    for (int m = 0; m < M; ++m) { mn[m] = vmin(mn[m], r[m]); mx[m] = vmax(mx[m], r[m]); }
                }
                const int oj_own = qj4.w;
                int oi, oj;
                if (a.sc.strategy == HCC_EPD1) { oi = oj = (oi_own < oj_own ? oi_own : oj_own); }
                else { oi = oi_own; oj = oj_own; }
                const bool below = a.sc.aligned && (a.sc.max_order == 1 || oi_own < a.sc.max_order ||
                                                    oj_own < a.sc.max_order);
                flux_slot<float, D, M, PDE, 1, false, false>(a, fi, gi, Fi, nullptr, r, r + M, oi, oj, below, dk,
                                                             wk, blk, i, k);
            };
            if constexpr (GROUP > 0) {
                for (int s0 = 0; s0 < mine; s0 += PF) {
                    int ln[PF];
#pragma unroll
                    for (int q = 0; q < PF; ++q) ln[q] = s0 + PF + q < mine ? int(lp[int64_t(q) * lstep]) : 0;
                    lp += int64_t(PF) * lstep;
#pragma unroll
                    for (int q = 0; q < PF; ++q) {
                        if (s0 + q >= mine) break;
                        slot(lb[q], h + 2 * (s0 + q));
                    }
#pragma unroll
                    for (int q = 0; q < PF; ++q) lb[q] = ln[q];
                }
            } else {
                for (int s = 0; s < mine; ++s) {
                    const int l = lb[0];
#pragma unroll
                    for (int q = 0; q + 1 < PF; ++q) lb[q] = lb[q + 1];
                    lb[PF - 1] = s + PF < mine ? int(*lp) : 0;
                    lp += lstep;
                    slot(l, h + 2 * s);
                }
            }
            blk.flush();
        } else if (need_ext) {
            for (int s = 0; s < mine; ++s) {
                const int l = lb[0];
#pragma unroll
                for (int q = 0; q + 1 < PF; ++q) lb[q] = lb[q + 1];
                lb[PF - 1] = s + PF < mine ? int(*lp) : 0;
                lp += lstep;
                float r[M];
                lds_words<M>(srow + l * W, r);
#pragma unroll
                for (int m = 0; m < M; ++m) { mn[m] = vmin(mn[m], r[m]); mx[m] = vmax(mx[m], r[m]); }
            }
        }
        if (h == 1) {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                parts[pl].s[m] = acc.s[m];
                parts[pl].c[m] = acc.c[m];
                parts[pl].mn[m] = mn[m];
                parts[pl].mx[m] = mx[m];
            }
        }
    }
    __syncthreads();
    if (h == 1) return;
    bool f = false, rough = false;
    if (i < a.g.n) {
        if (a.g.bnd[i]) {
            float z[M];
#pragma unroll
            for (int m = 0; m < M; ++m) z[m] = 0.0f;
            store_vec<float, M>(a.K + i * M, z);
        } else {
            // the two compensated partials: their sum, minus both compensations and the rounding error of that sum
            float Kv[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const float s1 = parts[pl].s[m];
                const float u = acc.s[m] + s1;
                const float cm = (u - acc.s[m]) - s1;
                Kv[m] = -(u - ((acc.c[m] + parts[pl].c[m]) + cm));
                mn[m] = vmin(mn[m], parts[pl].mn[m]);
                mx[m] = vmax(mx[m], parts[pl].mx[m]);
            }
            if (a.rough_words) {
                bool r = !need_ext;
#pragma unroll
                for (int m = 0; m < M; ++m) r = r || (mx[m] - mn[m]) > 1e-6f * (fabsf(mx[m]) + fabsf(mn[m]));
                rough = r;
            }
            f = stage_epilogue<float, D, M, PDE, 1>(a, i, fi, Kv, mn, mx);
        }
    }
    if (a.check) tile_failures(a, i >> 5, f);
    if (a.rough_words) {
        const unsigned b = __ballot_sync(0xffffffffu, rough);
        if ((threadIdx.x & 31) == 0 && (i >> 5) * 32 < a.g.n) a.rough_words[i >> 5] = b;
    }
}

// The opt-in shared-memory limit of a block on the current device (the tile passes' dynamic allocation may go up
// to it).
inline int tile_smem_optin() {
    int dev = 0, v = 48 * 1024;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

// Dynamic shared memory of the tile passes for the largest union.
template <int D, int M> inline size_t tile_gather_smem(int umax) {
    return (size_t(umax) * tile_gather_row<D, M>() + size_t(HCC_TILE) * D * M) * sizeof(float);
}
template <int D, int M> inline size_t tile_flux_smem(int umax) {
    return size_t(umax) * (4 + tile_flux_row<D, M>()) * sizeof(float) + size_t(HCC_TILE) * sizeof(FluxPart<float, M>);
}

// ----------------------------------------------------------------------------------- WENO (scalar)
// _cholesky_moment (Interpolators.jl:31-64) and C \ b for a fixed basis size B (FP64).
template <int B>
__device__ __forceinline__ bool chol_upper_fixed(const double *A, double *U) {
    for (int q = 0; q < B * B; ++q) U[q] = 0.0;
    for (int r = 0; r < B; ++r)
        for (int c = r; c < B; ++c) {
            double sm = A[r * B + c];
            for (int q = 0; q < r; ++q) sm = sm - U[q * B + r] * U[q * B + c];
            if (r == c) {
                if (!(sm > 0.0)) return false;
                U[r * B + r] = sqrt(sm);
            } else {
                U[r * B + c] = sm / U[r * B + r];
            }
        }
    return true;
}
template <int B>
__device__ __forceinline__ bool chol_moment_fixed(double *N, double *U) {
    bool ok = chol_upper_fixed<B>(N, U);
    if (ok) {
        for (int q = 0; q < B; ++q) {
            const double u = U[q * B + q];
            if (!(u * u > 10.0 * 2.220446049250313e-16 * N[q * B + q])) { ok = false; break; }
        }
    }
    if (ok) return true;
    double tr = 0.0;
    for (int q = 0; q < B; ++q) tr = tr + N[q * B + q];
    const double er = 1.4901161193847656e-08 * tr / double(B);
    for (int q = 0; q < B; ++q) N[q * B + q] = N[q * B + q] + er;
    return chol_upper_fixed<B>(N, U);
}
template <int B>
__device__ __forceinline__ void chol_solve_fixed(const double *U, const double *b, double *x) {
    double y[B];
    for (int r = 0; r < B; ++r) {
        double t = b[r];
        for (int q = 0; q < r; ++q) t = t - U[q * B + r] * y[q];
        y[r] = t / U[r * B + r];
    }
    for (int r = B - 1; r >= 0; --r) {
        double t = y[r];
        for (int q = r + 1; q < B; ++q) t = t - U[r * B + q] * x[q];
        x[r] = t / U[r * B + r];
    }
}

// _mls_solve_masked of degree Q (Interpolators.jl:412-443) over the slots of particle i, all of them (dsel < 0) or
// the one-sided stencil along axis dsel: side 1 x_d < 0, side 2 x_d >= 0 (WENO's upwind sides), side 3 x_d <= 0
// (Tiwari's upwind side for v_d > 0), of the per-particle field g (fi = its value at i); out[0..D) = the
// first-derivative coefficients (scaled by invL). Returns the factorisation status (out = 0 when it fails).
template <typename T, int D, int Q, typename Field>
__device__ bool weno_fit_f(const StageArgs<T> &a, int64_t i, int cnt, int dsel, int side, double fi, Field g,
                           double *out) {
    constexpr int B = ExpTable<D, Q>::B;
    const int64_t np = a.g.npad;
    double N[B * B], bs[B];
    for (int q = 0; q < B * B; ++q) N[q] = 0.0;
    for (int q = 0; q < B; ++q) bs[q] = 0.0;
    for (int k = 0; k < cnt; ++k) {
        if (dsel >= 0) {
            const double dd = double(a.g.dist[(int64_t(k) * D + dsel) * np + i]);
            if (!(side == 1 ? dd < 0.0 : side == 2 ? dd >= 0.0 : dd <= 0.0)) continue;
        }
        const int64_t s = int64_t(k) * np + i;
        double x[D], p[B];
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = double(a.g.dist[(int64_t(k) * D + d) * np + i]) * a.g.invL64;
        table_basis<D, Q, double>(x, p);
        const double w = double(a.g.wt[s]);
        const double df = g(int64_t(a.g.nidx[s])) - fi;
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) N[r * B + c] = N[r * B + c] + w * (p[r] * p[c]);
        for (int r = 0; r < B; ++r) bs[r] = bs[r] + w * (p[r] * df);
    }
#pragma unroll
    for (int d = 0; d < D; ++d) out[d] = 0.0;
    double U[B * B], xs[B];
    if (!chol_moment_fixed<B>(N, U)) return false;
    chol_solve_fixed<B>(U, bs, xs);
#pragma unroll
    for (int d = 0; d < D; ++d) out[d] = xs[d] * a.g.invL64;   // degree-1 scale factors
    return true;
}

template <typename T, int D, int Q>
__device__ bool weno_fit(const StageArgs<T> &a, int64_t i, int cnt, int dsel, int side, double fi, double *out) {
    return weno_fit_f<T, D, Q>(a, i, cnt, dsel, side, fi, [&a](int64_t j) { return double(a.U[j]); }, out);
}

template <typename T, int D>
__device__ __forceinline__ void weno_fit_q(int q, const StageArgs<T> &a, int64_t i, int cnt, int dsel, int side,
                                           double fi, double *out) {
    if (q == 1) weno_fit<T, D, 1>(a, i, cnt, dsel, side, fi, out);
    else if (q == 2) weno_fit<T, D, 2>(a, i, cnt, dsel, side, fi, out);
    else weno_fit<T, D, 3>(a, i, cnt, dsel, side, fi, out);
}

// Position of the upper-triangle entry (r, c), r <= c, of a B x B matrix stored packed by rows.
template <int B> __host__ __device__ constexpr int packed_upper(int r, int c) { return r * B - r * (r - 1) / 2 + (c - r); }
// chol_solve_fixed with the factor packed: the same entries, the same operations in the same order.
template <int B>
__device__ __forceinline__ void chol_solve_packed(const double *U, const double *b, double *x) {
    double y[B];
    for (int r = 0; r < B; ++r) {
        double t = b[r];
        for (int q = 0; q < r; ++q) t = t - U[packed_upper<B>(q, r)] * y[q];
        y[r] = t / U[packed_upper<B>(r, r)];
    }
    for (int r = B - 1; r >= 0; --r) {
        double t = y[r];
        for (int q = r + 1; q < B; ++q) t = t - U[packed_upper<B>(r, q)] * x[q];
        x[r] = t / U[packed_upper<B>(r, r)];
    }
}

// weno_fit_f with the moment matrix's Cholesky factor taken from the geometry pass (k_weno_geom64: the same matrix,
// the same factorisation): only the right-hand side is summed here, in the same order, so the fit is bit for bit
// that of weno_fit_f.
template <typename T, int D, int Q, typename Field>
__device__ bool weno_fit_cached(const StageArgs<T> &a, int64_t i, int cnt, int dsel, int side, double fi, Field g,
                                const double *Up, bool ok, double *out) {
    constexpr int B = ExpTable<D, Q>::B;
    const int64_t np = a.g.npad;
    double bs[B];
    for (int q = 0; q < B; ++q) bs[q] = 0.0;
    for (int k = 0; k < cnt; ++k) {
        if (dsel >= 0) {
            const double dd = double(a.g.dist[(int64_t(k) * D + dsel) * np + i]);
            if (!(side == 1 ? dd < 0.0 : side == 2 ? dd >= 0.0 : dd <= 0.0)) continue;
        }
        const int64_t s = int64_t(k) * np + i;
        double x[D], p[B];
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = double(a.g.dist[(int64_t(k) * D + d) * np + i]) * a.g.invL64;
        table_basis<D, Q, double>(x, p);
        const double w = double(a.g.wt[s]);
        const double df = g(int64_t(a.g.nidx[s])) - fi;
        for (int r = 0; r < B; ++r) bs[r] = bs[r] + w * (p[r] * df);
    }
#pragma unroll
    for (int d = 0; d < D; ++d) out[d] = 0.0;
    if (!ok) return false;
    double xs[B];
    chol_solve_packed<B>(Up, bs, xs);
#pragma unroll
    for (int d = 0; d < D; ++d) out[d] = xs[d] * a.g.invL64;
    return true;
}

// The WENO functor (WENO.jl:55-165): central fit over the whole stencil and one upwind one-sided fit per axis,
// blended with w_S = 1 / (1 + (a_S / a_C)^2) on smoothness indicators IS = Σ_d (∂_d u)^2 h^2 normalised by
// max(u_i^2, IS_C); the result is Σ_d v_d ∂_d u and K_E = -that. Fits in FP64 in both paths.
template <typename T, int D>
__device__ __forceinline__ bool weno_one(const StageArgs<T> &a, const int64_t i) {
    if (a.g.bnd[i]) {
        if (a.full) a.K[i] = T(0);
        return false;
    }
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    const T fiT = a.U[i];
    T mn = fiT, mx = fiT;
    if (a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2))
        for (int k = 0; k < cnt; ++k) {
            const T fj = a.U[a.g.nidx[int64_t(k) * np + i]];
            mn = vmin(mn, fj);
            mx = vmax(mx, fj);
        }
    const double fi = double(fiT);
    double div_total = 0.0;
    int p_order = a.orders[i];
    while (p_order > 1 && cnt < basis_count(D, p_order)) --p_order;
    if (cnt >= basis_count(D, p_order)) {
        const int DO = a.sc.DO;
        const double dx2 = a.g.h64 * a.g.h64;
        double resC[D];
        weno_fit_q<T, D>(DO == 0 ? p_order : (DO < p_order ? DO : p_order), a, i, cnt, -1, 0, fi, resC);
        double smoothC = (resC[0] * resC[0]) * dx2;
#pragma unroll
        for (int d = 1; d < D; ++d) smoothC = smoothC + (resC[d] * resC[d]) * dx2;
        double s2 = jmax(fi * fi, smoothC);
        s2 = s2 > 0.0 ? s2 : 1.0;
        const double aC = smoothC / s2 + 1e-12;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double vel = double(a.ph.c[d][0]);
            const bool use_left = vel > 0.0;
            int stencil = 0;
            for (int k = 0; k < cnt; ++k) {
                const double dd = double(a.g.dist[(int64_t(k) * D + d) * np + i]);
                stencil += (use_left && dd < 0.0) || (!use_left && dd >= 0.0);
            }
            int p_d = p_order;
            while (p_d > 1 && stencil < basis_count(D, p_d)) --p_d;
            if (stencil < basis_count(D, p_d)) {
                div_total = div_total + resC[d] * vel;
                continue;
            }
            double resS[D];
            weno_fit_q<T, D>(DO == 0 ? p_d : (DO < p_d ? DO : p_d), a, i, cnt, d, use_left ? 1 : 2, fi, resS);
            double smoothS = (resS[0] * resS[0]) * dx2;
#pragma unroll
            for (int e = 1; e < D; ++e) smoothS = smoothS + (resS[e] * resS[e]) * dx2;
            const double q = (smoothS / s2 + 1e-12) / aC;
            const double wS = 1.0 / (1.0 + q * q);
            const double wC = 1.0 - wS;
            const double div_d = wS * resS[d] + wC * resC[d];
            div_total = div_total + div_d * vel;
        }
    }
    const T Kv = T(-div_total);
    return stage_epilogue<T, D, 1, HCC_PDE_ADVECTION>(a, i, &fiT, &Kv, &mn, &mx);
}

// A full pass or a worklist pass over tiles, as the MUSCL flux pass.
template <typename T, int D>
__global__ void __launch_bounds__(128) k_weno(const StageArgs<T> a) {
    const int lane = int(threadIdx.x & 31);
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        const bool f = (i < a.g.n) ? weno_one<T, D>(a, i) : false;
        if (a.check) tile_failures(a, i >> 5, f);
        return;
    }
    const unsigned nt = *a.wcount;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool f = ((word >> lane) & 1u) ? weno_one<T, D>(a, i) : false;
        if (a.check) tile_failures(a, tile, f);
        if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
    }
}

template <typename T, int D, typename Field>
__device__ __forceinline__ void weno_fit_qf(int q, const StageArgs<T> &a, int64_t i, int cnt, int dsel, int side,
                                            double fi, Field g, double *out) {
    if (q == 1) weno_fit_f<T, D, 1>(a, i, cnt, dsel, side, fi, g, out);
    else weno_fit_f<T, D, 2>(a, i, cnt, dsel, side, fi, g, out);
}

// Component-wise meshless WENO of a system (an extension of the scalar functor WENO.jl:55-165, which the reference
// defines for M = 1 only), orders 1 and 2: the central and one-sided fits, smoothness indicators and weights of the
// scalar scheme applied to one field at a time. Linear fluxes F_d(U)_m = c_dm U_m (advection, the kinetic model):
// field U_m, upwind side by the sign of c_dm, divergence sum_d c_dm d_d U_m. Euler: local Lax-Friedrichs splitting
// F_d^+- = (F_d(U) +- alpha_d U) / 2 with alpha_d the largest lambda_d over {i} u N(i); d_d F_d^+ from the
// left-biased one-sided fit (x_d < 0), d_d F_d^- from the right-biased one (x_d >= 0). Fits in FP64 in both paths.
template <typename T, int D, int M, int PDE>
__device__ __forceinline__ bool weno_sys_one(const StageArgs<T> &a, const int64_t i) {
    if (a.g.bnd[i]) {
        if (a.full) {
            T z[M];
#pragma unroll
            for (int m = 0; m < M; ++m) z[m] = T(0);
            store_vec<T, M>(a.K + i * M, z);
        }
        return false;
    }
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    T fiT[M], mn[M], mx[M];
    load_vec<T, M>(a.U + i * M, fiT);
#pragma unroll
    for (int m = 0; m < M; ++m) mn[m] = mx[m] = fiT[m];
    if (a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2))
        for (int k = 0; k < cnt; ++k) {
            const int64_t j = a.g.nidx[int64_t(k) * np + i];
#pragma unroll
            for (int m = 0; m < M; ++m) { mn[m] = vmin(mn[m], a.U[j * M + m]); mx[m] = vmax(mx[m], a.U[j * M + m]); }
        }
    double div[M];
#pragma unroll
    for (int m = 0; m < M; ++m) div[m] = 0.0;
    int p_order = a.orders[i];
    while (p_order > 1 && cnt < basis_count(D, p_order)) --p_order;
    if (cnt >= basis_count(D, p_order)) {
        const int DO = a.sc.DO;
        const double dx2 = a.g.h64 * a.g.h64;
        const int qC = DO == 0 ? p_order : (DO < p_order ? DO : p_order);
        // fit degree of the one-sided stencil of axis d (side 1: x_d < 0, side 2: x_d >= 0), 0 when too small
        auto one_sided = [&](int d, int side) {
            int stencil = 0;
            if (a.g.wcnt) {
                stencil = a.g.wcnt[i * (2 * D) + 2 * d + side - 1];
            } else {
                for (int k = 0; k < cnt; ++k) {
                    const double dd = double(a.g.dist[(int64_t(k) * D + d) * np + i]);
                    stencil += side == 1 ? (dd < 0.0) : (dd >= 0.0);
                }
            }
            int p_d = p_order;
            while (p_d > 1 && stencil < basis_count(D, p_d)) --p_d;
            if (stencil < basis_count(D, p_d)) return 0;
            return DO == 0 ? p_d : (DO < p_d ? DO : p_d);
        };
        auto smooth = [&](const double *r) {
            double sm = (r[0] * r[0]) * dx2;
#pragma unroll
            for (int d = 1; d < D; ++d) sm = sm + (r[d] * r[d]) * dx2;
            return sm;
        };
        if constexpr (PDE != HCC_PDE_EULER) {
            for (int m = 0; m < M; ++m) {
                auto g = [&a, m](int64_t j) { return double(a.U[j * M + m]); };
                const double fi = double(fiT[m]);
                double resC[D];
                weno_fit_qf<T, D>(qC, a, i, cnt, -1, 0, fi, g, resC);
                const double smoothC = smooth(resC);
                double s2 = jmax(fi * fi, smoothC);
                s2 = s2 > 0.0 ? s2 : 1.0;
                const double aC = smoothC / s2 + 1e-12;
                double div_total = 0.0;
                for (int d = 0; d < D; ++d) {
                    const double vel = double(a.ph.c[d][m]);
                    const int side = vel > 0.0 ? 1 : 2;
                    const int qS = one_sided(d, side);
                    if (qS == 0) {
                        div_total = div_total + resC[d] * vel;
                        continue;
                    }
                    double resS[D];
                    weno_fit_qf<T, D>(qS, a, i, cnt, d, side, fi, g, resS);
                    const double smoothS = smooth(resS);
                    const double q = (smoothS / s2 + 1e-12) / aC;
                    const double wS = 1.0 / (1.0 + q * q);
                    const double wC = 1.0 - wS;
                    const double div_d = wS * resS[d] + wC * resC[d];
                    div_total = div_total + div_d * vel;
                }
                div[m] = div_total;
            }
        } else {
            const double gamma = double(a.ph.gamma), gm1 = double(a.ph.gm1);
            // Euler primitives and lambda_d of a state in FP64 (euler_prim and speeds, operation for operation)
            auto prim = [gm1](const double *Uj, double &inv_rho, double *u, double &p) {
                const double rho = Uj[0];
                inv_rho = 1.0 / rho;
                double q2 = 0.0;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    u[d] = Uj[1 + d] * inv_rho;
                    q2 = (d == 0) ? u[d] * u[d] : q2 + u[d] * u[d];
                }
                p = gm1 * (Uj[D + 1] - 0.5 * (rho * q2));
            };
            auto lam = [&](const double *Uj, int d) {
                double inv_rho, u[D], p;
                prim(Uj, inv_rho, u, p);
                return fabs(u[d]) + sqrt(gamma * p * inv_rho);
            };
            double Ui[M];
#pragma unroll
            for (int m = 0; m < M; ++m) Ui[m] = double(fiT[m]);
            // with the geometry pass's factors and this stage's flux table (k_weno_prep64): the same values, each
            // computed once instead of once per fit
            const bool cached = a.g.wchol != nullptr && a.wflux64 != nullptr;
            constexpr int FW = D * (M + 1);                 // flux table row: F_d(U)_m then lambda_d, per axis
            double alpha[D];
            for (int d = 0; d < D; ++d) {
                alpha[d] = cached ? a.wflux64[i * FW + d * (M + 1) + M] : lam(Ui, d);
                for (int k = 0; k < cnt; ++k) {
                    const int64_t j = a.g.nidx[int64_t(k) * np + i];
                    if (cached) {
                        alpha[d] = jmax(alpha[d], a.wflux64[j * FW + d * (M + 1) + M]);
                        continue;
                    }
                    double Uj[M];
#pragma unroll
                    for (int m = 0; m < M; ++m) Uj[m] = double(a.U[j * M + m]);
                    alpha[d] = jmax(alpha[d], lam(Uj, d));
                }
            }
            constexpr int B2 = cbasis_count(D, 2), PK = B2 * (B2 + 1) / 2, NS = 2 * D + 1;
            auto fit = [&](int q, int dsel, int side, double fi, auto g, double *res) {
                if (!cached) {
                    weno_fit_qf<T, D>(q, a, i, cnt, dsel, side, fi, g, res);
                    return;
                }
                const int st = dsel < 0 ? 0 : 1 + 2 * dsel + side - 1;
                const int64_t slot = (i * 2 + (q - 1)) * NS + st;
                if (q == 1) weno_fit_cached<T, D, 1>(a, i, cnt, dsel, side, fi, g, a.g.wchol + slot * PK, a.g.wok[slot], res);
                else weno_fit_cached<T, D, 2>(a, i, cnt, dsel, side, fi, g, a.g.wchol + slot * PK, a.g.wok[slot], res);
            };
            for (int d = 0; d < D; ++d)
                for (int sg = 0; sg < 2; ++sg) {
                    const int side = sg == 0 ? 1 : 2;
                    const int qS = one_sided(d, side);
                    for (int m = 0; m < M; ++m) {
                        // F_d^+-(U_j)_m, the physical flux component as flux_and_speed forms it
                        auto g = [&a, &prim, &alpha, d, m, sg, cached](int64_t j) {
                            double F, Ujm;
                            if (cached) {
                                F = a.wflux64[j * FW + d * (M + 1) + m];
                                Ujm = double(a.U[j * M + m]);
                            } else {
                                double Uj[M];
#pragma unroll
                                for (int c = 0; c < M; ++c) Uj[c] = double(a.U[j * M + c]);
                                double inv_rho, u[D], p;
                                prim(Uj, inv_rho, u, p);
                                if (m == 0) F = Uj[1 + d];
                                else if (m <= D) F = (m - 1 == d) ? Uj[m] * u[d] + p : Uj[m] * u[d];
                                else F = (Uj[D + 1] + p) * u[d];
                                Ujm = Uj[m];
                            }
                            const double aU = alpha[d] * Ujm;
                            return sg == 0 ? 0.5 * (F + aU) : 0.5 * (F - aU);
                        };
                        const double fi = g(i);
                        double resC[D];
                        fit(qC, -1, 0, fi, g, resC);
                        double deriv = resC[d];
                        if (qS > 0) {
                            const double smoothC = smooth(resC);
                            double s2 = jmax(fi * fi, smoothC);
                            s2 = s2 > 0.0 ? s2 : 1.0;
                            const double aC = smoothC / s2 + 1e-12;
                            double resS[D];
                            fit(qS, d, side, fi, g, resS);
                            const double smoothS = smooth(resS);
                            const double q = (smoothS / s2 + 1e-12) / aC;
                            const double wS = 1.0 / (1.0 + q * q);
                            const double wC = 1.0 - wS;
                            deriv = wS * resS[d] + wC * resC[d];
                        }
                        div[m] = div[m] + deriv;
                    }
                }
        }
    }
    T Kv[M];
#pragma unroll
    for (int m = 0; m < M; ++m) Kv[m] = T(-div[m]);
    return stage_epilogue<T, D, M, PDE>(a, i, fiT, Kv, mn, mx);
}

template <typename T, int D, int M, int PDE>
__global__ void __launch_bounds__(128) k_weno_sys(const StageArgs<T> a) {
    const int lane = int(threadIdx.x & 31);
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        const bool f = (i < a.g.n) ? weno_sys_one<T, D, M, PDE>(a, i) : false;
        if (a.check) tile_failures(a, i >> 5, f);
        return;
    }
    const unsigned nt = *a.wcount;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool f = ((word >> lane) & 1u) ? weno_sys_one<T, D, M, PDE>(a, i) : false;
        if (a.check) tile_failures(a, tile, f);
        if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
    }
}

// UpwindDivergence (Upwind.jl), scalar advection, first order. Tiwari (:158-202): per axis d the gradient fit on
// the upwind side v_d x_d <= 0 (order lowered while that side has fewer than basis_count(D, p) points; an axis
// without enough contributes 0), summed as v_d (d_d u). Praveen (:205-249, 2-D): from the moment matrix
// N = sum w (x/L)(x/L)^T, per slot c = N^-1 (w x/L) / L, the edge normal n and tangent s, the coefficient
// (n . c) min(v . n, 0) + min((s . c)(v . s), 0) on u_j - u_i, summed and doubled. K_E = -that. FP64 fits.
template <typename T, int D, int ALG>
__device__ __forceinline__ bool upwind_one(const StageArgs<T> &a, const int64_t i) {
    if (a.g.bnd[i]) {
        if (a.full) a.K[i] = T(0);
        return false;
    }
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    const T fiT = a.U[i];
    T mn = fiT, mx = fiT;
    if (a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2))
        for (int k = 0; k < cnt; ++k) {
            const T fj = a.U[a.g.nidx[int64_t(k) * np + i]];
            mn = vmin(mn, fj);
            mx = vmax(mx, fj);
        }
    const double fi = double(fiT);
    double total = 0.0;
    if constexpr (ALG == HCC_UPWIND_TIWARI) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double vel = double(a.ph.c[d][0]);
            int stencil = 0;
            for (int k = 0; k < cnt; ++k)
                stencil += vel * double(a.g.dist[(int64_t(k) * D + d) * np + i]) <= 0.0;
            int p_d = a.orders[i];
            while (p_d > 1 && stencil < basis_count(D, p_d)) --p_d;
            if (stencil < basis_count(D, p_d)) continue;
            const int q = a.sc.DO == 0 ? p_d : (a.sc.DO < p_d ? a.sc.DO : p_d);
            // v_d x_d <= 0: x_d <= 0 for v_d > 0, x_d >= 0 for v_d < 0, every slot for v_d = 0
            double res[D];
            weno_fit_q<T, D>(q, a, i, cnt, vel == 0.0 ? -1 : d, vel > 0.0 ? 3 : 2, fi, res);
            total = total + res[d] * vel;
        }
    } else if constexpr (D == 2) {
        if (cnt >= 3 && a.g.h64 >= 1e-14) {
            const double iL = a.g.invL64;
            const double vx = double(a.ph.c[0][0]), vy = double(a.ph.c[1][0]);
            double n11 = 0.0, n12 = 0.0, n22 = 0.0;
            for (int k = 0; k < cnt; ++k) {
                const double w = double(a.g.wt[int64_t(k) * np + i]);
                const double x = double(a.g.dist[(int64_t(k) * 2) * np + i]) * iL;
                const double y = double(a.g.dist[(int64_t(k) * 2 + 1) * np + i]) * iL;
                n11 = n11 + w * (x * x);
                n12 = n12 + w * (x * y);
                n22 = n22 + w * (y * y);
            }
            const double det = n11 * n22 - n12 * n12;
            const double tr = n11 + n22;
            if (!(fabs(det) <= 4.0 * 2.220446049250313e-16 * (tr * tr))) {
                double div = 0.0;
                for (int k = 0; k < cnt; ++k) {
                    const double w = double(a.g.wt[int64_t(k) * np + i]);
                    const double dx = double(a.g.dist[(int64_t(k) * 2) * np + i]);
                    const double dy = double(a.g.dist[(int64_t(k) * 2 + 1) * np + i]);
                    const double bx = w * dx * iL, by = w * dy * iL;
                    const double cx = ((n22 * bx - n12 * by) / det) * iL;
                    const double cy = ((n11 * by - n12 * bx) / det) * iL;
                    const double hyp = sqrt(dx * dx + dy * dy);
                    double nx = 1.0, ny = 0.0;
                    if (!(hyp <= 2.220446049250313e-16 * a.g.h64)) { nx = dx / hyp; ny = dy / hyp; }
                    const double sx = -ny, sy = nx;
                    const double alfa = nx * cx + ny * cy;
                    const double beta = sx * cx + sy * cy;
                    const double vn = vx * nx + vy * ny;
                    const double vs = vx * sx + vy * sy;
                    const double bv = beta * vs;
                    const double cij = alfa * (vn < 0.0 ? vn : 0.0) + (bv < 0.0 ? bv : 0.0);
                    div = div + cij * (double(a.U[a.g.nidx[int64_t(k) * np + i]]) - fi);
                }
                total = 2.0 * div;
            }
        }
    }
    const T Kv = T(-total);
    return stage_epilogue<T, D, 1, HCC_PDE_ADVECTION>(a, i, &fiT, &Kv, &mn, &mx);
}

template <typename T, int D, int ALG>
__global__ void __launch_bounds__(128) k_upwind(const StageArgs<T> a) {
    const int lane = int(threadIdx.x & 31);
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        const bool f = (i < a.g.n) ? upwind_one<T, D, ALG>(a, i) : false;
        if (a.check) tile_failures(a, i >> 5, f);
        return;
    }
    const unsigned nt = *a.wcount;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool f = ((word >> lane) & 1u) ? upwind_one<T, D, ALG>(a, i) : false;
        if (a.check) tile_failures(a, tile, f);
        if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
    }
}

// CentralDivergence (Central.jl:45-88): the particle's order, lowered while it has fewer than basis_count(D, p) + 1
// neighbours (zero divergence if even order 1 lacks them), capped by div_order, selects the degree-q intercept fit
// of the flux differences F(f_j) - F(f_i); its per-slot weights (the geometry cache) are applied slot by slot.
// K_E = -div; the MOOD check of the next candidate runs in the shared epilogue.
template <typename T, int D, int M, int PDE>
__device__ __forceinline__ bool central_one(const StageArgs<T> &a, const int64_t i) {
    if (a.g.bnd[i]) {
        if (a.full) {
            T z[M];
#pragma unroll
            for (int m = 0; m < M; ++m) z[m] = T(0);
            store_vec<T, M>(a.K + i * M, z);
        }
        return false;
    }
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    T fi[M], mn[M], mx[M];
    load_vec<T, M>(a.U + i * M, fi);
#pragma unroll
    for (int m = 0; m < M; ++m) mn[m] = mx[m] = fi[m];
    const bool ext = a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2);
    int p = a.orders[i];
    while (p > 1 && cnt < basis_count(D, p) + 1) --p;
    const int q = a.sc.DO == 0 ? p : (a.sc.DO < p ? a.sc.DO : p);
    const T *wq = (cnt >= basis_count(D, p) + 1 && a.g.okc[q - 1][i]) ? a.g.dwc[q - 1] : nullptr;
    T Fi[D][M], lam[D], div[M];
    flux_and_speed<T, D, M, PDE>(a.ph, fi, Fi, lam);
#pragma unroll
    for (int m = 0; m < M; ++m) div[m] = T(0);
    for (int k = 0; k < cnt; ++k) {
        const int64_t j = a.g.nidx[int64_t(k) * np + i];
        T fj[M];
        load_vec<T, M>(a.U + j * M, fj);
        if (ext) {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                mn[m] = vmin(mn[m], fj[m]);
                mx[m] = vmax(mx[m], fj[m]);
            }
        }
        if (wq) {
            T Fj[D][M], lj[D];
            flux_and_speed<T, D, M, PDE>(a.ph, fj, Fj, lj);
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const T c = wq[(int64_t(k) * D + d) * np + i];
#pragma unroll
                for (int m = 0; m < M; ++m) div[m] = div[m] + c * (Fj[d][m] - Fi[d][m]);
            }
        }
    }
    T Kv[M];
#pragma unroll
    for (int m = 0; m < M; ++m) Kv[m] = -div[m];
    return stage_epilogue<T, D, M, PDE>(a, i, fi, Kv, mn, mx);
}

// A full pass or a worklist pass over tiles (the changed particles: no order reach), as the MUSCL flux pass.
template <typename T, int D, int M, int PDE>
__global__ void __launch_bounds__(128) k_central(const StageArgs<T> a) {
    const int lane = int(threadIdx.x & 31);
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        const bool f = (i < a.g.n) ? central_one<T, D, M, PDE>(a, i) : false;
        if (a.check) tile_failures(a, i >> 5, f);
        return;
    }
    const unsigned nt = *a.wcount;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool f = ((word >> lane) & 1u) ? central_one<T, D, M, PDE>(a, i) : false;
        if (a.check) tile_failures(a, tile, f);
        if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
    }
}

// form_candidate!(ts, eq, pg, 1, dt, t) (TimeSteppers.jl:365-397) for stage 1: Y_1 = Uⁿ (interior),
// the start-of-step state (boundary), then the implicit part. Boundary conditions follow in their own kernel.
template <typename T, int D, int M, int PDE, int RDEG>
__global__ void k_stage1(const StageArgs<T> a) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.g.n) return;
    T Y[M];
#pragma unroll
    for (int m = 0; m < M; ++m) Y[m] = a.Un[i * M + m];
    if (!a.g.bnd[i] && a.implicit_mode) {
        T KIo[M];
        implicit_part<T, D, M, PDE>(a, i, Y, KIo);
#pragma unroll
        for (int m = 0; m < M; ++m) a.KInext[i * M + m] = KIo[m];
    }
#pragma unroll
    for (int m = 0; m < M; ++m) a.Ynext[i * M + m] = Y[m];
}

// _cfl_weights_body! (ParticleGrids.jl:439-450) + the minimum over particles (:414).
template <typename T, int D, int M, int PDE, int RDEG>
__global__ void k_cfl(const StageArgs<T> a, unsigned long long *dt_bits) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double dti = INFINITY;
    if (i < a.g.n && !a.g.bnd[i]) {
        const int cnt = a.g.cnt[i];
        if (cnt > 0) {
            const int64_t np = a.g.npad;
            T Li[D];
            speeds<T, D, M, PDE>(a.ph, a.U + i * M, Li);
            T sum_c = T(0);
            for (int k = 0; k < cnt; ++k) {
                const int32_t j = a.g.nidx[int64_t(k) * np + i];
                T Lj[D];
                speeds<T, D, M, PDE>(a.ph, a.U + int64_t(j) * M, Lj);
                T dot = T(0);
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    T pr = fabs(a.g.dw[(int64_t(k) * D + d) * np + i]) * jmax(Li[d], Lj[d]);
                    dot = (d == 0) ? pr : dot + pr;
                }
                sum_c = sum_c + dot;
            }
            if (sum_c > floatmin_of<T>()) dti = double((T(1) / T(D)) / sum_c);
        }
    }
    // positive doubles order like their bit patterns
    unsigned long long b = __double_as_longlong(dti);
    int cl = 0;
    bool whole_warp = true;
    if (a.cloud_id) {   // one minimum per cloud of a batch (a warp straddling two clouds: one atomic per lane)
        cl = i < a.g.n ? a.cloud_id[i] : -1;
        whole_warp = __match_any_sync(0xffffffffu, cl) == 0xffffffffu;
        if (!whole_warp) {
            if (cl >= 0) atomicMin(dt_bits + cl, b);
            return;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long ob = __shfl_down_sync(0xffffffffu, b, o);
        b = ob < b ? ob : b;
    }
    if ((threadIdx.x & 31) == 0 && cl >= 0) atomicMin(dt_bits + cl, b);
}

// The CFL step of an FP32 context with tile tables (the same formula as k_cfl): per tile of HCC_TILE particles the
// union's quantised positions and the axis speeds of its states are staged in shared memory, one speed evaluation per
// union entry instead of one per slot, and each slot reads only its neighbour's union place; the slot offsets and
// divergence weights are recomputed from the positions and the particle's fit rows as in the tile flux pass. Two
// threads per particle (alternate slots, the second's partial sum through shared memory), the per-particle loads
// issued before the staging, every staging load of a thread in flight at once, union places in groups of four. One
// minimum for the whole cloud (batches with a minimum per cloud take k_cfl).
template <int D, int M, int PDE>
__global__ void __launch_bounds__(2 * HCC_TILE) k_cfl_tile(const StageArgs<float> a, unsigned long long *dt_bits) {
    extern __shared__ __align__(16) float sm[];
    int4 *spos = reinterpret_cast<int4 *>(sm);
    float4 *sspd = reinterpret_cast<float4 *>(sm + 4 * a.tv.umax);
    float *parts = sm + 8 * a.tv.umax;           // [HCC_TILE] partial sums of the second threads
    const int64_t t = blockIdx.x;
    const int64_t u0 = a.tv.ustart[t];
    const int nu = int(a.tv.ustart[t + 1] - u0);
    const int pl = int(threadIdx.x) % HCC_TILE, h = int(threadIdx.x) / HCC_TILE;
    const int64_t i = t * HCC_TILE + pl;
    const int64_t np = a.g.npad;
    constexpr int PF = 4;
    const int64_t lstep = 2 * np;
    const uint16_t *lp = a.tv.lidx + int64_t(h) * np + i;
    int li = 0, mine = 0;
    int lb[PF];
    float A[D], B[D][D];
    if (i < a.g.n && !a.g.bnd[i]) {
        const int cnt = a.g.cnt[i];
        if (cnt > 0 && a.g.ok_d[i]) {
            li = int(a.tv.lself[i]);
            const float *cf = a.tv.coef + i * a.tv.cw;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                A[d] = cf[d];
#pragma unroll
                for (int e = 0; e < D; ++e) B[d][e] = cf[D + d * D + e];
            }
            mine = cnt > h ? (cnt - h + 1) / 2 : 0;
#pragma unroll
            for (int q = 0; q < PF; ++q) lb[q] = q < mine ? int(lp[int64_t(q) * lstep]) : 0;
            lp += int64_t(PF) * lstep;
        }
    }
    {
        constexpr int SU = 4;
        const int nt = int(blockDim.x);
        for (int e0 = threadIdx.x; e0 < nu; e0 += SU * nt) {
            int32_t jj[SU];
#pragma unroll
            for (int u = 0; u < SU; ++u) jj[u] = e0 + u * nt < nu ? a.tv.uid[u0 + e0 + u * nt] : 0;
            int4 qq[SU];
            float U[SU][M];
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                if (e0 + u * nt >= nu) break;
                qq[u] = a.tv.upos[u0 + e0 + u * nt];
#pragma unroll
                for (int m = 0; m < M; ++m) U[u][m] = a.U[int64_t(jj[u]) * M + m];
            }
#pragma unroll
            for (int u = 0; u < SU; ++u) {
                if (e0 + u * nt >= nu) break;
                float L[D];
                speeds<float, D, M, PDE>(a.ph, U[u], L);
                spos[e0 + u * nt] = qq[u];
                sspd[e0 + u * nt] = make_float4(L[0], D > 1 ? L[D > 1 ? 1 : 0] : 0.0f,
                                                D > 2 ? L[D > 2 ? 2 : 0] : 0.0f, 0.0f);
            }
        }
    }
    __syncthreads();
    float sum_c = 0.0f;
    if (mine > 0) {
        const int4 q4 = spos[li];
        const int qi[3] = {q4.x, q4.y, q4.z};
        const float4 l4 = sspd[li];
        const float Li[3] = {l4.x, l4.y, l4.z};
        const float qt = a.tv.quantum[t], ws = a.tv.wscale;
        auto slot = [&](const int l) {
            const int4 qj4 = spos[l];
            const int qj[3] = {qj4.x, qj4.y, qj4.z};
            const float4 lj4 = sspd[l];
            const float Lj[3] = {lj4.x, lj4.y, lj4.z};
            float dk[D];
            tile_offset<D>(qj, qi, qt, dk);
            float r2 = dk[0] * dk[0];
#pragma unroll
            for (int d = 1; d < D; ++d) r2 = r2 + dk[d] * dk[d];
            const float w = tile_weight(r2, ws);
            float dot = 0.0f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                float v = A[d];
#pragma unroll
                for (int e = 0; e < D; ++e) v = v + B[d][e] * dk[e];
                const float pr = fabsf(w * v) * jmax(Li[d], Lj[d]);
                dot = (d == 0) ? pr : dot + pr;
            }
            sum_c = sum_c + dot;
        };
        // groups of PF union places, the next group in flight while this one is summed (the slot body unrolled)
        for (int s0 = 0; s0 < mine; s0 += PF) {
            int ln[PF];
#pragma unroll
            for (int q = 0; q < PF; ++q) ln[q] = s0 + PF + q < mine ? int(lp[int64_t(q) * lstep]) : 0;
            lp += int64_t(PF) * lstep;
#pragma unroll
            for (int q = 0; q < PF; ++q) {
                if (s0 + q >= mine) break;
                slot(lb[q]);
            }
#pragma unroll
            for (int q = 0; q < PF; ++q) lb[q] = ln[q];
        }
    }
    if (h == 1) parts[pl] = sum_c;
    __syncthreads();
    if (h == 1) return;
    double dti = INFINITY;
    if (i < a.g.n && !a.g.bnd[i]) {
        sum_c = sum_c + parts[pl];
        if (sum_c > floatmin_of<float>()) dti = double((1.0f / float(D)) / sum_c);
    }
    // positive doubles order like their bit patterns
    unsigned long long b = __double_as_longlong(dti);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_down_sync(0xffffffffu, b, o);
        b = ob < b ? ob : b;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(dt_bits, b);
}

// ----------------------------------------------------------------------------------- FP32 meshless WENO of Euler
// The fits of the component-wise WENO (weno_sys_one) are linear in the fitted field: out_s = sum_k c_{s,k} df_k with
// c_{s,k} = invL R_s (w_k p_k), R_s the first D rows of the inverse moment matrix of stencil s (the central stencil
// and, per axis, the slots with x_d < 0 and with x_d >= 0). The moment matrices depend on the geometry only: this
// pass assembles and factorises them once in FP64 (degree 2; the degree-1 matrix is its leading block, the same
// products), and stores R_s for both degrees in FP32, with the one-sided stencil sizes. A failed factorisation
// stores zeros (the fit returns zero, as in weno_fit_f).
template <int D>
__global__ void k_weno_geom(const WenoGeomArgs g) {
    constexpr int B1 = cbasis_count(D, 1), B2 = cbasis_count(D, 2), NS = 2 * D + 1;
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    float *out = g.ops + i * int64_t(2 * NS * D * B2);
    for (int q = 0; q < 2 * NS * D * B2; ++q) out[q] = 0.0f;
    if (g.bnd[i]) return;
    const int cnt = g.cnt[i];
    const int64_t np = g.npad;
    for (int st = 0; st < NS; ++st) {
        const int dsel = st == 0 ? -1 : (st - 1) / 2, side = st == 0 ? 0 : 1 + (st - 1) % 2;
        double N[B2 * B2];
        for (int q = 0; q < B2 * B2; ++q) N[q] = 0.0;
        int members = 0;
        for (int k = 0; k < cnt; ++k) {
            if (dsel >= 0) {
                const double dd = g.dist[(int64_t(k) * D + dsel) * np + i];
                if (!(side == 1 ? dd < 0.0 : dd >= 0.0)) continue;
            }
            ++members;
            double x[D], p[B2];
#pragma unroll
            for (int d = 0; d < D; ++d) x[d] = g.dist[(int64_t(k) * D + d) * np + i] * g.invL64;
            table_basis<D, 2, double>(x, p);
            const double w = g.w[int64_t(k) * np + i];
            for (int r = 0; r < B2; ++r)
                for (int c = r; c < B2; ++c) N[r * B2 + c] = N[r * B2 + c] + w * (p[r] * p[c]);
        }
        for (int r = 1; r < B2; ++r)
            for (int c = 0; c < r; ++c) N[r * B2 + c] = N[c * B2 + r];
        if (st > 0) g.wcnt[i * (2 * D) + (st - 1)] = members;
        {   // degree 1: the leading block
            double N1[B1 * B1], U1[B1 * B1];
            for (int r = 0; r < B1; ++r)
                for (int c = 0; c < B1; ++c) N1[r * B1 + c] = N[r * B2 + c];
            if (chol_moment_fixed<B1>(N1, U1)) {
                float *o = out + (0 * NS + st) * D * B2;
                for (int b = 0; b < B1; ++b) {
                    double e[B1], xs[B1];
                    for (int r = 0; r < B1; ++r) e[r] = r == b ? 1.0 : 0.0;
                    chol_solve_fixed<B1>(U1, e, xs);
#pragma unroll
                    for (int d = 0; d < D; ++d) o[d * B2 + b] = float(xs[d] * g.invL64);
                }
            }
        }
        {   // degree 2
            double U2[B2 * B2];
            if (chol_moment_fixed<B2>(N, U2)) {
                float *o = out + (1 * NS + st) * D * B2;
                for (int b = 0; b < B2; ++b) {
                    double e[B2], xs[B2];
                    for (int r = 0; r < B2; ++r) e[r] = r == b ? 1.0 : 0.0;
                    chol_solve_fixed<B2>(U2, e, xs);
#pragma unroll
                    for (int d = 0; d < D; ++d) o[d * B2 + b] = float(xs[d] * g.invL64);
                }
            }
        }
    }
}

// The FP64 path's counterpart of k_weno_geom: the same masked moment matrices (upper triangles, the same products
// in the same order), factorised by chol_moment_fixed as weno_fit_f does at every stage, stored packed with their
// flags; and the one-sided stencil sizes. weno_sys_one then sums only the right-hand sides.
template <int D>
__global__ void k_weno_geom64(const WenoGeomArgs g) {
    constexpr int B1 = cbasis_count(D, 1), B2 = cbasis_count(D, 2), NS = 2 * D + 1;
    constexpr int PK = B2 * (B2 + 1) / 2;
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    double *out = g.chol + i * int64_t(2 * NS * PK);
    uint8_t *okf = g.ok + i * int64_t(2 * NS);
    for (int q = 0; q < 2 * NS * PK; ++q) out[q] = 0.0;
    for (int q = 0; q < 2 * NS; ++q) okf[q] = 0;
    if (g.bnd[i]) return;
    const int cnt = g.cnt[i];
    const int64_t np = g.npad;
    for (int st = 0; st < NS; ++st) {
        const int dsel = st == 0 ? -1 : (st - 1) / 2, side = st == 0 ? 0 : 1 + (st - 1) % 2;
        double N[B2 * B2];
        for (int q = 0; q < B2 * B2; ++q) N[q] = 0.0;
        int members = 0;
        for (int k = 0; k < cnt; ++k) {
            if (dsel >= 0) {
                const double dd = g.dist[(int64_t(k) * D + dsel) * np + i];
                if (!(side == 1 ? dd < 0.0 : dd >= 0.0)) continue;
            }
            ++members;
            double x[D], p[B2];
#pragma unroll
            for (int d = 0; d < D; ++d) x[d] = g.dist[(int64_t(k) * D + d) * np + i] * g.invL64;
            table_basis<D, 2, double>(x, p);
            const double w = g.w[int64_t(k) * np + i];
            for (int r = 0; r < B2; ++r)
                for (int c = r; c < B2; ++c) N[r * B2 + c] = N[r * B2 + c] + w * (p[r] * p[c]);
        }
        if (st > 0) g.wcnt[i * (2 * D) + (st - 1)] = members;
        {   // degree 1: the leading block (the degree-1 basis is the degree-2 basis's first B1 terms)
            double N1[B1 * B1], U1[B1 * B1];
            for (int r = 0; r < B1; ++r)
                for (int c = 0; c < B1; ++c) N1[r * B1 + c] = N[r * B2 + c];
            const bool ok = chol_moment_fixed<B1>(N1, U1);
            okf[0 * NS + st] = ok;
            double *o = out + (0 * NS + st) * PK;
            for (int r = 0; r < B1; ++r)
                for (int c = r; c < B1; ++c) o[packed_upper<B1>(r, c)] = U1[r * B1 + c];
        }
        {   // degree 2
            double U2[B2 * B2];
            const bool ok = chol_moment_fixed<B2>(N, U2);
            okf[1 * NS + st] = ok;
            double *o = out + (1 * NS + st) * PK;
            for (int r = 0; r < B2; ++r)
                for (int c = r; c < B2; ++c) o[packed_upper<B2>(r, c)] = U2[r * B2 + c];
        }
    }
}

// The FP64 flux table of one stage for weno_sys_one: per particle F_d(U)_m and lambda_d, each by the same
// operations as the fits' field functions compute them.
template <int D>
__global__ void k_weno_prep64(const StageArgs<double> a) {
    constexpr int M = D + 2, FW = D * (M + 1);
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= a.g.n) return;
    const double gamma = double(a.ph.gamma), gm1 = double(a.ph.gm1);
    double Uj[M];
#pragma unroll
    for (int m = 0; m < M; ++m) Uj[m] = double(a.U[j * M + m]);
    const double rho = Uj[0];
    const double inv_rho = 1.0 / rho;
    double u[D], q2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        u[d] = Uj[1 + d] * inv_rho;
        q2 = (d == 0) ? u[d] * u[d] : q2 + u[d] * u[d];
    }
    const double p = gm1 * (Uj[D + 1] - 0.5 * (rho * q2));
    double *row = a.wflux64 + j * FW;
#pragma unroll
    for (int d = 0; d < D; ++d) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
            double F;
            if (m == 0) F = Uj[1 + d];
            else if (m <= D) F = (m - 1 == d) ? Uj[m] * u[d] + p : Uj[m] * u[d];
            else F = (Uj[D + 1] + p) * u[d];
            row[d * (M + 1) + m] = F;
        }
        row[d * (M + 1) + M] = fabs(u[d]) + sqrt(gamma * p * inv_rho);
    }
}

// The component-wise WENO of weno_sys_one for Euler in FP32 with the cached operators. Per axis d one pass over the
// slots accumulates, with the central operator and the operator of the slot's side, the gradients of the
// differences F_d(U_j)_m - F_d(U_i)_m and U_j,m - U_i,m and the largest lambda_d of the stencil (alpha_d); the split
// fields F_d^+- = (F_d +- alpha_d U) / 2 are linear in those, so their central and one-sided gradients, smoothness
// indicators and WENO weights follow without another pass. Same degree and stencil rules as weno_sys_one.
template <int D>
__device__ __forceinline__ bool weno_euler_f32_one(const StageArgs<float> &a, const int64_t i, float *sop) {
    constexpr int M = D + 2, B2 = cbasis_count(D, 2), NS = 2 * D + 1, R = D * B2;
    if (a.g.bnd[i]) {
        if (a.full) {
            float z[M];
#pragma unroll
            for (int m = 0; m < M; ++m) z[m] = 0.0f;
            store_vec<float, M>(a.K + i * M, z);
        }
        return false;
    }
    const int cnt = a.g.cnt[i];
    const int64_t np = a.g.npad;
    float Ui[M], mn[M], mx[M];
    load_vec<float, M>(a.U + i * M, Ui);
#pragma unroll
    for (int m = 0; m < M; ++m) mn[m] = mx[m] = Ui[m];
    const bool need_ext = a.check && (a.sc.criterion == HCC_MOOD_U1 || a.sc.criterion == HCC_MOOD_U2);
    float div[M];
#pragma unroll
    for (int m = 0; m < M; ++m) div[m] = 0.0f;
    int p_order = a.orders[i];
    while (p_order > 1 && cnt < basis_count(D, p_order)) --p_order;
    if (cnt >= basis_count(D, p_order)) {
        const int DO = a.sc.DO;
        const float dx2 = float(a.g.h64 * a.g.h64);
        const int qC = DO == 0 ? p_order : (DO < p_order ? DO : p_order);
        auto one_sided = [&](int d, int side) {
            const int stencil = a.g.wcnt[i * (2 * D) + 2 * d + side - 1];
            int p_d = p_order;
            while (p_d > 1 && stencil < basis_count(D, p_d)) --p_d;
            if (stencil < basis_count(D, p_d)) return 0;
            return DO == 0 ? p_d : (DO < p_d ? DO : p_d);
        };
        float inv_rho_i, u_i[D], p_i;
        euler_prim<float, D>(a.ph, Ui, inv_rho_i, u_i, p_i);
        const float c_i = root(a.ph.gamma * p_i * inv_rho_i);
        const float *ops = a.g.wops + i * int64_t(2 * NS * R);
        for (int d = 0; d < D; ++d) {
            const int q1 = one_sided(d, 1), q2 = one_sided(d, 2);
            // this axis's operators (central, side 1, side 2) into this thread's shared-memory row
            const float *oC = ops + ((qC - 1) * NS + 0) * R;
            const float *o1 = ops + ((q1 > 0 ? q1 - 1 : 0) * NS + 1 + 2 * d) * R;
            const float *o2 = ops + ((q2 > 0 ? q2 - 1 : 0) * NS + 2 + 2 * d) * R;
            for (int q = 0; q < R; ++q) { sop[q] = oC[q]; sop[R + q] = o1[q]; sop[2 * R + q] = o2[q]; }
            // F_d of the own state (flux_and_speed's components)
            float Fi[M];
            Fi[0] = Ui[1 + d];
#pragma unroll
            for (int e = 0; e < D; ++e) Fi[1 + e] = (e == d) ? Ui[1 + e] * u_i[d] + p_i : Ui[1 + e] * u_i[d];
            Fi[D + 1] = (Ui[D + 1] + p_i) * u_i[d];
            float alpha = fabsf(u_i[d]) + c_i;
            float gCF[M][D], gCU[M][D], gSF[2][M][D], gSU[2][M][D];
#pragma unroll
            for (int m = 0; m < M; ++m)
#pragma unroll
                for (int e = 0; e < D; ++e) {
                    gCF[m][e] = gCU[m][e] = 0.0f;
                    gSF[0][m][e] = gSU[0][m][e] = gSF[1][m][e] = gSU[1][m][e] = 0.0f;
                }
            // the next slot's index, offsets, weight and state are loaded while this one is computed
            int64_t jn = 0;
            float xn[D], wn = 0.0f, Un[M];
            auto load_slot = [&](int k) {
                jn = a.g.nidx[int64_t(k) * np + i];
#pragma unroll
                for (int e = 0; e < D; ++e) xn[e] = a.g.dist[(int64_t(k) * D + e) * np + i];
                wn = a.g.wt[int64_t(k) * np + i];
                load_vec<float, M>(a.U + jn * M, Un);
            };
            if (cnt > 0) load_slot(0);
            for (int k = 0; k < cnt; ++k) {
                float x[D], Uj[M];
#pragma unroll
                for (int e = 0; e < D; ++e) x[e] = xn[e] * a.g.invL;
                const float w = wn;
#pragma unroll
                for (int m = 0; m < M; ++m) Uj[m] = Un[m];
                if (k + 1 < cnt) load_slot(k + 1);
                const int sd = x[d] < 0.0f ? 0 : 1;
                float pb[B2];
                table_basis<D, 2, float>(x, pb);
#pragma unroll
                for (int b = 0; b < B2; ++b) pb[b] = w * pb[b];
                float cC[D], cS[D];
                const float *oS = sop + (1 + sd) * R;
#pragma unroll
                for (int e = 0; e < D; ++e) {
                    float vc = 0.0f, vs = 0.0f;
#pragma unroll
                    for (int b = 0; b < B2; ++b) { vc = vc + sop[e * B2 + b] * pb[b]; vs = vs + oS[e * B2 + b] * pb[b]; }
                    cC[e] = vc;
                    cS[e] = vs;
                }
                if (d == 0 && need_ext) {
#pragma unroll
                    for (int m = 0; m < M; ++m) { mn[m] = vmin(mn[m], Uj[m]); mx[m] = vmax(mx[m], Uj[m]); }
                }
                float inv_rho, u[D], pj;
                euler_prim<float, D>(a.ph, Uj, inv_rho, u, pj);
                alpha = vmax(alpha, fabsf(u[d]) + root(a.ph.gamma * pj * inv_rho));
                float Fj[M];
                Fj[0] = Uj[1 + d];
#pragma unroll
                for (int e = 0; e < D; ++e) Fj[1 + e] = (e == d) ? Uj[1 + e] * u[d] + pj : Uj[1 + e] * u[d];
                Fj[D + 1] = (Uj[D + 1] + pj) * u[d];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float dU = Uj[m] - Ui[m], dF = Fj[m] - Fi[m];
#pragma unroll
                    for (int e = 0; e < D; ++e) {
                        gCU[m][e] = gCU[m][e] + cC[e] * dU;
                        gCF[m][e] = gCF[m][e] + cC[e] * dF;
                        if (sd == 0) {
                            gSU[0][m][e] = gSU[0][m][e] + cS[e] * dU;
                            gSF[0][m][e] = gSF[0][m][e] + cS[e] * dF;
                        } else {
                            gSU[1][m][e] = gSU[1][m][e] + cS[e] * dU;
                            gSF[1][m][e] = gSF[1][m][e] + cS[e] * dF;
                        }
                    }
                }
            }
            // the split fields F_d^+ (side 1: x_d < 0) and F_d^- (side 2)
#pragma unroll
            for (int sg = 0; sg < 2; ++sg) {
                const float sgn = sg == 0 ? 1.0f : -1.0f;
                const int qS = sg == 0 ? q1 : q2;
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float fi = 0.5f * (Fi[m] + sgn * alpha * Ui[m]);
                    float gC[D];
#pragma unroll
                    for (int e = 0; e < D; ++e) gC[e] = 0.5f * (gCF[m][e] + sgn * alpha * gCU[m][e]);
                    float deriv = gC[d];
                    if (qS > 0) {
                        float smoothC = (gC[0] * gC[0]) * dx2;
#pragma unroll
                        for (int e = 1; e < D; ++e) smoothC = smoothC + (gC[e] * gC[e]) * dx2;
                        float s2 = vmax(fi * fi, smoothC);
                        s2 = s2 > 0.0f ? s2 : 1.0f;
                        const float aC = smoothC / s2 + 1e-12f;
                        float gS[D];
#pragma unroll
                        for (int e = 0; e < D; ++e) gS[e] = 0.5f * (gSF[sg][m][e] + sgn * alpha * gSU[sg][m][e]);
                        float smoothS = (gS[0] * gS[0]) * dx2;
#pragma unroll
                        for (int e = 1; e < D; ++e) smoothS = smoothS + (gS[e] * gS[e]) * dx2;
                        const float qq = (smoothS / s2 + 1e-12f) / aC;
                        const float wS = 1.0f / (1.0f + qq * qq);
                        deriv = wS * gS[d] + (1.0f - wS) * gC[d];
                    }
                    div[m] = div[m] + deriv;
                }
            }
        }
    } else if (need_ext) {
        for (int k = 0; k < cnt; ++k) {
            const int64_t j = a.g.nidx[int64_t(k) * np + i];
#pragma unroll
            for (int m = 0; m < M; ++m) { mn[m] = vmin(mn[m], a.U[j * M + m]); mx[m] = vmax(mx[m], a.U[j * M + m]); }
        }
    }
    float Kv[M];
#pragma unroll
    for (int m = 0; m < M; ++m) Kv[m] = -div[m];
    return stage_epilogue<float, D, M, HCC_PDE_EULER>(a, i, Ui, Kv, mn, mx);
}

template <int D>
__global__ void __launch_bounds__(128) k_weno_euler_f32(const StageArgs<float> a) {
    constexpr int RS = (3 * D * cbasis_count(D, 2)) | 1;   // odd row stride: conflict-free per-thread rows
    extern __shared__ float wsm[];
    float *sop = wsm + int(threadIdx.x) * RS;
    const int lane = int(threadIdx.x & 31);
    if (a.full) {
        const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        const bool f = (i < a.g.n) ? weno_euler_f32_one<D>(a, i, sop) : false;
        if (a.check) tile_failures(a, i >> 5, f);
        return;
    }
    const unsigned nt = *a.wcount;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned q = warp; q < nt; q += nwarps) {
        const int32_t tile = a.wtiles[q];
        const uint32_t word = a.wmask[tile];
        const int64_t i = int64_t(tile) * 32 + lane;
        const bool f = ((word >> lane) & 1u) ? weno_euler_f32_one<D>(a, i, sop) : false;
        if (a.check) tile_failures(a, tile, f);
        if (lane == 0 && a.clear_wmask) a.wmask[tile] = 0u;
    }
}
template <int D> inline size_t weno_euler_smem() {
    return size_t(128) * ((3 * D * cbasis_count(D, 2)) | 1) * sizeof(float);
}

// ----------------------------------------------------------------------------------- launchers / registry
template <typename T, int D, int M, int PDE, int RDEG>
struct StageInst {
    static unsigned grid(int64_t n, int bs) { return unsigned((n + bs - 1) / bs); }
    static unsigned pass_grid(const StageArgs<T> &a, int64_t n, int bs) {
        const unsigned g = grid(n, bs);
        return a.full ? g : std::max(1u, std::min(g, unsigned(a.list_blocks)));
    }
    // block of a full pass of the other flux-like schemes (the tuned flux block); worklist passes keep 128
    static int fbs(const StageArgs<T> &a) { return a.full ? a.flux_block : 128; }
    static void gather(const void *args, int64_t n, cudaStream_t s) {
        const StageArgs<T> &a = *static_cast<const StageArgs<T> *>(args);
        if constexpr (sizeof(T) == 4 && RDEG == 1) {
            if (a.full && a.tile) {   // FP32 full pass with tile tables: neighbours staged in shared memory
                static bool attr = false;
                if (!attr) {
                    cudaFuncSetAttribute(k_gather_tile<D, M, PDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tile_smem_optin());
                    attr = true;
                }
                k_gather_tile<D, M, PDE><<<unsigned(a.tv.ntiles), 2 * HCC_TILE, tile_gather_smem<D, M>(a.tv.umax), s>>>(a);
                return;
            }
            if (!a.full) {   // FP32 degree-1 worklist pass: split tiles (four warps a tile)
                k_gather_tiles<T, D, M, PDE, RDEG><<<std::max(1u, unsigned(a.list_blocks)), 128, 0, s>>>(a);
                return;
            }
        }
        const int bs = a.full ? a.gather_block : 128;
        k_gather<T, D, M, PDE, RDEG><<<pass_grid(a, n, bs), bs, 0, s>>>(a);
    }
    template <bool MOM> static void flux_mom(const StageArgs<T> &a, int64_t n, cudaStream_t s) {
        if constexpr (sizeof(T) == 4) {
            if (!a.full) {
                const unsigned g = std::max(1u, unsigned(a.list_blocks));
                if (a.mover) k_flux_tiles<T, D, M, PDE, RDEG, true, MOM><<<g, 128, 0, s>>>(a);
                else k_flux_tiles<T, D, M, PDE, RDEG, false, MOM><<<g, 128, 0, s>>>(a);
                return;
            }
        }
        const int bs = a.full ? a.flux_block : HCC_FLUX_BLOCK;
        if (a.mover)
            k_flux<T, D, M, PDE, RDEG, true, MOM><<<pass_grid(a, n, bs), bs, 0, s>>>(a);
        else
            k_flux<T, D, M, PDE, RDEG, false, MOM><<<pass_grid(a, n, bs), bs, 0, s>>>(a);
    }
    static void flux(const void *args, int64_t n, cudaStream_t s) {
        const StageArgs<T> &a = *static_cast<const StageArgs<T> *>(args);
        // first-order MUSCL with the moment correction: its own instantiation (the per-slot correction costs the
        // plain pass registers)
        if constexpr (RDEG == 1) {
            if (a.g.mw) { flux_mom<true>(a, n, s); return; }
        }
        if constexpr (sizeof(T) == 4) {
            if constexpr (RDEG == 1) {
                if (a.full && a.tile) {   // full pass with tile tables: neighbours staged in shared memory
                    static bool attr = false;
                    if (!attr) {
                        cudaFuncSetAttribute(k_flux_tile<D, M, PDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             tile_smem_optin());
                        attr = true;
                    }
                    k_flux_tile<D, M, PDE><<<unsigned(a.tv.ntiles), 2 * HCC_TILE, tile_flux_smem<D, M>(a.tv.umax), s>>>(a);
                    return;
                }
            }
            if (!a.full) {   // FP32 worklist pass: split tiles (four warps a tile)
                const unsigned g = std::max(1u, unsigned(a.list_blocks));
                if (a.mover) k_flux_tiles<T, D, M, PDE, RDEG, true><<<g, 128, 0, s>>>(a);
                else k_flux_tiles<T, D, M, PDE, RDEG, false><<<g, 128, 0, s>>>(a);
                return;
            }
        }
        const int bs = a.full ? a.flux_block : HCC_FLUX_BLOCK;
        if (a.mover)     // moving grid: the ALE-frame instantiation (grid velocities, shifted fluxes and speeds)
            k_flux<T, D, M, PDE, RDEG, true><<<pass_grid(a, n, bs), bs, 0, s>>>(a);
        else
            k_flux<T, D, M, PDE, RDEG, false><<<pass_grid(a, n, bs), bs, 0, s>>>(a);
    }
    static void stage1(const void *args, int64_t n, cudaStream_t s) {
        k_stage1<T, D, M, PDE, RDEG><<<grid(n, 256), 256, 0, s>>>(*static_cast<const StageArgs<T> *>(args));
    }
    static void cfl(const void *args, int64_t n, unsigned long long *dt_bits, cudaStream_t s) {
        const StageArgs<T> &a = *static_cast<const StageArgs<T> *>(args);
        if constexpr (sizeof(T) == 4 && RDEG == 1) {
            if (a.tile && !a.cloud_id) {   // FP32 with tile tables: the union's speeds staged in shared memory
                const size_t smem = (size_t(a.tv.umax) * 8 + HCC_TILE) * sizeof(float);
                static bool attr = false;
                if (!attr) {
                    cudaFuncSetAttribute(k_cfl_tile<D, M, PDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tile_smem_optin());
                    attr = true;
                }
                k_cfl_tile<D, M, PDE><<<unsigned(a.tv.ntiles), 2 * HCC_TILE, smem, s>>>(a, dt_bits);
                return;
            }
        }
        k_cfl<T, D, M, PDE, RDEG><<<grid(n, 256), 256, 0, s>>>(a, dt_bits);
    }
    static void weno(const void *args, int64_t n, cudaStream_t s) {
        const StageArgs<T> &a = *static_cast<const StageArgs<T> *>(args);
        if constexpr (sizeof(T) == 4 && PDE == HCC_PDE_EULER && RDEG == 1) {
            if (a.g.wops) {   // FP32 Euler with the cached operators
                static bool attr = false;
                if (!attr) {
                    cudaFuncSetAttribute(k_weno_euler_f32<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(weno_euler_smem<D>()));
                    attr = true;
                }
                k_weno_euler_f32<D><<<pass_grid(a, n, 128), 128, weno_euler_smem<D>(), s>>>(a);
                return;
            }
        }
        if constexpr (sizeof(T) == 8 && PDE == HCC_PDE_EULER && RDEG == 1) {
            // the stage's flux table, once per stage state (the MOOD worklist passes reuse it)
            if (a.full && a.wflux64) k_weno_prep64<D><<<grid(n, 256), 256, 0, s>>>(a);
        }
        if constexpr (M == 1 && PDE == HCC_PDE_ADVECTION) {
            k_weno<T, D><<<pass_grid(a, n, fbs(a)), fbs(a), 0, s>>>(a);
        } else if constexpr (RDEG == 1) {       // systems (one instantiation: WENO has no reconstruction degree)
            k_weno_sys<T, D, M, PDE><<<pass_grid(a, n, fbs(a)), fbs(a), 0, s>>>(a);
        }
    }
    static void upwind(const void *args, int64_t n, cudaStream_t s) {
        if constexpr (M == 1 && PDE == HCC_PDE_ADVECTION) {
            const StageArgs<T> &a = *static_cast<const StageArgs<T> *>(args);
            if (a.sc.upwind_alg == HCC_UPWIND_TIWARI)
                k_upwind<T, D, HCC_UPWIND_TIWARI><<<pass_grid(a, n, fbs(a)), fbs(a), 0, s>>>(a);
            else if constexpr (D == 2)
                k_upwind<T, D, HCC_UPWIND_PRAVEEN><<<pass_grid(a, n, fbs(a)), fbs(a), 0, s>>>(a);
        }
    }
    static void weno_geom(const WenoGeomArgs &g, cudaStream_t s) {
        if constexpr (PDE == HCC_PDE_EULER && RDEG == 1) {
            if (g.n <= 0) return;
            if constexpr (sizeof(T) == 4) k_weno_geom<D><<<unsigned((g.n + 127) / 128), 128, 0, s>>>(g);
            else k_weno_geom64<D><<<unsigned((g.n + 127) / 128), 128, 0, s>>>(g);
        }
    }
    static void central(const void *args, int64_t n, cudaStream_t s) {
        const StageArgs<T> &a = *static_cast<const StageArgs<T> *>(args);
        k_central<T, D, M, PDE><<<pass_grid(a, n, fbs(a)), fbs(a), 0, s>>>(a);
    }
    static const StageOps *ops() {
        static const StageOps o = {D, M, PDE, RDEG, RBasis<D, RDEG>::B, &gather, &flux, &stage1, &cfl,
                                   ((M == 1 && PDE == HCC_PDE_ADVECTION) || RDEG == 1) ? &weno : nullptr,
                                   RDEG == 1 ? &central : nullptr,
                                   (RDEG == 1 && M == 1 && PDE == HCC_PDE_ADVECTION) ? &upwind : nullptr,
                                   (PDE == HCC_PDE_EULER && RDEG == 1) ? &weno_geom : nullptr};
        return &o;
    }
};

template <typename T, int RDEG>
const StageOps *lookup_rdeg(int D, int M, int pde) {
    if (pde == HCC_PDE_EULER) {
        if (D == 1 && M == 3) return StageInst<T, 1, 3, HCC_PDE_EULER, RDEG>::ops();
        if (D == 2 && M == 4) return StageInst<T, 2, 4, HCC_PDE_EULER, RDEG>::ops();
        if (D == 3 && M == 5) return StageInst<T, 3, 5, HCC_PDE_EULER, RDEG>::ops();
        return nullptr;
    }
    if (pde == HCC_PDE_BGK) {
        if (D == 2 && M == 16) return StageInst<T, 2, 16, HCC_PDE_BGK, RDEG>::ops();
        if (D == 1 && M == 2) return StageInst<T, 1, 2, HCC_PDE_BGK, RDEG>::ops();
        return nullptr;
    }
    if (D == 1 && M == 1) return StageInst<T, 1, 1, HCC_PDE_ADVECTION, RDEG>::ops();
    if (D == 2 && M == 1) return StageInst<T, 2, 1, HCC_PDE_ADVECTION, RDEG>::ops();
    if (D == 3 && M == 1) return StageInst<T, 3, 1, HCC_PDE_ADVECTION, RDEG>::ops();
    if (D == 2 && M == 2) return StageInst<T, 2, 2, HCC_PDE_ADVECTION, RDEG>::ops();
    return nullptr;
}


}  // namespace hcc
