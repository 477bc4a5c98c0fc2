// hcc_mls.cu — FP64 MLS geometry caches (compiled with -fmad=false).
//
// One thread per particle assembles the moment matrices of its stencil, factorises them with the reference's
// conditional-Tikhonov Cholesky rule and writes
//   * the inverse moment matrix of the full-order reconstruction fit (MLSWeights, Interpolators.jl:517-577),
//   * the inverse of the divergence fit with intercept, of the degree the stencil carries at full order
//     (_FullOrderDivDegree, MUSCL.jl:169-179), zero-padded,
//   * the per-slot divergence weights c_ij = (R (w_j p~_j)) invL (update_divergence_weights!, MUSCL.jl:197-223),
//   * for adaptive-degree schemes, the per-slot weights of the degree-1 fit that MOOD-lowered particles use
//     (_slot_weight(::DynamicWeights), MUSCL.jl:442-445).
// The outflow donor map (the state-independent part of OutflowBC, BoundaryConditions.jl:82-130) is built here too.
#include "hcc_internal.cuh"
#include <algorithm>
#include <array>
#include <mutex>

namespace hcc {
namespace {

constexpr int kMaxDeg = 3;
constexpr int kMaxB = 20;            // basis_count(3, 3) + 1

struct BasisTab {
    int B;
    int exps[kMaxB][3];
    double pref[kMaxB];
    int has_pref[kMaxB];
};

__constant__ BasisTab c_tabs[4][kMaxDeg + 1];   // [D][degree]

int factorial(int n) { return n <= 1 ? 1 : n * factorial(n - 1); }

// _generate_exponents (Interpolators.jl:138-155)
std::vector<std::array<int, 3>> generate_exponents(int D, int max_order) {
    std::vector<std::array<int, 3>> res;
    for (int order = 1; order <= max_order; ++order) {
        std::vector<std::array<int, 3>> cur;
        int n = order + 1, total = 1;
        for (int d = 0; d < D; ++d) total *= n;
        for (int lin = 0; lin < total; ++lin) {
            std::array<int, 3> t{0, 0, 0};
            int r = lin, s = 0;
            for (int d = 0; d < D; ++d) { t[d] = r % n; r /= n; s += t[d]; }
            if (s == order) cur.push_back(t);
        }
        std::stable_sort(cur.begin(), cur.end(), [D](const std::array<int, 3> &a, const std::array<int, 3> &b) {
            int ma = 0, mb = 0;
            for (int d = 0; d < D; ++d) { ma = std::max(ma, a[d]); mb = std::max(mb, b[d]); }
            if (ma != mb) return ma > mb;
            for (int d = D - 1; d >= 0; --d)
                if (a[d] != b[d]) return a[d] < b[d];
            return false;
        });
        res.insert(res.end(), cur.begin(), cur.end());
    }
    return res;
}

std::once_flag g_tabs_once;
cudaError_t g_tabs_err = cudaSuccess;

void upload_tables() {
    static BasisTab host[4][kMaxDeg + 1];
    for (int D = 1; D <= 3; ++D)
        for (int q = 0; q <= kMaxDeg; ++q) {
            auto ex = generate_exponents(D, q);
            BasisTab &t = host[D][q];
            t.B = int(ex.size());
            for (int k = 0; k < t.B; ++k) {
                int den = 1;
                for (int d = 0; d < 3; ++d) { t.exps[k][d] = ex[k][d]; den *= factorial(ex[k][d]); }
                t.pref[k] = 1.0 / double(den);
                t.has_pref[k] = den != 1;
            }
        }
    g_tabs_err = cudaMemcpyToSymbol(c_tabs, host, sizeof(host));
}

__device__ __forceinline__ double ipow(double x, int p) {
    if (p == 2) return x * x;
    if (p == 3) return x * x * x;
    double r = x;
    for (int i = 1; i < p; ++i) r = r * x;
    return r;
}

// build_basis (Interpolators.jl:194-218), table driven; `intercept` prepends the constant 1 (:354).
__device__ void gen_basis(int D, int q, bool intercept, const double *x, double *p) {
    const BasisTab &t = c_tabs[D][q];
    int o = 0;
    if (intercept) p[o++] = 1.0;
    for (int k = 0; k < t.B; ++k) {
        bool have = t.has_pref[k];
        double v = have ? t.pref[k] : 0.0;
        for (int i = 0; i < D; ++i) {
            int e = t.exps[k][i];
            if (e == 0) continue;
            double f = (e == 1) ? x[i] : ipow(x[i], e);
            v = have ? v * f : f;
            have = true;
        }
        p[o++] = v;
    }
}

// Cholesky with the pivot rule and Tikhonov retry (Interpolators.jl:31-64).
__device__ bool cholesky_upper(int B, const double *A, double *U) {
    for (int i = 0; i < B * B; ++i) U[i] = 0.0;
    for (int i = 0; i < B; ++i) {
        for (int j = i; j < B; ++j) {
            double s = A[i * B + j];
            for (int k = 0; k < i; ++k) s = s - U[k * B + i] * U[k * B + j];
            if (i == j) {
                if (!(s > 0.0)) return false;
                U[i * B + i] = sqrt(s);
            } else {
                U[i * B + j] = s / U[i * B + i];
            }
        }
    }
    return true;
}

__device__ bool cholesky_moment(int B, double *N, double *U) {
    bool ok = cholesky_upper(B, N, U);
    if (ok) {
        const double tol = 10.0 * 2.220446049250313e-16;
        for (int k = 0; k < B; ++k) {
            double u = U[k * B + k];
            if (!(u * u > tol * N[k * B + k])) { ok = false; break; }
        }
    }
    if (ok) return true;
    double tr = 0.0;
    for (int k = 0; k < B; ++k) tr = tr + N[k * B + k];
    double eps_reg = 1.4901161193847656e-08 * tr / double(B);   // sqrt(eps(Float64)) tr(N) / B
    for (int k = 0; k < B; ++k) N[k * B + k] = N[k * B + k] + eps_reg;
    return cholesky_upper(B, N, U);
}

template <int BM>
__device__ void chol_solve(int B, const double *U, const double *b, double *x) {
    double y[BM];
    for (int r = 0; r < B; ++r) {
        double t = b[r];
        for (int k = 0; k < r; ++k) t = t - U[k * B + r] * y[k];
        y[r] = t / U[r * B + r];
    }
    for (int r = B - 1; r >= 0; --r) {
        double t = y[r];
        for (int k = r + 1; k < B; ++k) t = t - U[r * B + k] * x[k];
        x[r] = t / U[r * B + r];
    }
}

// Moment matrix of particle i for a fit of degree q (optionally with intercept): N = Σ w (p p'). The upper
// triangle is summed and mirrored: p_r p_c and p_c p_r are the same IEEE product, so every entry equals the full
// matrix's sum of the same terms in the same order, bit for bit, with 37-45 % fewer FP64 instructions (the
// pass is bound by the FP64 unit).
template <int BM>
__device__ void assemble(const MlsArgs &a, int64_t i, int cnt, int q, bool intercept, int B, double *N) {
    for (int k = 0; k < B * B; ++k) N[k] = 0.0;
    double x[3], p[BM];
    for (int k = 0; k < cnt; ++k) {
        int64_t s = int64_t(k) * a.npad + i;
        for (int d = 0; d < a.D; ++d) x[d] = a.dist[(int64_t(k) * a.D + d) * a.npad + i] * a.invL;
        gen_basis(a.D, q, intercept, x, p);
        double w = a.w[s];
        for (int r = 0; r < B; ++r)
            for (int c = r; c < B; ++c) N[r * B + c] = N[r * B + c] + w * (p[r] * p[c]);
    }
    for (int r = 1; r < B; ++r)
        for (int c = 0; c < r; ++c) N[r * B + c] = N[c * B + r];
}

// Inverse (C \ e_j per column) of an assembled B×B moment matrix N (overwritten), padded into a Bpad×Bpad block.
template <int BM>
__device__ bool invert_assembled(int B, double *N, int Bpad, double *out) {
    double U[BM * BM];
    for (int k = 0; k < Bpad * Bpad; ++k) out[k] = 0.0;
    if (!cholesky_moment(B, N, U)) return false;
    double e[BM], x[BM];
    for (int j = 0; j < B; ++j) {
        for (int r = 0; r < B; ++r) e[r] = (r == j) ? 1.0 : 0.0;
        chol_solve<BM>(B, U, e, x);
        for (int r = 0; r < B; ++r) out[r * Bpad + j] = x[r];
    }
    return true;
}

// Inverse moment matrix of the fit of degree q, padded into a Bpad×Bpad block.
template <int BM>
__device__ bool inverse_moment(const MlsArgs &a, int64_t i, int cnt, int q, bool intercept, int Bpad, double *out) {
    const int B = c_tabs[a.D][q].B + (intercept ? 1 : 0);
    double N[BM * BM];
    assemble<BM>(a, i, cnt, q, intercept, B, N);
    return invert_assembled<BM>(B, N, Bpad, out);
}

// One instantiation per basis capacity BM (4: degree-1 fits in 3-D; 10: degree 3 in 2-D; 20: degree 3 in 3-D),
// so that the per-thread arrays stay as small as the context's largest fit.
template <int BM>
__global__ void k_mls(MlsArgs a) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int cnt = a.cnt[i];
    double inv[BM * BM];
    if (a.weno_cfl_degree > 0) {
        // per-slot CFL weights of the assembled Taylor fit (_compute_cfl_coeffs, ParticleGrids.jl:296-329):
        // rows 1..D of inv(N) times p, times w and invL (the CFL pass takes their absolute values)
        const int qc = a.weno_cfl_degree;
        const int Bq = c_tabs[a.D][qc].B;
        const bool ok = inverse_moment<BM>(a, i, cnt, qc, false, Bq, inv);
        a.ok_r[i] = ok;
        a.ok_d[i] = ok;
        double x[3], p[BM];
        for (int k = 0; k < cnt; ++k) {
            const int64_t s = int64_t(k) * a.npad + i;
            for (int d = 0; d < a.D; ++d) x[d] = a.dist[(int64_t(k) * a.D + d) * a.npad + i] * a.invL;
            gen_basis(a.D, qc, false, x, p);
            const double w = a.w[s];
            for (int d = 0; d < a.D; ++d) {
                double cv = inv[d * Bq + 0] * p[0];
                for (int jb = 1; jb < Bq; ++jb) cv = cv + inv[d * Bq + jb] * p[jb];
                a.dw[(int64_t(k) * a.D + d) * a.npad + i] = ok ? cv * w * a.invL : 0.0;
            }
        }
        return;
    }
    // reconstruction fit (every particle, MLSWeights without intercept) and the divergence fit of the degree the
    // stencil carries at full order (padded to Bd). Where the two degrees agree, the reconstruction moments are the
    // divergence moments without the intercept row and column -- the same products w (p_r p_c) summed in the same
    // order, bit for bit -- so one assembly serves both.
    const int q = divergence_index(a.DO, a.D, a.max_order, cnt) - 1;
    bool okr, okd;
    if (q == a.rdeg) {
        const int Bq = c_tabs[a.D][q].B, B1 = Bq + 1;
        double Nd[BM * BM], Nr[BM * BM];
        assemble<BM>(a, i, cnt, q, true, B1, Nd);
        for (int r = 0; r < Bq; ++r)
            for (int c = 0; c < Bq; ++c) Nr[r * Bq + c] = Nd[(r + 1) * B1 + (c + 1)];
        okr = invert_assembled<BM>(Bq, Nr, a.Br, inv);
        for (int k = 0; k < a.Br * a.Br; ++k) a.inv_r[i * a.Br * a.Br + k] = inv[k];
        okd = invert_assembled<BM>(B1, Nd, a.Bd, inv);
    } else {
        okr = inverse_moment<BM>(a, i, cnt, a.rdeg, false, a.Br, inv);
        for (int k = 0; k < a.Br * a.Br; ++k) a.inv_r[i * a.Br * a.Br + k] = inv[k];
        okd = inverse_moment<BM>(a, i, cnt, q, true, a.Bd, inv);
    }
    a.ok_r[i] = okr;
    for (int k = 0; k < a.Bd * a.Bd; ++k) a.inv_d[i * a.Bd * a.Bd + k] = inv[k];
    a.ok_d[i] = okd;
    double x[3], p[BM], v[BM];
    for (int k = 0; k < cnt; ++k) {
        int64_t s = int64_t(k) * a.npad + i;
        if (!okd) {
            for (int d = 0; d < a.D; ++d) a.dw[(int64_t(k) * a.D + d) * a.npad + i] = 0.0;
            continue;
        }
        for (int d = 0; d < a.D; ++d) x[d] = a.dist[(int64_t(k) * a.D + d) * a.npad + i] * a.invL;
        gen_basis(a.D, a.ddeg, true, x, p);
        double w = a.w[s];
        for (int b = 0; b < a.Bd; ++b) v[b] = w * p[b];
        for (int d = 0; d < a.D; ++d) {
            const double *row = inv + (1 + d) * a.Bd;
            double acc = row[0] * v[0];
            for (int b = 1; b < a.Bd; ++b) acc = acc + row[b] * v[b];
            a.dw[(int64_t(k) * a.D + d) * a.npad + i] = acc * a.invL;
        }
    }
    if (!a.need_dw1) return;
    // degree-1 fit with intercept: per-slot weights C \ (w p~), rows 2..D+1, times invL
    const int B1 = a.D + 1;
    double N[BM * BM], U[BM * BM];
    assemble<BM>(a, i, cnt, 1, true, B1, N);
    bool ok1 = cholesky_moment(B1, N, U);
    a.ok_1[i] = ok1;
    for (int k = 0; k < cnt; ++k) {
        int64_t s = int64_t(k) * a.npad + i;
        if (!ok1) {
            for (int d = 0; d < a.D; ++d) a.dw1[(int64_t(k) * a.D + d) * a.npad + i] = 0.0;
            continue;
        }
        for (int d = 0; d < a.D; ++d) x[d] = a.dist[(int64_t(k) * a.D + d) * a.npad + i] * a.invL;
        gen_basis(a.D, 1, true, x, p);
        double w = a.w[s];
        for (int b = 0; b < B1; ++b) p[b] = w * p[b];
        chol_solve<BM>(B1, U, p, v);
        for (int d = 0; d < a.D; ++d) a.dw1[(int64_t(k) * a.D + d) * a.npad + i] = v[d + 1] * a.invL;
    }
}

// CentralDivergence weight set of degree q (Central.jl:45-88 with compute_dynamic_divergence,
// Interpolators.jl:290-334, per slot as _slot_weight(::DynamicWeights), MUSCL.jl:442-445): C \ (w p~), rows 2..D+1,
// times invL, for the particles with basis_count(D, q) + 1 neighbours (the others never use degree q).
template <int BM>
__global__ void k_mls_central(MlsArgs a, int q) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int cnt = a.cnt[i];
    const int B = c_tabs[a.D][q].B + 1;
    double *dwq = a.dwc[q - 1];
    double N[BM * BM], U[BM * BM];
    bool ok = false;
    if (cnt >= B) {
        assemble<BM>(a, i, cnt, q, true, B, N);
        ok = cholesky_moment(B, N, U);
    }
    a.okc[q - 1][i] = ok;
    double x[3], p[BM], v[BM];
    for (int k = 0; k < cnt; ++k) {
        const int64_t s = int64_t(k) * a.npad + i;
        if (!ok) {
            for (int d = 0; d < a.D; ++d) dwq[(int64_t(k) * a.D + d) * a.npad + i] = 0.0;
            continue;
        }
        for (int d = 0; d < a.D; ++d) x[d] = a.dist[(int64_t(k) * a.D + d) * a.npad + i] * a.invL;
        gen_basis(a.D, q, true, x, p);
        const double w = a.w[s];
        for (int b = 0; b < B; ++b) p[b] = w * p[b];
        chol_solve<BM>(B, U, p, v);
        for (int d = 0; d < a.D; ++d) dwq[(int64_t(k) * a.D + d) * a.npad + i] = v[d + 1] * a.invL;
    }
}

// _moment_mu (MUSCL.jl:285-330) for particle i: mu with sum_k (x_k . mu)_+ x_k = b over the scaled offsets, by Newton
// steps on the active slots with Armijo backtracking; zero when b is zero, a Hessian fails the pivot test or 30
// steps do not converge. The operation order is the oracle's.
__device__ void moment_hessian(const MlsArgs &a, int64_t i, int cnt, const double *m, const double *b, double *H,
                               double *g, double *phi, bool all) {
    const int D = a.D;
    for (int q = 0; q < D * D; ++q) H[q] = 0.0;
    if (g) for (int d = 0; d < D; ++d) g[d] = -b[d];
    if (phi) {
        double t = b[0] * m[0];
        for (int d = 1; d < D; ++d) t = t + b[d] * m[d];
        *phi = -t;
    }
    for (int k = 0; k < cnt; ++k) {
        double x[3];
        for (int d = 0; d < D; ++d) x[d] = a.dist[(int64_t(k) * D + d) * a.npad + i] * a.invL;
        double t = 0.0;
        if (!all) {
            t = x[0] * m[0];
            for (int d = 1; d < D; ++d) t = t + x[d] * m[d];
            if (!(t > 0.0)) continue;
        }
        for (int r = 0; r < D; ++r)
            for (int c = 0; c < D; ++c) H[r * D + c] = H[r * D + c] + x[r] * x[c];
        if (g) for (int d = 0; d < D; ++d) g[d] = g[d] + t * x[d];
        if (phi) *phi = *phi + (t * t) / 2.0;
    }
}
__device__ bool moment_pivots_ok(int D, const double *H, double *U) {
    if (!cholesky_upper(D, H, U)) return false;
    for (int k = 0; k < D; ++k) {
        const double u = U[k * D + k];
        if (!(u * u > 10.0 * 2.220446049250313e-16 * H[k * D + k])) return false;
    }
    return true;
}
__device__ void moment_mu(const MlsArgs &a, int64_t i, int cnt, const double *b, double *mu) {
    const int D = a.D;
    for (int d = 0; d < D; ++d) mu[d] = 0.0;
    double nb2 = b[0] * b[0];
    for (int d = 1; d < D; ++d) nb2 = nb2 + b[d] * b[d];
    if (!(nb2 > 0.0)) return;
    double H[9], U[9], m[3], g[3], Dl[3], zero[3] = {0.0, 0.0, 0.0};
    moment_hessian(a, i, cnt, zero, b, H, nullptr, nullptr, true);
    if (!moment_pivots_ok(D, H, U)) return;
    chol_solve<3>(D, U, b, m);
    for (int d = 0; d < D; ++d) m[d] = 2.0 * m[d];
    const double tol = 1.4901161193847656e-08;    // sqrt(eps)
    for (int it = 0; it < 30; ++it) {
        double phi;
        moment_hessian(a, i, cnt, m, b, H, g, &phi, false);
        double gg = g[0] * g[0];
        for (int d = 1; d < D; ++d) gg = gg + g[d] * g[d];
        if (gg <= (tol * tol) * nb2) {
            for (int d = 0; d < D; ++d) mu[d] = m[d];
            return;
        }
        if (!moment_pivots_ok(D, H, U)) return;
        chol_solve<3>(D, U, g, Dl);
        double gD = g[0] * Dl[0];
        for (int d = 1; d < D; ++d) gD = gD + g[d] * Dl[d];
        double lam = 1.0;
        for (int ls = 0; ls < 40; ++ls) {
            double mn[3];
            for (int d = 0; d < D; ++d) mn[d] = m[d] - lam * Dl[d];
            double t0 = b[0] * mn[0];
            for (int d = 1; d < D; ++d) t0 = t0 + b[d] * mn[d];
            double phin = -t0;
            for (int k = 0; k < cnt; ++k) {
                double t = (a.dist[(int64_t(k) * D) * a.npad + i] * a.invL) * mn[0];
                for (int d = 1; d < D; ++d) t = t + (a.dist[(int64_t(k) * D + d) * a.npad + i] * a.invL) * mn[d];
                if (t > 0.0) phin = phin + (t * t) / 2.0;
            }
            if (phin <= phi - (lam * gD) / 4.0) break;
            lam = lam / 2.0;
        }
        for (int d = 0; d < D; ++d) m[d] = m[d] - lam * Dl[d];
    }
}

// update_moment_weights! (MUSCL.jl:224-283): per axis d the first moment b = sum_k g^d_k x_k of the dissipation
// coefficients g^d_k = (dir_d > 0 ? c^d_k : -c^d_k) (dir: the signs of c for AlignedRusanovFlux, the offset
// otherwise), mu_d = _moment_mu(-b), e^d_k = (x_k . mu_d)_+, scaled down so that sum e <= sum |c| (_MOMENT_CAP 1).
__global__ void k_mweights(MlsArgs a) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int D = a.D, cnt = a.cnt[i];
    const int64_t np = a.npad;
    double mus[3][3];
    for (int d = 0; d < D; ++d) {
        double b[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < cnt; ++k) {
            const double c = a.dw[(int64_t(k) * D + d) * np + i];
            const double dir = a.aligned ? (c > 0.0 ? 1.0 : (c < 0.0 ? -1.0 : 0.0)) : a.dist[(int64_t(k) * D + d) * np + i];
            const double gcoef = dir > 0.0 ? c : -c;
            for (int e = 0; e < D; ++e) b[e] = b[e] + gcoef * (a.dist[(int64_t(k) * D + e) * np + i] * a.invL);
        }
        double nb[3];
        for (int e = 0; e < D; ++e) nb[e] = -b[e];
        moment_mu(a, i, cnt, nb, mus[d]);
    }
    double sum_e = 0.0, sum_g = 0.0;
    for (int k = 0; k < cnt; ++k) {
        double x[3];
        for (int e = 0; e < D; ++e) x[e] = a.dist[(int64_t(k) * D + e) * np + i] * a.invL;
        double se = 0.0, sg = 0.0;
        for (int d = 0; d < D; ++d) {
            double t = x[0] * mus[d][0];
            for (int e = 1; e < D; ++e) t = t + x[e] * mus[d][e];
            const double ep = t > 0.0 ? t : 0.0;
            se = d == 0 ? ep : se + ep;
            const double ag = fabs(a.dw[(int64_t(k) * D + d) * np + i]);
            sg = d == 0 ? ag : sg + ag;
        }
        sum_e = sum_e + se;
        sum_g = sum_g + sg;
    }
    const double scale = sum_e > sum_g ? sum_g / sum_e : 1.0;
    for (int k = 0; k < cnt; ++k) {
        double x[3];
        for (int e = 0; e < D; ++e) x[e] = a.dist[(int64_t(k) * D + e) * np + i] * a.invL;
        for (int d = 0; d < D; ++d) {
            double t = x[0] * mus[d][0];
            for (int e = 1; e < D; ++e) t = t + x[e] * mus[d][e];
            a.mw[(int64_t(k) * D + d) * np + i] = scale * (t > 0.0 ? t : 0.0);
        }
    }
}

// ---- outflow donor map
__global__ void k_donor_init(DonorArgs a, int tag, int first) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    a.status[i] = !a.bnd[i] ? 1 : (a.tags[i] == tag ? 0 : -1);
    if (first) a.root[i] = a.bnd[i] ? -1 : int32_t(i);
}

// _outflow_pass! (BoundaryConditions.jl:106-126), propagating the donor's root instead of its state. A particle
// resolved in this pass gets status pass+1, which no other particle accepts in the same pass.
__global__ void k_donor_pass(DonorArgs a, int pass) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n || a.status[i] != 0) return;
    int32_t closest = -1;
    double mind = INFINITY;
    const int cnt = a.cnt[i];
    for (int k = 0; k < cnt; ++k) {
        int32_t j = a.nidx[int64_t(k) * a.npad + i];
        int32_t sj = a.status[j];
        if (0 < sj && sj <= pass) {
            double d2 = 0.0;
            for (int d = 0; d < a.D; ++d) {
                double x = a.dist[(int64_t(k) * a.D + d) * a.npad + i];
                d2 = (d == 0) ? x * x : d2 + x * x;
            }
            if (d2 < mind) { mind = d2; closest = j; }
        }
    }
    if (closest != -1) {
        a.root[i] = a.root[closest];
        a.status[i] = pass + 1;
    }
}

inline unsigned grid_for(int64_t n, int bs = HCC_BLOCK) { return unsigned((n + bs - 1) / bs); }

}  // namespace

hcc_status mls_prepare(MlsArgs &a, cudaStream_t s, std::string &err) {
    std::call_once(g_tabs_once, upload_tables);
    if (g_tabs_err != cudaSuccess) { err = std::string("basis tables: ") + cudaGetErrorString(g_tabs_err); return HCC_ERR_CUDA; }
    if (a.n == 0) return HCC_OK;
    int need = a.weno_cfl_degree > 0 ? basis_count(a.D, a.weno_cfl_degree)
                                     : std::max(std::max(a.Bd, a.Br), a.D + 1);
    if (a.central_qmax > 0) need = std::max(need, basis_count(a.D, a.central_qmax) + 1);
    if (need > kMaxB) { err = "basis too large for the MLS kernel"; return HCC_ERR_UNSUPPORTED; }
    if (need <= 4) k_mls<4><<<grid_for(a.n, 128), 128, 0, s>>>(a);
    else if (need <= 10) k_mls<10><<<grid_for(a.n, 128), 128, 0, s>>>(a);
    else k_mls<kMaxB><<<grid_for(a.n, 64), 64, 0, s>>>(a);
    if (a.mw) k_mweights<<<grid_for(a.n, 128), 128, 0, s>>>(a);
    for (int q = 1; q <= a.central_qmax; ++q) {
        if (need <= 4) k_mls_central<4><<<grid_for(a.n, 128), 128, 0, s>>>(a, q);
        else if (need <= 10) k_mls_central<10><<<grid_for(a.n, 128), 128, 0, s>>>(a, q);
        else k_mls_central<kMaxB><<<grid_for(a.n, 64), 64, 0, s>>>(a, q);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = std::string("mls kernel: ") + cudaGetErrorString(e); return HCC_ERR_CUDA; }
    return HCC_OK;
}

hcc_status donor_map(DonorArgs &a, int tag, cudaStream_t s, std::string &err) {
    if (a.n == 0) return HCC_OK;
    // tag < 0: first call, roots of interior particles point at themselves, boundary roots are unresolved
    k_donor_init<<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a, tag, tag < 0 ? 1 : 0);
    if (tag >= 0)
        for (int pass = 1; pass <= 5; ++pass) k_donor_pass<<<grid_for(a.n), HCC_BLOCK, 0, s>>>(a, pass);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { err = std::string("donor map: ") + cudaGetErrorString(e); return HCC_ERR_CUDA; }
    return HCC_OK;
}

}  // namespace hcc
