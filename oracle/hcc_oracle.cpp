// hcc_oracle.cpp — TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// CPU restatement of HyperCloudCore.jl's explicit right-hand-side path. Every function names the reference
// file:line it follows. Arithmetic is written in the reference's evaluation order (left folds, no contraction:
// build with -ffp-contract=off), with these deliberate, documented deviations:
//   * Cholesky factor, inverse and triangular solves are the textbook row-oriented algorithms (StaticArrays'
//     unrolled order is not reproduced; parity with the reference is to tolerance there, as its own tests pin).
//   * Additions of an exact zero that only change the sign of a zero result (the zero non-conservative jump,
//     `0 + x` at the start of a contraction) are left out.
//   * Diagonal advection systems apply c[d][m] * U_m (the reference multiplies by the full diagonal matrix).
// The CUDA library computes the same sequence, so its FP64 results are compared bit for bit where stated.

#include "oracle.h"
#include <cmath>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <array>
#include <algorithm>
#include <memory>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- Julia float helpers
inline bool jisnan(double x) { return x != x; }
// Base.min / Base.max for IEEE floats: NaN-propagating, -0 < +0.
inline double jmin(double x, double y) {
    bool take_y = (y < x) || (std::signbit(y) && !std::signbit(x));
    return take_y ? (jisnan(x) ? x : y) : (jisnan(y) ? y : x);
}
inline double jmax(double x, double y) {
    bool take_y = (y > x) || (!std::signbit(y) && std::signbit(x));
    return take_y ? (jisnan(x) ? x : y) : (jisnan(y) ? y : x);
}
// Base.mod for floats (fmod with the sign of the divisor).
inline double jmod(double x, double y) {
    double r = std::fmod(x, y);
    if (r == 0.0) return std::copysign(r, y);
    if ((r > 0) != (y > 0)) return r + y;
    return r;
}

// ---------------------------------------------------------------- MLS basis (Interpolators.jl:121-247)
struct BasisTable {
    int D = 0, deg = 0, B = 0;
    std::vector<std::array<int, 3>> exps;
    std::vector<double> pref;      // 1/prod(t!) (only meaningful if has_pref)
    std::vector<int> has_pref;
};

int factorial(int n) { return n <= 1 ? 1 : n * factorial(n - 1); }

// _generate_exponents(D, max_order) (Interpolators.jl:138-155): per order, all tuples with that sum in
// Iterators.product order (first index fastest), sorted by (-maximum(t), reverse(t)).
std::vector<std::array<int, 3>> generate_exponents(int D, int max_order) {
    std::vector<std::array<int, 3>> res;
    for (int order = 1; order <= max_order; ++order) {
        std::vector<std::array<int, 3>> cur;
        int n = order + 1;
        int total = 1;
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
            if (-ma != -mb) return -ma < -mb;
            for (int d = D - 1; d >= 0; --d) {   // reverse(t), lexicographic
                if (a[d] != b[d]) return a[d] < b[d];
            }
            return false;
        });
        res.insert(res.end(), cur.begin(), cur.end());
    }
    return res;
}

// basis_count(D, degree) (Interpolators.jl:170-177)
int basis_count(int D, int degree) {
    if (degree <= 0) return 0;
    long n = 1;
    for (int k = 1; k <= degree; ++k) n = (n * (D + k)) / k;
    return int(n - 1);
}

const BasisTable &basis_table(int D, int deg) {
    static BasisTable tables[4][6];
    static bool init = false;
    if (!init) {
        for (int d = 1; d <= 3; ++d)
            for (int q = 0; q <= 5; ++q) {
                BasisTable &t = tables[d][q];
                t.D = d; t.deg = q;
                t.exps = generate_exponents(d, q);
                t.B = int(t.exps.size());
                for (auto &e : t.exps) {
                    int den = 1;
                    for (int i = 0; i < d; ++i) den *= factorial(e[i]);
                    t.pref.push_back(1.0 / double(den));
                    t.has_pref.push_back(den != 1);
                }
            }
        init = true;
    }
    return tables[D][deg];
}

inline double ipow(double x, int p) {   // Base.literal_pow for p = 2, 3
    if (p == 2) return x * x;
    if (p == 3) return x * x * x;
    double r = x;
    for (int i = 1; i < p; ++i) r = r * x;
    return r;
}

// build_basis(Val(IO), d) (Interpolators.jl:194-218)
void build_basis(const BasisTable &bt, const double *d, double *out) {
    for (int k = 0; k < bt.B; ++k) {
        bool have = bt.has_pref[k];
        double v = have ? bt.pref[k] : 0.0;
        for (int i = 0; i < bt.D; ++i) {
            int t = bt.exps[k][i];
            if (t == 0) continue;
            double f = (t == 1) ? d[i] : ipow(d[i], t);
            v = have ? v * f : f;
            have = true;
        }
        out[k] = v;
    }
}

// build_scale_factors (Interpolators.jl:236-247)
void build_scales(const BasisTable &bt, double invL, double *out) {
    for (int k = 0; k < bt.B; ++k) {
        int deg = 0;
        for (int i = 0; i < bt.D; ++i) deg += bt.exps[k][i];
        out[k] = (deg == 1) ? invL : ipow(invL, deg);
    }
}

// ---------------------------------------------------------------- Cholesky (Interpolators.jl:31-64)
const double kEps = std::numeric_limits<double>::epsilon();

// Upper factor U (row-major B×B) with U'U = A. Fails on a pivot that is not > 0.
bool cholesky_upper(int B, const double *A, double *U) {
    for (int i = 0; i < B * B; ++i) U[i] = 0.0;
    for (int i = 0; i < B; ++i) {
        for (int j = i; j < B; ++j) {
            double s = A[i * B + j];
            for (int k = 0; k < i; ++k) s = s - U[k * B + i] * U[k * B + j];
            if (i == j) {
                if (!(s > 0.0)) return false;
                U[i * B + i] = std::sqrt(s);
            } else {
                U[i * B + j] = s / U[i * B + i];
            }
        }
    }
    return true;
}

// _cholesky_moment: plain factorisation, pivot test U[k,k]^2 > 10 eps N[k,k], else retry with
// N + (sqrt(eps) tr(N) / B) I; ok = success of the retry.
bool cholesky_moment(int B, const double *N, double *U, bool *plain_ok = nullptr) {
    bool ok = cholesky_upper(B, N, U);
    if (ok) {
        const double tol = 10.0 * kEps;
        for (int k = 0; k < B; ++k) {
            double u = U[k * B + k];
            if (!(u * u > tol * N[k * B + k])) { ok = false; break; }
        }
    }
    if (plain_ok) *plain_ok = ok;
    if (ok) return true;
    double tr = 0.0;
    for (int k = 0; k < B; ++k) tr = tr + N[k * B + k];
    double eps_reg = std::sqrt(kEps) * tr / double(B);
    double A2[400];
    for (int i = 0; i < B * B; ++i) A2[i] = N[i];
    for (int k = 0; k < B; ++k) A2[k * B + k] = A2[k * B + k] + eps_reg;
    return cholesky_upper(B, A2, U);
}

// C \ b for C = U'U: forward substitution with U', then back substitution with U.
void chol_solve(int B, const double *U, const double *b, double *x) {
    double y[32];
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

// inv(C) column by column (C \ e_j).
void chol_inverse(int B, const double *U, double *Inv) {
    double e[32], x[32];
    for (int j = 0; j < B; ++j) {
        for (int r = 0; r < B; ++r) e[r] = (r == j) ? 1.0 : 0.0;
        chol_solve(B, U, e, x);
        for (int r = 0; r < B; ++r) Inv[r * B + j] = x[r];
    }
}

// ---------------------------------------------------------------- MUSCL degree rules (MUSCL.jl:11-32)
int div_idx(int D, int o) {
    if (o <= 2) return 2;
    return ((o % 2 == 1) && (D < 3 || o <= 3)) ? o + 1 : o;
}
int divergence_index(int DO, int D, int p_order, int num_nb) {
    int idx = (DO == 0) ? div_idx(D, p_order) : div_idx(D, DO);
    int base = std::max(2, DO == 0 ? p_order : DO);
    if (idx > base && 2 * num_nb < 3 * (basis_count(D, idx - 1) + 1)) idx = base;
    while (idx > 2 && num_nb < basis_count(D, idx - 1) + 1) idx -= 1;
    return idx;
}

// ---------------------------------------------------------------- tableaus (ButcherTableaus.jl)
struct Tableau {
    int s = 0;
    double a[5][5]{}, at[5][5]{}, c[5]{}, ct[5]{}, b[5]{}, bt[5]{};
};

Tableau make_tableau(int id) {
    Tableau t;
    auto set_explicit = [&](int s, std::initializer_list<double> A, std::initializer_list<double> b,
                            std::initializer_list<double> c) {
        t.s = s;
        int k = 0;
        for (double v : A) { t.at[k / s][k % s] = v; ++k; }
        k = 0; for (double v : b) t.bt[k++] = v;
        k = 0; for (double v : c) { t.c[k] = v; t.ct[k] = v; ++k; }
    };
    const double g2 = 1.0 - 1.0 / std::sqrt(2.0);
    switch (id) {
    case HCC_TAB_RK1_EULER: set_explicit(1, {0.0}, {1.0}, {0.0}); break;
    case HCC_TAB_RK2_SSP: set_explicit(2, {0, 0, 1.0, 0}, {1.0 / 2, 1.0 / 2}, {0.0, 1.0}); break;
    case HCC_TAB_RK2_RALSTON: set_explicit(2, {0, 0, 2.0 / 3, 0}, {1.0 / 4, 3.0 / 4}, {0.0, 2.0 / 3}); break;
    case HCC_TAB_RK3_SSP:
        set_explicit(3, {0, 0, 0, 1.0, 0, 0, 0.25, 0.25, 0}, {1.0 / 6, 1.0 / 6, 2.0 / 3}, {0.0, 1.0, 0.5});
        break;
    case HCC_TAB_RK4_CLASSICAL:
        set_explicit(4, {0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1.0, 0}, {1.0 / 6, 1.0 / 3, 1.0 / 3, 1.0 / 6},
                     {0.0, 0.5, 0.5, 1.0});
        break;
    case HCC_TAB_RK4_SSP:
        set_explicit(5,
                     {0, 0, 0, 0, 0,
                      0.39175222657189002, 0, 0, 0, 0,
                      0.21766909626116876, 0.36841059305037099, 0, 0, 0,
                      0.082692086657810582, 0.13995850219189535, 0.25189177427169401, 0, 0,
                      0.067966283637114752, 0.11503469850463156, 0.20703489859738566, 0.54497475022852104, 0},
                     {0.14681187608478657, 0.24848290944497617, 0.10425883033198098, 0.2744389009013507, 0.226007483236906},
                     {0.0, 0.39175222657189002, 0.58607968931153975, 0.47454236312139997, 0.93501063096765302});
        break;
    case HCC_TAB_IMEX_EULER:
        t.s = 2;
        t.at[1][0] = 1.0; t.a[1][1] = 1.0;
        t.c[0] = 0; t.c[1] = 1; t.ct[0] = 0; t.ct[1] = 1;
        t.b[0] = 0; t.b[1] = 1; t.bt[0] = 1; t.bt[1] = 0;
        break;
    case HCC_TAB_IMEX_ARS233: {
        double g = (3.0 + std::sqrt(3.0)) / 6.0;
        t.s = 3;
        t.a[1][1] = g; t.a[2][1] = 1.0 - 2 * g; t.a[2][2] = g;
        t.at[1][0] = g; t.at[2][0] = g - 1.0; t.at[2][1] = 2.0 * (1 - g);
        t.c[0] = 0; t.c[1] = g; t.c[2] = 1.0 - g;
        for (int i = 0; i < 3; ++i) t.ct[i] = t.c[i];
        t.b[0] = 0; t.b[1] = 0.5; t.b[2] = 0.5;
        for (int i = 0; i < 3; ++i) t.bt[i] = t.b[i];
        break;
    }
    case HCC_TAB_IMEX_ARS222: {
        double g = g2, dl = 1 - 1 / (2 * g);
        t.s = 3;
        t.a[1][1] = g; t.a[2][1] = 1 - g; t.a[2][2] = g;
        t.at[1][0] = g; t.at[2][0] = dl; t.at[2][1] = 1 - dl;
        t.c[0] = 0; t.c[1] = g; t.c[2] = 1;
        for (int i = 0; i < 3; ++i) t.ct[i] = t.c[i];
        t.b[0] = 0; t.b[1] = 1 - g; t.b[2] = g;
        t.bt[0] = dl; t.bt[1] = 1 - dl; t.bt[2] = 0;
        break;
    }
    case HCC_TAB_IMEX_PRSSP3: {
        double g = g2;
        t.s = 3;
        t.at[1][0] = 1; t.at[2][0] = 0.25; t.at[2][1] = 0.25;
        t.a[0][0] = g; t.a[1][0] = 1 - 2 * g; t.a[1][1] = g; t.a[2][0] = 0.5 - g; t.a[2][2] = g;
        t.b[0] = 1.0 / 6; t.b[1] = 1.0 / 6; t.b[2] = 2.0 / 3;
        for (int i = 0; i < 3; ++i) t.bt[i] = t.b[i];
        t.c[0] = g; t.c[1] = 1 - g; t.c[2] = 0.5;
        t.ct[0] = 0; t.ct[1] = 1; t.ct[2] = 0.5;
        break;
    }
    case HCC_TAB_IMEX_SSP2332:
        t.s = 3;
        t.a[0][0] = 0.25; t.a[1][1] = 0.25; t.a[2][0] = 1.0 / 3; t.a[2][1] = 1.0 / 3; t.a[2][2] = 1.0 / 3;
        t.at[1][0] = 0.5; t.at[2][0] = 0.5; t.at[2][1] = 0.5;
        t.b[0] = t.b[1] = t.b[2] = 1.0 / 3;
        for (int i = 0; i < 3; ++i) t.bt[i] = t.b[i];
        t.c[0] = 0.25; t.c[1] = 0.25; t.c[2] = 1.0;
        t.ct[0] = 0; t.ct[1] = 0.5; t.ct[2] = 1.0;
        break;
    default: t.s = 0;
    }
    return t;
}

bool tableau_has_implicit(const Tableau &t) {
    for (int i = 0; i < t.s; ++i)
        for (int j = 0; j < t.s; ++j)
            if (t.a[i][j] != 0.0) return true;
    for (int i = 0; i < t.s; ++i) if (t.b[i] != 0.0) return true;
    return false;
}

// _ssp_coefficient by bisection (ButcherTableaus.jl:104-118): alpha = rK (I + rK)^-1 >= -1e-13 and
// (I - alpha) 1 >= -1e-13. K is strictly lower triangular, so (I + rK)^-1 is a unit lower triangular
// forward substitution.
double ssp_coefficient(const Tableau &t) {
    for (int i = 0; i < t.s; ++i)
        for (int j = 0; j < t.s; ++j)
            if (t.a[i][j] != 0.0) return 0.0;
    const int s = t.s, n = s + 1;
    double K[6][6] = {};
    for (int i = 0; i < s; ++i) for (int j = 0; j < s; ++j) K[i][j] = t.at[i][j];
    for (int j = 0; j < s; ++j) K[s][j] = t.bt[j];
    auto ok = [&](double r) {
        double A[6][6], Inv[6][6], al[6][6];
        for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) A[i][j] = (i == j ? 1.0 : 0.0) + r * K[i][j];
        for (int j = 0; j < n; ++j) {           // columns of the inverse by forward substitution
            for (int i = 0; i < n; ++i) {
                double v = (i == j) ? 1.0 : 0.0;
                for (int k = 0; k < i; ++k) v -= A[i][k] * Inv[k][j];
                Inv[i][j] = v / A[i][i];
            }
        }
        double mn = 1e300;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double v = 0.0;
                for (int k = 0; k < n; ++k) v += r * K[i][k] * Inv[k][j];
                al[i][j] = v;
                mn = std::min(mn, v);
            }
        if (mn < -1e-13) return false;
        for (int i = 0; i < n; ++i) {
            double v = 0.0;
            for (int j = 0; j < n; ++j) v += ((i == j ? 1.0 : 0.0) - al[i][j]);
            if (v < -1e-13) return false;
        }
        return true;
    };
    double r_lo = 1e-3, r_hi = 1e-3;
    if (!ok(r_lo)) return 0.0;
    while (ok(r_hi) && r_hi < 1e3) r_hi *= 2;
    r_lo = r_hi / 2;
    for (int it = 0; it < 60; ++it) {
        double mid = (r_lo + r_hi) / 2;
        if (ok(mid)) r_lo = mid; else r_hi = mid;
    }
    return r_lo;
}

// ---------------------------------------------------------------- physics modules
// LinearAdvection (test/PDEs/linear_advection.jl:24-32), diagonal systems; Euler (new: ideal gas);
// BGK kinetic relaxation (test/kinetic_source.jl:37-104) = advection of the kinetic variables + source.
struct Physics {
    int kind = HCC_PDE_ADVECTION;
    int D = 2, M = 1;
    double c[3][HCC_MAX_VARS]{};
    double amax[3]{};
    double gamma = 1.4, gm1 = 0.4;
    // BGK
    double inv_eps = 0.0, coeff = 1.0, a_macro[3]{};
    double sinv[HCC_MAX_VARS][3]{};   // scaled_inv_speeds

    void init(const hcc_config &cfg) {
        kind = cfg.pde; D = cfg.dim; M = cfg.n_vars;
        for (int d = 0; d < D; ++d) {
            amax[d] = 0.0;
            for (int m = 0; m < M; ++m) {
                c[d][m] = cfg.velocity[d][m];
                amax[d] = std::max(amax[d], std::fabs(c[d][m]));
            }
        }
        gamma = cfg.gamma; gm1 = gamma - 1.0;
        if (kind == HCC_PDE_BGK) {
            inv_eps = 1.0 / cfg.bgk_epsilon;
            coeff = cfg.bgk_coefficient;
            double fac = cfg.bgk_interior_factor;
            for (int d = 0; d < D; ++d) a_macro[d] = cfg.bgk_macro_velocity[d];
            for (int k = 0; k < M; ++k)
                for (int d = 0; d < D; ++d) {
                    double v = cfg.velocity[d][k];
                    sinv[k][d] = std::fabs(v) > 1e-14 ? fac / v : 0.0;
                }
        }
    }
    // Euler primitive quantities: inv_rho = 1/rho, u_d = m_d inv_rho, p = (gamma-1)(E - 0.5 (rho |u|^2)).
    void euler_prim(const double *U, double &inv_rho, double *u, double &p) const {
        double rho = U[0];
        inv_rho = 1.0 / rho;
        double q2 = 0.0;
        for (int d = 0; d < D; ++d) {
            u[d] = U[1 + d] * inv_rho;
            q2 = (d == 0) ? u[d] * u[d] : q2 + u[d] * u[d];
        }
        p = gm1 * (U[D + 1] - 0.5 * (rho * q2));
    }
    // flux(eq, U) -> F[d*M + m]
    void flux(const double *U, double *F) const {
        if (kind == HCC_PDE_EULER) {
            double inv_rho, u[3], p;
            euler_prim(U, inv_rho, u, p);
            for (int d = 0; d < D; ++d) {
                double *Fd = F + d * M;
                Fd[0] = U[1 + d];
                for (int e = 0; e < D; ++e) {
                    double v = U[1 + e] * u[d];
                    Fd[1 + e] = (e == d) ? v + p : v;
                }
                Fd[D + 1] = (U[D + 1] + p) * u[d];
            }
        } else {
            for (int d = 0; d < D; ++d)
                for (int m = 0; m < M; ++m) F[d * M + m] = c[d][m] * U[m];
        }
    }
    // max_eigenvalue(eq, U, d)
    double lam(const double *U, int d) const {
        if (kind == HCC_PDE_EULER) {
            double inv_rho, u[3], p;
            euler_prim(U, inv_rho, u, p);
            return std::fabs(u[d]) + std::sqrt(gamma * p * inv_rho);
        }
        return amax[d];
    }
    // fluid_velocity (API.jl:104-109): scalar advection c_d (test/PDEs/linear_advection.jl:41-43); Euler m_d / rho
    // (a module of this implementation); no other system defines one.
    bool has_fluid_velocity() const { return kind == HCC_PDE_EULER || (kind == HCC_PDE_ADVECTION && M == 1); }
    void fluid_velocity(const double *U, double *w) const {
        for (int d = 0; d < D; ++d) w[d] = (kind == HCC_PDE_EULER) ? U[1 + d] / U[0] : c[d][0];
    }
    // max_eigenvalue(eq, U, d, shift) (API.jl:51-58): scalar advection |c_d - w_d| (linear_advection.jl:35), Euler
    // |u_d - w_d| + c, otherwise the default max_eigenvalue + |w_d|.
    double lam_shift(const double *U, int d, double w) const {
        if (kind == HCC_PDE_EULER) {
            double inv_rho, u[3], p;
            euler_prim(U, inv_rho, u, p);
            return std::fabs(u[d] - w) + std::sqrt(gamma * p * inv_rho);
        }
        if (kind == HCC_PDE_ADVECTION && M == 1) return std::fabs(c[d][0] - w);
        return amax[d] + std::fabs(w);
    }
    // flux(ALEFrame(eq, w), U) (GridMovers.jl:77-81): F_d - w_d U
    void flux_ale(const double *U, const double *w, double *F) const {
        flux(U, F);
        for (int d = 0; d < D; ++d)
            for (int m = 0; m < M; ++m) F[d * M + m] = F[d * M + m] - w[d] * U[m];
    }
    // is_admissible (API.jl:48): finite; Euler additionally rho > 0 and p > 0.
    bool admissible(const double *U) const {
        for (int m = 0; m < M; ++m) if (!std::isfinite(U[m])) return false;
        if (kind == HCC_PDE_EULER) {
            double inv_rho, u[3], p;
            euler_prim(U, inv_rho, u, p);
            return U[0] > 0.0 && p > 0.0;
        }
        return true;
    }
    bool has_implicit_source() const { return kind == HCC_PDE_BGK; }
    // Maxwellian of the single macro moment (kinetic_source.jl:67-104)
    void maxwellian(const double *U, double *Mk) const {
        double u = U[0];
        for (int k = 1; k < M; ++k) u = u + U[k];
        double F[3];
        for (int d = 0; d < D; ++d) F[d] = a_macro[d] * u;
        for (int k = 0; k < M; ++k) {
            double fd = F[0] * sinv[k][0];
            for (int d = 1; d < D; ++d) fd = fd + F[d] * sinv[k][d];
            Mk[k] = coeff * (u + fd);
        }
    }
    // evaluate_source (kinetic_source.jl:67-78)
    void source(const double *U, double *S) const {
        double Mk[HCC_MAX_VARS];
        maxwellian(U, Mk);
        for (int k = 0; k < M; ++k) S[k] = (Mk[k] - U[k]) * inv_eps;
    }
    // implicit_solve (kinetic_source.jl:80-104)
    void implicit_solve(const double *Y, double dt_coeff, double *out) const {
        double dto = dt_coeff * inv_eps;
        double denom = 1.0 / (1.0 + dto);
        double Mk[HCC_MAX_VARS];
        maxwellian(Y, Mk);
        for (int k = 0; k < M; ++k) out[k] = (Y[k] + dto * Mk[k]) * denom;
    }
};

// ---------------------------------------------------------------- the solver
struct Solver {
    hcc_config cfg{};
    int D = 2, M = 1;
    Physics phys;
    std::string err;

    // cloud
    int64_t N = 0;
    std::vector<double> pos;         // N*D
    std::vector<uint8_t> bnd;
    std::vector<int32_t> tags;
    std::vector<double> vol;

    // neighbours, row-major (host layout, NeighborLogic.jl:282)
    bool have_nb = false;
    std::vector<int64_t> start;      // N+1
    std::vector<int32_t> nidx;
    std::vector<double> nw, ndist;   // slots, slots*D
    int32_t max_nb = 0;

    // domain
    double R = 0, R_sq = 0, invR2 = 0, alpha = 1;
    double cmin[3]{}, cmax[3]{}, Lwrap[3]{}, invLwrap[3]{}, Lphys[3]{};
    int per[3]{};

    // scheme
    int max_order = 2, DO = 0, rdeg = 1, Br = 1, full_div = 2, ddeg = 1, Bd = 2;
    bool weno = false;
    bool central = false;            // CentralDivergence (Central.jl)
    int upwind = 0;                  // UpwindDivergence algorithm (Upwind.jl): 1 Tiwari, 2 Praveen
    int qmax = 1;                    // Central: highest divergence degree
    std::vector<double> dwc[3];      // Central: per-slot weights of the intercept fit of degree q = 1..qmax
    std::vector<uint8_t> okc[3];
    double invL = 1.0;
    bool streamed = true;
    bool aligned = false;            // AlignedRusanovFlux
    bool moment = false;             // MUSCL(...; moment_correction = true) of a first-order scheme
    std::vector<double> mw;          // its per-slot weights e^d_ij (slots * D)
    // moving grid (GridMovers.jl): mover kind, its parameters, positions as stage variables
    hcc_mover mover{};
    std::vector<double> x_n, x_cand, Xst[5], KX[5];
    bool moving() const { return mover.kind != HCC_MOVER_NONE; }
    bool have_geom = false;
    std::vector<double> inv_r, inv_d, dw;
    std::vector<uint8_t> ok_r, ok_d;

    // state
    std::vector<double> rhos;
    std::vector<int32_t> orders;
    std::vector<double> grads;       // N*Br*M

    // stepper
    Tableau tab;
    double ssp_C = 0.0, ratio = 0.0;
    std::vector<double> rho_n, rho_cand, rho_sub;
    std::vector<uint8_t> prelowered;   // pre-lowered particles of the next step (empty: none)
    std::vector<std::vector<double>> Y, KE, KI;
    std::vector<uint8_t> triggered, changed, dirty, scratch, trig_step;
    int64_t inadmissible = 0, mood_iters = 0, steps = 0;

    bool init(const hcc_config &c) {
        cfg = c;
        D = c.dim; M = c.n_vars;
        if (D < 1 || D > 3 || M < 1 || M > HCC_MAX_VARS) { err = "dim/n_vars out of range"; return false; }
        if (c.pde == HCC_PDE_EULER && M != D + 2) { err = "Euler needs n_vars = dim + 2"; return false; }
        phys.init(c);
        R = c.radius; alpha = c.weight_alpha;
        R_sq = R * R;
        invR2 = 1.0 / (R * R);
        for (int d = 0; d < D; ++d) {
            per[d] = c.periodic[d];
            cmin[d] = c.canvas_min[d]; cmax[d] = c.canvas_max[d];
            Lphys[d] = c.domain_max[d] - c.domain_min[d];
            Lwrap[d] = per[d] ? Lphys[d] : 0.0;
            invLwrap[d] = per[d] ? 1.0 / Lphys[d] : 0.0;
        }
        max_order = c.muscl_order;
        aligned = c.flux == HCC_FLUX_ALIGNED;
        moment = c.moment_correction != 0 && max_order == 1 && c.scheme == HCC_SCHEME_MUSCL;
        weno = c.scheme == HCC_SCHEME_WENO;
        central = c.scheme == HCC_SCHEME_CENTRAL;
        upwind = c.scheme == HCC_SCHEME_UPWIND ? c.upwind_algorithm : 0;
        if (c.scheme == HCC_SCHEME_UPWIND) {
            if (M != 1 || c.pde != HCC_PDE_ADVECTION) { err = "UpwindDivergence :Tiwari/:Praveen are scalar"; return false; }
            if (c.muscl_order != 1) { err = "UpwindDivergence is first order"; return false; }
            if (upwind != HCC_UPWIND_TIWARI && upwind != HCC_UPWIND_PRAVEEN) { err = "unknown upwind algorithm"; return false; }
            if (upwind == HCC_UPWIND_PRAVEEN && D != 2) { err = "Praveen is two-dimensional"; return false; }
        }
        if (max_order < 1 || max_order > 3) { err = "muscl_order must be 1..3"; return false; }
        DO = c.div_order > max_order ? max_order : c.div_order;
        qmax = DO == 0 ? max_order : DO;
        rdeg = std::max(1, max_order - 1);
        Br = basis_count(D, rdeg);
        full_div = div_idx(D, DO == 0 ? max_order : DO);
        ddeg = full_div - 1;
        Bd = basis_count(D, ddeg) + 1;
        double h = c.dx[0];
        for (int d = 1; d < D; ++d) h = std::min(h, c.dx[d]);
        invL = 1.0 / h;
        tab = make_tableau(c.tableau);
        if (tab.s == 0) { err = "unknown tableau"; return false; }
        if (phys.has_implicit_source() && !tableau_has_implicit(tab)) {
            // explicit tableau with implicit sources: the implicit part is the explicit one (TimeSteppers.jl:236-237)
            for (int i = 0; i < tab.s; ++i) {
                for (int j = 0; j < tab.s; ++j) tab.a[i][j] = tab.at[i][j];
                tab.c[i] = tab.ct[i]; tab.b[i] = tab.bt[i];
            }
        }
        ssp_C = ssp_coefficient(make_tableau(c.tableau));
        bool crit = c.mood_criterion != HCC_MOOD_NONE;
        ratio = (c.mood_substeps && ssp_C > 0) ? 1.0 / ssp_C : 0.0;
        if (!crit) ratio = 0.0;
        Y.assign(tab.s, {}); KE.assign(tab.s, {}); KI.assign(tab.s, {});
        return true;
    }

    const double *P(int64_t i) const { return &pos[i * D]; }

    // get_distance (ParticleGrids.jl:209-219)
    void distance(int64_t i, int64_t j, double *out) const {
        for (int d = 0; d < D; ++d) {
            double dx = pos[j * D + d] - pos[i * D + d];
            out[d] = dx - Lwrap[d] * std::nearbyint(dx * invLwrap[d]);
        }
    }
    double sumsq(const double *x) const {
        double s = x[0] * x[0];
        for (int d = 1; d < D; ++d) s = s + x[d] * x[d];
        return s;
    }
    // ExponentialWeightFunction (MLSWeightFunctions.jl:68-82)
    double weight(double d2) const {
        double arg = (-alpha) * d2 * invR2;
        double y = -arg;
        double den = 1.0 + y * (1.0 + y * (0.5 + y * (0.16666666666666666 + y * 0.041666666666666664)));
        return 1.0 / den;
    }

    // ------------------------------------------------------------ neighbour search (NeighborLogic.jl)
    // cell list of the whole cloud: bins, their 3^D windows, the particles of each bin
    int NOFF = 1;
    int64_t nbins = 1;
    std::vector<int64_t> binnb, bin_of, cstart, cellp;

    void build_bins() {
        // _wrap_position! (NeighborLogic.jl:279-286): periodic axes back into [min, min + L)
        for (int64_t i = 0; i < N; ++i)
            for (int d = 0; d < D; ++d)
                if (per[d]) pos[i * D + d] = cmin[d] + jmod(pos[i * D + d] - cmin[d], Lphys[d]);
        // GlobalBins (NeighborLogic.jl:22-40)
        int dims[3] = {1, 1, 1};
        double csize[3] = {1, 1, 1};
        nbins = 1;
        for (int d = 0; d < D; ++d) {
            double sz = cmax[d] - cmin[d];
            dims[d] = std::max(1, int(std::floor(sz / R)));
            csize[d] = sz / double(dims[d]);
            nbins *= dims[d];
        }
        NOFF = (D == 1) ? 3 : (D == 2 ? 9 : 27);
        binnb.assign(nbins * NOFF, 0);
        // _fill_bin_neighbors! (NeighborLogic.jl:43-76): window in CartesianIndices order (x offset fastest)
        for (int64_t b = 0; b < nbins; ++b) {
            int cart[3] = {0, 0, 0};
            int64_t r = b;
            for (int d = 0; d < D; ++d) { cart[d] = int(r % dims[d]); r /= dims[d]; }
            int64_t raw[27];
            for (int w = 0; w < NOFF; ++w) {
                int off[3] = {0, 0, 0};
                int q = w;
                for (int d = 0; d < D; ++d) { off[d] = q % 3 - 1; q /= 3; }
                bool valid = true;
                int64_t lin = 0, stride = 1;
                for (int d = 0; d < D; ++d) {
                    int nc = cart[d] + off[d];
                    if (nc < 0 || nc >= dims[d]) {
                        if (per[d]) nc = ((nc % dims[d]) + dims[d]) % dims[d];
                        else { valid = false; nc = 0; }
                    }
                    lin += nc * stride; stride *= dims[d];
                }
                raw[w] = valid ? lin : nbins;    // dummy bin
            }
            for (int w = 0; w < NOFF; ++w) {
                bool rep = false;
                for (int k = 0; k < w; ++k) if (raw[k] == raw[w]) rep = true;
                binnb[b * NOFF + w] = rep ? nbins : raw[w];
            }
        }
        // build_global_bins! (NeighborLogic.jl:116-136) with get_flat_bin_index (:86-102)
        bin_of.assign(N, 0);
        std::vector<int64_t> count(nbins + 1, 0);
        cstart.assign(nbins + 2, 0);
        for (int64_t i = 0; i < N; ++i) {
            int64_t lin = 0, stride = 1;
            for (int d = 0; d < D; ++d) {
                double f = std::floor((pos[i * D + d] - cmin[d]) / csize[d]);
                int64_t id = int64_t(f) + 1;
                id = std::min<int64_t>(std::max<int64_t>(id, 1), dims[d]);
                lin += (id - 1) * stride; stride *= dims[d];
            }
            bin_of[i] = lin;
            count[lin]++;
        }
        cstart[0] = 0;
        for (int64_t b = 0; b < nbins; ++b) cstart[b + 1] = cstart[b] + count[b];
        cstart[nbins + 1] = N;
        cellp.assign(N, 0);
        std::vector<int64_t> cursor(nbins, 0);
        for (int64_t i = 0; i < N; ++i) { int64_t b = bin_of[i]; cellp[cstart[b] + cursor[b]++] = i; }
        for (int64_t b = 0; b < nbins; ++b)   // _bin_sort! (NeighborLogic.jl:153-167): descending index within a bin
            std::sort(cellp.begin() + cstart[b], cellp.begin() + cstart[b + 1], std::greater<int64_t>());
    }

    // _count_neighbours! (NeighborLogic.jl:288-301) of particle i
    int64_t count_of(int64_t i) const {
        int64_t c = 0;
        double dist[3];
        for (int w = 0; w < NOFF; ++w) {
            int64_t b = binnb[bin_of[i] * NOFF + w];
            for (int64_t s = cstart[b]; s < cstart[b + 1]; ++s) {
                int64_t j = cellp[s];
                if (i != j) { distance(i, j, dist); if (sumsq(dist) <= R_sq) ++c; }
            }
        }
        return c;
    }

    // _write_neighbours! (NeighborLogic.jl:309-329) of particle i into idx/w/dist from slot 0; returns the count
    int64_t write_of(int64_t i, int32_t *idx, double *w, double *dst) const {
        int64_t k = 0;
        double dist[3];
        for (int wn = 0; wn < NOFF; ++wn) {
            int64_t b = binnb[bin_of[i] * NOFF + wn];
            for (int64_t s = cstart[b]; s < cstart[b + 1]; ++s) {
                int64_t j = cellp[s];
                if (i == j) continue;
                distance(i, j, dist);
                double d2 = sumsq(dist);
                if (d2 <= R_sq) {
                    idx[k] = int32_t(j);
                    w[k] = weight(d2);
                    for (int d = 0; d < D; ++d) dst[k * D + d] = dist[d];
                    ++k;
                }
            }
        }
        return k;
    }

    bool build_neighbours() {
        if (N == 0) { err = "no cloud"; return false; }
        build_bins();
        // pass 1: counts
        std::vector<int64_t> cnt(N, 0);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < N; ++i) cnt[i] = count_of(i);
        start.assign(N + 1, 0);
        max_nb = 0;
        for (int64_t i = 0; i < N; ++i) { start[i + 1] = start[i] + cnt[i]; max_nb = std::max<int32_t>(max_nb, int32_t(cnt[i])); }
        int64_t total = start[N];
        nidx.assign(total, 0); nw.assign(total, 0.0); ndist.assign(total * D, 0.0);
        // pass 2: write
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < N; ++i) write_of(i, &nidx[start[i]], &nw[start[i]], &ndist[start[i] * D]);
        have_nb = true;
        have_geom = false;
        return true;
    }

    int nnb(int64_t i) const { return int(start[i + 1] - start[i]); }

    // ------------------------------------------------------------ MLS caches (Interpolators.jl:517-577, MUSCL.jl:172-223)
    // _inverse_moment of degree q (intercept optional) into a B×B (padded to Bpad) matrix; returns ok.
    bool inverse_moment(int64_t i, int q, bool intercept, int Bpad, double *out) const {
        const BasisTable &bt = basis_table(D, q);
        int B = bt.B + (intercept ? 1 : 0);
        double Nm[400] = {0}, U[400], Inv[400], p[32], sd[3];
        for (int k = 0; k < B * B; ++k) Nm[k] = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
            if (intercept) { p[0] = 1.0; build_basis(bt, sd, p + 1); } else build_basis(bt, sd, p);
            double w = nw[s];
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) Nm[r * B + c] = Nm[r * B + c] + w * (p[r] * p[c]);
        }
        for (int k = 0; k < Bpad * Bpad; ++k) out[k] = 0.0;
        if (!cholesky_moment(B, Nm, U)) return false;
        chol_inverse(B, U, Inv);
        for (int r = 0; r < B; ++r) for (int c = 0; c < B; ++c) out[r * Bpad + c] = Inv[r * B + c];
        return true;
    }

    bool prepare_geometry() {
        if (!have_nb) { err = "neighbour lists missing"; return false; }
        inv_r.assign(N * Br * Br, 0.0); ok_r.assign(N, 0);
        inv_d.assign(N * Bd * Bd, 0.0); ok_d.assign(N, 0);
        dw.assign(nidx.size() * D, 0.0);
        const BasisTable &btd = basis_table(D, ddeg);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < N; ++i) {
            // update_weights!(grad_weights): full reconstruction degree, no intercept, every particle
            ok_r[i] = inverse_moment(i, rdeg, false, Br, &inv_r[i * Br * Br]);
            // update_weights!(div_weights, _FullOrderDivDegree): degree of the stencil at full order, padded
            int q = divergence_index(DO, D, max_order, nnb(i)) - 1;
            ok_d[i] = inverse_moment(i, q, true, Bd, &inv_d[i * Bd * Bd]);
            // _weights_body! (MUSCL.jl:211-223): (R (w p~)) invL with R the derivative rows 2..D+1
            double p[32], sd[3];
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                if (!ok_d[i]) { for (int d = 0; d < D; ++d) dw[s * D + d] = 0.0; continue; }
                for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                p[0] = 1.0; build_basis(btd, sd, p + 1);
                double w = nw[s];
                double v[32];
                for (int b = 0; b < Bd; ++b) v[b] = w * p[b];
                for (int d = 0; d < D; ++d) {
                    const double *row = &inv_d[i * Bd * Bd + (1 + d) * Bd];
                    double acc = row[0] * v[0];
                    for (int b = 1; b < Bd; ++b) acc = acc + row[b] * v[b];
                    dw[s * D + d] = acc * invL;
                }
            }
        }
        if (central) central_weights();
        if (moment) moment_weights();
        have_geom = true;
        return true;
    }

    // _moment_mu (MUSCL.jl:285-330): mu with sum_k (x_k . mu)_+ x_k = b over the scaled offsets x_k of particle i,
    // the minimiser of the convex Phi(mu) = 1/2 sum_k (x_k . mu)_+^2 - b . mu by Newton steps on the active slots
    // with Armijo backtracking; zero when b is zero, a Hessian fails the pivot test, or 30 steps do not converge.
    void moment_mu(int64_t i, const double *b, double *mu) const {
        for (int d = 0; d < D; ++d) mu[d] = 0.0;
        double nb2 = b[0] * b[0];
        for (int d = 1; d < D; ++d) nb2 = nb2 + b[d] * b[d];
        if (!(nb2 > 0.0)) return;
        auto hessian = [&](const double *m, double *H, double *g, double *phi, bool all) {
            for (int q = 0; q < D * D; ++q) H[q] = 0.0;
            if (g) for (int d = 0; d < D; ++d) g[d] = -b[d];
            if (phi) {
                double t = b[0] * m[0];
                for (int d = 1; d < D; ++d) t = t + b[d] * m[d];
                *phi = -t;
            }
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                double x[3];
                for (int d = 0; d < D; ++d) x[d] = ndist[s * D + d] * invL;
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
        };
        auto pivots_ok = [&](const double *H, double *Uc) {
            if (!cholesky_upper(D, H, Uc)) return false;
            for (int k = 0; k < D; ++k) {
                const double u = Uc[k * D + k];
                if (!(u * u > 10.0 * kEps * H[k * D + k])) return false;
            }
            return true;
        };
        double H[9], Uc[9], m[3], g[3], Dl[3], zero[3] = {0.0, 0.0, 0.0};
        hessian(zero, H, nullptr, nullptr, true);
        if (!pivots_ok(H, Uc)) return;
        chol_solve(D, Uc, b, m);
        for (int d = 0; d < D; ++d) m[d] = 2.0 * m[d];
        const double tol = std::sqrt(kEps);
        for (int it = 0; it < 30; ++it) {
            double phi;
            hessian(m, H, g, &phi, false);
            double gg = g[0] * g[0];
            for (int d = 1; d < D; ++d) gg = gg + g[d] * g[d];
            if (gg <= (tol * tol) * nb2) {
                for (int d = 0; d < D; ++d) mu[d] = m[d];
                return;
            }
            if (!pivots_ok(H, Uc)) return;
            chol_solve(D, Uc, g, Dl);
            double gD = g[0] * Dl[0];
            for (int d = 1; d < D; ++d) gD = gD + g[d] * Dl[d];
            double lam = 1.0;
            for (int ls = 0; ls < 40; ++ls) {
                double mn[3];
                for (int d = 0; d < D; ++d) mn[d] = m[d] - lam * Dl[d];
                double t0 = b[0] * mn[0];
                for (int d = 1; d < D; ++d) t0 = t0 + b[d] * mn[d];
                double phin = -t0;
                for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                    double t = (ndist[s * D] * invL) * mn[0];
                    for (int d = 1; d < D; ++d) t = t + (ndist[s * D + d] * invL) * mn[d];
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
    // otherwise), mu_d = _moment_mu(-b), e^d_k = (x_k . mu_d)_+; scaled down so that sum e <= sum |c| (_MOMENT_CAP 1).
    void moment_weights() {
        mw.assign(nidx.size() * D, 0.0);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < N; ++i) {
            double mus[3][3] = {};
            for (int d = 0; d < D; ++d) {
                double b[3] = {0.0, 0.0, 0.0};
                for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                    const double c = dw[s * D + d];
                    const double dir = aligned ? (c > 0.0 ? 1.0 : (c < 0.0 ? -1.0 : 0.0)) : ndist[s * D + d];
                    const double gcoef = dir > 0.0 ? c : -c;
                    for (int e = 0; e < D; ++e) b[e] = b[e] + gcoef * (ndist[s * D + e] * invL);
                }
                double nb[3];
                for (int e = 0; e < D; ++e) nb[e] = -b[e];
                moment_mu(i, nb, mus[d]);
            }
            double sum_e = 0.0, sum_g = 0.0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                double x[3];
                for (int e = 0; e < D; ++e) x[e] = ndist[s * D + e] * invL;
                double se = 0.0, sg = 0.0;
                for (int d = 0; d < D; ++d) {
                    double t = x[0] * mus[d][0];
                    for (int e = 1; e < D; ++e) t = t + x[e] * mus[d][e];
                    const double ep = t > 0.0 ? t : 0.0;
                    se = d == 0 ? ep : se + ep;
                    const double ag = std::fabs(dw[s * D + d]);
                    sg = d == 0 ? ag : sg + ag;
                }
                sum_e = sum_e + se;
                sum_g = sum_g + sg;
            }
            const double scale = sum_e > sum_g ? sum_g / sum_e : 1.0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                double x[3];
                for (int e = 0; e < D; ++e) x[e] = ndist[s * D + e] * invL;
                for (int d = 0; d < D; ++d) {
                    double t = x[0] * mus[d][0];
                    for (int e = 1; e < D; ++e) t = t + x[e] * mus[d][e];
                    mw[s * D + d] = scale * (t > 0.0 ? t : 0.0);
                }
            }
        }
    }

    // CentralDivergence (Central.jl:45-88) takes the intercept fit of degree q = the particle's (starved-lowered)
    // order, capped by div_order, of the flux differences F_j - F_i (compute_dynamic_divergence,
    // Interpolators.jl:290-334). Its per-slot weights for every q, as _slot_weight(::DynamicWeights)
    // (MUSCL.jl:442-445): C \ (w p~), rows 2..D+1, times invL; a particle uses degree q only if it has
    // basis_count(D, q) + 1 neighbours.
    void central_weights() {
        for (int q = 1; q <= qmax; ++q) {
            dwc[q - 1].assign(nidx.size() * D, 0.0);
            okc[q - 1].assign(N, 0);
            const BasisTable &bt = basis_table(D, q);
            const int B = bt.B + 1;
#pragma omp parallel for schedule(dynamic, 256)
            for (int64_t i = 0; i < N; ++i) {
                if (nnb(i) < B) continue;
                double Nm[400], Uc[400], p[32], sd[3], c[32];
                for (int k = 0; k < B * B; ++k) Nm[k] = 0.0;
                for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                    for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                    p[0] = 1.0; build_basis(bt, sd, p + 1);
                    const double w = nw[s];
                    for (int r = 0; r < B; ++r)
                        for (int cc = 0; cc < B; ++cc) Nm[r * B + cc] = Nm[r * B + cc] + w * (p[r] * p[cc]);
                }
                const bool ok = cholesky_moment(B, Nm, Uc);
                okc[q - 1][i] = ok;
                if (!ok) continue;
                for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                    for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                    p[0] = 1.0; build_basis(bt, sd, p + 1);
                    const double w = nw[s];
                    for (int b = 0; b < B; ++b) p[b] = w * p[b];
                    chol_solve(B, Uc, p, c);
                    for (int d = 0; d < D; ++d) dwc[q - 1][s * D + d] = c[d + 1] * invL;
                }
            }
        }
    }

    // The divergence of particle i (streamed: per-slot weights times the flux differences, slot by slot).
    void central_particle(int64_t i, const double *U, double *div) const {
        for (int m = 0; m < M; ++m) div[m] = 0.0;
        const int num = nnb(i);
        int p_order = orders[i];
        while (p_order > 1 && num < basis_count(D, p_order) + 1) --p_order;
        if (num < basis_count(D, p_order) + 1) return;
        const int q = DO == 0 ? p_order : std::min(DO, p_order);
        if (!okc[q - 1][i]) return;
        double Fi[3 * HCC_MAX_VARS], Fj[3 * HCC_MAX_VARS];
        phys.flux(&U[i * M], Fi);
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            phys.flux(&U[int64_t(nidx[s]) * M], Fj);
            for (int d = 0; d < D; ++d) {
                const double c = dwc[q - 1][s * D + d];
                for (int m = 0; m < M; ++m) div[m] = div[m] + c * (Fj[d * M + m] - Fi[d * M + m]);
            }
        }
    }

    // ------------------------------------------------------------ gather pass (MUSCL.jl:351-384)
    void gather_particle(int64_t i, const double *U) {
        const double *fi = &U[i * M];
        int num = nnb(i);
        int p_order = orders[i];
        while (p_order > 1 && num < basis_count(D, p_order - 1)) p_order -= 1;
        if (p_order < orders[i]) orders[i] = p_order;
        double *g = &grads[i * Br * M];
        for (int k = 0; k < Br * M; ++k) g[k] = 0.0;
        if (p_order == 1) return;                       // ConstantReconstruction
        double bs[32 * HCC_MAX_VARS], p[32], sd[3], df[HCC_MAX_VARS];
        if (p_order == max_order && ok_r[i]) {
            // apply_weights (Interpolators.jl:585-602)
            const BasisTable &bt = basis_table(D, rdeg);
            for (int k = 0; k < Br * M; ++k) bs[k] = 0.0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                int64_t j = nidx[s];
                for (int m = 0; m < M; ++m) df[m] = U[j * M + m] - fi[m];
                for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                build_basis(bt, sd, p);
                double w = nw[s];
                for (int b = 0; b < Br; ++b)
                    for (int m = 0; m < M; ++m) bs[b * M + m] = bs[b * M + m] + w * (p[b] * df[m]);
            }
            double sc[32];
            build_scales(bt, invL, sc);
            const double *inv = &inv_r[i * Br * Br];
            for (int b = 0; b < Br; ++b)
                for (int m = 0; m < M; ++m) {
                    double acc = inv[b * Br + 0] * bs[0 * M + m];
                    for (int c = 1; c < Br; ++c) acc = acc + inv[b * Br + c] * bs[c * M + m];
                    g[b * M + m] = acc * sc[b];
                }
            if (cfg.limiter != HCC_LIMITER_NONE) limit_slopes(i, U, g);
            return;
        }
        // dispatch_interpolator: Interpolator{D, p_order-1, 1} _mls_solve (Interpolators.jl:372-400), padded
        const BasisTable &bt = basis_table(D, p_order - 1);
        int B = bt.B;
        double Nm[400];
        for (int k = 0; k < B * B; ++k) Nm[k] = 0.0;
        for (int k = 0; k < B * M; ++k) bs[k] = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            int64_t j = nidx[s];
            for (int m = 0; m < M; ++m) df[m] = U[j * M + m] - fi[m];
            for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
            build_basis(bt, sd, p);
            double w = nw[s];
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) Nm[r * B + c] = Nm[r * B + c] + w * (p[r] * p[c]);
            for (int b = 0; b < B; ++b)
                for (int m = 0; m < M; ++m) bs[b * M + m] = bs[b * M + m] + w * (p[b] * df[m]);
        }
        double Uc[400];
        if (cholesky_moment(B, Nm, Uc)) {
            double sc[32] = {0}, col[32] = {0}, x[32] = {0};
            build_scales(bt, invL, sc);
            for (int m = 0; m < M; ++m) {
                for (int b = 0; b < B; ++b) col[b] = bs[b * M + m];
                chol_solve(B, Uc, col, x);
                for (int b = 0; b < B; ++b) g[b * M + m] = x[b] * sc[b];
            }
        }
        if (cfg.limiter != HCC_LIMITER_NONE) limit_slopes(i, U, g);
    }

    // ------------------------------------------------------------ MOOD interface orders (MOOD.jl:66-87)
    int nb_min_order(int64_t p) const {
        int o = orders[p];
        for (int64_t s = start[p]; s < start[p + 1]; ++s) o = std::min(o, (int)orders[nidx[s]]);
        return o;
    }
    void interface_orders(int64_t i, int64_t j, int &oi, int &oj) const {
        switch (cfg.mood_strategy) {
        case HCC_EPD1: { int o = std::min(orders[i], orders[j]); oi = oj = o; break; }
        case HCC_EPD2: { int o = std::min(nb_min_order(i), nb_min_order(j)); oi = oj = o; break; }
        default: oi = orders[i]; oj = orders[j];
        }
    }

    // mask_basis (Interpolators.jl:265-284)
    void mask_basis(double *p, int order) const {
        int max_spatial = rdeg + 1;
        int keep = (order >= 2 && order <= max_spatial) ? basis_count(D, order - 1) : 0;
        for (int b = keep; b < Br; ++b) p[b] = 0.0;
    }

    // ------------------------------------------------------------ slope limiters (Limiter.jl:35-143)
    // limiter_phi: Barth-Jespersen min(1, r); Venkatakrishnan (r^2 + 2r)/(r^2 + r + 2), its r > 1 branch
    // written in s = 1/r (Limiter.jl:37-46).
    double limiter_phi(double r) const {
        int lim = cfg.limiter;
        if (lim == HCC_LIMITER_BJ_SOFT || lim == HCC_LIMITER_BJ_HARD) return jmin(1.0, r);
        double rp = jmax(0.0, r);
        double sv = 1.0 / jmax(1.0, rp);
        double small = (rp * rp + 2.0 * rp) / (rp * rp + rp + 2.0);
        double large = (1.0 + 2.0 * sv) / (1.0 + sv + 2.0 * (sv * sv));
        return rp > 1.0 ? large : small;
    }
    // _limit_slopes for BJ / VK (Limiter.jl:120-143) with _local_extrema, _bounding_phi and _update_phi (:61-100).
    void limit_slopes(int64_t i, const double *U, double *g) const {
        const double *fi = &U[i * M];
        double umax[HCC_MAX_VARS], umin[HCC_MAX_VARS], phi[HCC_MAX_VARS];
        for (int m = 0; m < M; ++m) { umax[m] = umin[m] = fi[m]; phi[m] = 1.0; }
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            const double *rj = &U[int64_t(nidx[s]) * M];
            for (int m = 0; m < M; ++m) { umax[m] = jmax(umax[m], rj[m]); umin[m] = jmin(umin[m], rj[m]); }
        }
        const BasisTable &bt = basis_table(D, rdeg);
        const double tol16 = 16.0 * kEps;
        double p[32], hd[3];
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            for (int d = 0; d < D; ++d) hd[d] = 0.5 * ndist[s * D + d];
            build_basis(bt, hd, p);
            for (int m = 0; m < M; ++m) {
                double recon = g[0 * M + m] * p[0];
                for (int b = 1; b < Br; ++b) recon = recon + g[b * M + m] * p[b];
                double bound = recon > 0.0 ? umax[m] : umin[m];
                double tol = tol16 * jmax(std::fabs(fi[m]), std::fabs(bound));
                if (std::fabs(recon) > tol) {
                    double r = (bound - fi[m]) / recon;
                    phi[m] = jmin(phi[m], limiter_phi(r));
                }
            }
        }
        bool hard = cfg.limiter == HCC_LIMITER_BJ_HARD || cfg.limiter == HCC_LIMITER_VK_HARD;
        for (int b = 0; b < Br; ++b)
            if (hard || b < D)
                for (int m = 0; m < M; ++m) g[b * M + m] = g[b * M + m] * phi[m];
    }

    // ------------------------------------------------------------ flux pass (MUSCL.jl:390-508)
    // Returns the divergence (before the factor 2) in div[M].
    void flux_particle(int64_t i, const double *U, double *div) {
        for (int m = 0; m < M; ++m) div[m] = 0.0;
        int num = nnb(i);
        if (num == 0) return;
        int eff = orders[i];
        int didx = divergence_index(DO, D, eff, num);
        bool cached = ok_d[i] && didx == divergence_index(DO, D, max_order, num);
        const BasisTable &btr = basis_table(D, rdeg);
        const double *fi = &U[i * M];
        const double *gi = &grads[i * Br * M];
        double Fi[3 * HCC_MAX_VARS];
        // moving grid: the flux of particle i in the frame of its grid velocity (ALEFrame(eq, w_i))
        const bool ale = moving();
        double wv[3] = {0.0, 0.0, 0.0};
        if (ale) {
            grid_velocity(i, fi, wv);
            for (int d = 0; d < D; ++d) (*KX_cur)[i * D + d] = wv[d];
            phys.flux_ale(fi, wv, Fi);
        } else {
            phys.flux(fi, Fi);
        }

        // dynamic fit data (streamed dynamic: MUSCL.jl:514-538; buffered: Interpolators.jl:308-334)
        int qdyn = didx - 1;
        const BasisTable &btq = basis_table(D, qdyn);
        int Bq = btq.B + 1;
        double Ucd[400];
        bool dyn_ok = false;
        if (!cached) {
            double Nm[400];
            for (int k = 0; k < Bq * Bq; ++k) Nm[k] = 0.0;
            double p[32], sd[3];
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                p[0] = 1.0; build_basis(btq, sd, p + 1);
                double w = nw[s];
                for (int r = 0; r < Bq; ++r)
                    for (int c = 0; c < Bq; ++c) Nm[r * Bq + c] = Nm[r * Bq + c] + w * (p[r] * p[c]);
            }
            dyn_ok = cholesky_moment(Bq, Nm, Ucd);
            if ((streamed || aligned) && !dyn_ok) return;   // singular moment matrix: zero divergence
        }
        // the streamed form, and the aligned flux off the cached fit, contract per slot (MUSCL.jl:405-409)
        const bool per_slot = streamed || (aligned && !cached);
        // buffered: per-slot flux differences
        std::vector<double> buf;
        if (!streamed) buf.assign(size_t(num) * D * M, 0.0);

        double pi_[32], pj_[32], hd[3], fij[HCC_MAX_VARS], fji[HCC_MAX_VARS];
        double Fij[3 * HCC_MAX_VARS], Fji[3 * HCC_MAX_VARS], dF[3 * HCC_MAX_VARS];
        double sd_axis[3] = {0.0, 0.0, 0.0}, extra[HCC_MAX_VARS];
        for (int m = 0; m < M; ++m) extra[m] = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            const double *dk = &ndist[s * D];
            int64_t j = nidx[s];
            const double *fj = &U[j * M];
            const double *gj = &grads[j * Br * M];
            for (int d = 0; d < D; ++d) hd[d] = 0.5 * dk[d];
            build_basis(btr, hd, pi_);
            for (int d = 0; d < D; ++d) hd[d] = (-0.5) * dk[d];
            build_basis(btr, hd, pj_);
            int oi, oj;
            interface_orders(i, j, oi, oj);
            mask_basis(pi_, oi);
            mask_basis(pj_, oj);
            for (int m = 0; m < M; ++m) {
                double si = gi[0 * M + m] * pi_[0];
                double sj = gj[0 * M + m] * pj_[0];
                for (int b = 1; b < Br; ++b) {
                    si = si + gi[b * M + m] * pi_[b];
                    sj = sj + gj[b * M + m] * pj_[b];
                }
                fij[m] = fi[m] + si;
                fji[m] = fj[m] + sj;
            }
            if (ale) {
                phys.flux_ale(fij, wv, Fij);
                phys.flux_ale(fji, wv, Fji);
            } else {
                phys.flux(fij, Fij);
                phys.flux(fji, Fji);
            }
            // the slot's divergence weights c_ij (_slot_weight, MUSCL.jl:429-445): the cached fit, or the dynamic
            // fit solved per slot; the streamed contraction and the aligned orientation use them
            double wk[3] = {0.0, 0.0, 0.0};
            if (streamed || aligned) {
                if (cached) {
                    for (int d = 0; d < D; ++d) wk[d] = dw[s * D + d];
                } else {
                    // _slot_weight(::DynamicWeights) (MUSCL.jl:442-445): C \ (w p~), rows 2..D+1, times invL
                    double p[32], sd[3], c[32];
                    for (int d = 0; d < D; ++d) sd[d] = dk[d] * invL;
                    p[0] = 1.0; build_basis(btq, sd, p + 1);
                    double w = nw[s];
                    for (int b = 0; b < Bq; ++b) p[b] = w * p[b];
                    chol_solve(Bq, Ucd, p, c);
                    for (int d = 0; d < D; ++d) wk[d] = c[d + 1] * invL;
                }
            }
            // AlignedRusanovFlux (FluxFunctions.jl:103-111, MUSCL.jl:331-338): where either particle is below the
            // full order, or always at order 1, the states are sorted by the signs of c_ij instead of the distance
            const bool below = max_order == 1 || eff < max_order || orders[j] < max_order;
            const double *dir = (aligned && below) ? wk : dk;
            // sort_flux (Utils.jl:95-102) + RusanovFlux (FluxFunctions.jl:66-76)
            for (int d = 0; d < D; ++d) {
                bool pos_ = dir[d] > 0.0;
                const double *fL = pos_ ? fij : fji;
                const double *fR = pos_ ? fji : fij;
                const double *FL = pos_ ? &Fij[d * M] : &Fji[d * M];
                const double *FR = pos_ ? &Fji[d * M] : &Fij[d * M];
                double sdd = ale ? jmax(phys.lam_shift(fL, d, wv[d]), phys.lam_shift(fR, d, wv[d]))
                                 : jmax(phys.lam(fL, d), phys.lam(fR, d));
                sd_axis[d] = sdd;
                for (int m = 0; m < M; ++m) {
                    double Fn = 0.5 * ((FL[m] + FR[m]) - sdd * (fR[m] - fL[m]));
                    dF[d * M + m] = Fn - Fi[d * M + m];
                }
            }
            if (per_slot) {
                // _contract (MUSCL.jl:452-458)
                for (int m = 0; m < M; ++m) {
                    double t = wk[0] * dF[0 * M + m];
                    for (int d = 1; d < D; ++d) t = t + wk[d] * dF[d * M + m];
                    div[m] = div[m] + t;
                }
            } else {
                double *dst = &buf[size_t(s - start[i]) * D * M];
                for (int q = 0; q < D * M; ++q) dst[q] = dF[q];
            }
            if (moment) {
                // moment correction of a first-order scheme (MUSCL.jl:501-505): -1/2 sum_d s_d e^d_ij (f_ji - f_ij)
                double se = sd_axis[0] * mw[s * D + 0];
                for (int d = 1; d < D; ++d) se = se + sd_axis[d] * mw[s * D + d];
                const double corr = 0.5 * se;
                double *tgt = per_slot ? div : extra;
                for (int m = 0; m < M; ++m) tgt[m] = tgt[m] - corr * (fji[m] - fij[m]);
            }
        }
        if (per_slot) return;
        // buffered fits
        if (cached) {
            // apply_weights_divergence (Interpolators.jl:610-626)
            const BasisTable &btd = basis_table(D, ddeg);
            std::vector<double> bs(size_t(Bd) * D * M, 0.0);
            double p[32], sd[3];
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                p[0] = 1.0; build_basis(btd, sd, p + 1);
                double w = nw[s];
                const double *row = &buf[size_t(s - start[i]) * D * M];
                for (int b = 0; b < Bd; ++b)
                    for (int q = 0; q < D * M; ++q) bs[b * D * M + q] = bs[b * D * M + q] + w * (p[b] * row[q]);
            }
            const double *inv = &inv_d[i * Bd * Bd];
            for (int m = 0; m < M; ++m) {
                double acc = 0.0;
                for (int d = 0; d < D; ++d) {
                    int q = d * M + m;
                    double Rdq = inv[(1 + d) * Bd + 0] * bs[0 * D * M + q];
                    for (int b = 1; b < Bd; ++b) Rdq = Rdq + inv[(1 + d) * Bd + b] * bs[b * D * M + q];
                    acc = (d == 0) ? Rdq : acc + Rdq;
                }
                div[m] = acc * invL;
            }
        } else {
            // _mls_divergence of degree qdyn: R = (C \ E)' b_s
            if (!dyn_ok) return;
            std::vector<double> bs(size_t(Bq) * D * M, 0.0);
            double p[32], sd[3];
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
                p[0] = 1.0; build_basis(btq, sd, p + 1);
                double w = nw[s];
                const double *row = &buf[size_t(s - start[i]) * D * M];
                for (int b = 0; b < Bq; ++b)
                    for (int q = 0; q < D * M; ++q) bs[b * D * M + q] = bs[b * D * M + q] + w * (p[b] * row[q]);
            }
            double E[32], X[3][32];
            for (int d = 0; d < D; ++d) {
                for (int b = 0; b < Bq; ++b) E[b] = (b == d + 1) ? 1.0 : 0.0;
                chol_solve(Bq, Ucd, E, X[d]);
            }
            for (int m = 0; m < M; ++m) {
                double acc = 0.0;
                for (int d = 0; d < D; ++d) {
                    int q = d * M + m;
                    double Rdq = X[d][0] * bs[0 * D * M + q];
                    for (int b = 1; b < Bq; ++b) Rdq = Rdq + X[d][b] * bs[b * D * M + q];
                    acc = (d == 0) ? Rdq : acc + Rdq;
                }
                div[m] = acc * invL;
            }
        }
        if (moment)   // fit + extra (MUSCL.jl:420)
            for (int m = 0; m < M; ++m) div[m] = div[m] + extra[m];
    }

    // ------------------------------------------------------------ WENO (WENO.jl:55-165), scalar
    // Tiwari (Upwind.jl:158-202): per axis d the particles with v_d x_d <= 0 (the upwind side); the order lowered
    // while that stencil has fewer than basis_count(D, p) points (then the axis contributes 0); the gradient fit
    // of degree q (div_order cap) on it; the result is sum_d v_d (d_d u).
    double tiwari_particle(int64_t i, const double *U) const {
        const int num = nnb(i);
        std::vector<uint8_t> mask(num, 0);
        double total = 0.0;
        for (int d = 0; d < D; ++d) {
            const double vel = phys.c[d][0];
            int stencil = 0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                const bool in = vel * ndist[s * D + d] <= 0.0;
                mask[s - start[i]] = in;
                stencil += in;
            }
            int p_d = orders[i];
            while (p_d > 1 && stencil < basis_count(D, p_d)) --p_d;
            if (stencil < basis_count(D, p_d)) continue;
            const int q = DO == 0 ? p_d : std::min(DO, p_d);
            double res[32];
            masked_fit(i, U, q, mask, res);
            total = total + res[d] * vel;
        }
        return total;
    }

    // Praveen (Upwind.jl:205-249), 2-D, first order: the moment matrix N = sum w (x/L)(x/L)^T; per slot
    // c = N \ (w x / L) / L, the edge normal n = x / |x| and tangent s = (-n_y, n_x); the coefficient
    // (n . c) min(v . n, 0) + min((s . c)(v . s), 0) times u_j - u_i, summed, doubled.
    double praveen_particle(int64_t i, const double *U) const {
        const int num = nnb(i);
        if (num < 3) return 0.0;
        const double scale = std::min(cfg.dx[0], cfg.dx[1]);
        if (scale < 1e-14) return 0.0;
        const double iL = 1.0 / scale;
        const double vx = phys.c[0][0], vy = phys.c[1][0];
        double n11 = 0.0, n12 = 0.0, n22 = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            const double w = nw[s];
            const double x = ndist[s * 2] * iL, y = ndist[s * 2 + 1] * iL;
            n11 = n11 + w * (x * x);
            n12 = n12 + w * (x * y);
            n22 = n22 + w * (y * y);
        }
        const double det = n11 * n22 - n12 * n12;
        const double tr = n11 + n22;
        if (std::fabs(det) <= 4.0 * 2.220446049250313e-16 * (tr * tr)) return 0.0;
        const double fi = U[i];
        double div = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            const double w = nw[s];
            const double dx = ndist[s * 2], dy = ndist[s * 2 + 1];
            const double bx = w * dx * iL, by = w * dy * iL;
            const double cx = ((n22 * bx - n12 * by) / det) * iL;
            const double cy = ((n11 * by - n12 * bx) / det) * iL;
            const double hyp = std::sqrt(dx * dx + dy * dy);
            double nx = 1.0, ny = 0.0;
            if (!(hyp <= 2.220446049250313e-16 * scale)) { nx = dx / hyp; ny = dy / hyp; }
            const double sx = -ny, sy = nx;
            const double alfa = nx * cx + ny * cy;
            const double beta = sx * cx + sy * cy;
            const double vn = vx * nx + vy * ny;
            const double vs = vx * sx + vy * sy;
            const double bv = beta * vs;
            const double cij = alfa * (vn < 0.0 ? vn : 0.0) + (bv < 0.0 ? bv : 0.0);
            div = div + cij * (U[nidx[s]] - fi);
        }
        return 2.0 * div;
    }

    // _mls_solve_masked (Interpolators.jl:412-443) of degree q over the slots with mask[k] of a per-particle field
    // g(j) (fi = g(i)); out[0..B) scaled.
    template <typename G>
    bool masked_fit_field(int64_t i, G g, double fi, int q, const std::vector<uint8_t> &mask, double *out) const {
        const BasisTable &bt = basis_table(D, q);
        const int B = bt.B;
        double Nm[400], bs[32], p[32], sd[3];
        for (int k = 0; k < B * B; ++k) Nm[k] = 0.0;
        for (int b = 0; b < B; ++b) bs[b] = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            if (!mask[s - start[i]]) continue;
            for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
            build_basis(bt, sd, p);
            double w = nw[s];
            double df = g(int64_t(nidx[s])) - fi;
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) Nm[r * B + c] = Nm[r * B + c] + w * (p[r] * p[c]);
            for (int b = 0; b < B; ++b) bs[b] = bs[b] + w * (p[b] * df);
        }
        for (int b = 0; b < B; ++b) out[b] = 0.0;
        double Uc[400], x[32], sc[32];
        if (!cholesky_moment(B, Nm, Uc)) return false;
        chol_solve(B, Uc, bs, x);
        build_scales(bt, invL, sc);
        for (int b = 0; b < B; ++b) out[b] = x[b] * sc[b];
        return true;
    }
    bool masked_fit(int64_t i, const double *U, int q, const std::vector<uint8_t> &mask, double *out) const {
        return masked_fit_field(i, [U](int64_t j) { return U[j]; }, U[i], q, mask, out);
    }

    // Component-wise meshless WENO of a system (an extension of the scalar functor WENO.jl:55-165, which the reference
    // defines for M = 1 only): the central and one-sided fits, smoothness indicators and weights of the scalar scheme
    // applied to one field at a time.
    //  * linear fluxes F_d(U)_m = c_dm U_m (advection, the kinetic model): field U_m, upwind side by the sign of c_dm,
    //    the divergence sum_d c_dm d_d U_m -- for M = 1 the scalar scheme, operation for operation;
    //  * Euler: local Lax-Friedrichs splitting F_d = F_d^+ + F_d^-, F_d^+- = (F_d(U) +- alpha_d U) / 2 with alpha_d the
    //    largest lambda_d over {i} u N(i); d_d F_d^+ from the left-biased one-sided fit (x_d < 0), d_d F_d^- from the
    //    right-biased one (x_d >= 0), each blended with the central fit of the same field.
    void weno_system(int64_t i, const double *U, double *div) const {
        for (int m = 0; m < M; ++m) div[m] = 0.0;
        const int num = nnb(i);
        int p_order = orders[i];
        while (p_order > 1) {
            if (num >= basis_count(D, p_order)) break;
            p_order -= 1;
        }
        if (num < basis_count(D, p_order)) return;
        double hmin = cfg.dx[0];
        for (int d = 1; d < D; ++d) hmin = std::min(hmin, cfg.dx[d]);
        const double dx2 = hmin * hmin;
        const int qC = DO == 0 ? p_order : std::min(DO, p_order);
        std::vector<uint8_t> all(num, 1), side(num, 0);
        // one-sided stencil of axis d: x_d < 0 (left) or x_d >= 0; returns the fit degree, or 0 when too small
        auto one_sided = [&](int d, bool left) {
            int stencil = 0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                const double dk = ndist[s * D + d];
                const bool in = left ? dk < 0.0 : dk >= 0.0;
                side[s - start[i]] = in;
                stencil += in;
            }
            int p_d = p_order;
            while (p_d > 1) {
                if (stencil >= basis_count(D, p_d)) break;
                p_d -= 1;
            }
            if (stencil < basis_count(D, p_d)) return 0;
            return DO == 0 ? p_d : std::min(DO, p_d);
        };
        auto smooth = [&](const double *res) {
            double sm = (res[0] * res[0]) * dx2;
            for (int k = 1; k < D; ++k) sm = sm + (res[k] * res[k]) * dx2;
            return sm;
        };
        if (cfg.pde != HCC_PDE_EULER) {
            for (int m = 0; m < M; ++m) {
                auto g = [U, m, this](int64_t j) { return U[j * M + m]; };
                const double fi = U[i * M + m];
                double resC[32];
                masked_fit_field(i, g, fi, qC, all, resC);
                const double smoothC = smooth(resC);
                double s2 = jmax(fi * fi, smoothC);
                s2 = s2 > 0.0 ? s2 : 1.0;
                const double aC = smoothC / s2 + 1e-12;
                double div_total = 0.0;
                for (int d = 0; d < D; ++d) {
                    const double vel = phys.c[d][m];
                    const int qS = one_sided(d, vel > 0.0);
                    if (qS == 0) {
                        div_total = div_total + resC[d] * vel;
                        continue;
                    }
                    double resS[32];
                    masked_fit_field(i, g, fi, qS, side, resS);
                    const double smoothS = smooth(resS);
                    const double q = (smoothS / s2 + 1e-12) / aC;
                    const double wS = 1.0 / (1.0 + q * q);
                    const double wC = 1.0 - wS;
                    const double div_d = wS * resS[d] + wC * resC[d];
                    div_total = div_total + div_d * vel;
                }
                div[m] = div_total;
            }
            return;
        }
        double alpha[3];
        for (int d = 0; d < D; ++d) {
            alpha[d] = phys.lam(&U[i * M], d);
            for (int64_t s = start[i]; s < start[i + 1]; ++s) alpha[d] = jmax(alpha[d], phys.lam(&U[int64_t(nidx[s]) * M], d));
        }
        for (int d = 0; d < D; ++d)
            for (int sg = 0; sg < 2; ++sg) {
                const bool plus = sg == 0;
                const int qS = one_sided(d, plus);
                for (int m = 0; m < M; ++m) {
                    auto g = [&, d, m, plus](int64_t j) {
                        double F[3 * HCC_MAX_VARS];
                        phys.flux(&U[j * M], F);
                        const double aU = alpha[d] * U[j * M + m];
                        return plus ? 0.5 * (F[d * M + m] + aU) : 0.5 * (F[d * M + m] - aU);
                    };
                    const double fi = g(i);
                    double resC[32];
                    masked_fit_field(i, g, fi, qC, all, resC);
                    double deriv = resC[d];
                    if (qS > 0) {
                        const double smoothC = smooth(resC);
                        double s2 = jmax(fi * fi, smoothC);
                        s2 = s2 > 0.0 ? s2 : 1.0;
                        const double aC = smoothC / s2 + 1e-12;
                        double resS[32];
                        masked_fit_field(i, g, fi, qS, side, resS);
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

    double weno_particle(int64_t i, const double *U) const {
        const int num = nnb(i);
        int p_order = orders[i];
        while (p_order > 1) {
            if (num >= basis_count(D, p_order)) break;
            p_order -= 1;
        }
        if (num < basis_count(D, p_order)) return 0.0;
        const double fi = U[i];
        double hmin = cfg.dx[0];                         // scale_val = minimum(pg.meta.dx)
        for (int d = 1; d < D; ++d) hmin = std::min(hmin, cfg.dx[d]);
        const double dx2 = hmin * hmin;
        std::vector<uint8_t> mask(num, 1);
        double resC[32];
        int div_idx_C = DO == 0 ? p_order : std::min(DO, p_order);
        masked_fit(i, U, div_idx_C, mask, resC);
        double smoothC = (resC[0] * resC[0]) * dx2;
        for (int k = 1; k < D; ++k) smoothC = smoothC + (resC[k] * resC[k]) * dx2;
        double s2 = jmax(fi * fi, smoothC);
        s2 = s2 > 0.0 ? s2 : 1.0;
        const double aC = smoothC / s2 + 1e-12;
        double div_total = 0.0;
        for (int d = 0; d < D; ++d) {
            const double vel = phys.c[d][0];
            const bool use_left = vel > 0.0;
            int stencil = 0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                double dk = ndist[s * D + d];
                bool in = (use_left && dk < 0.0) || (!use_left && dk >= 0.0);
                mask[s - start[i]] = in;
                stencil += in;
            }
            int p_d = p_order;
            while (p_d > 1) {
                if (stencil >= basis_count(D, p_d)) break;
                p_d -= 1;
            }
            if (stencil < basis_count(D, p_d)) {
                div_total = div_total + resC[d] * vel;
                continue;
            }
            int div_idx_S = DO == 0 ? p_d : std::min(DO, p_d);
            double resS[32];
            masked_fit(i, U, div_idx_S, mask, resS);
            double smoothS = (resS[0] * resS[0]) * dx2;
            for (int k = 1; k < D; ++k) smoothS = smoothS + (resS[k] * resS[k]) * dx2;
            double q = (smoothS / s2 + 1e-12) / aC;
            double wS = 1.0 / (1.0 + q * q);
            double wC = 1.0 - wS;
            double div_d = wS * resS[d] + wC * resC[d];
            div_total = div_total + div_d * vel;
        }
        return div_total;
    }

    // _cfl_body! (ParticleGrids.jl:427-436) with _compute_cfl_coeffs (:296-329): the assembled Taylor fit of
    // degree `degree` per particle (schemes without cached per-slot weights, WENO).
    double cfl_sum_assembled(int64_t i, const double *Lambda_i, int degree) const {
        const BasisTable &bt = basis_table(D, degree);
        const int B = bt.B;
        double Nm[400], Uc[400], Inv[400], p[32], sd[3];
        for (int k = 0; k < B * B; ++k) Nm[k] = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
            build_basis(bt, sd, p);
            double w = nw[s];
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) Nm[r * B + c] = Nm[r * B + c] + w * (p[r] * p[c]);
        }
        if (!cholesky_moment(B, Nm, Uc)) return 0.0;
        chol_inverse(B, Uc, Inv);
        double sum_c = 0.0;
        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
            for (int d = 0; d < D; ++d) sd[d] = ndist[s * D + d] * invL;
            build_basis(bt, sd, p);
            double w = nw[s];
            const double *Uj = &rhos[int64_t(nidx[s]) * M];
            double dot = 0.0;
            for (int d = 0; d < D; ++d) {
                double cv = Inv[d * B + 0] * p[0];
                for (int jb = 1; jb < B; ++jb) cv = cv + Inv[d * B + jb] * p[jb];
                double c = std::fabs(cv * w * invL);
                double pr = c * jmax(Lambda_i[d], phys.lam(Uj, d));
                dot = (d == 0) ? pr : dot + pr;
            }
            sum_c = sum_c + dot;
        }
        return sum_c;
    }

    // grid_velocity (GridMovers.jl:60-63) of particle p at its current (stage) position
    void grid_velocity(int64_t p, const double *U, double *w) const {
        double r[3] = {0.0, 0.0, 0.0};
        switch (mover.kind) {
        case HCC_MOVER_LAGRANGIAN: phys.fluid_velocity(U, w); break;
        case HCC_MOVER_SCALED:
            phys.fluid_velocity(U, w);
            for (int d = 0; d < D; ++d) w[d] = mover.alpha * w[d];
            break;
        case HCC_MOVER_PRESCRIBED:
            for (int d = 0; d < D; ++d) r[d] = pos[p * D + d] - mover.center[d];
            if (D == 1) {
                w[0] = mover.velocity[0];
            } else if (D == 2) {
                w[0] = mover.velocity[0] - mover.omega[2] * r[1];
                w[1] = mover.velocity[1] + mover.omega[2] * r[0];
            } else {
                w[0] = mover.velocity[0] + (mover.omega[1] * r[2] - mover.omega[2] * r[1]);
                w[1] = mover.velocity[1] + (mover.omega[2] * r[0] - mover.omega[0] * r[2]);
                w[2] = mover.velocity[2] + (mover.omega[0] * r[1] - mover.omega[1] * r[0]);
            }
            break;
        default: for (int d = 0; d < D; ++d) w[d] = 0.0;
        }
    }

    // refresh_geometry! (GridMovers.jl:95-121): distances and weights of the existing slots at the current positions,
    // weight 0 beyond R
    void refresh_geometry() {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < N; ++i)
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                double dist[3];
                distance(i, nidx[s], dist);
                for (int d = 0; d < D; ++d) ndist[s * D + d] = dist[d];
                double d2 = sumsq(dist);
                nw[s] = d2 <= R_sq ? weight(d2) : 0.0;
            }
    }

    // compute_explicit_rhs! (TimeSteppers.jl:312-356); on a moving grid K_X = w and the flux in the ALE frame
    std::vector<double> *KX_cur = nullptr;
    void compute_rhs(std::vector<double> &K, const double *Ystate, bool full) {
        if (upwind) {
#pragma omp parallel for schedule(dynamic, 256)
            for (int64_t p = 0; p < N; ++p) {
                if (bnd[p]) { if (full) K[p] = 0.0; continue; }
                if (!(full || dirty[p])) continue;
                K[p] = -(upwind == HCC_UPWIND_TIWARI ? tiwari_particle(p, Ystate) : praveen_particle(p, Ystate));
            }
            return;
        }
        if (central) {
#pragma omp parallel for schedule(dynamic, 256)
            for (int64_t p = 0; p < N; ++p) {
                if (bnd[p]) { if (full) for (int m = 0; m < M; ++m) K[p * M + m] = 0.0; continue; }
                if (!(full || dirty[p])) continue;
                double div[HCC_MAX_VARS];
                central_particle(p, Ystate, div);
                for (int m = 0; m < M; ++m) K[p * M + m] = -div[m];
            }
            return;
        }
        if (weno) {
#pragma omp parallel for schedule(dynamic, 256)
            for (int64_t p = 0; p < N; ++p) {
                if (bnd[p]) { if (full) for (int m = 0; m < M; ++m) K[p * M + m] = 0.0; continue; }
                if (!(full || dirty[p])) continue;
                if (M == 1 && cfg.pde != HCC_PDE_EULER) {
                    K[p] = -weno_particle(p, Ystate);
                } else {
                    double div[HCC_MAX_VARS];
                    weno_system(p, Ystate, div);
                    for (int m = 0; m < M; ++m) K[p * M + m] = -div[m];
                }
            }
            return;
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t p = 0; p < N; ++p) {
            if (bnd[p] || !(full || changed[p])) continue;
            gather_particle(p, Ystate);
        }
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t p = 0; p < N; ++p) {
            if (bnd[p]) {
                if (full) {
                    for (int m = 0; m < M; ++m) K[p * M + m] = 0.0;
                    if (moving()) for (int d = 0; d < D; ++d) (*KX_cur)[p * D + d] = 0.0;
                }
                continue;
            }
            if (!(full || dirty[p])) continue;
            double div[HCC_MAX_VARS];
            flux_particle(p, Ystate, div);
            for (int m = 0; m < M; ++m) K[p * M + m] = -(2.0 * div[m]);
        }
    }

    // ------------------------------------------------------------ boundary conditions (BoundaryConditions.jl)
    void apply_bcs(double *buf) {
        for (int tag = 1; tag <= HCC_MAX_TAGS; ++tag) {
            int kind = cfg.bc_by_tag[tag - 1];
            if (kind == HCC_BC_DIRICHLET) {
                for (int64_t i = 0; i < N; ++i)
                    if (bnd[i] && tags[i] == tag)
                        for (int m = 0; m < M; ++m) buf[i * M + m] = rhos[i * M + m];
            } else if (kind == HCC_BC_OUTFLOW) {
                std::vector<int32_t> status(N);
                for (int64_t i = 0; i < N; ++i) status[i] = !bnd[i] ? 1 : (tags[i] == tag ? 0 : -1);
                for (int pass = 1; pass <= 5; ++pass) {
                    std::vector<int32_t> st0 = status;   // per-particle writes read only earlier passes
                    for (int64_t i = 0; i < N; ++i) {
                        if (st0[i] != 0) continue;
                        int64_t closest = -1;
                        double mind = std::numeric_limits<double>::infinity();
                        for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                            int64_t j = nidx[s];
                            int32_t sj = st0[j];
                            if (0 < sj && sj <= pass) {
                                double d2 = sumsq(&ndist[s * D]);
                                if (d2 < mind) { mind = d2; closest = j; }
                            }
                        }
                        if (closest != -1) {
                            for (int m = 0; m < M; ++m) buf[i * M + m] = buf[closest * M + m];
                            status[i] = pass + 1;
                        }
                    }
                    bool any0 = false;
                    for (int64_t i = 0; i < N; ++i) if (status[i] == 0) { any0 = true; break; }
                    if (!any0) break;
                }
                for (int64_t i = 0; i < N; ++i)
                    if (status[i] == 0) for (int m = 0; m < M; ++m) buf[i * M + m] = rhos[i * M + m];
            }
        }
    }

    // ------------------------------------------------------------ stage assembly (TimeSteppers.jl:365-444)
    std::vector<double> &form_candidate(int i, double dt) {   // i: 1-based stage, s+1 = final
        const int s = tab.s;
        bool fin = i > s;
        std::vector<double> &target = fin ? rho_cand : Y[i - 1];
        int n_prev = fin ? s : i - 1;
        const bool mv = moving();
        std::vector<double> *xt = mv ? (fin ? &x_cand : &Xst[i - 1]) : nullptr;
        for (int64_t p = 0; p < N; ++p) {
            double *Yp = &target[p * M];
            if (bnd[p]) {
                for (int m = 0; m < M; ++m) Yp[m] = rhos[p * M + m];
                if (mv) for (int d = 0; d < D; ++d) (*xt)[p * D + d] = x_n[p * D + d];
                continue;
            }
            for (int m = 0; m < M; ++m) Yp[m] = rho_n[p * M + m];
            double *Xp = mv ? &(*xt)[p * D] : nullptr;
            if (mv) for (int d = 0; d < D; ++d) Xp[d] = x_n[p * D + d];
            for (int j = 1; j <= n_prev; ++j) {
                double a_t = fin ? tab.bt[j - 1] : tab.at[i - 1][j - 1];
                double a = fin ? tab.b[j - 1] : tab.a[i - 1][j - 1];
                if (a_t != 0.0) {
                    double h = dt * a_t;
                    for (int m = 0; m < M; ++m) Yp[m] = Yp[m] + h * KE[j - 1][p * M + m];
                    if (mv) for (int d = 0; d < D; ++d) Xp[d] = Xp[d] + h * KX[j - 1][p * D + d];
                }
                if (a != 0.0 && phys.has_implicit_source()) {
                    double h = dt * a;
                    for (int m = 0; m < M; ++m) Yp[m] = Yp[m] + h * KI[j - 1][p * M + m];
                }
            }
        }
        if (!fin && phys.has_implicit_source()) {
            double a_ii = tab.a[i - 1][i - 1];
            std::vector<double> &KIi = KI[i - 1];
            if (std::fabs(a_ii) > 1e-14) {
                double dt_ii = dt * a_ii, inv_dt_ii = 1.0 / (dt * a_ii);
                for (int64_t p = 0; p < N; ++p) {
                    if (bnd[p]) { for (int m = 0; m < M; ++m) KIi[p * M + m] = 0.0; continue; }
                    double out[HCC_MAX_VARS];
                    phys.implicit_solve(&target[p * M], dt_ii, out);
                    for (int m = 0; m < M; ++m) {
                        KIi[p * M + m] = (out[m] - target[p * M + m]) * inv_dt_ii;
                        target[p * M + m] = out[m];
                    }
                }
            } else {
                for (int64_t p = 0; p < N; ++p) {
                    if (bnd[p]) { for (int m = 0; m < M; ++m) KIi[p * M + m] = 0.0; continue; }
                    phys.source(&target[p * M], &KIi[p * M]);
                }
            }
        }
        apply_bcs(target.data());
        return target;
    }

    std::vector<double> &form_substep(int i, double dt) {
        double h = ratio * dt;
        bool withKI = phys.has_implicit_source();
        const std::vector<double> &Yp = Y[i - 2], &K = KE[i - 2], &Ki = KI[i - 2];
        for (int64_t p = 0; p < N; ++p) {
            for (int m = 0; m < M; ++m) {
                int64_t q = p * M + m;
                if (bnd[p]) rho_sub[q] = Yp[q];
                else rho_sub[q] = withKI ? Yp[q] + h * (K[q] + Ki[q]) : Yp[q] + h * K[q];
            }
        }
        return rho_sub;
    }

    // ------------------------------------------------------------ MOOD (MOOD.jl:151-405)
    bool criterion_flags(int64_t p, const double *prev, const double *cand) const {
        switch (cfg.mood_criterion) {
        case HCC_MOOD_ONLY: return true;
        case HCC_MOOD_PAD: return false;
        case HCC_MOOD_U1: {
            double dlt = cfg.mood_delta;
            double mn[HCC_MAX_VARS], mx[HCC_MAX_VARS];
            for (int m = 0; m < M; ++m) mn[m] = mx[m] = prev[p * M + m];
            for (int64_t s = start[p]; s < start[p + 1]; ++s) {
                const double *rj = &prev[int64_t(nidx[s]) * M];
                for (int m = 0; m < M; ++m) { mn[m] = jmin(mn[m], rj[m]); mx[m] = jmax(mx[m], rj[m]); }
            }
            double d3 = dlt * dlt * dlt;
            const double *nr = &cand[p * M];
            for (int m = 0; m < M; ++m)
                if (std::fabs(mx[m] - mn[m]) >= d3 && (nr[m] < mn[m] - dlt || nr[m] > mx[m] + dlt)) return true;
            return false;
        }
        case HCC_MOOD_U2: return u2_fails(p, prev, &cand[p * M]);
        default: return false;
        }
    }

    // _global_range(::MOODu2, U, N) (MOOD.jl:215-221): max - min per component over all particles of the stage
    // state, NaN-propagating; empty when the plateau test is off.
    std::vector<double> u2_range;
    void global_range(const double *prev) {
        u2_range.clear();
        if (!(cfg.mood_criterion == HCC_MOOD_U2 && cfg.u2_plateau > 0.0) || N == 0) return;
        std::vector<double> lo(prev, prev + M), hi(prev, prev + M);
        for (int64_t p = 1; p < N; ++p)
            for (int m = 0; m < M; ++m) {
                lo[m] = jmin(lo[m], prev[p * M + m]);
                hi[m] = jmax(hi[m], prev[p * M + m]);
            }
        u2_range.resize(M);
        for (int m = 0; m < M; ++m) u2_range[m] = hi[m] - lo[m];
    }

    // _u2_fails (MOOD.jl:223-271): the DMP-violating components that are not a plateau; below order 3 (no curvature
    // terms) any such component flags; otherwise per axis the curvature terms of the cached reconstruction over
    // {p} ∪ N(p) must keep one sign and, over the neighbours within 1.5h, comparable magnitudes.
    bool u2_fails(int64_t p, const double *prev, const double *nr) const {
        const double dlt = cfg.mood_delta, d3 = dlt * dlt * dlt;
        double mn[HCC_MAX_VARS], mx[HCC_MAX_VARS];
        for (int m = 0; m < M; ++m) mn[m] = mx[m] = prev[p * M + m];
        for (int64_t s = start[p]; s < start[p + 1]; ++s) {
            const double *rj = &prev[int64_t(nidx[s]) * M];
            for (int m = 0; m < M; ++m) { mn[m] = jmin(mn[m], rj[m]); mx[m] = jmax(mx[m], rj[m]); }
        }
        bool viol[HCC_MAX_VARS], any = false;
        for (int m = 0; m < M; ++m) {
            viol[m] = std::fabs(mx[m] - mn[m]) >= d3 && (nr[m] < mn[m] - dlt || nr[m] > mx[m] + dlt) &&
                      !(!u2_range.empty() && mx[m] - mn[m] < cfg.u2_plateau * u2_range[m]);
            any = any || viol[m];
        }
        if (!any) return false;
        if (max_order < 3 || orders[p] < 3) return true;
        double h = cfg.dx[0];
        for (int d = 1; d < D; ++d) h = std::min(h, cfg.dx[d]);
        const double h2 = h * h, near_sq = (1.5 * h) * (1.5 * h);
        for (int d = 0; d < D; ++d) {
            const int b = D + d;                                    // curvature term of axis d
            const double *ci = &grads[(size_t(p) * Br + b) * M];
            double mini[HCC_MAX_VARS], maxi[HCC_MAX_VARS], minA[HCC_MAX_VARS], maxA[HCC_MAX_VARS];
            for (int m = 0; m < M; ++m) { mini[m] = maxi[m] = ci[m]; minA[m] = maxA[m] = std::fabs(ci[m]); }
            for (int64_t s = start[p]; s < start[p + 1]; ++s) {
                const double *cj = &grads[(size_t(nidx[s]) * Br + b) * M];
                double r2 = 0.0;
                for (int e = 0; e < D; ++e) r2 = (e == 0) ? ndist[s * D] * ndist[s * D] : r2 + ndist[s * D + e] * ndist[s * D + e];
                const bool near = r2 <= near_sq;
                for (int m = 0; m < M; ++m) {
                    mini[m] = jmin(mini[m], cj[m]);
                    maxi[m] = jmax(maxi[m], cj[m]);
                    if (near) { minA[m] = jmin(minA[m], std::fabs(cj[m])); maxA[m] = jmax(maxA[m], std::fabs(cj[m])); }
                }
            }
            for (int m = 0; m < M; ++m) {
                if (!viol[m]) continue;
                if (jmax(std::fabs(mini[m]), std::fabs(maxi[m])) * h2 < dlt) continue;   // negligible curvature
                const bool same_sign = (mini[m] * h2) * (maxi[m] * h2) > -(dlt * dlt);
                const bool comparable = cfg.u2_ratio <= 0.0 || minA[m] >= cfg.u2_ratio * maxA[m];
                if (!(same_sign && comparable)) return true;
            }
        }
        return false;
    }

    bool detect_and_drop(const double *prev, const double *cand, bool full, bool with_eq) {
        if (cfg.mood_criterion == HCC_MOOD_NONE) return false;
        global_range(prev);
        std::fill(triggered.begin(), triggered.end(), 0);
        std::fill(changed.begin(), changed.end(), 0);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t p = 0; p < N; ++p) {
            if (bnd[p] || !(full || dirty[p])) continue;
            bool pad_fail = with_eq && !phys.admissible(&cand[p * M]);
            if (pad_fail || criterion_flags(p, prev, cand)) triggered[p] = 1;
        }
        bool any = false;
        for (int64_t p = 0; p < N; ++p) {
            if (!triggered[p]) continue;
            if (orders[p] > 1) { orders[p] -= 1; changed[p] = 1; trig_step[p] = 1; any = true; }
            else triggered[p] = 0;
        }
        if (!any || cfg.mood_strategy != HCC_STRICT_EPD0) return any;
        // StrictEPD0 forcing from the post-decrement snapshot (forced_order(::Halo{1}), MOOD.jl:54-64; _mood_force!,
        // :312-320): each interior particle takes the lowest order of its dropped neighbours, without cascade
        std::vector<int32_t> snap = orders;
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t j = 0; j < N; ++j) {
            if (bnd[j]) continue;
            int32_t o = snap[j];
            for (int64_t s = start[j]; s < start[j + 1]; ++s) {
                const int64_t p = nidx[s];
                if (triggered[p]) o = std::min(o, snap[p]);
            }
            if (o < snap[j]) { orders[j] = o; changed[j] = 1; }
        }
        return any;
    }

    void expand_mask(std::vector<uint8_t> &mask, int hops) {
        for (int h = 0; h < hops; ++h) {
#pragma omp parallel for schedule(static)
            for (int64_t j = 0; j < N; ++j) {
                uint8_t m = mask[j];
                if (!m)
                    for (int64_t s = start[j]; s < start[j + 1]; ++s)
                        if (mask[nidx[s]]) { m = 1; break; }
                scratch[j] = m;
            }
            for (int64_t j = 0; j < N; ++j) mask[j] = scratch[j];
        }
    }

    // _order_reach (MUSCL_hooks.jl:10-11; API.jl:250 default 0 for schemes that read no neighbour orders: WENO)
    int order_reach() const { return (weno || central || upwind) ? 0 : (cfg.mood_strategy == HCC_EPD2 ? 2 : 1); }

    bool mood_checkpoint(int i, double dt) {
        const std::vector<double> &Yprev = Y[i - 2];
        bool full = true;
        int cap = cfg.max_mood_iterations > 0 ? cfg.max_mood_iterations : 64;
        for (int it = 0;; ++it) {
            std::vector<double> &target = form_candidate(i, dt);
            const std::vector<double> &cand = (ratio > 0.0 && cfg.mood_criterion != HCC_MOOD_NONE) ? form_substep(i, dt) : target;
            if (!detect_and_drop(Yprev.data(), cand.data(), full, true)) {
                if (cfg.mood_criterion != HCC_MOOD_NONE)
                    for (int64_t p = 0; p < N; ++p)
                        if (!bnd[p] && !phys.admissible(&cand[p * M])) ++inadmissible;
                return true;
            }
            if (it >= cap) { err = "MOOD fixed point did not converge"; return false; }
            dirty = changed;
            expand_mask(dirty, order_reach());
            compute_rhs(KE[i - 2], Yprev.data(), false);
            full = false;
            ++mood_iters;
        }
    }

    void size_buffers() {
        rho_n.assign(N * M, 0.0); rho_cand.assign(N * M, 0.0); rho_sub.assign(N * M, 0.0);
        for (int s = 0; s < tab.s; ++s) { Y[s].assign(N * M, 0.0); KE[s].assign(N * M, 0.0); KI[s].assign(N * M, 0.0); }
        triggered.assign(N, 0); changed.assign(N, 0); dirty.assign(N, 0); scratch.assign(N, 0); trig_step.assign(N, 0);
        grads.assign(N * Br * M, 0.0);
    }

    // (ts::GeneralRKTimeStepper)(eq, pg, t, dt) (TimeSteppers.jl:531-577), static grid
    bool step(double t, double dt) {
        (void)t;
        if (!have_geom && !prepare_geometry()) return false;
        if ((int64_t)rho_n.size() != N * M) size_buffers();
        std::fill(grads.begin(), grads.end(), 0.0);
        rho_n = rhos;
        std::fill(orders.begin(), orders.end(), max_order);
        if (!prelowered.empty()) {
            // particles a troubled-point predictor pre-lowered start the step one order lower (interior only)
            for (int64_t q = 0; q < N; ++q)
                if (prelowered[q] && !bnd[q]) orders[q] = std::max(1, max_order - 1);
            prelowered.clear();
        }
        std::fill(trig_step.begin(), trig_step.end(), 0);
        inadmissible = 0; mood_iters = 0;
        const int s = tab.s;
        const bool mv = moving();
        if (mv) {
            x_n = pos;
            x_cand.assign(N * D, 0.0);
            for (int q = 0; q < s; ++q) { Xst[q].assign(N * D, 0.0); KX[q].assign(N * D, 0.0); }
        }
        for (int i = 1; i <= s; ++i) {
            if (i == 1) {
                form_candidate(1, dt);                     // X_1 == x_n: the grid is already there
            } else {
                if (!mood_checkpoint(i, dt)) return false; // geometry of stage i - 1
                if (mv) {
                    // _apply_stage_geometry! (TimeSteppers.jl:521-525): stage positions, then the geometry caches
                    pos = Xst[i - 1];
                    if (mover.full_search_per_stage) { if (!build_neighbours()) return false; }
                    else refresh_geometry();
                    if (!prepare_geometry()) return false;
                }
            }
            // reset_orders_per_stage (TimeSteppers.jl:556)
            if (cfg.reset_orders_per_stage) std::fill(orders.begin(), orders.end(), max_order);
            KX_cur = mv ? &KX[i - 1] : nullptr;
            compute_rhs(KE[i - 1], Y[i - 1].data(), true);
        }
        if (!mood_checkpoint(s + 1, dt)) return false;     // geometry of stage s
        rhos = rho_cand;
        if (mv) {
            // final positions, full search with periodic re-wrap for the next step (TimeSteppers.jl:571-575)
            pos = x_cand;
            if (!build_neighbours() || !prepare_geometry()) return false;
            // ts.volume_estimator (TimeSteppers.jl:574): ShepardVolumes(sweeps) unless the volumes are kept
            if (!mover.keep_volumes) update_volumes(mover.shepard_sweeps > 0 ? mover.shepard_sweeps : 1);
        }
        ++steps;
        return true;
    }

    // update_volumes!(pg, ShepardVolumes(sweeps)) (Volumes.jl:183-229): S_i = w(0) + sum_j w_ij, V_i = 1/S_i, then
    // sweeps V_i <- (w(0)/S_i) V_i + sum_j (w_ij/S_j) V_j, negatives clamped and sum V rescaled to the box volume.
    void update_volumes(int sweeps) {
        if (N == 0) return;
        const double w0 = weight(0.0);
        std::vector<double> S(N), Vt(N);
        vol.assign(N, 0.0);
        for (int64_t i = 0; i < N; ++i) {
            double sm = w0;
            for (int64_t q = start[i]; q < start[i + 1]; ++q) sm = sm + nw[q];
            S[i] = sm;
            vol[i] = 1.0 / sm;
        }
        for (int it = 0; it < sweeps; ++it) {
            for (int64_t i = 0; i < N; ++i) {
                double acc = (w0 / S[i]) * vol[i];
                for (int64_t q = start[i]; q < start[i + 1]; ++q) {
                    const int64_t j = nidx[q];
                    acc = acc + (nw[q] / S[j]) * vol[j];
                }
                Vt[i] = acc;
            }
            vol = Vt;
        }
        double sum = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            if (!(vol[i] > 0.0)) vol[i] = 0.0;
            sum = sum + vol[i];
        }
        double box = 1.0;
        for (int d = 0; d < D; ++d) box = box * (cfg.domain_max[d] - cfg.domain_min[d]);
        const double f = box / sum;
        for (int64_t i = 0; i < N; ++i) vol[i] = vol[i] * f;
    }

    // get_time_step (ParticleGrids.jl:386-450) with the cached slot weights
    double time_step() {
        if (N == 0) return std::numeric_limits<double>::infinity();
        if (!have_geom) prepare_geometry();
        double best = std::numeric_limits<double>::infinity();
        const double tol = std::numeric_limits<double>::min();
        const double inv_dim = 1.0 / double(D);
#pragma omp parallel for reduction(min : best) schedule(dynamic, 256)
        for (int64_t i = 0; i < N; ++i) {
            if (bnd[i] || nnb(i) == 0) continue;
            const double *Ui = &rhos[i * M];
            double Li[3];
            for (int d = 0; d < D; ++d) Li[d] = phys.lam(Ui, d);
            if (weno || central || upwind) {
                // dispatch_cfl: degree _divergence_degree(WENO / Central / Upwind) = its order, clamped to 3 in 3-D / 4
                // otherwise (API.jl:236)
                int degree = std::min(max_order, D == 3 ? 3 : 4);
                double sc = cfl_sum_assembled(i, Li, degree);
                if (sc > tol) best = std::min(best, inv_dim / sc);
                continue;
            }
            double sum_c = 0.0;
            for (int64_t s = start[i]; s < start[i + 1]; ++s) {
                const double *Uj = &rhos[int64_t(nidx[s]) * M];
                double dot = 0.0;
                for (int d = 0; d < D; ++d) {
                    double pr = std::fabs(dw[s * D + d]) * jmax(Li[d], phys.lam(Uj, d));
                    dot = (d == 0) ? pr : dot + pr;
                }
                sum_c = sum_c + dot;
            }
            if (sum_c > tol) best = std::min(best, inv_dim / sum_c);
        }
        return best;
    }
};

inline hcc_status fail(Solver *s, hcc_status st) { (void)s; return st; }

}  // namespace

struct orc_ctx {
    Solver s;
};

namespace {

// Stencil features of the learned troubled-point predictor (no counterpart in the reference; definitions in
// include/hcc.h): four quantities per particle, six FP32 features each, in the operation order of the GPU kernel.
void feature_quantities(const Solver &s, const double *u, float q[4]) {
    if (s.cfg.pde == HCC_PDE_EULER) {
        // density, rho * (rho e), |momentum|^2, total energy
        const float rho = float(u[0]);
        float msq = 0.f;
        for (int d = 0; d < s.D; ++d) {
            const float md = float(u[1 + d]);
            msq = std::fma(md, md, msq);
        }
        const float E = float(u[s.D + 1]);
        q[0] = rho;
        q[1] = std::fma(E, rho, -(0.5f * msq));
        q[2] = msq;
        q[3] = E;
    } else {
        for (int m = 0; m < 4; ++m) q[m] = float(u[m < s.M ? m : s.M - 1]);
    }
}

float clamp_feature(float f) {
    if (!(f == f)) return 0.f;
    return f > 8.f ? 8.f : (f < -8.f ? -8.f : f);
}

void point_features(const Solver &s, int64_t i, float h, float *f) {
    const int D = s.D;
    float qi[4], qmax[4], qmin[4], s1[4] = {0, 0, 0, 0}, s2[4] = {0, 0, 0, 0}, b[4][3] = {}, G[6] = {};
    feature_quantities(s, &s.rhos[i * s.M], qi);
    for (int m = 0; m < 4; ++m) { qmax[m] = qi[m]; qmin[m] = qi[m]; }
    const int64_t k0 = s.start[i], c = s.start[i + 1] - s.start[i];
    for (int64_t k = 0; k < c; ++k) {
        const int64_t slot = k0 + k;
        const int64_t j = s.nidx[slot];
        float x[3] = {0, 0, 0};
        for (int d = 0; d < D; ++d) x[d] = float(s.ndist[slot * D + d]);
        int e = 0;
        for (int p = 0; p < D; ++p)
            for (int q = p; q < D; ++q) { G[e] = std::fma(x[p], x[q], G[e]); ++e; }
        float qj[4];
        feature_quantities(s, &s.rhos[j * s.M], qj);
        for (int m = 0; m < 4; ++m) {
            const float dq = qj[m] - qi[m];
            s1[m] += dq;
            s2[m] = std::fma(dq, dq, s2[m]);
            for (int d = 0; d < D; ++d) b[m][d] = std::fma(dq, x[d], b[m][d]);
            qmax[m] = qj[m] > qmax[m] ? qj[m] : qmax[m];
            qmin[m] = qj[m] < qmin[m] ? qj[m] : qmin[m];
        }
    }
    float Gi[6] = {};
    float det;
    if (D == 1) {
        det = G[0];
        Gi[0] = 1.f;
    } else if (D == 2) {
        det = G[0] * G[2] - G[1] * G[1];
        Gi[0] = G[2]; Gi[1] = -G[1]; Gi[2] = G[0];
    } else {
        Gi[0] = G[3] * G[5] - G[4] * G[4];
        Gi[1] = G[2] * G[4] - G[1] * G[5];
        Gi[2] = G[1] * G[4] - G[2] * G[3];
        Gi[3] = G[0] * G[5] - G[2] * G[2];
        Gi[4] = G[1] * G[2] - G[0] * G[4];
        Gi[5] = G[0] * G[3] - G[1] * G[1];
        det = (G[0] * Gi[0] + G[1] * Gi[1]) + G[2] * Gi[2];
    }
    const bool solve = det > 0.f;
    const float idet = solve ? 1.f / det : 0.f;
    const float ic = c > 0 ? 1.f / float(c) : 0.f;
    for (int m = 0; m < 4; ++m) {
        float g[3] = {0, 0, 0};
        if (D == 1) {
            g[0] = b[m][0] * idet;
        } else if (D == 2) {
            g[0] = std::fma(Gi[0], b[m][0], Gi[1] * b[m][1]) * idet;
            g[1] = std::fma(Gi[1], b[m][0], Gi[2] * b[m][1]) * idet;
        } else {
            g[0] = std::fma(Gi[0], b[m][0], std::fma(Gi[1], b[m][1], Gi[2] * b[m][2])) * idet;
            g[1] = std::fma(Gi[1], b[m][0], std::fma(Gi[3], b[m][1], Gi[4] * b[m][2])) * idet;
            g[2] = std::fma(Gi[2], b[m][0], std::fma(Gi[4], b[m][1], Gi[5] * b[m][2])) * idet;
        }
        float bgb = 0.f, gg = 0.f;
        for (int d = 0; d < D; ++d) {
            bgb = std::fma(b[m][d], g[d], bgb);
            gg = std::fma(g[d], g[d], gg);
        }
        const float r = qmax[m] - qmin[m];
        const float sc = std::fabs(qmax[m]) + std::fabs(qmin[m]);
        float *o = f + 6 * m;
        o[0] = sc > 0.f ? r / sc : 0.f;
        if (c > 0 && r > 1e-6f * sc) {
            const float ir = 1.f / r;
            const float mean = s1[m] * ic;
            const float res = (s2[m] - bgb) * ic;
            const float var = s2[m] * ic - mean * mean;
            o[1] = ((2.f * qi[m] - qmax[m]) - qmin[m]) * ir;
            o[2] = -(mean * ir);
            o[3] = (res > 0.f ? std::sqrt(res) : 0.f) * ir;
            o[4] = (std::sqrt(gg) * h) * ir;
            o[5] = (var > 0.f ? std::sqrt(var) : 0.f) * ir;
        } else {
            o[1] = o[2] = o[3] = o[4] = o[5] = 0.f;
        }
        for (int t = 0; t < 6; ++t) o[t] = clamp_feature(o[t]);
    }
}

}  // namespace

extern "C" {

hcc_status orc_create(const hcc_config *cfg, orc_ctx **out) {
    if (!cfg || !out) return HCC_ERR_INVALID;
    auto *c = new orc_ctx();
    if (!c->s.init(*cfg)) { *out = c; return HCC_ERR_INVALID; }
    *out = c;
    return HCC_OK;
}
hcc_status orc_destroy(orc_ctx *ctx) { delete ctx; return HCC_OK; }
const char *orc_last_error(const orc_ctx *ctx) { return ctx ? ctx->s.err.c_str() : "null context"; }
hcc_status orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
    return HCC_OK;
}

hcc_status orc_upload_cloud(orc_ctx *ctx, int64_t n, const double *pos, const uint8_t *is_boundary,
                            const int32_t *tags, const double *volumes) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !is_boundary || !tags))) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    s.N = n;
    s.pos.assign(pos, pos + n * s.D);
    s.bnd.assign(is_boundary, is_boundary + n);
    s.tags.assign(tags, tags + n);
    double v0 = 1.0;
    for (int d = 0; d < s.D; ++d) v0 *= s.cfg.dx[d];
    s.vol.assign(n, v0);
    if (volumes) s.vol.assign(volumes, volumes + n);
    s.rhos.assign(n * s.M, 0.0);
    s.orders.assign(n, 0);
    s.have_nb = false; s.have_geom = false;
    s.rho_n.clear();
    return HCC_OK;
}
hcc_status orc_build_neighbours(orc_ctx *ctx) {
    if (!ctx) return HCC_ERR_INVALID;
    return ctx->s.build_neighbours() ? HCC_OK : HCC_ERR_STATE;
}
hcc_status orc_neighbour_total(orc_ctx *ctx, int64_t *total, int32_t *max_nb) {
    if (!ctx || !ctx->s.have_nb) return HCC_ERR_STATE;
    if (total) *total = int64_t(ctx->s.nidx.size());
    if (max_nb) *max_nb = ctx->s.max_nb;
    return HCC_OK;
}
hcc_status orc_download_neighbours(orc_ctx *ctx, int32_t *counts, int32_t *idx, double *w, double *dist) {
    if (!ctx || !ctx->s.have_nb) return HCC_ERR_STATE;
    Solver &s = ctx->s;
    if (counts) for (int64_t i = 0; i < s.N; ++i) counts[i] = s.nnb(i);
    if (idx) std::memcpy(idx, s.nidx.data(), s.nidx.size() * sizeof(int32_t));
    if (w) std::memcpy(w, s.nw.data(), s.nw.size() * sizeof(double));
    if (dist) std::memcpy(dist, s.ndist.data(), s.ndist.size() * sizeof(double));
    return HCC_OK;
}
hcc_status orc_neighbour_counts(orc_ctx *ctx, int32_t *counts) {
    if (!ctx || !counts) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if (s.N == 0) return HCC_OK;
    s.build_bins();
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < s.N; ++i) counts[i] = int32_t(s.count_of(i));
    return HCC_OK;
}
hcc_status orc_neighbours_of(orc_ctx *ctx, int64_t n_sel, const int64_t *ids, int32_t max_slots, int32_t *counts,
                             int32_t *idx, double *w, double *dist) {
    if (!ctx || n_sel < 0 || max_slots < 0 || (n_sel > 0 && (!ids || !counts || !idx || !w || !dist)))
        return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    for (int64_t q = 0; q < n_sel; ++q)
        if (ids[q] < 0 || ids[q] >= s.N) return HCC_ERR_INVALID;
    if (n_sel == 0) return HCC_OK;
    s.build_bins();
    bool over = false;
#pragma omp parallel for schedule(dynamic, 16) reduction(|| : over)
    for (int64_t q = 0; q < n_sel; ++q) {
        const int64_t i = ids[q];
        const int64_t c = s.count_of(i);
        counts[q] = int32_t(c);
        if (c > max_slots) { over = true; continue; }
        for (int64_t k = 0; k < max_slots; ++k) {            // slots past the count are zero
            idx[q * max_slots + k] = 0;
            w[q * max_slots + k] = 0.0;
            for (int d = 0; d < s.D; ++d) dist[(q * max_slots + k) * s.D + d] = 0.0;
        }
        s.write_of(i, idx + q * max_slots, w + q * max_slots, dist + q * max_slots * s.D);
    }
    return over ? HCC_ERR_CAPACITY : HCC_OK;
}
hcc_status orc_download_positions(orc_ctx *ctx, double *pos) {
    if (!ctx || !pos) return HCC_ERR_INVALID;
    std::memcpy(pos, ctx->s.pos.data(), ctx->s.pos.size() * sizeof(double));
    return HCC_OK;
}
hcc_status orc_prepare_geometry(orc_ctx *ctx) {
    if (!ctx) return HCC_ERR_INVALID;
    return ctx->s.prepare_geometry() ? HCC_OK : HCC_ERR_STATE;
}
hcc_status orc_download_geometry(orc_ctx *ctx, double *dweights, uint8_t *ok_recon, uint8_t *ok_div) {
    if (!ctx || !ctx->s.have_geom) return HCC_ERR_STATE;
    Solver &s = ctx->s;
    // CentralDivergence: the weights and flags of its full-degree fit
    const std::vector<double> &w = s.central ? s.dwc[s.qmax - 1] : s.dw;
    const std::vector<uint8_t> &okd = s.central ? s.okc[s.qmax - 1] : s.ok_d;
    if (dweights) std::memcpy(dweights, w.data(), w.size() * sizeof(double));
    if (ok_recon) std::memcpy(ok_recon, s.ok_r.data(), s.N);
    if (ok_div) std::memcpy(ok_div, okd.data(), s.N);
    return HCC_OK;
}
hcc_status orc_upload_state(orc_ctx *ctx, const double *U) {
    if (!ctx || !U) return HCC_ERR_INVALID;
    ctx->s.rhos.assign(U, U + ctx->s.N * ctx->s.M);
    return HCC_OK;
}
hcc_status orc_download_state(orc_ctx *ctx, double *U) {
    if (!ctx || !U) return HCC_ERR_INVALID;
    std::memcpy(U, ctx->s.rhos.data(), ctx->s.rhos.size() * sizeof(double));
    return HCC_OK;
}
hcc_status orc_time_step(orc_ctx *ctx, double *dt_out) {
    if (!ctx || !dt_out) return HCC_ERR_INVALID;
    if (!ctx->s.have_nb) return HCC_ERR_STATE;
    *dt_out = ctx->s.time_step();
    return HCC_OK;
}
hcc_status orc_compute_rhs(orc_ctx *ctx, double *K) {
    if (!ctx || !K) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if (!s.have_nb) return HCC_ERR_STATE;
    if (!s.have_geom && !s.prepare_geometry()) return HCC_ERR_STATE;
    if ((int64_t)s.rho_n.size() != s.N * s.M) s.size_buffers();
    std::fill(s.grads.begin(), s.grads.end(), 0.0);
    std::fill(s.orders.begin(), s.orders.end(), s.max_order);
    std::vector<double> Kv(s.N * s.M, 0.0);
    s.compute_rhs(Kv, s.rhos.data(), true);
    std::memcpy(K, Kv.data(), Kv.size() * sizeof(double));
    return HCC_OK;
}
hcc_status orc_compute_rhs_orders(orc_ctx *ctx, const int32_t *orders, double *K) {
    if (!ctx || !K || !orders) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if (!s.have_nb) return HCC_ERR_STATE;
    if (!s.have_geom && !s.prepare_geometry()) return HCC_ERR_STATE;
    if ((int64_t)s.rho_n.size() != s.N * s.M) s.size_buffers();
    std::fill(s.grads.begin(), s.grads.end(), 0.0);
    s.orders.assign(orders, orders + s.N);
    std::vector<double> Kv(s.N * s.M, 0.0);
    s.compute_rhs(Kv, s.rhos.data(), true);
    std::memcpy(K, Kv.data(), Kv.size() * sizeof(double));
    return HCC_OK;
}
hcc_status orc_features(orc_ctx *ctx, float *out) {
    if (!ctx || !out) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if (!s.have_nb) return HCC_ERR_STATE;
    double hm = s.cfg.dx[0];
    for (int d = 1; d < s.D; ++d) hm = std::min(hm, s.cfg.dx[d]);
    const float h = float(hm);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < s.N; ++i) point_features(s, i, h, out + i * HCC_MLP_FEATURES);
    return HCC_OK;
}
hcc_status orc_set_prelowered(orc_ctx *ctx, const uint8_t *mask) {
    if (!ctx) return HCC_ERR_INVALID;
    if (mask) ctx->s.prelowered.assign(mask, mask + ctx->s.N);
    else ctx->s.prelowered.clear();
    return HCC_OK;
}
hcc_status orc_step(orc_ctx *ctx, double t, double dt) {
    if (!ctx) return HCC_ERR_INVALID;
    if (!ctx->s.have_nb) return HCC_ERR_STATE;
    if (!std::isfinite(dt)) return HCC_ERR_NONFINITE;
    return ctx->s.step(t, dt) ? HCC_OK : HCC_ERR_TIMEOUT;
}
hcc_status orc_download_orders(orc_ctx *ctx, int32_t *orders) {
    if (!ctx || !orders) return HCC_ERR_INVALID;
    std::memcpy(orders, ctx->s.orders.data(), ctx->s.orders.size() * sizeof(int32_t));
    return HCC_OK;
}
hcc_status orc_upload_orders(orc_ctx *ctx, const int32_t *orders) {
    if (!ctx || !orders) return HCC_ERR_INVALID;
    ctx->s.orders.assign(orders, orders + ctx->s.N);
    return HCC_OK;
}
hcc_status orc_download_mood_flags(orc_ctx *ctx, uint8_t *flags) {
    if (!ctx || !flags) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    for (int64_t i = 0; i < s.N; ++i) flags[i] = i < (int64_t)s.trig_step.size() ? s.trig_step[i] : 0;
    return HCC_OK;
}
hcc_status orc_get_counters(orc_ctx *ctx, hcc_counters *out) {
    if (!ctx || !out) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    std::memset(out, 0, sizeof(*out));
    out->n_particles = s.N;
    int64_t ni = 0;
    int32_t mn = INT32_MAX;
    for (int64_t i = 0; i < s.N; ++i)
        if (!s.bnd[i]) { ++ni; if (s.have_nb) mn = std::min(mn, s.nnb(i)); }
    out->n_interior = ni;
    out->max_neighbours = s.max_nb;
    out->min_neighbours_interior = (mn == INT32_MAX) ? 0 : mn;
    out->total_neighbours = int64_t(s.nidx.size());
    out->mood_iterations = s.mood_iters;
    int64_t fl = 0;
    for (auto v : s.trig_step) fl += v;
    out->mood_flagged = fl;
    out->inadmissible = s.inadmissible;
    out->steps = s.steps;
    return HCC_OK;
}
hcc_status orc_total_mass(orc_ctx *ctx, double *out) {
    if (!ctx || !out) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    for (int m = 0; m < s.M; ++m) out[m] = 0.0;
    for (int64_t i = 0; i < s.N; ++i)
        for (int m = 0; m < s.M; ++m) out[m] += s.vol[i] * s.rhos[i * s.M + m];
    return HCC_OK;
}
hcc_status orc_update_volumes(orc_ctx *ctx, int32_t sweeps) {
    if (!ctx || sweeps < 0) return HCC_ERR_INVALID;
    if (!ctx->s.have_nb) return HCC_ERR_STATE;
    ctx->s.update_volumes(sweeps);
    return HCC_OK;
}
hcc_status orc_download_volumes(orc_ctx *ctx, double *out) {
    if (!ctx || !out) return HCC_ERR_INVALID;
    std::memcpy(out, ctx->s.vol.data(), ctx->s.vol.size() * sizeof(double));
    return HCC_OK;
}
hcc_status orc_set_streamed(orc_ctx *ctx, int streamed) {
    if (!ctx) return HCC_ERR_INVALID;
    ctx->s.streamed = streamed != 0;
    return HCC_OK;
}
hcc_status orc_download_gradients(orc_ctx *ctx, double *g, int32_t *br_out) {
    if (!ctx) return HCC_ERR_INVALID;
    if (br_out) *br_out = ctx->s.Br;
    if (g) std::memcpy(g, ctx->s.grads.data(), ctx->s.grads.size() * sizeof(double));
    return HCC_OK;
}

double orc_ssp_coefficient(int32_t tableau) { return ssp_coefficient(make_tableau(tableau)); }
int32_t orc_basis_count(int32_t D, int32_t degree) { return basis_count(D, degree); }
int32_t orc_div_idx(int32_t D, int32_t o) { return div_idx(D, o); }
int32_t orc_divergence_index(int32_t DO, int32_t D, int32_t p_order, int32_t num_nb) {
    return divergence_index(DO, D, p_order, num_nb);
}
int32_t orc_basis_exponents(int32_t D, int32_t degree, int32_t *exps) {
    const BasisTable &bt = basis_table(D, degree);
    if (exps)
        for (int k = 0; k < bt.B; ++k)
            for (int d = 0; d < D; ++d) exps[k * D + d] = bt.exps[k][d];
    return bt.B;
}
int32_t orc_mls_divergence(int32_t D, int32_t M, int32_t q, int32_t K, const double *dists, const double *w,
                           const double *dF, double scale, double *out) {
    const BasisTable &bt = basis_table(D, q);
    int B = bt.B + 1;
    double invL = 1.0 / scale;
    std::vector<double> Nm(B * B, 0.0), bs(size_t(B) * D * M, 0.0);
    double p[32], sd[3];
    for (int k = 0; k < K; ++k) {
        for (int d = 0; d < D; ++d) sd[d] = dists[k * D + d] * invL;
        p[0] = 1.0; build_basis(bt, sd, p + 1);
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) Nm[r * B + c] = Nm[r * B + c] + w[k] * (p[r] * p[c]);
        for (int b = 0; b < B; ++b)
            for (int qq = 0; qq < D * M; ++qq) bs[b * D * M + qq] = bs[b * D * M + qq] + w[k] * (p[b] * dF[k * D * M + qq]);
    }
    double U[400];
    for (int m = 0; m < M; ++m) out[m] = 0.0;
    if (!cholesky_moment(B, Nm.data(), U)) return 0;
    double E[32], X[3][32];
    for (int d = 0; d < D; ++d) {
        for (int b = 0; b < B; ++b) E[b] = (b == d + 1) ? 1.0 : 0.0;
        chol_solve(B, U, E, X[d]);
    }
    for (int m = 0; m < M; ++m) {
        double acc = 0.0;
        for (int d = 0; d < D; ++d) {
            int qq = d * M + m;
            double Rdq = X[d][0] * bs[qq];
            for (int b = 1; b < B; ++b) Rdq = Rdq + X[d][b] * bs[b * D * M + qq];
            acc = (d == 0) ? Rdq : acc + Rdq;
        }
        out[m] = acc * invL;
    }
    return 1;
}
int32_t orc_mls_solve(int32_t D, int32_t M, int32_t q, int32_t K, const double *dists, const double *w,
                      const double *df, double scale, double *out) {
    const BasisTable &bt = basis_table(D, q);
    int B = bt.B;
    double invL = 1.0 / scale;
    std::vector<double> Nm(B * B, 0.0), bs(size_t(B) * M, 0.0);
    double p[32], sd[3];
    for (int k = 0; k < K; ++k) {
        for (int d = 0; d < D; ++d) sd[d] = dists[k * D + d] * invL;
        build_basis(bt, sd, p);
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) Nm[r * B + c] = Nm[r * B + c] + w[k] * (p[r] * p[c]);
        for (int b = 0; b < B; ++b)
            for (int m = 0; m < M; ++m) bs[b * M + m] = bs[b * M + m] + w[k] * (p[b] * df[k * M + m]);
    }
    double U[400], sc[32] = {0}, col[32] = {0}, x[32] = {0};
    for (int k = 0; k < B * M; ++k) out[k] = 0.0;
    if (!cholesky_moment(B, Nm.data(), U)) return 0;
    build_scales(bt, invL, sc);
    for (int m = 0; m < M; ++m) {
        for (int b = 0; b < B; ++b) col[b] = bs[b * M + m];
        chol_solve(B, U, col, x);
        for (int b = 0; b < B; ++b) out[b * M + m] = x[b] * sc[b];
    }
    return 1;
}
int32_t orc_cholesky_moment(int32_t B, const double *Nmat, double *U, int32_t *plain_ok) {
    bool pok = false;
    bool ok = cholesky_moment(B, Nmat, U, &pok);
    if (plain_ok) *plain_ok = pok;
    return ok ? 1 : 0;
}
hcc_status orc_expand_mask(orc_ctx *ctx, uint8_t *mask, int32_t hops) {
    if (!ctx || !mask || !ctx->s.have_nb) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    std::vector<uint8_t> m(mask, mask + s.N);
    s.scratch.assign(s.N, 0);
    s.expand_mask(m, hops);
    std::memcpy(mask, m.data(), s.N);
    return HCC_OK;
}
hcc_status orc_interface_orders(orc_ctx *ctx, int64_t i, int64_t j, int32_t *oi, int32_t *oj) {
    if (!ctx || !ctx->s.have_nb) return HCC_ERR_INVALID;
    int a, b;
    ctx->s.interface_orders(i, j, a, b);
    *oi = a; *oj = b;
    return HCC_OK;
}
hcc_status orc_detect_and_drop(orc_ctx *ctx, const double *prev, const double *cand, int32_t full,
                               const uint8_t *dirty, int32_t with_eq, int32_t *changed_any) {
    if (!ctx || !prev || !cand || !ctx->s.have_nb) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if ((int64_t)s.rho_n.size() != s.N * s.M) s.size_buffers();
    if (dirty) s.dirty.assign(dirty, dirty + s.N); else std::fill(s.dirty.begin(), s.dirty.end(), 0);
    bool any = s.detect_and_drop(prev, cand, full != 0, with_eq != 0);
    if (changed_any) *changed_any = any ? 1 : 0;
    return HCC_OK;
}
hcc_status orc_set_mover(orc_ctx *ctx, const hcc_mover *mv) {
    if (!ctx || !mv) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if (mv->kind < HCC_MOVER_NONE || mv->kind > HCC_MOVER_PRESCRIBED) return HCC_ERR_INVALID;
    if ((mv->kind == HCC_MOVER_LAGRANGIAN || mv->kind == HCC_MOVER_SCALED) && !s.phys.has_fluid_velocity())
        return HCC_ERR_UNSUPPORTED;
    if (mv->kind != HCC_MOVER_NONE && (s.weno || s.central || s.upwind)) return HCC_ERR_UNSUPPORTED;
    s.mover = *mv;
    return HCC_OK;
}

// The MOOD criterion of particle p for hand-set stage states (N x M), reconstruction gradients (N x Br x M, the
// layout of orc_download_gradients), orders and a candidate state (M): the known-answer tests of MOODu2.
hcc_status orc_criterion_flags(orc_ctx *ctx, int64_t p, const double *prev, const double *grads, const int32_t *orders,
                               const double *cand, int32_t *flag) {
    if (!ctx || !prev || !grads || !orders || !cand || !flag) return HCC_ERR_INVALID;
    Solver &s = ctx->s;
    if (p < 0 || p >= s.N || !s.have_nb) return HCC_ERR_INVALID;
    s.grads.assign(grads, grads + size_t(s.N) * s.Br * s.M);
    s.orders.assign(orders, orders + s.N);
    s.global_range(prev);
    std::vector<double> c(size_t(s.N) * s.M, 0.0);
    for (int m = 0; m < s.M; ++m) c[size_t(p) * s.M + m] = cand[m];
    *flag = s.criterion_flags(p, prev, c.data()) ? 1 : 0;
    return HCC_OK;
}

hcc_status orc_apply_bcs(orc_ctx *ctx, double *buf) {
    if (!ctx || !buf || !ctx->s.have_nb) return HCC_ERR_INVALID;
    ctx->s.apply_bcs(buf);
    return HCC_OK;
}

}  // extern "C"
