// hcc_api.cu — the C ABI (include/hcc.h): context lifecycle, device buffers and the host orchestration of one
// time step (the GeneralRKTimeStepper functor, src/TimeStepping/TimeSteppers.jl:531-577) on one CUDA stream.
#include "hcc_internal.cuh"
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>

using namespace hcc;

namespace {

// ----------------------------------------------------------------------------------- tableaus
// The built-in Butcher tableaus of src/TimeStepping/ButcherTableaus.jl (explicit part a_t, b_t, c_t; implicit
// part a, b, c), stored as plain data.
struct Tableau {
    int s = 0;
    double a[5][5]{}, at[5][5]{}, c[5]{}, ct[5]{}, b[5]{}, bt[5]{};
};

Tableau make_tableau(int id) {
    Tableau t;
    auto expl = [&](int s, std::initializer_list<double> A, std::initializer_list<double> bb,
                    std::initializer_list<double> cc) {
        t.s = s;
        int k = 0;
        for (double v : A) { t.at[k / s][k % s] = v; ++k; }
        k = 0; for (double v : bb) t.bt[k++] = v;
        k = 0; for (double v : cc) { t.c[k] = v; t.ct[k] = v; ++k; }
    };
    const double g2 = 1.0 - 1.0 / std::sqrt(2.0);
    switch (id) {
    case HCC_TAB_RK1_EULER: expl(1, {0.0}, {1.0}, {0.0}); break;
    case HCC_TAB_RK2_SSP: expl(2, {0, 0, 1.0, 0}, {0.5, 0.5}, {0.0, 1.0}); break;
    case HCC_TAB_RK2_RALSTON: expl(2, {0, 0, 2.0 / 3, 0}, {0.25, 0.75}, {0.0, 2.0 / 3}); break;
    case HCC_TAB_RK3_SSP: expl(3, {0, 0, 0, 1.0, 0, 0, 0.25, 0.25, 0}, {1.0 / 6, 1.0 / 6, 2.0 / 3}, {0.0, 1.0, 0.5}); break;
    case HCC_TAB_RK4_CLASSICAL:
        expl(4, {0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1.0, 0}, {1.0 / 6, 1.0 / 3, 1.0 / 3, 1.0 / 6},
             {0.0, 0.5, 0.5, 1.0});
        break;
    case HCC_TAB_RK4_SSP:   // Spiteri & Ruuth SSPRK(5,4)
        expl(5,
             {0, 0, 0, 0, 0, 0.39175222657189002, 0, 0, 0, 0, 0.21766909626116876, 0.36841059305037099, 0, 0, 0,
              0.082692086657810582, 0.13995850219189535, 0.25189177427169401, 0, 0, 0.067966283637114752,
              0.11503469850463156, 0.20703489859738566, 0.54497475022852104, 0},
             {0.14681187608478657, 0.24848290944497617, 0.10425883033198098, 0.2744389009013507, 0.226007483236906},
             {0.0, 0.39175222657189002, 0.58607968931153975, 0.47454236312139997, 0.93501063096765302});
        break;
    case HCC_TAB_IMEX_EULER:
        t.s = 2; t.at[1][0] = 1; t.a[1][1] = 1; t.c[1] = 1; t.ct[1] = 1; t.b[1] = 1; t.bt[0] = 1;
        break;
    case HCC_TAB_IMEX_ARS233: {
        double g = (3.0 + std::sqrt(3.0)) / 6.0;
        t.s = 3;
        t.a[1][1] = g; t.a[2][1] = 1.0 - 2 * g; t.a[2][2] = g;
        t.at[1][0] = g; t.at[2][0] = g - 1.0; t.at[2][1] = 2.0 * (1 - g);
        t.c[1] = g; t.c[2] = 1.0 - g;
        for (int i = 0; i < 3; ++i) t.ct[i] = t.c[i];
        t.b[1] = 0.5; t.b[2] = 0.5;
        for (int i = 0; i < 3; ++i) t.bt[i] = t.b[i];
        break;
    }
    case HCC_TAB_IMEX_ARS222: {
        double g = g2, dl = 1 - 1 / (2 * g);
        t.s = 3;
        t.a[1][1] = g; t.a[2][1] = 1 - g; t.a[2][2] = g;
        t.at[1][0] = g; t.at[2][0] = dl; t.at[2][1] = 1 - dl;
        t.c[1] = g; t.c[2] = 1;
        for (int i = 0; i < 3; ++i) t.ct[i] = t.c[i];
        t.b[1] = 1 - g; t.b[2] = g;
        t.bt[0] = dl; t.bt[1] = 1 - dl;
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
        t.ct[1] = 1; t.ct[2] = 0.5;
        break;
    }
    case HCC_TAB_IMEX_SSP2332:
        t.s = 3;
        t.a[0][0] = 0.25; t.a[1][1] = 0.25; t.a[2][0] = 1.0 / 3; t.a[2][1] = 1.0 / 3; t.a[2][2] = 1.0 / 3;
        t.at[1][0] = 0.5; t.at[2][0] = 0.5; t.at[2][1] = 0.5;
        t.b[0] = t.b[1] = t.b[2] = 1.0 / 3;
        for (int i = 0; i < 3; ++i) t.bt[i] = t.b[i];
        t.c[0] = 0.25; t.c[1] = 0.25; t.c[2] = 1.0;
        t.ct[1] = 0.5; t.ct[2] = 1.0;
        break;
    default: t.s = 0;
    }
    return t;
}

// ssp_coefficient (ButcherTableaus.jl:86-118): bisection on r for non-negative canonical Shu–Osher
// coefficients alpha = rK (I + rK)^-1, v = (I - alpha) 1 (tolerance -1e-13); 0 for tableaus with an implicit part.
double ssp_coefficient(const Tableau &t) {
    for (int i = 0; i < t.s; ++i)
        for (int j = 0; j < t.s; ++j)
            if (t.a[i][j] != 0.0) return 0.0;
    const int s = t.s, n = s + 1;
    double K[6][6] = {};
    for (int i = 0; i < s; ++i) for (int j = 0; j < s; ++j) K[i][j] = t.at[i][j];
    for (int j = 0; j < s; ++j) K[s][j] = t.bt[j];
    auto ok = [&](double r) {
        double A[6][6], Inv[6][6];
        for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) A[i][j] = (i == j ? 1.0 : 0.0) + r * K[i][j];
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                double v = (i == j) ? 1.0 : 0.0;
                for (int k = 0; k < i; ++k) v -= A[i][k] * Inv[k][j];
                Inv[i][j] = v / A[i][i];
            }
        double al[6][6];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double v = 0.0;
                for (int k = 0; k < n; ++k) v += r * K[i][k] * Inv[k][j];
                al[i][j] = v;
                if (v < -1e-13) return false;
            }
        for (int i = 0; i < n; ++i) {
            double v = 0.0;
            for (int j = 0; j < n; ++j) v += (i == j ? 1.0 : 0.0) - al[i][j];
            if (v < -1e-13) return false;
        }
        return true;
    };
    double lo = 1e-3, hi = 1e-3;
    if (!ok(lo)) return 0.0;
    while (ok(hi) && hi < 1e3) hi *= 2;
    lo = hi / 2;
    for (int it = 0; it < 60; ++it) {
        double mid = (lo + hi) / 2;
        if (ok(mid)) lo = mid; else hi = mid;
    }
    return lo;
}

bool has_implicit_part(const Tableau &t) {
    for (int i = 0; i < t.s; ++i) {
        if (t.b[i] != 0.0) return true;
        for (int j = 0; j < t.s; ++j) if (t.a[i][j] != 0.0) return true;
    }
    return false;
}

const char *kStatusNames[] = {"HCC_OK", "HCC_ERR_INVALID", "HCC_ERR_CAPACITY", "HCC_ERR_CUDA", "HCC_ERR_STATE",
                              "HCC_ERR_NONFINITE", "HCC_ERR_TIMEOUT", "HCC_ERR_UNSUPPORTED"};

template <typename P> void dfree(P *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace

struct hcc_ctx {
    hcc_config cfg{};
    std::string err;
    cudaStream_t stream = nullptr;
    int D = 2, M = 1, f32 = 0;
    int64_t capacity = 0, n = 0, npad = 0, n_interior = 0;
    int kmax = 0;
    int64_t total_nb = 0;
    const StageOps *ops = nullptr;
    // scheme
    int max_order = 2, DO = 0, rdeg = 1, Br = 1, full_div = 2, ddeg = 1, Bd = 2, need_dw1 = 0;
    double invL = 1.0, h = 1.0;
    int weno = 0;
    int central = 0;                  // CentralDivergence: no reconstruction, per-degree divergence weight sets
    int upwind = 0;                   // UpwindDivergence :Tiwari / :Praveen (scalar, first order)
    int qmax = 1;
    double *dwc64[3] = {}; float *dwc32[3] = {}; uint8_t *okc[3] = {};
    double *mw64 = nullptr; float *mw32 = nullptr;   // moment-correction weights (first-order MUSCL)
    std::vector<int64_t> batch_offsets;              // clouds of the last hcc_upload_batch (empty: one cloud)
    int32_t *cloud_id = nullptr;                     // device: particle -> cloud of the batch
    unsigned long long *cloud_dt = nullptr;          // device: per-cloud CFL minima (ordered bits)
    bool per_cloud = false;                          // the step being enqueued uses one dt per cloud (step_dts)
    std::vector<double> step_dts;
    int coef_sets = 1;                               // coefficient sets the stage-coefficient buffers hold
    int graph_per_cloud = -1;                        // the per_cloud mode the step graphs were captured with
    bool moment() const { return cfg.moment_correction && max_order == 1 && !weno && !central && !upwind; }
    bool no_recon() const { return weno || central || upwind; }

    Tableau tab;
    double ssp_C = 0.0, ratio = 0.0;
    int has_source = 0;
    // cloud
    double *pos = nullptr; uint8_t *bnd = nullptr; int32_t *tags = nullptr; double *vol = nullptr;
    float *pos32 = nullptr; unsigned int *pmax32 = nullptr;   // FP32 positions of the search prefilter
    float *wops = nullptr; int32_t *wcnt = nullptr;             // FP32 Euler WENO operators, stencil sizes
    double *wchol = nullptr; uint8_t *wok = nullptr;             // FP64 Euler WENO: packed factors and flags
    double *wflux64 = nullptr;                                    // FP64 Euler WENO: the stage's flux table
    std::vector<uint8_t> h_bnd; std::vector<int32_t> h_tags;
    // cell list
    int dims[3] = {1, 1, 1}; double csize[3] = {1, 1, 1};
    int64_t nbins = 0; int noff = 1;
    int64_t *binnb = nullptr; int32_t *bin_of = nullptr, *cell_count = nullptr, *cell_cursor = nullptr, *cellp = nullptr;
    int64_t *cell_start = nullptr; int32_t *cnt = nullptr;
    // neighbours (FP64 master copy, slot-major)
    int32_t *nidx = nullptr; double *w64 = nullptr, *dist64 = nullptr;
    // geometry
    double *inv_r64 = nullptr, *inv_d64 = nullptr, *dw64 = nullptr, *dw1_64 = nullptr;
    uint8_t *ok_r = nullptr, *ok_d = nullptr, *ok_1 = nullptr;
    float *dist32 = nullptr, *w32 = nullptr, *dw32 = nullptr, *dw1_32 = nullptr, *inv_r32 = nullptr, *gw32 = nullptr;
    int32_t *status = nullptr, *status2 = nullptr, *root = nullptr;
    int32_t *blist = nullptr, *bsrc = nullptr; int64_t nbnd = 0;
    // state (element type double or float)
    void *rhos = nullptr, *cand = nullptr, *grad = nullptr;
    void *xfer = nullptr;                        // n*M doubles: staging of host-precision conversions
    void *Y[HCC_MAX_STAGES] = {}, *KE[HCC_MAX_STAGES] = {}, *KI[HCC_MAX_STAGES] = {};
    int8_t *orders = nullptr, *nbmin = nullptr;
    uint8_t *trig_step = nullptr, *inadm = nullptr;
    // MOOD tile worklists (failed candidates, changed orders, their reach): tile lists and member words
    int32_t *ttiles = nullptr, *ctiles = nullptr, *dtiles = nullptr, *ftiles = nullptr;
    uint32_t *tmask = nullptr, *cmask = nullptr, *dmask = nullptr, *words1 = nullptr, *fmask = nullptr;
    int32_t *forced = nullptr;                    // StrictEPD0 order offers (0x7f7f7f7f: none)
    ListCounts *lcounts = nullptr, *h_lcounts = nullptr;
    int list_blocks = 1, drop_blocks = 1;
    int sms = 1;                                 // SM count of the device
    hcc_tuning tune{128, 128, 8, 2};             // launch shapes of the step (hcc_set_tuning / hcc_autotune)
    TileTables tiles;                            // tile staging of the FP32 full passes (hcc_tiles.cu)
    int tile_enabled = 1;
    void apply_tuning() {
        list_blocks = std::max(1, sms) * tune.list_blocks_per_sm;
        drop_blocks = std::max(1, sms) * tune.drop_blocks_per_sm;
    }
    unsigned long long *u2_keys = nullptr;       // MOODu2 global range of the stage state (ordered keys)
    // learned troubled-point predictor: the attached network, its threshold (logit), the start-of-step features
    // (captured for training) and the mask of the particles it pre-lowered
    hcc_mlp *mlp = nullptr;
    float thr_logit = 0.f;
    int capture_feat = 0;
    float *feat = nullptr;
    uint8_t *pred = nullptr;
    uint4 *pred_rows = nullptr;       // compact list of the rows that passed the smoothness gate
    int32_t *pred_idx = nullptr;
    uint32_t *rough = nullptr;        // per tile: particles whose stencil was not flat at the last step's end
    void reset_rough() {
        if (rough) cudaMemset(rough, 0xff, size_t(npad / 32) * sizeof(uint32_t));
    }
    int64_t predicted = 0;
    bool feat_valid = false;
    // moving grid: mover, start-of-step / stage / final positions and the stage grid velocities (SoA FP64)
    hcc_mover mover{};
    double *x_n = nullptr, *x_cand = nullptr, *Xs[HCC_MAX_STAGES] = {}, *KXs[HCC_MAX_STAGES] = {};
    bool moving() const { return mover.kind != HCC_MOVER_NONE; }
    void free_mover_buffers() {
        dfree(x_n); dfree(x_cand);
        for (int q = 0; q < HCC_MAX_STAGES; ++q) { dfree(Xs[q]); dfree(KXs[q]); }
    }
    bool u2_plateau_on() const { return cfg.mood_criterion == HCC_MOOD_U2 && cfg.u2_plateau > 0.0; }
    unsigned long long *d_counters = nullptr;   // [0..1] drop counters, [2] dt bits, [3..4] search stats
    unsigned long long *h_counters = nullptr;   // pinned mirror
    double *d_mass = nullptr;
    bool have_cloud = false, have_nb = false, have_geom = false, have_state = false;
    // statistics
    int64_t launches = 0, mood_iters = 0, flagged = 0, inadmissible = 0, steps = 0, launches_total = 0,
            graph_steps = 0;
    int32_t min_nb_interior = 0;
    // step graphs
    cudaStream_t stream2 = nullptr;       // capture stream of the conditional bodies
    void *coef_dev = nullptr, *coef_host = nullptr;
    MoodStats *mood_stats = nullptr, *mood_stats_host = nullptr;
    struct StepGraphT {
        cudaGraphExec_t exec = nullptr;
        void *rhos = nullptr;
        int launches = 0, body_launches = 0;
        void reset() {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
            rhos = nullptr;
        }
    } graphs[2];
    bool use_graphs = true, graphs_failed = false;
    int n_checkpoints() const { return cfg.mood_criterion != HCC_MOOD_NONE ? tab.s : 0; }
    void drop_graphs() { graphs[0].reset(); graphs[1].reset(); }
    // profiling: event pairs around gather (kind 0) and flux (kind 1) launches of the current step
    int prof = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_kind;
    size_t ev_used = 0;
    hcc_kernel_times times{};

    void prof_begin(int kind) {
        if (!prof) return;
        if (ev_used + 2 > ev_pool.size()) {
            for (int k = 0; k < 64; ++k) {
                cudaEvent_t e;
                if (cudaEventCreate(&e) != cudaSuccess) { prof = 0; return; }
                ev_pool.push_back(e);
            }
        }
        if (ev_kind.size() < ev_pool.size() / 2) ev_kind.resize(ev_pool.size() / 2);
        ev_kind[ev_used / 2] = kind;
        cudaEventRecord(ev_pool[ev_used], stream);
    }
    void prof_end() {
        if (!prof) return;
        cudaEventRecord(ev_pool[ev_used + 1], stream);
        ev_used += 2;
    }
    void prof_collect() {   // after the stream was synchronised
        for (size_t q = 0; q < ev_used; q += 2) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev_pool[q], ev_pool[q + 1]);
            if (ev_kind[q / 2] == 0) { times.gather_ms += ms; times.gather_launches += 1; }
            else if (ev_kind[q / 2] == 1) { times.flux_ms += ms; times.flux_launches += 1; }
            else if (ev_kind[q / 2] == 3) { times.predict_ms += ms; times.predict_launches += 1; }
            else { times.recompute_ms += ms; times.recompute_launches += 1; }
        }
        ev_used = 0;
    }

    size_t esz() const { return f32 ? sizeof(float) : sizeof(double); }

    hcc_status fail(hcc_status st, const std::string &msg) {
        err = msg;
        return st;
    }
    hcc_status cuda(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return HCC_OK;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return HCC_ERR_CUDA;
    }
    template <typename P> hcc_status alloc(P *&p, size_t count, const char *what) {
        dfree(p);
        if (count == 0) count = 1;
        return cuda(cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(P)), what);
    }
    hcc_status valloc(void *&p, size_t bytes, const char *what) {
        if (p) cudaFree(p);
        p = nullptr;
        return cuda(cudaMalloc(&p, bytes ? bytes : 1), what);
    }
    hcc_status sync(const char *what) { return cuda(cudaStreamSynchronize(stream), what); }

    void free_particles() {
        drop_graphs();
        tiles.release();
        free_mover_buffers();
        dfree(pos); dfree(bnd); dfree(tags); dfree(vol); dfree(bin_of); dfree(cellp); dfree(cnt);
        dfree(pos32); dfree(pmax32); dfree(wops); dfree(wcnt); dfree(wchol); dfree(wok); dfree(wflux64);
        dfree(ok_r); dfree(ok_d); dfree(ok_1); dfree(inv_r64); dfree(inv_d64); dfree(inv_r32);
        dfree(status); dfree(status2); dfree(root); dfree(blist); dfree(bsrc);
        for (void **p : {&rhos, &cand, &grad, &xfer}) { if (*p) cudaFree(*p); *p = nullptr; }
        for (int s = 0; s < HCC_MAX_STAGES; ++s)
            for (void **p : {&Y[s], &KE[s], &KI[s]}) { if (*p) cudaFree(*p); *p = nullptr; }
        dfree(orders); dfree(nbmin); dfree(trig_step); dfree(inadm);
        dfree(ttiles); dfree(ctiles); dfree(dtiles); dfree(tmask); dfree(cmask); dfree(dmask); dfree(words1);
        dfree(ftiles); dfree(fmask); dfree(forced); dfree(feat); dfree(pred); dfree(pred_rows); dfree(pred_idx);
        dfree(rough);
        dfree(cloud_id); dfree(cloud_dt);
        per_cloud = false;
        feat_valid = false;
    }
    void free_slots() {
        drop_graphs();
        tiles.release();
        dfree(nidx); dfree(w64); dfree(dist64); dfree(dw64); dfree(dw1_64); dfree(dist32); dfree(w32); dfree(dw32);
        dfree(dw1_32); dfree(gw32);
        for (int q = 0; q < 3; ++q) { dfree(dwc64[q]); dfree(dwc32[q]); dfree(okc[q]); }
        dfree(mw64); dfree(mw32);
    }
    void free_bins() { dfree(binnb); dfree(cell_count); dfree(cell_cursor); dfree(cell_start); }
};

namespace {

const char *g_null_ctx_error = "null context";

// ------------------------------------------------------------------ argument assembly
template <typename T> PhysParams<T> phys_params(const hcc_ctx *c) {
    PhysParams<T> p{};
    const hcc_config &f = c->cfg;
    for (int d = 0; d < c->D; ++d) {
        double am = 0.0;
        for (int m = 0; m < c->M; ++m) {
            p.c[d][m] = T(f.velocity[d][m]);
            am = std::max(am, std::fabs(f.velocity[d][m]));
        }
        p.amax[d] = T(am);
        p.a_macro[d] = T(f.bgk_macro_velocity[d]);
    }
    p.gamma = T(f.gamma);
    p.gm1 = T(f.gamma - 1.0);
    if (f.pde == HCC_PDE_BGK) {
        p.inv_eps = T(1.0 / f.bgk_epsilon);
        p.coeff = T(f.bgk_coefficient);
        double fac = f.bgk_interior_factor;
        for (int k = 0; k < c->M; ++k)
            for (int d = 0; d < c->D; ++d) {
                double v = f.velocity[d][k];
                p.sinv[k][d] = T(std::fabs(v) > 1e-14 ? fac / v : 0.0);
            }
    }
    return p;
}

template <typename T> StageArgs<T> base_args(hcc_ctx *c) {
    StageArgs<T> a{};
    Geometry<T> &g = a.g;
    g.n = c->n;
    g.npad = c->npad;
    g.cnt = c->cnt;
    g.nidx = c->nidx;
    if constexpr (sizeof(T) == 8) {
        g.dist = c->dist64; g.wt = c->w64; g.dw = c->dw64; g.dw1 = c->need_dw1 ? c->dw1_64 : nullptr;
        g.inv_r = c->inv_r64;
    } else {
        g.dist = c->dist32; g.wt = c->w32; g.dw = c->dw32; g.dw1 = c->need_dw1 ? c->dw1_32 : nullptr;
        g.inv_r = c->inv_r32;
        g.gw = c->gw32;
    }
    g.ok_r = c->ok_r; g.ok_d = c->ok_d; g.ok_1 = c->ok_1;
    if constexpr (sizeof(T) == 8) g.mw = c->moment() ? c->mw64 : nullptr;
    else g.mw = c->moment() ? c->mw32 : nullptr;
    for (int q = 0; q < 3; ++q) {
        if constexpr (sizeof(T) == 8) g.dwc[q] = c->dwc64[q];
        else g.dwc[q] = c->dwc32[q];
        g.okc[q] = c->okc[q];
    }
    g.bnd = c->bnd;
    g.invL = T(c->invL);
    g.invL64 = c->invL;
    g.h64 = c->h;
    if constexpr (sizeof(T) == 4) {
        g.wops = c->wops;
        g.wcnt = c->wcnt;
    } else {
        g.wchol = c->wchol;
        g.wok = c->wok;
        g.wcnt = c->wcnt;
    }
    a.ph = phys_params<T>(c);
    a.sc.max_order = c->max_order;
    a.sc.DO = c->DO;
    a.sc.strategy = c->cfg.mood_strategy;
    a.sc.criterion = c->cfg.mood_criterion;
    a.sc.has_source = c->has_source;
    a.sc.limiter = c->cfg.limiter;
    a.sc.upwind_alg = c->upwind;
    a.sc.aligned = c->cfg.flux == HCC_FLUX_ALIGNED;
    a.orders = c->orders;
    a.nbmin = c->nbmin;
    a.grad = static_cast<T *>(c->grad);
    a.tmask = c->tmask;
    a.ttiles = c->ttiles;
    a.tcount = &c->lcounts->t;
    a.inadm = c->inadm;
    a.list_blocks = c->list_blocks;
    a.flux_block = c->tune.flux_block;
    a.gather_block = c->tune.gather_block;
    a.delta = T(c->cfg.mood_delta);
    a.u2_plateau = T(c->cfg.u2_plateau);
    a.u2_ratio = T(c->cfg.u2_ratio);
    a.u2_h = T(c->h);
    a.u2_range = c->u2_plateau_on() ? c->u2_keys : nullptr;
    if constexpr (sizeof(T) == 4) {
        if (c->tiles.ok && c->tile_enabled && !c->moving()) {
            a.tile = 1;
            TileView &v = a.tv;
            v.ntiles = c->tiles.ntiles; v.ustart = c->tiles.ustart; v.uid = c->tiles.uid; v.upos = c->tiles.upos;
            v.quantum = c->tiles.quantum; v.lidx = c->tiles.lidx; v.lself = c->tiles.lself; v.coef = c->tiles.coef;
            v.cw = c->tiles.cw; v.umax = c->tiles.umax; v.wscale = c->tiles.wscale;
        }
    } else {
        a.wflux64 = c->wflux64;
    }
    return a;
}

template <typename T> hcc_status run_step(hcc_ctx *c, double dt);
template <typename T> hcc_status run_rhs(hcc_ctx *c);
template <typename T> hcc_status run_cfl(hcc_ctx *c, double *dt_out);

hcc_status launch_check(hcc_ctx *c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c->cuda(e, what);
    return HCC_OK;
}

hcc_status read_counters(hcc_ctx *c, int count) {
    hcc_status st = c->cuda(cudaMemcpyAsync(c->h_counters, c->d_counters, sizeof(unsigned long long) * count,
                                            cudaMemcpyDeviceToHost, c->stream), "counter copy");
    if (st != HCC_OK) return st;
    return c->sync("counter sync");
}

// Implicit-part mode of the candidate of stage `i` (0-based): 1 solve, 2 explicit source evaluation, 0 none.
int implicit_mode(const hcc_ctx *c, int i) {
    if (!c->has_source) return 0;
    return std::fabs(c->tab.a[i][i]) > 1e-14 ? 1 : 2;
}

template <typename T> void apply_bcs(hcc_ctx *c, void *Y) {
    launch_bc_apply(Y, c->rhos, c->blist, c->bsrc, c->nbnd, c->M, c->f32, c->stream);
    c->launches += c->nbnd > 0;
}

// Coefficients of every candidate of the step (entry 0: stage 1; entry s+1: the candidate the flux pass of stage s
// forms), from dt and the tableau, into the pinned mirror and then to the device on the context stream.
template <typename T> void fill_coeffs(const hcc_ctx *c, double dt, StageCoeffs<T> *h) {
    const int S = c->tab.s;
    std::memset(h, 0, sizeof(StageCoeffs<T>) * (S + 1));
    h[0].dt_ii = T(dt * c->tab.a[0][0]);
    h[0].inv_dt_ii = T(implicit_mode(c, 0) == 1 ? 1.0 / (dt * c->tab.a[0][0]) : 0.0);
    for (int s = 0; s < S; ++s) {
        StageCoeffs<T> &e = h[s + 1];
        const bool fin = (s + 1 == S);
        for (int j = 0; j <= s; ++j) {
            const double at = fin ? c->tab.bt[j] : c->tab.at[s + 1][j];
            const double ai = fin ? c->tab.b[j] : c->tab.a[s + 1][j];
            e.hE[j] = at != 0.0 ? T(dt * at) : T(0);
            e.hEd[j] = at != 0.0 ? dt * at : 0.0;
            e.hI[j] = (ai != 0.0 && c->has_source) ? T(dt * ai) : T(0);
        }
        if (!fin) {
            e.dt_ii = T(dt * c->tab.a[s + 1][s + 1]);
            e.inv_dt_ii = T(implicit_mode(c, s + 1) == 1 ? 1.0 / (dt * c->tab.a[s + 1][s + 1]) : 0.0);
        }
        e.h_sub = T(c->ratio * dt);
    }
}

// Coefficients of every candidate of the step (entry 0: stage 1; entry s+1: the candidate the flux pass of stage s
// forms), from dt and the tableau (one set, or one set per cloud of a batch stepped with per-cloud dts), into the
// pinned mirror and then to the device on the context stream.
template <typename T> hcc_status upload_coeffs(hcc_ctx *c, double dt) {
    StageCoeffs<T> *h = static_cast<StageCoeffs<T> *>(c->coef_host);
    const int S = c->tab.s;
    const int sets = c->per_cloud ? int(c->step_dts.size()) : 1;
    for (int b = 0; b < sets; ++b) fill_coeffs<T>(c, c->per_cloud ? c->step_dts[b] : dt, h + size_t(b) * (S + 1));
    return c->cuda(cudaMemcpyAsync(c->coef_dev, h, sizeof(StageCoeffs<T>) * (S + 1) * sets, cudaMemcpyHostToDevice,
                                   c->stream), "coefficient upload");
}

// Kernel arguments of stage s (s = -1: the stage-1 candidate) for the current buffer assignment.
template <typename T> StageArgs<T> stage_args(hcc_ctx *c, int s) {
    const int S = c->tab.s;
    StageArgs<T> a = base_args<T>(c);
    a.Un = static_cast<const T *>(c->rhos);
    for (int q = 0; q < S; ++q) {
        a.KE[q] = static_cast<const T *>(c->KE[q]);
        a.KI[q] = static_cast<const T *>(c->KI[q]);
    }
    const StageCoeffs<T> *coef = static_cast<const StageCoeffs<T> *>(c->coef_dev);
    if (c->per_cloud) {
        a.cloud_id = c->cloud_id;
        a.coef_stride = S + 1;
    }
    // with a predictor, the final stage's full flux pass marks the tiles the next step's feature pass must visit
    if (c->mlp && s == S - 1 && !c->no_recon()) a.rough_words = c->rough;
    if (c->moving()) {
        a.mover = c->mover.kind;
        a.mv_alpha = T(c->mover.alpha);
        for (int d = 0; d < 3; ++d) {
            a.mv_v[d] = c->mover.velocity[d];
            a.mv_om[d] = c->mover.omega[d];
            a.mv_c[d] = c->mover.center[d];
        }
        a.pos = c->pos;
        a.x_n = c->x_n;
        for (int q = 0; q < S; ++q) a.KX[q] = c->KXs[q];
    }
    if (s < 0) {
        a.Ynext = static_cast<T *>(c->Y[0]);
        a.KInext = static_cast<T *>(c->KI[0]);
        a.implicit_mode = implicit_mode(c, 0);
        a.coef = coef;
        return a;
    }
    const bool fin = (s + 1 == S);
    a.U = static_cast<const T *>(c->Y[s]);
    a.K = static_cast<T *>(c->KE[s]);
    a.full = 1;
    a.form_next = 1;
    a.n_prev = s + 1;
    a.self_slot = s;
    a.coef = coef + (s + 1);
    a.Ynext = static_cast<T *>(fin ? c->cand : c->Y[s + 1]);
    if (!fin) {
        a.KInext = static_cast<T *>(c->KI[s + 1]);
        a.implicit_mode = implicit_mode(c, s + 1);
    }
    a.check = c->cfg.mood_criterion != HCC_MOOD_NONE;
    if (c->moving()) {
        a.KXout = c->KXs[s];
        a.Xnext = fin ? c->x_cand : c->Xs[s + 1];
    }
    a.check_substep = c->ratio > 0.0;
    a.KIs = c->has_source ? static_cast<const T *>(c->KI[s]) : nullptr;
    return a;
}

// The flux pass of the context's scheme (MUSCL, WENO or CentralDivergence).
using PassFn = void (*)(const void *, int64_t, cudaStream_t);
PassFn pass_op(const hcc_ctx *c) {
    return c->weno ? c->ops->weno : c->central ? c->ops->central : c->upwind ? c->ops->upwind : c->ops->flux;
}

// Full pass of stage s: reconstruction, (EPD2 neighbourhood orders), flux with its fused epilogue (the failed
// candidates go to the t list), and — without the MOOD check — the boundary conditions of the new candidate (with
// the check they are part of the decrement launch). Returns the kernels launched.
template <typename T> int enqueue_full(hcc_ctx *c, const StageArgs<T> &a, cudaStream_t st, bool prof) {
    const int64_t n = c->n;
    int k = 0;
    if (!c->no_recon()) {
        if (prof) c->prof_begin(0);
        c->ops->gather(&a, n, st);
        if (prof) c->prof_end();
        ++k;
    }
    if (c->cfg.mood_strategy == HCC_EPD2) {
        launch_nbmin(c->orders, c->nbmin, c->cnt, c->nidx, n, c->npad, nullptr, nullptr, nullptr, 0, st);
        ++k;
    }
    if (a.check && c->u2_plateau_on()) {
        launch_u2_range(a.U, n, c->M, c->f32, c->u2_keys, st);
        ++k;
    }
    if (prof) c->prof_begin(1);
    pass_op(c)(&a, n, st);
    if (prof) c->prof_end();
    ++k;
    if (!a.check) {
        launch_bc_apply(a.Ynext, c->rhos, c->blist, c->bsrc, c->nbnd, c->M, c->f32, st);
        k += (c->nbnd > 0);
    }
    return k;
}

// Boundary conditions of the candidate Y + MOOD decrement + decision (one launch). Returns the kernels launched.
int enqueue_drop(hcc_ctx *c, void *Y, cudaStream_t st, const cudaGraphConditionalHandle *h) {
    const int cap = c->cfg.max_mood_iterations > 0 ? c->cfg.max_mood_iterations : 64;
    DropArgs d{};
    d.Y = Y;
    d.rhos = c->rhos;
    d.blist = c->blist;
    d.bsrc = c->bsrc;
    d.nb = c->nbnd;
    d.M = c->M;
    // boundary conditions of the candidate: up to eight blocks per SM (a few boundary particles a thread; every
    // copy is a dependent load chain, so the pass is latency-bound and wants the whole GPU)
    d.bc_blocks = c->nbnd > 0 ? int(std::min<int64_t>((c->nbnd + HCC_BLOCK - 1) / HCC_BLOCK,
                                                      int64_t(8) * std::max(1, c->sms))) : 0;
    d.orders = c->orders;
    d.trig_step = c->trig_step;
    d.ttiles = c->ttiles;
    d.tmask = c->tmask;
    d.ctiles = c->ctiles;
    d.cmask = c->cmask;
    d.counts = c->lcounts;
    d.stats = c->mood_stats;
    d.has_handle = h != nullptr;
    if (h) d.h = *h;
    d.cap = cap;
    launch_drop_decide(d, c->f32, c->drop_blocks, st);
    return 1;
}

// One MOOD recompute (mood_checkpoint!, TimeSteppers.jl:471-475) over worklists: reconstruction of the changed
// particles, which also pushes their reach (one hop; a second for EPD2; expand_mask!, MOOD.jl:343-351; none for
// WENO, which reads no neighbour orders), then the flux and candidate of the reach. Its boundary conditions come
// with the decrement launch that follows. Schemes without a reconstruction (WENO, CentralDivergence,
// UpwindDivergence) read no neighbour orders: no gather and no reach. Returns the kernels launched.
template <typename T> int enqueue_recompute(hcc_ctx *c, const StageArgs<T> &a, cudaStream_t st, bool prof) {
    const int64_t n = c->n;
    const int hops = c->no_recon() ? 0 : (c->cfg.mood_strategy == HCC_EPD2) ? 2 : 1;
    int k = 0;
    if (c->cfg.mood_strategy == HCC_STRICT_EPD0) {
        launch_force(c->ctiles, c->cmask, c->lcounts, c->ctiles, c->orders, c->bnd, c->cnt, c->nidx, c->npad, c->forced,
                     c->fmask, c->ftiles, c->list_blocks, st);
        k += 2;
    }
    if (!c->no_recon()) {
        StageArgs<T> ga = a;
        ga.full = 0;
        ga.wtiles = c->ctiles;
        ga.wcount = &c->lcounts->c;
        ga.wmask = c->cmask;
        ga.clear_wmask = 1;
        ga.rmask = c->dmask;
        ga.rtiles = c->dtiles;
        ga.rcount = &c->lcounts->d;
        if (prof) c->prof_begin(2);
        c->ops->gather(&ga, n, st);
        if (prof) c->prof_end();
        ++k;
    }
    if (hops == 2) {
        launch_reach_hop2(c->lcounts, c->dtiles, c->dtiles, c->dmask, c->words1, c->cnt, c->nidx, c->npad,
                          c->list_blocks, st);
        launch_nbmin(c->orders, c->nbmin, c->cnt, c->nidx, n, c->npad, c->dtiles, c->words1, &c->lcounts->d1,
                     c->list_blocks, st);
        k += 3;
    }
    StageArgs<T> fa = a;
    fa.full = 0;
    fa.wtiles = hops > 0 ? c->dtiles : c->ctiles;
    fa.wcount = hops > 0 ? &c->lcounts->d : &c->lcounts->c;
    fa.wmask = hops > 0 ? c->dmask : c->cmask;
    fa.clear_wmask = 1;
    if (prof) c->prof_begin(2);
    pass_op(c)(&fa, n, st);
    if (prof) c->prof_end();
    return k + 1;
}

// Stencil-feature inputs of the current state.
FeatArgs feat_args(const hcc_ctx *c, const void *U) {
    FeatArgs fa{};
    fa.U = U;
    fa.f32 = c->f32;
    fa.D = c->D;
    fa.M = c->M;
    fa.pde = c->cfg.pde;
    fa.n = c->n;
    fa.npad = c->npad;
    fa.cnt = c->cnt;
    fa.nidx = c->nidx;
    fa.dist = c->f32 ? static_cast<const void *>(c->dist32) : static_cast<const void *>(c->dist64);
    fa.bnd = c->bnd;
    fa.h = float(c->h);
    fa.gm1 = float(c->cfg.gamma - 1.0);
    return fa;
}

// Buffers of the predictor and of the feature capture (before a step is enqueued or captured).
hcc_status ensure_learn_buffers(hcc_ctx *c) {
    hcc_status st = HCC_OK;
    if (c->capture_feat && !c->feat) st = c->alloc(c->feat, size_t(c->n) * HCC_MLP_FEATURES, "features");
    if (st == HCC_OK && c->mlp && !c->pred) {
        st = c->alloc(c->pred, size_t(c->n), "predicted mask");
        if (st == HCC_OK) st = c->cuda(cudaMemset(c->pred, 0, size_t(c->n)), "predicted mask");
        if (st == HCC_OK) st = c->alloc(c->pred_rows, size_t(c->n) * 4, "predictor rows");
        if (st == HCC_OK) st = c->alloc(c->pred_idx, size_t(c->n), "predictor rows");
        if (st == HCC_OK) st = c->alloc(c->rough, size_t(c->npad / 32), "predictor tiles");
        if (st == HCC_OK) c->reset_rough();
    }
    return st;
}

int enqueue_prologue(hcc_ctx *c, const void *args, cudaStream_t st) {
    cudaMemsetAsync(c->lcounts, 0, sizeof(ListCounts), st);
    cudaMemsetAsync(c->mood_stats, 0, sizeof(MoodStats), st);
    launch_fill_i8(c->orders, int8_t(c->max_order), c->n, st);
    cudaMemsetAsync(c->trig_step, 0, size_t(c->n), st);
    int k = 0;
    if (c->capture_feat || c->mlp) {
        const FeatArgs fa = feat_args(c, c->rhos);
        if (c->mlp) {
            // the predicted particles start the step one order lower (MOOD still judges every particle); the
            // captured training features come out of the same feature pass
            PredictOut po{};
            po.orders = c->orders;
            po.lowered = int8_t(std::max(1, c->max_order - 1));
            po.pred = c->pred;
            po.count = &c->mood_stats->predicted;
            po.thr_logit = c->thr_logit;
            po.rows = c->pred_rows;
            po.row_idx = c->pred_idx;
            po.nrows = &c->mood_stats->pred_rows;
            po.cap = c->n;
            po.rough = c->rough;
            const bool prof = c->prof && st == c->stream;
            if (prof) c->prof_begin(3);
            if (launch_predict(fa, mlp_weights(c->mlp), po, c->capture_feat ? c->feat : nullptr,
                               c->sms * 2, &c->mood_stats->tc_error, st))
                k += 2;
            if (prof) c->prof_end();
        } else if (launch_features(fa, c->feat, st)) {
            k += 1;
        }
    }
    c->ops->stage1(args, c->n, st);
    launch_bc_apply(c->Y[0], c->rhos, c->blist, c->bsrc, c->nbnd, c->M, c->f32, st);
    return k + 2 + (c->nbnd > 0);
}

// The step with the MOOD fixed points driven from the host (one counter read per decrement).
// Statistics of the step from the device record (both step forms).
hcc_status read_mood_stats(hcc_ctx *c, cudaStream_t st) {
    return c->cuda(cudaMemcpyAsync(c->mood_stats_host, c->mood_stats, sizeof(MoodStats), cudaMemcpyDeviceToHost, st),
                   "MOOD statistics");
}
void take_mood_stats(hcc_ctx *c) {
    const MoodStats &ms = *c->mood_stats_host;
    c->mood_iters = int64_t(ms.iterations);
    c->flagged = int64_t(ms.flagged);
    c->inadmissible = int64_t(ms.inadmissible);
    c->predicted = int64_t(ms.predicted);
}

hcc_status apply_positions(hcc_ctx *c, const double *src, bool full_search);

// The step with the MOOD fixed points driven from the host (one read of the decision per decrement). On a moving
// grid the positions are stage variables: after the fixed point of a candidate its stage geometry is applied
// (distances, weights and MLS caches at the new positions), and a full search follows the step.
template <typename T> hcc_status run_step_host(hcc_ctx *c, double dt) {
    const int64_t n = c->n;
    const int S = c->tab.s;
    const bool mv = c->moving();
    c->launches = 0;
    hcc_status st = upload_coeffs<T>(c, dt);
    if (st != HCC_OK) return st;
    if (mv) {
        const size_t pb = size_t(c->npad) * c->D * sizeof(double);
        if (!c->x_n) {
            const size_t cnt = size_t(c->npad) * c->D;
            if ((st = c->alloc(c->x_n, cnt, "start-of-step positions")) != HCC_OK) return st;
            if ((st = c->alloc(c->x_cand, cnt, "final positions")) != HCC_OK) return st;
            for (int q = 0; q < S; ++q) {
                if ((st = c->alloc(c->Xs[q], cnt, "stage positions")) != HCC_OK) return st;
                if ((st = c->alloc(c->KXs[q], cnt, "grid velocities")) != HCC_OK) return st;
                cudaMemsetAsync(c->KXs[q], 0, cnt * sizeof(double), c->stream);
            }
        }
        cudaMemcpyAsync(c->x_n, c->pos, pb, cudaMemcpyDeviceToDevice, c->stream);
        cudaMemcpyAsync(c->x_cand, c->pos, pb, cudaMemcpyDeviceToDevice, c->stream);
        for (int q = 0; q < S; ++q) cudaMemcpyAsync(c->Xs[q], c->pos, pb, cudaMemcpyDeviceToDevice, c->stream);
    }
    StageArgs<T> a1 = stage_args<T>(c, -1);
    c->launches += enqueue_prologue(c, &a1, c->stream);
    for (int s = 0; s < S; ++s) {
        StageArgs<T> a = stage_args<T>(c, s);
        if (s > 0 && c->cfg.reset_orders_per_stage) {     // TimeSteppers.jl:556
            launch_fill_i8(c->orders, int8_t(c->max_order), n, c->stream);
            c->launches += 1;
        }
        c->launches += enqueue_full<T>(c, a, c->stream, c->prof != 0);
        if ((st = launch_check(c, "stage kernels")) != HCC_OK) return st;
        if (!a.check) {
            if (mv && s + 1 < S &&
                (st = apply_positions(c, c->Xs[s + 1], c->mover.full_search_per_stage != 0)) != HCC_OK)
                return st;
            continue;
        }
        for (;;) {
            c->launches += enqueue_drop(c, a.Ynext, c->stream, nullptr);
            if ((st = c->cuda(cudaMemcpyAsync(c->h_lcounts, c->lcounts, sizeof(ListCounts), cudaMemcpyDeviceToHost,
                                              c->stream), "MOOD counts")) != HCC_OK) return st;
            if ((st = read_mood_stats(c, c->stream)) != HCC_OK) return st;
            if ((st = c->sync("MOOD counts")) != HCC_OK) return st;
            if (c->h_lcounts->c == 0) break;
            if (c->mood_stats_host->timeout) {
                take_mood_stats(c);
                return c->fail(HCC_ERR_TIMEOUT, "MOOD fixed point reached the iteration cap");
            }
            c->launches += enqueue_recompute<T>(c, a, c->stream, c->prof != 0);
            if ((st = launch_check(c, "MOOD recompute")) != HCC_OK) return st;
        }
        launch_count_inadmissible(c->inadm, c->bnd, n, &c->mood_stats->inadmissible, c->stream);
        c->launches += 1;
        if (mv && s + 1 < S && (st = apply_positions(c, c->Xs[s + 1], c->mover.full_search_per_stage != 0)) != HCC_OK)
            return st;
    }
    if (mv) {
        // final positions; full search with periodic re-wrap for the next step (TimeSteppers.jl:571-575), then the
        // volume estimator (:574)
        if ((st = apply_positions(c, c->x_cand, true)) != HCC_OK) return st;
        if (!c->mover.keep_volumes &&
            (st = hcc_update_volumes(c, c->mover.shepard_sweeps > 0 ? c->mover.shepard_sweeps : 1)) != HCC_OK)
            return st;
    }
    if ((st = read_mood_stats(c, c->stream)) != HCC_OK) return st;
    st = c->sync("step");
    if (st != HCC_OK) return st;
    take_mood_stats(c);
    if (c->mood_stats_host->tc_error) return c->fail(HCC_ERR_TIMEOUT, "predictor: a tensor-core wait gave up");
    c->feat_valid = c->capture_feat != 0;
    std::swap(c->rhos, c->cand);
    ++c->steps;
    c->launches_total += c->launches;
    if (c->prof) {
        c->prof_collect();
        c->times.steps += 1;
    }
    return HCC_OK;
}

// Capture of one step as a CUDA graph: every MOOD fixed point is a conditional WHILE node whose body (recompute,
// then the decrement launch that also decides) repeats until the decision finds no changed order, so the host never
// waits inside the step. The dt-dependent coefficients are read from device memory, so one graph serves every dt;
// two graphs alternate with the start-of-step / candidate buffers.
template <typename T> hcc_status capture_step(hcc_ctx *c, int parity) {
    const int S = c->tab.s;
    auto &G = c->graphs[parity];
    G.reset();
    cudaStream_t st = c->stream;
    hcc_status rs = c->cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (rs != HCC_OK) return rs;
    int launches = 0, body_launches = 0;
    cudaError_t err = cudaSuccess;
    StageArgs<T> a1 = stage_args<T>(c, -1);
    launches += enqueue_prologue(c, &a1, st);
    for (int s = 0; s < S && err == cudaSuccess; ++s) {
        StageArgs<T> a = stage_args<T>(c, s);
        if (s > 0 && c->cfg.reset_orders_per_stage) {     // TimeSteppers.jl:556
            launch_fill_i8(c->orders, int8_t(c->max_order), c->n, st);
            launches += 1;
        }
        launches += enqueue_full<T>(c, a, st, false);
        if (!a.check) continue;
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        err = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, nullptr, nullptr, nullptr);
        if (err != cudaSuccess) break;
        cudaGraphConditionalHandle h;
        err = cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault);
        if (err != cudaSuccess) break;
        launches += enqueue_drop(c, a.Ynext, st, &h);
        err = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &ndeps);
        if (err != cudaSuccess) break;
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        err = cudaGraphAddNode(&node, cg, deps, nullptr, ndeps, &np);
        if (err != cudaSuccess) break;
        cudaGraph_t body = np.conditional.phGraph_out[0];
        err = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (err != cudaSuccess) break;
        err = cudaStreamBeginCaptureToGraph(c->stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) break;
        int bl = enqueue_recompute<T>(c, a, c->stream2, false);
        bl += enqueue_drop(c, a.Ynext, c->stream2, &h);
        body_launches += bl;
        cudaGraph_t body_out = nullptr;
        err = cudaStreamEndCapture(c->stream2, &body_out);
        if (err != cudaSuccess) break;
        // interior candidates that are not admissible once the fixed point has converged
        launch_count_inadmissible(c->inadm, c->bnd, c->n, &c->mood_stats->inadmissible, st);
        launches += 1;
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(c->mood_stats_host, c->mood_stats, sizeof(MoodStats),
                                                  cudaMemcpyDeviceToHost, st);
    cudaGraph_t graph = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (err == cudaSuccess) err = e2;
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaGraphInstantiate(&G.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (err != cudaSuccess) {
        cudaGetLastError();
        G.reset();
        return c->cuda(err, "step graph capture");
    }
    G.rhos = c->rhos;
    G.launches = launches;
    G.body_launches = body_launches;
    return HCC_OK;
}

template <typename T> hcc_status run_step_graph(hcc_ctx *c, double dt) {
    int parity = -1;
    for (int q = 0; q < 2; ++q)
        if (c->graphs[q].exec && c->graphs[q].rhos == c->rhos) parity = q;
    hcc_status st;
    if (parity < 0) {
        parity = (c->graphs[0].exec == nullptr) ? 0 : 1;
        if ((st = capture_step<T>(c, parity)) != HCC_OK) return st;
    }
    auto &G = c->graphs[parity];
    if ((st = upload_coeffs<T>(c, dt)) != HCC_OK) return st;
    if ((st = c->cuda(cudaGraphLaunch(G.exec, c->stream), "step graph launch")) != HCC_OK) return st;
    if ((st = c->sync("step")) != HCC_OK) return st;
    take_mood_stats(c);
    const int nchk = c->n_checkpoints();
    c->launches = G.launches + (nchk > 0 ? c->mood_iters * (G.body_launches / nchk) : 0);
    c->launches_total += c->launches;
    if (c->mood_stats_host->timeout) return c->fail(HCC_ERR_TIMEOUT, "MOOD fixed point reached the iteration cap");
    if (c->mood_stats_host->tc_error) return c->fail(HCC_ERR_TIMEOUT, "predictor: a tensor-core wait gave up");
    c->feat_valid = c->capture_feat != 0;
    std::swap(c->rhos, c->cand);
    ++c->steps;
    ++c->graph_steps;
    return HCC_OK;
}

template <typename T> hcc_status run_step(hcc_ctx *c, double dt) {
    c->feat_valid = false;
    if (c->graph_per_cloud != int(c->per_cloud)) {   // graphs hold the coefficient addressing of their mode
        c->drop_graphs();
        c->graph_per_cloud = int(c->per_cloud);
    }
    hcc_status lst = ensure_learn_buffers(c);
    if (lst != HCC_OK) return lst;
    if (c->use_graphs && !c->prof && !c->moving()) {
        hcc_status st = run_step_graph<T>(c, dt);
        if (st != HCC_ERR_CUDA || c->graphs_failed) return st;
        // a graph that cannot be captured or launched on this driver: the host-driven step for this context
        c->graphs_failed = true;
        c->use_graphs = false;
        cudaGetLastError();
    }
    return run_step_host<T>(c, dt);
}

template <typename T> hcc_status run_rhs(hcc_ctx *c) {
    const int64_t n = c->n;
    launch_fill_i8(c->orders, int8_t(c->max_order), n, c->stream);
    StageArgs<T> a = base_args<T>(c);
    a.U = static_cast<const T *>(c->rhos);
    a.K = static_cast<T *>(c->KE[0]);
    a.full = 1;
    if (!c->no_recon()) c->ops->gather(&a, n, c->stream);
    if (c->cfg.mood_strategy == HCC_EPD2)
        launch_nbmin(c->orders, c->nbmin, c->cnt, c->nidx, n, c->npad, nullptr, nullptr, nullptr, 0, c->stream);
    pass_op(c)(&a, n, c->stream);
    hcc_status st = launch_check(c, "rhs kernels");
    if (st != HCC_OK) return st;
    return c->sync("rhs");
}

template <typename T> hcc_status run_cfl(hcc_ctx *c, double *dt_out) {
    StageArgs<T> a = base_args<T>(c);
    a.U = static_cast<const T *>(c->rhos);
    const unsigned long long inf_bits = 0x7ff0000000000000ull;
    hcc_status st = c->cuda(cudaMemcpyAsync(c->d_counters + 2, &inf_bits, sizeof(inf_bits), cudaMemcpyHostToDevice,
                                            c->stream), "dt init");
    if (st != HCC_OK) return st;
    c->ops->cfl(&a, c->n, c->d_counters + 2, c->stream);
    c->launches = 1;
    c->launches_total += 1;
    if ((st = launch_check(c, "cfl kernel")) != HCC_OK) return st;
    st = c->cuda(cudaMemcpyAsync(c->h_counters + 2, c->d_counters + 2, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, c->stream), "dt copy");
    if (st != HCC_OK) return st;
    if ((st = c->sync("cfl")) != HCC_OK) return st;
    double v;
    std::memcpy(&v, &c->h_counters[2], sizeof(v));
    *dt_out = v;
    return HCC_OK;
}

const StageOps *find_ops(const hcc_config &f, int rdeg) {
    if (f.precision == HCC_FP32)
        return rdeg == 1 ? stage_ops_f32_r1(f.dim, f.n_vars, f.pde) : stage_ops_f32_r2(f.dim, f.n_vars, f.pde);
    return rdeg == 1 ? stage_ops_f64_r1(f.dim, f.n_vars, f.pde) : stage_ops_f64_r2(f.dim, f.n_vars, f.pde);
}

}  // namespace

extern "C" {

void hcc_config_defaults(hcc_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->abi_version = HCC_ABI_VERSION;
    cfg->dim = 2;
    cfg->n_vars = 1;
    cfg->pde = HCC_PDE_ADVECTION;
    cfg->precision = HCC_FP64;
    cfg->muscl_order = 2;
    cfg->div_order = 0;
    cfg->mood_criterion = HCC_MOOD_U1;
    cfg->mood_strategy = HCC_EPD1;
    cfg->tableau = HCC_TAB_RK3_SSP;
    cfg->mood_substeps = 1;
    cfg->max_mood_iterations = 64;
    cfg->weight_alpha = 1.0;
    cfg->gamma = 1.4;
    cfg->bgk_epsilon = 1e-4;
    cfg->bgk_coefficient = 1.0;
    cfg->bgk_interior_factor = 2.0;
    cfg->u2_plateau = 1e-3;
    cfg->u2_ratio = 0.5;
    for (int d = 0; d < HCC_MAX_DIM; ++d) { cfg->dx[d] = 1.0; cfg->canvas_max[d] = 1.0; cfg->domain_max[d] = 1.0; }
}

const char *hcc_status_string(hcc_status s) {
    int k = int(s);
    return (k >= 0 && k < 8) ? kStatusNames[k] : "HCC_UNKNOWN";
}

const char *hcc_last_error(const hcc_ctx *ctx) { return ctx ? ctx->err.c_str() : g_null_ctx_error; }

hcc_status hcc_create(const hcc_config *cfg, int64_t capacity, hcc_ctx **out) {
    if (!cfg || !out) return HCC_ERR_INVALID;
    *out = nullptr;
    hcc_ctx *c = new (std::nothrow) hcc_ctx();
    if (!c) return HCC_ERR_INVALID;
    *out = c;
    c->cfg = *cfg;
    const hcc_config &f = c->cfg;
    if (f.abi_version != HCC_ABI_VERSION) return c->fail(HCC_ERR_INVALID, "abi_version mismatch");
    c->D = f.dim;
    // tile staging by default where it measured faster: the 3-D stencils (K ~ 66; flux 7.05 vs 10.4 ms at 8.0M
    // points); 2-D stencils (K ~ 19) ran faster stream-fed (flux 0.21 vs 0.30 ms at 1.0M)
    c->tile_enabled = f.dim == 3 ? 1 : 0;
    c->M = f.n_vars;
    c->f32 = f.precision == HCC_FP32;
    c->capacity = capacity;
    if (c->D < 1 || c->D > 3) return c->fail(HCC_ERR_INVALID, "dim must be 1, 2 or 3");
    if (c->M < 1 || c->M > HCC_MAX_VARS) return c->fail(HCC_ERR_INVALID, "n_vars out of range");
    if (f.pde == HCC_PDE_EULER && c->M != c->D + 2) return c->fail(HCC_ERR_INVALID, "Euler needs n_vars = dim + 2");
    if (f.precision != HCC_FP64 && f.precision != HCC_FP32) return c->fail(HCC_ERR_INVALID, "unknown precision");
    if (!(f.radius > 0.0)) return c->fail(HCC_ERR_INVALID, "radius must be positive");
    if (f.muscl_order < 1 || f.muscl_order > 3) return c->fail(HCC_ERR_UNSUPPORTED, "muscl_order must be 1, 2 or 3");
    if (f.mood_criterion < HCC_MOOD_NONE || f.mood_criterion > HCC_MOOD_U2) return c->fail(HCC_ERR_INVALID, "unknown MOOD criterion");
    if (f.mood_strategy < HCC_EPD_NONE || f.mood_strategy > HCC_STRICT_EPD0) return c->fail(HCC_ERR_INVALID, "unknown MOOD strategy");
    if (f.flux < HCC_FLUX_RUSANOV || f.flux > HCC_FLUX_ALIGNED) return c->fail(HCC_ERR_INVALID, "unknown numerical flux");
    if (f.pde == HCC_PDE_BGK && !(f.bgk_epsilon > 0.0)) return c->fail(HCC_ERR_INVALID, "bgk_epsilon must be positive");
    if (f.limiter < HCC_LIMITER_NONE || f.limiter > HCC_LIMITER_VK_HARD) return c->fail(HCC_ERR_INVALID, "unknown limiter");
    if (f.scheme != HCC_SCHEME_MUSCL && f.scheme != HCC_SCHEME_WENO && f.scheme != HCC_SCHEME_CENTRAL &&
        f.scheme != HCC_SCHEME_UPWIND)
        return c->fail(HCC_ERR_INVALID, "unknown scheme");
    c->max_order = f.muscl_order;
    c->DO = f.div_order > c->max_order ? c->max_order : f.div_order;
    if (c->DO < 0) return c->fail(HCC_ERR_INVALID, "div_order must be >= 0");
    c->rdeg = std::max(1, c->max_order - 1);
    c->Br = basis_count(c->D, c->rdeg);
    c->full_div = div_idx(c->D, c->DO == 0 ? c->max_order : c->DO);
    c->ddeg = c->full_div - 1;
    c->Bd = basis_count(c->D, c->ddeg) + 1;
    if (c->ddeg > 3) return c->fail(HCC_ERR_UNSUPPORTED, "divergence degree above 3");
    c->need_dw1 = (c->DO == 0 && c->full_div > 2) ? 1 : 0;
    double h = f.dx[0];
    for (int d = 1; d < c->D; ++d) h = std::min(h, f.dx[d]);
    if (!(h > 0.0)) return c->fail(HCC_ERR_INVALID, "dx must be positive");
    c->invL = 1.0 / h;
    c->h = h;
    c->weno = f.scheme == HCC_SCHEME_WENO;
    c->central = f.scheme == HCC_SCHEME_CENTRAL;
    c->upwind = f.scheme == HCC_SCHEME_UPWIND ? f.upwind_algorithm : 0;
    if (f.scheme == HCC_SCHEME_UPWIND) {
        if (c->M != 1 || f.pde != HCC_PDE_ADVECTION)
            return c->fail(HCC_ERR_INVALID, "UpwindDivergence :Tiwari / :Praveen are scalar (linear advection, n_vars 1)");
        if (c->max_order != 1) return c->fail(HCC_ERR_INVALID, "UpwindDivergence is first order (muscl_order 1)");
        if (c->upwind != HCC_UPWIND_TIWARI && c->upwind != HCC_UPWIND_PRAVEEN)
            return c->fail(HCC_ERR_INVALID, "unknown upwind algorithm");
        if (c->upwind == HCC_UPWIND_PRAVEEN && c->D != 2) return c->fail(HCC_ERR_INVALID, "Praveen is two-dimensional");
        for (int d = 1; d < c->D; ++d)
            if (f.dx[d] != f.dx[0])
                return c->fail(HCC_ERR_UNSUPPORTED, "UpwindDivergence with anisotropic spacing");
    }
    c->qmax = c->DO == 0 ? c->max_order : c->DO;
    if (c->weno && c->max_order > 2 && c->M > 1)
        return c->fail(HCC_ERR_UNSUPPORTED, "WENO for systems: orders 1 and 2 (degree-1 fits)");
    if (c->central && f.mood_criterion == HCC_MOOD_U2)
        return c->fail(HCC_ERR_INVALID, "MOODu2 needs cached reconstruction gradients (MUSCL)");
    c->tab = make_tableau(f.tableau);
    if (c->tab.s == 0) return c->fail(HCC_ERR_INVALID, "unknown tableau");
    c->has_source = f.pde == HCC_PDE_BGK;
    c->ssp_C = ssp_coefficient(c->tab);
    if (c->has_source && !has_implicit_part(c->tab)) {
        // implicit sources with an explicit tableau: applied explicitly with the explicit weights
        // (_explicit_implicit_part, TimeSteppers.jl:236-237)
        for (int i = 0; i < c->tab.s; ++i) {
            for (int j = 0; j < c->tab.s; ++j) c->tab.a[i][j] = c->tab.at[i][j];
            c->tab.c[i] = c->tab.ct[i];
            c->tab.b[i] = c->tab.bt[i];
        }
    }
    c->ratio = (f.mood_substeps && c->ssp_C > 0.0 && f.mood_criterion != HCC_MOOD_NONE) ? 1.0 / c->ssp_C : 0.0;
    c->ops = find_ops(f, (c->central || c->upwind) ? 1 : c->rdeg);
    if (!c->ops) return c->fail(HCC_ERR_UNSUPPORTED, "this (dim, n_vars, pde) combination is not instantiated");
    if (c->weno && (!c->ops->weno || c->max_order > 3))
        return c->fail(HCC_ERR_UNSUPPORTED, "WENO of this dimension / order is not instantiated");
    if (c->upwind && !c->ops->upwind)
        return c->fail(HCC_ERR_UNSUPPORTED, "UpwindDivergence of this combination is not instantiated");
    if (c->central && !c->ops->central)
        return c->fail(HCC_ERR_UNSUPPORTED, "CentralDivergence of this combination is not instantiated");
    hcc_status st = c->cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
    if (st != HCC_OK) return st;
    if ((st = c->alloc(c->d_counters, 8, "counters")) != HCC_OK) return st;
    if ((st = c->cuda(cudaMallocHost(reinterpret_cast<void **>(&c->h_counters), 8 * sizeof(unsigned long long)),
                      "pinned counters")) != HCC_OK) return st;
    if ((st = c->alloc(c->d_mass, HCC_MAX_VARS, "mass")) != HCC_OK) return st;
    if ((st = c->cuda(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking), "capture stream")) != HCC_OK)
        return st;
    const size_t coef_bytes = sizeof(StageCoeffs<double>) * (HCC_MAX_STAGES + 1);
    if ((st = c->valloc(c->coef_dev, coef_bytes, "stage coefficients")) != HCC_OK) return st;
    if ((st = c->cuda(cudaMallocHost(&c->coef_host, coef_bytes), "pinned stage coefficients")) != HCC_OK) return st;
    if ((st = c->alloc(c->mood_stats, 1, "MOOD statistics")) != HCC_OK) return st;
    if ((st = c->alloc(c->lcounts, 1, "MOOD worklist counts")) != HCC_OK) return st;
    if ((st = c->alloc(c->u2_keys, 2 * HCC_MAX_VARS + 1, "MOODu2 range")) != HCC_OK) return st;
    cudaMemsetAsync(c->lcounts, 0, sizeof(ListCounts), c->stream);
    if ((st = c->cuda(cudaMallocHost(reinterpret_cast<void **>(&c->h_lcounts), sizeof(ListCounts)),
                      "pinned MOOD worklist counts")) != HCC_OK) return st;
    {
        int dev = 0, sms = 0;
        if ((st = c->cuda(cudaGetDevice(&dev), "device")) != HCC_OK) return st;
        if ((st = c->cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count")) != HCC_OK)
            return st;
        c->sms = std::max(1, sms);
        c->apply_tuning();   // worklist passes: a few resident blocks per SM, grid-stride
    }
    if ((st = c->cuda(cudaMallocHost(reinterpret_cast<void **>(&c->mood_stats_host), sizeof(MoodStats)),
                      "pinned MOOD statistics")) != HCC_OK) return st;
    return HCC_OK;
}

hcc_status hcc_destroy(hcc_ctx *ctx) {
    if (!ctx) return HCC_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->free_particles();
    ctx->free_slots();
    ctx->free_bins();
    dfree(ctx->d_counters);
    dfree(ctx->d_mass);
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    ctx->drop_graphs();
    if (ctx->coef_dev) cudaFree(ctx->coef_dev);
    if (ctx->coef_host) cudaFreeHost(ctx->coef_host);
    dfree(ctx->mood_stats);
    dfree(ctx->lcounts);
    dfree(ctx->u2_keys);
    if (ctx->h_lcounts) cudaFreeHost(ctx->h_lcounts);
    if (ctx->mood_stats_host) cudaFreeHost(ctx->mood_stats_host);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HCC_OK;
}

hcc_status hcc_upload_cloud(hcc_ctx *c, int64_t n, const double *pos, const uint8_t *is_boundary, const int32_t *tags,
                            const double *volumes) {
    if (!c) return HCC_ERR_INVALID;
    if (!c->ops) return c->fail(HCC_ERR_STATE, "context was not created successfully");
    if (n < 0 || (n > 0 && (!pos || !is_boundary || !tags))) return c->fail(HCC_ERR_INVALID, "bad cloud arguments");
    if (c->capacity > 0 && n > c->capacity) return c->fail(HCC_ERR_CAPACITY, "particle count above the capacity");
    if (n > int64_t(INT32_MAX) - 64) return c->fail(HCC_ERR_CAPACITY, "particle count above 2^31");
    c->free_particles();
    c->free_slots();
    c->have_cloud = c->have_nb = c->have_geom = c->have_state = false;
    c->batch_offsets.clear();
    c->n = n;
    c->npad = ((n + 31) / 32) * 32;
    const int D = c->D, M = c->M;
    const int64_t np = c->npad;
    std::vector<double> soa(size_t(D) * np, 0.0);
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < D; ++d) soa[d * np + i] = pos[i * D + d];
    c->h_bnd.assign(is_boundary, is_boundary + n);
    c->h_tags.assign(tags, tags + n);
    c->n_interior = 0;
    for (int64_t i = 0; i < n; ++i) c->n_interior += is_boundary[i] ? 0 : 1;
    std::vector<double> v(size_t(std::max<int64_t>(n, 1)), 1.0);
    double v0 = 1.0;
    for (int d = 0; d < D; ++d) v0 *= c->cfg.dx[d];
    for (int64_t i = 0; i < n; ++i) v[i] = volumes ? volumes[i] : v0;
    hcc_status st;
#define HCC_TRY(x) do { if ((st = (x)) != HCC_OK) return st; } while (0)
    HCC_TRY(c->alloc(c->pos, size_t(D) * np, "positions"));
    HCC_TRY(c->alloc(c->pos32, size_t(D) * np, "FP32 positions"));
    HCC_TRY(c->alloc(c->pmax32, 1, "largest coordinate"));
    HCC_TRY(c->alloc(c->bnd, np, "is_boundary"));
    HCC_TRY(c->alloc(c->tags, np, "tags"));
    HCC_TRY(c->alloc(c->vol, np, "volumes"));
    HCC_TRY(c->alloc(c->bin_of, np, "bin_of"));
    HCC_TRY(c->alloc(c->cellp, np, "cell particles"));
    HCC_TRY(c->alloc(c->cnt, np, "counts"));
    HCC_TRY(c->alloc(c->ok_r, np, "ok_r"));
    HCC_TRY(c->alloc(c->ok_d, np, "ok_d"));
    HCC_TRY(c->alloc(c->ok_1, np, "ok_1"));
    HCC_TRY(c->alloc(c->inv_r64, size_t(np) * c->Br * c->Br, "inv_r"));
    HCC_TRY(c->alloc(c->inv_d64, size_t(np) * c->Bd * c->Bd, "inv_d"));
    if (c->f32) HCC_TRY(c->alloc(c->inv_r32, size_t(np) * c->Br * c->Br, "inv_r32"));
    HCC_TRY(c->alloc(c->status, np, "status"));
    HCC_TRY(c->alloc(c->status2, np, "status2"));
    HCC_TRY(c->alloc(c->root, np, "root"));
    const size_t sb = size_t(np) * M * c->esz();
    HCC_TRY(c->valloc(c->rhos, sb, "rhos"));
    HCC_TRY(c->valloc(c->cand, sb, "candidate"));
    HCC_TRY(c->valloc(c->grad, size_t(np) * c->Br * M * c->esz(), "gradients"));
    HCC_TRY(c->valloc(c->xfer, size_t(np) * M * sizeof(double), "conversion buffer"));
    for (int s = 0; s < c->tab.s; ++s) {
        HCC_TRY(c->valloc(c->Y[s], sb, "stage states"));
        HCC_TRY(c->valloc(c->KE[s], sb, "stage K_E"));
        HCC_TRY(c->valloc(c->KI[s], sb, "stage K_I"));
        cudaMemsetAsync(c->KE[s], 0, sb, c->stream);
        cudaMemsetAsync(c->KI[s], 0, sb, c->stream);
    }
    cudaMemsetAsync(c->grad, 0, size_t(np) * c->Br * M * c->esz(), c->stream);
    cudaMemsetAsync(c->rhos, 0, sb, c->stream);
    HCC_TRY(c->alloc(c->orders, np, "orders"));
    HCC_TRY(c->alloc(c->nbmin, np, "nbmin"));
    for (uint8_t **p : {&c->trig_step, &c->inadm}) {
        HCC_TRY(c->alloc(*p, np, "masks"));
        cudaMemsetAsync(*p, 0, np, c->stream);
    }
    const int64_t ntiles = np / 32;
    for (int32_t **p : {&c->ttiles, &c->ctiles, &c->dtiles, &c->ftiles}) HCC_TRY(c->alloc(*p, ntiles, "MOOD tile lists"));
    HCC_TRY(c->alloc(c->forced, np, "StrictEPD0 offers"));
    cudaMemsetAsync(c->forced, 0x7f, size_t(np) * sizeof(int32_t), c->stream);
    for (uint32_t **p : {&c->tmask, &c->cmask, &c->dmask, &c->words1, &c->fmask}) {
        HCC_TRY(c->alloc(*p, ntiles, "MOOD tile words"));
        cudaMemsetAsync(*p, 0, size_t(ntiles) * sizeof(uint32_t), c->stream);
    }
    launch_fill_i8(c->orders, int8_t(c->max_order), np, c->stream);
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->pos, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream), "upload positions"));
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->bnd, is_boundary, n, cudaMemcpyHostToDevice, c->stream), "upload is_boundary"));
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->tags, tags, n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream), "upload tags"));
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->vol, v.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "upload volumes"));
    HCC_TRY(c->sync("upload cloud"));
    c->have_cloud = true;
    return HCC_OK;
}

hcc_status hcc_build_neighbours(hcc_ctx *c) {
    if (c) c->drop_graphs();
    if (!c) return HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud uploaded");
    const hcc_config &f = c->cfg;
    const int D = c->D;
    hcc_status st;
    // GlobalBins (NeighborLogic.jl:22-40) and the 3^D window of every bin (_fill_bin_neighbors!, :43-76), on the host
    c->nbins = 1;
    for (int d = 0; d < 3; ++d) { c->dims[d] = 1; c->csize[d] = 1.0; }
    for (int d = 0; d < D; ++d) {
        double sz = f.canvas_max[d] - f.canvas_min[d];
        if (!(sz > 0.0)) return c->fail(HCC_ERR_INVALID, "empty canvas");
        c->dims[d] = std::max(1, int(std::floor(sz / f.radius)));
        c->csize[d] = sz / double(c->dims[d]);
        c->nbins *= c->dims[d];
    }
    if (c->nbins > (int64_t(1) << 30)) return c->fail(HCC_ERR_CAPACITY, "too many cell-list bins");
    c->noff = D == 1 ? 3 : (D == 2 ? 9 : 27);
    std::vector<int64_t> binnb(size_t(c->nbins) * c->noff);
    for (int64_t b = 0; b < c->nbins; ++b) {
        int cart[3] = {0, 0, 0};
        int64_t r = b;
        for (int d = 0; d < D; ++d) { cart[d] = int(r % c->dims[d]); r /= c->dims[d]; }
        int64_t raw[27];
        for (int w = 0; w < c->noff; ++w) {
            int q = w;
            bool valid = true;
            int64_t lin = 0, stride = 1;
            for (int d = 0; d < D; ++d) {
                int off = q % 3 - 1;
                q /= 3;
                int nc = cart[d] + off;
                if (nc < 0 || nc >= c->dims[d]) {
                    if (f.periodic[d]) nc = ((nc % c->dims[d]) + c->dims[d]) % c->dims[d];
                    else { valid = false; nc = 0; }
                }
                lin += nc * stride;
                stride *= c->dims[d];
            }
            raw[w] = valid ? lin : c->nbins;
        }
        for (int w = 0; w < c->noff; ++w) {
            bool rep = false;
            for (int k = 0; k < w; ++k) rep = rep || raw[k] == raw[w];
            binnb[size_t(b) * c->noff + w] = rep ? c->nbins : raw[w];
        }
    }
    c->free_bins();
    HCC_TRY(c->alloc(c->binnb, binnb.size(), "bin windows"));
    HCC_TRY(c->alloc(c->cell_count, c->nbins + 1, "cell counts"));
    HCC_TRY(c->alloc(c->cell_cursor, c->nbins + 1, "cell cursor"));
    HCC_TRY(c->alloc(c->cell_start, c->nbins + 2, "cell start"));
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->binnb, binnb.data(), binnb.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                    c->stream), "upload bin windows"));
    SearchArgs a{};
    a.n = c->n; a.npad = c->npad; a.D = D; a.pos = c->pos;
    const double R = f.radius;
    for (int d = 0; d < 3; ++d) {
        a.periodic[d] = d < D ? f.periodic[d] : 0;
        a.cmin[d] = f.canvas_min[d];
        a.csize[d] = c->csize[d];
        a.dims[d] = c->dims[d];
        double L = f.domain_max[d] - f.domain_min[d];
        a.Lphys[d] = L;
        a.Lwrap[d] = (d < D && f.periodic[d]) ? L : 0.0;
        a.invLwrap[d] = (d < D && f.periodic[d]) ? 1.0 / L : 0.0;
    }
    a.nbins = c->nbins; a.noff = c->noff; a.binnb = c->binnb;
    a.bin_of = c->bin_of; a.cell_count = c->cell_count; a.cell_start = c->cell_start; a.cell_cursor = c->cell_cursor;
    a.cellp = c->cellp; a.cnt = c->cnt;
    a.R_sq = R * R;
    a.alpha = f.weight_alpha;
    a.invR2 = 1.0 / (R * R);
    a.pos32 = c->pos32;
    a.pmax = c->pmax32;
    a.Lmax = 0.0;
    for (int d = 0; d < 3; ++d) {
        a.L32[d] = float(a.Lwrap[d]);
        a.invL32[d] = float(a.invLwrap[d]);
        a.Lmax = std::max(a.Lmax, a.Lwrap[d]);
    }
    if ((st = search_bins(a, c->stream, c->err)) != HCC_OK) return st;
    if ((st = search_count(a, c->stream, c->d_counters + 3, c->err)) != HCC_OK) return st;
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->h_counters + 3, c->d_counters + 3, 2 * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, c->stream), "search stats"));
    HCC_TRY(c->sync("neighbour count"));
    const int64_t kmax = int64_t(c->h_counters[3]);
    c->total_nb = int64_t(c->h_counters[4]);
    if (f.slot_capacity > 0 && kmax > f.slot_capacity)
        return c->fail(HCC_ERR_CAPACITY, "max neighbours above the reserved slot capacity");
    c->free_slots();
    c->kmax = int(kmax);
    const size_t slots = size_t(std::max<int64_t>(kmax, 1)) * c->npad;
    HCC_TRY(c->alloc(c->nidx, slots, "neighbour indices"));
    HCC_TRY(c->alloc(c->w64, slots, "neighbour weights"));
    HCC_TRY(c->alloc(c->dist64, slots * D, "neighbour distances"));
    a.nidx = c->nidx; a.w = c->w64; a.dist = c->dist64; a.kmax = c->kmax;
    if ((st = search_write(a, c->stream, c->err)) != HCC_OK) return st;
    HCC_TRY(c->sync("neighbour write"));
    c->launches_total += 7;
    {
        std::vector<int32_t> cnt(c->n);
        HCC_TRY(c->cuda(cudaMemcpy(cnt.data(), c->cnt, c->n * 4, cudaMemcpyDeviceToHost), "counts"));
        int32_t mn = INT32_MAX;
        for (int64_t i = 0; i < c->n; ++i) if (!c->h_bnd[i]) mn = std::min(mn, cnt[i]);
        c->min_nb_interior = mn == INT32_MAX ? 0 : mn;
    }
    c->have_nb = true;
    c->have_geom = false;
    return HCC_OK;
}

hcc_status hcc_set_mover(hcc_ctx *c, const hcc_mover *mv) {
    if (!c || !mv) return c ? c->fail(HCC_ERR_INVALID, "null mover") : HCC_ERR_INVALID;
    if (mv->kind < HCC_MOVER_NONE || mv->kind > HCC_MOVER_PRESCRIBED) return c->fail(HCC_ERR_INVALID, "unknown mover");
    const bool fluid = c->cfg.pde == HCC_PDE_EULER || (c->cfg.pde == HCC_PDE_ADVECTION && c->M == 1);
    if ((mv->kind == HCC_MOVER_LAGRANGIAN || mv->kind == HCC_MOVER_SCALED) && !fluid)
        return c->fail(HCC_ERR_UNSUPPORTED, "this system defines no fluid velocity (Lagrangian movers)");
    if (mv->kind != HCC_MOVER_NONE && c->no_recon())
        return c->fail(HCC_ERR_UNSUPPORTED, "moving grids with WENO / CentralDivergence / UpwindDivergence");
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->drop_graphs();
    if (mv->kind != HCC_MOVER_NONE) c->tiles.release();   // moving positions: the full passes read the slot streams
    c->mover = *mv;
    c->free_mover_buffers();
    return HCC_OK;
}

hcc_status hcc_download_positions(hcc_ctx *c, double *pos) {
    if (!c || !pos) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud");
    const int D = c->D;
    std::vector<double> soa(size_t(D) * c->npad);
    hcc_status st;
    HCC_TRY(c->sync("positions"));
    HCC_TRY(c->cuda(cudaMemcpy(soa.data(), c->pos, soa.size() * sizeof(double), cudaMemcpyDeviceToHost), "positions"));
    for (int64_t i = 0; i < c->n; ++i)
        for (int d = 0; d < D; ++d) pos[i * D + d] = soa[size_t(d) * c->npad + i];
    return HCC_OK;
}

// Snapshot file: magic, then a header of int64 fields, then positions (n x D FP64, SoA as held), state (n x M in the
// context's precision), orders (int8 n), MOOD flags (uint8 n).
static const char kSnapMagic[8] = {'H', 'C', 'C', 'S', 'N', 'A', 'P', '1'};
struct SnapHeader {
    int64_t abi, dim, n_vars, pde, precision, n, npad, steps;
};

hcc_status hcc_save_snapshot(hcc_ctx *c, const char *path) {
    if (!c || !path) return c ? c->fail(HCC_ERR_INVALID, "null path") : HCC_ERR_INVALID;
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    hcc_status st;
    HCC_TRY(c->sync("snapshot"));
    const int64_t n = c->n, np = c->npad;
    std::vector<double> pos(size_t(np) * c->D);
    std::vector<char> U(size_t(n) * c->M * c->esz());
    std::vector<int8_t> ord(n);
    std::vector<uint8_t> flags(n);
    HCC_TRY(c->cuda(cudaMemcpy(pos.data(), c->pos, pos.size() * sizeof(double), cudaMemcpyDeviceToHost), "positions"));
    HCC_TRY(c->cuda(cudaMemcpy(U.data(), c->rhos, U.size(), cudaMemcpyDeviceToHost), "state"));
    HCC_TRY(c->cuda(cudaMemcpy(ord.data(), c->orders, n, cudaMemcpyDeviceToHost), "orders"));
    HCC_TRY(c->cuda(cudaMemcpy(flags.data(), c->trig_step, n, cudaMemcpyDeviceToHost), "flags"));
    SnapHeader h{HCC_ABI_VERSION, c->D, c->M, c->cfg.pde, c->cfg.precision, n, np, c->steps};
    FILE *f = std::fopen(path, "wb");
    if (!f) return c->fail(HCC_ERR_INVALID, std::string("cannot open ") + path);
    bool ok = std::fwrite(kSnapMagic, 1, 8, f) == 8 && std::fwrite(&h, sizeof(h), 1, f) == 1 &&
              std::fwrite(pos.data(), sizeof(double), pos.size(), f) == pos.size() &&
              std::fwrite(U.data(), 1, U.size(), f) == U.size() && std::fwrite(ord.data(), 1, n, f) == size_t(n) &&
              std::fwrite(flags.data(), 1, n, f) == size_t(n);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? HCC_OK : c->fail(HCC_ERR_INVALID, std::string("write failed: ") + path);
}

hcc_status hcc_load_snapshot(hcc_ctx *c, const char *path) {
    if (!c || !path) return c ? c->fail(HCC_ERR_INVALID, "null path") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud uploaded");
    FILE *f = std::fopen(path, "rb");
    if (!f) return c->fail(HCC_ERR_INVALID, std::string("cannot open ") + path);
    char magic[8];
    SnapHeader h{};
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kSnapMagic, 8) == 0 &&
              std::fread(&h, sizeof(h), 1, f) == 1;
    if (!ok || h.abi != HCC_ABI_VERSION || h.dim != c->D || h.n_vars != c->M || h.pde != c->cfg.pde ||
        h.precision != c->cfg.precision || h.n != c->n || h.npad != c->npad) {
        std::fclose(f);
        return c->fail(HCC_ERR_INVALID, "snapshot does not match this context");
    }
    const int64_t n = c->n;
    std::vector<double> pos(size_t(c->npad) * c->D);
    std::vector<char> U(size_t(n) * c->M * c->esz());
    std::vector<int8_t> ord(n);
    std::vector<uint8_t> flags(n);
    ok = std::fread(pos.data(), sizeof(double), pos.size(), f) == pos.size() &&
         std::fread(U.data(), 1, U.size(), f) == U.size() && std::fread(ord.data(), 1, n, f) == size_t(n) &&
         std::fread(flags.data(), 1, n, f) == size_t(n);
    std::fclose(f);
    if (!ok) return c->fail(HCC_ERR_INVALID, "truncated snapshot");
    hcc_status st;
    HCC_TRY(c->sync("snapshot"));
    HCC_TRY(c->cuda(cudaMemcpy(c->pos, pos.data(), pos.size() * sizeof(double), cudaMemcpyHostToDevice), "positions"));
    HCC_TRY(hcc_build_neighbours(c));
    HCC_TRY(hcc_prepare_geometry(c));
    HCC_TRY(c->cuda(cudaMemcpy(c->rhos, U.data(), U.size(), cudaMemcpyHostToDevice), "state"));
    HCC_TRY(c->cuda(cudaMemcpy(c->orders, ord.data(), n, cudaMemcpyHostToDevice), "orders"));
    HCC_TRY(c->cuda(cudaMemcpy(c->trig_step, flags.data(), n, cudaMemcpyHostToDevice), "flags"));
    c->steps = h.steps;
    c->have_state = true;
    c->reset_rough();
    return HCC_OK;
}

hcc_status hcc_download_neighbours(hcc_ctx *c, int32_t *counts, int32_t *idx, double *w, double *dist) {
    if (!c) return HCC_ERR_INVALID;
    if (!c->have_nb) return c->fail(HCC_ERR_STATE, "neighbour lists missing");
    const int64_t n = c->n;
    std::vector<int32_t> cnt(n);
    hcc_status st;
    HCC_TRY(c->cuda(cudaMemcpy(cnt.data(), c->cnt, n * sizeof(int32_t), cudaMemcpyDeviceToHost), "counts"));
    if (counts) std::memcpy(counts, cnt.data(), n * sizeof(int32_t));
    if (!idx && !w && !dist) return HCC_OK;
    std::vector<int64_t> rs(n);
    int64_t tot = 0;
    for (int64_t i = 0; i < n; ++i) { rs[i] = tot; tot += cnt[i]; }
    int64_t *d_rs = nullptr;
    void *tmp = nullptr;
    HCC_TRY(c->alloc(d_rs, n, "row starts"));
    HCC_TRY(c->valloc(tmp, size_t(std::max<int64_t>(tot, 1)) * 8 * c->D, "row buffer"));
    cudaMemcpy(d_rs, rs.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice);
    auto pull = [&](const void *src, void *dst, int width, int eb) -> hcc_status {
        launch_gather_rows(src, tmp, c->cnt, d_rs, n, c->npad, width, eb, c->stream);
        hcc_status s2 = c->sync("row gather");
        if (s2 != HCC_OK) return s2;
        return c->cuda(cudaMemcpy(dst, tmp, size_t(tot) * width * eb, cudaMemcpyDeviceToHost), "row copy");
    };
    st = HCC_OK;
    if (idx && st == HCC_OK) st = pull(c->nidx, idx, 1, 4);
    if (w && st == HCC_OK) st = pull(c->w64, w, 1, 8);
    if (dist && st == HCC_OK) st = pull(c->dist64, dist, c->D, 8);
    cudaFree(d_rs);
    cudaFree(tmp);
    return st;
}

hcc_status hcc_download_neighbours_of(hcc_ctx *c, int64_t n_sel, const int64_t *ids, int32_t max_slots,
                                      int32_t *counts, int32_t *idx, double *w, double *dist) {
    if (!c) return HCC_ERR_INVALID;
    if (!c->have_nb) return c->fail(HCC_ERR_STATE, "neighbour lists missing");
    if (n_sel < 0 || max_slots < 0 || (n_sel > 0 && !ids)) return c->fail(HCC_ERR_INVALID, "bad selection");
    if (n_sel == 0) return HCC_OK;
    for (int64_t q = 0; q < n_sel; ++q)
        if (ids[q] < 0 || ids[q] >= c->n) return c->fail(HCC_ERR_INVALID, "selected particle out of range");
    hcc_status st;
    int64_t *d_ids = nullptr;
    void *tmp = nullptr;
    HCC_TRY(c->alloc(d_ids, n_sel, "selection"));
    const size_t rows = size_t(n_sel) * size_t(std::max(max_slots, 1));
    st = c->valloc(tmp, rows * 8 * c->D + 8, "selection rows");
    if (st != HCC_OK) { cudaFree(d_ids); return st; }
    st = c->cuda(cudaMemcpy(d_ids, ids, size_t(n_sel) * sizeof(int64_t), cudaMemcpyHostToDevice), "selection");
    if (counts && st == HCC_OK) {
        // counts of the selected particles (uncapped)
        std::vector<int32_t> all(c->n);
        st = c->cuda(cudaMemcpy(all.data(), c->cnt, size_t(c->n) * sizeof(int32_t), cudaMemcpyDeviceToHost), "counts");
        for (int64_t q = 0; q < n_sel && st == HCC_OK; ++q) counts[q] = all[ids[q]];
    }
    auto pull = [&](const void *src, void *dst, int width, int eb) -> hcc_status {
        launch_gather_rows_of(src, tmp, c->cnt, d_ids, n_sel, c->npad, width, max_slots, eb, c->stream);
        hcc_status s2 = c->sync("selected rows");
        if (s2 != HCC_OK) return s2;
        return c->cuda(cudaMemcpy(dst, tmp, rows * width * eb, cudaMemcpyDeviceToHost), "selected row copy");
    };
    if (max_slots > 0) {
        if (idx && st == HCC_OK) st = pull(c->nidx, idx, 1, 4);
        if (w && st == HCC_OK) st = pull(c->w64, w, 1, 8);
        if (dist && st == HCC_OK) st = pull(c->dist64, dist, c->D, 8);
    }
    cudaFree(d_ids);
    cudaFree(tmp);
    return st;
}

// Tile tables of an FP32 context whose full passes can be staged (MUSCL of order <= 2 with the degree-1 divergence
// fit, no moment correction, EPD0/EPD1/StrictEPD0 interface orders): every full gather and flux pass then reads
// its neighbours from shared memory and recomputes the slot offsets and weights. Contexts or clouds that do not
// qualify keep the stream-fed passes (tiles.ok = 0).
hcc_status build_tiles(hcc_ctx *c) {
    c->tiles.release();
    const int pde = c->cfg.pde;
    const bool eligible = c->f32 && c->rdeg == 1 && c->max_order <= 2 && c->ddeg == 1 && !c->no_recon() &&
                          !c->moment() && !c->moving() && c->cfg.mood_strategy != HCC_EPD2 &&
                          (pde == HCC_PDE_EULER || pde == HCC_PDE_ADVECTION || pde == HCC_PDE_BGK);
    if (!eligible || c->n == 0) return HCC_OK;
    const int D = c->D, M = c->M;
    // shared memory of the flux pass per union entry (floats): the int4 position and the state + gradient row in an
    // odd number of 16-byte groups (tile_flux_row in hcc_stage_impl.cuh)
    const int groups = (M + D * M + 3) / 4;
    const int W = 4 + 4 * (groups % 2 == 1 ? groups : groups + 1);
    const long budget = 200L * 1024 - long(HCC_TILE) * 4 * M * long(sizeof(float));
    TileBuild b{};
    b.n = c->n; b.npad = c->npad; b.D = D; b.kmax = std::max(c->kmax, 1);
    b.cnt = c->cnt; b.nidx = c->nidx; b.pos = c->pos;
    for (int d = 0; d < D; ++d) {
        b.periodic[d] = c->cfg.periodic[d];
        const double L = c->cfg.domain_max[d] - c->cfg.domain_min[d];
        b.Lwrap[d] = b.periodic[d] ? L : 0.0;
        b.invLwrap[d] = b.periodic[d] ? 1.0 / L : 0.0;
    }
    b.R = c->cfg.radius;
    b.inv_r = c->inv_r64; b.inv_d = c->inv_d64; b.ok_r = c->ok_r; b.ok_d = c->ok_d;
    b.invL = c->invL;
    b.wscale = c->cfg.weight_alpha / (c->cfg.radius * c->cfg.radius);
    b.max_union = int(std::max(0L, budget / (4L * W)));
    return build_tile_tables(b, c->tiles, c->stream, c->err);
}

hcc_status hcc_set_tile_staging(hcc_ctx *c, int32_t enable) {
    if (!c) return HCC_ERR_INVALID;
    c->drop_graphs();
    c->tile_enabled = enable != 0;
    return HCC_OK;
}

hcc_status hcc_get_tile_staging(hcc_ctx *c, int32_t *active, int64_t *union_entries, int32_t *largest_union) {
    if (!c) return HCC_ERR_INVALID;
    if (active) *active = (c->tiles.ok && c->tile_enabled && !c->moving()) ? 1 : 0;
    if (union_entries) *union_entries = c->tiles.utotal;
    if (largest_union) *largest_union = c->tiles.umax;
    return HCC_OK;
}

hcc_status hcc_prepare_geometry(hcc_ctx *c) {
    if (c) c->drop_graphs();
    if (!c) return HCC_ERR_INVALID;
    if (!c->have_nb) return c->fail(HCC_ERR_STATE, "neighbour lists missing");
    hcc_status st;
    const int D = c->D;
    const size_t slots = size_t(std::max(c->kmax, 1)) * c->npad;
    HCC_TRY(c->alloc(c->dw64, slots * D, "divergence weights"));
    if (c->need_dw1) HCC_TRY(c->alloc(c->dw1_64, slots * D, "degree-1 weights"));
    cudaMemsetAsync(c->dw64, 0, slots * D * sizeof(double), c->stream);
    MlsArgs m{};
    m.n = c->n; m.npad = c->npad; m.D = D; m.rdeg = c->rdeg; m.Br = c->Br; m.ddeg = c->ddeg; m.Bd = c->Bd;
    m.max_order = c->max_order; m.DO = c->DO; m.need_dw1 = c->need_dw1;
    m.cnt = c->cnt; m.nidx = c->nidx; m.dist = c->dist64; m.w = c->w64; m.invL = c->invL;
    m.inv_r = c->inv_r64; m.ok_r = c->ok_r; m.inv_d = c->inv_d64; m.ok_d = c->ok_d;
    m.dw = c->dw64; m.dw1 = c->dw1_64; m.ok_1 = c->ok_1;
    // WENO / CentralDivergence: the CFL weights of the assembled Taylor fit of degree = the scheme's order
    // (_divergence_degree, API.jl:236), and for Central its per-degree divergence weight sets
    m.weno_cfl_degree = c->no_recon() ? std::min(c->max_order, c->D == 3 ? 3 : 4) : 0;
    if (c->central) {
        m.central_qmax = c->qmax;
        for (int q = 0; q < c->qmax; ++q) {
            HCC_TRY(c->alloc(c->dwc64[q], slots * D, "central weights"));
            HCC_TRY(c->alloc(c->okc[q], size_t(c->npad), "central flags"));
            m.dwc[q] = c->dwc64[q];
            m.okc[q] = c->okc[q];
        }
    }
    if (c->moment()) {
        HCC_TRY(c->alloc(c->mw64, slots * D, "moment weights"));
        cudaMemsetAsync(c->mw64, 0, slots * D * sizeof(double), c->stream);
        m.mw = c->mw64;
        m.aligned = c->cfg.flux == HCC_FLUX_ALIGNED;
    }
    if ((st = mls_prepare(m, c->stream, c->err)) != HCC_OK) return st;
    if (c->f32) {
        HCC_TRY(c->alloc(c->dist32, slots * D, "distances f32"));
        HCC_TRY(c->alloc(c->w32, slots, "weights f32"));
        HCC_TRY(c->alloc(c->dw32, slots * D, "divergence weights f32"));
        launch_cast_f64_to_f32(c->dist64, c->dist32, int64_t(slots) * D, c->stream);
        launch_cast_f64_to_f32(c->w64, c->w32, int64_t(slots), c->stream);
        launch_cast_f64_to_f32(c->dw64, c->dw32, int64_t(slots) * D, c->stream);
        launch_cast_f64_to_f32(c->inv_r64, c->inv_r32, c->npad * c->Br * c->Br, c->stream);
        if (c->rdeg == 1 && !c->no_recon()) {
            HCC_TRY(c->alloc(c->gw32, slots * D, "gradient weights f32"));
            launch_grad_weights(c->n, c->npad, D, std::max(c->kmax, 1), c->cnt, c->dist64, c->w64, c->inv_r64, c->ok_r,
                                c->invL, c->gw32, c->stream);
        }
        if (c->need_dw1) {
            HCC_TRY(c->alloc(c->dw1_32, slots * D, "degree-1 weights f32"));
            launch_cast_f64_to_f32(c->dw1_64, c->dw1_32, int64_t(slots) * D, c->stream);
        }
        if (c->moment()) {
            HCC_TRY(c->alloc(c->mw32, slots * D, "moment weights f32"));
            launch_cast_f64_to_f32(c->mw64, c->mw32, int64_t(slots) * D, c->stream);
        }
        for (int q = 0; q < (c->central ? c->qmax : 0); ++q) {
            HCC_TRY(c->alloc(c->dwc32[q], slots * D, "central weights f32"));
            launch_cast_f64_to_f32(c->dwc64[q], c->dwc32[q], int64_t(slots) * D, c->stream);
        }
        if ((st = build_tiles(c)) != HCC_OK) return st;
        if (c->weno && c->ops->weno_geom) {   // FP32 Euler WENO: the fit operators of every stencil, once
            dfree(c->wops);
            dfree(c->wcnt);
            HCC_TRY(c->alloc(c->wops, size_t(c->npad) * weno_ops_floats(D), "WENO operators"));
            HCC_TRY(c->alloc(c->wcnt, size_t(c->npad) * 2 * D, "WENO stencil sizes"));
            WenoGeomArgs wg{};
            wg.n = c->n; wg.npad = c->npad; wg.cnt = c->cnt; wg.dist = c->dist64; wg.w = c->w64; wg.bnd = c->bnd;
            wg.invL64 = c->invL; wg.ops = c->wops; wg.wcnt = c->wcnt;
            c->ops->weno_geom(wg, c->stream);
            HCC_TRY(launch_check(c, "WENO operators"));
        }
    } else if (c->weno && c->ops->weno_geom) {   // FP64 Euler WENO: the factors of every stencil, once
        dfree(c->wchol);
        dfree(c->wok);
        dfree(c->wcnt);
        dfree(c->wflux64);
        HCC_TRY(c->alloc(c->wchol, size_t(c->npad) * weno_chol_doubles(D), "WENO factors"));
        HCC_TRY(c->alloc(c->wok, size_t(c->npad) * 2 * (2 * D + 1), "WENO factor flags"));
        HCC_TRY(c->alloc(c->wcnt, size_t(c->npad) * 2 * D, "WENO stencil sizes"));
        HCC_TRY(c->alloc(c->wflux64, size_t(c->npad) * D * (c->M + 1), "WENO flux table"));
        WenoGeomArgs wg{};
        wg.n = c->n; wg.npad = c->npad; wg.cnt = c->cnt; wg.dist = c->dist64; wg.w = c->w64; wg.bnd = c->bnd;
        wg.invL64 = c->invL; wg.chol = c->wchol; wg.ok = c->wok; wg.wcnt = c->wcnt;
        c->ops->weno_geom(wg, c->stream);
        HCC_TRY(launch_check(c, "WENO factors"));
    }
    // outflow donor roots, then the boundary list (tag -> condition)
    DonorArgs da{};
    da.n = c->n; da.npad = c->npad; da.D = D; da.cnt = c->cnt; da.nidx = c->nidx; da.dist = c->dist64;
    da.bnd = c->bnd; da.tags = c->tags; da.status = c->status; da.status_prev = c->status2; da.root = c->root;
    if ((st = donor_map(da, -1, c->stream, c->err)) != HCC_OK) return st;
    for (int tag = 1; tag <= HCC_MAX_TAGS; ++tag)
        if (c->cfg.bc_by_tag[tag - 1] == HCC_BC_OUTFLOW)
            if ((st = donor_map(da, tag, c->stream, c->err)) != HCC_OK) return st;
    std::vector<int32_t> root(c->n);
    HCC_TRY(c->sync("geometry kernels"));
    if (c->n) HCC_TRY(c->cuda(cudaMemcpy(root.data(), c->root, c->n * sizeof(int32_t), cudaMemcpyDeviceToHost), "donor roots"));
    std::vector<int32_t> bl, bs;
    for (int64_t i = 0; i < c->n; ++i) {
        if (!c->h_bnd[i]) continue;
        int tag = c->h_tags[i];
        int kind = (tag >= 1 && tag <= HCC_MAX_TAGS) ? c->cfg.bc_by_tag[tag - 1] : HCC_BC_KEEP;
        bl.push_back(int32_t(i));
        bs.push_back(kind == HCC_BC_OUTFLOW ? root[i] : -1);
    }
    c->nbnd = int64_t(bl.size());
    HCC_TRY(c->alloc(c->blist, std::max<size_t>(bl.size(), 1), "boundary list"));
    HCC_TRY(c->alloc(c->bsrc, std::max<size_t>(bs.size(), 1), "boundary sources"));
    if (!bl.empty()) {
        HCC_TRY(c->cuda(cudaMemcpy(c->blist, bl.data(), bl.size() * 4, cudaMemcpyHostToDevice), "boundary list"));
        HCC_TRY(c->cuda(cudaMemcpy(c->bsrc, bs.data(), bs.size() * 4, cudaMemcpyHostToDevice), "boundary sources"));
    }
    c->have_geom = true;
    return HCC_OK;
}

hcc_status hcc_download_geometry(hcc_ctx *c, double *dweights, uint8_t *ok_recon, uint8_t *ok_div) {
    if (!c) return HCC_ERR_INVALID;
    if (!c->have_geom) return c->fail(HCC_ERR_STATE, "geometry not prepared");
    hcc_status st;
    const int64_t n = c->n;
    // CentralDivergence: the weights and flags of its full-degree fit (no MUSCL caches)
    const uint8_t *okd = c->central ? c->okc[c->qmax - 1] : c->ok_d;
    const double *dwsrc = c->central ? c->dwc64[c->qmax - 1] : c->dw64;
    if (ok_recon) HCC_TRY(c->cuda(cudaMemcpy(ok_recon, c->ok_r, n, cudaMemcpyDeviceToHost), "ok_r"));
    if (ok_div) HCC_TRY(c->cuda(cudaMemcpy(ok_div, okd, n, cudaMemcpyDeviceToHost), "ok_d"));
    if (!dweights) return HCC_OK;
    std::vector<int32_t> cnt(n);
    HCC_TRY(c->cuda(cudaMemcpy(cnt.data(), c->cnt, n * 4, cudaMemcpyDeviceToHost), "counts"));
    std::vector<int64_t> rs(n);
    int64_t tot = 0;
    for (int64_t i = 0; i < n; ++i) { rs[i] = tot; tot += cnt[i]; }
    int64_t *d_rs = nullptr;
    void *tmp = nullptr;
    HCC_TRY(c->alloc(d_rs, n, "row starts"));
    HCC_TRY(c->valloc(tmp, size_t(std::max<int64_t>(tot, 1)) * 8 * c->D, "row buffer"));
    cudaMemcpy(d_rs, rs.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice);
    launch_gather_rows(dwsrc, tmp, c->cnt, d_rs, n, c->npad, c->D, 8, c->stream);
    st = c->sync("row gather");
    if (st == HCC_OK) st = c->cuda(cudaMemcpy(dweights, tmp, size_t(tot) * c->D * 8, cudaMemcpyDeviceToHost), "dweights");
    cudaFree(d_rs);
    cudaFree(tmp);
    return st;
}

static hcc_status upload_state_impl(hcc_ctx *c, const void *U, int src_f32) {
    if (!c || !U) return c ? c->fail(HCC_ERR_INVALID, "null state") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud uploaded");
    const int64_t cnt = c->n * c->M;
    hcc_status st;
    if (bool(src_f32) == bool(c->f32)) {
        HCC_TRY(c->cuda(cudaMemcpyAsync(c->rhos, U, size_t(cnt) * c->esz(), cudaMemcpyHostToDevice, c->stream), "upload state"));
    } else {
        // convert through the staging buffer (n*M doubles)
        HCC_TRY(c->cuda(cudaMemcpyAsync(c->xfer, U, size_t(cnt) * (src_f32 ? 4 : 8), cudaMemcpyHostToDevice, c->stream),
                        "upload state"));
        if (src_f32) launch_cast_f32_to_f64(static_cast<const float *>(c->xfer), static_cast<double *>(c->rhos), cnt, c->stream);
        else launch_cast_f64_to_f32(static_cast<const double *>(c->xfer), static_cast<float *>(c->rhos), cnt, c->stream);
    }
    HCC_TRY(c->sync("upload state"));
    c->have_state = true;
    c->reset_rough();            // a new state: the predictor visits every tile in the next step
    return HCC_OK;
}

static hcc_status download_state_impl(hcc_ctx *c, void *U, int dst_f32) {
    if (!c || !U) return c ? c->fail(HCC_ERR_INVALID, "null state") : HCC_ERR_INVALID;
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    const int64_t cnt = c->n * c->M;
    hcc_status st;
    if (bool(dst_f32) == bool(c->f32)) {
        HCC_TRY(c->cuda(cudaMemcpyAsync(U, c->rhos, size_t(cnt) * c->esz(), cudaMemcpyDeviceToHost, c->stream), "download state"));
    } else {
        if (dst_f32) launch_cast_f64_to_f32(static_cast<const double *>(c->rhos), static_cast<float *>(c->xfer), cnt, c->stream);
        else launch_cast_f32_to_f64(static_cast<const float *>(c->rhos), static_cast<double *>(c->xfer), cnt, c->stream);
        const void *src = c->xfer;
        HCC_TRY(c->cuda(cudaMemcpyAsync(U, src, size_t(cnt) * (dst_f32 ? 4 : 8), cudaMemcpyDeviceToHost, c->stream),
                        "download state"));
    }
    return c->sync("download state");
}

hcc_status hcc_upload_state(hcc_ctx *c, const double *U) { return upload_state_impl(c, U, 0); }
hcc_status hcc_download_state(hcc_ctx *c, double *U) { return download_state_impl(c, U, 0); }
hcc_status hcc_upload_state_f32(hcc_ctx *c, const float *U) { return upload_state_impl(c, U, 1); }
hcc_status hcc_download_state_f32(hcc_ctx *c, float *U) { return download_state_impl(c, U, 1); }

hcc_status hcc_time_step(hcc_ctx *c, double *dt_out) {
    if (!c || !dt_out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (c->n == 0) { *dt_out = std::numeric_limits<double>::infinity(); return HCC_OK; }
    if (!c->have_geom) { hcc_status st = hcc_prepare_geometry(c); if (st != HCC_OK) return st; }
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    return c->f32 ? run_cfl<float>(c, dt_out) : run_cfl<double>(c, dt_out);
}

hcc_status hcc_compute_rhs(hcc_ctx *c, double *K) {
    if (!c || !K) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_geom) { hcc_status st = hcc_prepare_geometry(c); if (st != HCC_OK) return st; }
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    hcc_status st = c->f32 ? run_rhs<float>(c) : run_rhs<double>(c);
    if (st != HCC_OK) return st;
    const int64_t cnt = c->n * c->M;
    if (c->f32) {
        launch_cast_f32_to_f64(static_cast<const float *>(c->KE[0]), static_cast<double *>(c->xfer), cnt, c->stream);
        HCC_TRY(c->sync("rhs cast"));
        return c->cuda(cudaMemcpy(K, c->xfer, cnt * 8, cudaMemcpyDeviceToHost), "download rhs");
    }
    return c->cuda(cudaMemcpy(K, c->KE[0], cnt * 8, cudaMemcpyDeviceToHost), "download rhs");
}

hcc_status hcc_step(hcc_ctx *c, double t, double dt) {
    (void)t;
    if (!c) return HCC_ERR_INVALID;
    if (!std::isfinite(dt) || !(dt >= 0.0)) return c->fail(HCC_ERR_NONFINITE, "dt must be finite and >= 0");
    if (!c->have_geom) { hcc_status st = hcc_prepare_geometry(c); if (st != HCC_OK) return st; }
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    if (c->n == 0) return HCC_OK;
    c->per_cloud = false;
    return c->f32 ? run_step<float>(c, dt) : run_step<double>(c, dt);
}

hcc_status hcc_batch_step(hcc_ctx *c, double t, const double *dts) {
    (void)t;
    if (!c) return HCC_ERR_INVALID;
    if (c->batch_offsets.size() < 2 || !c->cloud_id) return c->fail(HCC_ERR_STATE, "no batch uploaded");
    if (!dts) return c->fail(HCC_ERR_INVALID, "null time steps");
    const int nb = int(c->batch_offsets.size()) - 1;
    for (int b = 0; b < nb; ++b)
        if (!std::isfinite(dts[b]) || !(dts[b] >= 0.0)) return c->fail(HCC_ERR_NONFINITE, "dt must be finite and >= 0");
    if (!c->have_geom) { hcc_status st = hcc_prepare_geometry(c); if (st != HCC_OK) return st; }
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    if (c->n == 0) return HCC_OK;
    if (nb > c->coef_sets) {                      // room for one coefficient set per cloud
        if (c->stream) cudaStreamSynchronize(c->stream);
        c->drop_graphs();
        const size_t bytes = sizeof(StageCoeffs<double>) * (HCC_MAX_STAGES + 1) * size_t(nb);
        if (c->coef_host) cudaFreeHost(c->coef_host);
        c->coef_host = nullptr;
        hcc_status st = c->valloc(c->coef_dev, bytes, "stage coefficients");
        if (st == HCC_OK) st = c->cuda(cudaMallocHost(&c->coef_host, bytes), "pinned stage coefficients");
        if (st != HCC_OK) return st;
        c->coef_sets = nb;
    }
    c->per_cloud = true;
    c->step_dts.assign(dts, dts + nb);
    const hcc_status st = c->f32 ? run_step<float>(c, 0.0) : run_step<double>(c, 0.0);
    c->per_cloud = false;
    return st;
}

hcc_status hcc_batch_time_steps(hcc_ctx *c, double *dt_out) {
    if (!c || !dt_out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (c->batch_offsets.size() < 2 || !c->cloud_id) return c->fail(HCC_ERR_STATE, "no batch uploaded");
    if (!c->have_geom) { hcc_status st = hcc_prepare_geometry(c); if (st != HCC_OK) return st; }
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    const int nb = int(c->batch_offsets.size()) - 1;
    hcc_status st;
    if (!c->cloud_dt) HCC_TRY(c->alloc(c->cloud_dt, size_t(nb), "per-cloud steps"));
    std::vector<unsigned long long> bits(nb, 0x7ff0000000000000ull);
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->cloud_dt, bits.data(), size_t(nb) * sizeof(unsigned long long),
                                    cudaMemcpyHostToDevice, c->stream), "dt init"));
    if (c->f32) {
        StageArgs<float> a = base_args<float>(c);
        a.U = static_cast<const float *>(c->rhos);
        a.cloud_id = c->cloud_id;
        c->ops->cfl(&a, c->n, c->cloud_dt, c->stream);
    } else {
        StageArgs<double> a = base_args<double>(c);
        a.U = static_cast<const double *>(c->rhos);
        a.cloud_id = c->cloud_id;
        c->ops->cfl(&a, c->n, c->cloud_dt, c->stream);
    }
    c->launches = 1;
    c->launches_total += 1;
    HCC_TRY(launch_check(c, "cfl kernel"));
    HCC_TRY(c->cuda(cudaMemcpyAsync(bits.data(), c->cloud_dt, size_t(nb) * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, c->stream), "dt copy"));
    HCC_TRY(c->sync("cfl"));
    for (int b = 0; b < nb; ++b) std::memcpy(&dt_out[b], &bits[b], sizeof(double));
    return HCC_OK;
}

#define HCC_STR2(x) #x
#define HCC_STR(x) HCC_STR2(x)
const char *hcc_build_info(void) {
    return "flux_block=" HCC_STR(HCC_FLUX_BLOCK) " flux_minb=" HCC_STR(HCC_FLUX_MINB)
           " flux_minb_wide=" HCC_STR(HCC_FLUX_MINB_WIDE) " flux_minb64=" HCC_STR(HCC_FLUX_MINB64)
           " flux_minb_many=" HCC_STR(HCC_FLUX_MINB_MANY) " fp32_packed=" HCC_STR(HCC_FP32_PACKED)
           " tile_flux_pf=" HCC_STR(HCC_TILE_FLUX_PF) " tile_stage_unroll=" HCC_STR(HCC_TILE_STAGE_UNROLL)
           " flux_kahan_block=" HCC_STR(HCC_FLUX_KAHAN_BLOCK)
           " tile_flux_group=" HCC_STR(HCC_TILE_FLUX_GROUP) " tile_gather_group=" HCC_STR(HCC_TILE_GATHER_GROUP);
}

hcc_status hcc_fp64_fma_rate(double *tflops_out) {
    if (!tflops_out) return HCC_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return HCC_ERR_CUDA;
    cudaError_t e = cudaSuccess;
    const double r = hcc::fp64_fma_rate_tflops(sms, nullptr, &e);
    if (e != cudaSuccess) return HCC_ERR_CUDA;
    *tflops_out = r;
    return HCC_OK;
}

static bool tuning_ok(const hcc_tuning &t) {
    auto blk = [](int32_t b) { return b >= 32 && b <= 128 && b % 32 == 0; };
    return blk(t.flux_block) && blk(t.gather_block) && t.list_blocks_per_sm >= 1 && t.list_blocks_per_sm <= 32 &&
           t.drop_blocks_per_sm >= 1 && t.drop_blocks_per_sm <= 32;
}

hcc_status hcc_get_tuning(hcc_ctx *c, hcc_tuning *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    *out = c->tune;
    return HCC_OK;
}

hcc_status hcc_set_tuning(hcc_ctx *c, const hcc_tuning *t) {
    if (!c || !t) return c ? c->fail(HCC_ERR_INVALID, "null tuning") : HCC_ERR_INVALID;
    if (!tuning_ok(*t)) return c->fail(HCC_ERR_INVALID, "tuning out of range");
    c->tune = *t;
    c->apply_tuning();
    c->drop_graphs();
    return HCC_OK;
}

hcc_status hcc_autotune(hcc_ctx *c, double dt, int32_t steps, hcc_tune_report *report) {
    if (!c) return HCC_ERR_INVALID;
    if (!std::isfinite(dt) || !(dt >= 0.0)) return c->fail(HCC_ERR_NONFINITE, "dt must be finite and >= 0");
    if (steps < 1 || steps > 1000) return c->fail(HCC_ERR_INVALID, "steps must be in [1, 1000]");
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    if (c->moving()) return c->fail(HCC_ERR_STATE, "autotune on a moving grid (its steps move the particles)");
    if (!c->have_geom) { hcc_status st = hcc_prepare_geometry(c); if (st != HCC_OK) return st; }
    if (c->n == 0) {                       // nothing to time: the shapes stay
        if (report) *report = hcc_tune_report{c->tune, 0.0, 0.0, 0, steps};
        return HCC_OK;
    }
    hcc_status st;
    const size_t sbytes = size_t(c->n) * c->M * (c->f32 ? 4 : 8);
    const size_t rbytes = c->rough ? size_t(c->npad / 32) * sizeof(uint32_t) : 0;
    // what the tuning steps overwrite: the state, last step's orders / flags, the rough-tile marks, the counters
    char *save = nullptr;
    if ((st = c->alloc(save, sbytes + 2 * size_t(c->n) + rbytes, "autotune snapshot")) != HCC_OK) return st;
    char *s_orders = save + sbytes, *s_flags = s_orders + c->n, *s_rough = s_flags + c->n;
    const int64_t k_launches = c->launches, k_iters = c->mood_iters, k_flagged = c->flagged,
                  k_inadm = c->inadmissible, k_steps = c->steps, k_total = c->launches_total,
                  k_graph = c->graph_steps, k_pred = c->predicted;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int prof0 = c->prof;   // the tuning steps stay out of the kernel timings (and take the graph path)
    c->prof = 0;
    auto restore = [&]() -> hcc_status {
        hcc_status r = c->cuda(cudaMemcpyAsync(c->rhos, save, sbytes, cudaMemcpyDeviceToDevice, c->stream), "restore");
        if (r == HCC_OK && rbytes)
            r = c->cuda(cudaMemcpyAsync(c->rough, s_rough, rbytes, cudaMemcpyDeviceToDevice, c->stream), "restore");
        return r;
    };
    // ms per step of tuning t: drop the graphs (their launches hold the shapes), one warm-up step (captures the
    // graph), then `steps` timed steps, each sequence from the saved state
    auto time_of = [&](const hcc_tuning &t, double *ms) -> hcc_status {
        c->tune = t;
        c->apply_tuning();
        c->drop_graphs();
        hcc_status r;
        if ((r = restore()) != HCC_OK) return r;
        if ((r = hcc_step(c, 0.0, dt)) != HCC_OK) return r;
        if ((r = restore()) != HCC_OK) return r;
        if ((r = c->cuda(cudaEventRecord(e0, c->stream), "event")) != HCC_OK) return r;
        for (int q = 0; q < steps; ++q)
            if ((r = hcc_step(c, 0.0, dt)) != HCC_OK) return r;
        if ((r = c->cuda(cudaEventRecord(e1, c->stream), "event")) != HCC_OK) return r;
        if ((r = c->cuda(cudaEventSynchronize(e1), "event")) != HCC_OK) return r;
        float el = 0.f;
        if ((r = c->cuda(cudaEventElapsedTime(&el, e0, e1), "event")) != HCC_OK) return r;
        *ms = double(el) / steps;
        return HCC_OK;
    };
    const hcc_tuning start = c->tune;
    hcc_tuning best = start;
    double best_ms = 0.0, default_ms = 0.0;
    int cands = 0;
    st = c->cuda(cudaMemcpyAsync(save, c->rhos, sbytes, cudaMemcpyDeviceToDevice, c->stream), "snapshot");
    if (st == HCC_OK) st = c->cuda(cudaMemcpyAsync(s_orders, c->orders, c->n, cudaMemcpyDeviceToDevice, c->stream),
                                   "snapshot");
    if (st == HCC_OK) st = c->cuda(cudaMemcpyAsync(s_flags, c->trig_step, c->n, cudaMemcpyDeviceToDevice, c->stream),
                                   "snapshot");
    if (st == HCC_OK && rbytes)
        st = c->cuda(cudaMemcpyAsync(s_rough, c->rough, rbytes, cudaMemcpyDeviceToDevice, c->stream), "snapshot");
    if (st == HCC_OK) st = c->cuda(cudaEventCreate(&e0), "event");
    if (st == HCC_OK) st = c->cuda(cudaEventCreate(&e1), "event");
    if (st == HCC_OK) st = time_of(start, &default_ms);
    if (st == HCC_OK) {
        best_ms = default_ms;
        cands = 1;
        static const int32_t flux_c[] = {128, 96, 64}, gather_c[] = {128, 64}, list_c[] = {8, 4, 16, 2},
                             drop_c[] = {2, 1, 4};
        struct Knob { int32_t hcc_tuning::*field; const int32_t *vals; int nv; };
        const Knob knobs[] = {{&hcc_tuning::flux_block, flux_c, 3}, {&hcc_tuning::gather_block, gather_c, 2},
                              {&hcc_tuning::list_blocks_per_sm, list_c, 4},
                              {&hcc_tuning::drop_blocks_per_sm, drop_c, 3}};
        for (const Knob &kb : knobs) {
            for (int v = 0; v < kb.nv && st == HCC_OK; ++v) {
                if (kb.vals[v] == best.*kb.field) continue;
                hcc_tuning t = best;
                t.*kb.field = kb.vals[v];
                double ms = 0.0;
                st = time_of(t, &ms);
                ++cands;
                if (st == HCC_OK && ms < 0.99 * best_ms) { best = t; best_ms = ms; }
            }
        }
    }
    // put back what the timed steps overwrote, and the winner (or, after an error, the starting shapes)
    c->tune = (st == HCC_OK) ? best : start;
    c->apply_tuning();
    c->drop_graphs();
    hcc_status rs = restore();
    if (rs == HCC_OK)
        rs = c->cuda(cudaMemcpyAsync(c->orders, s_orders, c->n, cudaMemcpyDeviceToDevice, c->stream), "restore");
    if (rs == HCC_OK)
        rs = c->cuda(cudaMemcpyAsync(c->trig_step, s_flags, c->n, cudaMemcpyDeviceToDevice, c->stream), "restore");
    if (rs == HCC_OK) rs = c->sync("autotune");
    c->prof = prof0;
    c->launches = k_launches; c->mood_iters = k_iters; c->flagged = k_flagged; c->inadmissible = k_inadm;
    c->steps = k_steps; c->launches_total = k_total; c->graph_steps = k_graph; c->predicted = k_pred;
    c->feat_valid = false;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dfree(save);
    if (st == HCC_OK) st = rs;
    if (st == HCC_OK && report) {
        report->best = best;
        report->default_ms = default_ms;
        report->best_ms = best_ms;
        report->candidates = cands;
        report->steps = steps;
    }
    return st;
}

hcc_status hcc_download_orders(hcc_ctx *c, int32_t *orders) {
    if (!c || !orders) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud");
    std::vector<int8_t> o(c->n);
    hcc_status st;
    HCC_TRY(c->cuda(cudaMemcpy(o.data(), c->orders, c->n, cudaMemcpyDeviceToHost), "orders"));
    for (int64_t i = 0; i < c->n; ++i) orders[i] = o[i];
    return HCC_OK;
}

hcc_status hcc_download_mood_flags(hcc_ctx *c, uint8_t *flags) {
    if (!c || !flags) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud");
    return c->cuda(cudaMemcpy(flags, c->trig_step, c->n, cudaMemcpyDeviceToHost), "mood flags");
}

hcc_status hcc_get_counters(hcc_ctx *c, hcc_counters *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    out->n_particles = c->n;
    out->n_interior = c->n_interior;
    out->max_neighbours = c->kmax;
    out->total_neighbours = c->total_nb;
    out->mood_iterations = c->mood_iters;
    if (c->have_cloud && c->n) {
        std::vector<uint8_t> ts(c->n);
        if (cudaMemcpy(ts.data(), c->trig_step, c->n, cudaMemcpyDeviceToHost) == cudaSuccess) {
            int64_t f = 0;
            for (uint8_t v : ts) f += v;
            out->mood_flagged = f;
        }
    }
    out->inadmissible = c->inadmissible;
    out->kernel_launches = c->launches;
    out->steps = c->steps;
    out->kernel_launches_total = c->launches_total;
    out->graph_steps = c->graph_steps;
    out->predicted = c->predicted;
    out->min_neighbours_interior = c->min_nb_interior;
    return HCC_OK;
}

hcc_status hcc_total_mass(hcc_ctx *c, double *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    launch_total_mass(c->rhos, c->vol, c->n, c->M, c->f32, c->d_mass, c->stream);
    hcc_status st;
    HCC_TRY(c->sync("mass"));
    return c->cuda(cudaMemcpy(out, c->d_mass, c->M * sizeof(double), cudaMemcpyDeviceToHost), "mass copy");
}

hcc_status hcc_set_profiling(hcc_ctx *c, int enable) {
    if (!c) return HCC_ERR_INVALID;
    c->prof = enable ? 1 : 0;
    c->ev_used = 0;
    return HCC_OK;
}

hcc_status hcc_set_step_graphs(hcc_ctx *c, int enable) {
    if (!c) return HCC_ERR_INVALID;
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->drop_graphs();
    c->use_graphs = enable != 0 && !c->graphs_failed;
    return HCC_OK;
}

hcc_status hcc_get_kernel_times(hcc_ctx *c, hcc_kernel_times *out, int reset) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    *out = c->times;
    if (reset) c->times = hcc_kernel_times{};
    return HCC_OK;
}

hcc_status hcc_batch_layout(int32_t dim, double radius, int32_t n_clouds, const int64_t *offsets, const double *pos,
                            double *shifts, double *canvas) {
    if (dim < 1 || dim > 3 || !(radius > 0.0) || n_clouds < 1 || !offsets || offsets[0] != 0 || !shifts || !canvas)
        return HCC_ERR_INVALID;
    for (int b = 0; b < n_clouds; ++b)
        if (offsets[b + 1] < offsets[b]) return HCC_ERR_INVALID;
    const int D = dim;
    const int64_t n = offsets[n_clouds];
    if (n > 0 && !pos) return HCC_ERR_INVALID;
    // bounding boxes
    std::vector<double> lo(size_t(n_clouds) * 3, 0.0), hi(size_t(n_clouds) * 3, 0.0);
    for (int b = 0; b < n_clouds; ++b) {
        for (int d = 0; d < D; ++d) { lo[b * 3 + d] = INFINITY; hi[b * 3 + d] = -INFINITY; }
        for (int64_t i = offsets[b]; i < offsets[b + 1]; ++i)
            for (int d = 0; d < D; ++d) {
                const double x = pos[i * D + d];
                if (!std::isfinite(x)) return HCC_ERR_NONFINITE;
                lo[b * 3 + d] = std::min(lo[b * 3 + d], x);
                hi[b * 3 + d] = std::max(hi[b * 3 + d], x);
            }
        for (int d = 0; d < D; ++d)
            if (offsets[b + 1] == offsets[b]) { lo[b * 3 + d] = 0.0; hi[b * 3 + d] = 0.0; }
    }
    // shelf packing in the (x, y) plane, tallest first; z (3-D) aligned at 0; 1-D: one row
    const double gap = 2.0 * radius;
    std::vector<int> order(n_clouds);
    for (int b = 0; b < n_clouds; ++b) order[b] = b;
    auto ext = [&](int b, int d) { return hi[b * 3 + d] - lo[b * 3 + d]; };
    if (D >= 2)
        std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return ext(p, 1) > ext(q, 1); });
    double area = 0.0, widest = 0.0;
    for (int b = 0; b < n_clouds; ++b) {
        area += (ext(b, 0) + gap) * (D >= 2 ? ext(b, 1) + gap : 1.0);
        widest = std::max(widest, ext(b, 0) + gap);
    }
    const double row_w = D >= 2 ? std::max(widest, 1.2 * std::sqrt(area)) : INFINITY;
    std::vector<double> sh(size_t(n_clouds) * 3, 0.0);
    double x = 0.0, y = 0.0, row_h = 0.0;
    for (int b : order) {
        const double w = ext(b, 0) + gap;
        if (x > 0.0 && x + w > row_w) { x = 0.0; y += row_h; row_h = 0.0; }
        sh[b * 3 + 0] = x - lo[b * 3 + 0];
        if (D >= 2) sh[b * 3 + 1] = y - lo[b * 3 + 1];
        if (D == 3) sh[b * 3 + 2] = -lo[b * 3 + 2];
        x += w;
        if (D >= 2) row_h = std::max(row_h, ext(b, 1) + gap);
    }
    double cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = 0; b < n_clouds; ++b)
        for (int64_t i = offsets[b]; i < offsets[b + 1]; ++i)
            for (int d = 0; d < D; ++d) {
                const double v = pos[i * D + d] + sh[b * 3 + d];
                cmin[d] = std::min(cmin[d], v);
                cmax[d] = std::max(cmax[d], v);
            }
    for (int d = 0; d < D; ++d) {
        if (!(cmax[d] > cmin[d])) { cmin[d] -= gap; cmax[d] += gap; }
        canvas[d] = cmin[d];
        canvas[D + d] = cmax[d];
    }
    for (int b = 0; b < n_clouds; ++b)
        for (int d = 0; d < D; ++d) shifts[b * D + d] = sh[b * 3 + d];
    return HCC_OK;
}

hcc_status hcc_upload_batch(hcc_ctx *c, int32_t n_clouds, const int64_t *offsets, const double *pos,
                            const uint8_t *is_boundary, const int32_t *tags, const double *volumes, double *shifts,
                            double *canvas) {
    if (!c) return HCC_ERR_INVALID;
    if (n_clouds < 1 || !offsets || offsets[0] != 0) return c->fail(HCC_ERR_INVALID, "bad batch offsets");
    for (int b = 0; b < n_clouds; ++b)
        if (offsets[b + 1] < offsets[b]) return c->fail(HCC_ERR_INVALID, "batch offsets must not decrease");
    const int D = c->D;
    for (int d = 0; d < D; ++d)
        if (c->cfg.periodic[d]) return c->fail(HCC_ERR_INVALID, "batches of periodic clouds are not supported");
    const int64_t n = offsets[n_clouds];
    if (n > 0 && !pos) return c->fail(HCC_ERR_INVALID, "bad cloud arguments");
    std::vector<double> sh(size_t(n_clouds) * D), cv(2 * size_t(D));
    const hcc_status ls = hcc_batch_layout(D, c->cfg.radius, n_clouds, offsets, pos, sh.data(), cv.data());
    if (ls == HCC_ERR_NONFINITE) return c->fail(ls, "non-finite position");
    if (ls != HCC_OK) return c->fail(ls, "bad batch layout arguments");
    std::vector<double> up(size_t(n) * D);
    for (int b = 0; b < n_clouds; ++b)
        for (int64_t i = offsets[b]; i < offsets[b + 1]; ++i)
            for (int d = 0; d < D; ++d) up[i * D + d] = pos[i * D + d] + sh[size_t(b) * D + d];
    for (int d = 0; d < D; ++d) {
        c->cfg.canvas_min[d] = cv[d];
        c->cfg.canvas_max[d] = cv[D + d];
        c->cfg.domain_min[d] = cv[d];
        c->cfg.domain_max[d] = cv[D + d];
        if (canvas) { canvas[d] = cv[d]; canvas[D + d] = cv[D + d]; }
    }
    if (shifts) std::copy(sh.begin(), sh.end(), shifts);
    hcc_status st = hcc_upload_cloud(c, n, up.data(), is_boundary, tags, volumes);
    if (st != HCC_OK) return st;
    c->batch_offsets.assign(offsets, offsets + n_clouds + 1);
    std::vector<int32_t> ids(size_t(std::max<int64_t>(n, 1)), 0);
    for (int b = 0; b < n_clouds; ++b)
        for (int64_t i = offsets[b]; i < offsets[b + 1]; ++i) ids[i] = b;
    HCC_TRY(c->alloc(c->cloud_id, size_t(std::max<int64_t>(n, 1)), "cloud ids"));
    HCC_TRY(c->cuda(cudaMemcpy(c->cloud_id, ids.data(), size_t(std::max<int64_t>(n, 1)) * sizeof(int32_t),
                               cudaMemcpyHostToDevice), "cloud ids"));
    dfree(c->cloud_dt);
    return HCC_OK;
}

hcc_status hcc_batch_total_mass(hcc_ctx *c, double *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    if (c->batch_offsets.size() < 2) return c->fail(HCC_ERR_STATE, "no batch uploaded");
    hcc_status st;
    const size_t nb = c->batch_offsets.size() - 1;
    for (size_t b = 0; b < nb; ++b) {
        const int64_t o = c->batch_offsets[b], m = c->batch_offsets[b + 1] - o;
        const void *U = c->f32 ? static_cast<const void *>(static_cast<const float *>(c->rhos) + o * c->M)
                               : static_cast<const void *>(static_cast<const double *>(c->rhos) + o * c->M);
        launch_total_mass(U, c->vol + o, m, c->M, c->f32, c->d_mass, c->stream);
        HCC_TRY(c->sync("batch mass"));
        HCC_TRY(c->cuda(cudaMemcpy(out + b * c->M, c->d_mass, c->M * sizeof(double), cudaMemcpyDeviceToHost),
                        "batch mass copy"));
    }
    return HCC_OK;
}

hcc_status hcc_update_volumes(hcc_ctx *c, int32_t sweeps) {
    if (!c) return HCC_ERR_INVALID;
    if (sweeps < 0) return c->fail(HCC_ERR_INVALID, "sweeps must be >= 0");
    if (!c->have_nb) return c->fail(HCC_ERR_STATE, "neighbour lists missing");
    const int64_t n = c->n;
    if (n == 0) return HCC_OK;
    const double w0 = 1.0;     // ExponentialWeightFunction at zero distance: 1 / (1 + 0)
    double *S = nullptr, *Vt = nullptr, *part = nullptr;
    const unsigned nb = shepard_blocks(n);
    hcc_status st = c->alloc(S, size_t(n), "Shepard sums");
    if (st == HCC_OK) st = c->alloc(Vt, size_t(n), "Shepard sweep");
    if (st == HCC_OK) st = c->alloc(part, size_t(nb), "Shepard partials");
    if (st == HCC_OK) {
        launch_shepard(c->cnt, c->nidx, c->w64, n, c->npad, w0, sweeps, S, c->vol, Vt, part, c->stream);
        std::vector<double> hp(nb);
        st = c->cuda(cudaMemcpyAsync(hp.data(), part, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                     "Shepard partials");
        if (st == HCC_OK) st = c->sync("Shepard volumes");
        if (st == HCC_OK) {
            double sum = 0.0;
            for (double v : hp) sum = sum + v;
            double box = 1.0;
            for (int d = 0; d < c->D; ++d) box = box * (c->cfg.domain_max[d] - c->cfg.domain_min[d]);
            launch_scale(c->vol, n, box / sum, c->stream);
            st = c->sync("Shepard scale");
        }
    }
    dfree(S);
    dfree(Vt);
    dfree(part);
    return st;
}

hcc_status hcc_download_volumes(hcc_ctx *c, double *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud");
    return c->cuda(cudaMemcpy(out, c->vol, size_t(c->n) * sizeof(double), cudaMemcpyDeviceToHost), "volumes");
}

hcc_status hcc_set_predictor(hcc_ctx *c, hcc_mlp *mlp, double thr) {
    if (!c) return HCC_ERR_INVALID;
    if (mlp && !(thr > 0.0 && thr < 1.0)) return c->fail(HCC_ERR_INVALID, "predictor threshold outside (0, 1)");
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->drop_graphs();
    c->mlp = mlp;
    c->thr_logit = mlp ? float(std::log(thr / (1.0 - thr))) : 0.f;
    c->reset_rough();
    return HCC_OK;
}

hcc_status hcc_set_feature_capture(hcc_ctx *c, int enable) {
    if (!c) return HCC_ERR_INVALID;
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->drop_graphs();
    c->capture_feat = enable ? 1 : 0;
    c->feat_valid = false;
    return HCC_OK;
}

hcc_status hcc_download_features(hcc_ctx *c, float *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_state) return c->fail(HCC_ERR_STATE, "no state");
    if (!c->have_geom) { hcc_status gs = hcc_prepare_geometry(c); if (gs != HCC_OK) return gs; }
    if (c->n == 0) return HCC_OK;
    float *tmp = nullptr;
    hcc_status st = c->alloc(tmp, size_t(c->n) * HCC_MLP_FEATURES, "features");
    if (st != HCC_OK) return st;
    if (!launch_features(feat_args(c, c->rhos), tmp, c->stream)) {
        dfree(tmp);
        return c->fail(HCC_ERR_UNSUPPORTED, "no feature kernel for this physics");
    }
    st = c->sync("features");
    if (st == HCC_OK)
        st = c->cuda(cudaMemcpy(out, tmp, size_t(c->n) * HCC_MLP_FEATURES * sizeof(float), cudaMemcpyDeviceToHost),
                     "features");
    dfree(tmp);
    return st;
}

hcc_status hcc_download_predicted(hcc_ctx *c, uint8_t *out) {
    if (!c || !out) return c ? c->fail(HCC_ERR_INVALID, "null output") : HCC_ERR_INVALID;
    if (!c->have_cloud) return c->fail(HCC_ERR_STATE, "no cloud");
    if (!c->pred) {
        std::memset(out, 0, size_t(c->n));
        return HCC_OK;
    }
    return c->cuda(cudaMemcpy(out, c->pred, size_t(c->n), cudaMemcpyDeviceToHost), "predicted mask");
}

hcc_status hcc_mlp_collect(hcc_mlp *m, hcc_ctx *c) {
    if (!m || !c) return c ? c->fail(HCC_ERR_INVALID, "null predictor") : HCC_ERR_INVALID;
    if (!c->feat_valid || !c->feat)
        return c->fail(HCC_ERR_STATE, "collect: the last step did not capture features (hcc_set_feature_capture)");
    hcc_status st = mlp_append(m, c->feat, c->trig_step, c->bnd, c->n, c->stream);
    if (st != HCC_OK) return c->fail(st, hcc_mlp_last_error(m));
    return HCC_OK;
}

hcc_status hcc_synchronize(hcc_ctx *c) {
    if (!c) return HCC_ERR_INVALID;
    return c->sync("synchronize");
}

void *hcc_stream(hcc_ctx *c) { return c ? static_cast<void *>(c->stream) : nullptr; }

}  // extern "C"

namespace {

// _apply_stage_geometry! / set_positions! (TimeSteppers.jl:521-525, GridMovers.jl:123-133): the positions src
// become the grid's, then a full search (with periodic re-wrap) or the refresh of the existing slots, then the
// geometry caches (MLS inverses, divergence and gradient weights, donor map) at the new positions.
hcc_status apply_positions(hcc_ctx *c, const double *src, bool full_search) {
    hcc_status st;
    c->tiles.release();                           // the tile tables describe the positions being replaced
    HCC_TRY(c->cuda(cudaMemcpyAsync(c->pos, src, size_t(c->npad) * c->D * sizeof(double), cudaMemcpyDeviceToDevice,
                                    c->stream), "stage positions"));
    if (full_search) {
        HCC_TRY(hcc_build_neighbours(c));
    } else {
        const hcc_config &f = c->cfg;
        SearchArgs a{};
        a.n = c->n; a.npad = c->npad; a.D = c->D; a.pos = c->pos;
        for (int d = 0; d < 3; ++d) {
            const bool per = d < c->D && f.periodic[d];
            const double L = f.domain_max[d] - f.domain_min[d];
            a.periodic[d] = per ? 1 : 0;
            a.Lwrap[d] = per ? L : 0.0;
            a.invLwrap[d] = per ? 1.0 / L : 0.0;
        }
        a.cnt = c->cnt; a.nidx = c->nidx; a.w = c->w64; a.dist = c->dist64; a.kmax = c->kmax;
        a.R_sq = f.radius * f.radius;
        a.alpha = f.weight_alpha;
        a.invR2 = 1.0 / (f.radius * f.radius);
        HCC_TRY(search_refresh(a, c->stream, c->err));
        c->launches += 1;
    }
    return hcc_prepare_geometry(c);
}

}  // namespace
