"""GPU: the learned troubled-point predictor against the CPU oracle.

Stencil features: bit for bit (FP32, both sides in the same operation order). Tensor-core inference and the
training kernels' loss and gradient: within FP32 accumulation error of the numpy restatement (oracle/mlp.py), which
mirrors the kernels' BF16 rounding points — tolerances are stated per test. The in-step pre-lowering: the FP64 step
with a predictor attached equals the oracle's step with the same particles pre-lowered, bit for bit.
"""
import importlib.util
import sys

import numpy as np
import pytest

from conftest import ROOT, quadrant_ic, blast_ic, gaussian_ic, c1_cloud

pytestmark = pytest.mark.gpu

OUTFLOW = {t: 2 for t in range(1, 7)}


def _mlp_oracle():
    if "hcc_oracle_mlp" in sys.modules:
        return sys.modules["hcc_oracle_mlp"]
    spec = importlib.util.spec_from_file_location("hcc_oracle_mlp", ROOT / "oracle" / "mlp.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["hcc_oracle_mlp"] = mod
    spec.loader.exec_module(mod)
    return mod


def _pair(hcc, oracle, cfg, cloud):
    abi = sys.modules["hcc_gb300._abi"]
    g = hcc.Context(cfg)
    o = oracle.OracleContext(cfg, abi)
    for c in (g, o):
        c.upload_cloud(cloud)
        c.build_neighbours()
        c.prepare_geometry()
    return g, o


def _euler_cfg(hcc, cloud, h, precision="fp64", D=2):
    return hcc.make_config(hcc.Euler(D, 1.4), cloud, scheme=hcc.MUSCL(2, 2),
                           mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h ** D)), tableau="RK3_SSP",
                           bc_map=OUTFLOW, precision=precision)


def _random_params(seed, scale=0.4):
    m = _mlp_oracle()
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, scale, m.NPARAMS).astype(np.float32)
    norm = np.concatenate([rng.normal(0.0, 0.2, 24), rng.uniform(0.5, 2.0, 24)]).astype(np.float32)
    return p, norm


@pytest.mark.parametrize("case", ["euler2d_fp64", "euler2d_fp32", "euler3d_fp64", "advection2d"])
def test_features_bit_exact(hcc, oracle, cuda_lib, case):
    if case.startswith("euler2d"):
        h = 1 / 64
        cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
        U = quadrant_ic(cloud)
        prec = "fp32" if case.endswith("fp32") else "fp64"
        cfg = _euler_cfg(hcc, cloud, h, prec)
    elif case == "euler3d_fp64":
        h = 1 / 16
        cloud = hcc.rectangular_cloud((0.0,) * 3, (1.0,) * 3, h, 2.5 * h, jitter=0.25 * h, seed=5)
        U = blast_ic(cloud)
        cfg = _euler_cfg(hcc, cloud, h, "fp64", D=3)
    else:
        cloud = c1_cloud(hcc, h=0.02)
        U = gaussian_ic(cloud)
        cfg = hcc.make_config(hcc.LinearAdvection(((1.0,), (1.0,))), cloud, scheme=hcc.MUSCL(2, 2))
    if cfg.precision == 1:
        U = U.astype(np.float32).astype(np.float64)      # the FP32 context's state, exactly representable
    g, o = _pair(hcc, oracle, cfg, cloud)
    g.upload_state(U.astype(np.float32) if cfg.precision == 1 else U)
    o.upload_state(U)
    fg, fo = g.features(), o.features()
    assert fg.shape == (cloud.n, 24)
    assert np.array_equal(fg.view(np.uint32), fo.view(np.uint32))
    assert np.abs(fg).max() <= 8.0 and np.count_nonzero(fg) > 0


def test_inference_matches_oracle(hcc, cuda_lib):
    m = _mlp_oracle()
    pred = hcc.TroubledPointPredictor(capacity=1024, seed=1)
    p, norm = _random_params(11)
    pred.set_params(p, norm)
    rng = np.random.default_rng(2)
    X = rng.normal(0.0, 1.5, (1000, 24)).astype(np.float32)       # 7 full tiles + a partial one
    got = pred.predict_rows(X)
    want, _ = m.forward(p, norm, X)
    g = m.gated(X)
    assert 0 < g.sum() < len(g)
    assert np.all(np.isneginf(got[g]))          # below the smoothness gate: no network, never predicted
    # BF16 operands identical on both sides; FP32 tensor-core accumulation vs FP64: |diff| <= 2e-3 (1 + |logit|)
    d = np.abs(got[~g] - want[~g])
    assert np.all(d <= 2e-3 * (1.0 + np.abs(want[~g]))), d.max()


@pytest.mark.parametrize("n,pos_weight", [(300, 3.0), (128 * 400 + 17, 1.0)])
def test_loss_and_gradient_match_oracle(hcc, cuda_lib, n, pos_weight):
    """One forward/backward pass on the tensor cores vs the numpy restatement. n = 300: three tiles, the last partial;
    n = 51217: more tiles than SMs, so CTAs accumulate several tiles in tensor memory."""
    m = _mlp_oracle()
    pred = hcc.TroubledPointPredictor(capacity=1024, seed=2, pos_weight=pos_weight)
    p, norm = _random_params(21)
    pred.set_params(p, norm)
    rng = np.random.default_rng(3)
    X = rng.normal(0.0, 1.5, (n, 24)).astype(np.float32)
    y = (rng.random(n) < 0.3).astype(np.uint8)
    loss, grad = pred.loss_grad(X, y)
    lo, go = m.loss_grad(p, norm, X, y, pos_weight)
    assert abs(loss - lo) <= 1e-4 * abs(lo)
    # per block (W1, b1, W2, b2, w3, b3): relative L2 error <= 2e-3
    cuts = [0, m.OFF_B1, m.OFF_W2, m.OFF_B2, m.OFF_W3, m.OFF_B3, m.NPARAMS]
    for a, b in zip(cuts[:-1], cuts[1:]):
        err = np.linalg.norm(grad[a:b] - go[a:b]) / max(np.linalg.norm(go[a:b]), 1e-30)
        assert err <= 2e-3, (a, b, err)


def test_training_learns_a_separable_rule(hcc, cuda_lib):
    """Adam on the device: a rule on two features is learnt to > 97 % held-out accuracy."""
    rng = np.random.default_rng(4)
    n = 40000
    X = rng.normal(0.0, 1.0, (n, 24)).astype(np.float32)
    y = ((X[:, 0] > 0.3) & (X[:, 6] < 0.5)).astype(np.uint8)
    pred = hcc.TroubledPointPredictor(capacity=n, seed=5, lr=3e-3)
    pred.add_rows(X, y)
    assert pred.rows() == (n, int(y.sum()))
    pred.fit_norm(holdout=0.2)
    l0 = pred.loss_grad(X[:4096], y[:4096])[0]
    loss = pred.train(600, batch=4096, holdout=0.2)
    assert loss < 0.5 * l0
    ev = pred.evaluate(0.5, holdout=0.2)
    acc = (ev["tp"] + ev["tn"]) / (ev["tp"] + ev["tn"] + ev["fp"] + ev["fn"])
    assert ev["tp"] + ev["tn"] + ev["fp"] + ev["fn"] == n - int(n * 0.8)
    assert acc > 0.97, ev


def _prepare_predicted_step(hcc, oracle, frac=0.2, precision="fp64"):
    h = 1 / 64
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
    U = quadrant_ic(cloud)
    cfg = _euler_cfg(hcc, cloud, h, precision)
    g, o = _pair(hcc, oracle, cfg, cloud)
    g.upload_state(U)
    o.upload_state(U)
    pred = hcc.TroubledPointPredictor(capacity=1024, seed=9)
    p, norm = _random_params(31)
    pred.set_params(p, norm)
    logits = pred.predict_rows(g.features())
    interior = ~cloud.is_boundary.astype(bool)
    # uniform regions give equal features, hence equal logits: threshold halfway between two distinct values
    u = np.unique(logits[interior])
    k = max(1, int((1.0 - frac) * len(u)))
    thr_logit = 0.5 * (float(u[k - 1]) + float(u[k]))
    thr = 1.0 / (1.0 + np.exp(-thr_logit))
    want = (logits > np.float32(np.log(thr / (1.0 - thr)))) & interior
    return g, o, pred, thr, want, cloud


@pytest.mark.parametrize("graphs", [True, False])
def test_step_with_predictor_bit_exact(hcc, oracle, cuda_lib, graphs):
    g, o, pred, thr, want, cloud = _prepare_predicted_step(hcc, oracle)
    g.set_step_graphs(graphs)
    g.set_predictor(pred, thr)
    dt = 0.4 * g.time_step()
    g.step(0.0, dt)
    got = g.predicted().astype(bool)
    assert 0 < got.sum() < (~cloud.is_boundary.astype(bool)).sum()
    np.testing.assert_array_equal(got, want)      # the in-step tiles see the same features and weights
    assert g.counters()["predicted"] == int(got.sum())
    o.set_prelowered(got.astype(np.uint8))
    o.step(0.0, dt)
    Ug, Uo = g.download_state(), o.download_state()
    assert np.array_equal(Ug.view(np.uint64), Uo.view(np.uint64))
    np.testing.assert_array_equal(g.orders(), o.orders())
    np.testing.assert_array_equal(g.mood_flags(), o.mood_flags())
    # detaching restores the plain method
    g.set_predictor(None)
    g.step(dt, dt)
    o.step(dt, dt)
    assert np.array_equal(g.download_state().view(np.uint64), o.download_state().view(np.uint64))
    assert g.counters()["predicted"] == 0


def test_collect_appends_flagged_and_sampled_rows(hcc, oracle, cuda_lib):
    h = 1 / 64
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=3)
    cfg = _euler_cfg(hcc, cloud, h, "fp32")
    g = hcc.Context(cfg)
    g.upload_cloud(cloud)
    g.build_neighbours()
    g.prepare_geometry()
    g.upload_state(quadrant_ic(cloud).astype(np.float32))
    pred = hcc.TroubledPointPredictor(capacity=1 << 16, neg_keep=0.1, seed=3)
    g.set_feature_capture(True)
    F0 = g.features()
    g.step(0.0, 0.4 * g.time_step())
    flags = g.mood_flags().astype(bool) & ~cloud.is_boundary.astype(bool)
    pred.collect(g)
    rows, flagged = pred.rows()
    assert flagged == int(flags.sum()) > 0
    neg = rows - flagged
    n_neg = int((~flags & ~cloud.is_boundary.astype(bool)).sum())
    assert 0.05 * n_neg < neg < 0.15 * n_neg
    # the collected rows are the start-of-step features: every flagged particle's row is present
    pred2 = hcc.TroubledPointPredictor(capacity=1 << 16, neg_keep=0.0, seed=3)
    pred2.collect(g)
    assert pred2.rows() == (int(flags.sum()), int(flags.sum()))
    logits_rows = pred2.predict_rows(F0[flags])
    pred2.clear()
    assert pred2.rows() == (0, 0)
    # flagged particles whose stencil was flat at the start of the step are below the smoothness gate (the trouble
    # reached them within the step); every other row goes through the network
    g = _mlp_oracle().gated(F0[flags])
    assert np.all(np.isneginf(logits_rows[g])) and np.all(np.isfinite(logits_rows[~g])) and (~g).sum() > 0


def _voronoi_run(hcc, cloud, h, seed, steps, predictor=None, thr=0.7, dts=None, precision="fp32"):
    L = sys.modules["hcc_gb300.learned"]
    cfg = _euler_cfg(hcc, cloud, h, precision)
    ctx = hcc.Context(cfg)
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    U0 = L.voronoi_state(cloud.pos, seed)
    ctx.upload_state(U0.astype(np.float32) if precision == "fp32" else U0)
    if predictor is not None:
        ctx.set_predictor(predictor, thr)
    t, used = 0.0, []
    flagged = iters = predicted = 0
    for k in range(steps):
        dt = dts[k] if dts is not None else 0.4 * ctx.time_step()
        used.append(dt)
        ctx.step(t, dt)
        c = ctx.counters()
        flagged += c["mood_flagged"]
        iters += c["mood_iterations"]
        predicted += c["predicted"]
        t += dt
    U = ctx.download_state()
    ctx.close()
    return U, used, {"flagged": flagged, "iters": iters, "predicted": predicted}


def test_trained_predictor_gains_over_plain_mood(hcc, cuda_lib):
    """The shipped network (trained by train_predictor.py on seeds 0-199) on a held-out Voronoi state (seed 4242) at
    250k nodes, FP32 bulk, 30 steps with one dt sequence: MOOD's judge flags at least 3x fewer particles and its
    fixed points take fewer iterations than without the network, while the density stays within 2e-3 relative L1
    of the plain run."""
    L = sys.modules["hcc_gb300.learned"]
    pred = hcc.TroubledPointPredictor(capacity=16)
    pred.load(L.default_weights_path())
    h = 2e-3
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=42)
    U0, dts, s0 = _voronoi_run(hcc, cloud, h, 4242, 30)
    U1, _, s1 = _voronoi_run(hcc, cloud, h, 4242, 30, predictor=pred, dts=dts)
    assert s1["predicted"] > 0
    assert s1["flagged"] * 3 <= s0["flagged"], (s0, s1)
    assert s1["iters"] < s0["iters"], (s0, s1)
    inner = ~cloud.is_boundary.astype(bool)
    l1 = np.abs(U1[inner, 0] - U0[inner, 0]).sum() / np.abs(U0[inner, 0]).sum()
    assert l1 < 2e-3, l1
