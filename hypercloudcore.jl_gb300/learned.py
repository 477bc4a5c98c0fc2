"""Learned troubled-point predictor: the host side of the ``hcc_mlp_*`` entry points of include/hcc.h.

The reference's MOOD loop computes every particle at full order, checks the candidates and recomputes the ones it
dropped (src/TimeStepping/MOOD.jl:375-405, src/TimeStepping/TimeSteppers.jl:454-477). A ``TroubledPointPredictor``
attached to a ``Context`` reads 24 stencil features of each step's start state and pre-lowers the particles it
predicts to be troubled, so they skip the compute-high-order-then-recompute cycle; MOOD still judges every particle.

Network: 24 -> 64 -> 64 -> 1, GELU, BF16 weights and activations on the tensor cores (tcgen05, FP32 accumulators
in tensor memory), weighted binary cross-entropy, Adam — forward, backward and update run on the GPU
(csrc/hcc_learn.cu). Training data are (feature, MOOD-flag) pairs the solver generates (``collect``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional

import numpy as np

from . import _abi

NF = _abi.HCC_MLP_FEATURES
NPARAMS = _abi.HCC_MLP_NPARAMS


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class TroubledPointPredictor:
    """Owner of one ``hcc_mlp`` (parameters, Adam state and the training rows, all on the device)."""

    def __init__(self, capacity: int = 1 << 22, neg_keep: float = 0.05, seed: int = 0, lr: float = 1e-3,
                 beta1: float = 0.9, beta2: float = 0.999, adam_eps: float = 1e-8, pos_weight: float = 1.0,
                 lib: Optional[C.CDLL] = None):
        from . import HCCError, load_library
        self._err = HCCError
        self.lib = lib or load_library()
        cfg = _abi.HccMlpConfig()
        cfg.capacity = int(capacity)
        cfg.neg_keep = float(neg_keep)
        cfg.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        cfg.lr, cfg.beta1, cfg.beta2, cfg.adam_eps = float(lr), float(beta1), float(beta2), float(adam_eps)
        cfg.pos_weight = float(pos_weight)
        self.cfg = cfg
        self._h = C.c_void_p()
        st = self.lib.hcc_mlp_create(C.byref(cfg), C.byref(self._h))
        if st != 0:
            self._h = None
            raise HCCError(st, "hcc_mlp_create failed", "hcc_mlp_create")

    @property
    def handle(self):
        return self._h

    def _check(self, st: int, call: str):
        if st != 0:
            raise self._err(st, self.lib.hcc_mlp_last_error(self._h).decode(), call)

    def close(self):
        if self._h:
            self.lib.hcc_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters
    def params(self):
        """(params[HCC_MLP_NPARAMS], norm[48]) as FP32 arrays."""
        p = np.zeros(NPARAMS, dtype=np.float32)
        n = np.zeros(2 * NF, dtype=np.float32)
        self._check(self.lib.hcc_mlp_get_params(self._h, _ptr(p, C.c_float), _ptr(n, C.c_float)),
                    "hcc_mlp_get_params")
        return p, n

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        if p is not None and p.size != NPARAMS:
            raise ValueError(f"expected {NPARAMS} parameters")
        if n is not None and n.size != 2 * NF:
            raise ValueError(f"expected {2 * NF} normalisation values")
        self._check(self.lib.hcc_mlp_set_params(self._h, None if p is None else _ptr(p, C.c_float),
                                                None if n is None else _ptr(n, C.c_float)), "hcc_mlp_set_params")

    def save(self, path):
        p, n = self.params()
        np.savez(path, params=p, norm=n)

    def load(self, path):
        d = np.load(path)
        self.set_params(d["params"], d["norm"])

    # -- training set
    def collect(self, ctx):
        """Append the last step of ``ctx`` (features captured at its start, its MOOD flags as labels)."""
        self._check(self.lib.hcc_mlp_collect(self._h, ctx.handle), "hcc_mlp_collect")

    def add_rows(self, X: np.ndarray, y: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, NF)
        y = np.ascontiguousarray(y, dtype=np.uint8).reshape(-1)
        self._check(self.lib.hcc_mlp_add_rows(self._h, _ptr(X, C.c_float), _ptr(y, C.c_uint8), X.shape[0]),
                    "hcc_mlp_add_rows")

    def rows(self):
        r, f = C.c_int64(), C.c_int64()
        self._check(self.lib.hcc_mlp_rows(self._h, C.byref(r), C.byref(f)), "hcc_mlp_rows")
        return r.value, f.value

    def clear(self):
        self._check(self.lib.hcc_mlp_clear(self._h), "hcc_mlp_clear")

    # -- training
    def fit_norm(self, holdout: float = 0.0):
        self._check(self.lib.hcc_mlp_fit_norm(self._h, float(holdout)), "hcc_mlp_fit_norm")

    def train(self, iters: int, batch: int = 8192, holdout: float = 0.0) -> float:
        loss = C.c_double()
        self._check(self.lib.hcc_mlp_train(self._h, int(iters), int(batch), float(holdout), C.byref(loss)),
                    "hcc_mlp_train")
        return loss.value

    def evaluate(self, threshold: float = 0.5, holdout: float = 0.1) -> dict:
        c = (C.c_int64 * 4)()
        self._check(self.lib.hcc_mlp_evaluate(self._h, float(threshold), float(holdout), c), "hcc_mlp_evaluate")
        tp, fp, fn, tn = (int(v) for v in c)
        return {"tp": tp, "fp": fp, "fn": fn, "tn": tn,
                "precision": tp / (tp + fp) if tp + fp else 0.0, "recall": tp / (tp + fn) if tp + fn else 0.0}

    def loss_grad(self, X: np.ndarray, y: np.ndarray):
        """(mean loss, gradient) of one forward/backward pass on host rows, no update."""
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, NF)
        y = np.ascontiguousarray(y, dtype=np.uint8).reshape(-1)
        g = np.zeros(NPARAMS, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.hcc_mlp_loss_grad(self._h, _ptr(X, C.c_float), _ptr(y, C.c_uint8), X.shape[0],
                                               _ptr(g, C.c_float), C.byref(loss)), "hcc_mlp_loss_grad")
        return loss.value, g

    def predict_rows(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, NF)
        out = np.zeros(X.shape[0], dtype=np.float32)
        self._check(self.lib.hcc_mlp_predict_rows(self._h, _ptr(X, C.c_float), X.shape[0], _ptr(out, C.c_float)),
                    "hcc_mlp_predict_rows")
        return out


# ------------------------------------------------------------------------------------------ training data
def voronoi_state(pos: np.ndarray, seed: int, gamma: float = 1.4, regions=(2, 6)) -> np.ndarray:
    """Random piecewise-constant 2-D Euler state over 2-6 Voronoi regions of the unit square: per region
    rho, p ~ U[0.1, 2] and u, v ~ U[-1, 1]; conserved variables (rho, rho u, rho v, E)."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(regions[0], regions[1] + 1))
    sites = rng.random((k, 2))
    rho = rng.uniform(0.1, 2.0, k)
    p = rng.uniform(0.1, 2.0, k)
    u = rng.uniform(-1.0, 1.0, k)
    v = rng.uniform(-1.0, 1.0, k)
    d2 = ((pos[:, None, :2] - sites[None, :, :]) ** 2).sum(axis=2)
    r = np.argmin(d2, axis=1)
    R, Uu, Vv, Pp = rho[r], u[r], v[r], p[r]
    E = Pp / (gamma - 1.0) + 0.5 * R * (Uu * Uu + Vv * Vv)
    return np.ascontiguousarray(np.stack([R, R * Uu, R * Vv, E], axis=1))


def generate_training_set(hcc, predictor: TroubledPointPredictor, runs: int, h: float, t_end: float,
                          seed0: int = 0, cfl: float = 0.4, precision: str = "fp32", every: int = 1,
                          max_steps: Optional[int] = None, log=None) -> dict:
    """Seeded 2-D Euler runs on the jittered unit-square lattice of spacing h (MUSCL2 + MOOD(EPD1, MOODu1(1e-4 h^2)),
    Rusanov, SSP-RK3, transmissive walls) from Voronoi states to t_end; every `every`-th step is appended to the
    predictor's training set. Returns run statistics."""
    cloud = hcc.rectangular_cloud((0.0, 0.0), (1.0, 1.0), h, 2.5 * h, jitter=0.25 * h, seed=42)
    cfg = hcc.make_config(hcc.Euler(2, 1.4), cloud, scheme=hcc.MUSCL(2, 2),
                          mood=hcc.MOOD(hcc.EPD1, hcc.MOODu1(1e-4 * h * h)), tableau="RK3_SSP",
                          bc_map={t: hcc.BC_OUTFLOW for t in range(1, 5)}, precision=precision)
    ctx = hcc.Context(cfg)
    ctx.upload_cloud(cloud)
    ctx.build_neighbours()
    ctx.prepare_geometry()
    ctx.set_feature_capture(True)
    steps = 0
    for r in range(runs):
        U0 = voronoi_state(cloud.pos, seed0 + r)
        ctx.upload_state(U0.astype(np.float32) if precision == "fp32" else U0)
        t, k = 0.0, 0
        while t < t_end - 1e-12 and (max_steps is None or k < max_steps):
            dt = min(cfl * ctx.time_step(), t_end - t)
            ctx.step(t, dt)
            if k % every == 0:
                predictor.collect(ctx)
            t += dt
            k += 1
        steps += k
        if log:
            log(f"run {r}: {k} steps, rows {predictor.rows()}")
    ctx.close()
    rows, flagged = predictor.rows()
    return {"runs": runs, "steps": steps, "rows": rows, "flagged": flagged, "n": cloud.n}


def default_weights_path() -> Path:
    return Path(__file__).resolve().parent / "predictor_euler2d.npz"


def holdout_path() -> Path:
    return Path(__file__).resolve().parent / "predictor_euler2d_holdout.json"


def holdout_thresholds(hcc, weights, thresholds, runs: int = 8, h: float = 2e-3, t_end: float = 0.2,
                       every: int = 100, seed0: int = 900000, min_precision: float = 0.9, log=None) -> dict:
    """Precision and recall of a trained network on held-out runs: the training recipe's seeded 2-D Euler runs with
    seeds outside the training range, EVERY row kept (the training set keeps only a small share of the unflagged
    rows, so its held-out precision overstates the precision a step sees). The chosen threshold is the lowest one
    whose held-out precision reaches `min_precision`: a pre-lowered particle that MOOD would not have flagged costs
    accuracy, a missed one only a recompute."""
    pred = TroubledPointPredictor(capacity=1 << 26, neg_keep=1.0, seed=seed0)
    pred.load(weights)
    gen = generate_training_set(hcc, pred, runs, h, t_end, seed0=seed0, every=every, log=log)
    table = {}
    for thr in thresholds:
        table[f"{thr:g}"] = pred.evaluate(float(thr), holdout=1.0)
    chosen = next((thr for thr in sorted(thresholds) if table[f"{thr:g}"]["precision"] >= min_precision), None)
    pred.close()
    return {"runs": runs, "seeds": [seed0, seed0 + runs - 1], "rows": gen["rows"], "flagged": gen["flagged"],
            "every": every, "h": h, "t_end": t_end, "min_precision": min_precision, "table": table,
            "threshold": chosen}
