"""Train the troubled-point predictor shipped with the package (predictor_euler2d.npz).

Recipe: seeded 2-D Euler runs at 250k nodes (jittered lattice h = 2e-3 on the unit square, MUSCL2 + MOOD(EPD1,
MOODu1(1e-4 h^2)), Rusanov, SSP-RK3, CFL 0.4, transmissive walls, FP32 bulk) from random piecewise-constant states
over 2-6 Voronoi regions (rho, p ~ U[0.1, 2], u, v ~ U[-1, 1]) to t = 0.2. Every `every`-th step the features of
its start state and its MOOD flags are appended to the training rows on the device (every flagged particle,
unflagged ones with probability neg_keep). Then Adam on the GPU's tensor-core training kernels.

    python hypercloudcore.jl_gb300/train_predictor.py [--runs 200] [--out path]
    python hypercloudcore.jl_gb300/train_predictor.py --holdout-eval     # threshold table on held-out runs
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import sys
import time
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent


def package():
    if "hcc_gb300" in sys.modules:
        return sys.modules["hcc_gb300"]
    spec = importlib.util.spec_from_file_location("hcc_gb300", PKG / "__init__.py",
                                                  submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["hcc_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--runs", type=int, default=200)
    ap.add_argument("--h", type=float, default=2e-3)
    ap.add_argument("--t-end", type=float, default=0.2)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--neg-keep", type=float, default=0.02)
    ap.add_argument("--capacity", type=int, default=64 << 20)
    ap.add_argument("--iters", type=int, default=40000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--holdout", type=float, default=0.05)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", type=str, default=str(PKG / "predictor_euler2d.npz"))
    ap.add_argument("--holdout-eval", action="store_true",
                    help="only evaluate the weights in --out on held-out runs (every row kept) and write the "
                         "threshold table next to them")
    ap.add_argument("--holdout-runs", type=int, default=8)
    a = ap.parse_args(argv)
    hcc = package()
    learned = sys.modules["hcc_gb300.learned"]
    if a.holdout_eval:
        res = learned.holdout_thresholds(hcc, a.out, (0.9, 0.95, 0.97, 0.98, 0.99, 0.995, 0.998, 0.999),
                                         runs=a.holdout_runs, h=a.h, t_end=a.t_end, every=a.every,
                                         log=lambda m: print(m, flush=True))
        out = Path(a.out).with_name(Path(a.out).stem + "_holdout.json")
        out.write_text(json.dumps(res, indent=1) + "\n")
        print(json.dumps(res), flush=True)
        return res
    pred = hcc.TroubledPointPredictor(capacity=a.capacity, neg_keep=a.neg_keep, seed=a.seed, lr=a.lr)
    t0 = time.time()
    gen = learned.generate_training_set(hcc, pred, a.runs, a.h, a.t_end, seed0=a.seed * 100000, every=a.every,
                                        log=lambda m: print(m, flush=True))
    gen["seconds"] = time.time() - t0
    print(json.dumps({"generation": gen}), flush=True)
    t0 = time.time()
    pred.fit_norm(holdout=a.holdout)
    losses = []
    chunk = max(1, a.iters // 20)
    done = 0
    while done < a.iters:
        k = min(chunk, a.iters - done)
        losses.append(pred.train(k, batch=a.batch, holdout=a.holdout))
        done += k
    train_s = time.time() - t0
    ev = {str(t): pred.evaluate(t, a.holdout) for t in (0.3, 0.5, 0.7, 0.9)}
    meta = {"recipe": {k: v for k, v in vars(a).items() if k != "out"}, "generation": gen, "losses": losses,
            "train_seconds": train_s, "holdout_eval": ev}
    p, n = pred.params()
    np.savez(a.out, params=p, norm=n, meta=json.dumps(meta))
    print(json.dumps({"losses": losses[-3:], "train_seconds": train_s, "holdout_eval": ev}), flush=True)
    return meta


if __name__ == "__main__":
    main()
