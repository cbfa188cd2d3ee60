"""Train the warm-start network on fields the solver converges itself.

    python -m scft_gb300.train_warmstart [--train 20000] [--eval 4096] [--steps 8000] [--out PATH]

1. solves the training instances (L ~ U[2, 10], 64..512 elements, steps in
   {512..4096}) from the cold start to ||phi - f0||_inf <= 1e-6;
2. trains the network on the converged fields with the GPU kernels;
3. solves the tuning batch (warm-start evaluation workload, seed 43) cold and
   warm-started and reports iterations and converged solves/s of both;
4. saves the weights (npz) and the report (json next to it).
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import F32, ST_CONVERGED, api, workloads
from .warmstart import DEFAULT_WEIGHTS, generate_and_train


def evaluate(ws, held, tol=1e-6):
    out = {}
    with api.Batch(held) as b:
        for mode in ("cold", "warm"):
            b.reset()
            pred_ms = 0.0
            if mode == "warm":
                ws.predict(b)
                pred_ms = b.last_ms()
            r = b.solve(precision=F32, tol=tol)
            conv = int(((r["status"] & ST_CONVERGED) != 0).sum())
            ms = b.last_ms() + pred_ms
            out[mode] = {"converged": conv, "iterations_mean": float(r["iterations"].mean()),
                         "iterations_median": float(np.median(r["iterations"])), "ms": ms,
                         "solves_per_s": conv / (ms / 1e3), "predict_ms": pred_ms}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--eval", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    t0 = time.time()
    train = workloads.warmstart_train(a.train)
    ws, losses, stats = generate_and_train(train, steps=a.steps, batch=a.batch, lr=a.lr, seed=a.seed,
                                           log=lambda m: print(m, flush=True))
    t_train = time.time() - t0
    held = workloads.warmstart_eval(a.eval, seed=43)
    rep = evaluate(ws, held)
    rep.update({"train_instances": a.train, "train_converged": stats["solved"], "steps": a.steps,
                "batch": a.batch, "lr": a.lr, "final_loss": stats["final_loss"],
                "first_loss": float(np.mean(losses[:10])), "wall_s_generate_and_train": t_train,
                "iteration_ratio_warm_over_cold": rep["warm"]["iterations_mean"] / rep["cold"]["iterations_mean"],
                "speedup_warm_over_cold": rep["warm"]["solves_per_s"] / rep["cold"]["solves_per_s"]})
    ws.save(a.out, losses=losses)
    with open(os.path.splitext(a.out)[0] + ".json", "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    main()
