"""Train the warm-start MLP and evaluate it (the learned warm-start configuration).

    python -m tgvreconclaude_gb300.train_warmstart [--train 100] [--eval 20] [--out weights.npz]

1. Training data: (features, converged u - median indicator) pairs from the
   plain solver on `--train` seeded scenes alternating the torus and
   three-object kinds (16 cameras at 320x240); converged = reference
   initialisation run to a relative residual of 1e-6 (at most 6000 iterations
   per level); cubes whose converged |u| > 1.5 (no fixed point) are left out.
2. Training: this package's forward/backward/Adam kernels on the GPU.
3. Evaluation on `--eval` held-out seeds: iterations and time to a relative
   residual of 1e-4 for the solver from a zero start (every level from
   u = v = p = q = 0), from the network's prediction (every level from the
   predicted u), and from the reference initialisation (median, then the
   parent's u and v at each level); all three solve the reference's problem.
Prints one JSON line with the per-seed records and the medians.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import api, warmstart as WS


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=100)
    ap.add_argument("--eval", type=int, default=20)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--tol", type=float, default=1e-4)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "data", "warmstart_nb10.npz"))
    ap.add_argument("--load", default="", help="skip training, evaluate these weights")
    a = ap.parse_args(argv)

    t0 = time.time()
    if a.load:
        mlp = WS.WarmStartMLP.load(a.load)
        info = {"loaded": a.load}
    else:
        X, t = WS.dataset(range(a.train))
        t1 = time.time()
        mlp = WS.WarmStartMLP(10, seed=0)
        loss0, _ = mlp.grad(X[:200000], t[:200000])
        loss = mlp.train(X, t, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=0)
        t2 = time.time()
        os.makedirs(os.path.dirname(a.out), exist_ok=True)
        mlp.save(a.out)
        info = {"train_scenes": a.train, "samples": int(len(X)), "data_s": round(t1 - t0, 1),
                "train_s": round(t2 - t1, 1), "loss_initial": loss0, "loss_final": loss, "weights": a.out}

    recs, summary = WS.evaluate(mlp, range(1000, 1000 + a.eval), tol=a.tol)
    print(json.dumps({"info": info, "summary": summary, "records": recs}), flush=True)


if __name__ == "__main__":
    main()
