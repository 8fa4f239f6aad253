"""Trains the network of the Newton solvers' learned restart on the GPU.

Training cells come from the plain FP64 Newton solver itself: seeded
synthetic grids (the reference's own initial/ECMWF files are not available)
with random day of year and time of day, half of them with 30% of the
columns in polar winter (the distributions of reprobus_gb300.inputs). Each
grid gives, per chemistry cell, the 64 features of its start state and the
log10 ratios of the solver's end-of-step mixing ratios to the start ones.

    python -m reprobus_gb300.train_mlp --cases 9 --steps 20000 \
        --out reprobus_gb300/data/mlp_warmstart.npz
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def make_training_set(cases, nlon, nlat, seed0=100, log=print, npass=5):
    import torch
    from . import inputs, mlp
    rng = np.random.default_rng(seed0)
    Xs, Ys = [], []
    for c in range(cases):
        day = float(rng.uniform(0.0, 365.0))
        pf = 0.3 if c % 2 else 0.0
        t0 = time.time()
        case = inputs.make_case("grid", seed=seed0 + 1 + c, nlon=nlon, nlat=nlat, daynum=day, polar_frac=pf)
        X, Y = mlp.sample(case, npass=npass)
        Xs.append(X)
        Ys.append(Y)
        log(f"case {c}: day {day:.2f} polar {pf} cells {X.shape[0]} ({time.time() - t0:.1f} s)")
    return torch.cat(Xs), torch.cat(Ys)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--cases", type=int, default=9)
    ap.add_argument("--nlon", type=int, default=180)
    ap.add_argument("--nlat", type=int, default=91)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    import torch
    from . import mlp
    X, Y = make_training_set(args.cases, args.nlon, args.nlat)
    Xv, Yv = make_training_set(1, args.nlon, args.nlat, seed0=900)  # validation grid for the output gate
    net = mlp.Mlp(batch_cap=args.batch, seed=args.seed)
    net.set_params(None, mlp.normalisation(X, Y))
    t0 = time.time()
    hist = mlp.train(net, X, Y, args.steps, batch=args.batch, lr=args.lr, seed=args.seed,
                     log_every=max(1, args.steps // 20))
    torch.cuda.synchronize()
    dt = time.time() - t0
    tau = mlp.fit_thresholds(net, Xv, Yv)
    summary = {"cells": int(X.shape[0]), "npass": 5, "steps": args.steps, "batch": args.batch, "train_s": round(dt, 2),
               "loss_first": float(np.mean(hist[:10])), "loss_last": float(np.mean(hist[-100:])),
               "outputs_on": int(np.isfinite(tau).sum()),
               "thresholds": [None if not np.isfinite(t) else float(t) for t in tau[:mlp.NY]]}
    print(json.dumps(summary))
    if args.out:
        p, n = net.get_params()
        np.savez(args.out, params=p, norm=n, summary=json.dumps(summary))
    return net, summary


if __name__ == "__main__":
    main()
