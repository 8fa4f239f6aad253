"""Resident multi-step run of the chemistry step: N consecutive 15-min steps
on a grid whose state never leaves the GPU, the solar zenith angle following
the diurnal cycle (the day number advances by dt every step) and, between
steps, a seeded smooth multiplicative perturbation of the transported
species (+-amp, correlation length ~corr cells along longitude and latitude)
standing in for transport.

Two solvers run the same sequence (same perturbations); the report gives
cell-steps/s of each (CUDA events around the steps only) and the drift of the
O3 (ox), Cly and NOy family totals (sums of the mixing ratios of those
transported slots over all cells) of the first against the second.

    python -m reprobus_gb300.resident_run --config cfg4 --steps 96 --solver mlp --against newton64

torch supplies device memory, streams and the perturbation fields; the step
runs in libreprobus_gb300.so.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import chem, inputs
from .species import LONG

FAMILIES = {"ox": LONG.index("ox"), "cly": LONG.index("cly"), "noy": LONG.index("noy")}
SOLVERS = {"ref5": chem.SOLVER_REF5, "newton64": chem.SOLVER_NEWTON64, "mixed": chem.SOLVER_NEWTON_MIXED,
           "mlp": chem.SOLVER_NEWTON_MIXED}


def perturbation(shape_lonlat, nlev, amp, corr, gen):
    """exp(amp * f) with f a smooth unit-variance field: white noise smoothed
    by a separable box filter of width corr along longitude (periodic) and
    latitude, repeated over the levels."""
    import torch
    nlon, nlat = shape_lonlat
    w = torch.randn(nlat, nlon, device="cuda", generator=gen, dtype=torch.float64)
    k = max(1, int(corr))
    for _ in range(2):  # two box passes ~ a triangle filter
        w = sum(torch.roll(w, s, dims=1) for s in range(-(k // 2), k - k // 2)) / k
        wp = torch.nn.functional.pad(w[None, None], (0, 0, k // 2, k - 1 - k // 2), mode="replicate")[0, 0]
        w = sum(wp[i:i + nlat] for i in range(k)) / k
    w = (w - w.mean()) / w.std()
    return torch.exp(amp * w)  # (nlat, nlon): the (lat, lon) order of a level plane of the Fortran arrays


def run(case, solver, steps, amp, corr, seed, net=None, graph=True, log=None):
    import torch
    from .resident import DeviceCase
    dc = DeviceCase(case)
    h = chem.ChemStep.for_case(case, niter=5, flags=chem.FUSE_CONSERV)
    h.set_solver(SOLVERS[solver])
    if solver == "mlp":
        h.set_mlp(net)
    h.set_graph(graph)
    stream = torch.cuda.Stream()
    h.set_stream(stream)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    nlon, nlat, niv = case.nlon, case.nlat, case.niv
    q = dc["qj1"].view(43, niv, nlat, nlon)
    a = dc.args()
    # one untimed step on a copy: tunes the solve kernel and readies the graph
    warm = DeviceCase(case)
    h.step_dev(1, nlat, case.daynum, case.dt, *warm.args())
    del warm
    totals = []
    ms = 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for s in range(steps):
        day = case.daynum + s * case.dt / 86400.0
        with torch.cuda.stream(stream):
            e0.record(stream)
            h.step_dev(1, nlat, day, case.dt, *a)
            e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
        with torch.cuda.stream(stream):
            totals.append([float(q[i].sum()) for i in FAMILIES.values()])
            if s + 1 < steps:
                # transport stand-in: the 42 transported slots times a smooth field
                f = perturbation((nlon, nlat), niv, amp, corr, gen)
                q[:42] *= f[None, None, :, :]
        if log and s % max(1, steps // 8) == 0:
            log(f"{solver} step {s}: {ms / (s + 1):.1f} ms/step")
    torch.cuda.synchronize()
    h.close()
    return {"ms_per_step": ms / steps, "cell_steps_per_s": case.ncells * steps / (ms * 1e-3),
            "totals": np.array(totals)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--config", default="cfg4")
    ap.add_argument("--nlon", type=int, default=None)
    ap.add_argument("--nlat", type=int, default=None)
    ap.add_argument("--steps", type=int, default=96)
    ap.add_argument("--solver", default="mlp", choices=list(SOLVERS))
    ap.add_argument("--against", default="newton64", choices=list(SOLVERS) + ["none"])
    ap.add_argument("--amp", type=float, default=0.02)
    ap.add_argument("--corr", type=float, default=10.0)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    kw = {}
    if args.config == "grid":
        kw = {"nlon": args.nlon, "nlat": args.nlat}
    t0 = time.time()
    case = inputs.make_case(args.config, seed=1234, **kw)
    net = None
    if "mlp" in (args.solver, args.against):
        from . import mlp
        net = mlp.Mlp(batch_cap=128)
        net.load()
    print(f"case {args.config}: {case.ncells} cells ({time.time() - t0:.1f} s to build)", flush=True)
    res = {args.solver: run(case, args.solver, args.steps, args.amp, args.corr, args.seed, net,
                            graph=not args.no_graph, log=print)}
    if args.against != "none":
        res[args.against] = run(case, args.against, args.steps, args.amp, args.corr, args.seed, net,
                                graph=not args.no_graph, log=print)
    out = {"config": args.config, "cells": int(case.ncells), "steps": args.steps, "amp": args.amp,
           "corr": args.corr, "graph": not args.no_graph}
    for k, v in res.items():
        out[k] = {"ms_per_step": round(v["ms_per_step"], 3), "cell_steps_per_s": v["cell_steps_per_s"]}
    if args.against != "none":
        a, b = res[args.solver]["totals"], res[args.against]["totals"]
        drift = (a - b) / np.abs(b)
        out["drift_vs_" + args.against] = {
            name: {"final": float(drift[-1, i]), "max_abs": float(np.abs(drift[:, i]).max())}
            for i, name in enumerate(FAMILIES)}
        t0_ = b[0]
        out["change_over_run_" + args.against] = {name: float((b[-1, i] - t0_[i]) / t0_[i])
                                                  for i, name in enumerate(FAMILIES)}
    print(json.dumps(out))
    if args.out:
        with open(args.out, "w") as f:
            json.dump(out, f, indent=1)
    return out


if __name__ == "__main__":
    main()
