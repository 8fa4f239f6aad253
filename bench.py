"""Benchmark of the GB300 REPROBUS chemistry step.

One step = one 15-min chemistry step (55 species) over every cell of the
2 x 2 deg x L137 grid (180 x 91 x 137 = 2,244,060 cells), FP64, seeded
synthetic state (the reference's ECMWF/restart inputs are not available).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours       value: device-resident step through reprobus_chem_step_dev, CUDA
           events on the launching stream; e2e: the host entry point
           reprobus_chem_step with pinned host arrays (H2D + step + D2H).
reference  the reference's chemistry step restated on the CPU (oracle/,
           the reference itself is Fortran and cannot be compiled here),
           timed on the host cores on a bounded sample of the same grid.
N > 1 (torchrun): every rank integrates its own grid (weak scaling, no
exchange: the chemistry has no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s (55 sp, 15-min) 1 GB300: MLP+mixed vs plain FP64, same 1e-6 err"
WORKLOAD = "2x2deg L137 global grid, 180x91x137 = 2,244,060 cells, one 15-min step, 55 species, FP64 state"
BYTES_PER_CELL = 1008  # compulsory FP64 SoA traffic per cell-step: 63 reads + 63 writes
# Algorithmic FP64 work of the reference scheme per cell-step on the cfg1 grid:
# 6612 +-*/ (612 of them divisions) + 181 transcendentals, each counted once
# (python -m oracle.count_ops --config cfg1 --rows 12).
OPS_PER_CELL = 6793.08
# DRAM bytes per cell-iteration of the mixed solve kernel, from one ncu capture
# of the 394,560-cell grid (1.35 GB per launch at 3.60 iterations per cell):
# the cell records re-read from DRAM, proportional to the cell-iterations;
# scaled to the benchmark launch
SOLVE_DRAM_BYTES_PER_CELL_ITER = 950.0
# the accuracy leg: seeded columns of the grid (x 137 levels ~ 1.1e4 cells)
# checked against the CPU FP64 oracle after the timed steps
ACCURACY_COLUMNS = 80
ACCURACY_SEED = 2024
STEP_TOL = 1e-4  # the Newton solvers' default step tolerance (both solvers alike)


def newton_ops():
    """Arithmetic operators (+ - * /) of one Newton iteration, counted in the
    generated source (reprobus_gb300/csrc/newton_gen.cuh; an FMA counts 2, a
    quotient nt_div or reciprocal nt_rcp one): residual (day, night), Jacobian
    (day, night), factorisation + solve."""
    path = os.path.join(ROOT, "reprobus_gb300", "csrc", "newton_gen.cuh")
    src = open(path).read()

    def body(name):
        i = src.index(f"void {name}(")
        j = src.index("\n}\n", i)
        lines = [ln.split("//")[0] for ln in src[i:j].splitlines()[1:]]
        text = "\n".join(lines)
        return sum(text.count(op) for op in ("*", " + ", " - ", "/", "-=", "nt_div<", "nt_rcp<"))

    return {"res_day": body("nt_residual_day"), "res_night": body("nt_residual_night"),
            "jac_day": body("nt_jacobian_day"), "jac_night": body("nt_jacobian_night"),
            "factor": body("nt_factor_solve"), "update": 3 * 57, "rhs": 2 * 57}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        out.update(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=reasons, samples=len(rows))
        return out


def _gemm_peak_tflops(torch, dtype, n):
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def fp64_peak_tflops(torch):
    """cuBLAS DGEMM 4096^3, best of 5 (CUDA events): the FP64 denominator."""
    return _gemm_peak_tflops(torch, torch.float64, 4096)


def fp32_peak_tflops(torch):
    """cuBLAS SGEMM 8192^3 with TF32 off (FP32 FMA on the CUDA cores), best
    of 5: the FP32 denominator."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        return _gemm_peak_tflops(torch, torch.float32, 8192)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def _rows(case, nrows):
    """nrows latitude rows (1-based) spread evenly from pole to pole."""
    return sorted({int(round(x)) for x in np.linspace(1, case.nlat, nrows)})


CPU_ROWS = 12  # latitude rows of the CPU sample, the same in both CPU legs


def _time_rows(case, rows, nthreads=0):
    from oracle import oracle
    st = case.state_copy()
    t0 = time.perf_counter()
    for r in rows:
        oracle.step(case, niter=5, fuse=True, ilat0=r, ilat1=r, nthreads=nthreads, state=st)
    return time.perf_counter() - t0


def cpu_sample(case, nrows=CPU_ROWS, nthreads=0):
    """One timing of the oracle (the reference scheme restated on the CPU,
    OpenMP over longitude blocks of a row) on nrows latitude rows spread pole
    to pole: cell-steps/s. The per-cell rate does not depend on which rows
    are sampled beyond the day/night mix, which spreading them keeps."""
    import multiprocessing
    rows = _rows(case, nrows)
    dt = _time_rows(case, rows, nthreads)
    cells = len(rows) * case.nlon * case.nivbas
    cores = nthreads if nthreads > 0 else multiprocessing.cpu_count()
    return {"value": cells / dt, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(rows)} latitude rows spread pole to pole x {case.nlon} lon x {case.nivbas} levels "
                      f"= {cells} cells per step, oracle/chem_oracle.c restating the reference scheme "
                      f"(niter 5, conserv and clamps), OpenMP {cores} threads", "seconds": dt}


def cpu_baseline(case, target_s=10.0):
    """The oracle on the machine's host cores: all cores (median of repeats of the
    sample the reference arm times, about target_s in all) and one thread
    (the reference is serial: the same rows, one repeat)."""
    runs = [cpu_sample(case)]
    while sum(r["seconds"] for r in runs) < target_s and len(runs) < 20:
        runs.append(cpu_sample(case))
    out = dict(runs[0])
    out["value"] = statistics.median(r["value"] for r in runs)
    out["repeats"] = len(runs)
    out.pop("seconds", None)
    one = cpu_sample(case, nthreads=1)
    out["one_thread"] = {"value": one["value"], "unit": "cell-steps/s", "cores": 1,
                         "seconds": round(one["seconds"], 3), "sample": "the same rows, 1 thread"}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from reprobus_gb300 import inputs
    case = inputs.make_case("cfg1", seed=1234)
    for _ in range(args.warmup):
        cpu_sample(case)
    vals = [cpu_sample(case) for _ in range(args.steps)]
    v = statistics.median([x["value"] for x in vals])
    cb = dict(vals[0])
    cb["value"] = v
    cb.pop("seconds", None)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference inputs unavailable)",
            "config": {"workload": WORKLOAD, "sample": cb["sample"]},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def column_bench(torch, h, case, dc, stream, hbm_peak, reps=5):
    """Times the column physics around the step on the benchmark grid
    (device-resident arrays, CUDA events on the handle's stream): per entry
    point the mean device time, the algorithmic bytes (each array element the
    reference routine reads or writes, counted once) and the HBM fraction."""
    from reprobus_gb300 import ChemStep
    # the reference's level split: chemistry on levels 1..94, forcing below
    nlon, nlat, niv, nb, nh = case.nlon, case.nlat, case.niv, min(94, case.niv), case.nivhau
    ncol = nlon * nlat
    h = ChemStep(case.ajl, case.o3up, nlon, nlat, niv, nivbas=nb, nivhau=nh, nrappmax=case.nrappmax, niter=5,
                 flags=0, troe=case.troe)
    h.set_stream(stream)
    rng = np.random.default_rng(11)
    f64 = dict(dtype=torch.float64, device="cuda")
    vsed = torch.rand(ncol * nb, **f64) * 2e-3
    ph2o = torch.rand(ncol * nb, **f64)
    pno3 = torch.rand(ncol * nb, **f64)
    co = torch.full((ncol,), 1e-7, **f64)
    hj1 = torch.rand(ncol * niv, **f64) * 1e-3
    aaa, bbb = inputs_l137()
    aaa_d, bbb_d = torch.tensor(aaa, **f64), torch.tensor(bbb, **f64)
    psol = torch.tensor(rng.uniform(980., 1030., ncol), **f64)
    relief = torch.zeros(ncol, **f64)
    alt = torch.empty(ncol * niv, **f64)
    q0, h0 = dc["qj1"].clone(), dc["hc"].clone()
    h2o = dc["qj1"][2 * ncol * niv:3 * ncol * niv]  # regular-grid H2O (slot 3)
    nivh2o = min(59, nb + 1)
    ksed = max(nivh2o - nh, 0)
    calls = {
        "sedimentation": (lambda: h.sedimentation_dev(dc["trajpre"], dc["trajtem"], 1, dc["qj1"], vsed, nivh2o, ph2o,
                                                      pno3, 10800.),
                          ncol * 8 * (5 * (nb - nh + 2) + 2 * (ksed + 1) + ksed + 3 * (nb - nh + 1))),
        "forcing": (lambda: h.forcing_dev(2010, 3, 900., dc["trajpre"], 1, dc["qj1"], dc["hc"], co_month=co, hj1=hj1,
                                          nivh2oecmwf=nivh2o),
                    ncol * 8 * ((niv - nb) * 21 + 2 * (niv - nb + 1) + 1 + 2 * (niv - nivh2o + 1))),
        "altitude": (lambda: h.altitude_dev(relief, psol, aaa_d, bbb_d, dc["trajtem"], h2o, dc["trajlon"],
                                            dc["trajlat"], dc["trajpre"], alt),
                     ncol * 8 * (5 * niv + 2) + ncol * niv * 8 * 9),
    }
    out = {}
    for name, (fn, nbytes) in calls.items():
        fn()
        ms = 0.0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
        ms /= reps
        gbs = nbytes / (ms * 1e-3) / 1e9
        out[name] = {"ms": round(ms, 4), "bytes": int(nbytes), "achieved_gbs": round(gbs, 1),
                     "frac_hbm": round(gbs / hbm_peak, 4)}
    dc["qj1"].copy_(q0)
    dc["hc"].copy_(h0)
    h.close()
    return out


def inputs_l137():
    from reprobus_gb300 import inputs
    return inputs.l137_levels()


ARMS = {"ref5": "reference scheme, 5 fixed passes (drop-in)",
        "newton64": "Newton to the fixed point of the reference map, FP64 Jacobian",
        "mixed": "Newton to the fixed point, FP32 Jacobian+LU, FP64 residual/update",
        "mlp": "Newton to the fixed point, FP32 Jacobian+LU, FP64 residual/update, learned restart of the cells "
               "whose plain start misses (BF16 MLP on tensor cores)"}
SOLVER_ID = {"ref5": 0, "newton64": 1, "mixed": 2, "mlp": 2}  # REPROBUS_SOLVER_*


class Accuracy:
    """The accuracy leg: a seeded sample of whole columns of the grid, their
    answer from the CPU FP64 oracle (Oracle-C fixed point and the reference's
    5-pass answer, with conserv and the clamps), and per arm the error of the
    answer the GPU produced in its last timed step on those columns. Runs
    outside every timed region."""

    def __init__(self, case, ncol=ACCURACY_COLUMNS, seed=ACCURACY_SEED):
        from oracle import accuracy
        rng = np.random.default_rng(seed)
        pick = rng.choice(case.nlon * case.nlat, size=min(ncol, case.nlon * case.nlat), replace=False)
        self.ilon, self.ilat = pick % case.nlon, pick // case.nlon
        self.case = case
        self.sub = case.columns(self.ilon, self.ilat)
        t0 = time.perf_counter()
        self.ref = accuracy.Reference(self.sub, fuse=True)
        self.oracle_s = time.perf_counter() - t0

    def check(self, dc, against="fixed_point"):
        got = {f: self.case.gather_columns(dc[f].cpu().numpy().reshape(getattr(self.case, f).shape, order="F"),
                                           self.ilon, self.ilat) for f in ("qj1", "hc")}
        return self.ref.report(got, against=against)

    def describe(self):
        return {"columns": int(len(self.ilon)), "cells": int(self.sub.ncells), "seed": ACCURACY_SEED,
                "oracle": "Oracle-C (FP64 fixed point of the reference pass map) + conserv + clamps",
                "oracle_converged": int((self.ref.stat >= 0).sum()),
                "oracle_stages": np.bincount(self.ref.stage, minlength=7).tolist(),
                "oracle_s": round(self.oracle_s, 2)}


def time_arms(torch, h, case, dc, stream, arms, steps, warmup, net, npass_of, world, acc=None):
    """Times each solver arm on the device-resident state: warm-up steps, one
    step with statistics, then `steps` timed steps (CUDA events on the
    handle's stream, each from the same restored start state). With acc the
    last timed step's answer is checked against the oracle afterwards."""
    from reprobus_gb300.replicas import max_over_ranks, whole_job_rate
    a = dc.args()
    state = ("qj1", "hc", "vsed3d", "parth2osed", "parthno3sed", "surfarea", "sza3d")
    pristine = {f: dc[f].clone() for f in state}

    def restore():
        with torch.cuda.stream(stream):
            for f in state:
                dc[f].copy_(pristine[f])

    def step(stats=False):
        return h.step_dev(1, case.nlat, case.daynum, case.dt, *a, stats=stats)

    results = {}
    for name in arms:
        h.set_solver(SOLVER_ID[name], npass=npass_of(name), maxit=12, tol=STEP_TOL)
        h.set_mlp(net if name == "mlp" else None)
        for _ in range(max(warmup, 3)):
            restore()
            step()
        restore()
        st = step(stats=True)  # launches per step, kernel time, solver statistics
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for e0, e1 in evs:
            restore()
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(sum(e0.elapsed_time(e1) for e0, e1 in evs))
        conv = case.ncells - st["fallbacks"]
        day_frac = float((dc["sza3d"][:case.ncells] <= 95.0).double().mean())
        newton = name != "ref5"
        results[name] = {"cells_per_s": whole_job_rate(case.ncells, world, steps, ms * 1e-3),
                         "ms_per_step": ms / steps, "kernel_ms": st["device_ms"],
                         "solve_ms": st["solve_ms"] if newton else None,
                         "launches_per_step": st["kernel_launches"], "fallbacks": st["fallbacks"],
                         "mean_newton_iters": (st["newton_iters"] / conv) if newton and conv else None,
                         "iters_per_cell": ((st["newton_iters"] + st["failed_iters"]) / case.ncells
                                            if newton else None),
                         "warm_restarts": st["warm_restarts"] if name == "mlp" else None,
                         "day_frac": day_frac,
                         "max_newton_iters": st["max_newton_iters"] if newton else None,
                         "solve_shape": None if not newton else
                         {"lanes_per_block": st["lanes_per_block"], "blocks_per_sm": st["blocks_per_sm"],
                          "z_shared": st["z_shared"]}}
        if acc is not None:
            results[name]["accuracy"] = acc.check(dc, "ref5" if name == "ref5" else "fixed_point")
    restore()
    torch.cuda.synchronize()
    return results


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg1", help="cfg1 (180x91x137), cfg2, cfg4, or grid (--nlon x --nlat)")
    ap.add_argument("--nlon", type=int, default=180)
    ap.add_argument("--nlat", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-columns", action="store_true", help="skip timing the column physics kernels")
    ap.add_argument("--no-accuracy", action="store_true", help="skip checking the timed answers against the oracle")
    ap.add_argument("--no-polar", action="store_true", help="skip the 30%%-polar-winter grid block")
    ap.add_argument("--polar-steps", type=int, default=5, help="timed steps per arm on the polar-winter grid")
    ap.add_argument("--npass", type=int, default=0,
                    help="reference passes before Newton for the plain solvers (0: each solver's default)")
    ap.add_argument("--lanes", type=int, default=0,
                    help="Newton solve kernel lanes per block (0: autotune)")
    ap.add_argument("--bps", type=int, default=0, help="Newton solve kernel blocks per SM (0: all that fit)")
    ap.add_argument("--zshared", type=int, default=0, help="with --lanes: right-hand side in shared memory")
    ap.add_argument("--solver", default="all", choices=["all", "ref5", "newton64", "mixed", "mlp"],
                    help="all: time the four arms, headline = mlp")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from reprobus_gb300 import ChemStep, inputs
    from reprobus_gb300.chem import FUSE_CONSERV
    from reprobus_gb300.resident import DeviceCase

    from reprobus_gb300.replicas import max_over_ranks, replica_seed, whole_job_rate
    if args.config == "grid":
        case = inputs.make_case("grid", seed=replica_seed(1234, rank), nlon=args.nlon, nlat=args.nlat)
    else:
        case = inputs.make_case(args.config, seed=replica_seed(1234, rank))
    run = list(ARMS) if args.solver == "all" else [args.solver]
    headline = "mlp" if args.solver == "all" else args.solver
    net = None
    if "mlp" in run:
        from reprobus_gb300 import mlp as mlpmod
        net = mlpmod.Mlp(batch_cap=128, seed=0)
        net.load()  # reprobus_gb300/data/mlp_warmstart.npz, trained by reprobus_gb300.train_mlp
    h = ChemStep.for_case(case, niter=5, flags=FUSE_CONSERV)
    if args.lanes:
        h.set_tuning(args.lanes, args.bps, args.zshared)
    stream = torch.cuda.Stream()
    h.set_stream(stream)
    dc = DeviceCase(case)

    def npass_of(name):
        # the network is trained on the default 5-pass start
        if name == "mlp":
            return 5
        return args.npass if args.npass > 0 else 5

    # the oracle's answers for the accuracy leg (CPU, before any timing)
    acc = Accuracy(case) if (rank == 0 and not args.no_accuracy) else None

    clocks = Clocks(local)
    clocks.start()
    results = time_arms(torch, h, case, dc, stream, run, args.steps, args.warmup, net, npass_of, world, acc)
    clk = clocks.stop()
    h.set_solver(SOLVER_ID[headline], npass=npass_of(headline), maxit=12, tol=STEP_TOL)
    h.set_mlp(net if headline == "mlp" else None)
    R = results[headline]
    ms_step = R["ms_per_step"]
    kernel_ms = R["kernel_ms"]
    launches_per_step = R["launches_per_step"]
    ncell = case.ncells
    value = R["cells_per_s"]

    # end to end through the host entry point, pinned host arrays
    e2e = None
    if not args.no_e2e:
        pin = lambda x: torch.from_numpy(np.ascontiguousarray(x.reshape(-1, order="F"))).pin_memory()
        hp = {f: pin(getattr(case, f)) for f in ("alt", "trajlon", "trajlat", "trajpre", "trajtem")}
        st0 = case.state_copy()
        hs = {f: pin(st0[f]) for f in st0}
        view = lambda t, like: t.numpy().reshape(like.shape, order="F")
        harr = [view(hp[f], getattr(case, f)) for f in ("alt", "trajlon", "trajlat", "trajpre", "trajtem")]
        sarr = [view(hs[f], st0[f]) for f in ("qj1", "hc", "vsed3d", "parth2osed", "parthno3sed", "surfarea",
                                             "sza3d")]
        hstep = lambda: h.step(1, case.nlat, case.daynum, case.dt, *harr, case.irapp, *sarr, stats=False)
        def hrestore():  # every step integrates the same start state (outside the timed region)
            for f, arr in zip(("qj1", "hc", "vsed3d", "parth2osed", "parthno3sed", "surfarea", "sza3d"), sarr):
                np.copyto(arr, st0[f])

        hrestore()
        hstep()
        torch.cuda.synchronize()
        # single calls vary by a few ms from call to call (host side): the
        # median of several calls, the mean and the fastest beside it
        n_e2e = max(7, args.steps)
        calls = []
        for _ in range(n_e2e):
            hrestore()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            hstep()
            torch.cuda.synchronize()
            calls.append(time.perf_counter() - t0)
        te = max_over_ranks(statistics.median(calls))
        pl = case.nlon * case.nlat * case.niv * 8
        pb = case.nlon * case.nlat * case.nivbas * 8
        h2d = pb * 5 + pl * 43 + pb * 15
        d2h = pl * 43 + pb * 15 + pb * 4 + (case.nivbas - case.nivhau + 1) * case.nlon * case.nlat * 8
        e2e = {"value": whole_job_rate(ncell, world, 1, te), "unit": "cell-steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": te * 1e3, "calls": n_e2e, "statistic": "median",
               "ms_mean": statistics.mean(calls) * 1e3, "ms_min": min(calls) * 1e3}
        del hp, hs, harr, sarr

    # the 30 %-polar-winter grid at full size: the Newton arms, timed and checked
    polar = None
    parms = [x for x in ("newton64", "mixed", "mlp") if x in run]
    if not args.no_polar and args.config == "cfg1" and parms:
        pcase = inputs.make_case("cfg2", seed=replica_seed(4321, rank))
        pacc = Accuracy(pcase) if (rank == 0 and not args.no_accuracy) else None
        pdc = DeviceCase(pcase)
        ph = ChemStep.for_case(pcase, niter=5, flags=FUSE_CONSERV)  # the case's own tables (o3up is seeded)
        if args.lanes:
            ph.set_tuning(args.lanes, args.bps, args.zshared)
        ph.set_stream(stream)
        pres = time_arms(torch, ph, pcase, pdc, stream, parms, args.polar_steps, args.warmup, net, npass_of, world,
                         pacc)
        ph.close()
        polar = {"workload": f"cfg2: {pcase.nlon}x{pcase.nlat}x{pcase.niv} = {pcase.ncells} cells, 30% of the "
                             f"columns in polar winter (T 183-195 K, SZA > 95, active ClOx), day {pcase.daynum}",
                 "steps": args.polar_steps, "solvers": pres,
                 "mixed_vs_fp64_newton": (pres["mixed"]["cells_per_s"] / pres["newton64"]["cells_per_s"]
                                          if "mixed" in pres and "newton64" in pres else None),
                 "mlp_mixed_vs_fp64_newton": (pres["mlp"]["cells_per_s"] / pres["newton64"]["cells_per_s"]
                                              if "mlp" in pres and "newton64" in pres else None),
                 "accuracy_sample": pacc.describe() if pacc else None}
        del pdc
        torch.cuda.empty_cache()

    line = None
    if rank == 0:
        peak64 = fp64_peak_tflops(torch)
        peak32 = fp32_peak_tflops(torch)
        try:
            hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
            hbm_src = "MEASURED_PEAKS.json hbm_gbs (measured copy)"
        except Exception:
            hbm_peak = 6800.0
            hbm_src = "fallback 6.8 TB/s"
        ach_gbs = BYTES_PER_CELL * ncell / (kernel_ms * 1e-3) / 1e9
        # the work of a step: the reference scheme's FP64 operations per cell
        # (fixed across solvers so that their figures compare)
        step_tf = OPS_PER_CELL * ncell / (kernel_ms * 1e-3) / 1e12
        roof = {"bound": "fp64", "unit": "TFLOP/s", "peak": round(peak64, 4),
                "peak_source": "cuBLAS DGEMM 4096^3 measured live in this run",
                "flops_per_cell": OPS_PER_CELL,
                "flops_note": "algorithmic work = the reference scheme's FP64 operations per cell-step "
                              "(+-*/ and transcendentals counted once each, oracle operation counter), the same "
                              "for every solver; the peak counts an FMA as 2",
                "step": {"ms": round(kernel_ms, 4), "achieved": round(step_tf, 4),
                         "frac": round(step_tf / peak64, 4)},
                "hbm": {"achieved": round(ach_gbs, 2), "peak": hbm_peak, "peak_source": hbm_src, "unit": "GB/s",
                        "frac": round(ach_gbs / hbm_peak, 5), "bytes_per_cell": BYTES_PER_CELL}}
        if headline == "ref5":
            roof.update(kernel="whole step", kernel_ms=round(kernel_ms, 4), achieved=round(step_tf, 4),
                        frac=round(step_tf / peak64, 4), traffic=None)
        else:
            # dominant kernel: the persistent Newton solve kernel (k_nt_solve)
            ops = newton_ops()
            f = R["day_frac"]
            res = f * ops["res_day"] + (1 - f) * ops["res_night"]
            jac = f * ops["jac_day"] + (1 - f) * ops["jac_night"]
            mixed = headline in ("mixed", "mlp")
            fp64_it = res + ops["update"] + (0 if mixed else jac + ops["factor"] + ops["rhs"])
            fp32_it = (jac + ops["factor"] + ops["rhs"]) if mixed else 0
            iters = R["iters_per_cell"] * ncell
            sm = R["solve_ms"] * 1e-3
            ach = OPS_PER_CELL * ncell / sm / 1e12
            traffic = SOLVE_DRAM_BYTES_PER_CELL_ITER * iters if mixed else None
            fp32_tf = fp32_it * iters / sm / 1e12
            roof.update(kernel="k_nt_solve", kernel_ms=round(R["solve_ms"], 4), achieved=round(ach, 4),
                        frac=round(ach / peak64, 4), traffic=traffic,
                        traffic_ratio=(round(traffic / (BYTES_PER_CELL * ncell), 3) if traffic else None),
                        traffic_note="DRAM bytes per launch: 950 B per cell-iteration from an ncu capture of the "
                                     "394,560-cell grid, times this launch's cell-iterations; ratio against the "
                                     "step's algorithmic 1,008 B per cell",
                        solver_ops={"fp64_ops_per_iteration": round(fp64_it, 1),
                                    "fp32_ops_per_iteration": round(fp32_it, 1),
                                    "iterations_per_cell": round(R["iters_per_cell"], 3),
                                    "fp64_tflops": round(fp64_it * iters / sm / 1e12, 4),
                                    "fp64_frac": round(fp64_it * iters / sm / 1e12 / peak64, 4),
                                    "note": "operators the solver executes, counted in the generated source (an "
                                            "FMA counts 2), times the step's iterations, over the solve kernel's "
                                            "CUDA-event time"},
                        fp32={"achieved": round(fp32_tf, 4), "peak": round(peak32, 3),
                              "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured live in this run",
                              "frac": round(fp32_tf / peak32, 5) if mixed else None})
        cols = None
        if not args.no_columns:
            cols = column_bench(torch, h, case, dc, stream, hbm_peak)
        cb = None
        if not args.no_cpu_baseline:
            cb = cpu_baseline(case)
        line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference inputs unavailable)",
                "config": {"workload": WORKLOAD if args.config == "cfg1" else
                           f"{args.config}: {case.nlon}x{case.nlat}x{case.niv} = {case.ncells} cells, one 15-min step",
                           "solver": ARMS[headline],
                           "timing": "each timed step starts from the same restored device state",
                           "cells": ncell, "l2": "inputs larger than L2 (1.2 GB resident state)",
                           "parallelism": f"replicas x{world}"},
                "gpu_launches": launches_per_step * args.steps,
                "solvers": results,
                "mixed_vs_fp64_newton": (results["mixed"]["cells_per_s"] / results["newton64"]["cells_per_s"]
                                         if "mixed" in results and "newton64" in results else None),
                "mlp_mixed_vs_fp64_newton": (results["mlp"]["cells_per_s"] / results["newton64"]["cells_per_s"]
                                             if "mlp" in results and "newton64" in results else None),
                "accuracy_sample": acc.describe() if acc else None,
                "polar_winter": polar,
                "roofline": roof, "e2e": e2e, "cpu_baseline": cb, "clocks": clk, "columns": cols}
        print(json.dumps(line))
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
