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
# of the 394,560-cell grid (profiles/k_nt_solve_mixed_grid180x16.md: 1.35 GB
# per launch at 3.79 iterations per cell): the cell records re-read from DRAM,
# proportional to the cell-iterations; scaled to the benchmark launch
SOLVE_DRAM_BYTES_PER_CELL_ITER = 899.0


def newton_ops():
    """Arithmetic operators (+ - * /) of one Newton iteration, counted in the
    generated source (reprobus_gb300/csrc/newton_gen.cuh; an FMA counts 2):
    residual (day, night), Jacobian (day, night), factorisation + solve."""
    path = os.path.join(ROOT, "reprobus_gb300", "csrc", "newton_gen.cuh")
    src = open(path).read()

    def body(name):
        i = src.index(f"void {name}(")
        j = src.index("\n}\n", i)
        lines = [ln.split("//")[0] for ln in src[i:j].splitlines()[1:]]
        text = "\n".join(lines)
        return sum(text.count(op) for op in ("*", " + ", " - ", "/", "-=")) - text.count("J[") * 0

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


def fp64_peak_tflops(torch):
    """cuBLAS DGEMM 4096^3, best of 5 (CUDA events): the FP64 denominator."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
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


def _rows(case, nrows):
    """nrows latitude rows (1-based) spread evenly from pole to pole."""
    return sorted({int(round(x)) for x in np.linspace(1, case.nlat, nrows)})


def _time_rows(case, rows, nthreads=0):
    from oracle import oracle
    st = case.state_copy()
    t0 = time.perf_counter()
    for r in rows:
        oracle.step(case, niter=5, fuse=True, ilat0=r, ilat1=r, nthreads=nthreads, state=st)
    return time.perf_counter() - t0


def cpu_baseline(case, target_s=12.0, nthreads=0):
    """Times the oracle (the reference scheme restated on the CPU, OpenMP over
    longitude blocks) on latitude rows spread over the same grid, sized to
    about target_s of CPU time."""
    import multiprocessing
    dt = _time_rows(case, _rows(case, 2), nthreads)
    n = int(min(case.nlat, max(2, 2 * target_s / max(dt, 1e-3))))
    rows = _rows(case, n)
    dt = _time_rows(case, rows, nthreads)
    cells = len(rows) * case.nlon * case.nivbas
    cores = nthreads if nthreads > 0 else multiprocessing.cpu_count()
    return {"value": cells / dt, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(rows)} latitude rows spread pole to pole x {case.nlon} lon x {case.nivbas} levels "
                      f"= {cells} cells, one step, oracle/chem_oracle.c (OpenMP, {cores} threads), {dt:.2f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from reprobus_gb300 import inputs
    case = inputs.make_case("cfg1", seed=1234)
    for _ in range(args.warmup):
        cpu_baseline_one(case)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline_one(case))
    v = statistics.median([x["value"] for x in vals])
    cb = dict(vals[0])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference inputs unavailable)",
            "config": {"workload": WORKLOAD, "sample": cb["sample"]},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline_one(case, nrows=12):
    import multiprocessing
    rows = _rows(case, nrows)
    dt = _time_rows(case, rows)
    cells = len(rows) * case.nlon * case.nivbas
    cores = multiprocessing.cpu_count()
    return {"value": cells / dt, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(rows)} latitude rows spread pole to pole x {case.nlon} lon x {case.nivbas} levels "
                      f"= {cells} cells per step, oracle/chem_oracle.c restating the reference scheme, "
                      f"OpenMP {cores} threads"}


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
    ap.add_argument("--npass", type=int, default=0,
                    help="reference passes before Newton for the plain solvers (0: each solver's default)")
    ap.add_argument("--lanes", type=int, default=0,
                    help="Newton solve kernel lanes per block (0: autotune)")
    ap.add_argument("--bps", type=int, default=0, help="Newton solve kernel blocks per SM (0: all that fit)")
    ap.add_argument("--zshared", type=int, default=0, help="with --lanes: right-hand side in shared memory")
    ap.add_argument("--solver", default="all", choices=["all", "ref5", "newton64", "mixed", "mlp"],
                    help="all: time the three solvers, headline = mixed")
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
    from reprobus_gb300.chem import SOLVER_NEWTON64, SOLVER_NEWTON_MIXED, SOLVER_REF5
    solver_ids = {"ref5": SOLVER_REF5, "newton64": SOLVER_NEWTON64, "mixed": SOLVER_NEWTON_MIXED,
                  "mlp": SOLVER_NEWTON_MIXED}
    run = list(solver_ids) if args.solver == "all" else [args.solver]
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
    a = dc.args()
    state = ("qj1", "hc", "vsed3d", "parth2osed", "parthno3sed", "surfarea", "sza3d")
    pristine = {f: dc[f].clone() for f in state}

    def restore():
        with torch.cuda.stream(stream):
            for f in state:
                dc[f].copy_(pristine[f])

    def step(stats=False):
        return h.step_dev(1, case.nlat, case.daynum, case.dt, *a, stats=stats)

    def npass_of(name):
        # the warm start's network is trained on the default 5-pass start
        if name == "mlp":
            return 5
        return args.npass if args.npass > 0 else 5

    results = {}
    clocks = Clocks(local)
    clocks.start()
    for name in run:
        h.set_solver(solver_ids[name], npass=npass_of(name), maxit=12, tol=1e-5)
        h.set_mlp(net if name == "mlp" else None)
        for _ in range(max(args.warmup, 3)):
            restore()
            step()
        restore()
        st = step(stats=True)  # launches per step, kernel time, solver statistics
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for e0, e1 in evs:
            restore()
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(sum(e0.elapsed_time(e1) for e0, e1 in evs))
        conv = case.ncells - st["fallbacks"]
        day_frac = float((dc["sza3d"][:case.ncells] <= 95.0).double().mean())
        results[name] = {"cells_per_s": whole_job_rate(case.ncells, world, args.steps, ms * 1e-3),
                         "ms_per_step": ms / args.steps, "kernel_ms": st["device_ms"],
                         "solve_ms": st["solve_ms"] if name != "ref5" else None,
                         "launches_per_step": st["kernel_launches"], "fallbacks": st["fallbacks"],
                         "mean_newton_iters": (st["newton_iters"] / conv) if name != "ref5" and conv else None,
                         "iters_per_cell": ((st["newton_iters"] + st["failed_iters"]) / case.ncells
                                            if name != "ref5" else None),
                         "warm_restarts": st["warm_restarts"] if name == "mlp" else None,
                         "day_frac": day_frac,
                         "max_newton_iters": st["max_newton_iters"] if name != "ref5" else None,
                         "solve_shape": None if name == "ref5" else
                         {"lanes_per_block": st["lanes_per_block"], "blocks_per_sm": st["blocks_per_sm"],
                          "z_shared": st["z_shared"]}}
    clk = clocks.stop()
    h.set_solver(solver_ids[headline], npass=npass_of(headline), maxit=12, tol=1e-5)
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
        n_e2e = max(3, args.steps)
        te = 0.0
        for _ in range(n_e2e):
            hrestore()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            hstep()
            torch.cuda.synchronize()
            te += time.perf_counter() - t0
        te = max_over_ranks(te / n_e2e)
        pl = case.nlon * case.nlat * case.niv * 8
        pb = case.nlon * case.nlat * case.nivbas * 8
        h2d = pb * 5 + pl * 43 + pb * 15
        d2h = pl * 43 + pb * 15 + pb * 4 + (case.nivbas - case.nivhau + 1) * case.nlon * case.nlat * 8
        e2e = {"value": whole_job_rate(ncell, world, 1, te), "unit": "cell-steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": te * 1e3}

    line = None
    if rank == 0:
        peak64 = fp64_peak_tflops(torch)
        hbm_peak = None
        try:
            hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        except Exception:
            hbm_peak = 6800.0
        flops_cell = OPS_PER_CELL
        ach_gbs = BYTES_PER_CELL * ncell / (kernel_ms * 1e-3) / 1e9
        roof = {"bound": "fp64", "unit": "TFLOP/s", "peak": round(peak64, 4),
                "peak_source": "cuBLAS DGEMM 4096^3 measured live in this run",
                "achieved": None, "frac": None, "traffic": None,
                "kernel_ms": round(kernel_ms, 4),
                "hbm": {"achieved": round(ach_gbs, 2), "peak": hbm_peak, "unit": "GB/s",
                        "frac": round(ach_gbs / hbm_peak, 5), "bytes_per_cell": BYTES_PER_CELL}}
        if headline == "ref5" and flops_cell:
            ach = flops_cell * ncell / (kernel_ms * 1e-3) / 1e12
            roof.update(achieved=round(ach, 4), frac=round(ach / peak64, 4), flops_per_cell=flops_cell,
                        flops_note="algorithmic ops of the reference scheme per cell-step (+-*/ and "
                                   "transcendentals counted once each; the peak counts an FMA as 2)")
        elif headline != "ref5":
            # dominant kernel: the persistent Newton solve kernel (k_nt_solve)
            ops = newton_ops()
            f = R["day_frac"]
            res = f * ops["res_day"] + (1 - f) * ops["res_night"]
            jac = f * ops["jac_day"] + (1 - f) * ops["jac_night"]
            fp64_it = res + ops["update"] + (0 if headline in ("mixed", "mlp") else jac + ops["factor"] + ops["rhs"])
            fp32_it = (jac + ops["factor"] + ops["rhs"]) if headline in ("mixed", "mlp") else 0
            iters = R["iters_per_cell"] * ncell
            sm = R["solve_ms"] * 1e-3
            ach = fp64_it * iters / sm / 1e12
            traffic = (SOLVE_DRAM_BYTES_PER_CELL_ITER * iters if headline in ("mixed", "mlp") else None)
            roof.update(kernel="k_nt_solve", kernel_ms=round(R["solve_ms"], 4), achieved=round(ach, 4),
                        traffic=traffic, traffic_note="DRAM bytes per launch: 899 B per cell-iteration from an "
                        "ncu capture of the 394,560-cell grid, times this launch's cell-iterations",
                        frac=round(ach / peak64, 4), fp64_ops_per_iteration=round(fp64_it, 1),
                        fp32_ops_per_iteration=round(fp32_it, 1), iterations_per_cell=round(R["iters_per_cell"], 3),
                        fp32_tflops=round(fp32_it * iters / sm / 1e12, 4),
                        flops_note="arithmetic operators of one Newton iteration counted in the generated "
                                   "source (an FMA counts 2), times the iterations the step ran, over the "
                                   "solve kernel's CUDA-event time; FP64 part (residual, update) against the "
                                   "live DGEMM peak")
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
                           "solver": {"ref5": "reference scheme, 5 fixed passes (drop-in)",
                                      "mlp": "Newton to the fixed point, FP32 Jacobian+LU, FP64 residual/update, "
                                             "learned warm start (BF16 MLP on tensor cores)",
                                      "newton64": "Newton to the fixed point of the reference map, FP64 Jacobian",
                                      "mixed": "Newton to the fixed point, FP32 Jacobian+LU, FP64 residual/update"}
                           [headline],
                           "timing": "each timed step starts from the same restored device state",
                           "cells": ncell, "l2": "inputs larger than L2 (1.2 GB resident state)",
                           "parallelism": f"replicas x{world}"},
                "gpu_launches": launches_per_step * args.steps,
                "solvers": results,
                "mixed_vs_fp64_newton": (results["mixed"]["cells_per_s"] / results["newton64"]["cells_per_s"]
                                         if "mixed" in results and "newton64" in results else None),
                "mlp_mixed_vs_fp64_newton": (results["mlp"]["cells_per_s"] / results["newton64"]["cells_per_s"]
                                             if "mlp" in results and "newton64" in results else None),
                "roofline": roof, "e2e": e2e, "cpu_baseline": cb, "clocks": clk, "columns": cols}
        print(json.dumps(line))
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
