"""Per-species error of the GPU Newton solvers against the FP64 oracle on a
polar-winter mix (the distributions of the 30 %-polar-winter workload: 30 % of
the columns in polar night, T 183-195 K, active ClOx), at the solvers'
production settings (5 start passes, step tolerance 1e-4, maxit 16), for the
FP64 solver, the mixed-precision solver and the mixed solver with the
committed network's learned restart. Written as a table when
REPROBUS_SPECIES_REPORT names a file.

The oracle is Oracle-C: the reference pass map's fixed point by the oracle's
own finite-difference Newton, restarted from earlier pass states (and
finally by pseudo-transient continuation) where it does not converge from
the reference's 5-pass state. It must converge on at least 99.9 % of the
cells, and on those the GPU answer must lie within 1e-6 of it for every
species above 1e-20 mol/mol. On every remaining cell the solver did not hand
to its fallback, Oracle-C's Newton started from the GPU answer must converge
to an exact FP64 fixed point within 1e-6 of that answer."""
import json
import os

import numpy as np
import pytest

from oracle import accuracy, oracle
from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import SOLVER_NEWTON64, SOLVER_NEWTON_MIXED

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-6
MAP_TOL = 1e-8
COVER = 0.999


@pytest.fixture(scope="module")
def case():
    return inputs.make_case("grid", seed=77, nlon=36, nlat=8, daynum=355.5, polar_frac=0.3)


@pytest.fixture(scope="module")
def reference(case):
    return accuracy.Reference(case, fuse=False)


def _run(case, solver, net=None):
    from reprobus_gb300.resident import DeviceCase
    h = ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(solver, maxit=16)  # the default start and tolerance
    if net is not None:
        h.set_mlp(net)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    out = dc.state_host()
    h.close()
    return out, st


@pytest.mark.parametrize("arm", ["mixed", "fp64", "mlp"])
def test_species_errors_polar_winter(case, reference, arm):
    net = None
    if arm == "mlp":
        from reprobus_gb300 import mlp
        net = mlp.Mlp(batch_cap=128)
        net.load()
    solver = SOLVER_NEWTON64 if arm == "fp64" else SOLVER_NEWTON_MIXED
    got, st = _run(case, solver, net)
    if net is not None:
        net.close()
    fell_back = oracle.map_residual(case, got["qj1"], got["hc"]) > MAP_TOL
    conv = reference.converged
    ok = conv & ~fell_back
    rows = accuracy.species_errors(got, reference.fp, case.nivbas, ok)
    worst = max(r[1] for r in rows)
    # the cells Oracle-C did not converge on: Newton from the GPU answer
    rest = ~conv & ~fell_back
    polished, pstat, _ = oracle.newton_from(case, got["qj1"], got["hc"])
    dist = accuracy.cell_errors(got, polished, case.nivbas)
    report = {"solver": arm, "cells": int(case.ncells), "compared": int(ok.sum()),
              "fallbacks": int(st["fallbacks"]), "oracle_unconverged": int((~conv).sum()),
              "oracle_stages": np.bincount(reference.stage, minlength=7).tolist(),
              "checked_from_gpu_answer": int(rest.sum()),
              "max_dist_to_fixed_point_from_gpu_answer": float(dist[rest].max()) if rest.any() else None,
              "iters_per_cell": (st["newton_iters"] + st["failed_iters"]) / case.ncells,
              "max_newton_iters": st["max_newton_iters"], "warm_restarts": st["warm_restarts"],
              "species": {n: {"max": m, "p99": p, "n": k} for n, m, p, k in rows}}
    path = os.environ.get("REPROBUS_SPECIES_REPORT")
    if path:
        with open(path + f".{arm}.json", "w") as f:
            json.dump(report, f, indent=1)
    assert fell_back.sum() <= st["fallbacks"] <= 0.001 * case.ncells
    assert conv.mean() >= COVER, report["oracle_stages"]
    assert ok.mean() >= COVER
    assert worst <= ERR_TOL, sorted(rows, key=lambda r: -r[1])[:5]
    if rest.any():
        assert (pstat[rest] >= 0).all()
        assert dist[rest].max() <= ERR_TOL
