"""The learned restart on the GPU: a cell whose Newton iteration from the
plain start misses the convergence test gets a second attempt from the
network's prediction for that plain start, and only a cell that misses again
falls back to the reference passes.

Properties checked against the same step without the network: every cell
that converged from the plain start keeps its answer bit for bit (the
network touches only the cells that missed: at most stats.warm_restarts of
them differ); each restarted cell is one the plain solver handed to its
fallback (warm_restarts equals the plain solver's fallback count); the
restarted cells that converge reach the fixed point (Oracle-C and the
reference map, as for the plain start); and fewer cells fall back."""
import numpy as np
import pytest

from oracle import accuracy, oracle
from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import SOLVER_NEWTON_MIXED

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-6
MAP_TOL = 1e-8


@pytest.fixture(scope="module")
def net(lib_built):
    from reprobus_gb300 import mlp, train_mlp
    # trained for the one-pass start, which leaves more cells to miss
    X, Y = train_mlp.make_training_set(12, 36, 12, seed0=500, log=lambda *a: None, npass=1)
    Xv, Yv = train_mlp.make_training_set(1, 36, 12, seed0=900, log=lambda *a: None, npass=1)
    n = mlp.Mlp(batch_cap=4096, seed=1)
    n.set_params(None, mlp.normalisation(X, Y))
    hist = mlp.train(n, X, Y, 3000, batch=4096, lr=1e-3)
    assert np.mean(hist[-50:]) < 0.5 * np.mean(hist[:10])
    tau = mlp.fit_thresholds(n, Xv, Yv)
    print(f"loss {np.mean(hist[:10]):.3f} -> {np.mean(hist[-50:]):.4f}; outputs on: {int(np.isfinite(tau).sum())}")
    yield n
    n.close()


@pytest.fixture(scope="module")
def case():
    return inputs.make_case("cfg0", seed=2, nlon=16, nivbas=94)


def _run(case, net, npass=5, maxit=12):
    from reprobus_gb300.resident import DeviceCase
    h = ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(SOLVER_NEWTON_MIXED, npass=npass, maxit=maxit)  # npass: the start the network was trained for
    if net is not None:
        h.set_mlp(net)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    out = dc.state_host()
    h.close()
    # the first step of a handle autotunes the solve kernel; its trial solves are not counted
    assert st["newton_iters"] + st["failed_iters"] <= st["ncells"] * maxit * (2 if net is not None else 1)
    return out, st


def _changed_cells(a, b, nb):
    """Cells (diag order) where any of the 57 unknowns differs bitwise."""
    d = (a["qj1"][:, :, :nb, :42] != b["qj1"][:, :, :nb, :42]).any(-1) | (
        a["hc"][:, :, :nb, :] != b["hc"][:, :, :nb, :]).any(-1)
    return d.transpose(2, 1, 0).reshape(-1)


def _check(case, plain, st0, learned, st1):
    assert st1["warm_start"] == 1 and st0["warm_start"] == 0
    # only the cells that missed are touched, and every one of them was restarted
    assert st1["warm_restarts"] == st0["fallbacks"]
    assert _changed_cells(plain, learned, case.nivbas).sum() <= st1["warm_restarts"]
    assert st1["fallbacks"] <= st0["fallbacks"]
    # the restarted cells that converged are the fixed point
    fp, stat, _ = oracle.step_fixed_point(case, tol=1e-12, maxiter=60, fuse=False)
    fell_back = oracle.map_residual(case, learned["qj1"], learned["hc"]) > MAP_TOL
    assert fell_back.sum() <= st1["fallbacks"]
    ok = (stat >= 0) & ~fell_back
    assert accuracy.cell_errors(learned, fp, case.nivbas)[ok].max() <= ERR_TOL
    it0 = (st0["newton_iters"] + st0["failed_iters"]) / case.ncells
    it1 = (st1["newton_iters"] + st1["failed_iters"]) / case.ncells
    print(f"iterations per cell {it0:.3f} -> {it1:.3f}; restarted {st1['warm_restarts']}, "
          f"fallbacks {st0['fallbacks']} -> {st1['fallbacks']}")


def test_learned_restart_of_a_network_trained_here(case, net):
    # a one-pass start and a cap of 4 iterations leave enough cells to restart
    plain, st0 = _run(case, None, npass=1, maxit=4)
    learned, st1 = _run(case, net, npass=1, maxit=4)
    assert st0["fallbacks"] >= 20
    _check(case, plain, st0, learned, st1)
    assert st1["fallbacks"] < st0["fallbacks"]


def test_committed_network_on_a_fresh_grid(case):
    """The network shipped in reprobus_gb300/data (trained by
    reprobus_gb300.train_mlp on 2e7 solver cells for the default 5-pass
    start) on a grid it has not seen, at the production settings and with a
    cap of 4 iterations (more cells to restart). What it gains on the full
    grid is held in tests/test_gpu_fullsize.py."""
    from reprobus_gb300 import mlp
    n = mlp.Mlp(batch_cap=128)
    n.load()
    for maxit in (12, 4):
        plain, st0 = _run(case, None, maxit=maxit)
        learned, st1 = _run(case, n, maxit=maxit)
        _check(case, plain, st0, learned, st1)
    assert st0["fallbacks"] >= 20 and st1["warm_restarts"] == st0["fallbacks"]
    n.close()
