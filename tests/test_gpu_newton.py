"""Newton solvers of the step equations on the GPU, against the oracle.

The reference iterates its pass map a fixed 5 times; the Newton solvers
return the fixed point of that map. Parity is checked two independent ways:
  * against Oracle-C (the oracle's own Newton on the reference pass map with
    a finite-difference Jacobian), on the cells where Oracle-C converges:
    relative error <= 1e-6 for species above 1e-20 mol/mol (the accuracy
    bound of the solver work), measured ~1e-10;
  * on every cell the solver does not hand to its fallback, the oracle's
    reference pass evaluated at the GPU answer returns it: max|G(x)-x|/
    max(|x|, 1e-20 hnm) <= 1e-8.
"""
import numpy as np
import pytest

from conftest import relerr
from oracle import oracle
from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import FUSE_CONSERV, SOLVER_NEWTON64, SOLVER_NEWTON_MIXED

pytestmark = pytest.mark.gpu

ERR_TOL = 1e-6
MAP_TOL = 1e-8


@pytest.fixture(scope="module")
def case():
    return inputs.make_case("cfg0", seed=2, nlon=16, nivbas=94)


@pytest.fixture(scope="module")
def fixed_point(case):
    return oracle.step_fixed_point(case, tol=1e-12, maxiter=60, fuse=False)


def _run(case, solver, flags=0, npass=1):
    from reprobus_gb300.resident import DeviceCase
    h = ChemStep.for_case(case, niter=5, flags=flags)
    h.set_solver(solver, npass=npass, maxit=12, tol=1e-10)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    out = dc.state_host()
    h.close()
    return out, st


def _species_err(got, ref, nb):
    q, r = got["qj1"][:, :, :nb, :42], ref["qj1"][:, :, :nb, :42]
    big = np.abs(r) > 1e-20
    e = np.where(big, relerr(q, r), 0.0)
    h, hr = got["hc"][:, :, :nb, :], ref["hc"][:, :, :nb, :]
    eh = np.where(np.abs(hr) > 1e-20, relerr(h, hr), 0.0)
    # per cell (diag layout: lon fastest, then lat, then level)
    ec = np.maximum(e.max(axis=-1), eh.max(axis=-1))
    return np.moveaxis(ec, 2, 0).reshape(-1)[..., None].ravel() if False else ec.transpose(2, 1, 0).reshape(-1)


@pytest.mark.parametrize("solver", [SOLVER_NEWTON64, SOLVER_NEWTON_MIXED])
def test_newton_matches_oracle_fixed_point(case, fixed_point, solver):
    fp, stat, _ = fixed_point
    got, st = _run(case, solver)
    assert st["solver"] == solver and st["ncells"] == case.ncells
    err = _species_err(got, fp, case.nivbas)
    # cells the solver handed to its fallback (the reference's passes) are off the
    # fixed point by construction: they are the ones the map residual flags
    fell_back = oracle.map_residual(case, got["qj1"], got["hc"]) > MAP_TOL
    assert fell_back.sum() <= st["fallbacks"]
    ok = (stat >= 0) & ~fell_back
    assert ok.mean() > 0.9
    assert err[ok].max() <= ERR_TOL, (err[ok].max(), int(np.argmax(np.where(ok, err, 0))))
    assert np.percentile(err[ok], 99) <= 1e-9
    # mean iterations of a converged cell, and few fallbacks
    assert st["fallbacks"] <= 0.01 * case.ncells
    assert 1 <= st["newton_iters"] / (case.ncells - st["fallbacks"]) <= 8


@pytest.mark.parametrize("solver", [SOLVER_NEWTON64, SOLVER_NEWTON_MIXED])
def test_newton_answer_is_a_fixed_point_of_the_reference_map(case, solver):
    got, st = _run(case, solver)
    mr = oracle.map_residual(case, got["qj1"], got["hc"])
    bad = mr > MAP_TOL
    # the only cells allowed off the fixed point are the solver's fallbacks
    assert bad.sum() <= st["fallbacks"], (bad.sum(), st["fallbacks"], np.sort(mr)[-5:])


def test_newton_polar_winter_and_fused_conservation():
    case = inputs.make_case("grid", seed=61, nlon=16, nlat=6, nivbas=94, daynum=355.5, polar_frac=0.5)
    for solver in (SOLVER_NEWTON64, SOLVER_NEWTON_MIXED):
        got, st = _run(case, solver)
        mr = oracle.map_residual(case, got["qj1"], got["hc"])
        assert (mr > MAP_TOL).sum() <= st["fallbacks"]
        fused, st2 = _run(case, solver, flags=FUSE_CONSERV)
        ref = {k: v.copy(order="F") for k, v in got.items()}
        oracle.conserv(case, ref["qj1"], ref["hc"])
        oracle.clamp(case, ref["qj1"])
        assert relerr(fused["qj1"], ref["qj1"]).max() < 1e-12


def test_mixed_and_fp64_newton_agree(case):
    a, _ = _run(case, SOLVER_NEWTON64)
    b, _ = _run(case, SOLVER_NEWTON_MIXED)
    e = _species_err(b, a, case.nivbas)
    assert np.percentile(e, 99.9) <= 1e-9


@pytest.mark.parametrize("lanes", [128, 64])
def test_mixed_solve_kernel_shapes_agree_with_the_oracle(case, fixed_point, lanes):
    """Compiled shapes of the mixed solve kernel, forced (the autotuner's
    candidates): 128 and 64 lanes per block."""
    from reprobus_gb300.resident import DeviceCase
    fp, stat, _ = fixed_point
    h = ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(SOLVER_NEWTON_MIXED, npass=1, maxit=12, tol=1e-10)
    h.set_tuning(lanes, 0, 0)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    got = dc.state_host()
    h.close()
    assert st["lanes_per_block"] == lanes
    fell_back = oracle.map_residual(case, got["qj1"], got["hc"]) > MAP_TOL
    assert fell_back.sum() <= st["fallbacks"] <= 0.01 * case.ncells
    ok = (stat >= 0) & ~fell_back
    assert _species_err(got, fp, case.nivbas)[ok].max() <= ERR_TOL


@pytest.mark.parametrize("solver,lanes,form", [(SOLVER_NEWTON_MIXED, 256, 2), (SOLVER_NEWTON_MIXED, 128, 2),
                                               (SOLVER_NEWTON64, 128, 2), (SOLVER_NEWTON64, 64, 2),
                                               (SOLVER_NEWTON_MIXED, 128, 3), (SOLVER_NEWTON_MIXED, 64, 3),
                                               (SOLVER_NEWTON64, 64, 3), (SOLVER_NEWTON64, 32, 3),
                                               (SOLVER_NEWTON_MIXED, 128, 4), (SOLVER_NEWTON_MIXED, 64, 4),
                                               (SOLVER_NEWTON64, 64, 4), (SOLVER_NEWTON_MIXED, 32, 5),
                                               (SOLVER_NEWTON_MIXED, 64, 5), (SOLVER_NEWTON_MIXED, 32, 6),
                                               (SOLVER_NEWTON64, 32, 5), (SOLVER_NEWTON64, 32, 6)])
def test_two_group_solve_kernel_agrees_with_the_oracle(case, fixed_point, solver, lanes, form):
    """The solve kernels with two kinds of warps, forced, for both matrix
    precisions: two warp groups taking turns on one set of matrix slots
    (zshared 2), a matrix lane plus a residual lane per cell (zshared 3), the
    one-group kernel with its warps in lock-step (zshared 4), and 2 or 4
    warps per cell sharing the rows of the Jacobian and the residual (zshared
    5, 6; lanes = cells per block). Same accuracy bound and fixed-point
    property as the one-group kernel."""
    from reprobus_gb300.resident import DeviceCase
    fp, stat, _ = fixed_point
    h = ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(solver, npass=1, maxit=12, tol=1e-10)
    h.set_tuning(lanes, 0, form)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    got = dc.state_host()
    h.close()
    assert st["lanes_per_block"] == lanes and st["z_shared"] == form
    fell_back = oracle.map_residual(case, got["qj1"], got["hc"]) > MAP_TOL
    assert fell_back.sum() <= st["fallbacks"] <= 0.01 * case.ncells
    ok = (stat >= 0) & ~fell_back
    assert _species_err(got, fp, case.nivbas)[ok].max() <= ERR_TOL
