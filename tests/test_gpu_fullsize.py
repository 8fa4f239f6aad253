"""Checks at the benchmark's full size: the 2 x 2 degree L137 grid of
2,244,060 cells (cfg1), through properties that do not depend on the size.

* REF5 (the reference scheme) over the whole grid on the GPU equals the CPU
  oracle on latitude rows from pole to pole, at the tolerances of
  test_gpu_parity.py.
* The mixed-precision Newton answer is a fixed point of the reference's pass
  map in every cell the solver did not hand to its fallback (the oracle's
  pass evaluated at the GPU answer over the whole grid), with every value
  finite.
* With the conservation fused, the answer equals the oracle's conserv and
  clamps applied to the unfused answer, over the whole grid.
"""
import numpy as np
import pytest

from conftest import relerr
from oracle import oracle
from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import FUSE_CONSERV, SOLVER_NEWTON_MIXED

from test_gpu_parity import FIELDS, _compare

pytestmark = pytest.mark.gpu
MAP_TOL = 1e-8


@pytest.fixture(scope="module")
def torch():
    import torch as T
    assert T.cuda.is_available(), "GPU tests need CUDA"
    return T


@pytest.fixture(scope="module")
def case():
    return inputs.make_case("cfg1", seed=1234)


def _gpu(case, solver=None, flags=FUSE_CONSERV):
    from reprobus_gb300.resident import DeviceCase
    h = ChemStep.for_case(case, niter=5, flags=flags)
    if solver is not None:
        h.set_solver(solver)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    out = dc.state_host()
    h.close()
    return out, st


def test_ref5_full_grid_matches_oracle_on_rows(torch, case):
    got, st = _gpu(case)
    assert st["ncells"] == case.ncells == 2244060
    for f in FIELDS:
        assert np.all(np.isfinite(got[f])), f
    for r in (1, 23, 46, 70, 91):  # pole, mid-latitude, equator, mid-latitude, pole
        ref, _, _ = oracle.step(case, niter=5, fuse=True, ilat0=r, ilat1=r)
        _compare({f: got[f][:, r - 1] for f in FIELDS}, {f: ref[f][:, r - 1] for f in FIELDS})


def test_mixed_newton_full_grid_is_a_fixed_point_and_conserves(torch, case):
    got, st = _gpu(case, SOLVER_NEWTON_MIXED, flags=0)
    for f in ("qj1", "hc"):
        assert np.all(np.isfinite(got[f])), f
    res = oracle.map_residual(case, got["qj1"], got["hc"])
    fell_back = res > MAP_TOL
    assert fell_back.sum() <= st["fallbacks"] <= 1e-3 * case.ncells
    fused, st2 = _gpu(case, SOLVER_NEWTON_MIXED, flags=FUSE_CONSERV)
    q, hc = got["qj1"].copy(order="F"), got["hc"].copy(order="F")
    oracle.conserv(case, q, hc)
    oracle.clamp(case, q)
    assert relerr(fused["qj1"], q).max() < 1e-12
    assert relerr(fused["hc"], hc).max() < 1e-12


def test_learned_restart_halves_the_fallbacks(torch, case):
    """What the committed network gains on the full grid: cells whose Newton
    iteration from the plain start fails within the iteration cap would fall
    back to the reference's 5 passes (their answer is then the reference
    scheme's, not the fixed point); the learned restart gives them a second
    attempt from the network's prediction, and fewer fall back. Every other
    cell keeps its answer bit for bit; bench.py reports the time."""
    from reprobus_gb300 import mlp
    from reprobus_gb300.resident import DeviceCase
    net = mlp.Mlp(batch_cap=128)
    net.load()
    out = {}
    for name, n in (("plain", None), ("learned", net)):
        h = ChemStep.for_case(case, niter=5, flags=0)
        h.set_solver(SOLVER_NEWTON_MIXED)  # production settings: 5 passes, tol 1e-4, maxit 12
        h.set_mlp(n)
        dc = DeviceCase(case)
        st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
        out[name] = (dc.state_host(), st)
        h.close()
    net.close()
    (a, sa), (b, sb) = out["plain"], out["learned"]
    print(f"fallbacks: plain start {sa['fallbacks']}, with the learned restart {sb['fallbacks']}; iterations "
          f"per cell {(sa['newton_iters'] + sa['failed_iters']) / case.ncells:.4f} -> "
          f"{(sb['newton_iters'] + sb['failed_iters']) / case.ncells:.4f}; restarts {sb['warm_restarts']}")
    assert sa["fallbacks"] >= 100  # enough cells for the comparison to mean something
    assert sb["warm_restarts"] == sa["fallbacks"]
    assert sb["fallbacks"] <= 0.75 * sa["fallbacks"]
    from oracle import accuracy
    both = (oracle.map_residual(case, a["qj1"], a["hc"]) <= MAP_TOL) & (
        oracle.map_residual(case, b["qj1"], b["hc"]) <= MAP_TOL)
    assert both.mean() > 0.999
    assert accuracy.cell_errors(b, a, case.nivbas)[both].max() <= 1e-6
