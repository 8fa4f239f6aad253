"""Fault handling through the C-ABI, in forms that fault, trap or hang no GPU.

Poisoned host inputs (a NaN species, a negative temperature, HCl = 0, a
photolysis table whose BrCl rates are 0) make the reference itself divide by
zero or propagate NaN (src/reprobus_l137_20230723.f:1525-1526 divides by
J_BrCl, :3166-3167 by the HCl partial pressure; the oracle gives non-finite
values for each); with REPROBUS_CHECK_FINITE the call must return
REPROBUS_ERR_NONFINITE, count the values, finish, and leave the handle usable
for the next clean step. None of these inputs reaches an index computation:
the photolysis lookup takes its indices from the altitude, the zenith angle
(NaN selects the last node) and an O3 ratio clamped by fmin/fmax.

The tensor-core inference kernel's bounded waits: with a wait limit of 0 the
first wait on a weight copy gives up while the copy is in flight; the kernel
must wait for that copy with its default limit, release its tensor memory and
report REPROBUS_ERR_TIMEOUT, and the same network must then give the
reference output again. In a step, the learned restart's cells then start
from the plain start again and the step reports the timeout."""
import copy

import numpy as np
import pytest

from oracle import oracle
from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import (CHECK_FINITE, FUSE_CONSERV, SOLVER_NEWTON_MIXED, SOLVER_REF5,
                                 ReprobusError)
from reprobus_gb300.species import LONG, PHOT

pytestmark = pytest.mark.gpu

ERR_NONFINITE, ERR_TIMEOUT = 3, 5


@pytest.fixture(scope="module")
def case():
    return inputs.make_case("cfg0", seed=5, nlon=8, nivbas=94)


def _poisoned(case, kind):
    c = copy.deepcopy(case)
    if kind == "nan_species":
        c.qj1[3, 0, 20, LONG.index("ch4")] = np.nan
    elif kind == "negative_T":
        c.trajtem[5, 0, 30, c.irapp - 1] = -200.0
    elif kind == "hcl_zero":
        c.qj1[:, :, :, LONG.index("hcl")] = 0.0
    elif kind == "jbrcl_zero":
        c.ajl[PHOT.index("brcl")] = 0.0
    return c


def _host_step(h, c):
    st = c.state_copy()
    return h.step(1, c.nlat, c.daynum, c.dt, c.alt, c.trajlon, c.trajlat, c.trajpre, c.trajtem, c.irapp,
                  st["qj1"], st["hc"], st["vsed3d"], st["parth2osed"], st["parthno3sed"], st["surfarea"],
                  st["sza3d"]), st


@pytest.mark.parametrize("kind", ["nan_species", "negative_T", "hcl_zero", "jbrcl_zero"])
@pytest.mark.parametrize("solver", [SOLVER_REF5, SOLVER_NEWTON_MIXED])
def test_poisoned_input_is_reported_and_the_handle_stays_usable(case, kind, solver):
    bad = _poisoned(case, kind)
    ref_bad, _, _ = oracle.step(bad, niter=5, fuse=True)
    assert not all(np.isfinite(ref_bad[f]).all() for f in ("qj1", "hc"))  # the reference's own behaviour
    # the photolysis table is a handle constant: poison it in the handle
    h = ChemStep.for_case(bad, niter=5, flags=FUSE_CONSERV | CHECK_FINITE)
    h.set_solver(solver)
    with pytest.raises(ReprobusError) as ei:
        _host_step(h, bad)
    assert ei.value.code == ERR_NONFINITE, str(ei.value)
    h.close()
    # a handle that saw a poisoned step integrates the next clean one correctly
    h = ChemStep.for_case(case, niter=5, flags=FUSE_CONSERV | CHECK_FINITE)
    h.set_solver(solver)
    if kind != "jbrcl_zero":
        with pytest.raises(ReprobusError):
            _host_step(h, bad)
    st, got = _host_step(h, case)
    assert st["nonfinite"] == 0
    h.close()
    if solver == SOLVER_REF5:
        ref, _, _ = oracle.step(case, niter=5, fuse=True)
        for f in ("qj1", "hc"):
            e = np.abs(got[f] - ref[f]) / np.maximum(np.abs(ref[f]), 1e-300)
            assert e.max() < 1e-7, (f, e.max())


def test_inference_wait_gives_up_and_the_network_stays_usable():
    import torch
    from reprobus_gb300 import mlp
    net = mlp.Mlp(batch_cap=128)
    net.load()
    rng = np.random.default_rng(3)
    X = torch.tensor(rng.normal(size=(1000, 64)).astype(np.float32) + 1.0, device="cuda")
    Y0 = torch.zeros(1000, 64, device="cuda")
    Y1 = torch.full((1000, 64), float("nan"), device="cuda")
    net.forward(X, Y0)
    torch.cuda.synchronize()
    net.set_wait_limit(0)  # the first wait gives up with the weight copy in flight
    with pytest.raises(ReprobusError) as ei:
        net.forward(X, Y1)
    assert ei.value.code == ERR_TIMEOUT, str(ei.value)
    net.set_wait_limit(-1)
    net.forward(X, Y1)
    torch.cuda.synchronize()
    assert torch.equal(Y0, Y1)
    net.close()


def test_learned_restart_reports_the_inference_timeout(case):
    from reprobus_gb300 import mlp
    from reprobus_gb300.resident import DeviceCase
    net = mlp.Mlp(batch_cap=128)
    net.load()
    h = ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(SOLVER_NEWTON_MIXED, maxit=2)  # many cells miss: the restart's inference runs
    h.set_mlp(net)
    dc = DeviceCase(case)
    net.set_wait_limit(0)
    with pytest.raises(ReprobusError) as ei:
        h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    assert ei.value.code == ERR_TIMEOUT, str(ei.value)
    net.set_wait_limit(-1)
    h.set_solver(SOLVER_NEWTON_MIXED)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    got = dc.state_host()
    assert st["warm_start"] == 1
    fp, stat, _ = oracle.step_fixed_point(case, tol=1e-12, maxiter=60, fuse=False)
    from oracle import accuracy
    e = accuracy.cell_errors(got, fp, case.nivbas)
    ok = (stat >= 0) & (oracle.map_residual(case, got["qj1"], got["hc"]) <= 1e-8)
    assert ok.mean() > 0.99 and e[ok].max() <= 1e-6
    h.close()
    net.close()
