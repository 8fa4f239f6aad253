"""Parity of the CUDA chemistry step (through the C-ABI) with the CPU oracle.

Tolerances (FP64 throughout; the GPU uses fused multiply-add and CUDA's libm,
the oracle IEEE operations without contraction and glibc's libm, so single
operations agree to about one ulp):
  rate stage: 99 rate constants, 41 J, sza, hnm, O3 column,
              het1-4,6,8, vsed, surfarea, partitions         rel 1e-12
  het5, het7: the reference evaluates 1/tanh(x) - 1/x with
              x = rmean/l << 1 (F:3570-3571, F:3611-3612),
              whose relative rounding error is ~eps/x^2       rel 2e-5
  parthno3:   ternary-aerosol cubic (F:3015-3047) with
              cancelling coefficients                         rel 1e-7
  full step, 5 passes: qj1 and hc                            max rel 1e-7,
              (hno3_gas = ck5*parthno3/hnm inherits the       99.9th pct 1e-10
              parthno3 error; every other slot stays ~1e-9)
              sza3d, vsed3d, parth2osed, parthno3sed,
              surfarea                                        rel 1e-12
"""
import numpy as np
import pytest

from conftest import relerr
from oracle import oracle
from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import CHECK_FINITE, FUSE_CONSERV
from reprobus_gb300.species import DIAG_COUNT, DIAG_NAMES

pytestmark = pytest.mark.gpu

RATE_TOL = 1e-12
RATE_TOL_SPECIAL = {"het5": 2e-5, "het7": 2e-5, "parthno3": 1e-7}
STEP_TOL = 1e-7
STEP_P999 = 1e-10
OUT_TOL = 1e-12
STATE = ("qj1", "hc")
OUTS = ("sza3d", "vsed3d", "parth2osed", "parthno3sed", "surfarea")
FIELDS = STATE + OUTS


@pytest.fixture(scope="module")
def torch():
    import torch as T
    assert T.cuda.is_available(), "GPU tests need CUDA"
    return T


def _run_gpu(case, niter=5, flags=FUSE_CONSERV, ilat0=1, ilat1=None):
    from reprobus_gb300.resident import DeviceCase
    ilat1 = case.nlat if ilat1 is None else ilat1
    h = ChemStep.for_case(case, niter=niter, flags=flags)
    dc = DeviceCase(case)
    st = h.step_dev(ilat0, ilat1, case.daynum, case.dt, *dc.args(), stats=True)
    out = dc.state_host()
    h.close()
    return out, st


def _compare(got, ref, tol=STEP_TOL, p999=STEP_P999, out_tol=OUT_TOL, floor=1e-300):
    worst = {}
    for f in FIELDS:
        assert np.all(np.isfinite(got[f]) == np.isfinite(ref[f])), f"{f}: finiteness differs"
        e = relerr(got[f], ref[f], floor)
        worst[f] = (float(np.nanmax(e)), float(np.nanpercentile(e, 99.9))) if e.size else (0.0, 0.0)
    bad = {f: worst[f] for f in STATE if not (worst[f][0] <= tol and worst[f][1] <= p999)}
    bad.update({f: worst[f] for f in OUTS if not worst[f][0] <= out_tol})
    assert not bad, f"(max, p99.9) rel err out of tolerance: {bad} (all: {worst})"
    return worst


@pytest.mark.parametrize("nivbas", [94, 137])
def test_rate_stage_matches_oracle(torch, nivbas):
    from reprobus_gb300.resident import DeviceCase
    case = inputs.make_case("cfg0", seed=21, nlon=32, nivbas=nivbas)
    _, dref, _ = oracle.step(case, niter=1, fuse=False, diag=True)
    h = ChemStep.for_case(case)
    dc = DeviceCase(case)
    diag = torch.zeros(DIAG_COUNT * case.ncells, dtype=torch.float64, device="cuda")
    h.rates_dev(1, case.nlat, case.daynum, dc["alt"], dc["trajlon"], dc["trajlat"], dc["trajpre"], dc["trajtem"],
                case.irapp, dc["qj1"], dc["hc"], diag)
    d = diag.cpu().numpy().reshape(DIAG_COUNT, case.ncells)
    h.close()
    errs = {DIAG_NAMES[i]: float(relerr(d[i], dref[i]).max()) for i in range(DIAG_COUNT)}
    bad = {k: v for k, v in errs.items() if not v <= RATE_TOL_SPECIAL.get(k, RATE_TOL)}
    assert not bad, bad


TROE_RATES = ("a1", "b12", "b22", "b23", "c4", "d31", "d36", "d60", "e13")  # :930-1303, the 9 falloff terms


def test_troe_rates_over_a_temperature_and_density_sweep(torch):
    """The nine Troe falloff rate constants, which the rate stage evaluates as
    k = x kinf / (kinf + x) with log10(x / kinf) from logarithms, against the
    reference's direct formula (the oracle) over T = 150..330 K (one value per
    column) and every level's air density from the top of the L137 grid to
    the surface."""
    from reprobus_gb300.resident import DeviceCase
    from reprobus_gb300.species import DIAG_RATE
    case = inputs.make_case("cfg0", seed=22, nlon=64, nivbas=137)
    T = np.linspace(150.0, 330.0, case.nlon)
    case.trajtem[:, :, :, :] = T[:, None, None, None]
    _, dref, _ = oracle.step(case, niter=1, fuse=False, diag=True)
    h = ChemStep.for_case(case)
    dc = DeviceCase(case)
    diag = torch.zeros(DIAG_COUNT * case.ncells, dtype=torch.float64, device="cuda")
    h.rates_dev(1, case.nlat, case.daynum, dc["alt"], dc["trajlon"], dc["trajlat"], dc["trajpre"], dc["trajtem"],
                case.irapp, dc["qj1"], dc["hc"], diag)
    d = diag.cpu().numpy().reshape(DIAG_COUNT, case.ncells)
    h.close()
    worst = {k: float(relerr(d[DIAG_NAMES.index(k)], dref[DIAG_NAMES.index(k)]).max()) for k in TROE_RATES}
    assert all(DIAG_NAMES.index(k) >= DIAG_RATE for k in TROE_RATES)
    assert max(worst.values()) <= 1e-13, worst


@pytest.mark.parametrize("nivbas,seed", [(94, 31), (137, 32)])
def test_step_matches_oracle(torch, nivbas, seed):
    case = inputs.make_case("cfg0", seed=seed, nlon=64, nivbas=nivbas)
    ref, _, _ = oracle.step(case, niter=5, fuse=True)
    got, st = _run_gpu(case)
    assert st["ncells"] == case.ncells
    _compare(got, ref)


def test_step_unfused_matches_oracle(torch):
    case = inputs.make_case("cfg0", seed=33, nlon=32, nivbas=94)
    ref, _, _ = oracle.step(case, niter=5, fuse=False)
    got, st = _run_gpu(case, flags=0)
    _compare(got, ref)
    assert st["kernel_launches"] == 3  # columns, rate stage, passes


def test_polar_winter_cells(torch):
    # cold polar-night parcels: NAT/ice, ternary aerosol, night chemistry
    case = inputs.make_case("grid", seed=34, nlon=16, nlat=6, nivbas=94, daynum=355.5, polar_frac=0.5)
    ref, dref, _ = oracle.step(case, niter=5, fuse=True, diag=True)
    assert dref[DIAG_NAMES.index("vsed")].max() > 0, "no PSC cells in the workload"
    got, _ = _run_gpu(case)
    _compare(got, ref)


def test_dt_zero_is_exact(torch):
    case = inputs.make_case("cfg0", seed=35, nlon=16, nivbas=94, dt=0.0)
    ref, _, _ = oracle.step(case, niter=5, fuse=False)
    got, _ = _run_gpu(case, flags=0)
    assert np.array_equal(got["qj1"][..., :42], ref["qj1"][..., :42])


def test_host_entry_equals_device_entry(torch):
    case = inputs.make_case("cfg0", seed=36, nlon=16, nivbas=94)
    dev, _ = _run_gpu(case)
    h = ChemStep.for_case(case)
    st = case.state_copy()
    h.step(1, case.nlat, case.daynum, case.dt, case.alt, case.trajlon, case.trajlat, case.trajpre, case.trajtem,
           case.irapp, st["qj1"], st["hc"], st["vsed3d"], st["parth2osed"], st["parthno3sed"], st["surfarea"],
           st["sza3d"])
    h.close()
    for f in FIELDS:
        assert np.array_equal(st[f], dev[f]), f


def test_row_subset_and_other_rows_untouched(torch):
    case = inputs.make_case("grid", seed=37, nlon=12, nlat=7, nivbas=94)
    ref, _, _ = oracle.step(case, niter=5, fuse=True, ilat0=3, ilat1=5)
    got, st = _run_gpu(case, ilat0=3, ilat1=5)
    assert st["ncells"] == 12 * 3 * 94
    _compare(got, ref)
    for j in (0, 1, 5, 6):
        assert np.array_equal(got["qj1"][:, j], case.qj1[:, j])


def test_host_entry_row_subset(torch):
    case = inputs.make_case("grid", seed=38, nlon=10, nlat=5, nivbas=94)
    ref, _, _ = oracle.step(case, niter=5, fuse=True, ilat0=2, ilat1=3)
    h = ChemStep.for_case(case)
    st = case.state_copy()
    h.step(2, 3, case.daynum, case.dt, case.alt, case.trajlon, case.trajlat, case.trajpre, case.trajtem,
           case.irapp, st["qj1"], st["hc"], st["vsed3d"], st["parth2osed"], st["parthno3sed"], st["surfarea"],
           st["sza3d"])
    h.close()
    _compare(st, ref)


def test_irapp_slice(torch):
    case = inputs.make_case("cfg0", seed=39, nlon=16, nivbas=94, nrappmax=3, irapp=2)
    ref, _, _ = oracle.step(case, niter=5, fuse=True)
    got, _ = _run_gpu(case)
    _compare(got, ref)


def test_conserv_entry_matches_oracle(torch):
    from reprobus_gb300.resident import DeviceCase
    case = inputs.make_case("cfg0", seed=40, nlon=16, nivbas=94)
    st, _, _ = oracle.step(case, niter=5, fuse=False)
    q, hc = st["qj1"].copy(order="F"), st["hc"].copy(order="F")
    oracle.conserv(case, q, hc)
    oracle.clamp(case, q)
    dc = DeviceCase(case, state=st)
    h = ChemStep.for_case(case)
    h.conserv_dev(1, case.nlat, dc["qj1"], dc["hc"])
    got = dc.state_host()
    h.close()
    assert relerr(got["qj1"], q).max() < 1e-14
    assert relerr(got["hc"], hc).max() < 1e-14


def test_check_finite_and_stream(torch):
    from reprobus_gb300.resident import DeviceCase
    case = inputs.make_case("cfg0", seed=41, nlon=16, nivbas=94)
    ref, _, _ = oracle.step(case, niter=5, fuse=True)
    h = ChemStep.for_case(case, flags=FUSE_CONSERV | CHECK_FINITE)
    s = torch.cuda.Stream()
    h.set_stream(s)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    assert st["nonfinite"] == 0
    got = dc.state_host()
    h.close()
    _compare(got, ref)


def test_reference_shaped_interface(torch):
    # chem3d(ilat, ...) per row, then conserv, as the time loop calls them
    import reprobus_gb300 as R
    case = inputs.make_case("grid", seed=42, nlon=8, nlat=3, nivbas=94, nrappmax=2, irapp=1)
    ref, _, _ = oracle.step(case, niter=5, fuse=True)
    R.init(case.ajl, case.o3up, case.nlon, case.nlat, case.niv, 94, 14, case.nrappmax)
    st = case.state_copy()
    for ilat in range(1, case.nlat + 1):
        R.chem3d(ilat, case.daynum, case.dt, case.alt, case.trajlon, case.trajlat, case.trajpre, case.trajtem,
                 case.irapp, st["qj1"], st["hc"], st["vsed3d"], st["parth2osed"], st["parthno3sed"],
                 st["surfarea"], st["sza3d"])
    R.conserv(st["qj1"], st["hc"])
    _compare(st, ref)


@pytest.mark.parametrize("solver", ["ref5", "mixed", "fp64", "mlp"])
@pytest.mark.parametrize("chunks", ["4", "3"])
def test_host_entry_in_row_chunks_equals_device_entry(torch, solver, chunks, monkeypatch):
    """The host-array entry point pipelines calls of 32 rows or more in row
    chunks (copies of one chunk overlapping the integration of another); once
    a Newton solver is tuned, its step runs in phases (rate stage and start
    chunk by chunk, one solve over all rows, write-back chunk by chunk). Both
    the first (chunk by chunk) and the second (phased) host step are bit for
    bit the device-array entry point's on the same grid, and so are the
    solver statistics."""
    from reprobus_gb300 import mlp as mlpmod
    from reprobus_gb300.chem import SOLVER_NEWTON64, SOLVER_NEWTON_MIXED
    from reprobus_gb300.resident import DeviceCase
    monkeypatch.setenv("REPROBUS_HOST_CHUNKS", chunks)
    case = inputs.make_case("grid", seed=41, nlon=12, nlat=40, nivbas=94)
    net = None
    if solver == "mlp":
        net = mlpmod.Mlp(batch_cap=128, seed=0)
        net.load()
    outs, stats = [], []
    for host in (True, False):
        h = ChemStep.for_case(case, niter=5, flags=FUSE_CONSERV)
        if solver in ("mixed", "mlp"):
            # mlp: a cap of 4 iterations, so that cells of both work queues take the learned restart
            h.set_solver(SOLVER_NEWTON_MIXED, maxit=4 if solver == "mlp" else 12)
            h.set_tuning(64, 1, 0)
        elif solver == "fp64":
            h.set_solver(SOLVER_NEWTON64)
            h.set_tuning(32, 1, 0)
        if net is not None:
            h.set_mlp(net)
        if host:
            for _ in range(2):  # the second step takes the phased path
                st = case.state_copy()
                sd = h.step(1, case.nlat, case.daynum, case.dt, case.alt, case.trajlon, case.trajlat, case.trajpre,
                            case.trajtem, case.irapp, st["qj1"], st["hc"], st["vsed3d"], st["parth2osed"],
                            st["parthno3sed"], st["surfarea"], st["sza3d"])
                outs.append(st)
                stats.append(sd)
        else:
            dc = DeviceCase(case)
            stats.append(h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True))
            outs.append(dc.state_host())
        h.close()
    for k in (0, 1):
        for f in FIELDS:
            assert np.array_equal(outs[k][f], outs[2][f]), (k, f)
        for key in ("ncells", "newton_iters", "fallbacks", "max_newton_iters", "warm_restarts", "nonfinite"):
            assert stats[k][key] == stats[2][key], (k, key)
    if solver == "mlp":
        assert stats[2]["warm_restarts"] > 0
