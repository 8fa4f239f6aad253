"""Parity of the CUDA chemistry step (through the C-ABI) with the CPU oracle.

Tolerances (FP64 throughout; the GPU uses fused multiply-add and CUDA's libm,
the oracle IEEE operations without contraction and glibc's libm, so results
agree to a few ulp per operation, amplified by the fixed-point passes):
  rate stage (k, J, het, partitions, vsed, surfarea, sza):  rel 1e-12
  full step, 5 passes (qj1, hc, outputs):                   rel 1e-9
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
STEP_TOL = 1e-9
FIELDS = ("qj1", "hc", "sza3d", "vsed3d", "parth2osed", "parthno3sed", "surfarea")


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


def _compare(got, ref, tol, fields=FIELDS, floor=1e-300):
    worst = {}
    for f in fields:
        e = relerr(got[f], ref[f], floor)
        worst[f] = float(np.nanmax(e)) if e.size else 0.0
        assert np.all(np.isfinite(got[f]) == np.isfinite(ref[f])), f"{f}: finiteness differs"
    bad = {f: v for f, v in worst.items() if not v <= tol}
    assert not bad, f"rel err above {tol}: {bad} (all: {worst})"
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
    bad = {k: v for k, v in errs.items() if not v <= RATE_TOL}
    assert not bad, bad


@pytest.mark.parametrize("nivbas,seed", [(94, 31), (137, 32)])
def test_step_matches_oracle(torch, nivbas, seed):
    case = inputs.make_case("cfg0", seed=seed, nlon=64, nivbas=nivbas)
    ref, _, _ = oracle.step(case, niter=5, fuse=True)
    got, st = _run_gpu(case)
    assert st["ncells"] == case.ncells
    _compare(got, ref, STEP_TOL)


def test_step_unfused_matches_oracle(torch):
    case = inputs.make_case("cfg0", seed=33, nlon=32, nivbas=94)
    ref, _, _ = oracle.step(case, niter=5, fuse=False)
    got, st = _run_gpu(case, flags=0)
    _compare(got, ref, STEP_TOL)
    assert st["kernel_launches"] == 2


def test_polar_winter_cells(torch):
    # cold polar-night parcels: NAT/ice, ternary aerosol, night chemistry
    case = inputs.make_case("grid", seed=34, nlon=16, nlat=6, nivbas=94, daynum=355.5, polar_frac=0.5)
    ref, dref, _ = oracle.step(case, niter=5, fuse=True, diag=True)
    assert dref[DIAG_NAMES.index("vsed")].max() > 0, "no PSC cells in the workload"
    got, _ = _run_gpu(case)
    _compare(got, ref, STEP_TOL)


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
    _compare(got, ref, STEP_TOL)
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
    _compare(st, ref, STEP_TOL)


def test_irapp_slice(torch):
    case = inputs.make_case("cfg0", seed=39, nlon=16, nivbas=94, nrappmax=3, irapp=2)
    ref, _, _ = oracle.step(case, niter=5, fuse=True)
    got, _ = _run_gpu(case)
    _compare(got, ref, STEP_TOL)


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
    _compare(got, ref, STEP_TOL)


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
    _compare(st, ref, STEP_TOL)
