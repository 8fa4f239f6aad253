"""The allocation-free entry point (reprobus_chem_step_noalloc) against the
handle-based device entry point (reprobus_chem_step_dev).

It serves callers that may not allocate device memory while they run (their
GPU memory is reserved up front and handed out by their own runtime or pool,
or their process has a fixed device-memory budget): every array comes from the
caller and the step's scratch lives in one fixed device array of the library.
This file is collected last, so that a run that stops at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-7  # the full-step tolerance of tests/test_gpu_parity.py


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).cuda()


def test_noalloc_matches_device_entry_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "GPU test"
    from reprobus_gb300 import ChemStep, chem, inputs
    from reprobus_gb300.resident import DeviceCase

    case = inputs.make_case("grid", seed=51, nlon=24, nlat=6, nivbas=94)
    flags = chem.FUSE_CONSERV | chem.CHECK_FINITE
    # existing entry point: a handle, two steps in a row
    h = ChemStep.for_case(case, niter=5, flags=flags)
    ref = DeviceCase(case)
    # allocation-free entry point: caller-owned arrays, two steps in a row
    new = DeviceCase(case)
    ajl = _dev(torch, case.ajl)
    o3up = _dev(torch, case.o3up)
    for call in range(2):
        h.step_dev(1, case.nlat, case.daynum, case.dt, *ref.args())
        chem.step_noalloc(ajl, o3up, case.troe, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                          case.nrappmax, 5, flags, 1, case.nlat, case.daynum, case.dt, *new.args())
        torch.cuda.synchronize()
        a, b = new.state_host(), ref.state_host()
        for f in ("qj1", "hc", "sza3d", "vsed3d", "parth2osed", "parthno3sed", "surfarea"):
            assert np.all(np.isfinite(a[f]) == np.isfinite(b[f])), (call, f)
            assert relerr(a[f], b[f]).max() <= STEP_TOL, (call, f, relerr(a[f], b[f]).max())
    h.close()


def test_noalloc_row_subset_after_a_larger_call():
    # the scratch keeps the previous call's contents; a smaller call must not see them
    torch = pytest.importorskip("torch")
    from reprobus_gb300 import ChemStep, chem, inputs
    from reprobus_gb300.resident import DeviceCase

    case = inputs.make_case("grid", seed=52, nlon=16, nlat=5, nivbas=94)
    ajl, o3up = _dev(torch, case.ajl), _dev(torch, case.o3up)
    big = DeviceCase(case)
    chem.step_noalloc(ajl, o3up, case.troe, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                      case.nrappmax, 5, chem.FUSE_CONSERV, 1, case.nlat, case.daynum, case.dt, *big.args())
    sub = DeviceCase(case)
    chem.step_noalloc(ajl, o3up, case.troe, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                      case.nrappmax, 5, chem.FUSE_CONSERV, 2, 3, case.daynum, case.dt, *sub.args())
    h = ChemStep.for_case(case, niter=5, flags=chem.FUSE_CONSERV)
    ref = DeviceCase(case)
    h.step_dev(2, 3, case.daynum, case.dt, *ref.args())
    torch.cuda.synchronize()
    a, b = sub.state_host(), ref.state_host()
    for f in ("qj1", "hc", "sza3d", "vsed3d", "parth2osed", "parthno3sed", "surfarea"):
        assert relerr(a[f], b[f]).max() <= STEP_TOL, (f, relerr(a[f], b[f]).max())
    h.close()


def test_noalloc_on_a_caller_stream_back_to_back():
    # two calls on the caller's stream with no synchronisation between them
    # (calls on one stream run in order, so they do not race on the scratch)
    torch = pytest.importorskip("torch")
    from reprobus_gb300 import ChemStep, chem, inputs
    from reprobus_gb300.resident import DeviceCase

    case = inputs.make_case("grid", seed=54, nlon=20, nlat=4, nivbas=94)
    flags = chem.FUSE_CONSERV
    ajl, o3up = _dev(torch, case.ajl), _dev(torch, case.o3up)
    s = torch.cuda.Stream()
    new = DeviceCase(case)
    torch.cuda.synchronize()
    for _ in range(2):
        chem.step_noalloc(ajl, o3up, case.troe, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                          case.nrappmax, 5, flags, 1, case.nlat, case.daynum, case.dt, *new.args(), stream=s)
    s.synchronize()
    h = ChemStep.for_case(case, niter=5, flags=flags)
    h.set_stream(s)
    ref = DeviceCase(case)
    for _ in range(2):
        h.step_dev(1, case.nlat, case.daynum, case.dt, *ref.args())
    s.synchronize()
    a, b = new.state_host(), ref.state_host()
    for f in ("qj1", "hc", "sza3d", "vsed3d", "parth2osed", "parthno3sed", "surfarea"):
        assert relerr(a[f], b[f]).max() <= STEP_TOL, (f, relerr(a[f], b[f]).max())
    h.close()


def test_noalloc_refuses_troe_prefactors_that_are_not_positive():
    torch = pytest.importorskip("torch")
    from reprobus_gb300 import chem, inputs
    from reprobus_gb300.resident import DeviceCase

    case = inputs.make_case("grid", seed=55, nlon=8, nlat=2, nivbas=94)
    dc = DeviceCase(case)
    ajl, o3up = _dev(torch, case.ajl), _dev(torch, case.o3up)
    bad = np.array(case.troe, dtype=np.float64)
    bad[4] = -bad[4]
    with pytest.raises(chem.ReprobusError) as ei:
        chem.step_noalloc(ajl, o3up, bad, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                          case.nrappmax, 5, chem.FUSE_CONSERV, 1, case.nlat, case.daynum, case.dt, *dc.args())
    assert ei.value.code == 1 and "troe" in str(ei.value)


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from reprobus_gb300 import chem, inputs
    from reprobus_gb300.resident import DeviceCase

    case = inputs.make_case("grid", seed=53, nlon=180, nlat=30, nivbas=137)  # 3*180*30*137 > 2^20
    dc = DeviceCase(case)
    ajl, o3up = _dev(torch, case.ajl), _dev(torch, case.o3up)
    before = dc["qj1"].clone()
    with pytest.raises(chem.ReprobusError) as ei:
        chem.step_noalloc(ajl, o3up, case.troe, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                          case.nrappmax, 5, chem.FUSE_CONSERV, 1, case.nlat, case.daynum, case.dt, *dc.args())
    assert ei.value.code == 1 and "scratch" in str(ei.value)
    assert torch.equal(before, dc["qj1"])
