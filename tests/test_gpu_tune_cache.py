"""The autotuner's persisted choices (REPROBUS_TUNE_CACHE): the first handle
times the solve-kernel shapes and stores its choice; the next handle for the
same GPU, precision and cell count takes it from the file without timing;
a choice planted in the file is used as written."""
import pytest

from reprobus_gb300 import ChemStep, inputs
from reprobus_gb300.chem import SOLVER_NEWTON_MIXED

pytestmark = pytest.mark.gpu


def _run(case):
    from reprobus_gb300.resident import DeviceCase
    h = ChemStep.for_case(case, niter=5, flags=0)
    h.set_solver(SOLVER_NEWTON_MIXED)
    dc = DeviceCase(case)
    st = h.step_dev(1, case.nlat, case.daynum, case.dt, *dc.args(), stats=True)
    h.close()
    return st


def _shape(st):
    return st["lanes_per_block"], st["z_shared"], st["blocks_per_sm"]


def test_tune_cache_roundtrip(tmp_path, monkeypatch):
    path = tmp_path / "tune.txt"
    monkeypatch.setenv("REPROBUS_TUNE_CACHE", str(path))
    case = inputs.make_case("cfg0", seed=2, nlon=16, nivbas=94)
    st1 = _run(case)
    lines = path.read_text().splitlines()
    assert len(lines) == 1
    key, nth, zs, bps, _ = lines[0].split()
    assert "fp32" in key and f"{case.ncells}cells" in key
    assert (int(nth), int(zs), int(bps)) == _shape(st1)
    st2 = _run(case)
    assert _shape(st2) == _shape(st1)
    assert len(path.read_text().splitlines()) == 1  # taken from the file, not tuned again
    path.write_text(f"{key} 96 0 1 0.0\n")
    assert _shape(_run(case)) == (96, 0, 1)
