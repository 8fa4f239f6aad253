"""Column physics on the GPU (reprobus_gb300/csrc/column_kernels.cu) through
the C-ABI, against the CPU oracle (oracle/column_oracle.cpp) on the same
seeded inputs.

Tolerances: sedimentation and forcing round every operation as the oracle
does; only the logarithm (CUDA vs the C library, each within an ulp or two)
differs, so 1e-13 relative. Altitude adds cos() and a 137-level sum of
logarithms: 1e-12 relative. The history record is byte for byte."""
import os
import struct
import tempfile

import numpy as np
import pytest

from conftest import relerr
from oracle import column
from reprobus_gb300 import ChemStep, inputs

from test_column_oracle import grid_inputs, sed_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as T
    assert T.cuda.is_available(), "GPU tests need CUDA"
    return T


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))).cuda()


def _host(t, like):
    return t.cpu().numpy().reshape(like.shape, order="F")


def _handle(nlon, nlat, niv=137, nivbas=94):
    case = inputs.make_case("grid", seed=0, nlon=4, nlat=3, nivbas=nivbas)
    return ChemStep(case.ajl, case.o3up, nlon, nlat, niv, nivbas=nivbas, nivhau=14, nrappmax=1, niter=5, flags=0)


@pytest.mark.parametrize("rows", [None, (2, 3)])
def test_sedimentation_matches_oracle(torch, rows):
    case, pre, tem, vsed, ph2o, pno3 = sed_case(seed=5, nlon=40, nlat=5)
    ilat0, ilat1 = rows if rows else (1, case.nlat)
    ref = case.qj1.copy(order="F")
    column.sedimentation(94, 14, pre, tem, ref, vsed, 59, ph2o, pno3, 10800., ilat0, ilat1)
    h = _handle(case.nlon, case.nlat)
    q = _dev(torch, case.qj1)
    h.sedimentation_dev(_dev(torch, case.trajpre), _dev(torch, case.trajtem), 1, q, _dev(torch, vsed), 59,
                        _dev(torch, ph2o), _dev(torch, pno3), 10800., ilat0, ilat1)
    got = _host(q, ref)
    h.close()
    assert relerr(got, ref).max() <= 1e-13
    if rows:  # other rows untouched
        assert np.array_equal(got[:, 0], case.qj1[:, 0])


def test_forcing_matches_oracle(torch):
    case = inputs.make_case("grid", seed=6, nlon=30, nlat=7, nivbas=94)
    rng = np.random.default_rng(6)
    co = np.asfortranarray(rng.uniform(5e-8, 2e-7, (case.nlon, case.nlat)))
    hj1 = np.asfortranarray(rng.uniform(1e-6, 1e-2, (case.nlon, case.nlat, case.niv)))
    pre = np.asfortranarray(case.trajpre[..., 0])
    q, hc = case.qj1.copy(order="F"), case.hc.copy(order="F")
    column.forcing(94, 2015, 11, 900., pre, q, hc, co=co, hj1=hj1, nivh2o=59)
    h = _handle(case.nlon, case.nlat)
    qd, hd = _dev(torch, case.qj1), _dev(torch, case.hc)
    h.forcing_dev(2015, 11, 900., _dev(torch, case.trajpre), 1, qd, hd, co_month=_dev(torch, co),
                  hj1=_dev(torch, hj1), nivh2oecmwf=59)
    gq, gh = _host(qd, q), _host(hd, hc)
    assert relerr(gq, q).max() <= 1e-13 and relerr(gh, hc).max() <= 1e-13
    # without the optional fields: tropo alone
    q2, hc2 = case.qj1.copy(order="F"), case.hc.copy(order="F")
    column.forcing(94, 2015, 11, 900., pre, q2, hc2)
    qd, hd = _dev(torch, case.qj1), _dev(torch, case.hc)
    h.forcing_dev(2015, 11, 900., _dev(torch, case.trajpre), 1, qd, hd)
    assert relerr(_host(qd, q2), q2).max() <= 1e-13
    h.close()


def test_forcing_rejects_dates_outside_the_tables(torch):
    from reprobus_gb300.chem import ReprobusError
    case = inputs.make_case("grid", seed=6, nlon=4, nlat=3, nivbas=94)
    h = _handle(case.nlon, case.nlat)
    qd, hd = _dev(torch, case.qj1), _dev(torch, case.hc)
    with pytest.raises(ReprobusError):
        h.forcing_dev(1980, 1, 900., _dev(torch, case.trajpre), 1, qd, hd)
    assert np.array_equal(_host(qd, case.qj1), case.qj1)
    h.close()


def test_altitude_matches_oracle_on_moved_trajectories(torch):
    g = grid_inputs(7, nlon=36, nlat=19)
    rng = np.random.default_rng(7)
    shp = g["t"].shape
    # trajectories moved off their grid points (nearest-point lookup, the
    # pressure search and the clamp at the lowest level all act)
    g["trajlon"] = np.asfortranarray((g["trajlon"] + rng.uniform(-14., 14., shp)) % 360.)
    g["trajlat"] = np.asfortranarray(np.clip(g["trajlat"] + rng.uniform(-9., 9., shp), -90., 90.))
    g["trajpre"] = np.asfortranarray(g["trajpre"] * rng.uniform(0.8, 1.25, shp))
    ref = column.altitude(**g)
    h = _handle(shp[0], shp[1])
    alt = torch.zeros(ref.size, dtype=torch.float64, device="cuda")
    h.altitude_dev(*(_dev(torch, g[k]) for k in ("relief", "psol", "aaa", "bbb", "t", "h2o", "trajlon", "trajlat",
                                                  "trajpre")), alt, irapp=1)
    got = _host(alt, ref)
    h.close()
    assert np.all(np.isfinite(got))
    assert relerr(got, ref, floor=1e-3).max() <= 1e-12


def _hist_arrays(torch, nlon, nlat, niv, seed):
    rng = np.random.default_rng(seed)
    shapes = [(nlon, nlat), (nlon, nlat, niv), (nlon, nlat, niv), (nlon, nlat, niv), (nlon, nlat, niv),
              (nlon, nlat, niv, 43), (nlon, nlat, niv), (nlon, nlat, niv, 15)]
    host = [np.asfortranarray(rng.standard_normal(s) * 10.0 ** rng.uniform(-30, 5, s)) for s in shapes]
    return host, [_dev(torch, a) for a in host]


def _read_like_post_processor(path, nlon, nlat, niv):
    """The reading convention of post-process-reprobus.py:127-143 (the
    record marker and name in the first 10 bytes, then big-endian data)."""
    with open(path, "rb") as f:
        head = f.read(10)
        date = struct.unpack(">iiiii", f.read(20))
        out = [np.fromfile(f, dtype=">f8", count=nlon * nlat)]
        for n in (1, 1, 1, 1, 43, 1, 15):
            out.append(np.fromfile(f, dtype=">f8", count=nlon * nlat * niv * n))
        tail = f.read()
    return head, date, out, tail


def test_history_record_roundtrip_and_format(torch):
    nlon, nlat, niv = 12, 5, 137
    h = _handle(nlon, nlat, niv)
    host, dev = _hist_arrays(torch, nlon, nlat, niv, 8)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "MODEL_history_2010031512_001442")
        h.history_write_dev(path, "001442", (2010, 3, 15, 12, 0), *dev)
        head, date, arrs, tail = _read_like_post_processor(path, nlon, nlat, niv)
        nbytes = os.path.getsize(path)
        assert struct.unpack(">i", head[:4])[0] == nbytes - 8 and head[4:] == b"001442"
        assert date == (2010, 3, 15, 12, 0) and tail == head[:4]
        for a, b in zip(arrs, host):
            assert np.array_equal(a.astype(np.float64), b.reshape(-1, order="F"))
        # read back into fresh device arrays: bit for bit
        back = [torch.zeros_like(t) for t in dev]
        name, date2 = h.history_read_dev(path, *back)
        assert name == "001442" and date2 == (2010, 3, 15, 12, 0)
        for a, b in zip(back, dev):
            assert torch.equal(a.view(torch.int64), b.view(torch.int64))
        # a record for another grid is refused
        h2 = _handle(nlon + 1, nlat, niv)
        from reprobus_gb300.chem import ReprobusError
        with pytest.raises(ReprobusError):
            h2.history_read_dev(path, *[torch.zeros(1, dtype=torch.float64, device="cuda")] * 8)
        h2.close()
    h.close()


def test_history_reads_a_record_written_on_the_host(torch):
    # a record written by plain numpy in the reference's layout (the role of
    # the Fortran writer, F:587-588) is read on the GPU bit for bit
    nlon, nlat, niv = 7, 4, 137
    h = _handle(nlon, nlat, niv)
    host, _ = _hist_arrays(torch, nlon, nlat, niv, 9)
    payload = b"abc   " + struct.pack(">iiiii", 1999, 12, 31, 23, 45) + b"".join(
        a.reshape(-1, order="F").astype(">f8").tobytes() for a in host)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "restart")
        with open(path, "wb") as f:
            f.write(struct.pack(">i", len(payload)) + payload + struct.pack(">i", len(payload)))
        back = [torch.zeros(a.size, dtype=torch.float64, device="cuda") for a in host]
        name, date = h.history_read_dev(path, *back)
    assert name == "abc   " and date == (1999, 12, 31, 23, 45)
    for a, b in zip(back, host):
        assert np.array_equal(a.cpu().numpy(), b.reshape(-1, order="F"))
    h.close()
