"""The CPU oracle of the column physics (oracle/column_oracle.cpp), pinned by
known answers derived from the reference code, and the library's host-side
forcing interpolation against it (no GPU needed).

F = src/reprobus_l137_20230723.f of the reference."""
import math

import numpy as np
import pytest

from oracle import column
from reprobus_gb300 import inputs

# June values of the reference's data statements (subroutine tropo,
# F:4099-4411): year -> (n2o, ch4, cfc11) at table index year - 1988
KAT = {2000: (315.6e-9, None, None), 1988: (306.2e-9, 1.693e-6, 245.21e-12)}


def test_tropo_values_at_table_years():
    # yearccmval = ian + (imois - 1)/12 = Y + 0.5 in July: cinf = 0, the value
    # of year Y itself (F:4416-4424)
    v = column.tropo_values(2000, 7)
    assert v[0] == KAT[2000][0]
    v = column.tropo_values(1988, 7)
    assert v[0] == KAT[1988][0] and v[1] == KAT[1988][1] and v[4] == KAT[1988][2]
    assert v[2] == 0.3e-9 and v[3] == 40.e-12 and v[14] == 0.5e-12 and v[15] == 2.5e-12


def test_tropo_values_interpolate_linearly_and_lump():
    a, b = column.tropo_values(2004, 7), column.tropo_values(2005, 7)
    m = column.tropo_values(2005, 1)  # yearccmval = 2005.0: halfway between the Junes
    assert np.allclose(m, 0.5 * (a + b), rtol=1e-14, atol=0)
    # CFC-12 slot carries CFC-114 + CFC-115/2 (F:4476), 1988 table values
    v = column.tropo_values(1988, 7)
    assert v[5] == 445.e-12 + 14.57e-12 + 0.5 * 4.62e-12


def test_tropo_values_refuse_dates_outside_the_tables():
    for y, m in ((1988, 6), (1987, 12), (2024, 7), (2030, 1)):
        with pytest.raises(ValueError):
            column.tropo_values(y, m)


def test_library_host_interpolation_equals_oracle(lib_built):
    from reprobus_gb300 import chem
    for y in (1988, 1995, 2010, 2023, 2024):
        for m in range(1, 13):
            try:
                ref = column.tropo_values(y, m)
            except ValueError:
                with pytest.raises(chem.ReprobusError):
                    chem.tropo_values(y, m)
                continue
            assert np.array_equal(chem.tropo_values(y, m), ref)


def sed_case(seed=0, nlon=8, nlat=3):
    case = inputs.make_case("grid", seed=seed, nlon=nlon, nlat=nlat, nivbas=94)
    rng = np.random.default_rng(seed)
    shp = (nlon, nlat, 94)
    vsed = np.asfortranarray(rng.uniform(0., 2e-3, shp) * (rng.uniform(size=shp) < 0.7))
    vsed[rng.uniform(size=shp) < 0.05] = 5.0  # fractions clamped to 1 (F:2464-2465)
    ph2o = np.asfortranarray(rng.uniform(0., 1., shp))
    pno3 = np.asfortranarray(rng.uniform(0., 1., shp))
    pre = np.asfortranarray(case.trajpre[..., 0])
    tem = np.asfortranarray(case.trajtem[..., 0])
    return case, pre, tem, vsed, ph2o, pno3


def test_sedimentation_is_identity_without_settling():
    case, pre, tem, vsed, ph2o, pno3 = sed_case()
    q = case.qj1.copy(order="F")
    column.sedimentation(94, 14, pre, tem, q, np.zeros_like(vsed, order="F"), 59, ph2o, pno3, 10800.)
    assert np.array_equal(q, case.qj1)
    q = case.qj1.copy(order="F")  # everything in the non-sedimenting part
    column.sedimentation(94, 14, pre, tem, q, vsed, 59, np.ones_like(ph2o, order="F"),
                         np.ones_like(pno3, order="F"), 10800.)
    assert np.array_equal(q, case.qj1)


def test_sedimentation_moves_the_hno3_flux_into_noy():
    # the NOy update takes the HNO3 terms (F:2493-2500): both change alike
    case, pre, tem, vsed, ph2o, pno3 = sed_case(seed=1)
    q = case.qj1.copy(order="F")
    column.sedimentation(94, 14, pre, tem, q, vsed, 59, ph2o, pno3, 10800.)
    d4 = q[..., 3] - case.qj1[..., 3]
    d5 = q[..., 4] - case.qj1[..., 4]
    assert np.abs(d5).max() > 0
    assert np.allclose(d4, d5, rtol=0, atol=1e-15 * np.abs(case.qj1[..., 3:5]).max())
    # levels outside nivhau..nivbas untouched; H2O only on nivhau..nivh2o-1
    assert np.array_equal(q[:, :, :13], case.qj1[:, :, :13])
    assert np.array_equal(q[:, :, 94:], case.qj1[:, :, 94:])
    assert np.array_equal(q[:, :, 58:, 2], case.qj1[:, :, 58:, 2])


def test_forcing_writes_only_below_nivbas():
    case = inputs.make_case("grid", seed=2, nlon=6, nlat=4, nivbas=94)
    q, h = case.qj1.copy(order="F"), case.hc.copy(order="F")
    pre = np.asfortranarray(case.trajpre[..., 0])
    column.forcing(94, 2010, 3, 900., pre, q, h)
    v = column.tropo_values(2010, 3)
    slots = [1, 2, 4, 7] + list(range(31, 43))
    for n, s in enumerate(slots):
        assert np.all(q[:, :, 94:, s - 1] == v[n])
    assert np.array_equal(q[:, :, :93], case.qj1[:, :, :93])
    assert np.array_equal(h[:, :, 93:, 4], q[:, :, 93:, 7]) and np.array_equal(q[:, :, 93:, 10], q[:, :, 93:, 7])
    # Ox relaxes towards its limit with exp(-1/96) per 15 min (F:4528-4543)
    p = pre[:, :, 94:]
    lim = np.where(p > 370., -2.3825e-8 * np.log(p) + 1.9457e-7, case.qj1[:, :, 94:, 7])
    want = np.maximum(lim + (case.qj1[:, :, 94:, 7] - lim) * math.exp(-(900. / 86400.)), 0.)
    assert np.allclose(q[:, :, 94:, 7], want, rtol=1e-15, atol=0)


def grid_inputs(seed, nlon=36, nlat=19, relief=True):
    rng = np.random.default_rng(seed)
    aaa, bbb = inputs.l137_levels()
    niv = len(aaa)
    ps = rng.uniform(980., 1030., (nlon, nlat))
    p = aaa[None, None, :] + bbb[None, None, :] * ps[..., None]
    z = 7.0 * np.log(1013.25 / p)
    t = np.asfortranarray(np.clip(250. - 3. * np.minimum(z, 12.) + rng.uniform(-5, 5, p.shape), 185, 300))
    h2o = np.asfortranarray(5e-6 + 1e-2 * np.exp(-z / 2.2) * rng.uniform(0.5, 1.5, p.shape))
    rel = np.asfortranarray(rng.uniform(0., 3., (nlon, nlat)) if relief else np.zeros((nlon, nlat)))
    lon = np.arange(nlon) * (360. / nlon)
    lat = 90. - np.arange(nlat) * (180. / (nlat - 1))
    tl = np.asfortranarray(np.broadcast_to(lon[:, None, None], p.shape))
    tb = np.asfortranarray(np.broadcast_to(lat[None, :, None], p.shape))
    return dict(relief=rel, psol=np.asfortranarray(ps), aaa=aaa, bbb=bbb, t=t, h2o=h2o, trajlon=tl, trajlat=tb,
                trajpre=np.asfortranarray(p.copy()))


def test_altitude_oracle_matches_the_generator_restatement():
    # trajectories at their own grid points, no relief: the special case that
    # reprobus_gb300/inputs.py restates independently in numpy
    g = grid_inputs(3, relief=False)
    alt = column.altitude(**g)
    nlon, nlat, niv = g["t"].shape
    tv = g["t"] * (1. + 0.608 * g["h2o"] * 18. / 28.97)
    pc = lambda a: np.moveaxis(a, 2, 0).reshape(niv, -1, order="F")
    want = inputs._altitude(pc(g["trajpre"]), g["psol"].reshape(-1, order="F"), pc(tv),
                            pc(g["trajlat"])[0])
    got = pc(alt)
    assert np.allclose(got, want, rtol=1e-13, atol=1e-12)
    assert np.all(np.diff(got, axis=0) < 0)  # altitude decreases downwards


def test_altitude_oracle_interpolates_within_the_column():
    # a point halfway (in log p) between two regular levels of its own column
    # gets an altitude between theirs
    g = grid_inputs(4)
    base = column.altitude(**g)
    k = 60
    g2 = dict(g)
    pre = g["trajpre"].copy(order="F")
    pre[:, :, k] = np.sqrt(g["trajpre"][:, :, k] * g["trajpre"][:, :, k + 1])
    g2["trajpre"] = pre
    alt = column.altitude(**g2)
    assert np.all(alt[:, :, k] < base[:, :, k]) and np.all(alt[:, :, k] > base[:, :, k + 1])
