"""Known-answer tests of the CPU oracle, derived from the reference code.

The reference ships no tests or golden vectors (parity unpinned); these checks
pin the oracle's pieces against closed forms that the Fortran implies.
"""
import os

import numpy as np
import pytest

from conftest import relerr
from oracle import oracle
from reprobus_gb300 import inputs
from reprobus_gb300.species import DIAG_HET, DIAG_RATE, DIAG_SZA, DIAG_TJ, L, RATES, S, DIAG_HNM

pytestmark = pytest.mark.filterwarnings("ignore")


@pytest.fixture(scope="module")
def case():
    return inputs.make_case("cfg0", seed=11, nlon=24, nivbas=94)


def _hnm(case):
    k = case.irapp - 1
    return case.trajpre[..., k] / (case.trajtem[..., k] * 1.38e-19)


def test_troe_constants_match_const_formulas():
    # const, F:5927-5948: exact, same libm pow
    got = oracle.troe()
    assert np.array_equal(got, inputs.troe_constants())
    assert got[5] == 2.8e-11  # 300**0.0 == 1
    assert got[11] == 1.0e-10 * 300.0


def test_dt_zero_returns_initial_state(case):
    # F:2364-2369 with dt = 0: ck = ck0 after every pass; write-back ck/hnm
    case0 = inputs.make_case("cfg0", seed=11, nlon=24, nivbas=94, dt=0.0)
    st, dg, passes = oracle.step(case0, niter=5, fuse=False, diag=True)
    assert passes == 5
    hnm = _hnm(case0)[:, :, :94]
    for n in range(42):
        exp = (case0.qj1[:, :, :94, n] * hnm) / hnm
        assert np.array_equal(st["qj1"][:, :, :94, n], exp), n
    # hno3 gas, F:2392-2394: ck5*parthno3/hnm
    part = dg[53].reshape(hnm.shape, order="F")
    exp = ((case0.qj1[:, :, :94, 4] * hnm) * part) / hnm
    assert np.array_equal(st["qj1"][:, :, :94, 42], exp)
    # levels below nivbas are untouched without the fused epilogue
    assert np.array_equal(st["qj1"][:, :, 94:, :], case0.qj1[:, :, 94:, :])


def test_night_closed_forms(case):
    # night branch F:1673-1746 with dt = 0 (ck = ck0 in every pass)
    case0 = inputs.make_case("cfg0", seed=11, nlon=24, nivbas=94, dt=0.0)
    st, dg, _ = oracle.step(case0, niter=5, fuse=False, diag=True)
    shp = (case0.nlon, case0.nlat, 94)
    sza = dg[DIAG_SZA].reshape(shp, order="F")
    night = sza > 95.0
    assert night.sum() > 50, "need night cells"
    hnm = _hnm(case0)[:, :, :94]
    hc = st["hc"][:, :, :94, :]
    for sp in ("o1d", "oh", "cl", "o3p", "ho2", "no", "br", "n", "h", "ch3"):
        assert np.all(hc[..., S[sp]][night] == 0.0), sp
    ck = lambda sp: case0.qj1[:, :, :94, L[sp]] * hnm
    assert np.array_equal(hc[..., S["o3"]][night], (ck("ox") / hnm)[night])
    assert np.array_equal(hc[..., S["clo"]][night], (np.maximum(ck("clox"), 0.) / hnm)[night])
    assert np.array_equal(hc[..., S["bro"]][night], (np.maximum(ck("brox"), 0.) / hnm)[night])
    # NO2/NO3 fixed point of F:1721-1730, iterated 5 times from the input NO2
    b9 = dg[DIAG_RATE + RATES.index("b9")].reshape(shp, order="F")
    b12 = dg[DIAG_RATE + RATES.index("b12")].reshape(shp, order="F")
    cc7 = case0.hc[:, :, :94, S["no2"]] * hnm
    cc5 = ck("ox")
    for _ in range(5):
        r8 = b9 * cc5 / (b12 * np.maximum(cc7, 1e-30))
        cc7 = ck("nox") / (1. + r8)
        cc13 = r8 * cc7
    assert np.array_equal(hc[..., S["no2"]][night], (cc7 / hnm)[night])
    assert np.array_equal(hc[..., S["no3"]][night], (cc13 / hnm)[night])


def test_photolysis_zero_at_night_and_jno_top_switch(case):
    _, dg, _ = oracle.step(case, niter=1, fuse=False, diag=True)
    shp = (case.nlon, case.nlat, 94)
    sza = dg[DIAG_SZA].reshape(shp, order="F")
    tj = dg[DIAG_TJ:DIAG_TJ + 41].reshape((41,) + shp, order="F")
    assert np.all(tj[:40][:, sza > 95.0] == 0.0)
    assert np.all(tj[:40][:, sza <= 95.0] > 0.0)
    # jno uses the level-1 zenith angle of the column (JNO:139)
    top = sza[:, :, :1]
    dark_top = np.broadcast_to(top > 89.0, shp)
    assert np.all(tj[40][dark_top] == 0.0)
    assert np.all(tj[40][~dark_top] >= 1e-30)


def test_phot_weights_sum_to_one():
    # a table constant in (z, sza, o3) returns that constant (trilinear weights sum to 1)
    c = inputs.make_case("cfg0", seed=5, nlon=16, nivbas=94)
    vals = np.logspace(-9, -1, 40)
    c.ajl = np.asfortranarray(np.broadcast_to(vals[:, None, None, None], c.ajl.shape).copy(order="F"))
    _, dg, _ = oracle.step(c, niter=1, fuse=False, diag=True)
    shp = (c.nlon, c.nlat, 94)
    sza = dg[DIAG_SZA].reshape(shp, order="F")
    tj = dg[DIAG_TJ:DIAG_TJ + 40].reshape((40,) + shp, order="F")
    day = sza <= 95.0
    err = relerr(tj[:, day], np.broadcast_to(vals[:, None], tj[:, day].shape))
    assert err.max() < 1e-14


def test_arrhenius_rates_independent(case):
    # a few rate constants evaluated independently from the formulas of F:938-1303
    _, dg, _ = oracle.step(case, niter=1, fuse=False, diag=True)
    t = case.trajtem[..., 0][:, :, :94].reshape(-1, order="F")
    hnm = dg[DIAG_HNM]
    k = lambda name: dg[DIAG_RATE + RATES.index(name)]
    assert relerr(k("a2"), 1.4e-10 * np.exp(-470. / t)).max() < 4e-16
    assert relerr(k("d62"), 1.0e-12 * np.exp(-1590. / t) + 3.0e-11 * np.exp(-2450. / t)).max() < 1e-15
    assert relerr(k("hk2"), 6.0e-34 * (300. / t) ** 2.4 * hnm).max() < 1e-15
    assert np.all(k("c3") == 1.1e-10)
    # Troe, a1 (F:930-935) against its closed form
    tr = inputs.troe_constants()
    ak0 = tr[0] * np.exp(np.log(t) * -1.3)
    ak1 = tr[1] * np.exp(np.log(t) * 0.2)
    a1 = (ak0 * hnm) / (1. + ak0 * hnm / ak1) * np.exp(np.log(0.6) / (1. + np.log10(ak0 * hnm / ak1) ** 2))
    assert relerr(k("a1"), a1).max() < 1e-14
    # low-pressure limit of the fall-off form: k -> k0*M*0.6 when k0*M << kinf
    assert np.all(k("a1") <= ak0 * hnm)


def test_het_zero_above_aerosol_levels(case):
    _, dg, _ = oracle.step(case, niter=1, fuse=False, diag=True)
    shp = (case.nlon, case.nlat, 94)
    het = dg[DIAG_HET:DIAG_HET + 9].reshape((9,) + shp, order="F")
    assert np.all(het[:, :, :, :13] == 0.0)  # levels 1..nivhau-1
    assert np.all(het[8] == 0.0)             # het9 is switched off (F:4024)
    assert np.all(np.isfinite(het))


def test_conserv_restores_element_totals(case):
    st, _, _ = oracle.step(case, niter=5, fuse=False)
    q, h = st["qj1"].copy(order="F"), st["hc"].copy(order="F")
    brcl_before = q[:, :, :94, L["brcl"]].copy()
    brono2_before = q[:, :, :94, L["brono2"]].copy()
    oracle.conserv(case, q, h)
    Q = lambda sp: q[:, :, :94, L[sp]]
    cl = Q("oclo") + Q("hcl") + Q("clono2") + Q("hocl") + 2 * Q("cl2") + Q("clno2") + Q("clox") + 2 * Q("cl2o2")
    # the chlorine rescale (F:2555) uses BrCl before the bromine rescale (F:2609) changes it
    assert relerr(cl, Q("cly") - brcl_before).max() < 1e-14
    br = Q("hbr") + Q("brono2") + Q("brox") + Q("hobr") + Q("brcl")
    assert relerr(br, Q("bry")).max() < 1e-14
    n = Q("hno3") + 2 * Q("n2o5") + Q("nox") + Q("ho2no2")
    # nitrogen (F:2578) sees ClONO2/ClNO2 after the chlorine rescale, BrONO2 before the bromine one
    assert relerr(n, np.maximum(Q("noy") - Q("clono2") - Q("clno2") - brono2_before, 0.)).max() < 1e-14


def test_clamp_and_hno3_gas_below_nivbas(case):
    st, _, _ = oracle.step(case, niter=5, fuse=True)
    q = st["qj1"]
    assert q[..., :42].min() >= 1e-30
    assert np.array_equal(q[:, :, 94:, 42], q[:, :, 94:, 4])


def test_fixed_point_iteration_mostly_converges():
    # Iterating the reference's map (F:1348-2378) past its 5 passes converges
    # in most cells; in some warm night cells the lagged quadratic ClO loss
    # makes it oscillate with growing amplitude (Picard does not converge
    # there, the fixed point itself still exists).
    c = inputs.make_case("cfg0", seed=2, nlon=8, nivbas=94)
    a, _, _ = oracle.step(c, niter=400, fuse=False)
    b, _, _ = oracle.step(c, niter=401, fuse=False)
    qa, qb = a["qj1"][:, :, :94, :42], b["qj1"][:, :, :94, :42]
    ok = np.all(np.isfinite(qa) & np.isfinite(qb), axis=-1)
    ok &= np.nan_to_num(relerr(qb, qa, 1e-30), nan=1.0).max(axis=-1) < 1e-12
    assert ok.mean() > 0.9
    e = []
    for nit in (5, 20, 80):
        st, _, _ = oracle.step(c, niter=nit, fuse=False)
        e.append(np.median(relerr(st["qj1"][:, :, :94, :42], qa, 1e-30)[ok]))
    assert e[0] > e[1] > e[2]


def test_row_subset_leaves_other_rows():
    c = inputs.make_case("grid", seed=4, nlon=8, nlat=6, nivbas=94)
    st, _, _ = oracle.step(c, ilat0=2, ilat1=4, niter=5, fuse=True)
    for j in (0, 4, 5):
        assert np.array_equal(st["qj1"][:, j], c.qj1[:, j])
        assert np.array_equal(st["hc"][:, j], c.hc[:, j])
    assert not np.array_equal(st["qj1"][:, 2], c.qj1[:, 2])


def test_golden_regression_fixture():
    """Regression pin of the oracle on a fixed small workload (generated by
    tests/golden/make_golden.py from this oracle; it guards against changes
    to the oracle, it does not pin it to the reference)."""
    path = os.path.join(os.path.dirname(__file__), "golden", "oracle_cfg0_small.npz")
    g = np.load(path)
    c = inputs.make_case("cfg0", seed=int(g["seed"]), nlon=int(g["nlon"]), nivbas=int(g["nivbas"]))
    st, _, _ = oracle.step(c, niter=5, fuse=True)
    assert relerr(st["qj1"], g["qj1"]).max() < 1e-12
    assert relerr(st["hc"], g["hc"]).max() < 1e-12
