"""CPU checks of the generated step equations (reprobus_gb300/codegen/
gen_newton.py -> csrc/newton_gen.cuh), through a host build of the generated
code (tests/newton_host.cpp):
  * the committed header is what the generator writes;
  * its residual vanishes at the oracle's fixed point of the reference map;
  * its Jacobian matches finite differences of its residual;
  * the Newton iteration (FP64 and FP32 Jacobian) converges to that fixed point;
  * on a polar-winter mix, Oracle-C converges on at least 99.9 % of the cells
    and the Newton iteration at the production tolerance lands within 1e-6.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle
from reprobus_gb300 import inputs
from reprobus_gb300.species import DIAG_HET, DIAG_HNM, DIAG_NAMES, DIAG_RATE, DIAG_SZA, DIAG_TJ

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN = os.path.join(ROOT, "reprobus_gb300", "csrc", "newton_gen.cuh")


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("nt") / "libnthost.so")
    extra = os.environ.get("REPROBUS_SANITIZE_FLAGS", "").split()  # set by test_sanitizers.py
    subprocess.run(["g++", "-O1", "-std=c++17", "-fPIC", "-shared", *extra, "-o", out,
                    os.path.join(ROOT, "tests", "newton_host.cpp")], check=True)
    L = ctypes.CDLL(out)
    dp = ctypes.POINTER(ctypes.c_double)
    L.nt_host_residual.argtypes = [dp] * 5 + [ctypes.c_int, dp, dp]
    L.nt_host_jacobian.argtypes = [dp] * 4 + [ctypes.c_int, dp, dp]
    L.nt_host_newton.argtypes = [dp] * 5 + [ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp]
    L.nt_host_residual_groups.argtypes = [ctypes.c_int] + [dp] * 5 + [ctypes.c_int, dp, dp]
    L.nt_host_jacobian_groups.argtypes = [ctypes.c_int] + [dp] * 4 + [ctypes.c_int, dp, dp]
    return L


@pytest.fixture(scope="module")
def data():
    c = inputs.make_case("cfg0", seed=2, nlon=4, nivbas=94)
    _, dg, _ = oracle.step(c, niter=1, fuse=False, diag=True)
    fp, stat, _ = oracle.step_fixed_point(c, tol=1e-12, maxiter=60, fuse=False)
    r1, _, _ = oracle.step(c, niter=1, fuse=False)
    return c, dg, fp, stat, r1


def _P(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _cell_inputs(c, dg, cell):
    i, k = cell % c.nlon, cell // c.nlon
    hnm = dg[DIAG_HNM, cell]
    q0 = c.qj1[i, 0, k, :]
    rain = 1e-6 if (q0[2] * hnm) / hnm >= 100e-6 else 0.0
    fix = np.array([0.21 * hnm, 0.78 * hnm, 5e-7 * hnm, 360e-6 * hnm, hnm,
                    dg[DIAG_NAMES.index("parthno3"), cell], dg[DIAG_NAMES.index("parth2o"), cell],
                    dg[DIAG_NAMES.index("parthcl"), cell], 1.0, rain, rain, rain, rain, c.dt])
    return (np.ascontiguousarray(dg[DIAG_RATE:DIAG_RATE + 99, cell]), np.ascontiguousarray(dg[DIAG_TJ:DIAG_TJ + 41, cell]),
            np.ascontiguousarray(dg[DIAG_HET:DIAG_HET + 9, cell]), fix, np.ascontiguousarray(q0[:42] * hnm),
            int(dg[DIAG_SZA, cell] <= 95.0))


def _x(c, st, dg, cell):
    i, k = cell % c.nlon, cell // c.nlon
    hnm = dg[DIAG_HNM, cell]
    return np.concatenate([st["qj1"][i, 0, k, :42] * hnm, st["hc"][i, 0, k, :] * hnm])


def _pow2_scale(x, floor):
    """2^floor(log2(max(|x|, floor))), the generated code's unknown scales."""
    m, e = np.frexp(np.maximum(np.abs(x), floor))
    return np.ldexp(1.0, e - 1)


def test_generated_header_is_current(tmp_path):
    pytest.importorskip("sympy")
    from reprobus_gb300.codegen import gen_newton
    out = tmp_path / "newton_gen.cuh"
    gen_newton.generate(str(out))
    assert out.read_text() == open(GEN).read(), "rerun python -m reprobus_gb300.codegen.gen_newton"


def test_generated_quotients_go_through_nt_div():
    """Every quotient of the generated equations is an nt_div and every pivot
    reciprocal an nt_rcp (newton_num.cuh): no IEEE division sequence is left
    in the solve kernels' code."""
    code = "\n".join(line.split("//")[0] for line in open(GEN).read().splitlines())
    assert "/" not in code
    assert code.count("nt_rcp<T>(p)") == 57 * code.count("void nt_factor_solve(")
    assert code.count("nt_div<T>(") > 0


def test_residual_vanishes_at_the_reference_fixed_point(host, data):
    c, dg, fp, stat, _ = data
    worst = 0.0
    for cell in np.where(stat >= 0)[0]:
        K, tj, het, fix, ck0, day = _cell_inputs(c, dg, cell)
        x = _x(c, fp, dg, cell)
        R = np.zeros(57)
        host.nt_host_residual(_P(K), _P(tj), _P(het), _P(fix), _P(ck0), day, _P(x), _P(R))
        worst = max(worst, np.max(np.abs(R) / np.maximum(np.abs(x), 1e-20 * fix[4])))
    assert worst < 1e-9


def test_jacobian_matches_finite_differences(host, data):
    c, dg, fp, stat, _ = data
    for cell in np.where(stat >= 0)[0][::97][:4]:
        K, tj, het, fix, ck0, day = _cell_inputs(c, dg, cell)
        x = _x(c, fp, dg, cell)
        Jd = np.zeros(57 * 57)
        host.nt_host_jacobian(_P(K), _P(tj), _P(het), _P(fix), day, _P(x), _P(Jd))
        Jd = Jd.reshape(57, 57)
        s = _pow2_scale(x, 1e-20 * fix[4])
        for j in range(57):
            h = 1e-6 * s[j]
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            Rp, Rm = np.zeros(57), np.zeros(57)
            host.nt_host_residual(_P(K), _P(tj), _P(het), _P(fix), _P(ck0), day, _P(xp), _P(Rp))
            host.nt_host_residual(_P(K), _P(tj), _P(het), _P(fix), _P(ck0), day, _P(xm), _P(Rm))
            fd = (Rp - Rm) / (2 * h) * s[j] / s
            an = Jd[:, j]
            assert np.all(np.abs(an - fd) <= 1e-4 * np.abs(fd) + 1e-6), (cell, j)


@pytest.mark.parametrize("W", [2, 4])
def test_row_groups_reproduce_the_residual_and_jacobian(host, data, W):
    """The row groups that the warps of the warps-per-cell solve kernel
    evaluate cover every residual row and every stored Jacobian entry once,
    with the values of the whole functions, for day and night cells."""
    c, dg, fp, stat, r1 = data
    for cell in range(0, c.ncells, 7):
        K, tj, het, fix, ck0, day = _cell_inputs(c, dg, cell)
        x = _x(c, r1, dg, cell)
        R, Rg = np.zeros(57), np.zeros(57)
        host.nt_host_residual(_P(K), _P(tj), _P(het), _P(fix), _P(ck0), day, _P(x), _P(R))
        host.nt_host_residual_groups(W, _P(K), _P(tj), _P(het), _P(fix), _P(ck0), day, _P(x), _P(Rg))
        assert np.array_equal(R, Rg), (cell, np.where(R != Rg))
        Jd, Jg = np.zeros(57 * 57), np.zeros(57 * 57)
        host.nt_host_jacobian(_P(K), _P(tj), _P(het), _P(fix), day, _P(x), _P(Jd))
        host.nt_host_jacobian_groups(W, _P(K), _P(tj), _P(het), _P(fix), day, _P(x), _P(Jg))
        assert np.array_equal(Jd, Jg), (cell, np.where(Jd != Jg))


@pytest.mark.parametrize("mixed", [0, 1])
def test_newton_converges_to_the_fixed_point(host, data, mixed):
    c, dg, fp, stat, r1 = data
    fails, errs = 0, []
    for cell in range(c.ncells):
        K, tj, het, fix, ck0, day = _cell_inputs(c, dg, cell)
        x = _x(c, r1, dg, cell)
        last = ctypes.c_double()
        it = host.nt_host_newton(_P(K), _P(tj), _P(het), _P(fix), _P(ck0), day, _P(x), 12, 1e-10, mixed,
                                 ctypes.byref(last))
        if it < 0:
            fails += 1
            continue
        if stat[cell] >= 0:
            xs = _x(c, fp, dg, cell)
            errs.append(np.max(np.abs(x - xs) / np.maximum(np.abs(xs), 1e-20 * fix[4])))
    assert fails <= 2
    assert max(errs) < 1e-8


@pytest.fixture(scope="module")
def polar():
    """A polar-winter mix (30 % of the columns in polar night, T 183-195 K,
    active ClOx) on all 137 levels."""
    c = inputs.make_case("grid", seed=77, nlon=8, nlat=4, daynum=355.5, polar_frac=0.3)
    _, dg, _ = oracle.step(c, niter=1, fuse=False, diag=True)
    fp, stat, _, stage = oracle.step_fixed_point(c, tol=1e-12, maxiter=60, fuse=False, with_stage=True)
    r5, _, _ = oracle.step(c, niter=5, fuse=False)
    return c, dg, fp, stat, stage, r5


def test_oracle_fixed_point_covers_the_polar_winter_mix(polar):
    """Oracle-C converges on at least 99.9 % of the cells, and each cell's
    answer is an exact fixed point of the reference pass map."""
    c, dg, fp, stat, stage, _ = polar
    assert (stat >= 0).mean() >= 0.999, np.bincount(stage, minlength=7)
    mr = oracle.map_residual(c, fp["qj1"], fp["hc"])
    assert mr[stat >= 0].max() < 1e-10


def test_oracle_newton_from_a_fixed_point_stays_there(polar):
    """Newton started from a state (here Oracle-C's own answer) returns the
    fixed point nearest it: the check the GPU tests apply to the cells
    Oracle-C does not converge on."""
    c, dg, fp, stat, _, _ = polar
    st, pstat, _ = oracle.newton_from(c, fp["qj1"], fp["hc"])
    ok = stat >= 0
    assert (pstat[ok] >= 0).all()
    from oracle import accuracy
    assert accuracy.cell_errors(st, fp, c.nivbas)[ok].max() < 1e-9


@pytest.mark.parametrize("mixed", [0, 1])
def test_generated_newton_at_production_settings_matches_the_oracle(host, polar, mixed):
    """The generated equations' Newton iteration (host build) from the
    5-pass state with the production step tolerance 1e-4: within 1e-6 of
    Oracle-C for every species above 1e-20 mol/mol on every cell both
    converge on, for the FP64 and the FP32 Jacobian."""
    c, dg, fp, stat, _, r5 = polar
    fails, worst = 0, 0.0
    for cell in range(c.ncells):
        i, j, k = cell % c.nlon, (cell // c.nlon) % c.nlat, cell // (c.nlon * c.nlat)
        hnm = dg[DIAG_HNM, cell]
        q0 = c.qj1[i, j, k, :]
        rain = 1e-6 if q0[2] >= 100e-6 else 0.0
        fix = np.array([0.21 * hnm, 0.78 * hnm, 5e-7 * hnm, 360e-6 * hnm, hnm,
                        dg[DIAG_NAMES.index("parthno3"), cell], dg[DIAG_NAMES.index("parth2o"), cell],
                        dg[DIAG_NAMES.index("parthcl"), cell], 1.0, rain, rain, rain, rain, c.dt])
        K = np.ascontiguousarray(dg[DIAG_RATE:DIAG_RATE + 99, cell])
        tj = np.ascontiguousarray(dg[DIAG_TJ:DIAG_TJ + 41, cell])
        het = np.ascontiguousarray(dg[DIAG_HET:DIAG_HET + 9, cell])
        ck0 = np.ascontiguousarray(q0[:42] * hnm)
        x = np.concatenate([r5["qj1"][i, j, k, :42], r5["hc"][i, j, k, :]]) * hnm
        last = ctypes.c_double()
        it = host.nt_host_newton(_P(K), _P(tj), _P(het), _P(fix), _P(ck0), int(dg[DIAG_SZA, cell] <= 95.0), _P(x),
                                 16, 1e-4, mixed, ctypes.byref(last))
        if it < 0:
            fails += 1
            continue
        if stat[cell] >= 0:
            xs = np.concatenate([fp["qj1"][i, j, k, :42], fp["hc"][i, j, k, :]]) * hnm
            big = np.abs(xs) > 1e-20 * hnm
            e = np.where(big, np.abs(x - xs) / np.maximum(np.abs(xs), 1e-300), 0.0)
            worst = max(worst, float(e.max()))
    assert fails <= 0.001 * c.ncells
    assert worst <= 1e-6
