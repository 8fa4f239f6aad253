"""ctypes front end of the CPU FP64 oracle (chem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker, never as the measured or
shipped path. PARITY UNPINNED: see chem_oracle.c.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "chem_oracle.c")
# a prebuilt copy to load instead (the sanitizer runs of tests/ build one)
LIB_OVERRIDE = "REPROBUS_ORACLE_LIB"

CFLAGS = ["-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compiles the oracle with gcc (IEEE, no FMA contraction, OpenMP)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", *CFLAGS, "-o", LIB, SRC, "-lm"]
        subprocess.run(cmd, check=True)
    from . import column
    column.build(force)
    return LIB


class OrcGrid(ctypes.Structure):
    _fields_ = [
        ("nlon", ctypes.c_int), ("nlat", ctypes.c_int), ("niv", ctypes.c_int),
        ("nivbas", ctypes.c_int), ("nivhau", ctypes.c_int), ("nrappmax", ctypes.c_int),
        ("niter", ctypes.c_int), ("tol", ctypes.c_double), ("maxiter", ctypes.c_int),
        ("ajl", ctypes.POINTER(ctypes.c_double)), ("o3up", ctypes.POINTER(ctypes.c_double)),
        ("troe", ctypes.c_double * 18),
        ("newton", ctypes.c_int), ("cellstat", ctypes.POINTER(ctypes.c_int)),
        ("cellres", ctypes.POINTER(ctypes.c_double)),
        ("x_qj1", ctypes.POINTER(ctypes.c_double)), ("x_hc", ctypes.POINTER(ctypes.c_double)),
        ("cellstage", ctypes.POINTER(ctypes.c_int)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.environ.get(LIB_OVERRIDE)
        if not path:
            path = build()
        _lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.orc_step.restype = ctypes.c_int
        _lib.orc_step.argtypes = [ctypes.POINTER(OrcGrid), ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_double, dp, dp, dp, dp, dp, ctypes.c_int, dp, dp, dp, dp, dp, dp,
                                  dp, ctypes.c_int, dp, ctypes.c_int]
        _lib.orc_const.argtypes = [dp]
        _lib.orc_conserv.argtypes = [ctypes.POINTER(OrcGrid), ctypes.c_int, ctypes.c_int, dp, dp]
        _lib.orc_clamp.argtypes = [ctypes.POINTER(OrcGrid), ctypes.c_int, ctypes.c_int, dp]
    return _lib


def _p(a):
    assert a.dtype == np.float64
    assert a.flags.f_contiguous or a.ndim == 1
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def troe():
    out = np.zeros(18)
    lib().orc_const(_p(out))
    return out


def grid(case, niter=5, tol=0.0, maxiter=0, troe_vals=None, newton=False, cellstat=None, cellres=None):
    g = OrcGrid()
    g.cellres = cellres.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if cellres is not None else None
    g.newton = int(bool(newton))
    g.cellstat = cellstat.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if cellstat is not None else None
    g.nlon, g.nlat, g.niv = case.nlon, case.nlat, case.niv
    g.nivbas, g.nivhau, g.nrappmax = case.nivbas, case.nivhau, case.nrappmax
    g.niter, g.tol, g.maxiter = niter, tol, maxiter
    g.ajl = _p(case.ajl)
    g.o3up = _p(case.o3up)
    tv = case.troe if troe_vals is None else troe_vals
    for i in range(18):
        g.troe[i] = float(tv[i])
    return g


def step(case, niter=5, fuse=True, diag=False, nthreads=0, ilat0=1, ilat1=None, tol=0.0, maxiter=0,
         state=None):
    """Runs the chemistry block of the time loop on copies of the case state
    (or on `state`, a dict as returned by case.state_copy(), in place).
    ilat0/ilat1 are 1-based inclusive rows. Returns (state, diag or None, passes)."""
    L = lib()
    g = grid(case, niter=niter, tol=tol, maxiter=maxiter)
    return _run(L, g, case, fuse, diag, nthreads, ilat0, ilat1, state)


def step_fixed_point(case, tol=1e-13, maxiter=60, fuse=True, nthreads=0, ilat0=1, ilat1=None, state=None,
                     with_stage=False):
    """Oracle-C: the fixed point of the reference's pass map (5 passes, then
    Newton on G(x) - x, restarted from earlier pass states and finally by
    pseudo-transient continuation where it does not converge). Returns
    (state, cellstat, cellres[, cellstage]): per chemistry cell (diag layout)
    the Newton steps over all stages (>= 0 when converged, -steps-1 when not),
    the final max |G(x) - x| / max(|x|, 1e-40 hnm), and with with_stage the
    stage that converged (1: from the 5-pass state, 2-5: from the 0/1/2/3-pass
    state, 6: continuation, 0: none)."""
    L = lib()
    nc = case.nlon * case.nlat * case.nivbas
    stat = np.zeros(nc, dtype=np.int32)
    res = np.zeros(nc)
    stage = np.zeros(nc, dtype=np.int32)
    g = grid(case, niter=5, tol=tol, maxiter=maxiter, newton=True, cellstat=stat, cellres=res)
    g.cellstage = stage.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    st, _, _ = _run(L, g, case, fuse, False, nthreads, ilat0, ilat1, state)
    return (st, stat, res, stage) if with_stage else (st, stat, res)


def newton_from(case, qj1, hc, tol=1e-12, maxiter=60, nthreads=0):
    """Oracle-C's Newton (stage 1 alone) started from the given state
    x = (qj1, hc) instead of the 5-pass state: the FP64 fixed point of the
    reference's pass map nearest x. Returns (state, cellstat, cellres) as
    step_fixed_point does; a cell whose iteration converges with a state
    within e of x shows that x lies within e of an exact fixed point."""
    L = lib()
    nc = case.nlon * case.nlat * case.nivbas
    stat = np.zeros(nc, dtype=np.int32)
    res = np.zeros(nc)
    g = grid(case, niter=5, tol=tol, maxiter=maxiter, newton=True, cellstat=stat, cellres=res)
    qx = np.asfortranarray(qj1)
    hx = np.asfortranarray(hc)
    g.x_qj1 = _p(qx)
    g.x_hc = _p(hx)
    st, _, _ = _run(L, g, case, False, False, nthreads, 1, None, None)
    return st, stat, res


def map_residual(case, qj1, hc, nthreads=0):
    """One pass of the reference's map (F:1350-2372) evaluated at the state
    x = (qj1, hc) (mixing ratios; the step's start state still defines ck0 and
    the rates). Returns per chemistry cell (diag layout)
    max_i |G(x)_i - x_i| / max(|x_i|, 1e-20 hnm): zero at a fixed point."""
    L = lib()
    res = np.full(case.nlon * case.nlat * case.nivbas, np.nan)
    g = grid(case, niter=1, cellres=res)
    qx = np.asfortranarray(qj1)
    hx = np.asfortranarray(hc)
    g.x_qj1 = _p(qx)
    g.x_hc = _p(hx)
    _run(L, g, case, False, False, nthreads, 1, None, None)
    return res


def _run(L, g, case, fuse, diag, nthreads, ilat0, ilat1, state):
    st = case.state_copy() if state is None else state
    ilat1 = case.nlat if ilat1 is None else ilat1
    dg = None
    if diag:
        from reprobus_gb300.species import DIAG_COUNT
        dg = np.zeros(DIAG_COUNT * case.nlon * case.nlat * case.nivbas)
    passes = L.orc_step(ctypes.byref(g), ilat0 - 1, ilat1 - 1, case.daynum, case.dt, _p(case.alt),
                        _p(case.trajlon), _p(case.trajlat), _p(case.trajpre), _p(case.trajtem),
                        case.irapp - 1, _p(st["qj1"]), _p(st["hc"]), _p(st["vsed3d"]), _p(st["parth2osed"]),
                        _p(st["parthno3sed"]), _p(st["surfarea"]), _p(st["sza3d"]), int(bool(fuse)),
                        _p(dg) if dg is not None else None, nthreads)
    if dg is not None:
        dg = dg.reshape(DIAG_COUNT, case.nlon * case.nlat * case.nivbas)
    return st, dg, passes


def conserv(case, qj1, hc, ilat0=1, ilat1=None):
    g = grid(case)
    ilat1 = case.nlat if ilat1 is None else ilat1
    lib().orc_conserv(ctypes.byref(g), ilat0 - 1, ilat1 - 1, _p(qj1), _p(hc))


def clamp(case, qj1, ilat0=1, ilat1=None):
    g = grid(case)
    ilat1 = case.nlat if ilat1 is None else ilat1
    lib().orc_clamp(ctypes.byref(g), ilat0 - 1, ilat1 - 1, _p(qj1))


# --------------------------------------------------------------------------- #
# operation counts (op_count.cpp: the same oracle source with a counting type)
# --------------------------------------------------------------------------- #
COUNT_LIB = os.path.join(HERE, "liboracle_count.so")
COUNT_SRC = os.path.join(HERE, "op_count.cpp")
COUNT_CATS = ["add", "mul", "div", "exp", "log", "log10", "pow", "sqrt", "trig", "tanh", "cmp"]


def build_count(force: bool = False) -> str:
    deps = [COUNT_SRC, SRC, os.path.join(HERE, "chem_oracle.h")]
    if force or not os.path.exists(COUNT_LIB) or any(os.path.getmtime(d) > os.path.getmtime(COUNT_LIB)
                                                      for d in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o",
                        COUNT_LIB, COUNT_SRC, "-lm"], check=True)
    return COUNT_LIB


def op_counts(case, rows, niter=5):
    """Operations the reference scheme executes per cell-step, averaged over
    the cells of the given 1-based latitude rows (all lon, levels 1..nivbas).
    Returns a dict: the categories of COUNT_CATS, 'flops' (+-*/) and
    'transcendentals', all per cell."""
    build_count()
    L = ctypes.CDLL(COUNT_LIB)
    dp = ctypes.POINTER(ctypes.c_double)
    L.orc_step.restype = ctypes.c_int
    L.orc_step.argtypes = lib().orc_step.argtypes
    L.orc_count_read.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)]
    g = grid(case, niter=niter)
    st = case.state_copy()
    L.orc_count_reset()
    for r in rows:
        L.orc_step(ctypes.byref(g), r - 1, r - 1, case.daynum, case.dt, _p(case.alt), _p(case.trajlon),
                   _p(case.trajlat), _p(case.trajpre), _p(case.trajtem), case.irapp - 1, _p(st["qj1"]),
                   _p(st["hc"]), _p(st["vsed3d"]), _p(st["parth2osed"]), _p(st["parthno3sed"]), _p(st["surfarea"]),
                   _p(st["sza3d"]), 1, None, 1)
    out = (ctypes.c_ulonglong * len(COUNT_CATS))()
    L.orc_count_read(out)
    ncell = len(rows) * case.nlon * case.nivbas
    res = {k: out[i] / ncell for i, k in enumerate(COUNT_CATS)}
    res["flops"] = res["add"] + res["mul"] + res["div"]
    res["transcendentals"] = sum(res[k] for k in ("exp", "log", "log10", "pow", "sqrt", "trig", "tanh"))
    res["cells"] = ncell
    return res
