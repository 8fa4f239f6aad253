"""ctypes front end of the CPU FP64 oracle of the column physics
(column_oracle.cpp): sedimentation, tropospheric forcing, altitude.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA
kernels of reprobus_gb300/csrc/column_kernels.cu, never as the measured or
shipped path. PARITY UNPINNED: see column_oracle.cpp.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libcolumn_oracle.so")
SRC = os.path.join(HERE, "column_oracle.cpp")
LIB_OVERRIDE = "REPROBUS_COLUMN_ORACLE_LIB"  # a prebuilt copy to load instead
DEPS = [SRC, os.path.join(HERE, "..", "reprobus_gb300", "csrc", "tropo_tables.h")]


def build(force: bool = False) -> str:
    """Compiles the column oracle with g++ (IEEE, no FMA contraction)."""
    if force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in DEPS):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                        "-o", LIB, SRC, "-lm"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.environ.get(LIB_OVERRIDE)
        if not path:
            path = build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        i, d = ctypes.c_int, ctypes.c_double
        L.orc_sedimentation.argtypes = [i, i, i, i, i, i, i, dp, dp, dp, dp, i, dp, dp, d]
        L.orc_tropo_values.argtypes = [i, i, dp]
        L.orc_tropo_values.restype = i
        L.orc_forcing.argtypes = [i, i, i, i, i, i, dp, d, dp, dp, dp, i, dp, dp]
        L.orc_altitude.argtypes = [i, i, i] + [dp] * 11 + [ctypes.POINTER(ctypes.c_int)]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def sedimentation(nivbas, nivhau, pre, tem, qj1, vsed, nivh2o, ph2o, pno3, dt, ilat0=1, ilat1=None):
    """sedimentation (F:2416-2522) in place on qj1; pre/tem: one trajectory slice."""
    nlon, nlat, niv = pre.shape
    ilat1 = nlat if ilat1 is None else ilat1
    lib().orc_sedimentation(nlon, nlat, niv, nivbas, nivhau, ilat0, ilat1, _p(pre), _p(tem), _p(qj1), _p(vsed),
                            nivh2o, _p(ph2o), _p(pno3), float(dt))


def tropo_values(ian, imois):
    v = np.zeros(16)
    if lib().orc_tropo_values(int(ian), int(imois), _p(v)) != 0:
        raise ValueError(f"date {ian}/{imois} outside the forcing tables")
    return v


def forcing(nivbas, ian, imois, dt, pre, qj1, hc, co=None, hj1=None, nivh2o=59, ilat0=1, ilat1=None):
    """tropo + co_tropo + ecmwfh2o (F:4498-4571, 4617-4636, 8649-8655) in place."""
    nlon, nlat, niv = pre.shape
    ilat1 = nlat if ilat1 is None else ilat1
    v = tropo_values(ian, imois)
    lib().orc_forcing(nlon, nlat, niv, nivbas, ilat0, ilat1, _p(v), float(dt), _p(pre), _p(co), _p(hj1), nivh2o,
                      _p(qj1), _p(hc))


def altitude(relief, psol, aaa, bbb, t, h2o, trajlon, trajlat, trajpre):
    """altitude (altitude.f90:1-148); returns alt (nlon, nlat, niv)."""
    nlon, nlat, niv = t.shape
    alt = np.zeros((nlon, nlat, niv), order="F")
    work = np.zeros(3 * nlon * nlat * niv)
    iwork = np.zeros(3 * nlon * nlat * niv, dtype=np.int32)
    lib().orc_altitude(nlon, nlat, niv, _p(relief), _p(psol), _p(np.ascontiguousarray(aaa)),
                       _p(np.ascontiguousarray(bbb)), _p(t), _p(h2o), _p(trajlon), _p(trajlat), _p(trajpre),
                       _p(alt), _p(work), iwork.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return alt
