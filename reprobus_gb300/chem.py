"""Python host side of the GB300 chemistry step, over the C-ABI of
libreprobus_gb300.so (include/reprobus_chem.h).

Mirrors the reference's interface for this path:

* ``chem3d(ilat, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp,
  qj1, hc, vsed3d, parth2osed, parthno3sed, surfarea, sza3d)`` — the Fortran
  subroutine of src/reprobus_l137_20230723.f:601-616, same argument names,
  meaning and in-place update of Fortran-ordered FP64 arrays;
* ``conserv(qj1, hc)`` — :2526 (plus the clamps of :431-450);
* ``const()`` — the COMMON /constant/ values of :5927-5948.

``ChemStep`` is the object behind them (one device context, one handle). The
CUDA library is required: every entry point raises ``ReprobusError`` when the
library is missing or the GPU call fails; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .species import DIAG_COUNT

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libreprobus_gb300.so")

FUSE_CONSERV = 0x1
CHECK_FINITE = 0x2
USE_GRAPH = 0x4
SOLVER_REF5, SOLVER_NEWTON64, SOLVER_NEWTON_MIXED = 0, 1, 2

ERRORS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NONFINITE", 4: "ERR_NOCONV", 5: "ERR_TIMEOUT",
          6: "ERR_NODEVICE"}

# every entry point declared in include/reprobus_chem.h
EXPORTS = [
    "reprobus_version", "reprobus_last_error", "reprobus_chem_troe", "reprobus_chem_init",
    "reprobus_chem_free", "reprobus_chem_set_stream", "reprobus_chem_step", "reprobus_chem_step_dev",
    "reprobus_chem_rates_dev", "reprobus_conserv_dev", "reprobus_chem_step_noalloc", "reprobus_chem_set_solver",
    "reprobus_chem_set_tuning", "reprobus_mlp_create", "reprobus_mlp_free", "reprobus_mlp_nparams",
    "reprobus_mlp_set_params", "reprobus_mlp_get_params", "reprobus_mlp_train_step", "reprobus_mlp_grads",
    "reprobus_mlp_forward", "reprobus_chem_set_mlp", "reprobus_chem_features_dev", "reprobus_chem_set_graph",
    "reprobus_sedimentation_dev", "reprobus_tropo_values", "reprobus_forcing_dev", "reprobus_altitude_dev",
    "reprobus_history_write_dev", "reprobus_history_read_dev", "reprobus_mlp_set_wait_limit",
]
NOALLOC_SCRATCH_DOUBLES = 1 << 20


class ReprobusError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("ncells", ctypes.c_longlong), ("nonfinite", ctypes.c_longlong),
                ("kernel_launches", ctypes.c_int), ("passes", ctypes.c_int), ("device_ms", ctypes.c_double),
                ("newton_iters", ctypes.c_longlong), ("fallbacks", ctypes.c_longlong),
                ("max_newton_iters", ctypes.c_int), ("solver", ctypes.c_int),
                ("lanes_per_block", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("z_shared", ctypes.c_int),
                ("warm_start", ctypes.c_int), ("warm_restarts", ctypes.c_longlong),
                ("failed_iters", ctypes.c_longlong), ("solve_ms", ctypes.c_double), ("graph", ctypes.c_int),
                ("start64_cells", ctypes.c_longlong)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def load_library(path: str = LIBPATH):
    """Loads libreprobus_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ReprobusError(6, f"{path} is missing: build it with reprobus_gb300.build.build()")
    lib = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    i, d = ctypes.c_int, ctypes.c_double
    lib.reprobus_version.restype = ctypes.c_char_p
    lib.reprobus_last_error.restype = ctypes.c_char_p
    lib.reprobus_chem_troe.argtypes = [dp]
    lib.reprobus_chem_init.argtypes = [dp, dp, dp, i, i, i, i, i, i, i, i, ctypes.POINTER(vp)]
    lib.reprobus_chem_free.argtypes = [vp]
    lib.reprobus_chem_set_stream.argtypes = [vp, vp]
    lib.reprobus_chem_set_solver.argtypes = [vp, i, i, i, d]
    lib.reprobus_chem_set_tuning.argtypes = [vp, i, i, i]
    step_args = [vp, i, i, d, d, vp, vp, vp, vp, vp, i, vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Stats)]
    lib.reprobus_chem_step.argtypes = step_args
    lib.reprobus_chem_step_dev.argtypes = step_args
    lib.reprobus_chem_rates_dev.argtypes = [vp, i, i, d, vp, vp, vp, vp, vp, i, vp, vp, vp]
    lib.reprobus_conserv_dev.argtypes = [vp, i, i, vp, vp]
    lib.reprobus_chem_step_noalloc.argtypes = [vp, vp, dp, i, i, i, i, i, i, i, i, i, i, d, d, vp, vp, vp, vp, vp,
                                               i, vp, vp, vp, vp, vp, vp, vp, vp]
    fp = ctypes.POINTER(ctypes.c_float)
    lib.reprobus_mlp_create.argtypes = [i, ctypes.c_ulonglong, ctypes.POINTER(vp)]
    lib.reprobus_mlp_free.argtypes = [vp]
    lib.reprobus_mlp_nparams.argtypes = []
    lib.reprobus_mlp_set_params.argtypes = [vp, fp, fp]
    lib.reprobus_mlp_get_params.argtypes = [vp, fp, fp]
    lib.reprobus_mlp_train_step.argtypes = [vp, vp, vp, i, ctypes.c_float, fp, vp]
    lib.reprobus_mlp_grads.argtypes = [vp, vp, vp, i, fp, fp, vp]
    lib.reprobus_mlp_forward.argtypes = [vp, vp, vp, i, vp]
    lib.reprobus_mlp_set_wait_limit.argtypes = [vp, ctypes.c_longlong]
    lib.reprobus_chem_set_mlp.argtypes = [vp, vp]
    lib.reprobus_chem_set_graph.argtypes = [vp, i]
    lib.reprobus_chem_features_dev.argtypes = [vp, i, i, d, d, vp, vp, vp, vp, vp, i, vp, vp, vp]
    lib.reprobus_sedimentation_dev.argtypes = [vp, i, i, vp, vp, i, vp, vp, i, vp, vp, d]
    lib.reprobus_tropo_values.argtypes = [i, i, dp]
    lib.reprobus_forcing_dev.argtypes = [vp, i, i, i, i, d, vp, i, vp, vp, i, vp, vp]
    lib.reprobus_altitude_dev.argtypes = [vp] + [vp] * 9 + [i, vp]
    cp = ctypes.c_char_p
    lib.reprobus_history_write_dev.argtypes = [vp, cp, cp, i, i, i, i, i] + [vp] * 8
    lib.reprobus_history_read_dev.argtypes = [vp, cp, vp, ctypes.POINTER(ctypes.c_int)] + [vp] * 8
    for name in EXPORTS:
        if name not in ("reprobus_version", "reprobus_last_error"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        raise ReprobusError(rc, _lib.reprobus_last_error().decode())


def _hp(a):
    """Host pointer of a Fortran-ordered float64 numpy array."""
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not (a.flags.f_contiguous or a.ndim == 1):
        raise ReprobusError(1, "host arrays must be Fortran-ordered float64 numpy arrays")
    return ctypes.c_void_p(a.ctypes.data)


def _dp(a):
    """Device pointer: an int, or a CUDA tensor/array exposing data_ptr()."""
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    if hasattr(a, "data_ptr"):
        if not getattr(a, "is_cuda", True):
            raise ReprobusError(1, "device entry points need CUDA tensors")
        return ctypes.c_void_p(a.data_ptr())
    raise ReprobusError(1, f"cannot take a device pointer of {type(a)}")


def const():
    """COMMON /constant/ (the 18 fall-off prefactors), :5927-5948."""
    lib = load_library()
    out = np.zeros(18)
    _check(lib.reprobus_chem_troe(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out


class ChemStep:
    """One handle of the GB300 chemistry step for a fixed grid.

    ajl(40,101,27,7), o3up(0:79): COMMON /photodis/; troe: COMMON /constant/
    (defaults to const()). nivbas/nivhau/niter default to the reference's
    94 / 14 / 5 (:627, :2629, :630)."""

    def __init__(self, ajl, o3up, nlon, nlat, niv, nivbas=94, nivhau=14, nrappmax=12, niter=5,
                 flags=FUSE_CONSERV, troe=None):
        lib = load_library()
        troe = const() if troe is None else np.ascontiguousarray(troe, dtype=np.float64)
        ajl = np.asfortranarray(ajl, dtype=np.float64)
        o3up = np.ascontiguousarray(o3up, dtype=np.float64)
        if ajl.shape != (40, 101, 27, 7) or o3up.shape != (80,):
            raise ReprobusError(1, "ajl must be (40,101,27,7) and o3up (80,)")
        h = ctypes.c_void_p()
        dp = ctypes.POINTER(ctypes.c_double)
        _check(lib.reprobus_chem_init(ajl.ctypes.data_as(dp), o3up.ctypes.data_as(dp), troe.ctypes.data_as(dp),
                                      nlon, nlat, niv, nivbas, nivhau, nrappmax, niter, flags, ctypes.byref(h)))
        self._h = h
        self.nlon, self.nlat, self.niv, self.nivbas, self.nivhau = nlon, nlat, niv, nivbas, nivhau
        self.nrappmax, self.niter, self.flags = nrappmax, niter, flags
        self.lib = lib

    @classmethod
    def for_case(cls, case, niter=5, flags=FUSE_CONSERV):
        return cls(case.ajl, case.o3up, case.nlon, case.nlat, case.niv, case.nivbas, case.nivhau,
                   case.nrappmax, niter, flags, case.troe)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.reprobus_chem_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_solver(self, solver, npass=5, maxit=12, tol=1e-4):
        """SOLVER_REF5 (the reference's fixed passes), SOLVER_NEWTON64 or
        SOLVER_NEWTON_MIXED (fixed point of the pass map by Newton)."""
        _check(self.lib.reprobus_chem_set_solver(self._h, solver, npass, maxit, float(tol)))
        self.solver = solver

    def set_tuning(self, lanes_per_block=0, blocks_per_sm=0, zshared=0):
        """Shape of the persistent Newton solve kernel (lanes_per_block 0:
        autotune on the first Newton step of each matrix precision)."""
        _check(self.lib.reprobus_chem_set_tuning(self._h, int(lanes_per_block), int(blocks_per_sm), int(zshared)))

    def set_graph(self, on=True):
        """Launch each step as one CUDA graph (REPROBUS_USE_GRAPH)."""
        _check(self.lib.reprobus_chem_set_graph(self._h, 1 if on else 0))

    def set_mlp(self, net):
        """Attaches a reprobus_gb300.mlp.Mlp to the Newton solvers (None
        detaches): a cell whose plain start misses the convergence test is
        solved again from the network's prediction before it falls back."""
        _check(self.lib.reprobus_chem_set_mlp(self._h, ctypes.c_void_p(net.handle if net is not None else None)))
        self.mlp = net

    def features_dev(self, ilat0, ilat1, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc,
                     feat):
        """The network's 64 raw features of every chemistry cell of the rows
        at the plain start into feat (a CUDA float32 tensor of ncell x 64)."""
        _check(self.lib.reprobus_chem_features_dev(self._h, ilat0, ilat1, daynum, dt, _dp(alt), _dp(trajlon),
                                                   _dp(trajlat), _dp(trajpre), _dp(trajtem), irapp, _dp(qj1),
                                                   _dp(hc), _dp(feat)))

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream, a raw cudaStream_t int, or None."""
        ptr = None if stream is None else (stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))
        _check(self.lib.reprobus_chem_set_stream(self._h, ctypes.c_void_p(ptr)))

    def step(self, ilat0, ilat1, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc, vsed3d,
             parth2osed, parthno3sed, surfarea, sza3d, stats=True):
        """Host-array step for rows ilat0..ilat1 (1-based, inclusive); updates in place."""
        st = Stats() if stats else None
        _check(self.lib.reprobus_chem_step(
            self._h, ilat0, ilat1, float(daynum), float(dt), _hp(alt), _hp(trajlon), _hp(trajlat), _hp(trajpre),
            _hp(trajtem), irapp, _hp(qj1), _hp(hc), _hp(vsed3d), _hp(parth2osed), _hp(parthno3sed), _hp(surfarea),
            _hp(sza3d), ctypes.byref(st) if st is not None else None))
        return st.as_dict() if st is not None else None

    def step_dev(self, ilat0, ilat1, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc, vsed3d,
                 parth2osed, parthno3sed, surfarea, sza3d, stats=False):
        """Device-array step (torch CUDA tensors or raw pointers, Fortran layout).
        Asynchronous on the handle's stream unless stats=True."""
        st = Stats() if stats else None
        _check(self.lib.reprobus_chem_step_dev(
            self._h, ilat0, ilat1, float(daynum), float(dt), _dp(alt), _dp(trajlon), _dp(trajlat), _dp(trajpre),
            _dp(trajtem), irapp, _dp(qj1), _dp(hc), _dp(vsed3d), _dp(parth2osed), _dp(parthno3sed), _dp(surfarea),
            _dp(sza3d), ctypes.byref(st) if st is not None else None))
        return st.as_dict() if st is not None else None

    def rates_dev(self, ilat0, ilat1, daynum, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc, diag):
        _check(self.lib.reprobus_chem_rates_dev(
            self._h, ilat0, ilat1, float(daynum), _dp(alt), _dp(trajlon), _dp(trajlat), _dp(trajpre),
            _dp(trajtem), irapp, _dp(qj1), _dp(hc), _dp(diag)))

    def conserv_dev(self, ilat0, ilat1, qj1, hc):
        _check(self.lib.reprobus_conserv_dev(self._h, ilat0, ilat1, _dp(qj1), _dp(hc)))

    # column physics around the step (device arrays, Fortran layout)
    def sedimentation_dev(self, trajpre, trajtem, irapp, qj1, vsed3d, nivh2oecmwf, parth2osed, parthno3sed,
                          dtsedi, ilat0=1, ilat1=None):
        """subroutine sedimentation (:2416-2522), same arguments, rows ilat0..ilat1."""
        ilat1 = self.nlat if ilat1 is None else ilat1
        _check(self.lib.reprobus_sedimentation_dev(self._h, ilat0, ilat1, _dp(trajpre), _dp(trajtem), irapp,
                                                   _dp(qj1), _dp(vsed3d), int(nivh2oecmwf), _dp(parth2osed),
                                                   _dp(parthno3sed), float(dtsedi)))

    def forcing_dev(self, ian, imois, dt, trajpre, irapp, qj1, hc, co_month=None, hj1=None, nivh2oecmwf=59,
                    ilat0=1, ilat1=None):
        """tropo (:4077-4574), then co_tropo (:4577-4639) when co_month (the
        month's CO field, nlon x nlat) is given and ecmwfh2o (:8621-8658) when
        hj1 (the humidity field) is given."""
        ilat1 = self.nlat if ilat1 is None else ilat1
        _check(self.lib.reprobus_forcing_dev(self._h, ilat0, ilat1, int(ian), int(imois), float(dt), _dp(trajpre),
                                             irapp, _dp(co_month) if co_month is not None else None,
                                             _dp(hj1) if hj1 is not None else None, int(nivh2oecmwf), _dp(qj1),
                                             _dp(hc)))

    def altitude_dev(self, relief, psol, aaa, bbb, t, h2o, trajlon, trajlat, trajpre, alt, irapp=1):
        """subroutine altitude (altitude.f90:1-148) on slice irapp of the trajectories."""
        _check(self.lib.reprobus_altitude_dev(self._h, _dp(relief), _dp(psol), _dp(aaa), _dp(bbb), _dp(t), _dp(h2o),
                                              _dp(trajlon), _dp(trajlat), _dp(trajpre), irapp, _dp(alt)))

    def history_write_dev(self, path, namexp, date, pj1, uj1, vj1, alt, tj1, qj1, surfarea, hc):
        """write(78) of the history record (:587-588); date = (ian, imois, ijour, iheure, imin)."""
        ian, imois, ijour, iheure, imin = (int(x) for x in date)
        _check(self.lib.reprobus_history_write_dev(self._h, os.fsencode(path), namexp.encode()[:6], ian, imois, ijour,
                                                   iheure, imin, _dp(pj1), _dp(uj1), _dp(vj1), _dp(alt), _dp(tj1),
                                                   _dp(qj1), _dp(surfarea), _dp(hc)))

    def history_read_dev(self, path, pj1, uj1, vj1, alt, tj1, qj1, surfarea, hc):
        """read(90) of a history/restart record (:231-235) into device arrays;
        returns (namexp, (ian, imois, ijour, iheure, imin))."""
        name = ctypes.create_string_buffer(7)
        date = (ctypes.c_int * 5)()
        _check(self.lib.reprobus_history_read_dev(self._h, os.fsencode(path), name, date, _dp(pj1), _dp(uj1),
                                                  _dp(vj1), _dp(alt), _dp(tj1), _dp(qj1), _dp(surfarea), _dp(hc)))
        return name.value.decode(), tuple(date)


def tropo_values(ian, imois):
    """The 16 forcing mixing ratios tropo imposes below nivbas for the date
    (:4414-4495), ordered as the qj1 slots 1 2 4 7 31..42."""
    lib = load_library()
    out = np.zeros(16)
    _check(lib.reprobus_tropo_values(int(ian), int(imois), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out


def step_noalloc(ajl, o3up, troe, nlon, nlat, niv, nivbas, nivhau, nrappmax, niter, flags, ilat0, ilat1,
                 daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc, vsed3d, parth2osed,
                 parthno3sed, surfarea, sza3d, stream=None):
    """reprobus_chem_step_noalloc: the step with no device allocation (no
    handle). ajl/o3up and every array are DEVICE arrays (torch CUDA tensors or
    pointers); troe is a host sequence of 18 values. For callers that may not
    allocate device memory; see include/reprobus_chem.h for the scratch limit."""
    lib = load_library()
    tr = np.ascontiguousarray(troe, dtype=np.float64)
    sp = None if stream is None else (stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))
    _check(lib.reprobus_chem_step_noalloc(
        _dp(ajl), _dp(o3up), tr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nlon, nlat, niv, nivbas, nivhau,
        nrappmax, niter, flags, ilat0, ilat1, float(daynum), float(dt), _dp(alt), _dp(trajlon), _dp(trajlat),
        _dp(trajpre), _dp(trajtem), irapp, _dp(qj1), _dp(hc), _dp(vsed3d), _dp(parth2osed), _dp(parthno3sed),
        _dp(surfarea), _dp(sza3d), ctypes.c_void_p(sp)))


# --------------------------------------------------------------------------- #
# reference-shaped module interface
# --------------------------------------------------------------------------- #
_default: ChemStep | None = None


def init(ajl, o3up, nlon=180, nlat=91, niv=137, nivbas=94, nivhau=14, nrappmax=12, niter=5,
         flags=FUSE_CONSERV):
    """Plays the role of call const(relief) (:294): fills the GPU copies of
    COMMON /constant/ and /photodis/ for the module-level chem3d()."""
    global _default
    if _default is not None:
        _default.close()
    _default = ChemStep(ajl, o3up, nlon, nlat, niv, nivbas, nivhau, nrappmax, niter, flags & ~FUSE_CONSERV)
    return _default


def chem3d(ilat, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc, vsed3d, parth2osed,
           parthno3sed, surfarea, sza3d):
    """subroutine chem3d (:601-616): one latitude row, arrays updated in place."""
    if _default is None:
        raise ReprobusError(1, "call init(ajl, o3up, ...) first (the role of const)")
    _default.step(ilat, ilat, daynum, dt, alt, trajlon, trajlat, trajpre, trajtem, irapp, qj1, hc, vsed3d,
                  parth2osed, parthno3sed, surfarea, sza3d, stats=False)


def conserv(qj1, hc):
    """subroutine conserv (:2526) followed by the clamps of :431-450, on the GPU."""
    if _default is None:
        raise ReprobusError(1, "call init(ajl, o3up, ...) first")
    import torch
    q = torch.from_numpy(np.ascontiguousarray(qj1.reshape(-1, order="F"))).cuda()
    h = torch.from_numpy(np.ascontiguousarray(hc.reshape(-1, order="F"))).cuda()
    _default.conserv_dev(1, _default.nlat, q, h)
    qj1.reshape(-1, order="F")[:] = q.cpu().numpy()
    hc.reshape(-1, order="F")[:] = h.cpu().numpy()
