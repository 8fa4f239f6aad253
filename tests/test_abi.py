"""The C-ABI library loads and exports every entry point include/*.h declares;
host-only entry points work without a GPU; compute entry points fail loudly
(an error code, no CPU fallback) where no GPU is visible."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(reprobus_\w+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "reprobus_chem_step" in names and "reprobus_chem_init" in names
    from reprobus_gb300.chem import EXPORTS
    assert set(EXPORTS) <= set(names)


def test_library_exports_every_declared_symbol(lib_built):
    lib = ctypes.CDLL(lib_built)
    missing = [n for n in declared_entry_points() if not hasattr(lib, n)]
    assert not missing, missing


def test_troe_host_entry_matches_oracle(lib_built):
    from oracle import oracle
    from reprobus_gb300 import chem
    assert np.array_equal(chem.const(), oracle.troe())


def test_version_string(lib_built):
    from reprobus_gb300 import chem
    lib = chem.load_library()
    assert b"sm_103a" in lib.reprobus_version()


def test_bad_arguments_are_rejected(lib_built):
    from reprobus_gb300 import chem
    lib = chem.load_library()
    h = ctypes.c_void_p()
    rc = lib.reprobus_chem_init(None, None, None, 1, 1, 1, 1, 1, 1, 5, 0, ctypes.byref(h))
    assert rc == 1 and b"non-NULL" in lib.reprobus_last_error()
    z = np.zeros(40 * 101 * 27 * 7)
    o = np.zeros(80)
    t = chem.const()
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.reprobus_chem_init(z.ctypes.data_as(dp), o.ctypes.data_as(dp), t.ctypes.data_as(dp), 10, 5, 137,
                                140, 14, 1, 5, 0, ctypes.byref(h))
    assert rc == 1 and b"nivbas" in lib.reprobus_last_error()
    # Troe prefactors must be positive and finite (the rate stage takes their logarithms)
    for bad in (0.0, -1e-30, np.nan, np.inf):
        tb = t.copy()
        tb[5] = bad
        rc = lib.reprobus_chem_init(z.ctypes.data_as(dp), o.ctypes.data_as(dp), tb.ctypes.data_as(dp), 10, 5, 137,
                                    94, 14, 1, 5, 0, ctypes.byref(h))
        assert rc == 1 and b"troe[5]" in lib.reprobus_last_error(), bad
    assert lib.reprobus_chem_step(None, 1, 1, 0., 0., *([None] * 5), 1, *([None] * 7), None) == 1


def test_no_gpu_means_error_not_fallback(lib_built):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from reprobus_gb300 import chem, inputs
    c = inputs.make_case("cfg0", seed=1, nlon=4, nivbas=94)
    with pytest.raises(chem.ReprobusError) as ei:
        chem.ChemStep.for_case(c)
    assert ei.value.code in (2, 6)
