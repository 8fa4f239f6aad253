"""CPU checks of exp64 (reprobus_gb300/csrc/exp64.cuh), the table-driven
exponential of the rate stage, through its host build (tests/exp64_host.cpp):
the error against the exponential in long double (64-bit mantissa on x86,
128-bit on Arm; at least 11 bits beyond double) over the fast range
|y| < 64, densely and at the reduction's boundaries, the Arrhenius and Troe
arguments of the rate stage, and the fallback outside that range. The
generated table header must be current."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAX_ULP = 1.5


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("exp64") / "libexp64.so")
    extra = os.environ.get("REPROBUS_SANITIZE_FLAGS", "").split()  # set by test_sanitizers.py
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", *extra, "-o", out,
                    os.path.join(ROOT, "tests", "exp64_host.cpp")], check=True)
    L = ctypes.CDLL(out)
    L.exp64_many.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
    return L


def _exp64(L, y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.empty_like(y)
    L.exp64_many(y.ctypes.data, out.ctypes.data, y.size)
    return out


def _ulp_err(got, y):
    if np.finfo(np.longdouble).nmant < 63:
        pytest.skip("long double is no wider than double here")
    ref = np.exp(y.astype(np.longdouble))
    return (np.abs(got.astype(np.longdouble) - ref) / np.spacing(ref.astype(np.float64)).astype(np.longdouble)).astype(
        np.float64)


def test_fast_range_dense_and_at_the_reduction_boundaries(lib):
    rng = np.random.default_rng(7)
    y = np.concatenate([rng.uniform(-64.0, 64.0, 2_000_000), rng.uniform(-1e-3, 1e-3, 200_000),
                        np.array([0.0, -0.0, 1e-300, -1e-300, 5e-324, 63.999999, -63.999999])])
    L = np.log(2.0) / 512
    k = np.arange(-47000, 47000, 7, dtype=np.float64)
    y = np.concatenate([y, (k + 0.5) * L, (k + 0.5) * L * (1 + 1e-15), (k + 0.5) * L * (1 - 1e-15), k * L])
    y = y[np.abs(y) < 64.0]
    e = _ulp_err(_exp64(lib, y), y)
    print(f"max error {e.max():.3f} ulp, mean {e.mean():.3f} ulp over {y.size} arguments")
    assert e.max() <= MAX_ULP


def test_rate_stage_arguments(lib):
    # Arrhenius E / T and Troe n ln T over the temperatures of the grid
    T = np.linspace(150.0, 330.0, 20001)
    E = np.array([60, -470, 180, -940, -490, 200, 250, -1800, 270, 19, 920, 210, -1500, 100, -3600, -2450, 10900,
                  2199, 1335, 460, 380, 11000, 20, -1775, 300, 800, 125, -1600, -30, 390, -900, -115, -800, -200,
                  85, 290, -1280, -2270, 269, 230, -375, -250, -840, -500, -130, 8649, -1590, -1520, -1250, -780,
                  260, 550, -310, 215, -430, -1300, -2060, 110, 55], dtype=np.float64)
    n = np.array([-1.3, 0.2, -4.4, -0.7, -3.0, -3.4, -1.1, -3.6, 1.1, -3.4, -1.9, -2.0, -1.0, -4.5, -3.2, -2.9])
    y = np.concatenate([(E[:, None] * (1.0 / T)[None, :]).ravel(), (n[:, None] * np.log(T)[None, :]).ravel()])
    e = _ulp_err(_exp64(lib, y), y)
    assert e.max() <= MAX_ULP


def test_outside_the_fast_range_it_is_exp(lib):
    y = np.array([64.0, -64.0, 100.0, -700.0, 709.0, 710.0, -745.0, -745.13, -745.14, -745.2, -745.21, -746.0,
                  -1e4, -2.7e6, np.inf, -np.inf, np.nan])
    got = _exp64(lib, y)
    with np.errstate(over="ignore"):
        want = np.exp(y)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.allclose(got[ok], want[ok], rtol=2.5e-16, atol=0.0)


def test_generated_table_is_current():
    from reprobus_gb300.codegen import gen_exp_table
    with open(gen_exp_table.OUT) as f:
        assert f.read() == gen_exp_table.render()
