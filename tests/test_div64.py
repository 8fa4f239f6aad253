"""CPU checks of div64 and sqrt64 (reprobus_gb300/csrc/div64.cuh), the rate
stage's FP64 quotients and square roots, through their host build
(tests/div64_host.cpp): against the IEEE quotient over random operands of
the chemistry's magnitudes (1e-40 .. 1e30), unit-range operands, and the
operands that take the IEEE division (zero, subnormal, huge, inf, nan)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("div64") / "libdiv64.so")
    extra = os.environ.get("REPROBUS_SANITIZE_FLAGS", "").split()  # set by test_sanitizers.py
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", *extra, "-o", out,
                    os.path.join(ROOT, "tests", "div64_host.cpp")], check=True)
    L = ctypes.CDLL(out)
    L.div64_many.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long]
    L.sqrt64_many.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_long]
    return L


def _div64(L, a, b):
    a, b = (np.ascontiguousarray(v, dtype=np.float64) for v in (a, b))
    out = np.empty_like(a)
    L.div64_many(a.ctypes.data, b.ctypes.data, out.ctypes.data, a.size)
    return out


def test_quotients_are_the_ieee_ones_within_an_ulp(lib):
    rng = np.random.default_rng(3)
    n = 2_000_000
    a = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-40, 30, n)
    b = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-40, 30, n)
    u = rng.uniform(0.5, 2.0, (2, n))
    a, b = np.concatenate([a, u[0]]), np.concatenate([b, u[1]])
    got, want = _div64(lib, a, b), a / b
    ulp = np.abs(got - want) / np.spacing(np.abs(want))
    print(f"max {ulp.max():.2f} ulp; {np.mean(got != want):.2e} of the quotients differ from IEEE")
    assert ulp.max() <= 1.0
    assert np.mean(got != want) < 1e-4


def test_operands_outside_the_range_take_the_ieee_division(lib):
    a = np.array([0.0, -0.0, 1.0, 1.0, 5e-324, 1e300, 1.0, np.inf, np.nan, 1.0, 1e-300, 3.0])
    b = np.array([2.0, 2.0, 0.0, 5e-324, 1.0, 1e-300, np.inf, 2.0, 2.0, np.nan, 1e300, 1e-310])
    with np.errstate(all="ignore"):
        want = a / b
    got = _div64(lib, a, b)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.array_equal(got[ok], want[ok])


def test_square_roots_are_the_ieee_ones_within_an_ulp(lib):
    rng = np.random.default_rng(4)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 1_000_000), rng.uniform(0.25, 4.0, 1_000_000),
                        np.array([0.0, -0.0, -1.0, 5e-324, 1e-310, np.inf, np.nan, 1.0, 4.0, 2.0])])
    x = np.ascontiguousarray(x)
    got = np.empty_like(x)
    lib.sqrt64_many(x.ctypes.data, got.ctypes.data, x.size)
    with np.errstate(invalid="ignore"):
        want = np.sqrt(x)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    fin = np.isfinite(want) & (want > 0)
    ulp = np.abs(got[fin] - want[fin]) / np.spacing(want[fin])
    print(f"sqrt64: max {ulp.max():.2f} ulp; {np.mean(got[fin] != want[fin]):.2e} differ from IEEE")
    assert ulp.max() <= 1.0 and np.mean(got[fin] != want[fin]) < 1e-4
    rest = ~fin & ~np.isnan(want)
    assert np.array_equal(got[rest], want[rest])
