"""CPU checks of log64 (reprobus_gb300/csrc/log64.cuh), the table-driven
logarithm of the rate stage, through its host build (tests/log64_host.cpp):
the error against the logarithm in long double over positive normals of
every magnitude, densely near 1 (where the result is small) and at the
table's breakpoints, the rate stage's arguments, and the arguments that take
the library log. The generated table header must be current."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAX_ULP = 2.0  # measured: 0.5 ulp but for x just below 1 (hi and p cancel), 1.6 ulp there


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("log64") / "liblog64.so")
    extra = os.environ.get("REPROBUS_SANITIZE_FLAGS", "").split()  # set by test_sanitizers.py
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", *extra, "-o", out,
                    os.path.join(ROOT, "tests", "log64_host.cpp")], check=True)
    L = ctypes.CDLL(out)
    L.log64_many.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
    return L


def _log64(L, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    L.log64_many(x.ctypes.data, out.ctypes.data, x.size)
    return out


def _ulp_err(got, x):
    if np.finfo(np.longdouble).nmant < 63:
        pytest.skip("long double is no wider than double here")
    ref = np.log(x.astype(np.longdouble))
    return (np.abs(got.astype(np.longdouble) - ref) /
            np.spacing(np.abs(ref.astype(np.float64))).astype(np.longdouble)).astype(np.float64)


def test_positive_normals_near_one_and_at_the_breakpoints(lib):
    rng = np.random.default_rng(9)
    x = np.concatenate([10.0 ** rng.uniform(-307, 307, 1_500_000), rng.uniform(0.5, 2.0, 1_000_000),
                        1.0 + rng.uniform(-1e-3, 1e-3, 300_000), 1.0 + rng.uniform(-1e-9, 1e-9, 100_000)])
    j = np.arange(257)
    F = 1.0 + j / 256.0
    half = 1.0 + (j[:-1] + 0.5) / 256.0
    x = np.concatenate([x, F, F * (1 + 2e-16), half, np.nextafter(half, 0), np.nextafter(half, 3), F * 2.0 ** 37,
                        half * 2.0 ** -41, [1.0, 2.0, 0.5, 2.2250738585072014e-308, 1.7976931348623157e308]])
    x = x[x != 1.0]  # ln 1 = 0: checked exactly below
    e = _ulp_err(_log64(lib, x), x)
    print(f"max error {e.max():.3f} ulp, mean {e.mean():.3f} ulp over {x.size} arguments")
    assert e.max() <= MAX_ULP
    assert _log64(lib, np.array([1.0]))[0] == 0.0


def test_rate_stage_arguments(lib):
    # temperatures, number densities, partial pressures, water activities, weight fractions
    x = np.concatenate([np.linspace(150.0, 330.0, 20001), 10.0 ** np.linspace(12, 20, 20001),
                        10.0 ** np.linspace(-12, -2, 20001), np.linspace(1e-4, 1.0, 20001),
                        np.linspace(0.005, 100.0, 20001)])
    assert _ulp_err(_log64(lib, x), x).max() <= MAX_ULP


def test_other_arguments_take_the_library_log(lib):
    x = np.array([0.0, -0.0, -1.0, 5e-324, 1e-310, np.inf, -np.inf, np.nan])
    got = _log64(lib, x)
    with np.errstate(all="ignore"):
        want = np.log(x)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.allclose(got[ok], want[ok], rtol=2.5e-16, atol=0.0)


def test_generated_table_is_current():
    from reprobus_gb300.codegen import gen_log_table
    with open(gen_log_table.OUT) as f:
        assert f.read() == gen_log_table.render()
