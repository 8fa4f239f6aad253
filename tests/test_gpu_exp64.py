"""exp64 (reprobus_gb300/csrc/exp64.cuh) on the GPU: the device code gives
bit for bit the host build's results (whose error tests/test_exp64.py bounds
against long double), and stays within 2 ulp of CUDA's exp."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def libs(tmp_path_factory):
    d = tmp_path_factory.mktemp("exp64")
    dev, host = str(d / "libexp64_dev.so"), str(d / "libexp64_host.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-o", dev, os.path.join(ROOT, "tests", "exp64_dev.cu")], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", host,
                    os.path.join(ROOT, "tests", "exp64_host.cpp")], check=True)
    D, H = ctypes.CDLL(dev), ctypes.CDLL(host)
    D.exp64_dev.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long]
    H.exp64_many.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_long]
    return D, H


def test_device_equals_host_build_and_cuda_exp(libs):
    D, H = libs
    rng = np.random.default_rng(11)
    L = np.log(2.0) / 512
    k = np.arange(-47000, 47000, 3, dtype=np.float64)
    y = np.concatenate([rng.uniform(-64.0, 64.0, 4_000_000), rng.uniform(-1e-3, 1e-3, 100_000), (k + 0.5) * L,
                        k * L, np.array([0.0, -0.0, 1e-300, 64.0, -64.0, 300.0, -800.0, np.inf, -np.inf, np.nan])])
    a, b, h = np.empty_like(y), np.empty_like(y), np.empty_like(y)
    assert D.exp64_dev(y.ctypes.data, a.ctypes.data, b.ctypes.data, y.size) == 0
    H.exp64_many(y.ctypes.data, h.ctypes.data, y.size)
    fast = np.abs(y) < 64.0
    assert np.array_equal(a[fast], h[fast])  # bitwise
    ok = np.isfinite(b) & (b > 0)
    ulp = np.abs(a[ok] - b[ok]) / np.spacing(b[ok])
    print(f"exp64 vs CUDA exp: max {ulp.max():.2f} ulp, mean {ulp.mean():.3f} ulp")
    assert ulp.max() <= 2.0
    assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~fast & ~np.isnan(a)], b[~fast & ~np.isnan(b)])
