"""div64 and sqrt64 (reprobus_gb300/csrc/div64.cuh) on the GPU, from the
hardware's reciprocal (square root) estimates: within one ulp of the IEEE
quotient (square root) and equal to it but for rare operands, over the
chemistry's magnitudes."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_device_quotients_match_ieee(tmp_path):
    so = str(tmp_path / "libdiv64_dev.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-o", so, os.path.join(ROOT, "tests", "div64_dev.cu")], check=True)
    L = ctypes.CDLL(so)
    L.div64_dev.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_long]
    rng = np.random.default_rng(5)
    n = 4_000_000
    a = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-40, 30, n)
    b = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-40, 30, n)
    a = np.concatenate([a, rng.uniform(0.5, 2.0, n), [0.0, 1.0, 1.0, np.inf, np.nan]])
    b = np.concatenate([b, rng.uniform(0.5, 2.0, n), [2.0, 0.0, 1e-310, 2.0, 2.0]])
    q, ieee = np.empty_like(a), np.empty_like(a)
    assert L.div64_dev(a.ctypes.data, b.ctypes.data, q.ctypes.data, ieee.ctypes.data, a.size) == 0
    fin = np.isfinite(ieee) & (ieee != 0)
    ulp = np.abs(q[fin] - ieee[fin]) / np.spacing(np.abs(ieee[fin]))
    print(f"max {ulp.max():.2f} ulp; {np.mean(q[fin] != ieee[fin]):.2e} differ")
    assert ulp.max() <= 1.0 and np.mean(q[fin] != ieee[fin]) < 1e-4
    assert np.array_equal(np.isnan(q), np.isnan(ieee))
    assert np.array_equal(q[~fin & ~np.isnan(q)], ieee[~fin & ~np.isnan(ieee)])


def test_device_square_roots_match_ieee(tmp_path):
    so = str(tmp_path / "libdiv64_dev.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-o", so, os.path.join(ROOT, "tests", "div64_dev.cu")], check=True)
    L = ctypes.CDLL(so)
    L.sqrt64_dev.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long]
    rng = np.random.default_rng(6)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 3_000_000), rng.uniform(0.25, 4.0, 1_000_000),
                        np.array([0.0, -1.0, 1e-310, np.inf, np.nan, 1.0, 4.0])])
    q, ieee = np.empty_like(x), np.empty_like(x)
    assert L.sqrt64_dev(x.ctypes.data, q.ctypes.data, ieee.ctypes.data, x.size) == 0
    fin = np.isfinite(ieee) & (ieee > 0)
    ulp = np.abs(q[fin] - ieee[fin]) / np.spacing(ieee[fin])
    print(f"sqrt64: max {ulp.max():.2f} ulp; {np.mean(q[fin] != ieee[fin]):.2e} differ")
    assert ulp.max() <= 1.0 and np.mean(q[fin] != ieee[fin]) < 1e-4
    assert np.array_equal(np.isnan(q), np.isnan(ieee))


def test_generated_equation_quotients(tmp_path):
    """nt_div<double> (no range test) equals the IEEE quotient to one ulp over
    the chemistry's magnitudes and gives NaN for a zero divisor; nt_div<float>
    is within 2 ulp and nt_rcp<float> within 1 ulp of the exact quotient (2.5
    and 1.5 ulp of its FP32 rounding)."""
    so = str(tmp_path / "libnt_div_dev.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-o", so, os.path.join(ROOT, "tests", "nt_div_dev.cu")], check=True)
    L = ctypes.CDLL(so)
    L.nt_div_dev.argtypes = [ctypes.c_void_p] * 8 + [ctypes.c_long]
    rng = np.random.default_rng(7)
    n = 2_000_000
    a = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-40, 30, n)
    b = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-40, 30, n)
    a = np.concatenate([a, rng.uniform(0.5, 2.0, n), [1.0, 0.0]])
    b = np.concatenate([b, rng.uniform(0.5, 2.0, n), [0.0, 3.0]])
    m = a.size
    af = (rng.choice([-1.0, 1.0], m) * 10.0 ** rng.uniform(-15, 15, m)).astype(np.float32)
    bf = (rng.choice([-1.0, 1.0], m) * 10.0 ** rng.uniform(-15, 15, m)).astype(np.float32)
    qd, ieee = np.empty_like(a), np.empty_like(a)
    qf, rf = np.empty_like(af), np.empty_like(af)
    assert L.nt_div_dev(a.ctypes.data, b.ctypes.data, af.ctypes.data, bf.ctypes.data, qd.ctypes.data,
                        ieee.ctypes.data, qf.ctypes.data, rf.ctypes.data, m) == 0
    fin = np.isfinite(ieee) & (ieee != 0)
    fin[-2:] = False
    ulp = np.abs(qd[fin] - ieee[fin]) / np.spacing(np.abs(ieee[fin]))
    print(f"nt_div<double>: max {ulp.max():.2f} ulp; {np.mean(qd[fin] != ieee[fin]):.2e} differ")
    assert ulp.max() <= 1.0 and np.mean(qd[fin] != ieee[fin]) < 1e-4
    assert np.isnan(qd[-2]) and qd[-1] == 0.0  # 1 / 0 -> NaN (the cell fails); 0 / 3 -> 0
    ref = (af.astype(np.float64) / bf.astype(np.float64)).astype(np.float32)
    ulpf = np.abs(qf.astype(np.float64) - ref) / np.spacing(np.abs(ref)).astype(np.float64)
    rref = (1.0 / bf.astype(np.float64)).astype(np.float32)
    ulpr = np.abs(rf.astype(np.float64) - rref) / np.spacing(np.abs(rref)).astype(np.float64)
    print(f"nt_div<float>: max {ulpf.max():.2f} ulp; nt_rcp<float>: max {ulpr.max():.2f} ulp")
    assert ulpf.max() <= 2.5 and ulpr.max() <= 1.5
