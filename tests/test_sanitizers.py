"""AddressSanitizer + UndefinedBehaviorSanitizer runs of the host C/C++ code
that the CPU tests exercise: the chemistry oracle (oracle/chem_oracle.c, the
reference scheme, Oracle-C's Newton with its staged restarts, conserv), the
column oracle (oracle/column_oracle.cpp), the host build of the generated
Newton equations (tests/newton_host.cpp, which includes the same
newton_gen.cuh and newton_solve.cuh as the CUDA kernels) and that of the
rate stage's exponential (tests/exp64_host.cpp, exp64.cuh).

Each library is compiled again with -fsanitize=address,undefined (UBSan
errors fatal) into a temporary folder, and the CPU test files that drive it
run in a child pytest that loads those copies. Any sanitizer report fails
the test."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer", "-g1"]
FILES = ["tests/test_oracle_kat.py", "tests/test_column_oracle.py", "tests/test_newton_equations.py",
         "tests/test_exp64.py", "tests/test_div64.py", "tests/test_log64.py"]


def _runtime(name):
    p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_oracles_and_host_newton_under_asan_and_ubsan(tmp_path):
    asan = _runtime("libasan.so")
    if asan is None or _runtime("libubsan.so") is None:
        pytest.skip("gcc has no sanitizer runtimes here")
    from oracle import column, oracle
    orc = str(tmp_path / "liboracle_san.so")
    col = str(tmp_path / "libcolumn_oracle_san.so")
    subprocess.run(["gcc", "-O1", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
                    *SAN, "-o", orc, oracle.SRC, "-lm"], check=True)
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", *SAN,
                    "-o", col, column.SRC, "-lm"], check=True)
    env = dict(os.environ, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", OMP_NUM_THREADS="4",
               REPROBUS_SANITIZE_FLAGS=" ".join(SAN))
    env[oracle.LIB_OVERRIDE] = orc
    env[column.LIB_OVERRIDE] = col
    # the child loads the sanitized copies, with the ASan runtime
    probe = ("from oracle import column, oracle; oracle.lib(); column.lib(); "
             "print(open('/proc/self/maps').read())")
    maps = subprocess.run([sys.executable, "-c", probe], cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=300).stdout
    assert orc in maps and col in maps and "libasan" in maps
    # (the generator's own check is pure Python and runs in the plain suite)
    r = subprocess.run([sys.executable, "-m", "pytest", *FILES, "-q", "-x", "-m", "not gpu", "-p", "no:cacheprovider",
                        "-k", "not generated_header_is_current"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    out = r.stdout + r.stderr
    assert "AddressSanitizer" not in out and "runtime error:" not in out, out[-4000:]
    assert r.returncode == 0, out[-4000:]
    assert " passed" in r.stdout
