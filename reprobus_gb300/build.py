"""Builds the in-tree CUDA library libreprobus_gb300.so for sm_103a.

nvcc compiles each translation unit for compute_103a/sm_103a only; host code is
compiled with -ffp-contract=off so that the host-side per-step constants round
exactly as written on both x86_64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libreprobus_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["chem_kernels.cu", "nt_solve_f32_zr.cu", "nt_solve_f32_zs.cu", "nt_solve_f64_zr.cu",
           "nt_solve_f64_zs.cu", "nt_solve_pp.cu", "nt_solve_sp.cu", "nt_solve_ls.cu", "nt_solve_wc.cu", "mlp_kernels.cu",
           "column_kernels.cu"]
HEADERS = ["chem_cell.cuh", "chem_enums.h", "chem_params.cuh", "newton_gen.cuh", "newton_solve.cuh",
           "newton_kernel.cuh", "newton_launch.h", "newton_num.cuh", "tc_sm100.cuh", "handle_info.h",
           "tropo_tables.h", "exp64.cuh", "exp_table.h", "div64.cuh", "log64.cuh", "log_table.h", "mlp_net.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-diag-suppress", "550"]
if os.environ.get("REPROBUS_FMAD", "1") == "0":
    # strict IEEE variant (no FMA contraction) for parity studies
    NVFLAGS += ["--fmad=false"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libreprobus_gb300.so")
    return cand


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    include = os.path.join(os.path.dirname(HERE), "include", "reprobus_chem.h")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [include]
    objs, jobs = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs]):
            jobs.append([nvcc(), *ARCH, *NVFLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
