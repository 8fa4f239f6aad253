"""Generates reprobus_gb300/csrc/exp_table.h: the constants of the table-driven
exponential exp64 (exp64.cuh), computed with Python's decimal module at 60
significant digits and rounded once to double (or float) precision.

Method (P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989), with
N = 512 table entries: y = k L + r, L = ln 2 / 512, k an integer,
exp(y) = 2^(k >> 9) 2^((k & 511) / 512) exp(r).

  EXP64_TAB[j]   2^(j / 512), j = 0..511, correctly rounded doubles
  EXP64_L1       L rounded to 37 significant bits: k L1 is exact for |k| < 2^16
  EXP64_L2F      L - L1 rounded to float
  EXP64_INVF     512 / ln 2 rounded to float (picks k, within 0.01 of y / L)

    python -m reprobus_gb300.codegen.gen_exp_table
"""
from __future__ import annotations

import decimal
import os
import struct

import numpy as np

N = 512
L1_BITS = 37
OUT = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "csrc", "exp_table.h")


def _ctx():
    c = decimal.Context(prec=60)
    return c


def constants():
    c = _ctx()
    ln2 = c.ln(decimal.Decimal(2))
    L = c.divide(ln2, N)
    tab = [float(c.exp(c.multiply(L, j))) for j in range(N)]  # float(Decimal) rounds correctly
    # L1: the double nearest L with its 53 - L1_BITS low mantissa bits cleared
    b = struct.unpack("<Q", struct.pack("<d", float(L)))[0]
    b &= ~((1 << (53 - L1_BITS)) - 1)
    l1 = struct.unpack("<d", struct.pack("<Q", b))[0]
    l2 = float(c.subtract(L, decimal.Decimal(l1)))
    l2f = float(np.float32(l2))
    invf = float(np.float32(float(c.divide(N, ln2))))
    return tab, l1, l2f, invf


def render():
    tab, l1, l2f, invf = constants()
    lines = [
        "// exp_table.h — constants of the table-driven exponential exp64 (exp64.cuh).",
        "// Generated by reprobus_gb300/codegen/gen_exp_table.py; do not edit.",
        "#pragma once",
        "",
        "namespace rpb {",
        "",
        f"constexpr int EXP64_N = {N};",
        f"constexpr double EXP64_L1 = {l1.hex()};  // ln 2 / {N}, {L1_BITS} significant bits",
        f"constexpr float EXP64_L2F = {float(l2f).hex()}f;  // ln 2 / {N} - EXP64_L1",
        f"constexpr float EXP64_INVF = {float(invf).hex()}f;  // {N} / ln 2",
        "",
        "#ifdef __CUDACC__",
        "#define EXP64_TABLE static __device__ const",
        "#else",
        "#define EXP64_TABLE static const",
        "#endif",
        f"// 2^(j / {N}), j = 0..{N - 1}",
        f"EXP64_TABLE double EXP64_TAB[{N}] = {{",
    ]
    for i in range(0, N, 4):
        lines.append("    " + ", ".join(t.hex() for t in tab[i:i + 4]) + ",")
    lines += ["};", "#undef EXP64_TABLE", "", "}  // namespace rpb", ""]
    return "\n".join(lines)


def main():
    with open(OUT, "w") as f:
        f.write(render())
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
