"""Generates reprobus_gb300/csrc/log_table.h: the constants of the
table-driven logarithm log64 (log64.cuh), computed with Python's decimal
module at 60 significant digits and rounded once to double precision.

Method (P. T. P. Tang, "Table-driven implementation of the logarithm
function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990), with
N = 256: x = 2^m y, y in [1, 2), F = 1 + j / 256 the nearest such breakpoint
(j = 0..256), ln x = m ln 2 + ln F + ln(1 + (y - F) / F).

  LOG64_INV[j]          1 / F_j, correctly rounded
  LOG64_HI[j]           ln F_j rounded to a multiple of 2^-42, so that
                        m LN2_HI + LOG64_HI[j] is exact for |m| < 2^11
  LOG64_LO[j]           ln F_j - LOG64_HI[j], correctly rounded
  LOG64_LN2_HI / _LO    the same split of ln 2

    python -m reprobus_gb300.codegen.gen_log_table
"""
from __future__ import annotations

import decimal
import os

N = 256
QUANTUM_BITS = 42
OUT = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "csrc", "log_table.h")


def _split(c, v):
    """(hi, lo): hi = v rounded to a multiple of 2^-QUANTUM_BITS, lo = v - hi."""
    q = decimal.Decimal(2) ** -QUANTUM_BITS
    hi = (v / q).to_integral_value(rounding=decimal.ROUND_HALF_EVEN) * q
    return float(hi), float(c.subtract(v, hi))


def constants():
    c = decimal.Context(prec=60)
    decimal.setcontext(c)
    inv, hi, lo = [], [], []
    for j in range(N + 1):
        F = c.add(decimal.Decimal(1), c.divide(decimal.Decimal(j), N))
        inv.append(float(c.divide(decimal.Decimal(1), F)))
        h, l = _split(c, c.ln(F))
        hi.append(h)
        lo.append(l)
    ln2_hi, ln2_lo = _split(c, c.ln(decimal.Decimal(2)))
    return inv, hi, lo, ln2_hi, ln2_lo


def render():
    inv, hi, lo, ln2_hi, ln2_lo = constants()

    def table(name, vals):
        out = [f"LOG64_TABLE double {name}[{N + 1}] = {{"]
        for i in range(0, N + 1, 4):
            out.append("    " + ", ".join(v.hex() for v in vals[i:i + 4]) + ",")
        out.append("};")
        return out

    lines = [
        "// log_table.h — constants of the table-driven logarithm log64 (log64.cuh).",
        "// Generated by reprobus_gb300/codegen/gen_log_table.py; do not edit.",
        "#pragma once",
        "",
        "namespace rpb {",
        "",
        f"constexpr int LOG64_N = {N};",
        f"constexpr double LOG64_LN2_HI = {ln2_hi.hex()};  // ln 2 to a multiple of 2^-{QUANTUM_BITS}",
        f"constexpr double LOG64_LN2_LO = {ln2_lo.hex()};  // ln 2 - LOG64_LN2_HI",
        "",
        "#ifdef __CUDACC__",
        "#define LOG64_TABLE static __device__ const",
        "#else",
        "#define LOG64_TABLE static const",
        "#endif",
        f"// 1 / F_j and ln F_j = hi + lo for F_j = 1 + j / {N}, j = 0..{N}",
    ]
    lines += table("LOG64_INV", inv) + table("LOG64_HI", hi) + table("LOG64_LO", lo)
    lines += ["#undef LOG64_TABLE", "", "}  // namespace rpb", ""]
    return "\n".join(lines)


def main():
    with open(OUT, "w") as f:
        f.write(render())
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
