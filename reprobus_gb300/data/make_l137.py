"""Writes l137_ab.txt: the 138 half-level coefficients a [Pa], b of the ECMWF
L137 hybrid vertical grid, as tabulated in the REPROBUS source tree
(src/ecmwf_levels_table.csv, columns n, a [Pa], b).

The reference reads the same coefficients from ecmwf_137_levels.txt at run time
(src/reprobus_l137_20230723.f:79-91). Run once, with the reference checkout at
REPROBUS_SRC (the directory holding the reference's src files; required); the output is committed because the
reference tree is not available where the library runs.
"""
import csv
import os
import sys


def _src_dir():
    d = os.environ.get("REPROBUS_SRC")
    if not d:
        sys.exit("set REPROBUS_SRC to the reference checkout's src directory")
    return d

src = _src_dir()
rows = []
with open(os.path.join(src, "ecmwf_levels_table.csv")) as f:
    rd = csv.reader(f)
    next(rd)
    for r in rd:
        rows.append((int(r[0]), r[1], r[2]))
if len(rows) != 138:
    sys.exit(f"expected 138 half levels, got {len(rows)}")
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "l137_ab.txt")
with open(out, "w") as f:
    f.write("# ECMWF L137 half-level coefficients: n  a[Pa]  b\n")
    for n, a, b in rows:
        f.write(f"{n:4d} {a} {b}\n")
print("wrote", out)
