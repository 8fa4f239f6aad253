"""Writes ../csrc/tropo_tables.h: the yearly (June) forcing values that the
reference's tropospheric relaxation interpolates in time, as tabulated in the
`data s_*` statements of subroutine tropo (src/reprobus_l137_20230723.f:4099-4411;
37 values per species for 1988..2024).

These are observed surface mixing ratios (NOAA/GML, CCMVal), i.e. physical
data that the port must reproduce exactly. Run once with the reference
checkout at REPROBUS_SRC (the directory holding the reference's src files; required); the output is committed
because the reference tree is not available where the library is built and
runs.
"""
import os
import re
import sys


def _src_dir():
    d = os.environ.get("REPROBUS_SRC")
    if not d:
        sys.exit("set REPROBUS_SRC to the reference checkout's src directory")
    return d

NAMES = ["noy", "cly", "bry", "n2o", "ch4", "ch3cl", "cfc11", "cfc12", "cfc114", "cfc115", "cfc113", "ccl4",
         "ch3ccl3", "hcfc22", "hcfc141b", "hcfc142b", "ch3br", "h1211", "h1301", "h2402", "ch2br2"]
NYEAR = 37

src = os.path.join(_src_dir(), "reprobus_l137_20230723.f")
lines = open(src).read().splitlines()
lo, hi = 4077, 4574  # subroutine tropo
body = lines[lo - 1:hi]
tables = {}
i = 0
while i < len(body):
    m = re.match(r"\s+data\s+s_(\w+)\s*/(.*)", body[i])
    if not m:
        i += 1
        continue
    name, text = m.group(1), m.group(2)
    while "/" not in text:
        i += 1
        cont = body[i]
        if not re.match(r"     \$", cont):
            sys.exit(f"unexpected line in data s_{name}: {cont!r}")
        text += cont[6:]
    text = text.split("/")[0]
    vals = [v.strip() for v in text.split(",") if v.strip()]
    if len(vals) != NYEAR:
        sys.exit(f"s_{name}: {len(vals)} values")
    tables[name] = vals
    i += 1
missing = [n for n in NAMES if n not in tables]
if missing:
    sys.exit(f"tables not found: {missing}")


def c_literal(v):
    v = v.lower()
    if v.endswith("."):
        v += "0"
    if "e" in v:
        mant, ex = v.split("e")
        if mant.endswith("."):
            mant += "0"
        v = f"{mant}e{ex}"
    return v


out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "csrc", "tropo_tables.h")
with open(out, "w") as f:
    f.write("// tropo_tables.h -- GENERATED by reprobus_gb300/data/make_tropo.py from the\n")
    f.write("// `data s_*` statements of subroutine tropo (src/reprobus_l137_20230723.f:4099-4411):\n")
    f.write("// June surface mixing ratios (mol/mol) for the years 1988..2024. Do not edit.\n")
    f.write("#pragma once\n\nnamespace rpb {\n")
    f.write(f"constexpr int TROPO_NYEAR = {NYEAR};\nconstexpr int TROPO_YEAR0 = 1988;\n")
    f.write(f"constexpr int TROPO_NTAB = {len(NAMES)};\n")
    f.write("enum TropoTab {\n" + "".join(f"    TT_{n.upper()} = {k},\n" for k, n in enumerate(NAMES)) + "};\n")
    f.write("static const double kTropoTab[TROPO_NTAB][TROPO_NYEAR] = {\n")
    for n in NAMES:
        f.write(f"    /* {n} */ {{" + ", ".join(c_literal(v) for v in tables[n]) + "},\n")
    f.write("};\n}  // namespace rpb\n")
print("wrote", os.path.normpath(out))
