"""Species and photolysis-rate numbering of the REPROBUS chemistry.

Transported slots qj1(...,1..43): src/reprobus_l137_20230723.f:718-730.
Steady-state slots hc(...,1..15): :741-746.
Photolysis rates tj(...,1..41): :754-794.
All lists are 0-based in Python: LONG[0] is qj1 slot 1.
"""

LONG = [
    "n2o", "ch4", "h2o", "noy", "hno3", "n2o5", "cly", "ox", "co", "oclo",
    "ox_passive", "h2so4", "hcl", "clono2", "hocl", "cl2", "h2o2", "clno2", "hbr", "brono2",
    "nox", "ho2no2", "clox", "brox", "cl2o2", "hobr", "brcl", "ch2o", "ch3o2", "ch3o2h",
    "cfc11", "cfc12", "cfc113", "ccl4", "ch3ccl3", "ch3cl", "hcfc22", "ch3br", "h1211", "h1301",
    "bry", "ch2br2", "hno3_gas",
]
SHORT = [
    "o1d", "oh", "cl", "o3p", "o3", "ho2", "no2", "no", "br", "n",
    "clo", "bro", "no3", "h", "ch3",
]
PHOT = [
    "o2", "no2", "o3_o1d", "o3_o3p", "no3_no", "no3_no2", "n2o5", "hno3", "hno4", "h2o2",
    "h2o", "n2o", "hocl", "clono2_cl", "clono2_clo", "cl2o2", "hcl", "cl2", "clno2", "bro",
    "brono2", "hobr", "oclo", "brcl", "ch3o2h", "ch2o_hco", "ch2o_co", "cfc11", "cfc12", "cfc113",
    "ccl4", "ch3ccl3", "ch3cl", "hcfc22", "ch3br", "h1211", "h1301", "co2", "ch2br2", "hbr",
    "no",
]
RATES = (
    "a1 a1et a2 a5 a6 a6b a7 a17 a19 a26 a27 a30 a31 a36 "
    "b3 b4 b6 b7 b9 b12 b22 b23 b24 b27 b28 b32 b38 b39 "
    "c1a c1b c1c c2 c3 c4 c5 c7 c8 c9 c10 c12 c14 c15 c17a c17b c18 c19 "
    "d2 d3 d4 d5 d6 d7 d8 d9 d10 d11 d31 d32 d33 d34 d35 d36 d37 d60 d61 d62 "
    "d90 d91 d92 d93 d94 d95 d96 d97 "
    "e2 e3 e4 e5a e5b e5c e6 e7 e8 e9 e10 e11 e13 e15 e16 e50 e51 e52 e53 e54 "
    "hk1 hk2 hk3 hk4 hk5"
).split()

NBCON = len(LONG)   # 43
NCM = len(SHORT)    # 15
NPHOT = len(PHOT)   # 41
NRATE = len(RATES)  # 99
assert (NBCON, NCM, NPHOT, NRATE) == (43, 15, 41, 99)

L = {n: i for i, n in enumerate(LONG)}
S = {n: i for i, n in enumerate(SHORT)}

# per-cell diagnostics layout (include/reprobus_chem.h, REPROBUS_DIAG_*)
DIAG_HNM, DIAG_SZA, DIAG_O3T = 0, 1, 2
DIAG_TJ = 3
DIAG_HET = 44
DIAG_PARTHNO3, DIAG_PARTHNO3SL, DIAG_PARTH2O, DIAG_PARTHCL = 53, 54, 55, 56
DIAG_VSED, DIAG_SURFAREA = 57, 58
DIAG_RATE = 59
DIAG_COUNT = 158
DIAG_NAMES = (
    ["hnm", "sza", "o3t"] + [f"J_{p}" for p in PHOT] + [f"het{i}" for i in range(1, 10)]
    + ["parthno3", "parthno3sl", "parth2o", "parthcl", "vsed", "surfarea"] + RATES
)
assert len(DIAG_NAMES) == DIAG_COUNT
