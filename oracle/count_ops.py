"""Prints the algorithmic FP64 work per cell-step of the reference scheme
(operation counts of the oracle, op_count.cpp) for a workload.

    python -m oracle.count_ops [--config cfg1] [--rows 12]

Measurement infrastructure: the figure is the numerator of the benchmark's
roofline (algorithmic FLOP per cell-step), fixed once per workload.
"""
import argparse
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from oracle import oracle  # noqa: E402
from reprobus_gb300 import inputs  # noqa: E402

ap = argparse.ArgumentParser()
ap.add_argument("--config", default="cfg1")
ap.add_argument("--rows", type=int, default=12)
ap.add_argument("--seed", type=int, default=1234)
a = ap.parse_args()
case = inputs.make_case(a.config, seed=a.seed)
rows = sorted({int(round(x)) for x in np.linspace(1, case.nlat, a.rows)})
r = oracle.op_counts(case, rows)
r["ops"] = r["flops"] + r["transcendentals"]
print(json.dumps({k: (round(v, 2) if isinstance(v, float) else v) for k, v in r.items()}))
