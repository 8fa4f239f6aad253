"""Writes tests/golden/oracle_cfg0_small.npz: the oracle's output (5 passes,
fused conserv + clamps) on the seeded 4-column config-0 workload. A regression
fixture of the oracle (the reference itself cannot be run: no Fortran
compiler, no golden vectors of its own)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402
from reprobus_gb300 import inputs  # noqa: E402

seed, nlon, nivbas = 17, 4, 94
c = inputs.make_case("cfg0", seed=seed, nlon=nlon, nivbas=nivbas)
st, _, _ = oracle.step(c, niter=5, fuse=True)
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_cfg0_small.npz")
np.savez_compressed(out, seed=seed, nlon=nlon, nivbas=nivbas, qj1=st["qj1"], hc=st["hc"])
print("wrote", out)
