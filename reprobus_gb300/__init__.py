"""reprobus_gb300 — GB300-native (sm_103a) REPROBUS chemistry step.

The per-gridbox chemistry of the REPROBUS chemistry-transport model
(src/reprobus_l137_20230723.f:601-2412 and callees) as hand-written CUDA behind
a C-ABI (include/reprobus_chem.h); see chem.py for the Python front end.
"""
from .chem import (CHECK_FINITE, FUSE_CONSERV, ChemStep, ReprobusError, chem3d, conserv, const, init,
                   load_library)

__all__ = ["ChemStep", "ReprobusError", "chem3d", "conserv", "const", "init", "load_library",
           "FUSE_CONSERV", "CHECK_FINITE"]
