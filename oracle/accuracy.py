"""Accuracy of a chemistry-step answer against Oracle-C (test infrastructure).

TEST INFRASTRUCTURE ONLY: used by tests/ and by the accuracy leg of bench.py
(after and outside its timed region) as the checker of an answer the GPU
library produced; never part of the measured or shipped path.

The quantities follow the accuracy contract of the Newton solvers:
  * per species, |x - x_ref| / |x_ref| for values above 1e-20 mol/mol
    (the reference's mixing ratios, qj1 slots 1..42 and hc 1..15);
  * the element totals: the Cl, N and Br family tracers (Cly, NOy, Bry;
    qj1 slots 7, 4, 41) that conserv (src/reprobus_l137_20230723.f:2526-2616)
    rescales the members of each family to, relative to the oracle's.
    (The members do not close on all three totals at once after conserv:
    its Br step rescales BrCl and BrONO2, which the Cl and N totals count.)
"""
from __future__ import annotations

import numpy as np

from . import oracle

SPECIES_FLOOR = 1e-20  # mol/mol: species below it are not compared
ELEMENTS = (("Cl", 7), ("N", 4), ("Br", 41))  # element and its family tracer's qj1 slot


def _rel(a, b):
    d = np.where(a == b, 0.0, np.abs(a - b))
    return d / np.maximum(np.abs(b), 1e-300)


def cell_errors(got, ref, nb):
    """Per cell (diag layout: lon fastest, then lat, then level) the largest
    relative error over the 57 unknowns above SPECIES_FLOOR."""
    def one(a, b):
        return np.where(np.abs(b) > SPECIES_FLOOR, _rel(a, b), 0.0).max(axis=-1)
    eq = one(got["qj1"][:, :, :nb, :42], ref["qj1"][:, :, :nb, :42])
    eh = one(got["hc"][:, :, :nb, :], ref["hc"][:, :, :nb, :])
    return np.maximum(eq, eh).transpose(2, 1, 0).reshape(-1)


def species_errors(got, ref, nb, mask=None):
    """Rows (name, max, p99, cells above the floor) per species over the cells
    of mask (diag layout; None: all)."""
    from reprobus_gb300.species import LONG, SHORT
    rows = []
    for arr, n, names in (("qj1", 42, LONG), ("hc", 15, SHORT)):
        for s in range(n):
            g = got[arr][:, :, :nb, s].transpose(2, 1, 0).reshape(-1)
            r = ref[arr][:, :, :nb, s].transpose(2, 1, 0).reshape(-1)
            if mask is not None:
                g, r = g[mask], r[mask]
            big = np.abs(r) > SPECIES_FLOOR
            e = np.where(big, _rel(g, r), 0.0)
            rows.append((f"{arr}:{names[s]}", float(e.max()) if e.size else 0.0,
                         float(np.percentile(e, 99)) if e.size else 0.0, int(big.sum())))
    return rows


def element_errors(got, ref, nb, mask=None):
    """Per element the largest relative error of its family tracer over the
    chemistry cells of mask (diag layout; None: all)."""
    out = {}
    for name, slot in ELEMENTS:
        e = _rel(got["qj1"][:, :, :nb, slot - 1], ref["qj1"][:, :, :nb, slot - 1]).transpose(2, 1, 0).reshape(-1)
        e = e if mask is None else e[mask]
        out[name] = float(e.max()) if e.size else None
    return out


class Reference:
    """Oracle-C's answers for one case: the fixed point of the reference pass
    map (Newton, staged restarts) and the reference's own 5-pass answer, both
    with or without conserv and the clamps (fuse)."""

    def __init__(self, case, fuse=True, nthreads=0):
        self.case = case
        self.fuse = fuse
        self.fp, self.stat, self.res, self.stage = oracle.step_fixed_point(
            case, tol=1e-12, maxiter=60, fuse=fuse, nthreads=nthreads, with_stage=True)
        self.ref5, _, _ = oracle.step(case, niter=5, fuse=fuse, nthreads=nthreads)

    @property
    def converged(self):
        return self.stat >= 0

    def report(self, got, tol=1e-6, against="fixed_point"):
        """Accuracy of an answer `got` (dict with qj1 and hc of this case).
        against="fixed_point" (the Newton solvers): against Oracle-C's fixed
        point over the cells where it converged; cells above tol that equal
        the reference's 5-pass answer instead (the solver's fallbacks) are
        counted apart and left out of err_*/elem_err. against="ref5" (the
        reference-scheme solver): against the reference's own 5-pass answer
        over every cell."""
        nb = self.case.nivbas
        if against == "ref5":
            e = cell_errors(got, self.ref5, nb)
            return {"against": "reference 5-pass answer", "cells": int(e.size), "err_max": float(e.max()),
                    "err_p99": float(np.percentile(e, 99)), "cells_over_tol": int((e > tol).sum()), "tol": tol,
                    "elem_err": element_errors(got, self.ref5, nb)}
        e = cell_errors(got, self.fp, nb)
        conv = self.converged
        over = conv & (e > tol)
        fallback_like = over & (cell_errors(got, self.ref5, nb) <= tol)
        kept = conv & ~fallback_like
        return {"against": "fixed point (Oracle-C)", "cells": int(e.size), "oracle_converged": int(conv.sum()),
                "err_max": float(e[kept].max()) if kept.any() else None,
                "err_p99": float(np.percentile(e[kept], 99)) if kept.any() else None,
                "cells_over_tol": int(over.sum()), "over_tol_equal_to_ref5": int(fallback_like.sum()),
                "tol": tol, "elem_err": element_errors(got, self.fp, nb, kept)}
