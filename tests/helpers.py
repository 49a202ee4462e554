"""Shared test helpers: systems, scatter of packed blocks, pivot comparison."""

from __future__ import annotations

import numpy as np

import giaoint_gb300 as gi
from giaoint_gb300 import synthetic as syn


def basis_from_records(records):
    return gi.Basis([gi.Shell.from_record(r) for r in records])


def specs_to_basis(shells):
    out = []
    for s in shells:
        out.append(gi.Shell(tuple(s["center"]), s["l"], s["exponents"], np.asarray(s["coefficients"]),
                            normalize=bool(s["normalize"])))
    return gi.Basis(out)


def molecule(seed=2026, natoms=12):
    recs = syn.random_molecule(seed, natoms=natoms)
    return recs, basis_from_records(recs)


def pivots_agree(pivots, ref_pivots, residual_gap_ok):
    """Pivots must match wherever the decision was not a near tie."""
    n = min(len(pivots), len(ref_pivots))
    for k in range(n):
        if tuple(pivots[k]) != tuple(ref_pivots[k]):
            return residual_gap_ok(k)
    return True
