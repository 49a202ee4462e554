"""Molecule methods on the GPU equal the direct calls on its basis, nuclei
and field (python/giao_integrals/molecule.py:383-475)."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi

from test_molecule import ATOMS, BASIS

pytestmark = pytest.mark.gpu


def test_molecule_methods_match_direct_calls():
    field = gi.MagneticField((0.02, -0.05, 0.1), gauge_origin=(0.1, 0.0, -0.2))
    m = gi.Molecule(ATOMS, BASIS, field=field)
    v = m.nuclear_attraction()
    np.testing.assert_array_equal(v, gi.nuclear_attraction(m.basis, m.nuclei, field=field))
    assert np.abs(v - v.conj().T).max() < 1e-12
    full = m.eri()
    assert full.shape == (m.ao_count,) * 4
    np.testing.assert_array_equal(full, gi.eri(m.basis, field=field, storage="full",
                                               max_bytes=m.ao_count ** 4 * 16))
    batches = list(m.eri_batches(target_bytes=1 << 16))
    assert sum(len(b.quartets) for b in batches) == len(gi.canonical_quartets(len(m.basis.shells)))
    q = [(0, 4, 2, 6), (3, 3, 1, 7)]
    d = next(m.eri_derivative_batches(quartets=q))
    e = next(gi.eri_derivative_batches(m.basis, field=field, quartets=q))
    np.testing.assert_array_equal(d.values, e.values)
    chol = m.cholesky_eri(threshold=1e-8)
    n = m.ao_count
    L = chol.vectors.reshape(len(chol.pivots), n, n)
    rec = np.einsum("pij,plk->ijkl", L, L.conj())
    assert np.abs(rec - full).max() < 1e-7
