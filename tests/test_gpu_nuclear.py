"""GIAO nuclear attraction on the GPU against the reference library's values
(golden nuclear.npz) and the oracle: full matrix, shell blocks, single
primitives, validation and errors of the reference's Python API."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300 import synthetic as syn

from helpers import basis_from_records

pytestmark = pytest.mark.gpu

FIELD = gi.MagneticField((0.05, -0.1, 0.12), gauge_origin=(0.3, 0.1, -0.2))


def _nuclei(golden):
    g = golden.nuclear
    return [gi.Nucleus(float(z), tuple(c)) for z, c in zip(g["charges"], g["centers"])]


def test_matrix_matches_reference(golden):
    g = golden.nuclear
    basis = basis_from_records(syn.random_molecule(7, natoms=3))
    nuclei = _nuclei(golden)
    v1 = gi.nuclear_attraction(basis, nuclei, field=FIELD)
    v0 = gi.nuclear_attraction(basis, nuclei)
    np.testing.assert_allclose(v1, g["mol_field"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(v0, g["mol_zero"], rtol=1e-12, atol=1e-12)
    atom = basis_from_records(syn.full_tensor_atom())
    va = gi.nuclear_attraction(atom, [gi.Nucleus(10.0, (0.0, 0.0, 0.0))], field=gi.MagneticField((0.0, 0.0, 0.1)))
    np.testing.assert_allclose(va, g["atom"], rtol=1e-12, atol=1e-12)


def test_shell_blocks_primitives_and_out(golden, oracle):
    recs = syn.random_molecule(7, natoms=3)
    basis = basis_from_records(recs)
    nuclei = _nuclei(golden)
    full = gi.nuclear_attraction(basis, nuclei, field=FIELD)
    shells = basis.shells
    off = basis.ao_offsets
    for a, b in [(0, 0), (3, 5), (5, 3), (11, 17), (17, 2)]:
        blk = gi.nuclear_attraction_shell(shells[a], shells[b], nuclei, field=FIELD)
        ref = full[off[a]:off[a] + shells[a].ao_count, off[b]:off[b] + shells[b].ao_count]
        np.testing.assert_allclose(blk, ref, rtol=1e-12, atol=1e-12)
    out = np.empty((shells[3].ao_count, shells[5].ao_count), dtype=np.complex128)
    assert gi.nuclear_attraction_shell(shells[3], shells[5], nuclei, field=FIELD, out=out) is out
    with pytest.raises(ValueError, match="out has an incorrect shape"):
        gi.nuclear_attraction_shell(shells[3], shells[5], nuclei, out=np.empty((1, 1), dtype=np.complex128))
    with pytest.raises(ValueError, match="dtype complex128"):
        gi.nuclear_attraction(basis, nuclei, out=np.empty(full.shape, dtype=np.float64))
    # single primitives, normalised and not, against the oracle's shell of one primitive
    bra = gi.PrimitiveGaussian(0.7, (0.1, 0.0, -0.3), (1, 0, 1), coefficient=0.8)
    ket = gi.PrimitiveGaussian(1.3, (0.0, 0.5, 0.2), (0, 2, 0), coefficient=1.1, normalized=False)
    nucs = [(2.0, (0.0, 0.0, 0.0)), (1.0, (0.4, -0.3, 0.9))]
    v = gi.primitive_nuclear_attraction(bra, ket, [gi.Nucleus(z, c) for z, c in nucs], field=FIELD)
    prim_recs = [syn.ShellRecord(bra.center, 2, (0.7,), ((1.0,),), False),
                 syn.ShellRecord(ket.center, 2, (1.3,), ((1.0,),), False)]
    mat = oracle.nuclear(prim_recs, nucs, FIELD.B, FIELD.gauge_origin)
    comps = gi.cartesian_components(2)
    expect = mat[comps.index((1, 0, 1)), 6 + comps.index((0, 2, 0))] * 0.8 * 1.1 / gi.primitive_normalization(
        1.3, (0, 2, 0))
    assert abs(v - expect) <= 1e-12 * max(1.0, abs(expect))


def test_no_nuclei_and_validation():
    basis = basis_from_records(syn.random_molecule(7, natoms=2))
    z = gi.nuclear_attraction(basis, [])
    assert z.shape == (basis.ao_count, basis.ao_count) and not z.any()
    with pytest.raises(ValueError, match="nuclear charge must be finite and positive"):
        gi.Nucleus(0.0, (0.0, 0.0, 0.0))
    with pytest.raises(TypeError):
        gi.nuclear_attraction(basis, [(1.0, (0.0, 0.0, 0.0))])
