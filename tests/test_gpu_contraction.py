"""Per-atom ERI centre-derivative contraction on the GPU
(eri_derivative_contraction, python/giao_integrals/derivative_assembly.py)
against the reference library's contract_eri_derivatives (golden
contraction.npz), batching invariance, the Molecule method and validation."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi

from conftest import contraction_setup

pytestmark = pytest.mark.gpu


def _basis(specs):
    return gi.Basis([gi.Shell(s.center, s.l, s.exponents, np.asarray(s.coefficients), normalize=s.normalize)
                     for s in specs])


def test_contraction_matches_reference(golden):
    mg = contraction_setup()
    for name, specs, atoms, natom, complex_gamma in mg.contraction_cases():
        basis = _basis(specs)
        n = basis.ao_count
        coulomb, exchange, gamma = mg.contraction_densities(n, complex_gamma)
        for label, field in (("field", gi.MagneticField(mg.DERIV_FIELD, gauge_origin=mg.DERIV_ORIGIN)),
                             ("zero", None)):
            got = gi.eri_derivative_contraction(basis, atoms, natom, field=field, coulomb_pairs=coulomb,
                                                exchange_pairs=exchange, gamma=gamma)
            ref = golden.contraction[f"{name}_{label}"]
            assert got.shape == (natom, 3)
            assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max(), (name, label)
            # each density kind alone adds up to the combined result
            parts = (gi.eri_derivative_contraction(basis, atoms, natom, field=field, coulomb_pairs=coulomb)
                     + gi.eri_derivative_contraction(basis, atoms, natom, field=field, exchange_pairs=exchange)
                     + gi.eri_derivative_contraction(basis, atoms, natom, field=field, gamma=gamma))
            assert np.abs(parts - got).max() <= 1e-11 * np.abs(ref).max()


def test_batching_invariance_out_and_validation():
    mg = contraction_setup()
    name, specs, atoms, natom, _ = mg.contraction_cases()[1]
    basis = _basis(specs)
    n = basis.ao_count
    coulomb, exchange, gamma = mg.contraction_densities(n, True)
    field = gi.MagneticField((0.02, 0.05, -0.1))
    full = gi.eri_derivative_contraction(basis, atoms, natom, field=field, coulomb_pairs=coulomb,
                                         exchange_pairs=exchange)
    small = gi.eri_derivative_contraction(basis, atoms, natom, field=field, coulomb_pairs=coulomb,
                                          exchange_pairs=exchange, target_bytes=4096)
    # partial sums are added in quartet and slot order; the derivative blocks
    # of a smaller batch come from a plan whose ket chunking (and so the lane
    # split of each box sum) adapts to the batch size: equal to rounding
    assert np.abs(full - small).max() <= 1e-12 * np.abs(full).max()
    again = gi.eri_derivative_contraction(basis, atoms, natom, field=field, coulomb_pairs=coulomb,
                                          exchange_pairs=exchange)
    np.testing.assert_array_equal(full, again)  # same batching: bit for bit
    out = np.full((natom, 3), 7.0 + 0j)
    assert gi.eri_derivative_contraction(basis, atoms, natom, field=field, coulomb_pairs=coulomb,
                                         exchange_pairs=exchange, out=out) is out
    np.testing.assert_array_equal(out, full)
    with pytest.raises(ValueError, match="at least one density"):
        gi.eri_derivative_contraction(basis, atoms, natom)
    with pytest.raises(ValueError, match="shell_atoms"):
        gi.eri_derivative_contraction(basis, atoms[:-1], natom, coulomb_pairs=coulomb)
    with pytest.raises(ValueError, match="shape"):
        gi.eri_derivative_contraction(basis, atoms, natom, coulomb_pairs=[(coulomb[0][0][:2], coulomb[0][1])])
    with pytest.raises(ValueError, match="gamma"):
        gi.eri_derivative_contraction(basis, atoms, natom, gamma=gamma[:, :, :, :2])
    buf = np.zeros(n * n, dtype=np.complex128)
    with pytest.raises(ValueError, match="overlap"):
        gi.eri_derivative_contraction(basis, atoms, natom, coulomb_pairs=[(buf.reshape(n, n), coulomb[0][1])],
                                      out=buf[: natom * 3].reshape(natom, 3))
    # the Molecule method equals the function on its basis, owners and field
    from test_molecule import ATOMS, BASIS

    m = gi.Molecule(ATOMS, BASIS, field=field)
    nn = m.ao_count
    cj, kx, _ = mg.contraction_densities(nn, False)
    a = m.eri_derivative_contraction(coulomb_pairs=cj, exchange_pairs=kx)
    b = gi.eri_derivative_contraction(m.basis, m.shell_atoms, len(m.atoms), field=field, coulomb_pairs=cj,
                                      exchange_pairs=kx)
    np.testing.assert_array_equal(a, b)
