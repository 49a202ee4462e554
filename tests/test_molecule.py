"""Molecule wrapper (python/giao_integrals/molecule.py:285-475): atoms and
XYZ input, unit conversion, BSE-JSON bases (dictionary, text, file), shell
order and owners, and the reference's validation errors.  Host-only."""

from __future__ import annotations

import json

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300.molecule import BOHR_IN_ANGSTROM, Molecule

# a synthetic two-element basis in BSE-JSON layout (made-up exponents)
BASIS = {
    "elements": {
        "1": {"electron_shells": [
            {"function_type": "gto", "angular_momentum": [0], "exponents": ["2.5", "0.45"],
             "coefficients": [["0.3", "0.8"]]},
            {"function_type": "gto", "angular_momentum": [1], "exponents": ["0.7"], "coefficients": [["1.0"]]},
        ]},
        "8": {"electron_shells": [
            {"function_type": "gto", "angular_momentum": [2], "exponents": ["0.9"], "coefficients": [["1.0"]]},
            {"function_type": "gto", "angular_momentum": [0, 1], "exponents": ["5.0", "1.1D0"],
             "coefficients": [["0.4", "0.7"], ["0.5", "0.6"]]},
            {"function_type": "gto", "angular_momentum": [0], "exponents": ["30.0", "6.0", "1.5"],
             "coefficients": [["0.2", "0.5", "0.4"], ["0.0", "-0.3", "1.0"]]},
        ]},
    }
}
ATOMS = [("O", (0.0, 0.0, 0.1)), ("H", (0.0, 0.75, -0.45)), ("1", (0.0, -0.75, -0.45))]


def test_atoms_units_and_shell_layout(tmp_path):
    m = Molecule(ATOMS, BASIS)
    assert [s for s, _ in m.atoms] == ["O", "H", "H"]
    assert np.allclose(m.atoms[1][1], np.array([0.0, 0.75, -0.45]) / BOHR_IN_ANGSTROM)
    # O: s(2 contractions), s (from sp), p (from sp), d; H: s, p
    assert [s.angular_momentum for s in m.basis.shells] == [0, 0, 1, 2, 0, 1, 0, 1]
    assert m.shell_atoms == (0, 0, 0, 0, 1, 1, 2, 2)
    assert m.basis.shells[0].contraction_count in (1, 2)
    assert [n.charge for n in m.nuclei] == [8.0, 1.0, 1.0]
    assert m.ao_count == sum(s.ao_count for s in m.basis.shells)
    assert "cartesian_aos" in repr(m)
    b = Molecule(ATOMS, BASIS, unit="bohr")
    assert b.atoms[1][1] == (0.0, 0.75, -0.45)
    text = Molecule(ATOMS, json.dumps(BASIS))
    f = tmp_path / "basis.json"
    f.write_text(json.dumps(BASIS))
    path = Molecule(ATOMS, f)
    for other in (text, path):
        assert [s.angular_momentum for s in other.basis.shells] == [s.angular_momentum for s in m.basis.shells]
    xyz = "3\nwater\nO 0 0 0.1\nH 0 0.75 -0.45\nH 0 -0.75 -0.45\n"
    x = Molecule.from_xyz(xyz, BASIS)
    assert x.atoms == m.atoms
    field = gi.MagneticField((0.0, 0.0, 0.1))
    assert Molecule(ATOMS, BASIS, field=field).field is field


def test_validation_errors(tmp_path):
    with pytest.raises(ValueError, match="unit must be"):
        Molecule(ATOMS, BASIS, unit="nm")
    with pytest.raises(ValueError, match="Unknown element"):
        Molecule([("Xx", (0, 0, 0))], BASIS)
    with pytest.raises(ValueError, match="at least one atom"):
        Molecule([], BASIS)
    with pytest.raises(ValueError, match="Invalid atom 1"):
        Molecule([("H", (0, 0))], BASIS)
    with pytest.raises(ValueError, match="no data for element C"):
        Molecule([("C", (0, 0, 0))], BASIS)
    with pytest.raises(ValueError, match="ECP"):
        Molecule([("H", (0, 0, 0))], {"elements": {"1": {"ecp_electrons": 2, "electron_shells": []}}})
    with pytest.raises(ValueError, match="distinct angular momenta"):
        Molecule([("H", (0, 0, 0))], {"elements": {"1": {"electron_shells": [
            {"angular_momentum": [1, 1], "exponents": [1.0], "coefficients": [[1.0], [1.0]]}]}}})
    with pytest.raises(ValueError, match="basis_format must be"):
        Molecule(ATOMS, BASIS, basis_format="xml")
    with pytest.raises(ValueError, match="Invalid BSE JSON"):
        Molecule(ATOMS, "{not json")
    with pytest.raises(ValueError, match="Specify basis_format"):
        Molecule(ATOMS, "H 0\nS 1 1.0\n")
    with pytest.raises(TypeError, match="basis must be"):
        Molecule(ATOMS, 3.0)
    with pytest.raises(TypeError, match="field must be"):
        Molecule(ATOMS, BASIS, field=(0, 0, 1))
    try:
        import basis_set_exchange  # noqa: F401
    except ImportError:
        with pytest.raises(ImportError, match="basis-set-exchange"):
            Molecule(ATOMS, "sto-3g")
    with pytest.raises(ValueError, match="integer atom count"):
        Molecule.from_xyz("x\n\nH 0 0 0\n", BASIS)
    with pytest.raises(ValueError, match="one XYZ frame"):
        Molecule.from_xyz("1\n\nH 0 0 0\nH 1 1 1\n", BASIS)
