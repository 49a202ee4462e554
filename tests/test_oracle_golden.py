"""The CPU oracle pinned against the reference's golden vectors (no GPU)."""

import numpy as np
import pytest

from oracle import oracle as O
from giaoint_gb300 import synthetic as syn


def test_boys_oracle_matches_reference_and_mpmath(golden, oracle):
    orders = golden.boys["mpmath_orders"]
    for case in golden.boys["cases"]:
        z = complex(*case["z"])
        vals, diag = oracle.boys(z, 32)
        ref = np.array([complex(*v) for v in case["reference"]])
        np.testing.assert_allclose(vals, ref, rtol=1e-15, atol=1e-300)
        assert diag["region"] == case["region"]
        for n, mp in zip(orders, case["mpmath"], strict=True):
            expected = complex(*mp)
            assert abs(vals[n] - expected) <= 3e-14 + 8e-13 * abs(expected)


def test_boys_oracle_scaled_and_errors(golden, oracle):
    for case in golden.boys["scaled"]:
        vals, _ = oracle.boys(complex(*case["z"]), 16, scaled=True)
        np.testing.assert_allclose(vals, [complex(*v) for v in case["reference"]], rtol=1e-15)
    for err in golden.boys["errors"]:
        with pytest.raises(O.OracleError, match="outside the verified"):
            oracle.boys(complex(*err["z"]), err["order"])


def test_primitive_eri_oracle_against_frozen_m8(golden, oracle):
    for rec in golden.m8:
        prims = [(p["exponent"], p["center"], p["angular"], p["coefficient"], p["normalized"])
                 for p in rec["primitives"]]
        for fld, expected, ref in zip([(0, 0, 0), rec["field"]], rec["expected"], rec["reference"], strict=True):
            v = oracle.primitive_eri(prims, fld, rec["gauge"])
            e = complex(*expected)
            assert abs(v - e) <= 5e-14 + 5e-13 * abs(e)
            assert abs(v - complex(*ref)) <= 2e-15 * abs(complex(*ref))


def test_shell_quartets_oracle_bitwise_reference(golden, oracle):
    b = golden.blocks
    atom = syn.full_tensor_atom()
    vals, offs = oracle.eri_batch(atom, b["atom_quartets"], (0, 0, 0.1), None, 8)
    np.testing.assert_array_equal(offs, b["atom_offsets"])
    np.testing.assert_array_equal(vals, b["atom_values"])
    mol = syn.random_molecule(2026)
    vals, offs = oracle.eri_batch(mol, b["mol_quartets"], tuple(b["mol_field"]), None, 8)
    np.testing.assert_array_equal(vals, b["mol_values"])
    vals, _ = oracle.eri_batch(mol, b["mol_quartets"][:120], (0, 0, 0), None, 8)
    np.testing.assert_array_equal(vals, b["mol_zero_values"])


def test_cholesky_driver_restatement_matches_reference_driver(golden, oracle):
    g = golden.cholesky
    specs = {k: [O.ShellSpec(tuple(s["center"]), s["l"], s["exponents"], s["coefficients"], s["normalize"])
                 for s in v] for k, v in g["shells"].items()}
    for case in g["cases"]:
        if case["system"] == "molecule3" and case["threshold"] < 1e-6:
            continue  # the tight cases run in the GPU suite; keep the CPU suite short
        res = O.cholesky_eri(oracle, specs[case["system"]], case["B"], case["origin"], threshold=case["threshold"],
                             pivot_batch_size=case["pivot_batch_size"], threads=8)
        assert len(res.pivots) == case["rank"]
        np.testing.assert_array_equal(res.pivots, np.asarray(case["pivots"]))
        assert abs(res.max_residual_diagonal - case["max_residual_diagonal"]) <= 1e-15
        first = np.array([complex(*x) for x in case["first_vector"]])
        np.testing.assert_allclose(res.vectors[0].ravel()[: len(first)], first, atol=1e-15)


def test_canonical_quartet_enumeration(oracle):
    import giaoint_gb300 as gi

    for ns in (1, 2, 3, 5):
        np.testing.assert_array_equal(gi.canonical_quartets(ns), oracle.canonical_quartets(ns))
    assert len(oracle.canonical_quartets(72)) == 6722352


def test_nuclear_attraction_oracle_matches_reference(golden, oracle):
    """Oracle restatement of src/nuclear.cpp against the reference library's
    compute_nuclear_attraction_matrix (golden nuclear.npz)."""
    from giaoint_gb300 import synthetic as syn

    g = golden.nuclear
    recs = syn.random_molecule(7, natoms=3)
    nuclei = [(float(z), tuple(c)) for z, c in zip(g["charges"], g["centers"])]
    v1 = oracle.nuclear(recs, nuclei, (0.05, -0.1, 0.12), (0.3, 0.1, -0.2))
    v0 = oracle.nuclear(recs, nuclei, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    va = oracle.nuclear(syn.full_tensor_atom(), [(10.0, (0.0, 0.0, 0.0))], (0.0, 0.0, 0.1), (0.0, 0.0, 0.0))
    np.testing.assert_allclose(v1, g["mol_field"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(v0, g["mol_zero"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(va, g["atom"], rtol=1e-13, atol=1e-13)
    # Hermitian, and the field changes it
    assert np.abs(v1 - v1.conj().T).max() < 1e-12
    assert np.abs(v1 - v0).max() > 1e-6

