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



def test_eri_center_derivatives_oracle_matches_reference(golden, oracle):
    """Oracle restatement of compute_eri_center_derivatives
    (src/derivatives.cpp:53-87, 215-245, 556-640) against the reference
    library's blocks (golden derivatives.npz), zero and finite field."""
    from conftest import derivative_systems

    g = golden.derivatives
    B, origin = tuple(g["field"]), tuple(g["origin"])
    for name, specs, q in derivative_systems(g):
        for label, field, o in (("field", B, origin), ("zero", None, None)):
            vals, offsets = oracle.eri_center_derivatives(specs, q, field, o)
            np.testing.assert_array_equal(offsets, g[f"{name}_offsets"])
            ref = g[f"{name}_{label}"]
            assert np.abs(vals - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), (name, label)
        # zero and finite field differ
        assert np.abs(g[f"{name}_field"] - g[f"{name}_zero"]).max() > 1e-6


def derivative_sum_rule_residual(specs, q, offsets, values, eri, eri_offsets, B, origin) -> float:
    """max over blocks of |sum_slots d/dR - i (k_a - k_b + k_c - k_d) (ab|cd)| / max(1, max |block|).

    Translating all four centres by delta multiplies a London-orbital ERI
    (orbitals exp(-i k.r) phi(r - C), k = B x (C - O) / 2, fixed gauge
    origin) by exp(i (k_a - k_b + k_c - k_d).delta), so the four slot
    derivatives sum to i (k_a - k_b + k_c - k_d) times the ERI block."""
    B = np.asarray(B, dtype=float)
    O = np.asarray(origin, dtype=float)

    def k(c):
        return 0.5 * np.cross(B, np.asarray(c, dtype=float) - O)

    worst = 0.0
    for i, x in enumerate(np.asarray(q)):
        blk = values[offsets[i]:offsets[i + 1]].reshape(4, 3, -1)
        e = eri[eri_offsets[i]:eri_offsets[i + 1]]
        K = k(specs[x[0]].center) - k(specs[x[1]].center) + k(specs[x[2]].center) - k(specs[x[3]].center)
        r = np.abs(blk.sum(axis=0) - 1j * K[:, None] * e[None, :]).max()
        worst = max(worst, r / max(1.0, np.abs(blk).max()))
    return worst


def test_eri_center_derivatives_translation_sum_rule_oracle(golden, oracle):
    """The reference's derivative blocks obey the translation sum rule with
    the oracle's ERI blocks, at zero and finite field."""
    from conftest import derivative_systems

    g = golden.derivatives
    B, origin = tuple(g["field"]), tuple(g["origin"])
    for name, specs, q in derivative_systems(g):
        for label, field, o in (("field", B, origin), ("zero", (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))):
            eri, eoff = oracle.eri_batch(specs, q, field, o)
            r = derivative_sum_rule_residual(specs, q, g[f"{name}_offsets"], g[f"{name}_{label}"], eri, eoff,
                                             field, o)
            assert r <= 1e-11, (name, label, r)


def test_eri_derivative_bounds_oracle_matches_reference(golden, oracle):
    """Oracle restatement of EriDerivativeSchwarzBounds
    (src/derivatives.cpp:1307-1372) against the reference library's factors,
    and the oracle's ordinary Schwarz factors against the reference's."""
    from conftest import derivative_systems

    g = golden.derivatives
    B, origin = tuple(g["field"]), tuple(g["origin"])
    for name, specs, _q in derivative_systems(g):
        for label, field, o in (("field", B, origin), ("zero", None, None)):
            np.testing.assert_allclose(oracle.eri_derivative_bounds(specs, field, o), g[f"{name}_bounds_{label}"],
                                       rtol=1e-14, atol=0)
            np.testing.assert_allclose(oracle.schwarz(specs, field, o), g[f"{name}_schwarz_{label}"],
                                       rtol=1e-14, atol=0)


def test_eri_magnetic_derivatives_oracle_matches_reference(golden, oracle):
    """Oracle restatement of compute_eri_magnetic_derivatives
    (src/derivatives.cpp:88-106, 268-280, 961-966) against the reference
    library's (3, na, nb, nc, nd) blocks, zero and finite field."""
    from conftest import derivative_systems

    g = golden.derivatives
    B, origin = tuple(g["field"]), tuple(g["origin"])
    for name, specs, q in derivative_systems(g):
        for label, field, o in (("field", B, origin), ("zero", None, None)):
            vals, _ = oracle.eri_magnetic_derivatives(specs, q, field, o)
            ref = g[f"{name}_magnetic_{label}"]
            assert np.abs(vals - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), (name, label)


def test_eri_mixed_derivatives_oracle_matches_reference(golden, oracle):
    """Oracle restatement of compute_eri_mixed_derivatives
    (src/derivatives.cpp:160-181, 232-259, 968-973) against the reference
    library's (4, 3, 3, na, nb, nc, nd) blocks, zero and finite field."""
    from conftest import derivative_systems

    g = golden.derivatives
    B, origin = tuple(g["field"]), tuple(g["origin"])
    for name, specs, _q in derivative_systems(g):
        q = g[f"{name}_mixed_quartets"]
        for label, field, o in (("field", B, origin), ("zero", None, None)):
            vals, _ = oracle.eri_mixed_derivatives(specs, q, field, o)
            ref = g[f"{name}_mixed_{label}"]
            assert np.abs(vals - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), (name, label)


def test_eri_derivative_contraction_oracle_matches_reference(golden, oracle):
    """Oracle restatement of detail::contract_eri_derivatives
    (src/assembly.cpp:87-158) over all 5292 canonical quartets of a two-atom
    molecule at finite field, with the fixture's closed-form Coulomb,
    exchange and real two-particle densities, against the reference library."""
    from conftest import contraction_setup
    from oracle.oracle import contract_eri_derivatives

    mg = contraction_setup()
    name, specs, atoms, natom, complex_gamma = mg.contraction_cases()[1]
    n = sum(s.nao for s in specs)
    coulomb, exchange, gamma = mg.contraction_densities(n, complex_gamma)
    q = oracle.canonical_quartets(len(specs))
    vals, off = oracle.eri_center_derivatives(specs, q, mg.DERIV_FIELD, mg.DERIV_ORIGIN)
    got = contract_eri_derivatives(specs, atoms, natom, q, off, vals, coulomb, exchange, gamma)
    ref = golden.contraction[f"{name}_field"]
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
