"""Cholesky selections and the pivoted factorisation against the reference."""

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300.eri import _eri_batch
from giaoint_gb300.cholesky import _cholesky_columns, _cholesky_diagonal
from helpers import specs_to_basis

pytestmark = pytest.mark.gpu


def test_selected_diagonal_and_columns_against_oracle(golden, oracle):
    shells = golden.cholesky["shells"]["molecule3"]
    basis = specs_to_basis(shells)
    from oracle.oracle import ShellSpec

    specs = [ShellSpec(tuple(s["center"]), s["l"], s["exponents"], s["coefficients"], s["normalize"]) for s in shells]
    n = basis.ao_count
    ns = len(specs)
    pairs = [(a, b) for a in range(ns) for b in range(a, ns)]
    for B, O in (((0, 0, 0), (0, 0, 0)), ((0.05, -0.03, 0.2), (0.37, -0.29, 0.43))):
        field = gi.MagneticField(B, O)
        d = _cholesky_diagonal(basis, pairs, field=field)
        np.testing.assert_allclose(d, oracle.cholesky_diagonal(specs, pairs, B, O), atol=1e-12)
        off = basis.ao_offsets
        for sa, sb in ((3, 4), (5, 5), (0, 11)):
            piv = [(off[sa] + i, off[sb] + j) for i in range(basis.shells[sa].ao_count)
                   for j in range(basis.shells[sb].ao_count)][:8]
            c = _cholesky_columns(basis, piv, field=field)
            r = oracle.cholesky_columns(specs, piv, B, O)
            assert c.dtype == r.dtype
            assert np.abs(c - r).max() <= 1e-12
            assert c.shape == (len(piv), n * n)


def first_divergence_is_a_tie(basis, field, res, ref_pivots, gap=1e-10):
    """Pivots must equal the reference's wherever the residual-diagonal gap
    between the two choices exceeds 1e-10; after the first (tied) divergence
    the sequences may legitimately differ.  Returns the common prefix length."""
    n = basis.ao_count
    k = 0
    while k < min(len(res.pivots), len(ref_pivots)) and tuple(res.pivots[k]) == tuple(ref_pivots[k]):
        k += 1
    if k == min(len(res.pivots), len(ref_pivots)):
        return k
    ns = len(basis.shells)
    shells = basis.shells
    single = all(s.center == shells[0].center for s in shells)
    diag = _cholesky_diagonal(basis, [(a, b) for a in range(ns) for b in range(a, ns)],
                              field=None if single else field)
    resid = diag.ravel() - np.sum(np.abs(res.vectors[:k].reshape(k, n * n)) ** 2, axis=0)
    mine = res.pivots[k][0] * n + res.pivots[k][1]
    theirs = ref_pivots[k][0] * n + ref_pivots[k][1]
    assert abs(resid[mine] - resid[theirs]) <= gap, (k, resid[mine], resid[theirs])
    return k


def test_cholesky_against_reference_driver(golden):
    """Every golden case of the reference's own driver, including the
    generally contracted two-centre system whose pivots the complex local
    block rule and the reference's raw-column cache decide: the pivot
    sequence must agree up to an exact tie, and in full when there is none."""
    g = golden.cholesky
    for case in g["cases"]:
        basis = specs_to_basis(g["shells"][case["system"]])
        field = gi.MagneticField(case["B"], case["origin"])
        res = gi.cholesky_eri(basis, field=field, threshold=case["threshold"],
                              pivot_batch_size=case["pivot_batch_size"])
        k = first_divergence_is_a_tie(basis, field, res, np.asarray(case["pivots"]))
        if k == len(case["pivots"]):
            assert len(res.pivots) == case["rank"], (case["system"], case["field_label"], case["threshold"])
        assert abs(len(res.pivots) - case["rank"]) <= max(3, case["rank"] // 50)
        assert res.max_residual_diagonal <= max(case["threshold"], 2e-12)
        first = np.array([complex(*x) for x in case["first_vector"]])
        np.testing.assert_allclose(res.vectors[0].ravel()[: len(first)], first, atol=1e-11)


@pytest.mark.parametrize("system", ["contracted", "molecule3"])
def test_cholesky_every_pivot_is_the_reference_choice_or_a_tie(golden, oracle, system):
    """The whole pivot sequence, not only its prefix: the oracle restatement
    of the reference driver (pinned bitwise to the reference's own driver by
    the CPU suite) is replayed along the GPU's pivots, making its own choice
    at every step -- global argmax, the complex local block rule, the
    raw-column cache state -- and every GPU pivot must be that choice or tied
    with it (residual gap <= 1e-10).  The generally contracted two-centre
    system at finite field puts the local rule and the cache in charge."""
    from oracle import oracle as O

    g = golden.cholesky
    specs = [O.ShellSpec(tuple(s["center"]), s["l"], s["exponents"], s["coefficients"], s["normalize"])
             for s in g["shells"][system]]
    basis = specs_to_basis(g["shells"][system])
    for case in [c for c in g["cases"] if c["system"] == system and c["field_label"] == "field"]:
        field = gi.MagneticField(case["B"], case["origin"])
        res = gi.cholesky_eri(basis, field=field, threshold=case["threshold"],
                              pivot_batch_size=case["pivot_batch_size"])
        rep = O.cholesky_eri(oracle, specs, case["B"], case["origin"], threshold=case["threshold"],
                             pivot_batch_size=case["pivot_batch_size"], threads=8, follow=res.pivots)
        assert rep.max_forced_gap <= 1e-10, (case["threshold"], case["pivot_batch_size"], rep.max_forced_gap)
        assert len(rep.pivots) == len(res.pivots) and rep.stopped_by_threshold
        np.testing.assert_allclose(res.vectors, rep.vectors, atol=1e-10)


def test_cholesky_atom140_against_oracle(oracle):
    """The 140-AO even-tempered atom (10s 8p 6d 4f 2g) at B = (0, 0, 0.1),
    threshold 1e-8: rank 873 as the reference path, residual below the
    threshold, pivots equal to the oracle port's up to an exact tie, and the
    reconstruction of seeded blocks within the threshold."""
    import os

    from giaoint_gb300 import synthetic as syn
    from giaoint_gb300.eri import _eri_batch
    from oracle import oracle as O

    recs = syn.cholesky_atom()
    basis = gi.Basis([gi.Shell.from_record(r) for r in recs])
    field = gi.MagneticField((0.0, 0.0, 0.1))
    res = gi.cholesky_eri(basis, field=field, threshold=1e-8)
    assert len(res.pivots) == 873
    assert res.max_residual_diagonal <= 1e-8
    ref = O.cholesky_eri(oracle, recs, (0.0, 0.0, 0.1), None, threshold=1e-8, threads=os.cpu_count() or 1)
    k = first_divergence_is_a_tie(basis, field, res, ref.pivots)
    assert k >= 10
    np.testing.assert_allclose(res.vectors[:k], ref.vectors[:k], atol=1e-10)
    rng = np.random.default_rng(11)
    qs = rng.integers(0, len(recs), size=(24, 4))
    _, shapes, offs, vals, _, _ = _eri_batch(basis, qs, field=field, precision="fp64_exact")
    off = basis.ao_offsets
    worst = 0.0
    for i, q in enumerate(qs):
        sl = tuple(slice(off[x], off[x] + basis.shells[x].ao_count) for x in q)
        blk = vals[offs[i]:offs[i + 1]].reshape(tuple(shapes[i]))
        worst = max(worst, float(np.abs(res.reconstruct(sl) - blk).max()))
    assert worst <= 1e-8 + 2e-12


def test_cholesky_factor_handle_and_stats():
    """gx_cholesky_factor keeps the factors on the device and reports the
    work of the factorisation; the rows grow on the device past the initial
    capacity (8 n rows) without a restart; a rank limit from max_bytes raises
    the reference's MemoryError."""
    from giaoint_gb300.cholesky import _cholesky_device

    # two centres at finite field: rank 254 at 1e-11 on the oracle, n = 24
    basis = gi.Basis([gi.Shell(c, l, [e], [1.0]) for c in ((0.0, 0.0, 0.0), (0.9, -0.4, 0.5)) for l in (0, 1)
                      for e in (0.4, 1.5, 5.0)])
    n = basis.ao_count
    field = gi.MagneticField((0.05, -0.1, 0.2))
    stats = {}
    res = _cholesky_device(basis, field, 1e-11, 0.0, None, 32, stats=stats)
    assert stats["rank"] == len(res.pivots) > 8 * n  # grown past the first 8 n rows
    assert stats["block_evaluations"] >= 1 and stats["column_ms"] > 0 and stats["update_ms"] > 0
    assert stats["update_flops"] > 0 and stats["column_model_flops"] > 0
    assert res.max_residual_diagonal <= 1e-11
    with pytest.raises(MemoryError, match="Cholesky ERI output requires"):
        gi.cholesky_eri(basis, field=field, threshold=1e-11, max_bytes=3 * (n * n * 16 + 16))


def test_cholesky_reconstruction_df(golden):
    shells = golden.cholesky["shells"]["df"]
    basis = specs_to_basis(shells)
    for B in ((0, 0, 0), (0.05, -0.03, 0.2)):
        field = gi.MagneticField(B, (0.37, -0.29, 0.43))
        n = basis.ao_count
        exact = gi.eri(basis, field=field, storage="full", max_bytes=n**4 * 16)
        w = exact.transpose(1, 0, 2, 3).reshape(n * n, -1)
        np.testing.assert_allclose(w, w.conj().T, atol=1e-13)
        for tau in (1e-4, 1e-6, 1e-8, 1e-10, 0):
            res = gi.cholesky_eri(basis, field=field, threshold=tau)
            rec = res.reconstruct()
            atol = tau + 2e-12 if tau else 2e-12
            assert np.max(np.abs(exact - rec)) <= atol
            assert res.max_residual_diagonal <= max(tau, 2e-12)
            residual = w.diagonal().real - np.sum(abs(res.vectors) ** 2, axis=0).ravel()
            assert abs(res.max_residual_diagonal - max(0, residual.max())) < 2e-12
            assert len(np.unique(res.pivots, axis=0)) == len(res.vectors)
            if B == (0, 0, 0):
                np.testing.assert_array_equal(res.vectors.imag, 0)
