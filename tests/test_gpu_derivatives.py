"""ERI centre derivatives on the GPU against the reference library's blocks
(golden derivatives.npz) and the oracle, the translation sum rule at larger
sizes, and the reference Python API (eri_derivative_batches,
eri_center_derivatives_shell, primitive_eri_center_derivatives).

Tolerance: FP64 blocks agree with the reference within 1e-12 of
max(1, max |block|) per element (the derivative of a steep primitive is
sqrt(alpha) larger than its integral)."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300 import _native as nat
from giaoint_gb300 import synthetic as syn
from giaoint_gb300.eri import _eri_batch, _eri_derivative_batch

from conftest import derivative_systems
from helpers import basis_from_records
from test_oracle_golden import derivative_sum_rule_residual

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _basis(specs):
    return gi.Basis([gi.Shell(s.center, s.l, s.exponents, np.asarray(s.coefficients), normalize=s.normalize)
                     for s in specs])


def _field(B, origin):
    return gi.MagneticField(tuple(B), gauge_origin=tuple(origin))


def _close(vals, ref):
    assert vals.shape == ref.shape
    return np.abs(vals - ref).max() <= TOL * max(1.0, np.abs(ref).max())


def test_blocks_match_reference(golden):
    g = golden.derivatives
    for name, specs, q in derivative_systems(g):
        basis = _basis(specs)
        for label, field in (("field", _field(g["field"], g["origin"])), ("zero", None)):
            kq, shapes, offsets, values, requested, screened = _eri_derivative_batch(basis, q, field=field)
            np.testing.assert_array_equal(kq, q)
            np.testing.assert_array_equal(offsets, g[f"{name}_offsets"])
            assert requested == len(q) and screened == 0
            assert (shapes[:, :2] == (4, 3)).all()
            assert _close(values, g[f"{name}_{label}"]), (name, label)


def test_molecule_matches_oracle(oracle):
    """Seeded quartets of the 12-atom molecule (s, p, d shells, contracted)
    at a finite field against the oracle."""
    recs = syn.random_molecule(2026, natoms=12)
    basis = basis_from_records(recs)
    ns = len(recs)
    rng = np.random.default_rng(7)
    q = rng.integers(0, ns, size=(40, 4)).astype(np.uint32)
    B, O = (0.03, 0.11, -0.07), (0.5, -0.2, 0.3)
    _, _, offsets, values, _, _ = _eri_derivative_batch(basis, q, field=gi.MagneticField(B, gauge_origin=O))
    ref, roff = oracle.eri_center_derivatives(recs, q, B, O)
    np.testing.assert_array_equal(offsets, roff)
    assert _close(values, ref)


def test_translation_sum_rule_full_size():
    """2000 canonical quartets of the 12-atom molecule: the four slot
    derivatives sum to i (k_a - k_b + k_c - k_d) times the GPU's own ERI
    block (a size-independent property), at zero and finite field."""
    from oracle.oracle import as_specs

    recs = syn.random_molecule(2026, natoms=12)
    basis = basis_from_records(recs)
    specs = as_specs(recs)
    q = gi.canonical_quartets(len(recs))
    q = q[np.random.default_rng(3).choice(len(q), 2000, replace=False)]
    for B, O in (((0.0, 0.0, 0.0), (0.0, 0.0, 0.0)), ((0.05, -0.08, 0.12), (0.4, 0.1, -0.6))):
        field = gi.MagneticField(B, gauge_origin=O)
        _, _, offsets, values, _, _ = _eri_derivative_batch(basis, q, field=field)
        _, _, eoff, eri, _, _ = _eri_batch(basis, q, field=field, precision="fp64_exact")
        assert derivative_sum_rule_residual(specs, q, offsets, values, eri, eoff, B, O) <= 1e-11


def test_batches_stream_and_validate(golden):
    g = golden.derivatives
    (name, specs, q), _ = derivative_systems(g)
    basis = _basis(specs)
    field = _field(g["field"], g["origin"])
    one = list(gi.eri_derivative_batches(basis, field=field, quartets=q.tolist()))
    assert len(one) == 1 and isinstance(one[0], gi.EriDerivativeBatch)
    small = list(gi.eri_derivative_batches(basis, field=field, quartets=q.tolist(), target_bytes=20000))
    assert len(small) > 3
    joined = np.concatenate([b.values for b in small])
    np.testing.assert_array_equal(joined, one[0].values)
    blk = one[0].block(2)
    assert blk.shape == tuple(one[0].shapes[2]) and blk.shape[:2] == (4, 3)
    assert np.shares_memory(blk, one[0].values)
    assert _close(one[0].values, g[f"{name}_field"])
    assert list(gi.eri_derivative_batches(basis, quartets=[])) == []
    with pytest.raises(IndexError):
        list(gi.eri_derivative_batches(basis, quartets=[(0, 0, 0, len(specs))]))
    with pytest.raises(ValueError, match="four indices"):
        list(gi.eri_derivative_batches(basis, quartets=[(0, 0, 0)]))
    with pytest.raises(ValueError, match="target_bytes"):
        list(gi.eri_derivative_batches(basis, target_bytes=0))
    with pytest.raises(ValueError, match="screening_threshold"):
        list(gi.eri_derivative_batches(basis, screening_threshold=-1.0))
    with pytest.raises(ValueError, match="derivative bounds"):
        _eri_derivative_batch(basis, q, screening_threshold=1e-10)


def test_shell_and_primitive_api(golden, oracle):
    g = golden.derivatives
    _, (name, specs, q) = derivative_systems(g)
    basis = _basis(specs)
    field = _field(g["field"], g["origin"])
    shells = basis.shells
    off = g[f"{name}_offsets"]
    for i, x in enumerate(q):
        blk = gi.eri_center_derivatives_shell(*(shells[k] for k in x), field=field)
        ref = g[f"{name}_field"][off[i]:off[i + 1]].reshape(blk.shape)
        assert _close(blk, ref)
    x = q[1]
    shape = (4, 3) + tuple(shells[k].ao_count for k in x)
    out = np.empty(shape, dtype=np.complex128)
    assert gi.eri_center_derivatives_shell(*(shells[k] for k in x), field=field, out=out) is out
    with pytest.raises(ValueError, match="incorrect shape"):
        gi.eri_center_derivatives_shell(*(shells[k] for k in x),
                                        out=np.empty((4, 3, 1, 1, 1, 1), dtype=np.complex128))
    # single primitives, normalised and not, against the oracle's one-primitive shells
    prims = [gi.PrimitiveGaussian(0.7, (0.1, 0.0, -0.3), (1, 0, 1), coefficient=0.8),
             gi.PrimitiveGaussian(1.3, (0.0, 0.5, 0.2), (0, 2, 0), coefficient=1.1, normalized=False),
             gi.PrimitiveGaussian(0.4, (-0.6, 0.2, 0.1), (0, 0, 0)),
             gi.PrimitiveGaussian(2.1, (0.3, -0.4, 0.5), (1, 1, 1), coefficient=-0.5)]
    v = gi.primitive_eri_center_derivatives(*prims, field=field)
    assert v.shape == (4, 3)
    recs = [syn.ShellRecord(p.center, sum(p.angular), (p.exponent,), ((1.0,),), False) for p in prims]
    blk, _ = oracle.eri_center_derivatives(recs, [(0, 1, 2, 3)], tuple(g["field"]), tuple(g["origin"]))
    dims = [len(gi.cartesian_components(sum(p.angular))) for p in prims]
    blk = blk.reshape([4, 3] + dims)
    picks = [gi.cartesian_components(sum(p.angular)).index(tuple(p.angular)) for p in prims]
    expect = blk[:, :, picks[0], picks[1], picks[2], picks[3]] * (0.8 * 1.1 * -0.5)
    expect = expect / gi.primitive_normalization(1.3, (0, 2, 0))
    assert np.abs(v - expect).max() <= TOL * max(1.0, np.abs(expect).max())


def test_device_entry_matches_host(golden):
    torch = pytest.importorskip("torch")
    g = golden.derivatives
    (name, specs, q), _ = derivative_systems(g)
    basis = _basis(specs)
    ctx = nat.default_context()
    B = np.ascontiguousarray(g["field"], dtype=np.float64)
    O = np.ascontiguousarray(g["origin"], dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.uint32)
    total = int(g[f"{name}_offsets"][-1])
    dev = torch.empty(total, dtype=torch.complex128, device="cuda:0")
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    ms = ctypes.c_float()
    nat.check(nat.lib().gx_eri_center_derivatives_device(
        ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), nat.u32ptr(q), len(q), nat.i64ptr(offsets),
        ctypes.c_void_p(dev.data_ptr()), total, ctypes.byref(ms)))
    torch.cuda.synchronize()
    host = _eri_derivative_batch(basis, q, field=_field(B, O))[3]
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    np.testing.assert_array_equal(offsets, g[f"{name}_offsets"])
    # a too-small buffer is an error, not an overrun
    with pytest.raises(ValueError, match="too small"):
        nat.check(nat.lib().gx_eri_center_derivatives_device(
            ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), nat.u32ptr(q), len(q), nat.i64ptr(offsets),
            ctypes.c_void_p(dev.data_ptr()), total - 1, ctypes.byref(ms)))


def test_derivative_bounds_match_reference_and_bound_blocks(golden):
    """GPU derivative Schwarz factors against the reference's
    (EriDerivativeSchwarzBounds), and every block bounded by its quartet
    bound (the reference's own property, test_eri_derivative_batches.py)."""
    from giaoint_gb300.eri import _EriDerivativeSchwarzBounds

    g = golden.derivatives
    for name, specs, q in derivative_systems(g):
        basis = _basis(specs)
        for label, field in (("field", _field(g["field"], g["origin"])), ("zero", None)):
            bounds = _EriDerivativeSchwarzBounds(basis, field=field)
            ns = len(specs)
            np.testing.assert_allclose(bounds.values.reshape(ns, ns), g[f"{name}_bounds_{label}"], rtol=1e-12)
            np.testing.assert_allclose(bounds.ordinary.reshape(ns, ns), g[f"{name}_schwarz_{label}"], rtol=1e-12)
            off = g[f"{name}_offsets"]
            vals = g[f"{name}_{label}"]
            qb = bounds.quartet_bounds(q)
            for i in range(len(q)):
                assert np.abs(vals[off[i]:off[i + 1]]).max() <= qb[i] * (1 + 1e-13)
                assert qb[i] == bounds.quartet_bound(tuple(int(x) for x in q[i]))
            with pytest.raises(IndexError):
                bounds.quartet_bound((0, 0, 0, ns))


def test_derivative_screening_is_safe_and_tied_to_basis_and_field(golden):
    """Screening at the median quartet bound drops only quartets whose every
    derivative component is below the threshold, keeps the rest unchanged,
    and refuses bounds built for another basis object or field."""
    from giaoint_gb300.eri import _EriDerivativeSchwarzBounds

    shells = [gi.Shell((0.1, -0.2, 0.3), 0, [0.8], [1.0]), gi.Shell((4.0, 0.0, 0.0), 1, [0.9], [1.0]),
              gi.Shell((0.5, 0.3, -0.2), 2, [1.1, 0.4], [0.6, 0.5])]
    basis = gi.Basis(shells)
    q = [tuple(int(x) for x in r) for r in np.ndindex(3, 3, 3, 3)]
    for field in (None, gi.MagneticField((0.05, -0.02, 0.1), gauge_origin=(0.3, -0.1, 0.2))):
        bounds = _EriDerivativeSchwarzBounds(basis, field=field)
        threshold = float(np.median(bounds.quartet_bounds(q)))
        full = {tuple(int(x) for x in r): b.block(i) for b in gi.eri_derivative_batches(basis, field=field, quartets=q)
                for i, r in enumerate(b.quartets)}
        batches = list(gi.eri_derivative_batches(basis, field=field, quartets=q, screening_threshold=threshold,
                                                 target_bytes=4000))
        assert sum(b.requested_count for b in batches) == len(q)
        screened = sum(b.screened_count for b in batches)
        assert 0 < screened < len(q)
        kept = set()
        for b in batches:
            for i, r in enumerate(b.quartets):
                r = tuple(int(x) for x in r)
                kept.add(r)
                np.testing.assert_array_equal(b.block(i), full[r])
        dropped = [np.abs(full[r]).max() for r in q if r not in kept]
        assert len(dropped) == screened
        assert max(dropped) < threshold and any(v > 1e-20 for v in dropped)
        other = gi.Basis(shells)
        for changed_basis, changed_field in ((other, field), (basis, gi.MagneticField((0.0, 0.0, 0.3)))):
            with pytest.raises(ValueError, match="do not match"):
                _eri_derivative_batch(changed_basis, [(0, 0, 0, 0)], field=changed_field, screening_threshold=1e-8,
                                      bounds=bounds)


def test_derivatives_match_finite_differences():
    """Slot derivatives of a shell moved as a whole (both occurrences of a
    repeated shell) against a Richardson-extrapolated central difference of
    the GPU's own ERIs with displaced centres."""
    centers = np.array([[0.1, -0.2, 0.3], [-0.3, 0.4, 0.2]])

    def shells(c):
        return [gi.Shell(tuple(c[0]), 0, [0.8], [1.0]), gi.Shell(tuple(c[1]), 1, [0.6], [1.0])]

    q = (0, 1, 0, 1)
    for field in (None, gi.MagneticField((0.05, -0.1, 0.2), gauge_origin=(0.1, 0.2, -0.3))):
        block = next(gi.eri_derivative_batches(gi.Basis(shells(centers)), quartets=[q], field=field)).block(0)
        for center in range(2):
            for axis in range(3):
                def value(step):
                    c = centers.copy()
                    c[center, axis] += step
                    s = shells(c)
                    return gi.eri_shell(*[s[k] for k in q], field=field)

                h = 1e-3
                d1 = (value(h) - value(-h)) / (2 * h)
                d2 = (value(h / 2) - value(-h / 2)) / h
                expected = (4 * d2 - d1) / 3
                actual = block[[k for k, s in enumerate(q) if s == center], axis].sum(axis=0)
                np.testing.assert_allclose(actual, expected, atol=3e-10, rtol=3e-9)


def test_magnetic_derivatives_match_reference(golden, oracle):
    """d/dB_b blocks (3, na, nb, nc, nd) against the reference library's
    (golden) and the oracle's, through the batch entry, the shell API and
    the primitive API."""
    from giaoint_gb300.eri import _eri_magnetic_derivative_blocks

    g = golden.derivatives
    for name, specs, q in derivative_systems(g):
        basis = _basis(specs)
        for label, field in (("field", _field(g["field"], g["origin"])), ("zero", None)):
            offsets, values = _eri_magnetic_derivative_blocks(basis, q, field=field)
            ref = g[f"{name}_magnetic_{label}"]
            assert _close(values, ref), (name, label)
            if name == "hand":
                for i, x in enumerate(q):
                    blk = gi.eri_magnetic_derivatives_shell(*(basis.shells[k] for k in x), field=field)
                    assert _close(blk.ravel(), ref[offsets[i]:offsets[i + 1]])
    field = _field(g["field"], g["origin"])
    prims = [gi.PrimitiveGaussian(0.9, (0.2, -0.1, 0.0), (0, 1, 1), coefficient=1.2),
             gi.PrimitiveGaussian(0.5, (-0.4, 0.3, 0.2), (1, 0, 0), normalized=False),
             gi.PrimitiveGaussian(1.7, (0.1, 0.6, -0.3), (2, 0, 0), coefficient=0.7),
             gi.PrimitiveGaussian(0.3, (0.0, -0.5, 0.4), (0, 0, 0))]
    v = gi.primitive_eri_magnetic_derivatives(*prims, field=field)
    recs = [syn.ShellRecord(p.center, sum(p.angular), (p.exponent,), ((1.0,),), False) for p in prims]
    blk, _ = oracle.eri_magnetic_derivatives(recs, [(0, 1, 2, 3)], tuple(g["field"]), tuple(g["origin"]))
    dims = [len(gi.cartesian_components(sum(p.angular))) for p in prims]
    picks = [gi.cartesian_components(sum(p.angular)).index(tuple(p.angular)) for p in prims]
    expect = blk.reshape([3] + dims)[:, picks[0], picks[1], picks[2], picks[3]] * (1.2 * 0.7)
    expect = expect / gi.primitive_normalization(0.5, (1, 0, 0))
    assert v.shape == (3,)
    assert np.abs(v - expect).max() <= TOL * max(1.0, np.abs(expect).max())


def test_magnetic_derivatives_match_field_differences():
    """2000 canonical quartets of the 12-atom molecule: d/dB_b against a
    Richardson-extrapolated central difference of the GPU's own FP64-exact
    ERIs at B +- h e_b (fixed gauge origin), at zero and finite field."""
    from giaoint_gb300.eri import _eri_magnetic_derivative_blocks

    recs = syn.random_molecule(2026, natoms=12)
    basis = basis_from_records(recs)
    q = gi.canonical_quartets(len(recs))
    q = q[np.random.default_rng(11).choice(len(q), 2000, replace=False)]
    O = (0.4, 0.1, -0.6)
    for B in ((0.0, 0.0, 0.0), (0.05, -0.08, 0.12)):
        offsets, values = _eri_magnetic_derivative_blocks(basis, q, field=gi.MagneticField(B, gauge_origin=O))

        def eri_at(b, step):
            Bs = list(B)
            Bs[b] += step
            return _eri_batch(basis, q, field=gi.MagneticField(tuple(Bs), gauge_origin=O),
                              precision="fp64_exact")[3]

        _, _, eoff, _, _, _ = _eri_batch(basis, q, field=gi.MagneticField(B, gauge_origin=O))
        sizes = np.diff(eoff)
        for b in range(3):
            h = 1e-3
            d1 = (eri_at(b, h) - eri_at(b, -h)) / (2 * h)
            d2 = (eri_at(b, h / 2) - eri_at(b, -h / 2)) / h
            fd = (4 * d2 - d1) / 3
            got = np.concatenate([values[offsets[i] + b * sizes[i]:offsets[i] + (b + 1) * sizes[i]]
                                  for i in range(len(q))])
            assert np.abs(got - fd).max() <= 1e-9 * max(1.0, np.abs(fd).max())


def test_mixed_derivatives_match_reference(golden, oracle):
    """d2/dR dB blocks (4, 3, 3, na, nb, nc, nd) against the reference
    library's (golden) through the quartet entry and the shell API, and the
    primitive API against the oracle's one-primitive shells."""
    from giaoint_gb300.eri import _eri_mixed_derivative_blocks

    g = golden.derivatives
    for name, specs, _q in derivative_systems(g):
        basis = _basis(specs)
        q = g[f"{name}_mixed_quartets"]
        for label, field in (("field", _field(g["field"], g["origin"])), ("zero", None)):
            offsets, values = _eri_mixed_derivative_blocks(basis, q, field=field)
            ref = g[f"{name}_mixed_{label}"]
            assert _close(values, ref), (name, label)
            x = q[0]
            blk = gi.eri_mixed_derivatives_shell(*(basis.shells[k] for k in x), field=field)
            assert blk.shape[:3] == (4, 3, 3)
            assert _close(blk.ravel(), ref[offsets[0]:offsets[1]])
    field = _field(g["field"], g["origin"])
    prims = [gi.PrimitiveGaussian(0.9, (0.2, -0.1, 0.0), (0, 1, 0), coefficient=1.2),
             gi.PrimitiveGaussian(0.5, (-0.4, 0.3, 0.2), (1, 0, 0), normalized=False),
             gi.PrimitiveGaussian(1.7, (0.1, 0.6, -0.3), (0, 0, 1), coefficient=0.7),
             gi.PrimitiveGaussian(0.3, (0.0, -0.5, 0.4), (0, 0, 0))]
    v = gi.primitive_eri_mixed_derivatives(*prims, field=field)
    recs = [syn.ShellRecord(p.center, sum(p.angular), (p.exponent,), ((1.0,),), False) for p in prims]
    blk, _ = oracle.eri_mixed_derivatives(recs, [(0, 1, 2, 3)], tuple(g["field"]), tuple(g["origin"]))
    dims = [len(gi.cartesian_components(sum(p.angular))) for p in prims]
    picks = [gi.cartesian_components(sum(p.angular)).index(tuple(p.angular)) for p in prims]
    expect = blk.reshape([4, 3, 3] + dims)[:, :, :, picks[0], picks[1], picks[2], picks[3]] * (1.2 * 0.7)
    expect = expect / gi.primitive_normalization(0.5, (1, 0, 0))
    assert v.shape == (4, 3, 3)
    assert np.abs(v - expect).max() <= TOL * max(1.0, np.abs(expect).max())


def test_mixed_derivatives_match_field_differences_of_centre_derivatives():
    """d2/dR dB against a Richardson central difference in B of the GPU's
    own centre derivatives (fixed gauge origin), on 40 quartets of a
    three-atom molecule."""
    from giaoint_gb300.eri import _eri_mixed_derivative_blocks

    recs = syn.random_molecule(5, natoms=3, box=4.0)
    basis = basis_from_records(recs)
    q = gi.canonical_quartets(len(recs))
    q = q[np.random.default_rng(17).choice(len(q), 40, replace=False)]
    B0, O = np.array([0.04, -0.06, 0.09]), (0.3, -0.2, 0.1)
    offsets, mixed = _eri_mixed_derivative_blocks(basis, q, field=gi.MagneticField(tuple(B0), gauge_origin=O))

    def centre(Bv):
        return _eri_derivative_batch(basis, q, field=gi.MagneticField(tuple(Bv), gauge_origin=O))

    _, _, coff, _, _, _ = centre(B0)
    sizes = np.diff(coff) // 12
    for b in range(3):
        h = 1e-3
        e = np.eye(3)[b]
        d1 = (centre(B0 + h * e)[3] - centre(B0 - h * e)[3]) / (2 * h)
        d2 = (centre(B0 + h / 2 * e)[3] - centre(B0 - h / 2 * e)[3]) / h
        fd = (4 * d2 - d1) / 3
        for i in range(len(q)):
            m = mixed[offsets[i]:offsets[i + 1]].reshape(4, 3, 3, -1)[:, :, b, :]
            f = fd[coff[i]:coff[i + 1]].reshape(4, 3, -1)
            assert np.abs(m - f).max() <= 1e-8 * max(1.0, np.abs(f).max())
