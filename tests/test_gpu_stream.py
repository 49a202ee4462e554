"""Streaming consumer (gx_eri_for_each): every kept quartet reaches the
consumer once, in input order, with the values of the packed batch call;
screening drops the same quartets; a list of many chunks streams through the
two host buffers; a consumer that raises stops the call and the context stays
usable."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300 import _native as nat
from giaoint_gb300 import synthetic as syn
from giaoint_gb300.eri import _eri_batch, evaluate_eri_shell_quartets

pytestmark = pytest.mark.gpu


def _molecule(natoms, seed):
    recs = syn.random_molecule(seed, natoms=natoms)
    return recs, gi.Basis([gi.Shell.from_record(r) for r in recs]), gi.MagneticField(syn.random_field(seed))


def _collect(basis, q, field, **kw):
    got_q, got_v = [], []

    def consumer(quartet, block):
        got_q.append(quartet)
        got_v.append(block.copy())

    stats = evaluate_eri_shell_quartets(basis, q, consumer, field=field, **kw)
    return got_q, got_v, stats


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stream_equals_packed_batch(precision):
    recs, basis, field = _molecule(4, 11)
    rng = np.random.default_rng(5)
    ns = len(recs)
    q = rng.integers(0, ns, size=(3000, 4))  # arbitrary order, repeats and non-canonical quartets
    got_q, got_v, st = _collect(basis, q, field, precision=precision, screening_threshold=1e-9)
    kept, shapes, off, val, requested, screened = _eri_batch(basis, q, field=field, precision=precision,
                                                             screening_threshold=1e-9)
    assert requested == st["requested"] == len(q)
    assert screened == st["screened"] and st["computed"] == len(kept) == len(got_q)
    assert screened > 0  # the threshold really screens some quartets of this list
    assert [tuple(x) for x in kept.tolist()] == got_q
    for i, blk in enumerate(got_v):
        assert blk.shape == tuple(shapes[i])
        np.testing.assert_array_equal(blk.ravel(), val[off[i]:off[i + 1]])


def test_stream_against_oracle(oracle):
    recs, basis, field = _molecule(3, 17)
    q = gi.canonical_quartets(len(recs))
    got_q, got_v, _ = _collect(basis, q, field)
    assert got_q == [tuple(x) for x in q.tolist()]
    pick = np.arange(0, len(q), max(1, len(q) // 300))
    ref, _ = oracle.eri_batch(list(recs), q[pick], tuple(field.B), None, 8)
    got = np.concatenate([got_v[i].ravel() for i in pick])
    assert float(np.abs(got - ref).max()) <= 1e-12


def test_stream_many_chunks():
    # the 200,000 widest quartets of the 12-atom molecule in a shuffled order:
    # ~8e7 complex elements, about ten chunks of 2^23 through the two host
    # buffers
    recs, basis, field = _molecule(12, 2026)
    q = gi.canonical_quartets(len(recs))
    sizes = np.array([s.ao_count for s in basis.shells])
    widest = np.argsort(-np.prod(sizes[q.astype(np.int64)], axis=1), kind="stable")[:200_000]
    q = q[np.random.default_rng(8).permutation(widest)]
    kept, shapes, off, val, _, _ = _eri_batch(basis, q, field=field)
    count = [0]
    worst = [0.0]

    def consumer(quartet, block):
        i = count[0]
        assert quartet == tuple(kept[i].tolist())
        worst[0] = max(worst[0], float(np.abs(block.ravel() - val[off[i]:off[i + 1]]).max()))
        count[0] += 1

    st = evaluate_eri_shell_quartets(basis, q, consumer, field=field)
    assert count[0] == len(q) == st["computed"]
    assert int(off[-1]) > 8 * (1 << 23)  # more than eight chunks
    assert worst[0] <= 1e-12  # chunk plans group primitive sums differently from the whole list's


def test_consumer_exception_stops_and_context_survives():
    recs, basis, field = _molecule(3, 4)
    q = gi.canonical_quartets(len(recs))
    seen = []

    class Stop(Exception):
        pass

    def consumer(quartet, block):
        seen.append(quartet)
        if len(seen) == 5:
            raise Stop("enough")

    with pytest.raises(Stop):
        evaluate_eri_shell_quartets(basis, q, consumer, field=field)
    assert len(seen) == 5
    got_q, _, st = _collect(basis, q[:10], field)
    assert len(got_q) == 10 and st["computed"] == 10


def test_stream_validation():
    recs, basis, field = _molecule(3, 4)
    with pytest.raises(ValueError, match="must not be null"):
        evaluate_eri_shell_quartets(basis, [(0, 0, 0, 0)], None)
    with pytest.raises(IndexError):
        evaluate_eri_shell_quartets(basis, [(0, 0, 0, 99)], lambda q, b: None)
    with pytest.raises(ValueError, match="finite and non-negative"):
        evaluate_eri_shell_quartets(basis, [(0, 0, 0, 0)], lambda q, b: None, screening_threshold=-1.0)
    assert evaluate_eri_shell_quartets(basis, np.zeros((0, 4), dtype=np.int64), lambda q, b: None)["computed"] == 0
    rc = nat.lib().gx_eri_for_each(nat.default_context().handle, basis._device(nat.default_context()), None, None,
                                   None, 0, 0, 0.0, 0.0, nat.QUARTET_CONSUMER(), None, None)
    assert rc == -1 and "must not be null" in nat.last_error()


def test_overlapped_host_copies_equal_one_range():
    # host output in page-locked memory, copied after the evaluation, in input
    # ranges whose copies overlap the evaluation of later ranges, or class by
    # class as the classes finish: with size-independent launch configurations
    # the values are bit for bit the same
    torch = pytest.importorskip("torch")
    import ctypes

    recs, basis, field = _molecule(12, 2026)
    q = gi.canonical_quartets(len(recs))
    sizes = np.array([s.ao_count for s in basis.shells])
    widest = np.argsort(-np.prod(sizes[q.astype(np.int64)], axis=1), kind="stable")[:100_000]
    q = np.ascontiguousarray(q[np.sort(widest)])
    total = int(np.prod(sizes[q.astype(np.int64)], axis=1).sum())
    assert total >= 1 << 25
    ctx = nat.Context(0)
    lib = nat.lib()
    nat.check(lib.gx_context_set_stable_launch(ctx.handle, 1))
    from giaoint_gb300._types import field_arrays

    Bv, Ov = field_arrays(field)
    results = []
    for parts, share in ((1, 0.0), (3, 0.0), (2, 0.7), (0, 0.0)):
        nat.check(lib.gx_context_set_copy_parts(ctx.handle, parts, share))
        host = torch.zeros(2 * total, dtype=torch.float64, pin_memory=True)
        off = np.zeros(len(q) + 1, dtype=np.int64)
        st = nat.GxStats()
        nat.check(lib.gx_eri_batch(ctx.handle, basis._device(ctx), nat.dptr(Bv), nat.dptr(Ov), nat.u32ptr(q),
                                   len(q), 1, 1e-6, 0.0, None, nat.i64ptr(off),
                                   ctypes.cast(host.data_ptr(), ctypes.POINTER(ctypes.c_double)), total,
                                   ctypes.byref(st)))
        assert st.computed == len(q) and int(off[-1]) == total
        results.append(host.numpy().copy())
    for other in results[1:]:  # ranges, and (parts 0) each class copied as it finishes
        assert np.array_equal(results[0], other)
    with pytest.raises(ValueError):
        nat.check(lib.gx_context_set_copy_parts(ctx.handle, -1, 0.0))
    ctx.close()
