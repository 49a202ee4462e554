"""Packed requests (gx_eri_batch_packed): ERI requests of different molecules
and fields evaluated in one class-sorted execution.  On a context with stable
launch configurations every request's blocks are bit for bit those of the
request packed alone, in both precision modes, and agree with the ordinary
per-request call and with the oracle."""

from __future__ import annotations

import numpy as np
import pytest

import giaoint_gb300 as gi
from giaoint_gb300 import _native as nat
from giaoint_gb300 import synthetic as syn
from giaoint_gb300.eri import _eri_batch, _eri_batch_packed

pytestmark = pytest.mark.gpu


def _items(count=4, seed=21):
    reqs = syn.serving_requests(count=count, rate=100.0, seed=seed, atoms=(3, 5), max_entries=1 << 17,
                                cholesky_fraction=0.0)
    return [(gi.Basis([gi.Shell.from_record(s) for s in r.shells]), r.quartets, gi.MagneticField(r.field), r)
            for r in reqs]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_packed_equals_alone_bitwise(precision):
    ctx = nat.Context(0)
    nat.check(nat.lib().gx_context_set_stable_launch(ctx.handle, 1))
    items = _items()
    packed = _eri_batch_packed([i[:3] for i in items], precision=precision, context=ctx)
    for it, (off, val) in zip(items, packed):
        (off1, val1), = _eri_batch_packed([it[:3]], precision=precision, context=ctx)
        assert np.array_equal(off, off1)
        assert np.array_equal(val, val1)
        _, _, off2, val2, _, _ = _eri_batch(it[0], it[1], field=it[2], precision=precision, context=ctx)
        assert np.array_equal(off, off2)
        tol = 1e-12 if precision == "fp64" else 1e-10
        assert float(np.abs(val - val2).max(initial=0.0)) <= tol
    ctx.close()


def test_packed_against_oracle(oracle):
    items = _items(3, seed=33)
    packed = _eri_batch_packed([i[:3] for i in items], precision="fp64")
    for (basis, q, field, r), (off, val) in zip(items, packed):
        rng = np.random.default_rng(3)
        pick = np.sort(rng.choice(len(q), min(len(q), 200), replace=False))
        ref, _ = oracle.eri_batch(list(r.shells), np.asarray(q)[pick], tuple(r.field), None, 8)
        got = np.concatenate([val[off[i]:off[i + 1]] for i in pick])
        assert float(np.abs(got - ref).max()) <= 1e-12


def test_packed_validation():
    items = _items(2)
    bad = [(items[0][0], np.array([[0, 0, 0, 99]]), items[0][2])]
    with pytest.raises(IndexError):
        _eri_batch_packed(bad)
    assert _eri_batch_packed([]) == []
