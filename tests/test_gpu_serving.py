"""Serving on the GPU: every request gives the same result alone and in a
mix of overlapping requests (ERI blocks bit for bit, Cholesky vectors and
pivots within 1e-12), and the trace reports p50/p99 latency."""

from __future__ import annotations

import numpy as np
import pytest

from giaoint_gb300 import synthetic as syn
from giaoint_gb300.serving import Server, latency_summary

pytestmark = pytest.mark.gpu


def _compare(kind, a, b):
    if kind == "eri":
        for x, y in zip(a[:4], b[:4]):
            assert np.array_equal(x, y)
    else:
        assert np.array_equal(a.pivots, b.pivots)
        assert float(np.max(np.abs(a.vectors - b.vectors), initial=0.0)) <= 1e-12


def test_results_alone_equal_results_in_the_mix():
    reqs = syn.serving_requests(count=10, rate=1000.0, seed=9, atoms=(3, 6), max_entries=1 << 18,
                                cholesky_fraction=0.3, cholesky_atoms=(3, 3), thresholds=(1e-6, 1e-7))
    with Server(slots=1) as alone:
        ref = [alone.submit(r).result() for r in reqs]
    with Server(slots=4) as mix:
        done = mix.run(reqs)
    assert mix.max_inflight >= 2  # the requests really overlapped
    with Server(slots=1, precision="fp64") as packed:
        done_packed = packed.run(reqs, realtime=False)  # a queue forms behind one slot: ERI requests are packed
    for r, c0, c1 in zip(reqs, ref, done_packed):
        assert c1.error is None
        _compare(r.kind, c0.result, c1.result)
    for r, c0, c1 in zip(reqs, ref, done):
        assert c1.error is None
        _compare(r.kind, c0.result, c1.result)
    s = latency_summary(done)
    assert s["completed"] == len(reqs) and s["p99_ms"] >= s["p50_ms"] > 0.0
