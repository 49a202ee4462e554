"""Host logic of the serving loop (no GPU): admission by device footprint,
arrival-order admission, overlap up to the slot count, the slot kept for ERI
requests while Cholesky requests hold the others, rejection of requests
larger than the whole budget, latency summary."""

from __future__ import annotations

import threading
import time

import pytest

from giaoint_gb300 import synthetic as syn
from giaoint_gb300.serving import Server, footprint_bytes, latency_summary


def _trace(count=16):
    return syn.serving_requests(count=count, rate=400.0, seed=5, atoms=(3, 5), max_entries=1 << 16,
                                cholesky_fraction=0.3, cholesky_atoms=(3, 3))


def test_admission_respects_budget_slots_and_arrival_order():
    reqs = _trace()
    fps = [footprint_bytes(r) for r in reqs]
    budget = max(fps) + min(fps)  # the largest request plus one more at most
    lock = threading.Lock()
    live = {"n": 0, "bytes": 0, "max_n": 0, "max_bytes": 0}
    order = []

    def runner(slot, req):
        fp = footprint_bytes(req)
        with lock:
            live["n"] += 1
            live["bytes"] += fp
            live["max_n"] = max(live["max_n"], live["n"])
            live["max_bytes"] = max(live["max_bytes"], live["bytes"])
            order.append(req.arrival)
        time.sleep(0.01)
        with lock:
            live["n"] -= 1
            live["bytes"] -= fp
        return req.kind, 10

    with Server(slots=3, hbm_budget=budget, runner=runner) as srv:
        done = srv.run(reqs)
    assert all(c.error is None for c in done)
    assert live["max_bytes"] <= budget
    assert 1 <= live["max_n"] <= 3
    assert srv.max_reserved <= budget
    by_arrival = sorted(done, key=lambda c: c.arrival)
    admitted = [c.admitted for c in by_arrival]
    assert admitted == sorted(admitted)  # admitted in arrival order
    assert sorted(order) == [c.arrival for c in by_arrival]
    s = latency_summary(done)
    assert s["completed"] == len(reqs)
    assert s["p99_ms"] >= s["p50_ms"] > 0.0
    assert s["eris"] == 10 * len(reqs)


def test_requests_overlap_when_they_fit():
    reqs = _trace(8)
    started = []
    gate = threading.Barrier(2, timeout=5)

    def runner(slot, req):
        started.append(slot)
        if len(started) <= 2:
            gate.wait()  # the first two requests must run at the same time
        return None, 0

    with Server(slots=2, hbm_budget=1 << 50, runner=runner) as srv:
        done = srv.run(reqs, realtime=False)
    assert all(c.error is None for c in done)
    assert srv.max_inflight == 2


def test_oversize_request_is_rejected():
    reqs = _trace(4)
    with Server(slots=1, hbm_budget=1024, runner=lambda s, r: (None, 0)) as srv:
        fut = srv.submit(reqs[0])
        with pytest.raises(MemoryError, match="serving budget"):
            fut.result(timeout=5)


def test_runner_errors_reach_the_caller():
    reqs = _trace(3)

    def runner(slot, req):
        raise ValueError("bad request")

    with Server(slots=2, hbm_budget=1 << 50, runner=runner) as srv:
        fut = srv.submit(reqs[0])
        with pytest.raises(ValueError, match="bad request"):
            fut.result(timeout=5)


def test_per_request_limit_refuses_and_counts():
    """A request estimated above the per-request device-memory limit is
    refused with MemoryError at submission; the rest of the trace is served
    and the summary counts the refusals."""
    reqs = _trace(12)
    fps = sorted(footprint_bytes(r) for r in reqs)
    limit = fps[len(fps) // 2]
    with Server(slots=2, hbm_budget=1 << 50, max_request_bytes=limit, runner=lambda s, r: (None, 1)) as srv:
        done = srv.run(reqs, realtime=False)
    over = sum(footprint_bytes(r) > limit for r in reqs)
    assert over > 0 and srv.refused == over
    refused = [c for c in done if c.error is not None]
    assert len(refused) == over and all(isinstance(c.error, MemoryError) for c in refused)
    assert all("per-request limit" in str(c.error) for c in refused)
    s = latency_summary(done)
    assert s["refused_memory"] == over and s["completed"] == len(reqs) - over


def test_waiting_eri_requests_are_packed_cholesky_never():
    """ERI requests queued behind an admitted ERI request join its pack (up to
    the pack size); a Cholesky request is never packed and ends a pack."""
    reqs = _trace(16)
    packs = []

    def pack_runner(slot, rs):
        packs.append([r.kind for r in rs])
        return [(None, 1) for _ in rs]

    def runner(slot, r):
        packs.append([r.kind])
        if len(packs) == 1:
            time.sleep(0.2)  # the rest of the trace queues up behind the first request
        return None, 1

    with Server(slots=1, hbm_budget=1 << 50, runner=runner, pack_runner=pack_runner, pack=4) as srv:
        done = srv.run(reqs, realtime=False)
    assert all(c.error is None for c in done)
    assert sum(len(p) for p in packs) == len(reqs)
    assert max(len(p) for p in packs) <= 4
    assert srv.max_pack == max(len(p) for p in packs) >= 2
    for p in packs:
        if len(p) > 1:
            assert all(k == "eri" for k in p)
    # arrival order is kept across packs
    kinds = [k for p in packs for k in p]
    assert kinds == [r.kind for r in reqs]


def test_eri_requests_pass_cholesky_requests_beyond_the_long_slots():
    """With two slots, Cholesky requests hold at most one: a second Cholesky
    request waits, and an ERI request queued behind it is admitted at once on
    the free slot and finishes first."""
    reqs = syn.serving_requests(count=16, rate=400.0, seed=5, atoms=(3, 5), max_entries=1 << 16,
                                cholesky_fraction=0.5, cholesky_atoms=(3, 3))
    chol = [r for r in reqs if r.kind == "cholesky"][:2]
    eri = [r for r in reqs if r.kind == "eri"][:1]
    assert len(chol) == 2 and len(eri) == 1

    def runner(slot, r):
        time.sleep(0.3 if r.kind == "cholesky" else 0.0)
        return r.kind, 1

    with Server(slots=2, hbm_budget=1 << 50, runner=runner, long_slots=1) as srv:
        assert srv.long_slots == 1
        futs = [srv.submit(chol[0], 0), srv.submit(chol[1], 1), srv.submit(eri[0], 2)]
        a, b, c = (f.result(timeout=10) for f in futs)
    assert c.admitted < b.admitted  # the ERI request passed the waiting Cholesky request
    assert c.finished < a.finished
    assert b.admitted >= a.finished - 1e-3  # the second Cholesky request waited for the first
    with pytest.raises(ValueError, match="long_slots"):
        Server(slots=2, long_slots=3, runner=lambda s_, r: (None, 0))
