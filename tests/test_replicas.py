"""Multi-rank replica logic on the CPU: two gloo ranks share units without
overlap, agree on the max/sum of per-rank values, and draw distinct fields."""

from __future__ import annotations

import os
import socket

import pytest

from giaoint_gb300.replicas import field_for_rank, partition


def test_partition_covers_without_overlap():
    for count in (0, 1, 7, 64, 6722352):
        for world in (1, 2, 3, 8):
            parts = [partition(count, r, world) for r in range(world)]
            flat = [i for p in parts for i in (p if count < 100 else (p.start, p.stop - 1))]
            if count < 100:
                assert sorted(flat) == list(range(count))
            assert sum(len(p) for p in parts) == count
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        partition(10, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from giaoint_gb300.replicas import field_for_rank, max_over_ranks, partition, sum_over_ranks

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        share = partition(64, rank, world)
        mine = float(len(share)) * (rank + 1)
        q.put((rank, list(share), max_over_ranks(mine), sum_over_ranks(len(share)), field_for_rank(rank)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_and_shares():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, m0, n0, f0), (r1, s1, m1, n1, f1) = out
    assert set(s0).isdisjoint(s1) and sorted(s0 + s1) == list(range(64))
    assert m0 == m1 == 64.0  # 32 units x (rank 1 + 1)
    assert n0 == n1 == 64.0
    assert f0 == field_for_rank(0) and f1 == field_for_rank(1) and f0 != f1
