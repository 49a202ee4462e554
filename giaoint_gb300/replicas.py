"""Replica sharding for several GPUs: independent work, no data-path collective.

The ERI path shards into independent units (fields of a sweep, quartet
subsets, requests); each rank owns one GPU and evaluates its share alone.
The only cross-rank operations are timing and bookkeeping: a barrier around
the timed region and the maximum of the per-rank times (the whole job ends
when the slowest rank ends).  The Cholesky pivot loop is sequential per
factorisation, so across GPUs it is replicas only.
"""

from __future__ import annotations

import os

__all__ = ["dist_env", "partition", "field_for_rank", "max_over_ranks", "sum_over_ranks"]


def dist_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def partition(count: int, rank: int, world: int) -> range:
    """Contiguous share of ``count`` units for ``rank`` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(count), world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def field_for_rank(rank: int, seed: int = 2026, bmax: float = 0.2) -> tuple[float, float, float]:
    """The field a rank evaluates in the weak-scaling bench: rank 0 the seeded
    random field of the single-GPU workload, rank r > 0 point r of a seeded
    grid in the same ball, so every rank does the same amount of work on a
    different field."""
    from . import synthetic as syn

    if rank == 0:
        return syn.random_field(seed, bmax=bmax)
    return syn.field_grid(64, bmax, seed)[rank % 64]


def _reduce(value: float, op) -> float:
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    device = "cpu"
    if dist.get_backend() == "nccl":
        device = f"cuda:{torch.cuda.current_device()}"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value: float) -> float:
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.MAX)


def sum_over_ranks(value: float) -> float:
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.SUM)
