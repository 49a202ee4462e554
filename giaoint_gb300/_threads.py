"""Thread-count policy kept for API compatibility.

The reference resolves an OpenMP thread budget for every native call
(python/giao_integrals/_threads.py:20-110).  Here all work runs on one GPU, so
``threads`` is validated with the same rules and messages and otherwise has
no effect; ``build_info`` reports the GPU build instead of OpenMP.
"""

from __future__ import annotations

import os
from operator import index

import numpy as np

_override: int | None = None


def _positive(value, name="threads") -> int:
    if isinstance(value, (bool, np.bool_)):
        raise ValueError(f"{name} must be a positive integer")
    try:
        n = index(value)
    except TypeError as error:
        raise ValueError(f"{name} must be a positive integer") from error
    if not 1 <= n <= 2**31 - 1:
        raise ValueError(f"{name} must be a positive integer <= 2147483647")
    return n


def set_num_threads(n: int | None) -> None:
    """Set the process-wide default thread budget (validated, unused on the GPU)."""
    global _override
    _override = None if n is None else _positive(n, "n")


def resolve_num_threads(threads: int | None = None) -> int:
    if threads is not None:
        return _positive(threads)
    if _override is not None:
        return _override
    for name in ("GIAO_NUM_THREADS", "OMP_NUM_THREADS"):
        if name in os.environ:
            try:
                return _positive(int(os.environ[name]), name)
            except ValueError as error:
                raise ValueError(f"{name} must be a positive integer") from error
    return os.cpu_count() or 1


def build_info() -> dict:
    from . import _native as nat

    return {
        "version": nat.lib().gx_version().decode(),
        "backend": "cuda",
        "arch": "sm_103a",
        "library": str(nat.library_path()),
        "openmp_enabled": False,
        "default_threads": resolve_num_threads(),
    }
