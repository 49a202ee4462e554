"""On-demand pivoted Cholesky of the Hermitian ordered-pair Coulomb matrix.

Mirrors python/giao_integrals/cholesky.py:16-297: the same ``CholeskyERI``
result type, conventions, validation, pivot policy and stopping rule, with
the selected integrals (``_cholesky_diagonal`` / ``_cholesky_columns``,
src/bindings.cpp:2306-2330) generated on the GPU.  The whole pivot loop
(residual diagonal, argmax, column generation, factor update) runs on the
device through ``gx_cholesky``; only the pivots and factors come back.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

from . import _native as nat
from ._threads import resolve_num_threads
from ._types import Basis, MagneticField, field_arrays

__all__ = ["CholeskyERI", "cholesky_eri", "_cholesky_diagonal", "_cholesky_columns"]


@dataclass(frozen=True)
class CholeskyERI:
    r"""Coulomb factors in the AO order and normalisation of :func:`eri`.

    ``vectors`` is complex128 (rank, nao, nao) with
    (mu nu|lam sig) ~= sum_P L[P,mu,nu] conj(L[P,sig,lam]);
    W[(mu,nu),(lam,sig)] = (nu mu|lam sig) ~= sum_P conj(L[P,mu,nu]) L[P,lam,sig].
    """

    vectors: npt.NDArray[np.complex128]
    pivots: npt.NDArray[np.int64]
    threshold: float
    max_residual_diagonal: float

    def reconstruct(self, slices=None) -> npt.NDArray[np.complex128]:
        if slices is None:
            slices = (slice(None),) * 4
        if len(slices) != 4 or not all(isinstance(s, slice) for s in slices):
            raise ValueError("slices must contain four slices")
        a, b, c, d = slices
        return np.einsum("Pmn,Psl->mnls", self.vectors[:, a, b], self.vectors[:, d, c].conj(), optimize=True)


def _cholesky_diagonal(basis: Basis, pairs, *, field: MagneticField | None = None, threads=None, context=None):
    """float64[n, n] diagonal (mu nu|nu mu) for shell pairs a <= b (src/cholesky.cpp:285-314)."""
    resolve_num_threads(threads)
    ctx = context or nat.default_context()
    p = np.ascontiguousarray(np.asarray(pairs, dtype=np.int64).reshape(-1, 2))
    n = basis.ao_count
    out = np.zeros((n, n), dtype=np.float64)
    B, O = field_arrays(field)
    nat.check(nat.lib().gx_cholesky_diagonal(ctx.handle, basis._device(ctx), nat.i64ptr(p), len(p), nat.dptr(B),
                                             nat.dptr(O), nat.dptr(out.reshape(-1))))
    return out


def _cholesky_columns(basis: Basis, pivots, *, field: MagneticField | None = None, threads=None, context=None):
    """Columns (mu nu|p1 p0) for pivots sharing one shell pair (src/cholesky.cpp:203-323):
    float64[k, n*n] when B == 0 exactly, else complex128[k, n*n]."""
    resolve_num_threads(threads)
    ctx = context or nat.default_context()
    p = np.ascontiguousarray(np.asarray(pivots, dtype=np.int64).reshape(-1, 2))
    n = basis.ao_count
    B, O = field_arrays(field)
    real = bool(np.all(B == 0.0))
    out = np.zeros((len(p), n * n), dtype=np.float64 if real else np.complex128)
    if len(p):
        nat.check(nat.lib().gx_cholesky_columns(ctx.handle, basis._device(ctx), nat.i64ptr(p), len(p), nat.dptr(B),
                                                nat.dptr(O), nat.dptr(out.view(np.float64).reshape(-1))))
    return out


def _validate(threshold, screening_threshold, pivot_batch_size, max_bytes):
    threshold = float(threshold)
    screening_threshold = float(screening_threshold)
    for name, value in (("threshold", threshold), ("screening_threshold", screening_threshold)):
        if not np.isfinite(value) or value < 0:
            raise ValueError(f"{name} must be finite and non-negative")
    if (isinstance(pivot_batch_size, (bool, np.bool_)) or not isinstance(pivot_batch_size, (int, np.integer))
            or pivot_batch_size < 1):
        raise ValueError("pivot_batch_size must be a positive integer")
    if max_bytes is not None and (isinstance(max_bytes, (bool, np.bool_)) or not isinstance(max_bytes, (int, np.integer))
                                  or max_bytes < 0):
        raise ValueError("max_bytes must be a non-negative integer or None")
    return threshold, screening_threshold


def cholesky_eri(basis: Basis, *, field: MagneticField | None = None, threshold: float = 1e-8,
                 screening_threshold: float = 0.0, threads: int | None = None, max_bytes: int | None = None,
                 pivot_batch_size: int = 32) -> CholeskyERI:
    """Factor ERIs without forming the AO tensor or the ordered-pair matrix.

    Pivoted Cholesky acts on W[(mu,nu),(lam,sig)] = (nu mu|lam sig) and stops
    when the largest residual diagonal is <= max(threshold, 64 eps max diag).
    """
    threshold, screening_threshold = _validate(threshold, screening_threshold, pivot_batch_size, max_bytes)
    resolve_num_threads(threads)
    return _cholesky_device(basis, field, threshold, screening_threshold, max_bytes, pivot_batch_size)


def _cholesky_device(basis, field, threshold, screening_threshold, max_bytes, pivot_batch_size, context=None,
                     stats=None):
    """gx_cholesky_factor: the pivot loop resident on the device, the factor
    rows growing there; the vectors are copied out once at the end.  With
    ``stats`` (a dict), the factorisation's work and device times are added
    to it."""
    ctx = context or nat.default_context()
    n = basis.ao_count
    row_bytes = n * n * 16 + 16
    limit = n * n if max_bytes is None else min(n * n, max_bytes // row_bytes)
    B, O = field_arrays(field)
    opts = nat.GxCholeskyOptions(threshold, screening_threshold, int(limit), int(pivot_batch_size))
    lib = nat.lib()
    handle = ctypes.c_void_p()
    rc = lib.gx_cholesky_factor(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), ctypes.byref(opts),
                                ctypes.byref(handle))
    if rc == -6 and "rank capacity" in nat.last_error():
        st = nat.GxCholeskyStats()
        nat.check(lib.gx_cholesky_last_stats(ctx.handle, ctypes.byref(st)))
        raise MemoryError(f"Cholesky ERI output requires at least {(int(st.rank) + 1) * row_bytes} bytes, "
                          f"exceeding max_bytes={max_bytes}")
    nat.check(rc)
    try:
        rank = ctypes.c_int64()
        resid = ctypes.c_double()
        nat.check(lib.gx_cholesky_factors_info(handle, ctypes.byref(rank), None, ctypes.byref(resid), None))
        r = int(rank.value)
        vectors = np.empty((r, n, n), dtype=np.complex128)
        pivots = np.empty((r, 2), dtype=np.int64)
        if r:
            nat.check(lib.gx_cholesky_factors_copy(handle, nat.dptr(vectors.view(np.float64).reshape(-1)),
                                                   nat.i64ptr(pivots)))
        if stats is not None:
            st = nat.GxCholeskyStats()
            nat.check(lib.gx_cholesky_factors_stats(handle, ctypes.byref(st)))
            stats.update(st.as_dict())
    finally:
        lib.gx_cholesky_factors_destroy(handle)
    return CholeskyERI(vectors, pivots, threshold, float(resid.value))
