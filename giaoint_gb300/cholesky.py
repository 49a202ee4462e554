"""On-demand pivoted Cholesky of the Hermitian ordered-pair Coulomb matrix.

Mirrors python/giao_integrals/cholesky.py:16-297: the same ``CholeskyERI``
result type, conventions, validation, pivot policy and stopping rule, with
the selected integrals (``_cholesky_diagonal`` / ``_cholesky_columns``,
src/bindings.cpp:2306-2330) generated on the GPU.  ``backend="device"``
(the default) runs the whole pivot loop on the GPU through ``gx_cholesky``;
``backend="host"`` keeps the reference's NumPy loop over GPU columns.
"""

from __future__ import annotations

import ctypes
from collections import OrderedDict
from dataclasses import dataclass

import numpy as np
import numpy.typing as npt

from . import _native as nat
from ._threads import resolve_num_threads
from ._types import Basis, MagneticField, field_arrays
from .eri import eri_schwarz_bounds

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
                 pivot_batch_size: int = 32, backend: str = "device") -> CholeskyERI:
    """Factor ERIs without forming the AO tensor or the ordered-pair matrix.

    Pivoted Cholesky acts on W[(mu,nu),(lam,sig)] = (nu mu|lam sig) and stops
    when the largest residual diagonal is <= max(threshold, 64 eps max diag).
    """
    threshold, screening_threshold = _validate(threshold, screening_threshold, pivot_batch_size, max_bytes)
    threads = resolve_num_threads(threads)
    if backend == "device":
        return _cholesky_device(basis, field, threshold, screening_threshold, max_bytes, pivot_batch_size)
    if backend != "host":
        raise ValueError("backend must be 'device' or 'host'")
    return _cholesky_host(basis, field, threshold, screening_threshold, threads, max_bytes, pivot_batch_size)


def _cholesky_device(basis, field, threshold, screening_threshold, max_bytes, pivot_batch_size, context=None):
    """gx_cholesky: the pivot loop resident on the device."""
    ctx = context or nat.default_context()
    n = basis.ao_count
    row_bytes = n * n * 16 + 16
    limit = n * n if max_bytes is None else min(n * n, max_bytes // row_bytes)
    B, O = field_arrays(field)
    opts = nat.GxCholeskyOptions(threshold, screening_threshold, int(limit), int(pivot_batch_size))
    cap = max(int(limit), 1)
    # grow the host output on demand: start with a modest capacity and retry
    guess = min(cap, max(64, 8 * n))
    while True:
        vectors = np.empty((guess, n, n), dtype=np.complex128)
        pivots = np.empty((guess, 2), dtype=np.int64)
        rank = ctypes.c_int64()
        resid = ctypes.c_double()
        opts.max_rank = guess
        rc = nat.lib().gx_cholesky(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), ctypes.byref(opts),
                                   nat.dptr(vectors.view(np.float64).reshape(-1)), nat.i64ptr(pivots),
                                   ctypes.byref(rank), ctypes.byref(resid))
        if rc == -6 and guess < cap and "rank capacity" in nat.last_error():
            guess = min(cap, guess * 2)
            continue
        if rc == -6 and "rank capacity" in nat.last_error():
            r = int(rank.value)
            raise MemoryError(f"Cholesky ERI output requires at least {(r + 1) * row_bytes} bytes, "
                              f"exceeding max_bytes={max_bytes}")
        nat.check(rc)
        r = int(rank.value)
        return CholeskyERI(vectors[:r].copy(), pivots[:r].copy(), threshold, float(resid.value))


def _cholesky_host(basis, field, threshold, screening_threshold, threads, max_bytes, pivot_batch_size):
    """The reference's NumPy pivot loop (cholesky.py:128-297) over GPU-generated integrals."""
    n = basis.ao_count
    shells = basis.shells
    single_center = all(s.center == shells[0].center for s in shells)
    integral_field = None if single_center else field
    offsets = basis.ao_offsets
    spans = [slice(o, o + s.ao_count) for o, s in zip(offsets, shells, strict=False)]
    owners = np.repeat(np.arange(len(shells)), [s.ao_count for s in shells])
    diagonal = np.zeros((n, n))
    bounds = eri_schwarz_bounds(basis, field=integral_field) ** 2 if screening_threshold else None
    skipped, quartets = [], []
    for a in range(len(shells)):
        for b in range(a, len(shells)):
            if bounds is not None and bounds[a, b] <= min(threshold, screening_threshold):
                diagonal[spans[a], spans[b]] = bounds[a, b]
                diagonal[spans[b], spans[a]] = bounds[a, b]
                skipped.append((a, b))
            else:
                quartets.append((a, b))

    def read_diagonal(pairs):
        if not pairs:
            return
        measured = _cholesky_diagonal(basis, pairs, field=integral_field, threads=threads)
        for a, b in pairs:
            diagonal[spans[a], spans[b]] = measured[spans[a], spans[b]]
            diagonal[spans[b], spans[a]] = measured[spans[b], spans[a]]

    read_diagonal(quartets)
    residual = diagonal.ravel().copy()
    floor = 64 * np.finfo(float).eps * float(np.max(residual, initial=0.0))
    tolerance = max(threshold, floor)
    real = field is None or all(x == 0 for x in field.B) or single_center
    dtype = np.float64 if real else np.complex128
    row_bytes = n * n * 16 + 16
    limit = n * n if max_bytes is None else min(n * n, max_bytes // row_bytes)
    factors = np.empty((0, n * n), dtype=dtype)
    pivots: list[tuple[int, int]] = []
    reuse = not single_center or any(s.contraction_count > 1 or s.primitive_count > 1 for s in shells)
    candidate_count = 32 if reuse else 8
    raw_cache: OrderedDict[int, np.ndarray] = OrderedDict()
    block_candidates = np.empty(0, dtype=int)
    candidates = np.empty(0, dtype=int)
    columns = np.empty((0, n * n), dtype=dtype)
    while float(np.max(residual, initial=0.0)) > tolerance:
        pivot = int(np.argmax(residual))
        if reuse and not real and pivot_batch_size > 1 and len(block_candidates):
            local = int(block_candidates[np.argmax(residual[block_candidates])])
            if residual[local] > tolerance and residual[local] >= 0.01 * residual[pivot]:
                pivot = local
        rank = len(pivots)
        if rank >= limit:
            raise MemoryError(f"Cholesky ERI output requires at least {(rank + 1) * row_bytes} bytes, "
                              f"exceeding max_bytes={max_bytes}")
        if rank == len(factors):
            capacity = min(limit, max(8, 2 * len(factors)))
            grown = np.empty((capacity, n * n), dtype=dtype)
            grown[:rank] = factors[:rank]
            factors = grown
        if reuse and pivot in raw_cache:
            candidates = np.array([pivot])
            columns = raw_cache.pop(pivot)[None, :]
        match = np.flatnonzero(candidates == pivot)
        if not len(match):
            mu, nu = divmod(pivot, n)
            a, b = int(owners[mu]), int(owners[nu])
            if reuse:
                ca, cb = shells[a].cartesian_count, shells[b].cartesian_count
                left = offsets[a] + (mu - offsets[a]) % ca + ca * np.arange(shells[a].contraction_count)
                right = offsets[b] + (nu - offsets[b]) % cb + cb * np.arange(shells[b].contraction_count)
                indices = (left[:, None] * n + right).ravel()
            else:
                indices = np.arange(n * n).reshape(n, n)[spans[a], spans[b]].ravel()
            indices = indices[residual[indices] > tolerance]
            candidates = indices[np.argsort(-residual[indices], kind="stable")[:candidate_count]]
            if pivot not in candidates:
                candidates[-1] = pivot
            block_candidates = candidates[: min(32, pivot_batch_size)]
            cmu, cnu = np.divmod(candidates, n)
            columns = _cholesky_columns(basis, list(zip(cmu.tolist(), cnu.tolist(), strict=True)),
                                        field=integral_field, threads=threads)
            if reuse:
                for index, candidate in enumerate(candidates):
                    if candidate != pivot:
                        raw_cache[int(candidate)] = columns[index].copy()
                capacity = min(1024, max(8, rank + 8))
                while len(raw_cache) > capacity:
                    raw_cache.popitem(last=False)
            match = np.flatnonzero(candidates == pivot)
        if reuse:
            raw_cache.pop(pivot, None)
        column = columns[int(match[0])].copy()
        if rank:
            column -= factors[:rank, pivot].conj() @ factors[:rank]
        if real:
            square = column.reshape(n, n)
            column = ((square + square.T) * 0.5).ravel()
        column /= np.sqrt(residual[pivot])
        factors[rank] = column
        pivots.append(divmod(pivot, n))
        residual -= np.abs(column) ** 2
        if float(np.min(residual, initial=0.0)) < -max(floor * 16, 1e-12):
            raise RuntimeError("Coulomb Cholesky residual lost positive semidefiniteness")
        np.maximum(residual, 0, out=residual)
        residual[pivot] = 0
    if skipped:
        read_diagonal(skipped)
        residual = diagonal.ravel() - np.sum(np.abs(factors[: len(pivots)]) ** 2, axis=0)
    vectors = np.array(factors[: len(pivots)], dtype=np.complex128).reshape(len(pivots), n, n)
    return CholeskyERI(vectors, np.asarray(pivots, dtype=np.int64).reshape(-1, 2), threshold,
                       float(np.max(residual, initial=0.0)))
