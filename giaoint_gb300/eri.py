"""Electron-repulsion entry points on the GPU, with the reference's Python API.

Mirrors python/giao_integrals/eri.py:1-208 and the native entry points
``primitive_eri``, ``eri_shell``, ``_eri_full``, ``_eri_batch`` and
``_EriSchwarzBounds`` (src/bindings.cpp:409-425, 599-731): same names,
keyword arguments, validation and error types.  ``threads`` is accepted and
validated for compatibility and has no effect (the work runs on one GPU).
Two keyword arguments are additions: ``precision`` and ``mixed_cutoff``.
``precision="fp64"`` (default) skips primitive quartets whose Schwarz
product is below 1e-18 (they move no result by more than ~1e-15);
``"fp64_exact"`` evaluates every primitive quartet as the reference does;
``"mixed"`` evaluates primitive quartets with Schwarz product below
``mixed_cutoff`` in FP32 (FP64 Boys values, FP64 final summation) and skips
those below 1e-15.
"""

from __future__ import annotations

import ctypes
from collections.abc import Iterable, Iterator, Sequence
from dataclasses import dataclass
from itertools import product
from math import prod

import numpy as np
import numpy.typing as npt

from . import _native as nat
from ._threads import resolve_num_threads
from ._types import Basis, MagneticField, PrimitiveGaussian, Shell, field_arrays

Quartet = tuple[int, int, int, int]

PRECISIONS = {"fp64": 0, "mixed": 1, "fp64_exact": 2}
DEFAULT_MIXED_CUTOFF = 1.0e-6


def _precision(precision: str) -> int:
    try:
        return PRECISIONS[precision]
    except KeyError:
        raise ValueError("precision must be 'fp64', 'mixed' or 'fp64_exact'") from None


@dataclass(frozen=True)
class EriBatch:
    """Packed shell-quartet results and screening counts.

    ``values[offsets[i]:offsets[i + 1]]`` reshaped to ``shapes[i]`` is the
    C-contiguous block for ``quartets[i]``.
    """

    quartets: npt.NDArray[np.uint32]
    shapes: npt.NDArray[np.int64]
    offsets: npt.NDArray[np.int64]
    values: npt.NDArray[np.complex128]
    requested_count: int = 0
    screened_count: int = 0

    def block(self, index: int) -> npt.NDArray[np.complex128]:
        start = int(self.offsets[index])
        stop = int(self.offsets[index + 1])
        return self.values[start:stop].reshape(tuple(self.shapes[index]))


def _checked_quartets(shell_count: int, quartets: Iterable[Sequence[int]] | None) -> Iterator[Quartet]:
    if quartets is None:
        for quartet in product(range(shell_count), repeat=4):
            a, b, c, d = quartet
            if min(quartet, (c, d, a, b), (b, a, d, c), (d, c, b, a)) == quartet:
                yield quartet
        return
    for value in quartets:
        if len(value) != 4:
            raise ValueError("each shell quartet must contain four indices")
        if any(isinstance(index, (bool, np.bool_)) for index in value):
            raise ValueError("shell-quartet indices must be integers")
        try:
            quartet = tuple(int(index) for index in value)
        except (TypeError, ValueError, OverflowError) as error:
            raise ValueError("shell-quartet indices must be integers") from error
        if any(converted != original for converted, original in zip(quartet, value, strict=True)):
            raise ValueError("shell-quartet indices must be integers")
        if any(index < 0 or index >= shell_count for index in quartet):
            raise IndexError("shell-quartet index is out of range")
        yield quartet  # type: ignore[misc]


def canonical_quartets(shell_count: int) -> np.ndarray:
    """All canonical representatives of the finite-field orbit
    {(ab|cd), (cd|ab), (ba|dc)*, (dc|ba)*} (src/eri.cpp:414-429), uint32[k, 4],
    in the reference's enumeration order (native host enumeration)."""
    n = int(shell_count)
    count = nat.lib().gx_canonical_quartets(n, None)
    out = np.empty((max(count, 1), 4), dtype=np.uint32)
    if count:
        nat.lib().gx_canonical_quartets(n, nat.u32ptr(out))
    return out[:count]


def _eri_batch(basis: Basis, quartets, *, field: MagneticField | None = None, screening_threshold: float = 0.0,
               threads=None, bounds=None, precision: str = "fp64", mixed_cutoff: float = DEFAULT_MIXED_CUTOFF,
               context=None, stats: dict | None = None):
    """Native packed batch (src/bindings.cpp:672-731): returns
    (quartets uint32[k,4], shapes int64[k,4], offsets int64[k+1],
    values complex128, requested, screened).  A ``stats`` dict, when given,
    receives the primitive-quartet counts (evaluated, FP32, skipped) and the
    kernel time."""
    resolve_num_threads(threads)
    ctx = context or nat.default_context()
    q = np.ascontiguousarray(np.asarray(quartets, dtype=np.int64).reshape(-1, 4))
    ns = len(basis.shells)
    if len(q) and (q.min() < 0 or q.max() >= ns):
        raise IndexError("ERI shell-quartet index is out of range")
    q = q.astype(np.uint32)
    screening_threshold = float(screening_threshold)
    if not np.isfinite(screening_threshold) or screening_threshold < 0.0:
        raise ValueError("ERI screening threshold must be finite and non-negative")
    sizes = np.array([s.ao_count for s in basis.shells], dtype=np.int64)
    total = int(np.prod(sizes[q.astype(np.int64)], axis=1).sum()) if len(q) else 0
    values = np.empty(max(total, 1), dtype=np.complex128)
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    kept = np.empty((max(len(q), 1), 4), dtype=np.uint32)
    stats_out = stats
    st = nat.GxStats()
    B, O = field_arrays(field)
    nat.check(nat.lib().gx_eri_batch(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), nat.u32ptr(q),
                                     len(q), _precision(precision), float(mixed_cutoff), screening_threshold,
                                     nat.u32ptr(kept), nat.i64ptr(offsets), nat.dptr(values.view(np.float64)),
                                     total, ctypes.byref(st)))
    if stats_out is not None:
        stats_out.update(primitive_quartets=int(st.primitive_quartets),
                         fp32_primitive_quartets=int(st.fp32_primitive_quartets),
                         skipped_primitive_quartets=int(st.skipped_primitive_quartets), kernel_ms=float(st.kernel_ms))
    k = int(st.computed)
    kept = kept[:k]
    offsets = offsets[: k + 1]
    shapes = sizes[kept.astype(np.int64)] if k else np.zeros((0, 4), dtype=np.int64)
    return kept, shapes, offsets, values[: int(offsets[-1])], int(st.requested), int(st.screened)


def eri_batches(basis: Basis, *, field: MagneticField | None = None, quartets: Iterable[Sequence[int]] | None = None,
                target_bytes: int = 64 * 1024 * 1024, screening_threshold: float = 0.0, threads: int | None = None,
                precision: str = "fp64", mixed_cutoff: float = DEFAULT_MIXED_CUTOFF) -> Iterator[EriBatch]:
    """Yield packed shell-quartet batches without allocating an AO tensor
    (python/giao_integrals/eri.py:80-146)."""
    if isinstance(target_bytes, (bool, np.bool_)) or not isinstance(target_bytes, (int, np.integer)):
        raise ValueError("target_bytes must be a positive integer")
    if target_bytes <= 0:
        raise ValueError("target_bytes must be a positive integer")
    screening_threshold = float(screening_threshold)
    if not np.isfinite(screening_threshold) or screening_threshold < 0.0:
        raise ValueError("screening_threshold must be finite and non-negative")
    threads = resolve_num_threads(threads)
    _precision(precision)
    shells = basis.shells
    sizes = [s.ao_count for s in shells]
    packed: list[Quartet] = []
    packed_bytes = 0

    def emit() -> EriBatch:
        q, shapes, offsets, values, requested, screened = _eri_batch(
            basis, packed, field=field, screening_threshold=screening_threshold, threads=threads,
            precision=precision, mixed_cutoff=mixed_cutoff)
        return EriBatch(q, shapes, offsets, values, requested, screened)

    for quartet in _checked_quartets(len(shells), quartets):
        block_bytes = prod(sizes[i] for i in quartet) * 16
        if packed and packed_bytes + block_bytes > target_bytes:
            yield emit()
            packed.clear()
            packed_bytes = 0
        packed.append(quartet)
        packed_bytes += int(block_bytes)
    if packed:
        yield emit()


def evaluate_eri_shell_quartets(basis: Basis, quartets, consumer, *, field: MagneticField | None = None,
                                screening_threshold: float = 0.0, precision: str = "fp64",
                                mixed_cutoff: float = DEFAULT_MIXED_CUTOFF, context=None) -> dict:
    """Stream the blocks of ``quartets`` to ``consumer(quartet, block)`` in
    input order, as the reference's C++ ``evaluate_eri_shell_quartets``
    (include/giao_integrals/eri.hpp:127-135, src/eri.cpp:644-767), through
    ``gx_eri_for_each``.  ``block`` is a C-order complex128 view of shape
    (na, nb, nc, nd) into a host buffer of the call, valid only while the
    consumer runs (copy it to keep it).  Quartets below the Schwarz
    ``screening_threshold`` are skipped.  An exception raised by the consumer
    stops the evaluation and propagates.  Returns the counts of the call
    (requested, computed, screened) and its timings."""
    if consumer is None:
        raise ValueError("ERI quartet consumer must not be null")
    ctx = context or nat.default_context()
    q = np.ascontiguousarray(np.asarray(quartets, dtype=np.int64).reshape(-1, 4))
    ns = len(basis.shells)
    if len(q) and (q.min() < 0 or q.max() >= ns):
        raise IndexError("ERI shell-quartet index is out of range")
    q = q.astype(np.uint32)
    failure: list[BaseException] = []

    def trampoline(blk_ptr, _user):
        try:
            blk = blk_ptr.contents
            shape = tuple(int(x) for x in blk.shape)
            flat = np.ctypeslib.as_array(blk.values, shape=(2 * int(blk.count),))
            consumer(tuple(int(x) for x in blk.shells), flat.view(np.complex128).reshape(shape))
            return 0
        except BaseException as exc:  # handed back to the caller after the call returns
            failure.append(exc)
            return 1

    callback = nat.QUARTET_CONSUMER(trampoline)
    st = nat.GxStats()
    B, O = field_arrays(field)
    rc = nat.lib().gx_eri_for_each(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), nat.u32ptr(q), len(q),
                                   _precision(precision), float(mixed_cutoff), float(screening_threshold), callback,
                                   None, ctypes.byref(st))
    if failure:
        raise failure[0]
    nat.check(rc)
    return {"requested": int(st.requested), "computed": int(st.computed), "screened": int(st.screened),
            "primitive_quartets": int(st.primitive_quartets), "kernel_ms": float(st.kernel_ms),
            "call_ms": float(st.call_ms)}


def _eri_batch_packed(items, *, precision: str = "fp64", mixed_cutoff: float = DEFAULT_MIXED_CUTOFF, context=None,
                      stats: dict | None = None):
    """Several requests in one class-sorted execution (gx_eri_batch_packed).

    ``items`` is a sequence of (basis, quartets, field); returns one
    (offsets int64[k+1], values complex128) pair per item, in the packed
    block layout that ``_eri_batch`` gives the item alone (no screening)."""
    ctx = context or nat.default_context()
    n = len(items)
    qs, offs, vals, caps = [], [], [], []
    Bs = np.zeros((max(n, 1), 3))
    Os = np.zeros((max(n, 1), 3))
    for r, (basis, quartets, field) in enumerate(items):
        q = np.ascontiguousarray(np.asarray(quartets, dtype=np.int64).reshape(-1, 4))
        if len(q) and (q.min() < 0 or q.max() >= len(basis.shells)):
            raise IndexError("ERI shell-quartet index is out of range")
        q = q.astype(np.uint32)
        sizes = np.array([s.ao_count for s in basis.shells], dtype=np.int64)
        total = int(np.prod(sizes[q.astype(np.int64)], axis=1).sum()) if len(q) else 0
        qs.append(q)
        offs.append(np.zeros(len(q) + 1, dtype=np.int64))
        vals.append(np.empty(max(total, 1), dtype=np.complex128))
        caps.append(total)
        Bs[r], Os[r] = field_arrays(field)
    lib = nat.lib()
    handles = (ctypes.c_void_p * max(n, 1))(*[b._device(ctx).value for b, _, _ in items])
    qptr = (nat._u32 * max(n, 1))(*[nat.u32ptr(q) for q in qs])
    optr = (nat._i64 * max(n, 1))(*[nat.i64ptr(o) for o in offs])
    vptr = (nat._d * max(n, 1))(*[nat.dptr(v.view(np.float64)) for v in vals])
    nq = np.array([len(q) for q in qs] or [0], dtype=np.int64)
    cap = np.array(caps or [0], dtype=np.int64)
    ms = ctypes.c_double()
    nat.check(lib.gx_eri_batch_packed(ctx.handle, n, handles, nat.dptr(Bs.reshape(-1)), nat.dptr(Os.reshape(-1)), qptr,
                                      nat.i64ptr(nq), _precision(precision), float(mixed_cutoff), optr, vptr,
                                      nat.i64ptr(cap), ctypes.byref(ms)))
    if stats is not None:
        stats["kernel_ms"] = ms.value
    return [(o, v[: int(o[-1])]) for o, v in zip(offs, vals)]


def _eri_full(basis: Basis, *, field: MagneticField | None = None, screening_threshold: float = 0.0, threads=None,
              precision: str = "fp64", mixed_cutoff: float = DEFAULT_MIXED_CUTOFF, context=None):
    """Native full tensor (src/bindings.cpp:640-671)."""
    resolve_num_threads(threads)
    ctx = context or nat.default_context()
    n = basis.ao_count
    out = np.empty((n, n, n, n), dtype=np.complex128)
    B, O = field_arrays(field)
    nat.check(nat.lib().gx_eri_full(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O),
                                    _precision(precision), float(mixed_cutoff), float(screening_threshold),
                                    nat.dptr(out.view(np.float64).reshape(-1))))
    return out


def eri(basis: Basis, *, field: MagneticField | None = None, storage: str = "blocks", max_bytes: int | None = None,
        target_bytes: int = 64 * 1024 * 1024, screening_threshold: float = 0.0, threads: int | None = None,
        precision: str = "fp64", mixed_cutoff: float = DEFAULT_MIXED_CUTOFF):
    """Streamed blocks or an explicitly guarded full tensor (eri.py:149-200)."""
    screening_threshold = float(screening_threshold)
    if not np.isfinite(screening_threshold) or screening_threshold < 0.0:
        raise ValueError("screening_threshold must be finite and non-negative")
    threads = resolve_num_threads(threads)
    if storage == "blocks":
        if max_bytes is not None:
            raise ValueError("max_bytes is only valid with storage='full'")
        return eri_batches(basis, field=field, target_bytes=target_bytes, screening_threshold=screening_threshold,
                           threads=threads, precision=precision, mixed_cutoff=mixed_cutoff)
    if storage != "full":
        raise ValueError("storage must be 'blocks' or 'full'")
    if max_bytes is None:
        raise ValueError("storage='full' requires an explicit max_bytes limit")
    if isinstance(max_bytes, (bool, np.bool_)) or not isinstance(max_bytes, (int, np.integer)):
        raise ValueError("max_bytes must be a non-negative integer")
    if max_bytes < 0:
        raise ValueError("max_bytes must be a non-negative integer")
    required = basis.ao_count**4 * 16
    if required > max_bytes:
        raise MemoryError(f"full ERI tensor requires {required} bytes, exceeding max_bytes={max_bytes}")
    return _eri_full(basis, field=field, screening_threshold=screening_threshold, threads=threads,
                     precision=precision, mixed_cutoff=mixed_cutoff)


class _EriSchwarzBounds:
    """Shell-pair Schwarz factors (src/eri.cpp:587-635)."""

    def __init__(self, basis: Basis, *, field: MagneticField | None = None, context=None):
        ctx = context or nat.default_context()
        ns = len(basis.shells)
        out = np.zeros((ns, ns), dtype=np.float64)
        B, O = field_arrays(field)
        if ns:
            nat.check(nat.lib().gx_schwarz(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O),
                                           nat.dptr(out.reshape(-1))))
        self.values = out

    def bound(self, a: int, b: int) -> float:
        ns = self.values.shape[0]
        if a < 0 or b < 0 or a >= ns or b >= ns:
            raise IndexError("ERI Schwarz shell-pair index is out of range")
        return float(self.values[a, b])


def eri_schwarz_bounds(basis: Basis, *, field: MagneticField | None = None) -> npt.NDArray[np.float64]:
    """The shell-pair Schwarz factors used by ERI screening."""
    return np.asarray(_EriSchwarzBounds(basis, field=field).values, dtype=np.float64)


def _validate_out(out, shape):
    if out is None:
        return np.empty(shape, dtype=np.complex128)
    if not isinstance(out, np.ndarray):
        raise ValueError("out must be a NumPy array")
    if out.dtype != np.complex128:
        raise ValueError("out must have dtype complex128")
    if out.ndim != len(shape):
        raise ValueError("out has an incorrect number of dimensions")
    if tuple(out.shape) != tuple(shape):
        raise ValueError("out has an incorrect shape")
    if not out.flags.c_contiguous:
        raise ValueError("out must be C-contiguous")
    if not out.flags.writeable:
        raise ValueError("out must be writable")
    return out


def eri_shell(a: Shell, b: Shell, c: Shell, d: Shell, *, field: MagneticField | None = None, out=None,
              context=None):
    """One shell quartet (compute_eri; src/bindings.cpp:616-639)."""
    shape = (a.ao_count, b.ao_count, c.ao_count, d.ao_count)
    result = _validate_out(out, shape)
    ctx = context or nat.default_context()
    basis = Basis([a, b, c, d])
    buf = np.empty(shape, dtype=np.complex128)
    B, O = field_arrays(field)
    nat.check(nat.lib().gx_eri_shell(ctx.handle, basis._device(ctx), 0, 1, 2, 3, nat.dptr(B), nat.dptr(O),
                                     nat.dptr(buf.view(np.float64).reshape(-1))))
    result[...] = buf
    return result


def primitive_eri(a: PrimitiveGaussian, b: PrimitiveGaussian, c: PrimitiveGaussian, d: PrimitiveGaussian, *,
                  field: MagneticField | None = None, context=None) -> complex:
    """One primitive quartet (src/bindings.cpp:599-614)."""
    prims = (a, b, c, d)
    ctx = context or nat.default_context()
    exps = np.ascontiguousarray([p.exponent for p in prims], dtype=np.float64)
    centers = np.ascontiguousarray([x for p in prims for x in p.center], dtype=np.float64)
    ang = np.ascontiguousarray([x for p in prims for x in p.angular], dtype=np.int32)
    coefs = np.ascontiguousarray([p.coefficient for p in prims], dtype=np.float64)
    norm = np.ascontiguousarray([int(p.normalized) for p in prims], dtype=np.int32)
    out = np.zeros(2, dtype=np.float64)
    B, O = field_arrays(field)
    nat.check(nat.lib().gx_primitive_eri(ctx.handle, nat.dptr(exps), nat.dptr(centers), nat.iptr(ang),
                                         nat.dptr(coefs), nat.iptr(norm), nat.dptr(B), nat.dptr(O), nat.dptr(out)))
    return complex(out[0], out[1])


# ---------------------------------------------------------------------------
# centre and magnetic derivatives (src/derivatives.cpp:53-106, 215-280, 556-640, 954-966;
# python/giao_integrals/eri.py:210-284; src/bindings.cpp:979-992, 1308-1324,
# 2255-2303)
# ---------------------------------------------------------------------------


@dataclass(frozen=True)
class EriDerivativeBatch(EriBatch):
    """Packed local centre derivatives, with blocks (4, 3, na, nb, nc, nd).

    Centre slots follow quartet order, independent even for repeated shells.
    ``block()`` returns a view of ``values``.  Counts include screened requests.
    """


def _derivative_call(ctx, basis: Basis, q: np.ndarray, field, total: int, values: np.ndarray,
                     offsets: np.ndarray) -> float:
    B, O = field_arrays(field)
    ms = ctypes.c_float()
    nat.check(nat.lib().gx_eri_center_derivatives(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O),
                                                  nat.u32ptr(q), len(q), nat.i64ptr(offsets),
                                                  nat.dptr(values.view(np.float64)), total, ctypes.byref(ms)))
    return float(ms.value)


def _eri_derivative_batch(basis: Basis, quartets, *, field: MagneticField | None = None,
                          screening_threshold: float = 0.0, threads=None, bounds=None, context=None):
    """Native packed derivative batch (src/bindings.cpp:2255-2303): returns
    (quartets uint32[k,4], shapes int64[k,6], offsets int64[k+1], values
    complex128, requested, screened)."""
    resolve_num_threads(threads)
    threshold = float(screening_threshold)
    if not np.isfinite(threshold) or threshold < 0.0:
        raise ValueError("screening_threshold must be finite and non-negative")
    if threshold > 0.0 and bounds is None:
        raise ValueError("derivative screening requires derivative bounds")
    if bounds is not None and not bounds.matches(basis, field):
        raise ValueError("derivative bounds do not match basis and field")
    ctx = context or nat.default_context()
    requested = np.ascontiguousarray(np.asarray(quartets, dtype=np.int64).reshape(-1, 4))
    ns = len(basis.shells)
    if len(requested) and (requested.min() < 0 or requested.max() >= ns):
        raise IndexError("derivative shell quartet index is out of range")
    q = requested
    if threshold > 0.0 and len(q):
        keep = bounds.quartet_bounds(q) >= threshold
        q = q[keep]
    q = np.ascontiguousarray(q.astype(np.uint32))
    sizes = np.array([s.ao_count for s in basis.shells], dtype=np.int64)
    block = np.prod(sizes[q.astype(np.int64)], axis=1) if len(q) else np.zeros(0, dtype=np.int64)
    total = int(12 * block.sum())
    values = np.empty(max(total, 1), dtype=np.complex128)
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    if len(q):
        _derivative_call(ctx, basis, q, field, total, values, offsets)
    shapes = np.zeros((len(q), 6), dtype=np.int64)
    if len(q):
        shapes[:, 0] = 4
        shapes[:, 1] = 3
        shapes[:, 2:] = sizes[q.astype(np.int64)]
    return q, shapes, offsets, values[:total], len(requested), len(requested) - len(q)


def eri_derivative_batches(basis: Basis, *, field: MagneticField | None = None,
                           quartets: Iterable[Sequence[int]] | None = None, target_bytes: int = 64 * 1024 * 1024,
                           screening_threshold: float = 0.0, threads: int | None = None,
                           ) -> Iterator[EriDerivativeBatch]:
    """Stream ERI centre derivatives without a full derivative AO tensor
    (python/giao_integrals/eri.py:220-284).

    Each block has axes (quartet centre slot, nuclear xyz, mu, nu, lambda,
    sigma); the London-phase centre response is included at fixed B and gauge
    origin.  ``target_bytes`` bounds the packed complex values per batch (a
    single oversized quartet is emitted alone).  Positive
    ``screening_threshold`` values drop quartets whose derivative Schwarz
    bound is below it."""
    if (isinstance(target_bytes, (bool, np.bool_)) or not isinstance(target_bytes, (int, np.integer))
            or target_bytes <= 0):
        raise ValueError("target_bytes must be a positive integer")
    threshold = float(screening_threshold)
    if not np.isfinite(threshold) or threshold < 0:
        raise ValueError("screening_threshold must be finite and non-negative")
    thread_count = resolve_num_threads(threads)
    bounds = _EriDerivativeSchwarzBounds(basis, field=field, threads=thread_count) if threshold > 0 else None
    shells = basis.shells
    packed: list[Quartet] = []
    packed_bytes = 0

    def emit() -> EriDerivativeBatch:
        q, shapes, offsets, values, requested, screened = _eri_derivative_batch(
            basis, packed, field=field, screening_threshold=threshold, threads=thread_count, bounds=bounds)
        return EriDerivativeBatch(q, shapes, offsets, values, requested, screened)

    for quartet in _checked_quartets(len(shells), quartets):
        block_bytes = 12 * prod(shells[index].ao_count for index in quartet) * 16
        if packed and packed_bytes + block_bytes > target_bytes:
            yield emit()
            packed.clear()
            packed_bytes = 0
        packed.append(quartet)
        packed_bytes += block_bytes
    if packed:
        yield emit()


def eri_center_derivatives_shell(a: Shell, b: Shell, c: Shell, d: Shell, *, field: MagneticField | None = None,
                                 out=None, context=None) -> npt.NDArray[np.complex128]:
    """Centre derivatives of one shell quartet, complex (4, 3, na, nb, nc, nd)
    (compute_eri_center_derivatives; src/bindings.cpp:1308-1324)."""
    for s in (a, b, c, d):
        if not isinstance(s, Shell):
            raise TypeError("a, b, c and d must be Shell objects")
    shape = (4, 3, a.ao_count, b.ao_count, c.ao_count, d.ao_count)
    result = _validate_out(out, shape)
    ctx = context or nat.default_context()
    basis = Basis([a, b, c, d])
    q = np.array([[0, 1, 2, 3]], dtype=np.uint32)
    total = int(np.prod(shape))
    values = np.empty(total, dtype=np.complex128)
    offsets = np.zeros(2, dtype=np.int64)
    _derivative_call(ctx, basis, q, field, total, values, offsets)
    result[...] = values.reshape(shape)
    return result


def primitive_eri_center_derivatives(a: PrimitiveGaussian, b: PrimitiveGaussian, c: PrimitiveGaussian,
                                     d: PrimitiveGaussian, *, field: MagneticField | None = None,
                                     context=None) -> npt.NDArray[np.complex128]:
    """Centre derivatives of one primitive quartet, complex (4, 3)
    (primitive_eri_center_derivatives; src/derivatives.cpp:836-842,
    src/bindings.cpp:979-992)."""
    shells, picks, scale = _primitive_shells((a, b, c, d))
    full = eri_center_derivatives_shell(*shells, field=field, context=context)
    return full[:, :, picks[0], picks[1], picks[2], picks[3]] * scale


def _eri_magnetic_derivative_blocks(basis: Basis, quartets, *, field: MagneticField | None = None, context=None):
    """Magnetic-derivative blocks (3, na, nb, nc, nd) of ``quartets`` packed
    in input order (gx_eri_magnetic_derivatives): returns (offsets, values)."""
    ctx = context or nat.default_context()
    q = np.ascontiguousarray(np.asarray(quartets, dtype=np.int64).reshape(-1, 4))
    if len(q) and (q.min() < 0 or q.max() >= len(basis.shells)):
        raise IndexError("derivative shell quartet index is out of range")
    q = np.ascontiguousarray(q.astype(np.uint32))
    sizes = np.array([s.ao_count for s in basis.shells], dtype=np.int64)
    total = int(3 * np.prod(sizes[q.astype(np.int64)], axis=1).sum()) if len(q) else 0
    values = np.empty(max(total, 1), dtype=np.complex128)
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    if len(q):
        B, O = field_arrays(field)
        ms = ctypes.c_float()
        nat.check(nat.lib().gx_eri_magnetic_derivatives(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O),
                                                        nat.u32ptr(q), len(q), nat.i64ptr(offsets),
                                                        nat.dptr(values.view(np.float64)), total, ctypes.byref(ms)))
    return offsets, values[:total]


def eri_magnetic_derivatives_shell(a: Shell, b: Shell, c: Shell, d: Shell, *, field: MagneticField | None = None,
                                   out=None, context=None) -> npt.NDArray[np.complex128]:
    """Field derivatives d/dB_b of one shell quartet at fixed gauge origin,
    complex (3, na, nb, nc, nd) (compute_eri_magnetic_derivatives;
    src/bindings.cpp:1326-1342)."""
    for s in (a, b, c, d):
        if not isinstance(s, Shell):
            raise TypeError("a, b, c and d must be Shell objects")
    shape = (3, a.ao_count, b.ao_count, c.ao_count, d.ao_count)
    result = _validate_out(out, shape)
    _, values = _eri_magnetic_derivative_blocks(Basis([a, b, c, d]), [(0, 1, 2, 3)], field=field, context=context)
    result[...] = values.reshape(shape)
    return result


def primitive_eri_magnetic_derivatives(a: PrimitiveGaussian, b: PrimitiveGaussian, c: PrimitiveGaussian,
                                       d: PrimitiveGaussian, *, field: MagneticField | None = None,
                                       context=None) -> npt.NDArray[np.complex128]:
    """Field derivatives of one primitive quartet, complex (3,)
    (primitive_eri_magnetic_derivatives; src/derivatives.cpp:844-850,
    src/bindings.cpp:995-1010)."""
    shells, picks, scale = _primitive_shells((a, b, c, d))
    full = eri_magnetic_derivatives_shell(*shells, field=field, context=context)
    return full[:, picks[0], picks[1], picks[2], picks[3]] * scale


def _eri_mixed_derivative_blocks(basis: Basis, quartets, *, field: MagneticField | None = None, context=None):
    """Mixed field/centre derivative blocks (4, 3, 3, na, nb, nc, nd) of
    ``quartets`` packed in input order (gx_eri_mixed_derivatives): returns
    (offsets, values).  Meant for small bases (two levels of derived shells)."""
    ctx = context or nat.default_context()
    q = np.ascontiguousarray(np.asarray(quartets, dtype=np.int64).reshape(-1, 4))
    if len(q) and (q.min() < 0 or q.max() >= len(basis.shells)):
        raise IndexError("derivative shell quartet index is out of range")
    q = np.ascontiguousarray(q.astype(np.uint32))
    sizes = np.array([s.ao_count for s in basis.shells], dtype=np.int64)
    total = int(36 * np.prod(sizes[q.astype(np.int64)], axis=1).sum()) if len(q) else 0
    values = np.empty(max(total, 1), dtype=np.complex128)
    offsets = np.zeros(len(q) + 1, dtype=np.int64)
    if len(q):
        B, O = field_arrays(field)
        nat.check(nat.lib().gx_eri_mixed_derivatives(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O),
                                                     nat.u32ptr(q), len(q), nat.i64ptr(offsets),
                                                     nat.dptr(values.view(np.float64)), total))
    return offsets, values[:total]


def eri_mixed_derivatives_shell(a: Shell, b: Shell, c: Shell, d: Shell, *, field: MagneticField | None = None,
                                out=None, context=None) -> npt.NDArray[np.complex128]:
    """Mixed second derivatives d2/dR dB of one shell quartet at fixed gauge
    origin, complex (4, 3, 3, na, nb, nc, nd): centre slot, nuclear axis,
    field axis (compute_eri_mixed_derivatives; src/bindings.cpp:2155-2165)."""
    for s in (a, b, c, d):
        if not isinstance(s, Shell):
            raise TypeError("a, b, c and d must be Shell objects")
    shape = (4, 3, 3, a.ao_count, b.ao_count, c.ao_count, d.ao_count)
    result = _validate_out(out, shape)
    _, values = _eri_mixed_derivative_blocks(Basis([a, b, c, d]), [(0, 1, 2, 3)], field=field, context=context)
    result[...] = values.reshape(shape)
    return result


def primitive_eri_mixed_derivatives(a: PrimitiveGaussian, b: PrimitiveGaussian, c: PrimitiveGaussian,
                                    d: PrimitiveGaussian, *, field: MagneticField | None = None,
                                    context=None) -> npt.NDArray[np.complex128]:
    """Mixed second derivatives of one primitive quartet, complex (4, 3, 3)
    (primitive_eri_mixed_derivatives; src/derivatives.cpp:1252-1256,
    src/bindings.cpp:2139-2145)."""
    shells, picks, scale = _primitive_shells((a, b, c, d))
    full = eri_mixed_derivatives_shell(*shells, field=field, context=context)
    return full[:, :, :, picks[0], picks[1], picks[2], picks[3]] * scale


def _primitive_shells(prims):
    """Unit-coefficient one-primitive shells whose components carry
    N(alpha, component), the component index of each primitive, and the
    scale (coefficients; unnormalised primitives divide N out again)."""
    shells, picks = [], []
    scale = 1.0
    for g in prims:
        if not isinstance(g, PrimitiveGaussian):
            raise TypeError("a, b, c and d must be PrimitiveGaussian objects")
        l = sum(g.angular)
        shells.append(Shell(g.center, l, [g.exponent], [1.0], normalize=False))
        comps = [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]
        picks.append(comps.index(tuple(g.angular)))
        scale *= g.coefficient
        if not g.normalized:
            scale /= nat.lib().gx_primitive_normalization(g.exponent, *g.angular)
    return shells, picks, scale


class _EriDerivativeSchwarzBounds:
    """Derivative-density Schwarz factors (src/derivatives.cpp:1307-1387,
    src/bindings.cpp:2242-2253), computed on the GPU (gx_eri_derivative_schwarz).

    A quartet's bound max(D_ab Q_cd, Q_ab D_cd), padded by (1 + 128 eps) and
    one ulp, bounds every local derivative component of its block.  The
    object is tied to the basis object and the exact field it was built for."""

    def __init__(self, basis: Basis, *, field: MagneticField | None = None, threads=None, context=None):
        if not isinstance(basis, Basis):
            raise TypeError("basis must be a Basis")
        resolve_num_threads(threads)
        ctx = context or nat.default_context()
        self._basis = basis
        B, O = field_arrays(field)
        self._field = (tuple(B.tolist()), tuple(O.tolist()))
        ns = len(basis.shells)
        self._n = ns
        values = np.zeros(max(ns * ns, 1), dtype=np.float64)
        ordinary = np.zeros(max(ns * ns, 1), dtype=np.float64)
        nat.check(nat.lib().gx_eri_derivative_schwarz(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O),
                                                      nat.dptr(values), nat.dptr(ordinary)))
        self.values = values[: ns * ns]
        self.ordinary = ordinary[: ns * ns]

    def matches(self, basis, field) -> bool:
        B, O = field_arrays(field)
        return basis is self._basis and (tuple(B.tolist()), tuple(O.tolist())) == self._field

    def quartet_bounds(self, quartets) -> np.ndarray:
        q = np.asarray(quartets, dtype=np.int64).reshape(-1, 4)
        if len(q) and (q.min() < 0 or q.max() >= self._n):
            raise IndexError("derivative shell quartet index is out of range")
        n = self._n
        ab = q[:, 0] * n + q[:, 1]
        cd = q[:, 2] * n + q[:, 3]
        bound = np.maximum(self.values[ab] * self.ordinary[cd], self.ordinary[ab] * self.values[cd])
        return np.nextafter(bound * (1.0 + 128.0 * np.finfo(np.float64).eps), np.inf)

    def quartet_bound(self, quartet) -> float:
        if len(quartet) != 4:
            raise ValueError("each shell quartet must contain four indices")
        return float(self.quartet_bounds([quartet])[0])
