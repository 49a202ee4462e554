"""Input model mirroring the reference's value types.

``Shell``, ``Basis``, ``MagneticField``, ``PrimitiveGaussian`` and
``CartesianExponent`` keep the reference's constructor signatures, property
names and validation messages (src/bindings.cpp:286-425,
include/giao_integrals/types.hpp:14-132).  Contraction normalisation runs in
the native host library (gx_shell_normalize, src/types.cpp:92-159).  A
``Basis`` uploads itself to the device once, on first use, and stays
resident for every later call.
"""

from __future__ import annotations

import ctypes
import sys
import threading
from collections.abc import Sequence

import numpy as np

from . import _native as nat

__all__ = [
    "CartesianExponent",
    "PrimitiveGaussian",
    "Shell",
    "Basis",
    "MagneticField",
    "Nucleus",
    "cartesian_components",
    "primitive_normalization",
]


def _vec3(value, name: str) -> tuple[float, float, float]:
    arr = np.asarray(value, dtype=float) if not isinstance(value, np.ndarray) else value.astype(float)
    if arr.ndim != 1 or arr.shape[0] != 3:
        raise ValueError(f"{name} must be a one-dimensional array with length 3")
    return (float(arr[0]), float(arr[1]), float(arr[2]))


def _finite3(v, name):
    if not all(np.isfinite(v)):
        raise ValueError(f"{name} values must be finite")


def _total_angular(value) -> int:
    if isinstance(value, (bool, np.bool_)) or not isinstance(value, (int, np.integer)):
        raise ValueError("shell angular momentum must be a non-negative integer")
    if value < 0 or value > 65535:
        raise ValueError("shell angular momentum must fit non-negative uint16")
    return int(value)


def _angular3(value) -> tuple[int, int, int]:
    if isinstance(value, (str, bytes)) or not isinstance(value, (Sequence, np.ndarray, CartesianExponent)):
        raise ValueError("angular momentum must contain exactly three integers")
    items = tuple(value)
    if len(items) != 3:
        raise ValueError("angular momentum must contain exactly three integers")
    out = []
    for x in items:
        if isinstance(x, (bool, np.bool_)) or not isinstance(x, (int, np.integer)):
            raise ValueError("angular momentum values must be integers")
        if x < 0 or x > 65535:
            raise ValueError("angular momentum values must fit non-negative uint16")
        out.append(int(x))
    return tuple(out)  # type: ignore[return-value]


def cartesian_components(angular_momentum) -> tuple[tuple[int, int, int], ...]:
    """x-major Cartesian powers of total degree l (src/types.cpp:74-90)."""
    l = _total_angular(angular_momentum)
    return tuple((x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1))


def primitive_normalization(exponent: float, angular) -> float:
    """Normalisation of a Cartesian primitive (src/types.cpp:60-72)."""
    a = float(exponent)
    if not np.isfinite(a) or a <= 0:
        raise ValueError("Gaussian exponent must be finite and positive")
    lx, ly, lz = _angular3(angular)
    return float(nat.lib().gx_primitive_normalization(a, lx, ly, lz))


class CartesianExponent:
    def __init__(self, values):
        self.x, self.y, self.z = _angular3(values)

    @property
    def total(self) -> int:
        return self.x + self.y + self.z

    def __iter__(self):
        return iter((self.x, self.y, self.z))


class MagneticField:
    """Uniform field B with gauge origin; London wave vector k = B x (R - O) / 2."""

    def __init__(self, B=(0.0, 0.0, 0.0), gauge_origin=(0.0, 0.0, 0.0)):
        self._B = _vec3(B, "B")
        self._O = _vec3(gauge_origin, "gauge_origin")
        _finite3(self._B, "B")
        _finite3(self._O, "gauge_origin")

    @property
    def B(self) -> tuple[float, float, float]:
        return self._B

    @property
    def gauge_origin(self) -> tuple[float, float, float]:
        return self._O

    def london_wave_vector(self, center):
        c = _vec3(center, "center")
        B, O = self._B, self._O
        d = (c[0] - O[0], c[1] - O[1], c[2] - O[2])
        return (0.5 * (B[1] * d[2] - B[2] * d[1]), 0.5 * (B[2] * d[0] - B[0] * d[2]),
                0.5 * (B[0] * d[1] - B[1] * d[0]))

    def _arrays(self):
        return np.ascontiguousarray(self._B, dtype=np.float64), np.ascontiguousarray(self._O, dtype=np.float64)


class Nucleus:
    def __init__(self, charge: float, center):
        charge = float(charge)
        if not np.isfinite(charge) or charge <= 0:
            raise ValueError("nuclear charge must be finite and positive")
        self.charge = charge
        self.center = _vec3(center, "center")
        _finite3(self.center, "nuclear center")


class PrimitiveGaussian:
    def __init__(self, exponent, center, angular=(0, 0, 0), coefficient=1.0, normalized=True):
        exponent = float(exponent)
        coefficient = float(coefficient)
        if not np.isfinite(exponent) or exponent <= 0:
            raise ValueError("Gaussian exponent must be finite and positive")
        if not np.isfinite(coefficient):
            raise ValueError("primitive coefficient must be finite")
        if not isinstance(normalized, (bool, np.bool_)):
            raise ValueError("normalized must be a bool")
        self.exponent = exponent
        self.coefficient = coefficient
        self.center = _vec3(center, "center")
        _finite3(self.center, "center")
        self.angular = _angular3(angular)
        self.normalized = bool(normalized)


class Shell:
    """Contracted Cartesian shell: Shell(center, angular_momentum, exponents,
    coefficients, *, normalize=True).  ``coefficients`` is 1-D (one
    contraction) or 2-D [contraction, primitive]."""

    def __init__(self, center, angular_momentum, exponents, coefficients, *, normalize=True):
        exps = np.asarray(exponents, dtype=np.float64)
        if exps.ndim != 1:
            raise ValueError("exponents must be one-dimensional")
        coefs = np.asarray(coefficients, dtype=np.float64)
        if coefs.ndim not in (1, 2):
            raise ValueError("coefficients must be one- or two-dimensional")
        coefs2 = coefs[None, :] if coefs.ndim == 1 else coefs
        if coefs2.shape[1] != exps.shape[0]:
            raise ValueError("the final coefficient dimension must equal the exponent count")
        if not isinstance(normalize, (bool, np.bool_)):
            raise ValueError("normalize must be a bool")
        self._center = _vec3(center, "center")
        _finite3(self._center, "center")
        self._l = _total_angular(angular_momentum)
        self._exps = np.ascontiguousarray(exps)
        self._raw = np.ascontiguousarray(coefs2)
        self._normalize = bool(normalize)
        out = np.empty_like(self._raw)
        nat.check(nat.lib().gx_shell_normalize(self._l, int(exps.shape[0]), int(coefs2.shape[0]),
                                               nat.dptr(self._exps), nat.dptr(self._raw), int(self._normalize),
                                               nat.dptr(out)))
        self._coefs = out

    # reference properties
    @property
    def center(self) -> tuple[float, float, float]:
        return self._center

    @property
    def angular_momentum(self) -> int:
        return self._l

    @property
    def primitive_count(self) -> int:
        return int(self._exps.shape[0])

    @property
    def contraction_count(self) -> int:
        return int(self._raw.shape[0])

    @property
    def cartesian_count(self) -> int:
        return (self._l + 1) * (self._l + 2) // 2

    @property
    def ao_count(self) -> int:
        return self.contraction_count * self.cartesian_count

    @property
    def components(self) -> tuple[tuple[int, int, int], ...]:
        return cartesian_components(self._l)

    # data accessors (not in the reference's Python surface)
    @property
    def exponents(self) -> np.ndarray:
        return self._exps.copy()

    @property
    def coefficients(self) -> np.ndarray:
        """Contraction-normalised coefficients [contraction, primitive]."""
        return self._coefs.copy()

    @property
    def raw_coefficients(self) -> np.ndarray:
        return self._raw.copy()

    @property
    def normalize(self) -> bool:
        return self._normalize

    @classmethod
    def from_record(cls, record) -> "Shell":
        """Build from any object with center, angular_momentum, exponents,
        raw_coefficients and normalize attributes (e.g. synthetic.ShellRecord)."""
        return cls(record.center, record.angular_momentum, list(record.exponents),
                   np.asarray(record.raw_coefficients, dtype=float), normalize=bool(record.normalize))


class Basis:
    """Ordered shells with contraction-major AO offsets (types.hpp:108-124)."""

    def __init__(self, shells):
        shells = list(shells)
        for s in shells:
            if not isinstance(s, Shell):
                raise TypeError("Basis requires Shell objects")
        self._shells = tuple(shells)
        offsets, total = [], 0
        for s in shells:
            offsets.append(total)
            total += s.ao_count
        self._offsets = tuple(offsets)
        self._nao = total
        self._handles: dict[int, ctypes.c_void_p] = {}
        self._lock = threading.Lock()

    @property
    def shells(self) -> list[Shell]:
        return list(self._shells)

    @property
    def ao_offsets(self) -> tuple[int, ...]:
        return self._offsets

    @property
    def ao_count(self) -> int:
        return self._nao

    def _device(self, ctx: "nat.Context | None" = None):
        """The device-resident copy on ``ctx`` (uploaded on first use)."""
        ctx = ctx or nat.default_context()
        key = id(ctx)
        h = self._handles.get(key)
        if h is not None:
            return h[0]
        with self._lock:
            h = self._handles.get(key)
            if h is None:
                s = self._shells
                centers = np.ascontiguousarray([c for sh in s for c in sh.center] or [0.0], dtype=np.float64)
                ls = np.ascontiguousarray([sh.angular_momentum for sh in s] or [0], dtype=np.int32)
                nps = np.ascontiguousarray([sh.primitive_count for sh in s] or [0], dtype=np.int32)
                ncs = np.ascontiguousarray([sh.contraction_count for sh in s] or [0], dtype=np.int32)
                exps = np.ascontiguousarray(np.concatenate([sh._exps for sh in s]) if s else [0.0])
                coefs = np.ascontiguousarray(np.concatenate([sh._coefs.ravel() for sh in s]) if s else [0.0])
                handle = ctypes.c_void_p()
                nat.check(nat.lib().gx_basis_create(ctx.handle, len(s), nat.dptr(centers), nat.iptr(ls),
                                                    nat.iptr(nps), nat.iptr(ncs), nat.dptr(exps), nat.dptr(coefs),
                                                    None, ctypes.byref(handle)))
                self._handles[key] = (handle, ctx)  # the basis keeps its context alive
                h = (handle, ctx)
        return h[0]

    def __del__(self):  # pragma: no cover
        # At interpreter exit the process teardown frees device memory; only
        # release bases whose context is still open during normal execution.
        if sys.is_finalizing():
            return
        try:
            for handle, ctx in self._handles.values():
                if getattr(ctx, "handle", None):
                    nat.lib().gx_basis_destroy(handle)
        except Exception:
            pass


def field_arrays(field: MagneticField | None):
    if field is None:
        z = np.zeros(3, dtype=np.float64)
        return z, z.copy()
    if not isinstance(field, MagneticField):
        raise TypeError("field must be a MagneticField or None")
    return field._arrays()
