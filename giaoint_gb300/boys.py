"""Complex Boys function F_0..F_n(z) on the GPU.

Mirrors ``boys`` and ``boys_with_diagnostics`` (src/bindings.cpp:444-482,
src/boys.cpp:245-294): same arguments, domain errors and region
classification.  The values come from the device kernel (Taylor grid,
asymptotic form or adaptive Gauss-Legendre quadrature); the diagnostics
report the reference's region for the argument and the method used here.
"""

from __future__ import annotations

import enum

import numpy as np

from . import _native as nat
from ._native import BoysNumericalError

__all__ = ["BoysRegion", "BoysNumericalError", "boys", "boys_with_diagnostics", "boys_many"]


class BoysRegion(enum.IntEnum):
    POWER_SERIES = 0
    ADAPTIVE_QUADRATURE = 1
    SCALED_QUADRATURE = 2
    POSITIVE_ASYMPTOTIC = 3


def _order(maximum_order) -> int:
    if isinstance(maximum_order, (bool, np.bool_)) or not isinstance(maximum_order, (int, np.integer)):
        raise TypeError("maximum_order must be an integer")
    if maximum_order < 0:
        raise TypeError("maximum_order must be non-negative")
    if maximum_order > 32:
        raise ValueError("complex Boys supports orders through 32")
    return int(maximum_order)


def boys_many(arguments, maximum_order: int, *, scaled: bool = False, context=None):
    """Vectorised form: complex128[count, maximum_order + 1] and region codes."""
    n = _order(maximum_order)
    z = np.ascontiguousarray(np.asarray(arguments, dtype=np.complex128).reshape(-1))
    ctx = context or nat.default_context()
    out = np.empty((len(z), n + 1), dtype=np.complex128)
    region = np.zeros(len(z), dtype=np.int32)
    nat.check(nat.lib().gx_boys(ctx.handle, nat.dptr(z.view(np.float64)), len(z), n, int(bool(scaled)),
                                nat.dptr(out.view(np.float64).reshape(-1)), nat.iptr(region)))
    return out, region


def boys(argument, maximum_order: int, *, scaled: bool = False) -> np.ndarray:
    """F_0..F_n(argument) (or e^z F_n when scaled) as complex128[n + 1]."""
    values, _ = boys_many([complex(argument)], maximum_order, scaled=scaled)
    return values[0]


def boys_with_diagnostics(argument, maximum_order: int, *, scaled: bool = False):
    values, region = boys_many([complex(argument)], maximum_order, scaled=scaled)
    z = complex(argument)
    r = BoysRegion(int(region[0]))
    if r == BoysRegion.POSITIVE_ASYMPTOTIC:
        method = "asymptotic"
    elif -16.0 <= z.real <= 108.0 and abs(z.imag) <= 12.0 and not (
            z.real >= 2 * maximum_order + 44 and abs(z.imag) <= 0.5 * z.real):
        method = "taylor_grid"
    elif z.real >= 2 * maximum_order + 44 and abs(z.imag) <= 0.5 * z.real:
        method = "asymptotic"
    else:
        method = "quadrature"
    details = {
        "region": r,
        "estimated_absolute_error": 1e-16 * float(np.max(np.abs(values[0]))),
        "quadrature_segments": 0 if method != "quadrature" else int(max(1, np.ceil(max(abs(z.real), abs(z.imag)) / 8))),
        "scaled": bool(scaled),
        "method": method,
    }
    return values[0], details
