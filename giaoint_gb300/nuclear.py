"""GIAO nuclear-attraction integrals on the GPU, with the reference's Python API.

Mirrors ``primitive_nuclear_attraction``, ``nuclear_attraction_shell`` and
``nuclear_attraction`` of the reference module (src/bindings.cpp:541-600,
src/nuclear.cpp:27-330): V[mu][nu] = sum_C -Z_C <mu| 1/|r - C| |nu> with
London orbitals, complex128, AO order of the basis.  The matrix is computed
by one device kernel (gx_nuclear_attraction) from the same primitive-pair
records and Boys function as the electron-repulsion path.
"""

from __future__ import annotations

from collections.abc import Sequence

import numpy as np

from . import _native as nat
from ._types import Basis, MagneticField, Nucleus, PrimitiveGaussian, Shell, field_arrays
from .eri import _validate_out

__all__ = ["nuclear_attraction", "nuclear_attraction_shell", "primitive_nuclear_attraction"]


def _nuclei_arrays(nuclei: Sequence[Nucleus]):
    nuclei = list(nuclei)
    for n in nuclei:
        if not isinstance(n, Nucleus):
            raise TypeError("nuclei must be Nucleus objects")
    charges = np.ascontiguousarray([n.charge for n in nuclei] or [0.0], dtype=np.float64)
    centers = np.ascontiguousarray([c for n in nuclei for c in n.center] or [0.0, 0.0, 0.0], dtype=np.float64)
    return len(nuclei), charges, centers


def _matrix(basis: Basis, nuclei, field, context=None) -> np.ndarray:
    ctx = context or nat.default_context()
    count, charges, centers = _nuclei_arrays(nuclei)
    B, O = field_arrays(field)
    n = basis.ao_count
    out = np.zeros((n, n), dtype=np.complex128)
    if n:
        nat.check(nat.lib().gx_nuclear_attraction(ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), count,
                                                  nat.dptr(charges), nat.dptr(centers),
                                                  nat.dptr(out.view(np.float64).reshape(-1))))
    return out


def nuclear_attraction(basis: Basis, nuclei: Sequence[Nucleus], *, field: MagneticField | None = None, out=None,
                       context=None) -> np.ndarray:
    """Full AO nuclear-attraction matrix (src/nuclear.cpp:304-330)."""
    if not isinstance(basis, Basis):
        raise TypeError("basis must be a Basis")
    n = basis.ao_count
    result = _validate_out(out, (n, n))
    result[...] = _matrix(basis, nuclei, field, context)
    return result


def nuclear_attraction_shell(a: Shell, b: Shell, nuclei: Sequence[Nucleus], *, field: MagneticField | None = None,
                             out=None, context=None) -> np.ndarray:
    """Shell-pair block, C-contiguous complex128 (a.ao_count, b.ao_count)
    (src/nuclear.cpp:207-302)."""
    if not isinstance(a, Shell) or not isinstance(b, Shell):
        raise TypeError("a and b must be Shell objects")
    result = _validate_out(out, (a.ao_count, b.ao_count))
    full = _matrix(Basis([a, b]), nuclei, field, context)
    result[...] = full[: a.ao_count, a.ao_count:]
    return result


def primitive_nuclear_attraction(bra: PrimitiveGaussian, ket: PrimitiveGaussian, nuclei: Sequence[Nucleus], *,
                                 field: MagneticField | None = None, context=None) -> complex:
    """One primitive pair (src/nuclear.cpp:181-205): coefficients and, when
    ``normalized``, the primitive normalisations of both Gaussians applied."""
    shells = []
    picks = []
    scale = 1.0
    for g in (bra, ket):
        if not isinstance(g, PrimitiveGaussian):
            raise TypeError("bra and ket must be PrimitiveGaussian objects")
        l = sum(g.angular)
        # raw unit-coefficient shell; the component's normalisation is folded in by the kernel
        shells.append(Shell(g.center, l, [g.exponent], [1.0], normalize=False))
        comps = [(x, y, l - x - y) for x in range(l, -1, -1) for y in range(l - x, -1, -1)]
        picks.append(comps.index(tuple(g.angular)))
        scale *= g.coefficient
        if not g.normalized:
            scale /= nat.lib().gx_primitive_normalization(g.exponent, *g.angular)
    full = _matrix(Basis(shells), nuclei, field, context)
    na = shells[0].ao_count
    return complex(full[picks[0], na + picks[1]] * scale)
