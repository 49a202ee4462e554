"""Per-atom contraction of ERI centre derivatives with fixed densities, on
the GPU (python/giao_integrals/derivative_assembly.py:14-148).

``eri_derivative_contraction`` returns, for each atom A and nuclear axis r,
the sum over canonical shell quartets and their distinct orbit images of
dI/dR[A, r] times the density weight: Coulomb pairs P[nu,mu] Q[sig,lam],
exchange pairs P[nu,lam] Q[sig,mu] and a dense gamma[mu,nu,lam,sig].  The
derivative blocks never leave the device: gx_eri_derivative_contraction
computes them in bounded batches, contracts each quartet in one warp and
returns twelve partial sums per quartet, which are added to the atoms in
quartet and slot order: repeated calls give identical results.  A different
``target_bytes`` changes the batches and with them the launch configuration
of the derived integrals (the lane split of their sums), so results across
batch sizes agree to rounding, not bit for bit as in the reference.  Densities are not conjugated and no
1/2, spin, exchange or force sign is applied, as in the reference.
"""

from __future__ import annotations

from operator import index

import numpy as np

from . import _native as nat
from ._threads import resolve_num_threads
from ._types import Basis, MagneticField, field_arrays
from .eri import _EriDerivativeSchwarzBounds, canonical_quartets

__all__ = ["eri_derivative_contraction"]


def eri_derivative_contraction(basis: Basis, shell_atoms, natom, *, field: MagneticField | None = None,
                               coulomb_pairs=(), exchange_pairs=(), gamma=None, target_bytes=64 * 1024 ** 2,
                               screening_threshold=0.0, threads=None, out=None, context=None):
    """Per-atom ERI centre-derivative contractions, complex128 (natom, 3)."""
    try:
        if isinstance(natom, (bool, np.bool_)):
            raise TypeError
        natom = index(natom)
        atoms = [index(a) if not isinstance(a, (bool, np.bool_)) else -1 for a in shell_atoms]
    except TypeError as error:
        raise ValueError("natom and shell_atoms must be integers") from error
    if natom < 0 or len(atoms) != len(basis.shells) or any(a < 0 or a >= natom for a in atoms):
        raise ValueError("shell_atoms must map every shell to an atom in [0,natom)")
    n = basis.ao_count
    originals = []

    def pairs(values):
        result = []
        for pair in values:
            if len(pair) != 2:
                raise ValueError("each density pair must contain P and Q")
            originals.extend(m for m in pair if isinstance(m, np.ndarray))
            p, q = (np.ascontiguousarray(m, dtype=np.complex128) for m in pair)
            if p.shape != (n, n) or q.shape != (n, n):
                raise ValueError("density matrices must have shape (nao,nao)")
            result.append((p, q))
        return result

    coulomb = pairs(coulomb_pairs)
    exchange = pairs(exchange_pairs)
    if gamma is not None and (not isinstance(gamma, np.ndarray) or gamma.shape != (n,) * 4
                              or not gamma.flags.c_contiguous
                              or gamma.dtype not in (np.dtype("float64"), np.dtype("complex128"))):
        raise ValueError("gamma must be a C-contiguous float64/complex128 (nao,)*4 ndarray")
    if not coulomb and not exchange and gamma is None:
        raise ValueError("at least one density pair or gamma is required")
    if (isinstance(target_bytes, (bool, np.bool_)) or not isinstance(target_bytes, (int, np.integer))
            or target_bytes <= 0):
        raise ValueError("target_bytes must be a positive integer")
    threshold = float(screening_threshold)
    if not np.isfinite(threshold) or threshold < 0:
        raise ValueError("screening_threshold must be finite and non-negative")
    count = resolve_num_threads(threads)
    if out is None:
        result = np.zeros((natom, 3), dtype=np.complex128)
    else:
        if (not isinstance(out, np.ndarray) or out.shape != (natom, 3) or out.dtype != np.complex128
                or not out.flags.c_contiguous or not out.flags.writeable):
            raise ValueError("out must be writable C-contiguous complex128 (natom,3)")
        result = out
        dens = [m for pair in coulomb + exchange for m in pair] + originals + ([gamma] if gamma is not None else [])
        for m in dens:
            if np.shares_memory(result, m):
                raise ValueError("out must not overlap input densities")
        result.fill(0)
    q = canonical_quartets(len(basis.shells))
    if threshold > 0 and len(q):
        bounds = _EriDerivativeSchwarzBounds(basis, field=field, threads=count)
        q = q[bounds.quartet_bounds(q) >= threshold]
    if len(q) == 0 or natom == 0:
        return result
    ctx = context or nat.default_context()
    B, O = field_arrays(field)
    cj = np.ascontiguousarray([m for pair in coulomb for m in pair] or [np.zeros((1,), np.complex128)])
    kx = np.ascontiguousarray([m for pair in exchange for m in pair] or [np.zeros((1,), np.complex128)])
    g = None if gamma is None else gamma
    at = np.ascontiguousarray(atoms, dtype=np.int64)
    acc = np.zeros(2 * natom * 3, dtype=np.float64)
    q = np.ascontiguousarray(q)
    nat.check(nat.lib().gx_eri_derivative_contraction(
        ctx.handle, basis._device(ctx), nat.dptr(B), nat.dptr(O), nat.u32ptr(q), len(q), nat.i64ptr(at), int(natom),
        len(coulomb), nat.dptr(cj.view(np.float64).reshape(-1)), len(exchange),
        nat.dptr(kx.view(np.float64).reshape(-1)),
        None if g is None else nat.dptr(g.view(np.float64).reshape(-1)), int(g is not None and np.iscomplexobj(g)),
        max(1, int(target_bytes) // 16), nat.dptr(acc)))
    result += acc.view(np.complex128).reshape(natom, 3)
    return result
