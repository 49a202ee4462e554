"""Seeded synthetic inputs for the electron-repulsion workloads.

The reference quotes its numbers on real basis sets and molecules that need
``basis_set_exchange`` and network access.  These generators stand in for
them with fixed seeds, sizes and value distributions:

* ``atom_even_tempered``: one atom at the origin with uncontracted
  even-tempered Cartesian shells (the 19-AO full-tensor case and the 140-AO
  Cholesky case);
* ``random_molecule``: atoms uniform in a cube with a minimum separation,
  each carrying contracted shells s(6), s(1), s(1), p(3), p(1), d(1) with
  log-uniform exponents and uniform coefficients (normalised by ``Shell``);
* ``random_field`` / ``field_grid``: magnetic fields drawn uniformly in a
  ball by rejection;
* ``serving_requests``: a Poisson request stream of mixed ERI-block and
  Cholesky requests on molecules of varying size.

Every draw comes from ``numpy.random.default_rng(seed)`` in a fixed order, so
the same seed gives the same inputs on every machine.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

__all__ = [
    "ShellRecord",
    "atom_even_tempered",
    "full_tensor_atom",
    "cholesky_atom",
    "random_molecule",
    "random_field",
    "field_grid",
    "serving_requests",
    "MOLECULE_RECIPE",
]


@dataclass(frozen=True)
class ShellRecord:
    """Plain shell description: the constructor arguments of ``Shell``."""

    center: tuple[float, float, float]
    angular_momentum: int
    exponents: tuple[float, ...]
    raw_coefficients: tuple[tuple[float, ...], ...]
    normalize: bool = True


# (angular momentum, primitive count) per atom, in shell order
MOLECULE_RECIPE = ((0, 6), (0, 1), (0, 1), (1, 3), (1, 1), (2, 1))


def atom_even_tempered(counts, first, ratio=2.5, center=(0.0, 0.0, 0.0)) -> list[ShellRecord]:
    """Uncontracted even-tempered shells: ``counts[l]`` shells of angular
    momentum l with exponents ``first[l] * ratio**k``."""
    shells = []
    for l, count in enumerate(counts):
        for k in range(count):
            shells.append(ShellRecord(tuple(map(float, center)), l, (float(first[l] * ratio**k),), ((1.0,),)))
    return shells


def full_tensor_atom() -> list[ShellRecord]:
    """4 s (0.2*2.5^k), 3 p (0.3*2.5^k), 1 d (0.8): 19 Cartesian AOs."""
    return atom_even_tempered([4, 3, 1], [0.2, 0.3, 0.8])


def cholesky_atom() -> list[ShellRecord]:
    """10 s, 8 p, 6 d, 4 f, 2 g, ratio 2.5 from 0.05: 140 Cartesian AOs."""
    return atom_even_tempered([10, 8, 6, 4, 2], [0.05] * 5)


def random_molecule(seed: int = 2026, natoms: int = 12, box: float = 10.0, min_separation: float = 1.8,
                    exponent_range=(0.1, 5000.0), recipe=MOLECULE_RECIPE, rng=None) -> list[ShellRecord]:
    """Atoms uniform in [0, box)^3 (each redrawn until it is at least
    ``min_separation`` from every earlier atom), then per atom the shells of
    ``recipe`` with exponents exp(U(ln lo, ln hi)) and coefficients U(0.1, 1)."""
    rng = np.random.default_rng(seed) if rng is None else rng
    atoms: list[np.ndarray] = []
    while len(atoms) < natoms:
        c = rng.uniform(0.0, box, 3)
        if all(np.linalg.norm(c - a) >= min_separation for a in atoms):
            atoms.append(c)
    lo, hi = np.log(exponent_range[0]), np.log(exponent_range[1])
    shells = []
    for a in atoms:
        for l, k in recipe:
            exps = np.exp(rng.uniform(lo, hi, k))
            coefs = rng.uniform(0.1, 1.0, k)
            shells.append(ShellRecord(tuple(float(x) for x in a), int(l), tuple(float(e) for e in exps),
                                      (tuple(float(c) for c in coefs),)))
    return shells


def random_field(seed: int = 2026, bmax: float = 0.2, rng=None) -> tuple[float, float, float]:
    """B uniform in the ball |B| <= bmax (rejection from the cube)."""
    rng = np.random.default_rng(seed + 7919) if rng is None else rng
    while True:
        b = rng.uniform(-bmax, bmax, 3)
        if np.linalg.norm(b) <= bmax:
            return tuple(float(x) for x in b)


def field_grid(count: int = 64, bmax: float = 0.5, seed: int = 2026) -> list[tuple[float, float, float]]:
    """``count`` seeded fields in the ball |B| <= bmax, sorted by |B|."""
    rng = np.random.default_rng(seed + 104729)
    fields = [random_field(bmax=bmax, rng=rng) for _ in range(count)]
    return sorted(fields, key=lambda b: float(np.linalg.norm(b)))


@dataclass(frozen=True)
class Request:
    arrival: float                      # seconds from stream start
    kind: str                           # "eri" or "cholesky"
    shells: tuple[ShellRecord, ...]
    field: tuple[float, float, float]
    quartets: np.ndarray | None         # uint32[k,4] for "eri"
    threshold: float | None             # for "cholesky"


def serving_requests(count: int = 200, rate: float = 200.0, seed: int = 2026, atoms=(3, 40), bmax: float = 0.3,
                     max_entries: int = 1 << 24, cholesky_fraction: float = 0.25, cholesky_atoms=(3, 6),
                     thresholds=(1e-6, 1e-7, 1e-8)) -> list[Request]:
    """Poisson arrivals at ``rate`` req/s.  ERI requests draw a molecule of
    U{atoms} atoms and a seeded subset of its canonical quartets holding at
    most ``max_entries`` complex entries; Cholesky requests draw a smaller
    molecule and a threshold from ``thresholds``."""
    rng = np.random.default_rng(seed + 31337)
    t = 0.0
    out = []
    for _ in range(count):
        t += float(rng.exponential(1.0 / rate))
        field = random_field(bmax=bmax, rng=rng)
        if rng.uniform() < cholesky_fraction:
            nat = int(rng.integers(cholesky_atoms[0], cholesky_atoms[1] + 1))
            shells = random_molecule(natoms=nat, rng=rng)
            out.append(Request(t, "cholesky", tuple(shells), field, None,
                               float(thresholds[int(rng.integers(len(thresholds)))])))
        else:
            nat = int(rng.integers(atoms[0], atoms[1] + 1))
            shells = random_molecule(natoms=nat, rng=rng)
            sizes = np.array([(s.angular_momentum + 1) * (s.angular_momentum + 2) // 2 for s in shells])
            ns = len(shells)
            budget = int(rng.integers(1 << 16, max_entries + 1))
            picked = []
            used = 0
            while used < budget:
                q = rng.integers(0, ns, size=4)
                a, b, c, d = (int(x) for x in q)
                orbit = ((a, b, c, d), (c, d, a, b), (b, a, d, c), (d, c, b, a))
                canon = min(orbit)
                size = int(np.prod(sizes[list(canon)]))
                if used + size > budget:
                    break
                picked.append(canon)
                used += size
            out.append(Request(t, "eri", tuple(shells), field, np.asarray(picked, dtype=np.uint32).reshape(-1, 4),
                               None))
    return out
