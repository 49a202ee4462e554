"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module, and only as the checker or as the timed CPU
baseline.  The product package never imports it.

Two native libraries sit behind the same Python functions:

* ``Oracle`` -- ``oracle/giao_oracle.c``, a plain-C restatement of the
  reference algorithm (builds anywhere gcc is present);
* ``Reference`` -- ``oracle/_ref/libgiaoref.so``, the reference library's own
  C++ sources compiled in place with a thin C shim (only where the reference
  checkout exists; used to pin the restatement and to generate fixtures).

``cholesky_eri`` restates the reference's NumPy pivot driver
(python/giao_integrals/cholesky.py:60-297) on top of either backend's
diagonal/column generators.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from collections import OrderedDict
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_l = ctypes.POINTER(ctypes.c_long)
_u32 = ctypes.POINTER(ctypes.c_uint32)


class OracleError(RuntimeError):
    """Raised with the oracle's status code and message."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def build(force: bool = False) -> Path:
    """Compile oracle/giao_oracle.c into oracle/_build/liboracle.so."""
    src = HERE / "giao_oracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(
        ["gcc", "-std=gnu11", "-O3", "-fPIC", "-fopenmp", "-shared", "-o", str(tmp), str(src), "-lm"],
        check=True,
    )
    os.replace(tmp, LIB)
    return LIB


# --------------------------------------------------------------------------
# basis description shared by both backends
# --------------------------------------------------------------------------


@dataclass
class ShellSpec:
    """One shell: centre, angular momentum, exponents, coefficients[ncontr][nprim]."""

    center: tuple[float, float, float]
    l: int
    exponents: list[float]
    coefficients: list[list[float]]
    normalize: bool = True

    @property
    def nprim(self) -> int:
        return len(self.exponents)

    @property
    def ncontr(self) -> int:
        return len(self.coefficients)

    @property
    def ncart(self) -> int:
        return (self.l + 1) * (self.l + 2) // 2

    @property
    def nao(self) -> int:
        return self.ncontr * self.ncart


def as_specs(shells) -> list[ShellSpec]:
    """Accept ShellSpec objects or objects exposing the reference Shell surface."""
    out = []
    for s in shells:
        if isinstance(s, ShellSpec):
            out.append(s)
            continue
        coefs = np.atleast_2d(np.asarray(s.raw_coefficients, dtype=float))
        out.append(
            ShellSpec(tuple(float(x) for x in s.center), int(s.angular_momentum),
                      [float(x) for x in s.exponents], coefs.tolist(), bool(s.normalize))
        )
    return out


@dataclass
class _Arrays:
    ns: int
    centers: np.ndarray
    ls: np.ndarray
    nprims: np.ndarray
    ncontrs: np.ndarray
    exps: np.ndarray
    coefs: np.ndarray
    normalize: np.ndarray
    nao: int
    ao_offsets: list[int] = field(default_factory=list)

    def args(self):
        return (
            ctypes.c_int(self.ns),
            self.centers.ctypes.data_as(_d),
            self.ls.ctypes.data_as(_i),
            self.nprims.ctypes.data_as(_i),
            self.ncontrs.ctypes.data_as(_i),
            self.exps.ctypes.data_as(_d),
            self.coefs.ctypes.data_as(_d),
        )


def _arrays(specs: list[ShellSpec]) -> _Arrays:
    ns = len(specs)
    centers = np.ascontiguousarray([c for s in specs for c in s.center], dtype=np.float64)
    ls = np.ascontiguousarray([s.l for s in specs], dtype=np.int32)
    nprims = np.ascontiguousarray([s.nprim for s in specs], dtype=np.int32)
    ncontrs = np.ascontiguousarray([s.ncontr for s in specs], dtype=np.int32)
    exps = np.ascontiguousarray([e for s in specs for e in s.exponents], dtype=np.float64)
    coefs = np.ascontiguousarray([c for s in specs for row in s.coefficients for c in row], dtype=np.float64)
    normalize = np.ascontiguousarray([int(s.normalize) for s in specs], dtype=np.int32)
    offsets, total = [], 0
    for s in specs:
        offsets.append(total)
        total += s.nao
    return _Arrays(ns, centers if ns else np.zeros(3), ls, nprims, ncontrs,
                   exps if len(exps) else np.zeros(1), coefs if len(coefs) else np.zeros(1),
                   normalize, total, offsets)


def _nuclei(nuclei):
    ch = np.ascontiguousarray([float(z) for z, _ in nuclei] or [0.0], dtype=np.float64)
    cc = np.ascontiguousarray([float(x) for _, c in nuclei for x in c] or [0.0, 0.0, 0.0], dtype=np.float64)
    return ch, cc


def _derivative_layout(shells, quartets, ncomp: int = 12):
    """Quartet array, offsets and total of packed (ncomp, na, nb, nc, nd) blocks."""
    q = np.ascontiguousarray(np.asarray(quartets, dtype=np.uint32).reshape(-1, 4))
    specs = as_specs(shells)
    sizes = [ncomp * int(np.prod([specs[k].nao for k in row])) for row in q]
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return q, offsets, int(offsets[-1])


def _vec3(v) -> np.ndarray:
    return np.ascontiguousarray([0.0, 0.0, 0.0] if v is None else v, dtype=np.float64)


class _Backend:
    prefix = ""

    def __init__(self, lib: ctypes.CDLL):
        self.lib = lib
        getattr(self.lib, self.prefix + "last_error").restype = ctypes.c_char_p

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def _check(self, rc: int):
        if rc != 0:
            msg = self._fn("last_error")().decode()
            raise OracleError(rc, msg)

    # subclasses provide _basis(specs) -> (_Arrays, extra args tuple)

    def boys(self, z: complex, nmax: int, scaled: bool = False):
        out = np.zeros(2 * (nmax + 1), dtype=np.float64)
        region = ctypes.c_int()
        err = ctypes.c_double()
        segs = ctypes.c_long()
        self._check(self._fn("boys")(ctypes.c_double(z.real), ctypes.c_double(z.imag), ctypes.c_int(nmax),
                                     ctypes.c_int(int(scaled)), out.ctypes.data_as(_d), ctypes.byref(region),
                                     ctypes.byref(err), ctypes.byref(segs)))
        return out.view(np.complex128), {"region": region.value, "estimated_absolute_error": err.value,
                                         "quadrature_segments": segs.value}

    def primitive_eri(self, prims, B=None, O=None) -> complex:
        """prims: 4 tuples (exponent, center, angular, coefficient, normalized)."""
        exps = np.ascontiguousarray([p[0] for p in prims], dtype=np.float64)
        centers = np.ascontiguousarray([c for p in prims for c in p[1]], dtype=np.float64)
        ang = np.ascontiguousarray([a for p in prims for a in p[2]], dtype=np.int32)
        coefs = np.ascontiguousarray([p[3] for p in prims], dtype=np.float64)
        norm = np.ascontiguousarray([int(p[4]) for p in prims], dtype=np.int32)
        out = np.zeros(2, dtype=np.float64)
        self._check(self._fn("primitive_eri")(exps.ctypes.data_as(_d), centers.ctypes.data_as(_d),
                                              ang.ctypes.data_as(_i), coefs.ctypes.data_as(_d),
                                              norm.ctypes.data_as(_i), _vec3(B).ctypes.data_as(_d),
                                              _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return complex(out[0], out[1])


class Oracle(_Backend):
    """The plain-C restatement (oracle/giao_oracle.c)."""

    prefix = "or_"

    def __init__(self):
        super().__init__(ctypes.CDLL(str(build())))
        self.lib.or_canonical_quartets.restype = ctypes.c_long
        self.lib.or_primitive_normalization.restype = ctypes.c_double

    def normalized_coefficients(self, spec: ShellSpec) -> list[list[float]]:
        c = np.ascontiguousarray(spec.coefficients, dtype=np.float64)
        if spec.normalize:
            e = np.ascontiguousarray(spec.exponents, dtype=np.float64)
            self._check(self.lib.or_normalize_shell(ctypes.c_int(spec.l), ctypes.c_int(spec.nprim),
                                                    ctypes.c_int(spec.ncontr), e.ctypes.data_as(_d),
                                                    c.ctypes.data_as(_d)))
        return c.tolist()

    def _basis(self, shells):
        specs = as_specs(shells)
        normed = [ShellSpec(s.center, s.l, s.exponents, self.normalized_coefficients(s), False) for s in specs]
        return _arrays(normed)

    def primitive_normalization(self, alpha, ang) -> float:
        return self.lib.or_primitive_normalization(ctypes.c_double(alpha), *[ctypes.c_int(a) for a in ang])

    def canonical_quartets(self, ns: int) -> np.ndarray:
        n = self.lib.or_canonical_quartets(ctypes.c_int(ns), None)
        out = np.zeros((max(n, 1), 4), dtype=np.uint32)
        self.lib.or_canonical_quartets(ctypes.c_int(ns), out.ctypes.data_as(_u32))
        return out[:n]

    def eri_shell(self, shells, quartet, B=None, O=None) -> np.ndarray:
        a = self._basis(shells)
        sh = np.ascontiguousarray(quartet, dtype=np.int32)
        shape = tuple(as_specs(shells)[k].nao for k in quartet)
        out = np.zeros(int(np.prod(shape)), dtype=np.complex128)
        self._check(self.lib.or_eri_shell(*a.args(), sh.ctypes.data_as(_i), _vec3(B).ctypes.data_as(_d),
                                          _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out.reshape(shape)

    def eri_batch(self, shells, quartets, B=None, O=None, threads: int = 1):
        a = self._basis(shells)
        q = np.ascontiguousarray(np.asarray(quartets, dtype=np.uint32).reshape(-1, 4))
        specs = as_specs(shells)
        total = int(sum(np.prod([specs[k].nao for k in row]) for row in q)) if len(q) else 0
        out = np.zeros(max(total, 1), dtype=np.complex128)
        offsets = np.zeros(len(q) + 1, dtype=np.int64)
        self._check(self.lib.or_eri_batch(*a.args(), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                          _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                          ctypes.c_int(threads), out.ctypes.data_as(_d),
                                          offsets.ctypes.data_as(_l)))
        return out[:total], offsets

    def eri_full(self, shells, B=None, O=None, threads: int = 1) -> np.ndarray:
        a = self._basis(shells)
        n = a.nao
        out = np.zeros(max(n**4, 1), dtype=np.complex128)
        self._check(self.lib.or_eri_full(*a.args(), _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                         ctypes.c_int(threads), out.ctypes.data_as(_d)))
        return out[: n**4].reshape(n, n, n, n)

    def nuclear(self, shells, nuclei, B=None, O=None) -> np.ndarray:
        """Nuclear-attraction matrix; nuclei = [(charge, (x, y, z)), ...]."""
        a = self._basis(shells)
        n = a.nao
        ch, cc = _nuclei(nuclei)
        out = np.zeros(max(n * n, 1), dtype=np.complex128)
        self._check(self.lib.or_nuclear_matrix(*a.args(), ctypes.c_int(len(nuclei)), ch.ctypes.data_as(_d),
                                               cc.ctypes.data_as(_d), _vec3(B).ctypes.data_as(_d),
                                               _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out[: n * n].reshape(n, n)

    def eri_center_derivatives(self, shells, quartets, B=None, O=None):
        """Centre-derivative blocks (4, 3, na, nb, nc, nd) of each quartet,
        packed in input order; returns (values, offsets)."""
        a = self._basis(shells)
        q, offsets, total = _derivative_layout(shells, quartets)
        out = np.zeros(max(total, 1), dtype=np.complex128)
        self._check(self.lib.or_eri_center_derivatives(*a.args(), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                                       _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                       out.ctypes.data_as(_d)))
        return out[:total], offsets

    def eri_magnetic_derivatives(self, shells, quartets, B=None, O=None):
        """Magnetic-derivative blocks (3, na, nb, nc, nd) of each quartet,
        packed in input order; returns (values, offsets)."""
        a = self._basis(shells)
        q, offsets, total = _derivative_layout(shells, quartets, 3)
        out = np.zeros(max(total, 1), dtype=np.complex128)
        self._check(self.lib.or_eri_magnetic_derivatives(*a.args(), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                                         _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                         out.ctypes.data_as(_d)))
        return out[:total], offsets

    def eri_mixed_derivatives(self, shells, quartets, B=None, O=None):
        """Mixed field/centre derivative blocks (4, 3, 3, na, nb, nc, nd) of
        each quartet, packed in input order; returns (values, offsets)."""
        a = self._basis(shells)
        q, offsets, total = _derivative_layout(shells, quartets, 36)
        out = np.zeros(max(total, 1), dtype=np.complex128)
        self._check(self.lib.or_eri_mixed_derivatives(*a.args(), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                                      _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                      out.ctypes.data_as(_d)))
        return out[:total], offsets

    def eri_derivative_bounds(self, shells, B=None, O=None) -> np.ndarray:
        """Derivative Schwarz factors of every ordered shell pair, [ns, ns]."""
        a = self._basis(shells)
        out = np.zeros((max(a.ns, 1), max(a.ns, 1)), dtype=np.float64)
        self._check(self.lib.or_eri_derivative_bounds(*a.args(), _vec3(B).ctypes.data_as(_d),
                                                      _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out[: a.ns, : a.ns]

    def schwarz(self, shells, B=None, O=None) -> np.ndarray:
        a = self._basis(shells)
        out = np.zeros((max(a.ns, 1), max(a.ns, 1)), dtype=np.float64)
        self._check(self.lib.or_schwarz(*a.args(), _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                        out.ctypes.data_as(_d)))
        return out[: a.ns, : a.ns]

    def cholesky_diagonal(self, shells, pairs, B=None, O=None, threads: int = 1) -> np.ndarray:
        a = self._basis(shells)
        p = np.ascontiguousarray(np.asarray(pairs, dtype=np.int64).reshape(-1, 2))
        out = np.zeros((a.nao, a.nao), dtype=np.float64)
        self._check(self.lib.or_cholesky_diagonal(*a.args(), p.ctypes.data_as(_l), ctypes.c_long(len(p)),
                                                  _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                  ctypes.c_int(threads), out.ctypes.data_as(_d)))
        return out

    def cholesky_columns(self, shells, pivots, B=None, O=None, threads: int = 1) -> np.ndarray:
        a = self._basis(shells)
        p = np.ascontiguousarray(np.asarray(pivots, dtype=np.int64).reshape(-1, 2))
        real = B is None or all(x == 0 for x in B)
        n = a.nao
        out = np.zeros((len(p), n * n), dtype=np.float64 if real else np.complex128)
        self._check(self.lib.or_cholesky_columns(*a.args(), p.ctypes.data_as(_l), ctypes.c_long(len(p)),
                                                 _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                 ctypes.c_int(threads), ctypes.c_int(int(real)),
                                                 out.ctypes.data_as(_d)))
        return out


class Reference(_Backend):
    """The reference library's own sources (oracle/_ref), where they were built."""

    prefix = "ref_"

    def __init__(self, path: Path | None = None):
        if path is None:
            path = HERE / "_ref" / "libgiaoref.so"
        if not Path(path).exists():
            raise FileNotFoundError(f"{path} not built (oracle/build_ref.py needs the reference checkout)")
        super().__init__(ctypes.CDLL(str(path)))

    def _basis(self, shells):
        return _arrays(as_specs(shells))

    def _bargs(self, a: _Arrays):
        return a.args() + (a.normalize.ctypes.data_as(_i),)

    def normalized_coefficients_all(self, shells) -> np.ndarray:
        a = self._basis(shells)
        out = np.zeros(max(len(a.coefs), 1))
        self._check(self.lib.ref_shell_coefficients(*self._bargs(a), out.ctypes.data_as(_d)))
        return out[: len(a.coefs)]

    def eri_batch(self, shells, quartets, B=None, O=None, threads: int = 1, screening: float = 0.0):
        a = self._basis(shells)
        q = np.ascontiguousarray(np.asarray(quartets, dtype=np.uint32).reshape(-1, 4))
        specs = as_specs(shells)
        sizes = [int(np.prod([specs[k].nao for k in row])) for row in q]
        out = np.zeros(max(sum(sizes), 1), dtype=np.complex128)
        stats = np.zeros(3, dtype=np.int64)
        self._check(self.lib.ref_eri_batch(*self._bargs(a), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                           _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                           ctypes.c_int(threads), ctypes.c_double(screening),
                                           out.ctypes.data_as(_d), stats.ctypes.data_as(_l)))
        offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        return out[: sum(sizes)], offsets, stats

    def eri_shell(self, shells, quartet, B=None, O=None) -> np.ndarray:
        vals, _, _ = self.eri_batch(shells, [quartet], B, O)
        specs = as_specs(shells)
        return vals.reshape(tuple(specs[k].nao for k in quartet))

    def eri_full(self, shells, B=None, O=None, threads: int = 1) -> np.ndarray:
        a = self._basis(shells)
        n = a.nao
        out = np.zeros(max(n**4, 1), dtype=np.complex128)
        self._check(self.lib.ref_eri_full(*self._bargs(a), _vec3(B).ctypes.data_as(_d),
                                          _vec3(O).ctypes.data_as(_d), ctypes.c_int(threads),
                                          out.ctypes.data_as(_d)))
        return out[: n**4].reshape(n, n, n, n)

    def nuclear(self, shells, nuclei, B=None, O=None) -> np.ndarray:
        a = self._basis(shells)
        n = a.nao
        ch, cc = _nuclei(nuclei)
        out = np.zeros(max(n * n, 1), dtype=np.complex128)
        self._check(self.lib.ref_nuclear_matrix(*self._bargs(a), ctypes.c_int(len(nuclei)), ch.ctypes.data_as(_d),
                                                cc.ctypes.data_as(_d), _vec3(B).ctypes.data_as(_d),
                                                _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out[: n * n].reshape(n, n)

    def eri_center_derivatives(self, shells, quartets, B=None, O=None):
        a = self._basis(shells)
        q, offsets, total = _derivative_layout(shells, quartets)
        out = np.zeros(max(total, 1), dtype=np.complex128)
        self._check(self.lib.ref_eri_center_derivatives(*self._bargs(a), q.ctypes.data_as(_u32),
                                                        ctypes.c_long(len(q)), _vec3(B).ctypes.data_as(_d),
                                                        _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out[:total], offsets

    def eri_magnetic_derivatives(self, shells, quartets, B=None, O=None):
        """Magnetic-derivative blocks (3, na, nb, nc, nd) of each quartet,
        packed in input order; returns (values, offsets)."""
        a = self._basis(shells)
        q, offsets, total = _derivative_layout(shells, quartets, 3)
        out = np.zeros(max(total, 1), dtype=np.complex128)
        self._check(self.lib.ref_eri_magnetic_derivatives(*self._bargs(a), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                                         _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                         out.ctypes.data_as(_d)))
        return out[:total], offsets

    def eri_mixed_derivatives(self, shells, quartets, B=None, O=None):
        """Mixed field/centre derivative blocks (4, 3, 3, na, nb, nc, nd) of
        each quartet, packed in input order; returns (values, offsets)."""
        a = self._basis(shells)
        q, offsets, total = _derivative_layout(shells, quartets, 36)
        out = np.zeros(max(total, 1), dtype=np.complex128)
        self._check(self.lib.ref_eri_mixed_derivatives(*self._bargs(a), q.ctypes.data_as(_u32), ctypes.c_long(len(q)),
                                                      _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                      out.ctypes.data_as(_d)))
        return out[:total], offsets

    def contract_eri_derivatives(self, shells, atoms, natom, quartets, offsets, values, coulomb=(), exchange=(),
                                 gamma=None) -> np.ndarray:
        """Reference per-atom contraction (complex (natom, 3))."""
        a = self._basis(shells)
        n = a.nao
        q = np.ascontiguousarray(np.asarray(quartets, dtype=np.uint32).reshape(-1, 4))
        at = np.ascontiguousarray(atoms, dtype=np.int64)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        vals = np.ascontiguousarray(values, dtype=np.complex128)
        cj = np.ascontiguousarray([m for pair in coulomb for m in pair] or [np.zeros((n, n))], dtype=np.complex128)
        kx = np.ascontiguousarray([m for pair in exchange for m in pair] or [np.zeros((n, n))], dtype=np.complex128)
        g = None if gamma is None else np.ascontiguousarray(gamma, dtype=np.complex128)
        out = np.zeros((natom, 3), dtype=np.complex128)
        self._check(self.lib.ref_contract_eri_derivatives(
            *self._bargs(a), at.ctypes.data_as(_l), ctypes.c_long(natom), q.ctypes.data_as(_u32),
            ctypes.c_long(len(q)), off.ctypes.data_as(_l), vals.ctypes.data_as(_d), ctypes.c_int(len(coulomb)),
            cj.ctypes.data_as(_d), ctypes.c_int(len(exchange)), kx.ctypes.data_as(_d),
            None if g is None else g.ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out

    def eri_derivative_bounds(self, shells, B=None, O=None) -> np.ndarray:
        a = self._basis(shells)
        out = np.zeros((max(a.ns, 1), max(a.ns, 1)), dtype=np.float64)
        self._check(self.lib.ref_eri_derivative_bounds(*self._bargs(a), _vec3(B).ctypes.data_as(_d),
                                                       _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out[: a.ns, : a.ns]

    def schwarz(self, shells, B=None, O=None) -> np.ndarray:
        a = self._basis(shells)
        out = np.zeros((max(a.ns, 1), max(a.ns, 1)), dtype=np.float64)
        self._check(self.lib.ref_schwarz(*self._bargs(a), _vec3(B).ctypes.data_as(_d),
                                         _vec3(O).ctypes.data_as(_d), out.ctypes.data_as(_d)))
        return out[: a.ns, : a.ns]

    def cholesky_diagonal(self, shells, pairs, B=None, O=None, threads: int = 1) -> np.ndarray:
        a = self._basis(shells)
        p = np.ascontiguousarray(np.asarray(pairs, dtype=np.int64).reshape(-1, 2))
        out = np.zeros((a.nao, a.nao), dtype=np.float64)
        self._check(self.lib.ref_cholesky_diagonal(*self._bargs(a), p.ctypes.data_as(_l), ctypes.c_long(len(p)),
                                                   _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                   ctypes.c_int(threads), out.ctypes.data_as(_d)))
        return out

    def cholesky_columns(self, shells, pivots, B=None, O=None, threads: int = 1) -> np.ndarray:
        a = self._basis(shells)
        p = np.ascontiguousarray(np.asarray(pivots, dtype=np.int64).reshape(-1, 2))
        real = B is None or all(x == 0 for x in B)
        n = a.nao
        out = np.zeros((len(p), n * n), dtype=np.float64 if real else np.complex128)
        self._check(self.lib.ref_cholesky_columns(*self._bargs(a), p.ctypes.data_as(_l), ctypes.c_long(len(p)),
                                                  _vec3(B).ctypes.data_as(_d), _vec3(O).ctypes.data_as(_d),
                                                  ctypes.c_int(threads), out.ctypes.data_as(_d)))
        return out


# --------------------------------------------------------------------------
# pivoted Cholesky driver (python/giao_integrals/cholesky.py:60-297)
# --------------------------------------------------------------------------


@dataclass
class CholeskyResult:
    vectors: np.ndarray
    pivots: np.ndarray
    threshold: float
    max_residual_diagonal: float


def cholesky_eri(backend: _Backend, shells, B=None, O=None, threshold: float = 1e-8,
                 screening_threshold: float = 0.0, threads: int = 1, max_bytes: int | None = None,
                 pivot_batch_size: int = 32, max_pivots: int | None = None, follow=None) -> CholeskyResult:
    """Restatement of the reference driver with the given integral backend.

    Checker-only options (not reference options):
    ``max_pivots`` stops after that many pivots and returns the partial
    factorisation, so that the pivot sequence and factors of a large system
    can be compared on a prefix.
    ``follow`` (pivots (M, 2) of another factorisation) replays the driver
    along that sequence: at every step the driver makes its own choice by
    the reference rules (global argmax, local block rule, raw-column cache
    state), and where the followed pivot differs it records the residual gap
    between the two and continues with the followed one.  The result's
    ``forced_steps`` and ``max_forced_gap`` then say whether every choice of
    the other factorisation was the reference's or tied with it."""
    specs = as_specs(shells)
    n = sum(s.nao for s in specs)
    offsets = []
    t = 0
    for s in specs:
        offsets.append(t)
        t += s.nao
    spans = [slice(o, o + s.nao) for o, s in zip(offsets, specs)]
    owners = np.repeat(np.arange(len(specs)), [s.nao for s in specs])
    # single centre: the London phase cancels, use the zero-field backend (cholesky.py:130-133)
    single = all(tuple(s.center) == tuple(specs[0].center) for s in specs)
    zero = [0.0, 0.0, 0.0]
    iB = zero if single or B is None else list(B)
    iO = zero if single or O is None else list(O)
    diagonal = np.zeros((n, n))
    bounds = backend.schwarz(shells, iB, iO) ** 2 if screening_threshold else None
    skipped, quartets = [], []
    for a in range(len(specs)):
        for b in range(a, len(specs)):
            if bounds is not None and bounds[a, b] <= min(threshold, screening_threshold):
                diagonal[spans[a], spans[b]] = bounds[a, b]
                diagonal[spans[b], spans[a]] = bounds[a, b]
                skipped.append((a, b))
            else:
                quartets.append((a, b))

    def read_diagonal(pairs):
        if not pairs:
            return
        measured = backend.cholesky_diagonal(shells, pairs, iB, iO, threads)
        for a, b in pairs:
            diagonal[spans[a], spans[b]] = measured[spans[a], spans[b]]
            diagonal[spans[b], spans[a]] = measured[spans[b], spans[a]]

    read_diagonal(quartets)
    residual = diagonal.ravel().copy()
    floor = 64 * np.finfo(float).eps * float(np.max(residual, initial=0.0))
    tolerance = max(threshold, floor)
    real = B is None or all(x == 0 for x in B) or single
    dtype = np.float64 if real else np.complex128
    row_bytes = n * n * 16 + 16
    limit = n * n if max_bytes is None else min(n * n, max_bytes // row_bytes)
    factors = np.empty((0, n * n), dtype=dtype)
    pivots: list[tuple[int, int]] = []
    reuse = not single or any(s.ncontr > 1 or s.nprim > 1 for s in specs)
    candidate_count = 32 if reuse else 8
    raw_cache: OrderedDict[int, np.ndarray] = OrderedDict()
    block_candidates = np.empty(0, dtype=int)
    candidates = np.empty(0, dtype=int)
    columns = np.empty((0, n * n), dtype=dtype)
    forced_steps, max_forced_gap = 0, 0.0
    while float(np.max(residual, initial=0.0)) > tolerance:
        if max_pivots is not None and len(pivots) >= max_pivots:
            break
        if follow is not None and len(pivots) >= len(follow):
            break
        pivot = int(np.argmax(residual))
        if reuse and not real and pivot_batch_size > 1 and len(block_candidates):
            local = int(block_candidates[np.argmax(residual[block_candidates])])
            if residual[local] > tolerance and residual[local] >= 0.01 * residual[pivot]:
                pivot = local
        if follow is not None:
            other = int(follow[len(pivots)][0]) * n + int(follow[len(pivots)][1])
            if other != pivot:
                forced_steps += 1
                max_forced_gap = max(max_forced_gap, abs(float(residual[pivot]) - float(residual[other])))
                pivot = other
        rank = len(pivots)
        if rank >= limit:
            raise MemoryError(f"Cholesky ERI output requires at least {(rank + 1) * row_bytes} bytes, "
                              f"exceeding max_bytes={max_bytes}")
        if rank == len(factors):
            cap = min(limit, max(8, 2 * len(factors)))
            grown = np.empty((cap, n * n), dtype=dtype)
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
                ca, cb = specs[a].ncart, specs[b].ncart
                left = offsets[a] + (mu - offsets[a]) % ca + ca * np.arange(specs[a].ncontr)
                right = offsets[b] + (nu - offsets[b]) % cb + cb * np.arange(specs[b].ncontr)
                idx = (left[:, None] * n + right).ravel()
            else:
                idx = np.arange(n * n).reshape(n, n)[spans[a], spans[b]].ravel()
            idx = idx[residual[idx] > tolerance]
            candidates = idx[np.argsort(-residual[idx], kind="stable")[:candidate_count]]
            if pivot not in candidates:
                candidates[-1] = pivot
            block_candidates = candidates[: min(32, pivot_batch_size)]
            cmu, cnu = np.divmod(candidates, n)
            columns = backend.cholesky_columns(shells, list(zip(cmu.tolist(), cnu.tolist())), iB, iO, threads)
            if reuse:
                for k, cand in enumerate(candidates):
                    if cand != pivot:
                        raw_cache[int(cand)] = columns[k].copy()
                cap = min(1024, max(8, rank + 8))
                while len(raw_cache) > cap:
                    raw_cache.popitem(last=False)
            match = np.flatnonzero(candidates == pivot)
        if reuse:
            raw_cache.pop(pivot, None)
        column = columns[int(match[0])].copy()
        if rank:
            column -= factors[:rank, pivot].conj() @ factors[:rank]
        if real:
            sq = column.reshape(n, n)
            column = ((sq + sq.T) * 0.5).ravel()
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
    out = CholeskyResult(vectors, np.asarray(pivots, dtype=np.int64).reshape(-1, 2), threshold,
                         float(np.max(residual, initial=0.0)))
    out.forced_steps = forced_steps
    out.max_forced_gap = max_forced_gap
    out.stopped_by_threshold = float(np.max(residual, initial=0.0)) <= tolerance
    return out


# --------------------------------------------------------------------------
# per-atom contraction of ERI centre derivatives (src/assembly.cpp:87-158)
# --------------------------------------------------------------------------

_ORBIT = ((0, 1, 2, 3), (2, 3, 0, 1), (1, 0, 3, 2), (3, 2, 1, 0))


def contract_eri_derivatives(shells, atoms, natom, quartets, offsets, values, coulomb=(), exchange=(), gamma=None):
    """Restatement of detail::contract_eri_derivatives: for every canonical
    quartet, every distinct orbit image (identity, pair exchange, conjugate
    reversal, conjugate exchanged reversal; images with equal shell quartets
    counted once) contributes derivative x weight, the weight being
    sum_pairs P[nu,mu] Q[sig,lam] (Coulomb), P[nu,lam] Q[sig,mu] (exchange)
    and gamma[mu,nu,lam,sig] at the image's AO indices; the derivative is
    conjugated for the last two images.  Twelve partial sums per quartet,
    added to the slot shells' atoms in quartet and slot order.  NumPy, one
    quartet at a time (small cases)."""
    specs = as_specs(shells)
    nao = [s.nao for s in specs]
    start = np.concatenate([[0], np.cumsum(nao)]).astype(np.int64)
    out = np.zeros((natom, 3), dtype=np.complex128)
    q = np.asarray(quartets, dtype=np.int64).reshape(-1, 4)
    for row, x in enumerate(q):
        shape = [nao[s] for s in x]
        size = int(np.prod(shape))
        blk = np.asarray(values[offsets[row]:offsets[row + 1]]).reshape(4, 3, size)
        grids = np.meshgrid(*[start[s] + np.arange(nao[s]) for s in x], indexing="ij")
        ao = [g.ravel() for g in grids]
        active = []
        for orbit, perm in enumerate(_ORBIT):
            image = tuple(x[perm[k]] for k in range(4))
            if any(image == tuple(x[_ORBIT[p][k]] for k in range(4)) for p in range(orbit)):
                continue
            active.append(orbit)
        partial = np.zeros((4, 3), dtype=np.complex128)
        for orbit in active:
            perm = _ORBIT[orbit]
            mu, nu, lam, sig = (ao[perm[k]] for k in range(4))
            w = np.zeros(size, dtype=np.complex128)
            for P, Q in coulomb:
                w += np.asarray(P)[nu, mu] * np.asarray(Q)[sig, lam]
            for P, Q in exchange:
                w += np.asarray(P)[nu, lam] * np.asarray(Q)[sig, mu]
            if gamma is not None:
                w += np.asarray(gamma)[mu, nu, lam, sig]
            d = np.conj(blk) if orbit >= 2 else blk
            partial += (d * w[None, None, :]).sum(axis=2)
        for slot in range(4):
            out[atoms[x[slot]]] += partial[slot]
    return out
