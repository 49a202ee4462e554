"""Molecules from atoms or XYZ and BSE-JSON Gaussian bases, with the
integral methods of this library (python/giao_integrals/molecule.py:285-475).

``Molecule(atoms, basis, *, unit, basis_format, field)`` builds the
Cartesian basis in atom order with shells of increasing angular momentum per
atom (general contractions kept as one shell, combined sp-type shells split),
converts coordinates to bohr, and carries the nuclei and the field.  Bases are
accepted as a BSE-JSON dictionary, a JSON file or inline JSON text; named
bases and Gaussian94/NWChem text need the basis_set_exchange package, as in
the reference, and raise ImportError without it.  The methods cover the
integrals this library computes: nuclear attraction, ERIs (full tensor or
streamed batches), Cholesky ERI factors and ERI centre derivatives.
"""

from __future__ import annotations

import json
import math
from collections.abc import Iterable, Mapping, Sequence
from os import PathLike
from pathlib import Path
from typing import Any

import numpy as np

from ._types import Basis, MagneticField, Nucleus, Shell
from .cholesky import cholesky_eri as _cholesky_eri
from .derivative_assembly import eri_derivative_contraction as _eri_derivative_contraction
from .eri import eri as _eri
from .eri import eri_batches as _eri_batches
from .eri import eri_derivative_batches as _eri_derivative_batches
from .nuclear import nuclear_attraction as _nuclear_attraction

__all__ = ["BOHR_IN_ANGSTROM", "Molecule"]

BOHR_IN_ANGSTROM = 0.529177210544  # CODATA 2022

ELEMENTS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
    "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr "
    "Rf Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og"
).split()
Z_OF = {sym: z for z, sym in enumerate(ELEMENTS, start=1)}
_FORMAT_BY_SUFFIX = {".json": "json", ".gbs": "gaussian94", ".g94": "gaussian94", ".nw": "nwchem",
                     ".nwchem": "nwchem"}


def _float(x: Any) -> float:
    """A number, accepting Fortran D exponents in strings."""
    if isinstance(x, str):
        x = x.replace("D", "E").replace("d", "e")
    return float(x)


def _element(value: Any) -> str:
    s = str(value).strip().capitalize()
    if s.isdecimal() and 1 <= int(s) <= len(ELEMENTS):
        s = ELEMENTS[int(s) - 1]
    if s not in Z_OF:
        raise ValueError(f"Unknown element {value!r}; use an element symbol or atomic number")
    return s


def _atoms_bohr(atoms, unit: str):
    scale = {"angstrom": 1.0 / BOHR_IN_ANGSTROM, "bohr": 1.0}
    if unit not in scale:
        raise ValueError("unit must be 'angstrom' or 'bohr'")
    out = []
    for n, atom in enumerate(atoms, start=1):
        try:
            sym, xyz = atom
            pos = tuple(_float(c) * scale[unit] for c in xyz)
            if len(pos) != 3 or not all(math.isfinite(c) for c in pos):
                raise ValueError("coordinates must be three finite numbers")
            out.append((_element(sym), pos))
        except (TypeError, ValueError, OverflowError) as e:
            raise ValueError(f"Invalid atom {n}: {e}") from e
    if not out:
        raise ValueError("A molecule must contain at least one atom")
    return tuple(out)


def _xyz_atoms(source):
    """Atoms of one XYZ frame from a path or multi-line text."""
    if isinstance(source, PathLike) or ("\n" not in source and "\r" not in source):
        text = Path(source).read_text(encoding="utf-8-sig")
    else:
        text = source.lstrip("\ufeff")
    lines = text.lstrip("\r\n").splitlines()
    try:
        count = int(lines[0].strip())
    except (IndexError, ValueError) as e:
        raise ValueError("XYZ must start with an integer atom count") from e
    if count < 1:
        raise ValueError("XYZ atom count must be positive")
    if len(lines) < count + 2:
        raise ValueError(f"XYZ requires a comment line and {count} atom lines")
    if any(line.strip() for line in lines[count + 2:]):
        raise ValueError("Expected one XYZ frame; extra atoms or frames follow the declared count")
    atoms = []
    for n, line in enumerate(lines[2:count + 2], start=3):
        fields = line.split()
        if len(fields) != 4:
            raise ValueError(f"XYZ line {n} must contain an element and three coordinates")
        atoms.append((fields[0], fields[1:]))
    return atoms


def _need_bse():
    try:
        import basis_set_exchange  # noqa: F401
    except ImportError as e:
        raise ImportError("Named, Gaussian94, and NWChem bases require basis-set-exchange; "
                          "BSE JSON input works without it.") from e
    return basis_set_exchange


def _basis_source(source, symbols, fmt):
    """The BSE-JSON dictionary of ``source``."""
    if fmt is not None and fmt not in ("json", "gaussian94", "nwchem"):
        raise ValueError("basis_format must be 'json', 'gaussian94', or 'nwchem'")
    if isinstance(source, Mapping):
        if fmt not in (None, "json"):
            raise ValueError("A basis dictionary uses basis_format='json'")
        return source
    if not isinstance(source, (str, PathLike)):
        raise TypeError("basis must be a basis name, file path, formatted text, or BSE dictionary")
    if isinstance(source, str) and ("\n" in source or "\r" in source or source.lstrip().startswith("{")):
        text = source
        if fmt is None:
            if not text.lstrip().startswith("{"):
                raise ValueError("Specify basis_format for inline Gaussian94 or NWChem text")
            fmt = "json"
    else:
        path = Path(source)
        looks_like_path = (isinstance(source, PathLike) or path.is_file() or path.suffix.lower() in _FORMAT_BY_SUFFIX
                           or "/" in str(source) or "\\" in str(source) or fmt is not None)
        if not looks_like_path:
            bse = _need_bse()
            try:
                return bse.get_basis(str(source), elements=sorted(set(symbols)))
            except (KeyError, ValueError) as e:
                raise ValueError(f"Could not load basis {source!r}: {e}") from e
        text = path.read_text(encoding="utf-8-sig")
        fmt = fmt or _FORMAT_BY_SUFFIX.get(path.suffix.lower())
        if fmt is None:
            raise ValueError("Cannot infer basis format; specify basis_format='gaussian94', 'nwchem', or 'json'")
    if fmt != "json":
        bse = _need_bse()
        try:
            return bse.read_formatted_basis_str(text, fmt, validate=True)
        except Exception as e:  # noqa: BLE001 - parser errors of any kind are reported as ValueError
            raise ValueError(f"Invalid {fmt} basis: {e}") from e
    try:
        data = json.loads(text)
    except ValueError as e:
        raise ValueError(f"Invalid BSE JSON basis: {e}") from e
    if not isinstance(data, Mapping):
        raise ValueError("BSE JSON basis must be an object containing 'elements'")
    return data


def _shells_for(atoms, data):
    """Shells in atom order, increasing angular momentum within an atom, and
    the owner atom of each shell."""
    elements = data.get("elements")
    if not isinstance(elements, Mapping):
        raise ValueError("BSE basis data must contain an 'elements' object keyed by atomic number")
    shells, owners = [], []
    for ia, (sym, pos) in enumerate(atoms):
        el = elements.get(str(Z_OF[sym]))
        if not isinstance(el, Mapping):
            raise ValueError(f"Basis has no data for element {sym}")
        if el.get("ecp_potentials") or el.get("ecp_electrons", 0):
            raise ValueError(f"Basis for {sym} contains an ECP; only all-electron bases are supported")
        entries = el.get("electron_shells")
        if not isinstance(entries, list) or not entries:
            raise ValueError(f"Basis for {sym} has no electron shells")
        specs = []
        for n, entry in enumerate(entries):
            try:
                if entry.get("function_type", "gto") not in ("gto", "gto_cartesian", "gto_spherical"):
                    raise ValueError("only Gaussian orbital shells are supported")
                ls = entry["angular_momentum"]
                if not ls or any(type(l) is not int or l < 0 for l in ls):
                    raise ValueError("angular momenta must be non-negative integers")
                if len(set(ls)) != len(ls):
                    raise ValueError("combined shells must have distinct angular momenta")
                exps = [_float(x) for x in entry["exponents"]]
                rows = [[_float(x) for x in row] for row in entry["coefficients"]]
                if len(ls) == 1:
                    specs.append((ls[0], exps, rows))
                elif len(rows) == len(ls):
                    specs.extend((l, exps, [row]) for l, row in zip(ls, rows))
                else:
                    raise ValueError("combined shells require one coefficient row per angular momentum")
            except (AttributeError, KeyError, TypeError, ValueError, OverflowError) as e:
                raise ValueError(f"Invalid basis shell {n} for {sym}: {e}") from e
        for l, exps, rows in sorted(specs, key=lambda t: t[0]):
            try:
                shells.append(Shell(pos, l, exps, np.asarray(rows, dtype=float)))
            except (TypeError, ValueError, OverflowError) as e:
                raise ValueError(f"Invalid basis shell for {sym}: {e}") from e
            owners.append(ia)
    return Basis(shells), tuple(owners)


class Molecule:
    """Geometry (bohr), Cartesian basis, nuclei and field, with the integral
    methods of this library."""

    def __init__(self, atoms: Iterable[tuple[str, Sequence[float]]], basis, *, unit: str = "angstrom",
                 basis_format: str | None = None, field: MagneticField | None = None) -> None:
        if field is not None and not isinstance(field, MagneticField):
            raise TypeError("field must be a MagneticField or None")
        self._atoms = _atoms_bohr(atoms, unit)
        data = _basis_source(basis, [s for s, _ in self._atoms], basis_format)
        self._basis, self._shell_atoms = _shells_for(self._atoms, data)
        self._nuclei = tuple(Nucleus(float(Z_OF[s]), p) for s, p in self._atoms)
        self._field = field if field is not None else MagneticField()

    @classmethod
    def from_xyz(cls, source, basis, *, unit: str = "angstrom", basis_format: str | None = None,
                 field: MagneticField | None = None) -> "Molecule":
        """One XYZ frame from a path or multi-line text (comment line required)."""
        return cls(_xyz_atoms(source), basis, unit=unit, basis_format=basis_format, field=field)

    @property
    def atoms(self):
        return self._atoms

    @property
    def basis(self) -> Basis:
        return self._basis

    @property
    def nuclei(self):
        return self._nuclei

    @property
    def shell_atoms(self) -> tuple[int, ...]:
        return self._shell_atoms

    @property
    def field(self) -> MagneticField:
        return self._field

    @property
    def ao_count(self) -> int:
        return self._basis.ao_count

    def __repr__(self) -> str:
        return f"Molecule(atoms={len(self._atoms)}, shells={len(self._shell_atoms)}, cartesian_aos={self.ao_count})"

    def nuclear_attraction(self):
        return _nuclear_attraction(self._basis, self._nuclei, field=self._field)

    def eri(self, *, max_bytes: int | None = None, screening_threshold: float = 0.0, threads: int | None = None):
        """Full (nao, nao, nao, nao) tensor; ``max_bytes=None`` lifts the cap."""
        return _eri(self._basis, field=self._field, storage="full",
                    max_bytes=self.ao_count ** 4 * 16 if max_bytes is None else max_bytes,
                    screening_threshold=screening_threshold, threads=threads)

    def cholesky_eri(self, *, threshold: float = 1e-8, screening_threshold: float = 0.0, threads: int | None = None,
                     max_bytes: int | None = None, pivot_batch_size: int = 32):
        return _cholesky_eri(self._basis, field=self._field, threshold=threshold,
                             screening_threshold=screening_threshold, threads=threads, max_bytes=max_bytes,
                             pivot_batch_size=pivot_batch_size)

    def eri_batches(self, *, target_bytes: int = 64 * 1024 ** 2, screening_threshold: float = 0.0,
                    threads: int | None = None):
        return _eri_batches(self._basis, field=self._field, target_bytes=target_bytes,
                            screening_threshold=screening_threshold, threads=threads)

    def eri_derivative_batches(self, *, quartets=None, target_bytes: int = 64 * 1024 ** 2,
                               screening_threshold: float = 0.0, threads: int | None = None):
        """Centre-derivative blocks (4, 3, na, nb, nc, nd); ``shell_atoms``
        maps shells to atoms (repeated slots add)."""
        return _eri_derivative_batches(self._basis, field=self._field, quartets=quartets, target_bytes=target_bytes,
                                       screening_threshold=screening_threshold, threads=threads)

    def eri_derivative_contraction(self, *, coulomb_pairs=(), exchange_pairs=(), gamma=None,
                                   target_bytes=64 * 1024 ** 2, screening_threshold=0.0, threads=None, out=None):
        """Per-atom contraction of the ERI centre derivatives with this
        molecule's field and shell owners, complex128 (natom, 3)."""
        return _eri_derivative_contraction(self._basis, self._shell_atoms, len(self._atoms), field=self._field,
                                           coulomb_pairs=coulomb_pairs, exchange_pairs=exchange_pairs, gamma=gamma,
                                           target_bytes=target_bytes, screening_threshold=screening_threshold,
                                           threads=threads, out=out)
