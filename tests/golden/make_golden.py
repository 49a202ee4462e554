"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference checkout exists (GIAO_REFERENCE_ROOT, default a
``reference`` directory beside the repository; the same checkout oracle/_ref
is built from):

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py nuclear    # one fixture (boys, m8, blocks, nuclear,
                                                  # derivatives, contraction, cholesky)

Inputs and outputs:

* ``boys.json`` -- the reference's Boys test map (tests/python/
  test_boys_production.py:13-37 arguments x orders 0,3,12,32) and its
  reachable-domain sample (test_boys_reachable_domain.py:7-44, seed 410404),
  with the reference library's F_0..F_32 and 40-digit mpmath values;
* ``primitive_eri_m8.json`` -- the 96 frozen primitive quartets of
  tests/data/eri_recursive_m8.jsonl (zero and finite field) with their
  recorded expected values and the reference library's values;
* ``eri_blocks.npz`` -- reference ``evaluate_eri_shell_quartets`` output for
  the 19-AO atom (all canonical quartets, B=(0,0,0.1)) and a seeded subset of
  the 12-atom molecule's canonical quartets;
* ``nuclear.npz`` -- reference ``compute_nuclear_attraction_matrix`` for a
  seeded three-atom molecule (nuclei at the atoms, charges 1, 2, 3; finite
  field with a shifted gauge origin, and zero field) and for the 19-AO atom
  (Z = 10 at the origin, B = (0, 0, 0.1));
* ``derivatives.npz`` -- reference ``compute_eri_center_derivatives``
  blocks (4, 3, na, nb, nc, nd) for a seeded three-atom molecule (seeded
  canonical and arbitrary quartets, repeated shells) and a hand-made f/g
  system with a two-contraction p shell, at a finite field with a shifted
  gauge origin and at zero field, with the magnetic-derivative blocks
  (3, na, nb, nc, nd) of the same quartets, the mixed field/centre blocks
  (4, 3, 3, na, nb, nc, nd) of a subset, and the reference's derivative
  and ordinary Schwarz factors of every ordered shell pair;
* ``contraction.npz`` -- reference ``contract_eri_derivatives`` (per-atom
  (natom, 3)) over all canonical quartets of the hand-made f/g system and a
  seeded two-atom molecule, with the closed-form densities of
  ``contraction_densities`` (complex and real gamma), zero and finite field;
* ``cholesky.json`` -- the reference's own NumPy Cholesky driver
  (python/giao_integrals/cholesky.py, executed unmodified over the reference
  library's native diagonal/column generators) on the two-shell d/f system of
  tests/python/test_cholesky.py:14-22 and on a small three-atom molecule.

The product never reads these files at run time; tests compare against them.
"""

from __future__ import annotations

import importlib.util
import json
import os
import random
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from giaoint_gb300 import synthetic as syn  # noqa: E402
from oracle import build_ref  # noqa: E402
from oracle import oracle as O  # noqa: E402

# the reference checkout: GIAO_REFERENCE_ROOT, else a "reference" directory beside the repository
REFERENCE = Path(os.environ.get("GIAO_REFERENCE_ROOT", str(ROOT.parent / "reference")))

BOYS_MAP = [0.0, 1.0e-14 + 1.0e-14j, 0.749999, 0.750001, 1.0 + 4.0j, 20.0 - 35.0j, -1.0 + 2.0j, -30.0 - 12.0j,
            -100.0 + 20.0j, 123.999, 124.001, 130.0 + 10.0j, 159.999j, 1000.0 - 25.0j]


def reachable_arguments():
    """The argument construction of the reference's reachable-domain test."""
    g = random.Random(410404)
    out = []
    for _ in range(120):
        ea = 10 ** g.uniform(-1.3, 1.3)
        eb = 10 ** g.uniform(-1.3, 1.3)
        e = ea + eb
        ca = tuple(g.uniform(-2.0, 2.0) for _ in range(3))
        cb = tuple(g.uniform(-2.0, 2.0) for _ in range(3))
        nuc = tuple(g.uniform(-2.0, 2.0) for _ in range(3))
        direction = tuple(g.gauss(0.0, 1.0) for _ in range(3))
        norm = sum(v * v for v in direction) ** 0.5
        mag = g.random()
        field = tuple(mag * v / norm for v in direction)
        sep = tuple(cb[i] - ca[i] for i in range(3))
        q = (0.5 * (field[1] * sep[2] - field[2] * sep[1]), 0.5 * (field[2] * sep[0] - field[0] * sep[2]),
             0.5 * (field[0] * sep[1] - field[1] * sep[0]))
        P = tuple((ea * ca[i] + eb * cb[i]) / e for i in range(3))
        cc = tuple(P[i] - 0.5j * q[i] / e for i in range(3))
        out.append(e * sum((cc[i] - nuc[i]) ** 2 for i in range(3)))
    return out


def boys_fixture(ref):
    import mpmath as mp

    def hyp(n, z):
        with mp.workdps(40):
            zz = mp.mpc(z)
            return complex(mp.hyp1f1(n + mp.mpf("0.5"), n + mp.mpf("1.5"), -zz) / (2 * n + 1))

    cases = []
    for z in BOYS_MAP + reachable_arguments():
        z = complex(z)
        vals, diag = ref.boys(z, 32)
        cases.append({"z": [z.real, z.imag], "region": diag["region"],
                      "reference": [[v.real, v.imag] for v in vals],
                      "mpmath": [[hyp(n, z).real, hyp(n, z).imag] for n in (0, 1, 3, 8, 12, 16, 32)]})
    scaled = []
    for z in (-0.3 + 0.2j, -20.0 + 5.0j, -120.0 - 8.0j, 3.0 - 7.0j):
        vals, _ = ref.boys(z, 16, scaled=True)
        scaled.append({"z": [z.real, z.imag], "reference": [[v.real, v.imag] for v in vals]})
    errors = []
    for z, n in ((10.0 + 500.0j, 4), (160.001j, 4)):
        try:
            ref.boys(z, n)
            raise SystemExit("expected a Boys domain error")
        except O.OracleError as e:
            errors.append({"z": [z.real, z.imag], "order": n, "message": str(e)})
    return {"mpmath_orders": [0, 1, 3, 8, 12, 16, 32], "cases": cases, "scaled": scaled, "errors": errors}


def m8_fixture(ref):
    records = [json.loads(x) for x in (REFERENCE / "tests/data/eri_recursive_m8.jsonl").read_text().splitlines()]
    out = []
    for r in records:
        prims = [(p["exponent"], p["center"], p["angular"], p["coefficient"], p["normalized"])
                 for p in r["primitives"]]
        vals = []
        for fld in ((0.0, 0.0, 0.0), tuple(r["field"])):
            v = ref.primitive_eri(prims, fld, r["gauge"])
            vals.append([v.real, v.imag])
        out.append({"primitives": r["primitives"], "field": r["field"], "gauge": r["gauge"],
                    "expected": r["expected"], "reference": vals})
    return out


def blocks_fixture(ref, orc):
    atom = syn.full_tensor_atom()
    q1 = orc.canonical_quartets(len(atom))
    v1, o1, _ = ref.eri_batch(atom, q1, (0.0, 0.0, 0.1), None, 8)
    mol = syn.random_molecule(2026)
    B = syn.random_field(2026)
    qall = orc.canonical_quartets(len(mol))
    pick = np.random.default_rng(7).choice(len(qall), 400, replace=False)
    q2 = qall[np.sort(pick)]
    v2, o2, _ = ref.eri_batch(mol, q2, B, None, 8)
    # zero-field variant of the same subset
    v3, o3, _ = ref.eri_batch(mol, q2[:120], (0.0, 0.0, 0.0), None, 8)
    np.savez_compressed(HERE / "eri_blocks.npz", atom_quartets=q1, atom_values=v1, atom_offsets=o1,
                        mol_quartets=q2, mol_values=v2, mol_offsets=o2, mol_field=np.asarray(B),
                        mol_zero_values=v3, mol_zero_offsets=o3)


def reference_cholesky_module(ref):
    """Execute the reference's cholesky.py unmodified over the reference library."""

    class Shell:
        def __init__(self, spec):
            self.spec = spec
            self.center = tuple(spec.center)
            self.cartesian_count = spec.ncart
            self.contraction_count = spec.ncontr
            self.primitive_count = spec.nprim
            self.ao_count = spec.nao

    class Basis:
        def __init__(self, specs):
            self.specs = specs
            self.shells = [Shell(s) for s in specs]
            offs, t = [], 0
            for s in specs:
                offs.append(t)
                t += s.nao
            self.ao_offsets = tuple(offs)
            self.ao_count = t

    class MagneticField:
        def __init__(self, B, gauge_origin=(0.0, 0.0, 0.0)):
            self.B = tuple(B)
            self.gauge_origin = tuple(gauge_origin)

    def fb(field):
        return (None, None) if field is None else (field.B, field.gauge_origin)

    native = types.ModuleType("giao_integrals._giao_integrals")
    native.Basis = Basis
    native.MagneticField = MagneticField
    native._cholesky_diagonal = lambda basis, pairs, field=None, threads=None: ref.cholesky_diagonal(
        basis.specs, pairs, *fb(field), threads or 1)
    native._cholesky_columns = lambda basis, pivots, field=None, threads=None: ref.cholesky_columns(
        basis.specs, pivots, *fb(field), threads or 1)
    threads_mod = types.ModuleType("giao_integrals._threads")
    threads_mod.resolve_num_threads = lambda t=None: 1 if t is None else int(t)
    eri_mod = types.ModuleType("giao_integrals.eri")
    eri_mod.eri_schwarz_bounds = lambda basis, field=None: ref.schwarz(basis.specs, *fb(field))
    pkg = types.ModuleType("giao_integrals")
    pkg.__path__ = []
    for name, mod in (("giao_integrals", pkg), ("giao_integrals._giao_integrals", native),
                      ("giao_integrals._threads", threads_mod), ("giao_integrals.eri", eri_mod)):
        sys.modules[name] = mod
    spec = importlib.util.spec_from_file_location("giao_integrals.cholesky",
                                                  REFERENCE / "python/giao_integrals/cholesky.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["giao_integrals.cholesky"] = mod
    spec.loader.exec_module(mod)
    return mod, Basis, MagneticField


def cholesky_fixture(ref):
    mod, Basis, MagneticField = reference_cholesky_module(ref)
    df = [O.ShellSpec((0.2, -0.1, 0.3), 2, [0.8], [[1.0]]), O.ShellSpec((-0.3, 0.4, -0.2), 3, [0.6], [[1.0]])]
    tri = O.as_specs(syn.random_molecule(11, natoms=3, box=4.0))
    # generally contracted shells (two contraction rows each) on two centres:
    # the complex local block rule and the raw-column cache of the reference
    # decide pivots here
    gen = [O.ShellSpec((0.0, 0.0, 0.0), 0, [9.0, 1.6, 0.35], [[0.15, 0.55, 0.45], [-0.1, -0.2, 1.0]]),
           O.ShellSpec((0.0, 0.0, 0.0), 1, [2.2, 0.45], [[0.5, 0.6], [-0.3, 1.0]]),
           O.ShellSpec((1.3, 0.4, -0.6), 0, [5.5, 0.9, 0.2], [[0.2, 0.6, 0.4], [0.05, -0.4, 1.0]]),
           O.ShellSpec((1.3, 0.4, -0.6), 1, [1.4, 0.3], [[0.6, 0.5], [-0.2, 1.0]]),
           O.ShellSpec((1.3, 0.4, -0.6), 2, [0.7], [[1.0]])]
    cases = []
    for name, specs in (("df", df), ("molecule3", tri), ("contracted", gen)):
        for label, B, origin in (("zero", (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
                                 ("field", (0.05, -0.03, 0.2), (0.37, -0.29, 0.43))):
            for tau in (1e-4, 1e-8):
                for pbs in (32, 1):
                    if name == "df" and pbs == 1:
                        continue
                    res = mod.cholesky_eri(Basis(specs), field=MagneticField(B, origin), threshold=tau,
                                           pivot_batch_size=pbs)
                    v = res.vectors
                    cases.append({
                        "system": name, "field_label": label, "B": list(B), "origin": list(origin),
                        "threshold": tau, "pivot_batch_size": pbs, "rank": int(len(res.pivots)),
                        "pivots": res.pivots.tolist(), "max_residual_diagonal": res.max_residual_diagonal,
                        "vector_sum": [float(v.sum().real), float(v.sum().imag)],
                        "vector_abs_sum": float(np.abs(v).sum()),
                        "first_vector": [[x.real, x.imag] for x in v[0].ravel()[:256]],
                    })
    shells = {"df": [s.__dict__ for s in df], "molecule3": [s.__dict__ for s in tri],
              "contracted": [s.__dict__ for s in gen]}
    return {"shells": shells, "cases": cases}


NUCLEAR_FIELD = (0.05, -0.1, 0.12)
NUCLEAR_ORIGIN = (0.3, 0.1, -0.2)


def nuclear_molecule():
    recs = syn.random_molecule(7, natoms=3)
    atoms = []
    for r in recs:
        if r.center not in atoms:
            atoms.append(r.center)
    return recs, [(1.0 + i, c) for i, c in enumerate(atoms)]


def nuclear_fixture(ref):
    recs, nuclei = nuclear_molecule()
    v1 = ref.nuclear(recs, nuclei, NUCLEAR_FIELD, NUCLEAR_ORIGIN)
    v0 = ref.nuclear(recs, nuclei, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    atom = syn.full_tensor_atom()
    va = ref.nuclear(atom, [(10.0, (0.0, 0.0, 0.0))], (0.0, 0.0, 0.1), (0.0, 0.0, 0.0))
    np.savez_compressed(HERE / "nuclear.npz", mol_field=v1, mol_zero=v0, atom=va,
                        charges=np.asarray([z for z, _ in nuclei]),
                        centers=np.asarray([c for _, c in nuclei]))


DERIV_FIELD = (0.07, -0.04, 0.15)
DERIV_ORIGIN = (0.2, -0.35, 0.1)


def derivative_cases():
    """Systems and quartet lists of the centre-derivative fixture: a seeded
    three-atom molecule (seeded canonical and non-canonical quartets, plus
    every slot repeating one shell), and a hand-made f/g system with a
    two-contraction p shell."""
    mol = O.as_specs(syn.random_molecule(5, natoms=3, box=4.0))
    ns = len(mol)
    rng = random.Random(20261203)
    canon = [tuple(int(x) for x in q) for q in O.Oracle().canonical_quartets(ns)]
    quartets = rng.sample(canon, min(24, len(canon)))
    quartets += [tuple(rng.randrange(ns) for _ in range(4)) for _ in range(6)]
    quartets += [(s, s, s, s) for s in range(0, ns, max(1, ns // 3))]
    hand = [O.ShellSpec((0.1, -0.2, 0.3), 3, [0.9, 0.35], [[0.6, 0.5]]),
            O.ShellSpec((-0.4, 0.5, 0.0), 4, [0.7], [[1.0]]),
            O.ShellSpec((0.6, 0.2, -0.5), 1, [1.3, 0.4], [[0.5, 0.6], [0.3, -0.8]]),
            O.ShellSpec((0.0, 0.0, 0.9), 0, [2.0, 0.5], [[0.4, 0.7]])]
    hq = [(1, 3, 3, 3), (0, 3, 1, 3), (2, 0, 3, 3), (3, 3, 3, 3), (2, 3, 2, 3), (3, 2, 0, 3)]
    return {"molecule3": (mol, quartets), "hand": (hand, hq)}


# quartets (indices into each system's list) of the mixed field/centre
# derivative fixture: (4, 3, 3, ...) blocks are 36 components per element
MIXED_SUBSET = {"molecule3": [0, 1, 2, 3, 30], "hand": [0, 3, 4]}


def derivative_fixture(ref):
    out = {}
    for name, (specs, quartets) in derivative_cases().items():
        q = np.asarray(quartets, dtype=np.uint32)
        out[f"{name}_quartets"] = q
        out[f"{name}_shells"] = np.asarray(json.dumps([s.__dict__ for s in specs]))
        for label, B, origin in (("field", DERIV_FIELD, DERIV_ORIGIN), ("zero", (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))):
            vals, offsets = ref.eri_center_derivatives(specs, q, B, origin)
            out[f"{name}_{label}"] = vals
            out[f"{name}_magnetic_{label}"] = ref.eri_magnetic_derivatives(specs, q, B, origin)[0]
            mq = q[MIXED_SUBSET[name]]
            out[f"{name}_mixed_quartets"] = mq
            out[f"{name}_mixed_{label}"] = ref.eri_mixed_derivatives(specs, mq, B, origin)[0]
            out[f"{name}_bounds_{label}"] = ref.eri_derivative_bounds(specs, B, origin)
            out[f"{name}_schwarz_{label}"] = ref.schwarz(specs, B, origin)
            out[f"{name}_offsets"] = offsets
    out["field"] = np.asarray(DERIV_FIELD)
    out["origin"] = np.asarray(DERIV_ORIGIN)
    np.savez_compressed(HERE / "derivatives.npz", **out)


def contraction_densities(n: int, complex_gamma: bool):
    """Closed-form (reproducible anywhere) Coulomb pair, two exchange pairs
    and a two-particle density of an n-AO system."""
    i = np.arange(n)[:, None]
    j = np.arange(n)[None, :]
    mats = [np.cos(0.3 * i + 0.7 * j + t) + 1j * np.sin(0.5 * i - 0.2 * j + 2 * t) for t in range(6)]
    coulomb = [(mats[0], mats[1])]
    exchange = [(mats[2], mats[3]), (mats[4], mats[5])]
    a, b, c, d = np.meshgrid(*(np.arange(n),) * 4, indexing="ij")
    gamma = 0.1 * np.sin(a + 2.0 * b + 3.0 * c + 5.0 * d)
    if complex_gamma:
        gamma = gamma + 0.1j * np.cos(7.0 * a - b + c - 2.0 * d)
    return coulomb, exchange, np.ascontiguousarray(gamma)


def contraction_cases():
    """(name, shell specs, shell atoms, natom, complex gamma) of the
    contraction fixture."""
    hand = derivative_cases()["hand"][0]
    small = O.as_specs(syn.random_molecule(9, natoms=2, box=3.0))
    cen = []
    small_atoms = []
    for s in small:
        if s.center not in cen:
            cen.append(s.center)
        small_atoms.append(cen.index(s.center))
    return [("hand", hand, [0, 1, 0, 2], 3, True), ("small", small, small_atoms, len(cen), False)]


def contraction_fixture(ref, orc):
    out = {}
    for name, specs, atoms, natom, cg in contraction_cases():
        n = sum(s.nao for s in specs)
        coulomb, exchange, gamma = contraction_densities(n, cg)
        q = orc.canonical_quartets(len(specs))
        for label, B, origin in (("field", DERIV_FIELD, DERIV_ORIGIN), ("zero", (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))):
            vals, offsets = ref.eri_center_derivatives(specs, q, B, origin)
            out[f"{name}_{label}"] = ref.contract_eri_derivatives(specs, atoms, natom, q, offsets, vals, coulomb,
                                                                  exchange, gamma)
    np.savez_compressed(HERE / "contraction.npz", **out)


def main():
    if build_ref.build() is None:
        raise SystemExit("the reference checkout is required to generate fixtures")
    ref = O.Reference()
    orc = O.Oracle()
    only = set(sys.argv[1:])
    if not only or "boys" in only:
        (HERE / "boys.json").write_text(json.dumps(boys_fixture(ref)))
    if not only or "m8" in only:
        (HERE / "primitive_eri_m8.json").write_text(json.dumps(m8_fixture(ref)))
    if not only or "blocks" in only:
        blocks_fixture(ref, orc)
    if not only or "nuclear" in only:
        nuclear_fixture(ref)
    if not only or "derivatives" in only:
        derivative_fixture(ref)
    if not only or "contraction" in only:
        contraction_fixture(ref, orc)
    if not only or "cholesky" in only:
        (HERE / "cholesky.json").write_text(json.dumps(cholesky_fixture(ref)))
    for p in sorted(HERE.iterdir()):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
