"""Compile the reference's hot-path C++ sources in place into oracle/_ref.

Test infrastructure only.  The reference's electron-repulsion path builds from
nine of its own source files (src/types.cpp, overlap.cpp, hermite.cpp, boys.cpp,
eri.cpp, cholesky.cpp, nuclear.cpp, derivatives.cpp, property.cpp) with no generated headers and no external libraries, so
this recipe runs g++ on them directly (no CMake) together with
oracle/ref_shim.cpp, and writes only into oracle/_ref/.  It needs the
reference checkout, which exists only where fixtures are generated; the
resulting library is never shipped or imported by the product.
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference checkout: GIAO_REFERENCE_ROOT, else a "reference" directory beside the repository
REFERENCE = Path(os.environ.get("GIAO_REFERENCE_ROOT", str(HERE.parent.parent / "reference")))
SOURCES = ["types.cpp", "overlap.cpp", "hermite.cpp", "boys.cpp", "eri.cpp", "cholesky.cpp", "nuclear.cpp",
           "derivatives.cpp", "property.cpp", "assembly.cpp"]
FLAGS = ["-std=c++20", "-O3", "-fPIC", "-fopenmp", "-DGIAO_HAS_OPENMP"]


def available() -> bool:
    return all((REFERENCE / "src" / s).is_file() for s in SOURCES)


def build(force: bool = False) -> Path | None:
    """Build oracle/_ref/libgiaoref.so; return its path, or None without the reference."""
    if not available():
        return None
    lib = OUT / "libgiaoref.so"
    inputs = [REFERENCE / "src" / s for s in SOURCES] + [HERE / "ref_shim.cpp"]
    if lib.exists() and not force and all(lib.stat().st_mtime >= p.stat().st_mtime for p in inputs):
        return lib
    OUT.mkdir(exist_ok=True)
    includes = ["-I", str(REFERENCE / "include"), "-I", str(REFERENCE / "src")]

    def compile_one(src: Path) -> Path:
        obj = OUT / (src.stem + ".o")
        subprocess.run(["g++", *FLAGS, *includes, "-c", str(src), "-o", str(obj)], check=True)
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        objs = list(pool.map(compile_one, inputs))
    subprocess.run(["g++", "-shared", "-fopenmp", "-o", str(lib), *map(str, objs)], check=True)
    for o in objs:
        o.unlink()
    return lib


if __name__ == "__main__":
    path = build(force="--force" in sys.argv)
    print(path if path else "reference sources not present; nothing built")
