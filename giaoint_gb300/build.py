"""Build the in-tree CUDA library ``giaoint_gb300/_build/libgiao_gb300.so``.

Each ``csrc/*.cu`` translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked into
one shared library exporting the C ABI of ``include/giao_gb300.h``.  The
build is incremental: a unit is recompiled only when it or a header is newer
than its object file.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libgiao_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "giao_gb300.h"]


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library; return its path."""
    BUILD.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    newest_header = max(p.stat().st_mtime for p in _headers())
    flags = ["-std=c++20", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-fopenmp", "-I", str(ROOT / "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]
    compiler = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        if (not force and obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime
                and obj.stat().st_mtime >= newest_header):
            return obj
        tmp = obj.with_suffix(f".{os.getpid()}.o")
        subprocess.run([compiler, *flags, "-c", str(src), "-o", str(tmp)], check=True)
        os.replace(tmp, obj)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(sources))) as pool:
        objs = list(pool.map(compile_one, sources))
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(f".{os.getpid()}.so")
        subprocess.run([compiler, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart", "-lgomp"], check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
