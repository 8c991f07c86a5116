"""Build the sm_103a CUDA library ``libloki_gb300.so`` in-tree.

``python -m pyloki_gb300.build`` compiles every ``csrc/*.cu`` translation unit
in parallel with nvcc (one ``-gencode`` for sm_103a) and links the shared
library next to this file. ``--fmad=false`` (device) and ``-ffp-contract=off`` (host) keep numpy's
rounding (no contracted multiply-adds), which the bit-exact kernels rely on.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libloki_gb300.so"

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "--fmad=false", "--expt-relaxed-constexpr",
    "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "-Xcompiler", "-ffp-contract=off",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        msg = "nvcc not found: the CUDA toolkit is required to build libloki_gb300"
        raise RuntimeError(msg)
    return cand


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if needed) and return the path of ``libloki_gb300.so``."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((PKG.parent / "include").glob("*.h"))
    objs = [BUILD / (s.stem + ".o") for s in sources]

    def compile_one(src: Path, obj: Path) -> None:
        if not force and not _stale(obj, [src, *headers]):
            return
        cmd = [nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(compile_one, sources, objs))
    if force or _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a",
               *map(str, objs), "-o", str(LIB) + ".tmp", "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
