"""Build the native library libamfls_gb300.so in-tree (sm_103a only).

    python -m amfls_solver_gb300.build          # or amfls_solver_gb300.build.build()

Each CUDA translation unit in csrc/ is compiled by its own nvcc process in
parallel, then linked into amfls_solver_gb300/_build/libamfls_gb300.so.  The
build is skipped when the library is newer than every source and header.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libamfls_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-diag-suppress", "177"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")
    return cand


def _sources():
    return sorted(SRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(SRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()

    def compile_one(src: Path) -> Path:
        obj = OUT / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-I", str(SRC), "-I", str(INCLUDE), "-c", str(src), "-o",
               str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=workers) as pool:
        objs = list(pool.map(compile_one, srcs))
    tmp = OUT / "libamfls_gb300.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
