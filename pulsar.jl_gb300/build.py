"""Build libpulsar_gb300.so (sm_103a) in-tree with nvcc.

Translation units compile in parallel into ``_build/`` at the repository root
and link into ``pulsar.jl_gb300/libpulsar_gb300.so``.  One ``-gencode``
(compute_103a -> sm_103a), no cmake.
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
INCLUDE = ROOT / "include"
BUILD = ROOT / "_build"
LIB = PKG / "libpulsar_gb300.so"

SOURCES = ["pgx_kernels.cu", "pgx_mixed.cu", "pgx_runtime.cu", "pgx_optimize.cu", "pgx_batch.cu",
           "pgx_noalloc.cu", "pgx_server.cu", "pgx_stack.cu", "pgx_lbfgs.cu", "pgx_penalty.cu", "pgx_tc.cu",
           "pgx_checkpoint.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpulsar_gb300.so")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def _deps():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")) + list(CSRC.glob("*.cuh")) +
                  list(CSRC.glob("*.h")) +
                  list(INCLUDE.glob("*.h")))


def build(force: bool = False, verbose: bool = False) -> Path:
    deps = _deps()
    if not force and _newer(LIB, deps):
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run([cc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", str(tmp),
                        *map(str, objs)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
