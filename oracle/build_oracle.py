"""Build the oracle's C restatement (test infrastructure, never shipped).

gcc -O3 -fopenmp on oracle/cpu_baseline.c -> oracle/libpgx_cpu_oracle.so.
No -march flags: the same source builds on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "cpu_baseline.c"
LIB = HERE / "libpgx_cpu_oracle.so"


def build(force: bool = False) -> Path:
    deps = [SRC, ROOT / "include" / "pgx.h"]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-fcx-limited-range",
           f"-I{ROOT / 'include'}", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
