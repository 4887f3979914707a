"""Builds the CPU oracle ``oracle/_build/liboracle.so`` (test infrastructure).

Plain gcc, OpenMP, no host-specific flags, so the same recipe builds the same
arithmetic on x86-64 and on aarch64 hosts.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "day_phase_oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"
HEADER = HERE.parent / "include" / "axicor_day.h"


def build() -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, HEADER.stat().st_mtime,
                                                    Path(__file__).stat().st_mtime):
        return LIB
    cc = shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fwrapv", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build())
    sys.exit(0)
