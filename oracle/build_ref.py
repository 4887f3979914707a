"""Compiles the reference's own Day Phase kernels into oracle/_ref/ (test infrastructure).

genesis-compute/src/cuda/physics.cu is self-contained (its __constant__ LUT is
defined in the same file), so nvcc builds it from the source where it lies
into a device-only cubin for sm_103a.  The tests load it with the CUDA driver
API and launch the reference kernels in the order of cu_step_day_phase
(physics.cu:441-495) to check the oracle against the reference itself on the
GPU.  Nothing is copied: the source is read in place, only the cubin is
written, and oracle/_ref/ is not committed.

Where the reference lies: the `root` argument, else the environment variable
AXC_REFERENCE_ROOT, else a checkout named `reference` beside this repository's
directory.  Without the sources the build is a no-op (an existing cubin is
kept).

    python oracle/build_ref.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "physics_ref.cubin"
REL = Path("genesis-compute") / "src" / "cuda" / "physics.cu"
NVCC = str(Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc")


def reference_root(root: str | os.PathLike | None = None) -> Path:
    if root:
        return Path(root)
    env = os.environ.get("AXC_REFERENCE_ROOT")
    if env:
        return Path(env)
    return HERE.parents[1] / "reference"


def build(root: str | os.PathLike | None = None) -> Path | None:
    """Builds the cubin when the reference sources are present; returns its path or None."""
    src = reference_root(root) / REL
    if not src.exists():
        return OUT if OUT.exists() else None
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= src.stat().st_mtime:
        return OUT
    cmd = [NVCC, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", str(src), "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference cubin build failed: {' '.join(cmd)}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
    sys.exit(0)
