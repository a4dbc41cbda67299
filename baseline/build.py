"""Build of the comparison-only library baseline/_lib/libref_thrust.so
(thrust_sort.cu: the reference's GPU local sort, thrust::sort / CUB radix
sort) for sm_103a. bench.py times it beside the engine; nothing in the
engine links or loads it."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "thrust_sort.cu"
LIB = HERE / "_lib" / "libref_thrust.so"


def build() -> Path:
    """Compile the library if it is missing or older than its source."""
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "-Xcompiler", "-fPIC", "-shared", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB
