"""Build libd2f.so (the CUDA step kernels behind the C ABI of include/d2f.h) in-tree.

    python -m diff_2d_fem_gb300.build

One translation unit, one -gencode (sm_103a), no CMake. The library lands in
diff_2d_fem_gb300/_build/libd2f.so and is rebuilt when a source is newer than it.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libd2f.so")
SOURCES = [os.path.join(HERE, "csrc", "pncg_step.cu")]
DEPS = SOURCES + [os.path.join(HERE, "csrc", "d2f_math.cuh"), os.path.join(ROOT, "include", "d2f.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in DEPS + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-lineinfo",
           "--use_fast_math" if os.environ.get("D2F_FAST_MATH") else "-ftz=false",
           "-I", os.path.join(ROOT, "include")] + ARCH + ["-o", tmp] + SOURCES
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
