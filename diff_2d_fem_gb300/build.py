"""Build libd2f.so (the CUDA step kernels behind the C ABI of include/d2f.h) in-tree.

    python -m diff_2d_fem_gb300.build

Seven translation units (FP64 step kernels, mixed step kernels with every term, mixed step kernels with
reduced feature sets, mixed cluster kernels, C ABI, adjoint kernels, read-out kernels) compiled in parallel, one
-gencode (sm_103a), no CMake. The library lands in
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
CSRC = os.path.join(HERE, "csrc")
SOURCES = [os.path.join(CSRC, f) for f in ("pncg_fp64.cu", "pncg_mixed.cu", "pncg_mixed_feat.cu", "pncg_mixed_cluster.cu",
                                               "d2f_capi.cu", "adjoint.cu", "readouts.cu")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("pncg_kernel.cuh", "pncg_mixed_kernel.cuh", "d2f_math.cuh", "d2f_solver.h")] + [
                  os.path.join(ROOT, "include", "d2f.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the translation units in parallel, link libd2f.so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in DEPS + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tag = f"{os.getpid()}"
    flags = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", "-I", os.path.join(ROOT, "include")] + ARCH
    if verbose:
        flags.append("-Xptxas=-v")
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.basename(src) + f".{tag}.o")
        objs.append(obj)
        procs.append(subprocess.Popen([nvcc(), "-c"] + flags + ["-o", obj, src]))
    rcs = [p.wait() for p in procs]
    if any(rcs):
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
        raise RuntimeError(f"nvcc failed ({rcs})")
    tmp = LIB + f".tmp{tag}"
    subprocess.run([nvcc(), "-shared"] + ARCH + ["-o", tmp] + objs, check=True)
    for o in objs:
        os.remove(o)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
