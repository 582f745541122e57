"""Build the CPU oracle (plain C, FP64) into oracle/_build/liboracle.so.

    python oracle/build.py

No fused multiply-add (-ffp-contract=off): the oracle reproduces the reference's serial
FP64 arithmetic operation for operation, and gcc on aarch64 would otherwise contract
a*b + c into one rounding. Host-portable: no -march flags, builds on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "oracle.c")]
HDR = [os.path.join(HERE, "oracle.h")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRC + HDR + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-o", tmp] + SRC + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
