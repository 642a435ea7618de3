"""Build recipe for the CPU oracle (test infrastructure only).

``build()`` compiles ``oracle/cvf_oracle.c`` into ``oracle/_build/libcvf_oracle.so`` with gcc,
OpenMP and ``-ffp-contract=off`` (the FP64 volume move must round exactly as on the GPU).
The library is loaded only by tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg, as the checker or as the timed CPU baseline.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libcvf_oracle.so")
SRC = [os.path.join(HERE, "cvf_oracle.c")]
HDR = [os.path.join(HERE, "cvf_oracle.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SRC + HDR)


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or _stale():
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-Wall", "-Wno-unused-function", "-o", tmp] + SRC + ["-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
