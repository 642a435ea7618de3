"""Build recipe for oracle/_ref/ (test infrastructure only):

  libref_correlator.so  the reference's own multi-tau correlator, compiled from
                        SOURCE/gpu_water3D.cu and SOURCE/mersenne_inline.cu where they lie in the
                        reference checkout (main renamed, nothing else changed), linked with
                        oracle/ref_correlator.cpp, which calls its initialize / add / evaluate;
  AlphaPderivate, CPderivate, KTderivate
                        the reference's finite-difference programs of
                        CVF_ThermodynamicAnalysis/*.c, compiled as they are with gcc (tools()).

Run where the reference checkout exists: its path is the argument, else the environment variable
CVF_REFERENCE_DIR (__graft_entry__.build() passes it). Without a checkout every call returns what
an earlier build left in oracle/_ref/ (None or {} where nothing was built, as on the GPU machine), and
the tests that need these builds skip. Nothing from the reference is copied into the repository;
the output stays in the git-ignored oracle/_ref/.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def checkout(ref: str | None = None) -> str | None:
    """The reference checkout to build from (the argument, else CVF_REFERENCE_DIR), or None."""
    for cand in (ref, os.environ.get("CVF_REFERENCE_DIR")):
        if cand and os.path.isdir(os.path.join(cand, "SOURCE")):
            return cand
    return None
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_correlator.so")


def build(ref: str | None = None, force: bool = False):
    ref = checkout(ref)
    if ref is None:
        return LIB if os.path.exists(LIB) else None
    src = os.path.join(ref, "SOURCE", "gpu_water3D.cu")
    if not os.path.exists(src):
        return None
    harness = os.path.join(HERE, "ref_correlator.cpp")
    newest = max(os.path.getmtime(harness), os.path.getmtime(os.path.abspath(__file__)))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    os.makedirs(OUT, exist_ok=True)
    objs = []
    for name in ("gpu_water3D.cu", "mersenne_inline.cu"):  # the reference's own two sources
        obj = os.path.join(OUT, name + ".o")
        subprocess.run(["nvcc", "-c", "-w", "-Xcompiler", "-fPIC", "-Dmain=cvf_reference_main",
                        "-gencode", "arch=compute_103a,code=sm_103a", "-o", obj,
                        os.path.join(ref, "SOURCE", name)], check=True)
        objs.append(obj)
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run(["nvcc", "-shared", "-Xcompiler", "-fPIC", "-o", tmp, harness] + objs + ["-cudart", "static", "-lm"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


TOOLS = ("AlphaPderivate", "CPderivate", "KTderivate")


def tools(ref: str | None = None):
    """{name: path} of the three analysis programs, built from the reference's own .c files with
    gcc -O2 (empty where the checkout is absent)."""
    ref = checkout(ref)
    if ref is None:
        built = {name: os.path.join(OUT, name) for name in TOOLS}
        return built if all(os.path.exists(p) for p in built.values()) else {}
    src_dir = os.path.join(ref, "CVF_ThermodynamicAnalysis")
    out = {}
    for name in TOOLS:
        src = os.path.join(src_dir, name + ".c")
        if not os.path.exists(src):
            return {}
        exe = os.path.join(OUT, name)
        if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
            os.makedirs(OUT, exist_ok=True)
            tmp = exe + f".tmp{os.getpid()}"
            subprocess.run(["gcc", "-O2", "-w", "-o", tmp, src, "-lm"], check=True)
            os.replace(tmp, exe)
        out[name] = exe
    return out


if __name__ == "__main__":
    print(build(*(sys.argv[1:2])))
    print(tools(*(sys.argv[1:2])))
