"""Builds the engine library and the drop-in driver in-tree for sm_103a.

Outputs (git-ignored):
  cvfbulkwater_gb300/_build/libcvf_gb300.so   C-ABI of include/cvf.h
  cvfbulkwater_gb300/_build/gpu_water3D       drop-in replacement of SOURCE/gpu_water3D

CUDA sources are compiled with ``-gencode arch=compute_103a,code=sm_103a``; host sources with
``-ffp-contract=off`` so that acceptance tables and FP64 observables round like the CPU oracle.
Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcvf_gb300.so")
EXE = os.path.join(BUILD, "gpu_water3D")

CU = ["cvf_mc.cu", "cvf_sw.cu", "cvf_reweight.cu", "cvf_noalloc.cu", "cvf_config.cu", "cvf_stats.cu", "cvf_corr.cu", "cvf_hist2d.cu", "cvf_nhb.cu"]
CPP = ["cvf_engine.cpp", "cvf_host.cpp", "cvf_io.cpp", "cvf_isobar.cpp"]
DRIVER = ["gpu_water3D.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "cvf.h"))
    return files


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in _deps())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library (and driver) if any source is newer; return the library path."""
    if not force and not _stale(LIB) and not (DRIVER and _stale(EXE)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cuda = _cuda_home()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    nvcc = os.path.join(cuda, "bin", "nvcc") if os.path.exists(os.path.join(cuda, "bin", "nvcc")) else "nvcc"
    jobs = []
    for f in CU:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [nvcc, "-c", os.path.join(CSRC, f), "-o", obj, "-O3", "-lineinfo", "-std=c++17",
               "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off"] + ARCH + inc
        if verbose:
            cmd += ["-Xptxas", "-v"]
        cmd += os.environ.get("CVF_NVCC_EXTRA", "").split()  # tuning experiments only
        jobs.append((obj, cmd))
    for f in CPP + DRIVER:
        obj = os.path.join(BUILD, f + ".o")
        cmd = ["g++", "-c", os.path.join(CSRC, f), "-o", obj, "-O2", "-std=c++17", "-fPIC",
               "-ffp-contract=off", "-Wall", "-I" + os.path.join(cuda, "include")] + inc
        jobs.append((obj, cmd))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(lambda j: _run(j[1]), jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    lib_objs = [os.path.join(BUILD, f + ".o") for f in CU + CPP]
    tmp = LIB + f".tmp{os.getpid()}"
    _run([nvcc, "-shared", "-o", tmp] + lib_objs + ARCH + ["-cudart", "static", "-Xlinker", "-z,defs", "-lpthread"])
    os.replace(tmp, LIB)
    if DRIVER:
        drv_objs = [os.path.join(BUILD, f + ".o") for f in DRIVER]
        tmpe = EXE + f".tmp{os.getpid()}"
        _run(["g++", "-o", tmpe] + drv_objs + ["-L" + BUILD, "-lcvf_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
        os.replace(tmpe, EXE)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
