"""Isobar analysis of the reference's CVF_ThermodynamicAnalysis/ scripts on the engine's results.

  Lattice.run_statistics()   the awk stage of script_analisi.sh:35, on the GPU from the on-device
                             sample stream (one row per replica)
  isobar_point(stats)        calculadora.sh:41-61: per-cell means and errors, density, C_P, K_T
  to_si(point, P)            conversor.sh: SI units
  alpha_p_derivative(...)    AlphaPderivate.c: alpha_P by finite differences along an isobar

The host steps run in the engine library (cvf_isobar.cpp) through its C ABI.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check, lib


def _as_dict(st, names):
    return {n: getattr(st, n) for n in names}


def stats_struct(d) -> abi.RunStats:
    s = abi.RunStats()
    s.L, s.P, s.T, s.n = int(d["L"]), float(d["P"]), float(d["T"]), int(d["n"])
    for k in range(6):
        s.mean[k] = float(d["mean"][k])
        s.var[k] = float(d["var"][k])
    return s


def isobar_point(stats) -> dict:
    """stats: a row of Lattice.run_statistics() (dict) -> per-cell isobar point (dict)."""
    p = abi.IsobarPoint()
    check(lib().cvf_isobar_point_from_stats(C.byref(stats_struct(stats)), C.byref(p)))
    return _as_dict(p, abi._POINT)


def to_si(point: dict, P: float) -> dict:
    p = abi.IsobarPoint(*[float(point[n]) for n in abi._POINT])
    o = abi.IsobarPointSI()
    check(lib().cvf_isobar_point_to_si(C.byref(p), float(P), C.byref(o)))
    return _as_dict(o, abi._POINT_SI)


def alpha_p_derivative(T, V, V2, n):
    """Arrays of one isobar (any order) -> (T, alpha_P, error) for the sorted points 2 .. m-3."""
    T, V, V2 = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, V, V2))
    n = np.ascontiguousarray(n, dtype=np.int64)
    m = len(T)
    outs = [np.zeros(max(m, 1)) for _ in range(3)]
    k = C.c_int()
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(lib().cvf_alpha_p_derivative(ptr(T), ptr(V), ptr(V2), ptr(n), m, ptr(outs[0]), ptr(outs[1]),
                                       ptr(outs[2]), C.byref(k)))
    return tuple(o[: k.value] for o in outs)
