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


class Histogram2D:
    """Binned (E, rho) histogram reweighting of the reference's F90 reweighting program on the GPU
    (cvf_h2d_*): h = H/N and rho = N/V per sample (internal units), the run of each sample and
    the runs' internal (T, P)."""

    def __init__(self, h, rho, run_of, That, Phat, L, bin_factor=1.0, steps=300, device=0):
        h, rho = (np.ascontiguousarray(a, dtype=np.float64) for a in (h, rho))
        run_of = np.ascontiguousarray(run_of, dtype=np.int32)
        That, Phat = (np.ascontiguousarray(a, dtype=np.float64) for a in (That, Phat))
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        self._h = C.c_void_p()
        self.n_runs = len(That)
        check(lib().cvf_h2d_create(device, ptr(h), ptr(rho), ptr(run_of), len(h), ptr(That), ptr(Phat),
                                   self.n_runs, int(L), float(bin_factor), int(steps), C.byref(self._h)))
        nb, nbm = C.c_int(), C.c_int()
        e0, de, d0, dd = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        self.ctes = np.zeros(self.n_runs)
        check(lib().cvf_h2d_info(self._h, C.byref(nb), C.byref(nbm), C.byref(e0), C.byref(de), C.byref(d0),
                                 C.byref(dd), ptr(self.ctes)))
        self.n_bin2d, self.n_bin_mixed = nb.value, nbm.value
        self.Emin, self.dE, self.Dmin, self.dD = e0.value, de.value, d0.value, dd.value

    def reweight(self, T_hat, P_hat, grid=True):
        g = np.zeros((self.n_bin2d, self.n_bin2d)) if grid else None
        be, br = C.c_double(), C.c_double()
        check(lib().cvf_h2d_reweight(self._h, float(T_hat), float(P_hat),
                                     g.ctypes.data_as(C.c_void_p) if grid else None, C.byref(be), C.byref(br)))
        return g, be.value, br.value

    def mixed(self, alpha):
        x, q = np.zeros(self.n_bin_mixed), np.zeros(self.n_bin_mixed)
        b = C.c_double()
        check(lib().cvf_h2d_mixed(self._h, float(alpha), x.ctypes.data_as(C.c_void_p), q.ctypes.data_as(C.c_void_p),
                                  C.byref(b)))
        return x, q, b.value

    def close(self):
        if getattr(self, "_h", None):
            lib().cvf_h2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
