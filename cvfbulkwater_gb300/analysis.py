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


def cp_derivative(T, H, H2, n):
    """CPderivate.c: arrays of one isobar (any order) -> (T, C_P, error) for the sorted points
    2 .. m-3."""
    T, H, H2 = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, H, H2))
    n = np.ascontiguousarray(n, dtype=np.int64)
    m = len(T)
    outs = [np.zeros(max(m, 1)) for _ in range(3)]
    k = C.c_int()
    check(lib().cvf_cp_derivative(_ptr(T), _ptr(H), _ptr(H2), _ptr(n), m, _ptr(outs[0]), _ptr(outs[1]),
                                  _ptr(outs[2]), C.byref(k)))
    return tuple(o[: k.value] for o in outs)


KT_NOT_VALUE = -10.0


def kt_derivative(T, P, rho, Erho):
    """KTderivate.c: points (T in K, P in MPa, rho and its error in kg/m^3, any order) ->
    (K_T, error) per point in MPa^-1, KT_NOT_VALUE where the reference gives none."""
    T, P, rho, Erho = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, P, rho, Erho))
    m = len(T)
    kt, ekt = np.zeros(max(m, 1)), np.zeros(max(m, 1))
    check(lib().cvf_kt_derivative(_ptr(T), _ptr(P), _ptr(rho), _ptr(Erho), m, _ptr(kt), _ptr(ekt)))
    return kt[:m], ekt[:m]


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def f90_range(start, stop, step, inclusive=True):
    """The values a Fortran `do while (v <= stop)` (or `< stop`) loop with `v = v + step` visits,
    accumulated as the F90's search does (F90:732-891)."""
    out, v = [], float(start)
    while (v <= stop) if inclusive else (v < stop):
        out.append(v)
        v = v + step
    return np.array(out)


def ising_compare(x, q, B=1.0):
    """ConfrontIsing, ZeroTest and HeightTest of the F90 on a mixed distribution (cvf_h2d_ising):
    dict of liu_2D, liu_3D, kl_2D, kl_3D, zero, height."""
    x, q = (np.ascontiguousarray(v, dtype=np.float64) for v in (x, q))
    out = np.zeros(6)
    check(lib().cvf_h2d_ising(_ptr(x), _ptr(q), len(x), float(B), _ptr(out)))
    return dict(zip(("liu_2D", "liu_3D", "kl_2D", "kl_3D", "zero", "height"), out.tolist()))


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

    def mixed_batch(self, alphas):
        """x, q (n x n_bin_mixed) and the Binder cumulants of n angles, binned in one pass."""
        a = np.ascontiguousarray(alphas, dtype=np.float64).ravel()
        x, q, b = np.zeros((len(a), self.n_bin_mixed)), np.zeros((len(a), self.n_bin_mixed)), np.zeros(len(a))
        check(lib().cvf_h2d_mixed_batch(self._h, _ptr(a), len(a), _ptr(x), _ptr(q), _ptr(b)))
        return x, q, b

    def set_constants(self, ctes):
        """The runs' constants as given (the F90's Constants_L file) instead of iterated."""
        c = np.ascontiguousarray(ctes, dtype=np.float64)
        if c.shape != (self.n_runs,):
            raise ValueError("one constant per run")
        check(lib().cvf_h2d_set_constants(self._h, _ptr(c)))
        self.ctes = c.copy()

    def scan(self, T_hats, P_hats, S_list, B=1.0):
        """The F90's search over pressures (outer), temperatures and angles (inner), internal
        units: (tp_rows [n_P, n_T, 2] = binder_e, binder_rho; rows [n_P, n_T, n_S, 7] = binder_m,
        liu_2D, liu_3D, kl_2D, kl_3D, zero, height; best: dict of the (P, T, S) indices of the
        smallest liu_2D, liu_3D, zero, height and zero + height, None where none)."""
        T, P, S = (np.ascontiguousarray(v, dtype=np.float64).ravel() for v in (T_hats, P_hats, S_list))
        tp = np.zeros((len(P), len(T), 2))
        rows = np.zeros((len(P), len(T), len(S), 7))
        best = np.zeros(5, dtype=np.int64)
        check(lib().cvf_h2d_scan(self._h, _ptr(T), len(T), _ptr(P), len(P), _ptr(S), len(S), float(B), _ptr(tp),
                                 _ptr(rows), _ptr(best)))
        names = ("liu_2D", "liu_3D", "zero", "height", "zero_height")
        return tp, rows, {k: (None if r < 0 else np.unravel_index(int(r), (len(P), len(T), len(S))))
                          for k, r in zip(names, best)}

    def close(self):
        if getattr(self, "_h", None):
            lib().cvf_h2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
