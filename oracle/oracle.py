"""ctypes wrapper around the CPU oracle (test infrastructure only; see cvf_oracle.h).

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as the checker
or as the timed CPU baseline, never by the GPU product.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class Obs(C.Structure):
    _fields_ = [("n_hb2", C.c_int64), ("n_sigma", C.c_int64), ("r_cell", C.c_double),
                ("volume", C.c_double), ("e_vdw", C.c_double), ("n_hb", C.c_double),
                ("energy", C.c_double), ("enthalpy", C.c_double), ("v_total", C.c_double),
                ("m", C.c_double)]


class CStats(C.Structure):
    _fields_ = [("largest", C.c_int64), ("second", C.c_int64), ("n_percolating", C.c_int64),
                ("n_clusters", C.c_int64), ("sum_size", C.c_int64), ("sum_size2", C.c_int64),
                ("sum_size2_wrap32", C.c_int64)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.oracle_create.restype = P
        L.oracle_create.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int64, C.c_float, C.c_uint32, C.c_int]
        L.oracle_create_mode.restype = P
        L.oracle_create_mode.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int64, C.c_float, C.c_uint32, C.c_int,
                                         C.c_int]
        L.oracle_get_nhb.argtypes = [P, P]
        L.oracle_destroy.argtypes = [P]
        L.oracle_set_threads.argtypes = [P, C.c_int]
        L.oracle_set_config.argtypes = [P, P, C.c_int64]
        L.oracle_get_config.argtypes = [P, P, C.c_int64]
        L.oracle_get_cubes.argtypes = [P, P, P]
        for f in ("oracle_cube_move", "oracle_volume_move", "oracle_sweep", "oracle_sw_step", "oracle_wolff_step"):
            getattr(L, f).argtypes = [P]
        L.oracle_step.argtypes = [P, C.c_int, C.c_int]
        L.oracle_set_wolff.argtypes = [P, C.c_int]
        L.oracle_wolff_stats.argtypes = [P, P]
        L.oracle_measure.argtypes = [P, C.POINTER(Obs)]
        L.oracle_cluster_stats.argtypes = [P, C.POINTER(CStats)]
        L.oracle_get_labels.argtypes = [P, P]
        L.oracle_get_state.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), P]
        L.oracle_set_state.argtypes = [P, C.c_double, C.c_double, P]
        L.oracle_get_thresholds.argtypes = [P, P, P, P]
        L.oracle_evdw.restype = C.c_double
        L.oracle_evdw.argtypes = [P, C.c_double]
        L.oracle_philox4x32_10.argtypes = [P, P, P]
        L.oracle_exp.restype = C.c_double
        L.oracle_exp.argtypes = [C.c_double]
        L.oracle_log.restype = C.c_double
        L.oracle_log.argtypes = [C.c_double]
        L.oracle_distances.restype = C.c_int
        L.oracle_distances.argtypes = [C.c_int, C.c_float, P, P, C.c_int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def distances(L: int, Rc: float):
    d = np.zeros(512, dtype=np.float32)
    f = np.zeros(512, dtype=np.int32)
    n = lib().oracle_distances(L, Rc, _ptr(d), _ptr(f), 512)
    if n < 0:
        raise RuntimeError("too many shells")
    return d[:n].copy(), f[:n].copy()


class Oracle:
    """One lattice of the CPU oracle."""

    def __init__(self, L, T, P, seed, Rc=6.0, replica=0, start=0, threads=1, flag_chessboard=1):
        self.L = L
        self.N = L ** 3
        self._h = lib().oracle_create_mode(L, T, P, seed, Rc, replica, start, flag_chessboard)
        if not self._h:
            raise ValueError("oracle_create failed")
        lib().oracle_set_threads(self._h, threads)

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    __del__ = close

    def set_threads(self, n):
        lib().oracle_set_threads(self._h, n)

    def set_config(self, cells12: np.ndarray):
        a = np.ascontiguousarray(cells12, dtype=np.int32).reshape(-1)
        rc = lib().oracle_set_config(self._h, _ptr(a), a.size // 12)
        if rc:
            raise ValueError(f"oracle_set_config rc={rc}")

    def nhb(self) -> np.ndarray:
        """Flag_chessboard = 0: the bond count of every cell (cell = x + L*(y + L*z))."""
        a = np.zeros(self.N, dtype=np.uint8)
        lib().oracle_get_nhb(self._h, _ptr(a))
        return a

    def get_config(self) -> np.ndarray:
        a = np.zeros((self.N, 12), dtype=np.int32)
        lib().oracle_get_config(self._h, _ptr(a), self.N)
        return a

    def get_cubes(self):
        n = (self.L // 2) ** 3
        ev = np.zeros(n, dtype=np.uint8)
        od = np.zeros(n, dtype=np.uint8)
        lib().oracle_get_cubes(self._h, _ptr(ev), _ptr(od))
        return ev, od

    def cube_move(self):
        lib().oracle_cube_move(self._h)

    def volume_move(self):
        lib().oracle_volume_move(self._h)

    def sweep(self):
        lib().oracle_sweep(self._h)

    def sw_step(self):
        lib().oracle_sw_step(self._h)

    def step(self, n_metropolis=1, n_cluster=0):
        lib().oracle_step(self._h, n_metropolis, n_cluster)

    def wolff_step(self):
        lib().oracle_wolff_step(self._h)

    def set_wolff(self, on: bool):
        """Cluster steps of step() are Wolff steps (GW:2199-2357) instead of Swendsen-Wang."""
        lib().oracle_set_wolff(self._h, 1 if on else 0)

    def wolff_stats(self):
        """The last Wolff step: (pokes, summed cluster sizes, largest cluster, poke counter)."""
        a = np.zeros(4, dtype=np.int64)
        lib().oracle_wolff_stats(self._h, _ptr(a))
        return tuple(int(v) for v in a)

    def measure(self) -> Obs:
        o = Obs()
        lib().oracle_measure(self._h, C.byref(o))
        return o

    def cluster_stats(self) -> CStats:
        s = CStats()
        lib().oracle_cluster_stats(self._h, C.byref(s))
        return s

    def labels(self) -> np.ndarray:
        a = np.zeros(6 * self.N, dtype=np.int32)
        lib().oracle_get_labels(self._h, _ptr(a))
        return a

    def state(self):
        r, v, e = C.c_double(), C.c_double(), C.c_double()
        ctr = np.zeros(4, dtype=np.uint32)
        lib().oracle_get_state(self._h, C.byref(r), C.byref(v), C.byref(e), _ptr(ctr))
        return r.value, v.value, e.value, ctr

    def set_state(self, r_cell, volume, counters):
        ctr = np.asarray(counters, dtype=np.uint32)
        lib().oracle_set_state(self._h, r_cell, volume, _ptr(ctr))

    def thresholds(self):
        s = np.zeros(33, dtype=np.uint64)
        c = np.zeros(9, dtype=np.uint64)
        w = np.zeros(2, dtype=np.uint64)
        lib().oracle_get_thresholds(self._h, _ptr(s), _ptr(c), _ptr(w))
        return s, c, w

    def evdw(self, r):
        return lib().oracle_evdw(self._h, r)
