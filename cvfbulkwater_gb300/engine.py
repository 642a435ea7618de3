"""Python face of the engine: one handle of one or more replicas behind the C ABI.

Mirrors the calls a reference user makes through gpu_water3D: load a configuration
(input_config), run Monte Carlo steps (MonteCarlo_Step, GW:1346-1733), measure (measure,
GW:2014-2160) and read cluster statistics (print_cluster_statistics, GW:2677-2721).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .abi import check, lib


@dataclass
class Params:
    L: int
    T: float
    P: float
    seed: int
    R_cutoff: float = 6.0
    start: int = 0            # Flag_config: 0 disordered, 1 from set_config, 2 ordered
    flag_chessboard: int = 1
    replica: int = 0
    device: int = 0
    sample_capacity: int = 0

    def to_c(self) -> abi.Params:
        return abi.Params(self.L, self.T, self.P, self.seed, self.R_cutoff, self.start,
                          self.flag_chessboard, self.replica, self.device, self.sample_capacity)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Lattice:
    """A handle of n >= 1 replicas on one GPU."""

    def __init__(self, params):
        if isinstance(params, Params):
            params = [params]
        arr = (abi.Params * len(params))(*[p.to_c() for p in params])
        h = C.c_void_p()
        if len(params) == 1:
            check(lib().cvf_create(arr, C.byref(h)))
        else:
            check(lib().cvf_batch_create(arr, len(params), C.byref(h)))
        self._h = h
        self.params = list(params)

    def close(self):
        if getattr(self, "_h", None):
            lib().cvf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def n_replicas(self) -> int:
        return lib().cvf_num_replicas(self._h)

    def N(self, r=0) -> int:
        return self.params[r].L ** 3

    # -- configuration
    def set_config(self, cells12: np.ndarray, r: int = 0):
        a = np.ascontiguousarray(cells12, dtype=np.int32)
        check(lib().cvf_set_config(self._h, r, _ptr(a), a.size // 12))

    def get_config(self, r: int = 0, out: np.ndarray = None) -> np.ndarray:
        """cells12 of replica r; pass `out` (int32, (N, 12), C-contiguous) to reuse a buffer."""
        a = np.empty((self.N(r), 12), dtype=np.int32) if out is None else out
        if a.dtype != np.int32 or a.shape != (self.N(r), 12) or not a.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous int32 array of shape (N, 12)")
        check(lib().cvf_get_config(self._h, r, _ptr(a), self.N(r)))
        return a

    def set_arms(self, s: np.ndarray, active_bond: np.ndarray, r: int = 0):
        """The reference's host arrays s[arm*N + cell] and active_bond[arm*N + cell] (uint8)."""
        a = np.ascontiguousarray(s, dtype=np.uint8).reshape(-1)
        b = np.ascontiguousarray(active_bond, dtype=np.uint8).reshape(-1)
        check(lib().cvf_set_arms(self._h, r, _ptr(a), _ptr(b), a.size))

    def get_arms(self, r: int = 0, out=None):
        """(s, active_bond) of replica r as uint8 arrays of 6N bytes (arm-major); pass `out`, a pair
        of such arrays, to reuse buffers."""
        n = 6 * self.N(r)
        a, b = (np.empty(n, dtype=np.uint8), np.empty(n, dtype=np.uint8)) if out is None else out
        for x in (a, b):
            if x.dtype != np.uint8 or x.size != n or not x.flags.c_contiguous:
                raise ValueError("out must hold two C-contiguous uint8 arrays of 6 N bytes")
        check(lib().cvf_get_arms(self._h, r, _ptr(a), _ptr(b), n))
        return a, b

    def packed_size(self, r: int = 0) -> int:
        n = C.c_longlong()
        check(lib().cvf_packed_size(self._h, r, C.byref(n)))
        return n.value

    def get_packed(self, r: int = 0, out: np.ndarray = None) -> np.ndarray:
        """The replica's packed state (colour words, then cube states) as uint8; pass `out` to
        reuse a buffer."""
        n = self.packed_size(r)
        a = np.empty(n, dtype=np.uint8) if out is None else out
        if a.dtype != np.uint8 or a.size != n or not a.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous uint8 array of packed_size() bytes")
        check(lib().cvf_get_packed(self._h, r, _ptr(a), n))
        return a

    def set_packed(self, buf: np.ndarray, r: int = 0):
        a = np.ascontiguousarray(buf, dtype=np.uint8)
        check(lib().cvf_set_packed(self._h, r, _ptr(a), a.size))

    def set_distances(self, dist, freq, r: int = 0):
        d = np.ascontiguousarray(dist, dtype=np.float32)
        f = np.ascontiguousarray(freq, dtype=np.int32)
        check(lib().cvf_set_distances(self._h, r, _ptr(d), _ptr(f), d.size))

    def get_distances(self, r: int = 0):
        d = np.zeros(512, dtype=np.float32)
        f = np.zeros(512, dtype=np.int32)
        n = C.c_int()
        check(lib().cvf_get_distances(self._h, r, _ptr(d), _ptr(f), 512, C.byref(n)))
        return d[: n.value].copy(), f[: n.value].copy()

    def autotune(self) -> int:
        """Pick the fastest sweep tile (cells per thread) for these replicas; returns it."""
        v = C.c_int()
        check(lib().cvf_autotune(self._h, C.byref(v)))
        return v.value

    def tuning(self):
        """(tile, log2 of the row patch or -1, launch mode) in effect."""
        t, g, m = C.c_int(), C.c_int(), C.c_int()
        check(lib().cvf_get_tuning(self._h, C.byref(t), C.byref(g), C.byref(m)))
        return t.value, g.value, m.value

    def set_row_tile(self, lg_rows: int):
        check(lib().cvf_set_row_tile(self._h, int(lg_rows)))

    @property
    def replica_groups(self) -> int:
        """Groups of consecutive replicas captured on parallel graph branches (count in effect)."""
        g = C.c_int()
        check(lib().cvf_get_replica_groups(self._h, C.byref(g)))
        return g.value

    @replica_groups.setter
    def replica_groups(self, groups: int):
        check(lib().cvf_set_replica_groups(self._h, int(groups)))

    def set_cluster_algorithm(self, wolff: bool):
        """Cluster steps of run() are Wolff steps (pokes until their clusters cover 6N sites)
        instead of Swendsen-Wang steps."""
        check(lib().cvf_set_cluster_algorithm(self._h, 1 if wolff else 0))

    def wolff_stats(self, r: int = 0):
        """The last Wolff step of replica r: (pokes, summed cluster sizes, largest cluster,
        poke counter)."""
        a = np.zeros(4, dtype=np.int64)
        check(lib().cvf_wolff_stats(self._h, r, _ptr(a)))
        return tuple(int(v) for v in a)

    def set_wolff_counter(self, r: int, pokes: int):
        check(lib().cvf_set_wolff_counter(self._h, r, int(pokes)))

    def set_correlation(self, enable: bool):
        """Start (and reset) or stop the per-step multi-tau autocorrelation of every replica."""
        check(lib().cvf_set_correlation(self._h, 1 if enable else 0))

    def correlation(self, r: int = 0):
        """(t, f) of replica r's correlator, evaluated as the reference does at the end of a run."""
        n = C.c_int()
        cap = 32 * 16
        t, f = np.zeros(cap), np.zeros(cap)
        check(lib().cvf_get_correlation(self._h, r, _ptr(t), _ptr(f), cap, C.byref(n)))
        return t[: n.value].copy(), f[: n.value].copy()

    def run_statistics(self):
        """Mean and <x^2> - <x>^2 of the data.out columns over each replica's recorded samples,
        computed on the GPU (the awk stage of the reference's isobar analysis)."""
        n = self.n_replicas
        rows = (abi.RunStats * n)()
        check(lib().cvf_run_statistics(self._h, rows, n))
        return [{"L": r.L, "P": r.P, "T": r.T, "mean": list(r.mean), "var": list(r.var), "n": r.n} for r in rows]

    def set_sweep_tile(self, vec: int) -> int:
        """Set the sweep tile (cells per thread) by hand; returns the tile in effect."""
        v = C.c_int()
        check(lib().cvf_set_sweep_tile(self._h, int(vec), C.byref(v)))
        return v.value

    @property
    def io_mode(self) -> int:
        """1: set_config / get_config read and write the caller's array in host memory from the
        GPU; 0: host packing and unpacking."""
        m = C.c_int()
        check(lib().cvf_get_io_mode(self._h, C.byref(m)))
        return m.value

    @io_mode.setter
    def io_mode(self, mode: int):
        check(lib().cvf_set_io_mode(self._h, int(mode)))

    @property
    def launch_mode(self) -> int:
        """1: Metropolis-only steps run as one persistent launch per graph; 0: one launch per phase."""
        m = C.c_int()
        check(lib().cvf_get_launch_mode(self._h, C.byref(m)))
        return m.value

    @launch_mode.setter
    def launch_mode(self, mode: int):
        check(lib().cvf_set_launch_mode(self._h, int(mode)))

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        check(lib().cvf_get_stream(self._h, C.byref(s)))
        return s.value or 0

    # -- running
    def run(self, n_steps: int, n_metropolis: int = 1, n_cluster: int = 0):
        check(lib().cvf_run_steps(self._h, n_steps, n_metropolis, n_cluster))

    def run_sampled(self, n_steps: int, n_metropolis: int, n_cluster: int, interval: int):
        check(lib().cvf_run_sampled(self._h, n_steps, n_metropolis, n_cluster, interval))

    def synchronize(self):
        check(lib().cvf_synchronize(self._h))

    # -- measurement
    def observables(self, r: int = 0) -> abi.Obs:
        o = abi.Obs()
        check(lib().cvf_observables(self._h, r, C.byref(o)))
        return o

    def cluster_stats(self, r: int = 0) -> abi.CStats:
        s = abi.CStats()
        check(lib().cvf_cluster_stats(self._h, r, C.byref(s)))
        return s

    def labels(self, r: int = 0) -> np.ndarray:
        a = np.zeros(6 * self.N(r), dtype=np.int32)
        check(lib().cvf_get_labels(self._h, r, _ptr(a), a.size))
        return a

    def samples(self, r: int = 0) -> np.ndarray:
        n = C.c_longlong()
        check(lib().cvf_sample_count(self._h, r, C.byref(n)))
        buf = (abi.Sample * max(n.value, 1))()
        got = C.c_longlong()
        check(lib().cvf_get_samples(self._h, r, buf, n.value, C.byref(got)))
        dt = np.dtype([("n_hb2", np.int64), ("n_sigma", np.int64), ("r_cell", np.float64),
                       ("volume", np.float64)])
        return np.frombuffer(bytes(buf), dtype=dt, count=got.value).copy()

    def cstats_stream(self, r: int = 0):
        n = C.c_longlong()
        check(lib().cvf_sample_count(self._h, r, C.byref(n)))
        buf = (abi.CStats * max(n.value, 1))()
        got = C.c_longlong()
        check(lib().cvf_get_cstats_stream(self._h, r, buf, n.value, C.byref(got)))
        return [buf[i] for i in range(got.value)]

    def clear_samples(self):
        check(lib().cvf_clear_samples(self._h))

    def sample_observables(self, s, r: int = 0) -> abi.Obs:
        smp = abi.Sample(int(s["n_hb2"]), int(s["n_sigma"]), float(s["r_cell"]), float(s["volume"]))
        o = abi.Obs()
        check(lib().cvf_sample_observables(self._h, r, C.byref(smp), C.byref(o)))
        return o

    def state(self, r: int = 0):
        s = abi.State()
        check(lib().cvf_get_state(self._h, r, C.byref(s)))
        return s.r_cell, s.volume, s.e_vdw, np.array(list(s.counters), dtype=np.uint32)

    def set_state(self, r_cell: float, volume: float, counters, r: int = 0):
        s = abi.State(r_cell, volume, 0.0, (C.c_uint * 4)(*[int(c) for c in counters]))
        check(lib().cvf_set_state(self._h, r, C.byref(s)))

    def thresholds(self, r: int = 0):
        a = np.zeros(44, dtype=np.uint64)
        check(lib().cvf_get_thresholds(self._h, r, _ptr(a)))
        return a[:33], a[33:42], a[42:44]
