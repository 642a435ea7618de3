"""Reweighted density along the isobar against the reference's processed results.

The reference's multiple-histogram reweighting (HistogramReweighting/
histogram_reweighting_mixed_paramSI_norm_x.f90:1003-1124) cannot be compiled here (no Fortran
compiler), so its only reference pin is physical: the L = 32 density along P = 0.45 in the
reference's own archive (PROCESSED_DATA/CVF_isobars.tar.gz, L32_P0.45_density.dat, rho = N / <V>
with its error). Twelve engine runs along the isobar, reweighted by the GPU kernels
(cvf_reweight_forward with WHAM free energies) to temperatures between the runs, must reproduce
that density within 2 combined standard errors: the archive's error and the jackknife error of
the reweighted value over 10 blocks of every run.
"""
import ctypes as C
import math
import os

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from cvfbulkwater_gb300.engine import Lattice, Params

GOLD = os.path.join(os.path.dirname(__file__), "golden")
pytestmark = pytest.mark.gpu

L, N, P0 = 32, 32 ** 3, 0.45
NB = 10


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _rho(s, ro, runs, f, T, n_iter):
    """Reweighted N / <V> at temperature T (f refined in place by n_iter WHAM iterations)."""
    th = np.array([1.0 / T, float(np.float32(P0)), 0.0, 0.0, 0.0])
    ids = np.array([1], dtype=np.int32)  # V
    out = np.zeros(2)
    abi.check(abi.lib().cvf_reweight_forward(0, _ptr(s), _ptr(ro), len(s), _ptr(runs), len(runs), _ptr(f), n_iter,
                                             1e-10, float(N), _ptr(th), _ptr(ids), 1, _ptr(out)))
    return N / out[0]


def test_reweighted_density_matches_reference_isobar(engine_lib):
    temps = np.linspace(0.60, 0.90, 12)
    lat = Lattice([Params(L=L, T=float(t), P=P0, seed=8800 + i, start=0, replica=i, sample_capacity=12000)
                   for i, t in enumerate(temps)])
    lat.run(10000, 1, 0)
    lat.run_sampled(40000, 1, 0, 4)
    cols = []
    for r in range(len(temps)):
        smp = lat.samples(r)
        obs = [lat.sample_observables(x, r) for x in smp]
        cols.append(np.stack([[o.energy for o in obs], [o.v_total for o in obs], [o.n_hb for o in obs],
                              smp["n_sigma"].astype(np.float64)], 1))
    lat.close()
    n_per = min(len(c) for c in cols) // NB * NB
    cols = [c[:n_per] for c in cols]
    runs = np.ascontiguousarray([[1.0 / float(np.float32(t)), float(np.float32(P0))] for t in temps])

    def stack(keep):
        s = np.ascontiguousarray(np.concatenate([c[keep] for c in cols]))
        ro = np.ascontiguousarray(np.repeat(np.arange(len(cols), dtype=np.int32), keep.sum()))
        return s, ro

    all_rows = np.ones(n_per, dtype=bool)
    s, ro = stack(all_rows)
    f = np.zeros(len(temps))
    _rho(s, ro, runs, f, 0.75, 400)
    table = {round(t, 3): (rho, err) for t, rho, err in np.loadtxt(os.path.join(GOLD, "isobar_P0.45_density.txt"))}
    targets = [0.66, 0.74, 0.82]  # between the runs' temperatures
    full = {t: _rho(s, ro, runs, f.copy(), t, 0) for t in targets}
    jack = {t: [] for t in targets}
    blk = n_per // NB
    for k in range(NB):
        keep = all_rows.copy()
        keep[k * blk:(k + 1) * blk] = False
        sk, rk = stack(keep)
        fk = f.copy()
        _rho(sk, rk, runs, fk, 0.75, 100)
        for t in targets:
            jack[t].append(_rho(sk, rk, runs, fk.copy(), t, 0))
    for t in targets:
        v = np.asarray(jack[t])
        err = math.sqrt((NB - 1) / NB * ((v - v.mean()) ** 2).sum())
        want, want_err = table[t]
        z = (full[t] - want) / math.hypot(err, want_err)
        assert abs(z) < 2.0, (t, full[t], want, err, want_err, z)
