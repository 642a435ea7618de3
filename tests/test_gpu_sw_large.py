"""Swendsen-Wang steps at the sizes of the Swendsen-Wang workload, bit for bit against the oracle.

The reference labels each of the 6N arm sites with the minimum site id of its cluster
(SOURCE/gpu_water3D.cu:2440-2529, min-label scans repeated until nothing changes) and reports
the statistics of print_cluster_statistics (:2677-2780). The engine's labelling is a lock-free
union-find whose roots are hooked with atomicMin; at L = 64 (1.57 M sites) and L = 128
(12.6 M sites) thousands of hooks contend at once, so these sizes are where a scheduling
dependence would show. Every step compares the lattice, all 6N labels and the seven cluster
statistics with the oracle.

The last case starts ordered at T = 0.1, where one cluster spans almost the whole lattice
(about 658 k of 663 k sites at L = 48), so s*s exceeds 2^31 and the reference's int32
accumulation of s*s (:2697) wraps: the wrapped sum is compared as well as the exact one.
"""
import os

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu

FIELDS = ("largest", "second", "n_percolating", "n_clusters", "sum_size", "sum_size2", "sum_size2_wrap32")


def _pair(oracle_mod, L, T, P, seed, start):
    eng = Lattice(Params(L=L, T=T, P=P, seed=seed, start=start))
    ora = oracle_mod.Oracle(L, T, P, seed, 6.0, 0, start, threads=os.cpu_count() or 1)
    return eng, ora


def _compare_step(eng, ora, step):
    ce, co = eng.get_config(), ora.get_config()
    bad = np.argwhere(ce != co)
    assert bad.size == 0, f"step {step}: {len(bad)} lattice entries differ, first {bad[:5].tolist()}"
    le, lo = eng.labels(), ora.labels()
    diff = np.flatnonzero(le != lo)
    assert diff.size == 0, f"step {step}: {diff.size} labels differ, first sites {diff[:5].tolist()}"
    a, b = eng.cluster_stats(), ora.cluster_stats()
    for f in FIELDS:
        assert getattr(a, f) == getattr(b, f), (step, f, getattr(a, f), getattr(b, f))
    oe, oo = eng.observables(), ora.measure()
    assert (oe.n_hb2, oe.n_sigma) == (oo.n_hb2, oo.n_sigma)
    assert eng.state()[:2] == ora.state()[:2]
    return b


@pytest.mark.parametrize("L", [64, 128])
@pytest.mark.parametrize("T", [0.60, 0.75])
def test_swendsen_wang_workload_sizes(engine_lib, oracle_mod, L, T):
    """Random start, P = 0.45, Cluster_Steps = 1, Metropolis_Steps = 0 (one cube move, one volume
    move and one Swendsen-Wang step per step), three steps."""
    eng, ora = _pair(oracle_mod, L, T, 0.45, 44648604 + L, 0)
    for step in range(3):
        eng.run(1, 0, 1)
        ora.step(0, 1)
        cs = _compare_step(eng, ora, step)
        assert cs.sum_size == 6 * L ** 3 and cs.n_clusters > 1
    eng.close()


def test_swendsen_wang_negative_jeff_l64(engine_lib, oracle_mod):
    """P = 1.0 > J_hb / v_hb: Jeff < 0, hydrogen-bond links join unequal sigmas (GW:2413-2425)."""
    eng, ora = _pair(oracle_mod, 64, 0.7, 1.0, 31, 0)
    for step in range(3):
        eng.run(1, 0, 1)
        ora.step(0, 1)
        _compare_step(eng, ora, step)
    eng.close()


def test_swendsen_wang_int32_wrap_of_size_squares(engine_lib, oracle_mod):
    """A spanning cluster larger than 46341 sites: the wrapped int32 sum of s*s differs from the
    exact sum, and both match the oracle (with the percolation count of the spanning cluster)."""
    eng, ora = _pair(oracle_mod, 48, 0.1, 0.45, 777, 2)
    for step in range(3):
        eng.run(1, 0, 1)
        ora.step(0, 1)
        cs = _compare_step(eng, ora, step)
        assert cs.largest > 46341, cs.largest
        assert cs.sum_size2_wrap32 != cs.sum_size2
        assert cs.n_percolating >= 1
    eng.close()
