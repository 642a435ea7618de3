"""Wolff cluster steps (GW:2199-2357) on the GPU against the oracle's restatement.

The engine grows one poke per warp in speculative batches and commits the pokes before the
first one that read a cell an earlier poke of the batch changes; a poke whose cluster outgrows
its warp is grown by the whole grid. Whatever the batching, the lattice, the poke counter and
the step's pokes, summed and largest cluster sizes must equal the oracle's sequential pokes.
"""
import os

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def _pair(oracle_mod, L, T, P, seed, start, flag_chessboard=1):
    eng = Lattice(Params(L=L, T=T, P=P, seed=seed, start=start, flag_chessboard=flag_chessboard))
    eng.set_cluster_algorithm(True)
    ora = oracle_mod.Oracle(L, T, P, seed, 6.0, 0, start, threads=os.cpu_count() or 1,
                            flag_chessboard=flag_chessboard)
    ora.set_wolff(True)
    return eng, ora


def _compare(eng, ora, step):
    assert np.array_equal(eng.get_config(), ora.get_config()), f"step {step}: lattices differ"
    assert eng.wolff_stats() == ora.wolff_stats(), (step, eng.wolff_stats(), ora.wolff_stats())
    oe, oo = eng.observables(), ora.measure()
    assert (oe.n_hb2, oe.n_sigma) == (oo.n_hb2, oo.n_sigma)
    assert eng.state()[:2] == ora.state()[:2]


@pytest.mark.parametrize("L,T,P,start,nmet", [(8, 0.7, 0.45, 0, 1), (16, 0.6, 0.45, 0, 0), (24, 0.75, 0.45, 0, 1),
                                              (32, 0.6, 0.45, 2, 1)])
def test_wolff_matches_oracle(engine_lib, oracle_mod, L, T, P, start, nmet):
    eng, ora = _pair(oracle_mod, L, T, P, 4100 + L, start)
    for step in range(3):
        eng.run(1, nmet, 1)
        ora.step(nmet, 1)
        _compare(eng, ora, step)
    pokes, total, largest, counter = eng.wolff_stats()
    assert total >= 6 * L ** 3 and pokes > 1 and counter > 2 * pokes
    eng.close()


def test_wolff_large_clusters_grown_by_the_grid(engine_lib, oracle_mod):
    """T = 0.1 from the ordered start: clusters far larger than a warp's 128 sites, grown level by
    level by the whole grid."""
    eng, ora = _pair(oracle_mod, 16, 0.1, 0.45, 77, 2)
    for step in range(3):
        eng.run(1, 1, 1)
        ora.step(1, 1)
        _compare(eng, ora, step)
        assert eng.wolff_stats()[2] > 128
    eng.close()


def test_wolff_negative_jeff_and_nhb_mode(engine_lib, oracle_mod):
    """P = 1.0 (Jeff < 0: hydrogen-bond links join unequal sigmas) and the nhb<=4 mode (eta as
    stored, every arm active)."""
    eng, ora = _pair(oracle_mod, 12, 0.7, 1.0, 31, 0)
    for step in range(2):
        eng.run(1, 1, 1)
        ora.step(1, 1)
        _compare(eng, ora, step)
    eng.close()
    eng, ora = _pair(oracle_mod, 12, 0.7, 0.45, 32, 0, flag_chessboard=0)
    for step in range(2):
        eng.run(1, 1, 1)
        ora.step(1, 1)
        assert np.array_equal(eng.get_config(), ora.get_config())
        assert eng.wolff_stats() == ora.wolff_stats()
    eng.close()


def test_wolff_batch_and_counter_restore(engine_lib, oracle_mod):
    """Replicas of uneven L step one after another through the same scratch; a handle whose poke
    counter is set continues the oracle's chain."""
    specs = [(8, 0.65), (16, 0.8), (12, 0.7)]
    eng = Lattice([Params(L=L, T=T, P=0.45, seed=900 + i, start=0, replica=i) for i, (L, T) in enumerate(specs)])
    eng.set_cluster_algorithm(True)
    oras = []
    for i, (L, T) in enumerate(specs):
        o = oracle_mod.Oracle(L, T, 0.45, 900 + i, 6.0, i, 0)
        o.set_wolff(True)
        oras.append(o)
    eng.run(2, 1, 1)
    for o in oras:
        o.step(1, 1)
        o.step(1, 1)
    for i, o in enumerate(oras):
        assert np.array_equal(eng.get_config(i), o.get_config()), i
        assert eng.wolff_stats(i) == o.wolff_stats(), i
    eng.close()
    # resume: a fresh handle given the configuration, the counters and the poke counter
    L, T = specs[1]
    o = oras[1]
    e2 = Lattice(Params(L=L, T=T, P=0.45, seed=901, start=1, replica=1))
    e2.set_cluster_algorithm(True)
    e2.set_config(o.get_config())
    r_cell, volume, _, counters = o.state()
    e2.set_state(r_cell, volume, counters)
    e2.set_wolff_counter(0, o.wolff_stats()[3])
    e2.run(1, 0, 1)
    o.step(0, 1)
    assert np.array_equal(e2.get_config(), o.get_config())
    assert e2.wolff_stats()[:3] == o.wolff_stats()[:3]
    e2.close()


def test_wolff_switching_sampled_and_tiny(engine_lib, oracle_mod):
    """Swendsen-Wang and Wolff steps alternate on one handle as the oracle alternates them; a
    sampled run records after Wolff steps; an L=4 lattice (48 sites, far fewer than a batch's
    pokes) steps like the oracle."""
    eng, ora = _pair(oracle_mod, 12, 0.7, 0.45, 55, 0)
    eng.set_cluster_algorithm(False)
    ora.set_wolff(False)
    eng.run(1, 1, 1)
    ora.step(1, 1)
    eng.set_cluster_algorithm(True)
    ora.set_wolff(True)
    eng.run(2, 1, 1)
    ora.step(1, 1)
    ora.step(1, 1)
    eng.set_cluster_algorithm(False)
    ora.set_wolff(False)
    eng.run(1, 0, 1)
    ora.step(0, 1)
    assert np.array_equal(eng.get_config(), ora.get_config())
    assert np.array_equal(eng.labels(), ora.labels())
    eng.set_cluster_algorithm(True)
    ora.set_wolff(True)
    eng.run_sampled(4, 1, 1, 2)
    rec = []
    for k in range(4):
        ora.step(1, 1)
        if k % 2 == 0:
            rec.append(ora.measure())
    smp = eng.samples()
    assert len(smp) == 2
    for got, want in zip(smp, rec):
        assert (got["n_hb2"], got["n_sigma"], got["r_cell"]) == (want.n_hb2, want.n_sigma, want.r_cell)
    assert np.array_equal(eng.get_config(), ora.get_config())
    assert eng.wolff_stats() == ora.wolff_stats()
    eng.close()
    eng, ora = _pair(oracle_mod, 4, 0.7, 0.45, 56, 0)
    for step in range(3):
        eng.run(1, 1, 1)
        ora.step(1, 1)
        _compare(eng, ora, step)
    eng.close()
