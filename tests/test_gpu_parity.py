"""GPU engine vs CPU oracle, bit for bit, through the C ABI.

Lattice (sigma and eta of every arm), cube-derived eta, r_cell / volume bits, move counters and
the exact int64 counts must agree after any number of steps; Swendsen-Wang labels and cluster
statistics likewise.
"""
import os

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

GOLD = os.path.join(os.path.dirname(__file__), "golden")
pytestmark = pytest.mark.gpu


def pair(oracle_mod, L, T, P, seed, start, replica=0, threads=1):
    eng = Lattice(Params(L=L, T=T, P=P, seed=seed, start=start, replica=replica))
    ora = oracle_mod.Oracle(L, T, P, seed, 6.0, replica, start, threads=threads)
    return eng, ora


def assert_same(eng, ora, r=0):
    ce, co = eng.get_config(r), ora.get_config()
    bad = np.argwhere(ce != co)
    assert bad.size == 0, f"{len(bad)} mismatching entries, first {bad[:5].tolist()}"
    re_, ve, _, ke = eng.state(r)
    ro, vo, _, ko = ora.state()
    assert re_ == ro and ve == vo, (re_, ro, ve, vo)
    assert list(ke) == list(ko)
    oe, oo = eng.observables(r), ora.measure()
    assert oe.n_hb2 == oo.n_hb2 and oe.n_sigma == oo.n_sigma
    assert oe.energy == oo.energy and oe.enthalpy == oo.enthalpy and oe.v_total == oo.v_total


def test_thresholds_identical(engine_lib, oracle_mod):
    eng, ora = pair(oracle_mod, 8, 0.815, 0.45, 5, 0)
    s, c, w = eng.thresholds()
    so, co, wo = ora.thresholds()
    assert np.array_equal(s, so) and np.array_equal(c, co) and np.array_equal(w, wo)


@pytest.mark.parametrize("L,start", [(4, 0), (6, 0), (8, 2), (12, 0), (16, 0), (16, 2)])
def test_initial_lattice(engine_lib, oracle_mod, L, start):
    eng, ora = pair(oracle_mod, L, 0.815, 0.45, 44648604 + L, start)
    assert_same(eng, ora)


@pytest.mark.parametrize("L", [4, 6, 8, 10, 16])
@pytest.mark.parametrize("steps", [1, 2, 10])
def test_metropolis_steps(engine_lib, oracle_mod, L, steps):
    eng, ora = pair(oracle_mod, L, 0.815, 0.45, 1234 + L, 0)
    eng.run(steps, 1, 0)
    for _ in range(steps):
        ora.step(1, 0)
    assert_same(eng, ora)


def test_many_steps_low_temperature(engine_lib, oracle_mod):
    eng, ora = pair(oracle_mod, 8, 0.55, 0.0, 99, 2)
    eng.run(100, 2, 0)
    for _ in range(100):
        ora.step(2, 0)
    assert_same(eng, ora)


def test_reference_input_config(engine_lib, oracle_mod):
    cfg = np.load(os.path.join(GOLD, "input_config_L32.npz"))["cells12"].astype(np.int32)
    eng, ora = pair(oracle_mod, 32, 0.815, 0.45, 44648604, 1, threads=os.cpu_count() or 1)
    eng.set_config(cfg)
    ora.set_config(cfg)
    assert np.array_equal(eng.get_config(), cfg)
    assert_same(eng, ora)
    eng.run(20, 1, 0)
    for _ in range(20):
        ora.step(1, 0)
    assert_same(eng, ora)


@pytest.mark.parametrize("L,T", [(4, 0.6), (8, 0.6), (8, 0.75), (16, 0.6)])
def test_swendsen_wang(engine_lib, oracle_mod, L, T):
    eng, ora = pair(oracle_mod, L, T, 0.45, 777 + L, 0)
    for step in range(3):
        eng.run(1, 1 if step == 1 else 0, 1)
        ora.step(1 if step == 1 else 0, 1)
        assert_same(eng, ora)
        assert np.array_equal(eng.labels(), ora.labels())
        a, b = eng.cluster_stats(), ora.cluster_stats()
        for f in ("largest", "second", "n_percolating", "n_clusters", "sum_size", "sum_size2", "sum_size2_wrap32"):
            assert getattr(a, f) == getattr(b, f), f


def test_high_pressure_negative_jeff(engine_lib, oracle_mod):
    # P > J_hb / v_hb makes Jeff < 0: SW bonds join unequal sigmas (GW:2413-2425)
    eng, ora = pair(oracle_mod, 8, 0.7, 1.0, 31, 0)
    eng.run(3, 1, 1)
    for _ in range(3):
        ora.step(1, 1)
    assert_same(eng, ora)
    assert np.array_equal(eng.labels(), ora.labels())


def test_batch_matches_individual_oracles(engine_lib, oracle_mod):
    specs = [(16, 0.6, 0.0), (8, 0.9, 0.6), (24, 0.75, 0.3), (12, 0.55, 0.45)]
    params = [Params(L=L, T=T, P=P, seed=1000 + i, start=0, replica=i) for i, (L, T, P) in enumerate(specs)]
    eng = Lattice(params)
    eng.run(5, 1, 0)
    for i, (L, T, P) in enumerate(specs):
        ora = oracle_mod.Oracle(L, T, P, 1000 + i, 6.0, i, 0)
        for _ in range(5):
            ora.step(1, 0)
        assert_same(eng, ora, r=i)


def test_sampled_run_matches_observables(engine_lib, oracle_mod):
    eng, ora = pair(oracle_mod, 8, 0.815, 0.45, 4242, 0)
    eng.run_sampled(25, 1, 0, 10)
    smp = eng.samples()
    assert len(smp) == 3
    for i in range(25):
        ora.step(1, 0)
        if i % 10 == 0:
            ob = ora.measure()
            s = smp[i // 10]
            assert s["n_hb2"] == ob.n_hb2 and s["n_sigma"] == ob.n_sigma and s["r_cell"] == ob.r_cell


def test_checkpoint_resume_is_exact(engine_lib, oracle_mod):
    a = Lattice(Params(L=8, T=0.7, P=0.45, seed=5, start=0))
    a.run(7, 1, 0)
    cfg, st = a.get_config(), a.state()
    b = Lattice(Params(L=8, T=0.7, P=0.45, seed=5, start=1))
    b.set_config(cfg)
    b.set_state(st[0], st[1], st[3])
    a.run(5, 1, 0)
    b.run(5, 1, 0)
    assert np.array_equal(a.get_config(), b.get_config())
    assert a.state()[:2] == b.state()[:2]


def test_l256_bit_exact_after_ten_sweeps(engine_lib, oracle_mod):
    """Bandwidth-bound workload: L=256, ordered start, T=0.70, P=0.45, Metropolis only."""
    eng, ora = pair(oracle_mod, 256, 0.70, 0.45, 44648604, 2, threads=os.cpu_count() or 1)
    eng.run(10, 1, 0)
    for _ in range(10):
        ora.step(1, 0)
    assert_same(eng, ora)


@pytest.mark.parametrize("tile", [1, 2, 4, 8])
def test_recorded_samples_every_tile(engine_lib, oracle_mod, tile):
    """Recorded steps fuse the measurement into the last colour-1 sweep; every tile must give the
    oracle's counts (L=16: H=8 admits all four tiles)."""
    eng, ora = pair(oracle_mod, 16, 0.72, 0.45, 99, 0)
    assert eng.set_sweep_tile(tile) == tile
    eng.run_sampled(9, 2, 0, 3)
    smp = eng.samples()
    assert len(smp) == 3
    for i in range(9):
        ora.step(2, 0)
        if i % 3 == 0:
            ob = ora.measure()
            s = smp[i // 3]
            assert s["n_hb2"] == ob.n_hb2 and s["n_sigma"] == ob.n_sigma and s["r_cell"] == ob.r_cell
    assert_same(eng, ora)
