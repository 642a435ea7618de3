"""Persistent step kernel (one cooperative launch per captured chunk of Metropolis steps) against
the per-phase launches and the CPU oracle, bit for bit.

Both launch modes must leave the same lattices, cube states, move counters, volume chain and
recorded samples for a batch of uneven replicas, for any number of sweeps per step and any
sampling interval; the persistent mode must be captured into the graph, not fall back.
"""
import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu

SPECS = [(6, 0.6, 0.0), (16, 0.9, 0.6), (24, 0.75, 0.3), (12, 0.55, 0.45), (40, 0.8, 0.2), (8, 0.7, 0.45)]


def batch(seed=77, start=0):
    return Lattice([Params(L=L, T=T, P=P, seed=seed + i, start=start, replica=i) for i, (L, T, P) in enumerate(SPECS)])


def snapshot(lat):
    out = []
    for r in range(len(SPECS)):
        out.append((lat.get_config(r), lat.state(r), lat.samples(r)))
    return out


def assert_snapshots_equal(a, b):
    for r, ((ca, sa, pa), (cb, sb, pb)) in enumerate(zip(a, b)):
        assert np.array_equal(ca, cb), f"replica {r}: lattices differ"
        assert sa[0] == sb[0] and sa[1] == sb[1] and list(sa[3]) == list(sb[3]), (r, sa, sb)
        assert len(pa) == len(pb), (r, len(pa), len(pb))
        for x, y in zip(pa, pb):
            assert x == y, (r, x, y)


def test_persistent_mode_is_captured(engine_lib):
    """The cooperative launch is captured into the graph (no silent fallback to mode 0)."""
    lat = batch()
    assert lat.launch_mode == 0
    lat.launch_mode = 1
    lat.run(3, 1, 0)
    lat.run_sampled(4, 1, 0, 2)
    lat.synchronize()
    assert lat.launch_mode == 1


@pytest.mark.parametrize("nmet", [1, 2])
def test_modes_identical_plain_runs(engine_lib, nmet):
    snaps = []
    for mode in (0, 1):
        lat = batch()
        lat.launch_mode = mode
        lat.run(33, nmet, 0)  # one chunk of 32 steps plus a remainder of 1
        lat.run(5, nmet, 0)
        snaps.append(snapshot(lat))
        assert lat.launch_mode == mode
        lat.close()
    assert_snapshots_equal(*snaps)


@pytest.mark.parametrize("interval", [1, 4, 7])
def test_modes_identical_sampled_runs(engine_lib, interval):
    snaps = []
    for mode in (0, 1):
        lat = batch(seed=91, start=2)
        lat.launch_mode = mode
        lat.run_sampled(29, 1, 0, interval)
        lat.run(3, 1, 0)
        lat.run_sampled(6, 2, 0, interval)
        snaps.append(snapshot(lat))
        lat.close()
    assert_snapshots_equal(*snaps)
    assert len(snaps[1][0][2]) == -(-29 // interval) + -(-6 // interval)


def test_mode_switch_mid_chain(engine_lib):
    """Switching modes between calls continues the same Markov chain."""
    ref = batch(seed=5)
    ref.launch_mode = 0
    ref.run(20, 1, 0)
    mix = batch(seed=5)
    mix.launch_mode = 1
    mix.run(7, 1, 0)
    mix.launch_mode = 0
    mix.run(6, 1, 0)
    mix.launch_mode = 1
    mix.run(7, 1, 0)
    assert_snapshots_equal(snapshot(ref), snapshot(mix))


def test_persistent_matches_oracle_two_sweeps(engine_lib, oracle_mod):
    eng = Lattice(Params(L=10, T=0.65, P=0.3, seed=2024, start=0, replica=3))
    eng.launch_mode = 1
    ora = oracle_mod.Oracle(10, 0.65, 0.3, 2024, 6.0, 3, 0)
    eng.run_sampled(12, 2, 0, 5)
    smp = eng.samples()
    for i in range(12):
        ora.step(2, 0)
        if i % 5 == 0:
            ob = ora.measure()
            s = smp[i // 5]
            assert s["n_hb2"] == ob.n_hb2 and s["n_sigma"] == ob.n_sigma and s["r_cell"] == ob.r_cell
    assert np.array_equal(eng.get_config(), ora.get_config())
    assert list(eng.state()[3]) == list(ora.state()[3])
