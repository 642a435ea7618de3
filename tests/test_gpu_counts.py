"""Reads of cvf_observables between runs: a Metropolis-only run that follows cvf_observables
measures its last step on that step's colour-1 sweep, and the next cvf_observables reads that
record instead of measuring the lattice again (as it does after a sampled run whose last step was
recorded). The reads must equal the oracle's full measurement after every step, through the rare
exact (16-bit tie) path, and across the calls that leave no current record (a run without a
following read, sampled runs off the interval grid, cluster steps, new configurations)."""
import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def pair(om, L, T, P, seed, start=0):
    return (Lattice(Params(L=L, T=T, P=P, seed=seed, start=start)),
            om.Oracle(L, T, P, seed, 6.0, 0, start))


def same_counts(eng, ora, r=0):
    oe, oo = eng.observables(r), ora.measure()
    assert (oe.n_hb2, oe.n_sigma) == (oo.n_hb2, oo.n_sigma)
    assert oe.energy == oo.energy and oe.v_total == oo.v_total


@pytest.mark.parametrize("L,T,start", [(8, 0.5, 0), (16, 0.815, 0), (24, 0.3, 2), (32, 0.7, 2)])
def test_read_after_every_step(engine_lib, oracle_mod, L, T, start):
    eng, ora = pair(oracle_mod, L, T, 0.45, 300 + L, start)
    for _ in range(40):
        eng.run(1, 1, 0)
        ora.step(1, 0)
        same_counts(eng, ora)
    # a few steps between reads (the run after a read measures only its last step)
    eng.run(7, 2, 0)
    for _ in range(7):
        ora.step(2, 0)
    same_counts(eng, ora)
    eng.close()


@pytest.mark.parametrize("L", [32, 48])
def test_eight_cell_tile(engine_lib, oracle_mod, L):
    # a handle on the 8-cell sweep tile: its last step measured with the 8-cell measuring sweep
    eng, ora = pair(oracle_mod, L, 0.7, 0.45, 40 + L, 2)
    assert eng.set_sweep_tile(8) == 8
    for _ in range(12):
        eng.run(1, 1, 0)
        ora.step(1, 0)
        same_counts(eng, ora)
    eng.run(3, 1, 0)  # plain 8-cell steps between reads
    eng.run(2, 1, 0)
    for _ in range(5):
        ora.step(1, 0)
    same_counts(eng, ora)
    assert np.array_equal(eng.get_config(), ora.get_config())
    eng.close()


def test_through_the_exact_path(engine_lib, oracle_mod):
    # L=16 x 6 arms x 400 steps: some 150 arm decisions need the low half of the uniform
    eng, ora = pair(oracle_mod, 16, 0.6, 0.45, 77)
    for _ in range(400):
        eng.run(1, 1, 0)
        ora.step(1, 0)
        o = eng.observables()
    oo = ora.measure()
    assert (o.n_hb2, o.n_sigma) == (oo.n_hb2, oo.n_sigma)
    eng.close()


def test_mixed_calls(engine_lib, oracle_mod):
    eng, ora = pair(oracle_mod, 12, 0.6, 0.45, 9)
    seq = []

    def run(n, nmet=1, ncl=0):
        eng.run(n, nmet, ncl)
        for _ in range(n):
            ora.step(nmet, ncl)

    run(5)
    same_counts(eng, ora)
    for _ in range(5):
        run(1)
        same_counts(eng, ora)
    eng.run_sampled(4, 1, 0, 2)  # last step off the interval grid: the read measures in full
    for _ in range(4):
        ora.step(1, 0)
    same_counts(eng, ora)
    eng.run_sampled(5, 1, 0, 2)  # last step recorded: the read takes its record
    for _ in range(5):
        ora.step(1, 0)
    same_counts(eng, ora)
    # a state set after the record: the read takes r_cell and volume from it
    r_cell, vol, _, ctr = eng.state()
    eng.set_state(r_cell * 1.001, vol * 1.001 ** 3, ctr)
    ora.set_state(r_cell * 1.001, vol * 1.001 ** 3, ctr)
    same_counts(eng, ora)
    run(3, 0, 1)  # Swendsen-Wang steps leave no record: the next read measures in full
    same_counts(eng, ora)
    run(2)
    same_counts(eng, ora)
    cfg = ora.get_config()
    run(3)
    eng.set_config(cfg)  # back to the configuration of three steps ago
    ora.set_config(cfg)
    same_counts(eng, ora)
    run(2)
    same_counts(eng, ora)
    eng.close()


def test_batch_reads(engine_lib, oracle_mod):
    specs = [(8, 0.5), (12, 0.7), (16, 0.9)]
    eng = Lattice([Params(L=L, T=T, P=0.45, seed=40 + i, start=0, replica=i) for i, (L, T) in enumerate(specs)])
    oras = [oracle_mod.Oracle(L, T, 0.45, 40 + i, 6.0, i, 0) for i, (L, T) in enumerate(specs)]
    for _ in range(10):
        eng.run(1, 1, 0)
        for i, o in enumerate(oras):
            o.step(1, 0)
        for i, o in enumerate(oras):
            same_counts(eng, o, i)
    eng.close()


def test_reads_in_persistent_mode(engine_lib, oracle_mod):
    # plain steps in the persistent kernel, the measured last step in the per-phase kernels
    eng, ora = pair(oracle_mod, 12, 0.7, 0.45, 21)
    eng.launch_mode = 1
    same_counts(eng, ora)
    for n in (1, 3, 2, 1):
        eng.run(n, 2, 0)
        for _ in range(n):
            ora.step(2, 0)
        same_counts(eng, ora)
    assert np.array_equal(eng.get_config(), ora.get_config())
    eng.close()


def test_grouped_batch_reads(engine_lib, oracle_mod):
    # eight replicas run as replica groups on parallel graph branches; the measured last step too
    specs = [(8 + 4 * (i % 3), 0.5 + 0.05 * i) for i in range(8)]
    eng = Lattice([Params(L=L, T=T, P=0.45, seed=60 + i, start=0, replica=i) for i, (L, T) in enumerate(specs)])
    oras = [oracle_mod.Oracle(L, T, 0.45, 60 + i, 6.0, i, 0) for i, (L, T) in enumerate(specs)]
    for i, o in enumerate(oras):
        same_counts(eng, o, i)
    for n in (1, 2, 1):
        eng.run(n, 1, 0)
        for o in oras:
            for _ in range(n):
                o.step(1, 0)
        for i, o in enumerate(oras):
            same_counts(eng, o, i)
    eng.close()
