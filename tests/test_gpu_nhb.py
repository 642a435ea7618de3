"""Flag_chessboard = 0 (the nhb<=4 compatibility mode) on the GPU against the oracle, bit for
bit: lattice, eta, r_cell / volume, move counters and the exact counts of the measurement,
whose N_hb is the reference's greedy typewriter-order count with the cap of 4 (GW:2064-2099);
recorded samples, configurations with arbitrary eta, batches of replicas, Swendsen-Wang steps
(which leave the bond counts stale, as the reference's do) and the rejections (mixed flags)."""
import numpy as np
import pytest

from cvfbulkwater_gb300.abi import CvfError
from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def pair(om, L, T, P, seed, start, replica=0):
    eng = Lattice(Params(L=L, T=T, P=P, seed=seed, start=start, replica=replica, flag_chessboard=0))
    ora = om.Oracle(L, T, P, seed, 6.0, replica, start, flag_chessboard=0)
    return eng, ora


def assert_same(eng, ora, r=0):
    ce, co = eng.get_config(r), ora.get_config()
    bad = np.argwhere(ce != co)
    assert bad.size == 0, f"{len(bad)} mismatching entries, first {bad[:5].tolist()}"
    re_, ve, _, ke = eng.state(r)
    ro, vo, _, ko = ora.state()
    assert re_ == ro and ve == vo
    assert list(ke) == list(ko)
    oe, oo = eng.observables(r), ora.measure()
    assert (oe.n_hb2, oe.n_sigma) == (oo.n_hb2, oo.n_sigma)
    assert oe.energy == oo.energy and oe.enthalpy == oo.enthalpy and oe.v_total == oo.v_total


@pytest.mark.parametrize("L,start", [(4, 0), (6, 2), (8, 0), (10, 0), (16, 2)])
def test_initial_lattice(engine_lib, oracle_mod, L, start):
    eng, ora = pair(oracle_mod, L, 0.6, 0.45, 300 + L, start)
    assert_same(eng, ora)
    eng.close()


@pytest.mark.parametrize("L", [4, 6, 8, 12, 16])
@pytest.mark.parametrize("T,nmet", [(0.7, 1), (0.35, 2)])
def test_metropolis_steps(engine_lib, oracle_mod, L, T, nmet):
    eng, ora = pair(oracle_mod, L, T, 0.45, 900 + L, 0)
    for k in range(3):
        eng.run(3, nmet, 0)
        for _ in range(3):
            ora.step(nmet, 0)
        assert_same(eng, ora)
    eng.close()


def test_ordered_start_low_temperature(engine_lib, oracle_mod):
    # every cell starts with six matched bonds: the greedy count refuses many of them
    eng, ora = pair(oracle_mod, 8, 0.2, 0.45, 21, 2)
    assert eng.observables().n_hb2 < 6 * 512
    for _ in range(5):
        eng.run(4, 1, 0)
        for _ in range(4):
            ora.step(1, 0)
        assert_same(eng, ora)
    eng.close()


@pytest.mark.parametrize("L,T,start", [(34, 0.2, 2), (66, 0.5, 0), (96, 0.3, 2), (130, 0.4, 0)])
def test_long_rows(engine_lib, oracle_mod, L, T, start):
    # rows of more than 32 cells: each lane replays several cells (ragged at 34, 66, 130) and the
    # chain of x bonds crosses lanes; the ordered starts mark most cells
    eng, ora = pair(oracle_mod, L, T, 0.45, 77 + L, start)
    assert_same(eng, ora)
    for _ in range(2):
        eng.run(2, 1, 0)
        for _ in range(2):
            ora.step(1, 0)
        assert_same(eng, ora)
    eng.close()


def test_sampled_run_records(engine_lib, oracle_mod):
    eng, ora = pair(oracle_mod, 6, 0.5, 0.45, 4, 0)
    eng.run_sampled(12, 1, 0, 3)
    smp = eng.samples()
    assert len(smp) == 4
    for k in range(12):
        ora.step(1, 0)
        if k % 3 == 0:
            m = ora.measure()
            s = smp[k // 3]
            assert (int(s["n_hb2"]), int(s["n_sigma"])) == (m.n_hb2, m.n_sigma)
            assert s["r_cell"] == m.r_cell and s["volume"] == m.volume
    eng.close()


def test_config_with_arbitrary_eta(engine_lib, oracle_mod):
    L = 8
    rng = np.random.default_rng(3)
    cfg = np.zeros((L ** 3, 12), dtype=np.int32)
    cfg[:, :6] = rng.integers(0, 6, (L ** 3, 6))
    cfg[:, 6:] = rng.integers(0, 2, (L ** 3, 6))
    eng, ora = pair(oracle_mod, L, 0.5, 0.45, 17, 1)
    for mode in (1, 0):
        if mode == 1 and eng.io_mode != 1:
            continue
        eng.io_mode = mode
        eng.set_config(cfg)
        assert np.array_equal(eng.get_config(), cfg)
    ora.set_config(cfg)
    eng.run(6, 1, 0)
    for _ in range(6):
        ora.step(1, 0)
    assert_same(eng, ora)
    eng.close()


def test_batch_of_replicas(engine_lib, oracle_mod):
    specs = [(4, 0.6, 0.45, 0), (8, 0.4, 0.30, 2), (6, 0.8, 0.10, 0)]
    eng = Lattice([Params(L=L, T=T, P=P, seed=60 + i, start=st, replica=i, flag_chessboard=0)
                   for i, (L, T, P, st) in enumerate(specs)])
    oras = [oracle_mod.Oracle(L, T, P, 60 + i, 6.0, i, st, flag_chessboard=0) for i, (L, T, P, st) in enumerate(specs)]
    eng.run(7, 1, 0)
    for o in oras:
        for _ in range(7):
            o.step(1, 0)
    for i, o in enumerate(oras):
        assert_same(eng, o, i)
    eng.close()


@pytest.mark.parametrize("L,T", [(6, 0.6), (8, 0.45)])
def test_cluster_steps_leave_counts_stale(engine_lib, oracle_mod, L, T):
    # Swendsen-Wang with Flag_chessboard = 0: bonds from the stored eta, counts untouched
    eng, ora = pair(oracle_mod, L, T, 0.45, 40 + L, 0)
    eng.run(5, 1, 1)
    for _ in range(5):
        ora.step(1, 1)
    assert_same(eng, ora)
    assert np.array_equal(eng.labels(), ora.labels())
    eng.run_sampled(4, 1, 1, 2)
    for _ in range(4):
        ora.step(1, 1)
    assert_same(eng, ora)
    eng.close()


def test_rejections(engine_lib):
    with pytest.raises(CvfError):
        Lattice([Params(L=4, T=0.6, P=0.45, seed=1, flag_chessboard=0), Params(L=4, T=0.6, P=0.45, seed=2)])
    with pytest.raises(CvfError):
        Lattice(Params(L=4, T=0.6, P=0.45, seed=1, flag_chessboard=2))
