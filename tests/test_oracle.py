"""CPU oracle pinned against the reference's own artefacts (no GPU needed).

Pins: Philox4x32-10 known-answer vectors (Salmon et al. SC'11; Random123 kat_vectors), the
reference's SOURCE/distances file (exact), SOURCE/input_config and config.out (chessboard
invariants, exact round trip) and the statistics of SOURCE/data.out (L=32, T=0.815, P=0.45).
"""
import json
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load_cfg(name):
    return np.load(os.path.join(GOLD, name))["cells12"].astype(np.int32)


def test_philox_known_answers(oracle_mod):
    O = oracle_mod
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert list(O.philox(ctr, key)) == want


def test_distances_match_reference_file(oracle_mod):
    d, f = oracle_mod.distances(32, 6.0)
    lines = open(os.path.join(GOLD, "distances_L32_Rc6.txt")).read().splitlines()
    assert lines[0].split() == ["32", "32", "32"]
    mine = ["%f %d" % (a, b) for a, b in zip(d, f)]
    assert mine == lines[1:]


@pytest.mark.parametrize("L", [4, 6, 8, 10])
def test_distances_small_lattices_follow_reference_rules(oracle_mod, L):
    # counts are halved with integer division then scaled by N (GW:912-915)
    d, f = oracle_mod.distances(L, 6.0)
    N = L ** 3
    assert np.all(f % N == 0)
    assert len(set(d.tolist())) == len(d)
    assert np.all(d < 6.0)


@pytest.mark.parametrize("name", ["input_config_L32.npz", "config_out_L32.npz"])
def test_reference_config_roundtrip_and_invariants(oracle_mod, name):
    cfg = load_cfg(name)
    assert cfg.shape == (32768, 12)
    eta = cfg[:, 6:]
    assert np.all(eta.sum(1) == 4)  # four active arms per cell (chessboard rule)
    o = oracle_mod.Oracle(32, 0.815, 0.45, 44648604, 6.0, 0, 1)
    o.set_config(cfg)
    assert np.array_equal(o.get_config(), cfg)
    # both ends of every bond carry the same eta
    L = 32
    idx = np.arange(L ** 3)
    x, y, z = idx % L, (idx // L) % L, idx // (L * L)
    nb = [((x + 1) % L) + L * (y + L * z), x + L * (((y + 1) % L) + L * z), x + L * (y + L * ((z + 1) % L))]
    for d in range(3):
        assert np.array_equal(eta[:, 2 * d], eta[nb[d], 2 * d + 1])


def test_config_out_observables_decompose(oracle_mod):
    # GW:2138-2150: e = E_vdW - J_hb N_hb - J_s N_s, v = N r^3 + v_hb N_hb, h = e + P v
    o = oracle_mod.Oracle(32, 0.815, 0.45, 1, 6.0, 0, 1)
    o.set_config(load_cfg("config_out_L32.npz"))
    ob = o.measure()
    assert ob.n_hb2 % 2 == 0
    e = ob.e_vdw - 0.5 * ob.n_hb - float(np.float32(0.08)) * ob.n_sigma
    assert ob.energy == pytest.approx(e, rel=1e-14)
    assert ob.v_total == pytest.approx(32768 * 1.0001 ** 3 + float(np.float32(0.6)) * ob.n_hb, rel=1e-14)
    assert ob.enthalpy == pytest.approx(ob.energy + float(np.float32(0.45)) * ob.v_total, rel=1e-14)
    assert ob.m == pytest.approx(ob.n_sigma / (15 * 32768))
    # the sample run's final configuration sits at the sample run's statistics
    stats = json.load(open(os.path.join(GOLD, "data_out_stats.json")))["columns"]
    assert abs(ob.n_hb - stats["n_hb"]["mean"]) < 5 * stats["n_hb"]["std"]
    assert abs(ob.m - stats["m"]["mean"]) < 5 * stats["m"]["std"]


def test_own_exp_log_accuracy(oracle_mod):
    lib = oracle_mod.lib()
    rng = np.random.default_rng(1)
    for x in np.concatenate([rng.uniform(-700, 700, 2000), rng.uniform(-1, 1, 2000)]):
        v = lib.oracle_exp(float(x))
        assert v == pytest.approx(math.exp(x), rel=4e-16)
    for x in np.concatenate([rng.uniform(1e-300, 1e300, 500), rng.uniform(0.9, 1.1, 2000), [1.0]]):
        v = lib.oracle_log(float(x))
        assert v == pytest.approx(math.log(x), rel=4e-16, abs=4e-16)


def test_thresholds(oracle_mod):
    o = oracle_mod.Oracle(8, 0.7, 0.45, 1, 6.0, 0, 0)
    s, c, w = o.thresholds()
    beta = 1.0 / float(np.float32(0.7))
    jeff = float(np.float32(np.float32(0.5) - np.float32(0.45) * np.float32(0.6)))
    js = float(np.float32(0.08))
    for dhb in (-1, 0, 1):
        for dns in range(-5, 6):
            de = -jeff * dhb - js * dns
            p = min(1.0, math.exp(-beta * de))
            want = 1 << 32 if p >= 1 else int(math.floor(p * 2 ** 32 + 0.5))
            assert int(s[(dhb + 1) * 11 + dns + 5]) == want
    assert int(c[4]) == 1 << 32 and int(c[5]) == 1 << 32 and int(c[3]) < 1 << 32
    assert 0 < int(w[0]) < 1 << 32 and 0 < int(w[1]) < 1 << 32


def test_cube_states_are_two_factors(oracle_mod):
    # every state of every cube gives each of its 8 vertices exactly two active edges, so each
    # cell ends with 4 active arms (CB:415-476)
    for start in (0, 2):
        o = oracle_mod.Oracle(8, 0.7, 0.45, 7 + start, 6.0, 0, start)
        for _ in range(3):
            cfg = o.get_config()
            assert np.all(cfg[:, 6:].sum(1) == 4)
            assert cfg[:, :6].max() <= 5
            o.step(1, 1)


def test_ordered_start_is_ordered(oracle_mod):
    o = oracle_mod.Oracle(8, 0.7, 0.45, 3, 6.0, 0, 2)
    s = o.get_config()[:, :6]
    assert np.all(s == s[0, 0])


def test_sw_labels_are_canonical_minimum(oracle_mod):
    o = oracle_mod.Oracle(6, 0.6, 0.45, 11, 6.0, 0, 0)
    o.step(0, 1)
    lab = o.labels()
    N = 6 ** 3
    assert lab.shape == (6 * N,)
    assert np.all(lab <= np.arange(6 * N))
    assert np.all(lab[lab] == lab)  # labels are roots
    cs = o.cluster_stats()
    sizes = np.bincount(lab, minlength=6 * N)
    sizes = sizes[sizes > 0]
    assert cs.n_clusters == len(sizes)
    assert cs.largest == sizes.max()
    assert cs.sum_size2 == int((sizes.astype(np.int64) ** 2).sum())


def test_no_sw_cluster_stats_match_reference_cluster_out(oracle_mod):
    # SOURCE/cluster.out with Cluster_Steps=0: labels never set, one cluster of 6N sites
    o = oracle_mod.Oracle(32, 0.815, 0.45, 1, 6.0, 0, 0)
    cs = o.cluster_stats()
    line = open(os.path.join(GOLD, "cluster_out_head.txt")).readline().split()
    n = cs.n_clusters
    avg = np.float32(cs.sum_size) / np.float32(n)
    avg2 = np.float32(cs.sum_size2_wrap32) / np.float32(n) - avg * avg
    mine = "%d %d %d %d %f %f %d" % (0, cs.largest, cs.second, cs.n_percolating, avg, avg2, n)
    assert mine.split() == line


def test_statistics_match_reference_data_out(oracle_mod):
    """Oracle at the sample run's state point vs the reference's own data.out: every observable
    within 2 combined standard errors (10-block errors of this run and of the reference's run)."""
    stats = json.load(open(os.path.join(GOLD, "data_out_stats.json")))["columns"]
    o = oracle_mod.Oracle(32, 0.815, 0.45, 44648604, 6.0, 0, 1, threads=os.cpu_count() or 1)
    o.set_config(load_cfg("input_config_L32.npz"))
    for _ in range(1000):
        o.step(1, 0)
    obs = {k: [] for k in ("e", "v", "n_hb", "m", "r_cell")}
    for i in range(4000):
        o.step(1, 0)
        if i % 10 == 0:
            ob = o.measure()
            obs["e"].append(ob.energy)
            obs["v"].append(ob.v_total)
            obs["n_hb"].append(ob.n_hb)
            obs["m"].append(ob.m)
            obs["r_cell"].append(ob.r_cell)
    for k, xs in obs.items():
        xs = np.asarray(xs)
        b = xs.reshape(10, -1).mean(1)
        err = b.std(ddof=1) / np.sqrt(10)
        z = (xs.mean() - stats[k]["mean"]) / math.hypot(err, stats[k]["block_err"])
        assert abs(z) < 2.0, (k, xs.mean(), stats[k]["mean"], z)
