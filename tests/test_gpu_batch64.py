"""The batched-replica workload as specified, every replica against the oracle.

64 replicas with L drawn from {16, 24, 32, 48, 64} (seeded), on the 8 x 8 grid of T in
[0.55, 0.95] and P in [0.0, 0.60], disordered starts from per-replica seeds, one Metropolis sweep
and one volume move per step: one handle steps them all (replica groups on parallel graph
branches, the autotuner's tile, row order and launch mode). After six steps, recorded every
third, every replica's lattice, volume state, counters and recorded counts equal the oracle's.
"""
import os

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def batch_specs():
    rng = np.random.default_rng(20261203)
    Ls = rng.choice([16, 24, 32, 48, 64], size=64)
    Ts = np.linspace(0.55, 0.95, 8)
    Ps = np.linspace(0.0, 0.60, 8)
    return [(int(Ls[i]), float(Ts[i % 8]), float(Ps[i // 8]), 44648604 + i) for i in range(64)]


def test_batch64_every_replica_matches_oracle(engine_lib, oracle_mod):
    specs = batch_specs()
    eng = Lattice([Params(L=L, T=T, P=P, seed=s, start=0, replica=i) for i, (L, T, P, s) in enumerate(specs)])
    eng.autotune()
    eng.run(3, 1, 0)
    eng.run_sampled(3, 1, 0, 2)
    threads = os.cpu_count() or 1
    for i, (L, T, P, s) in enumerate(specs):
        ora = oracle_mod.Oracle(L, T, P, s, 6.0, i, 0, threads=threads)
        rec = []
        for k in range(6):
            ora.step(1, 0)
            if k >= 3 and (k - 3) % 2 == 0:
                rec.append(ora.measure())
        assert np.array_equal(eng.get_config(i), ora.get_config()), f"replica {i} (L={L})"
        re_, ve, _, ke = eng.state(i)
        ro, vo, _, ko = ora.state()
        assert (re_, ve) == (ro, vo) and list(ke) == list(ko), i
        smp = eng.samples(i)
        assert len(smp) == len(rec) == 2
        for got, want in zip(smp, rec):
            assert (got["n_hb2"], got["n_sigma"], got["r_cell"]) == (want.n_hb2, want.n_sigma, want.r_cell), i
        ora.close()
    eng.close()
