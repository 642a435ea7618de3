"""Replica groups: a batch's Metropolis-only steps captured as one kernel chain per group of
replicas on parallel graph branches. Any grouping must leave the same lattices, counters,
volume chains, recorded samples and correlators as one chain for the whole batch."""
import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu

SPECS = [(6, 0.6, 0.0), (16, 0.9, 0.6), (24, 0.75, 0.3), (12, 0.55, 0.45), (40, 0.8, 0.2), (8, 0.7, 0.45),
         (16, 0.65, 0.1), (10, 0.85, 0.5), (32, 0.72, 0.4)]


def run(groups, corr):
    lat = Lattice([Params(L=L, T=T, P=P, seed=300 + i, start=0, replica=i) for i, (L, T, P) in enumerate(SPECS)])
    lat.replica_groups = groups
    assert lat.replica_groups == min(groups, len(SPECS)) if groups else lat.replica_groups == 4
    lat.run(5, 1, 0)
    if corr:
        lat.set_correlation(True)
    lat.run(35, 1, 0)
    lat.run_sampled(23, 2, 0, 4)
    out = []
    for r in range(len(SPECS)):
        item = [lat.get_config(r), lat.state(r), lat.samples(r)]
        if corr:
            item.append(lat.correlation(r))
        out.append(item)
    lat.close()
    return out


@pytest.mark.parametrize("corr", [False, True])
def test_groupings_identical(engine_lib, corr):
    ref = run(1, corr)
    for g in (0, 2, 3, 9):
        got = run(g, corr)
        for r, (a, b) in enumerate(zip(ref, got)):
            assert np.array_equal(a[0], b[0]), (g, r)
            assert a[1][0] == b[1][0] and a[1][1] == b[1][1] and list(a[1][3]) == list(b[1][3]), (g, r)
            assert len(a[2]) == len(b[2]) and all(x == y for x, y in zip(a[2], b[2])), (g, r)
            if corr:
                assert np.array_equal(a[3][0], b[3][0]) and np.array_equal(a[3][1], b[3][1]), (g, r)


def test_batch_run_and_sample_stream_exports(engine_lib):
    """cvf_batch_run steps a batch as cvf_run_steps does; cvf_sample_stream returns the records of
    cvf_get_samples."""
    import ctypes as C
    from cvfbulkwater_gb300 import abi
    specs = [(8, 0.6), (12, 0.8)]
    a = Lattice([Params(L=L, T=T, P=0.45, seed=70 + i, start=0, replica=i) for i, (L, T) in enumerate(specs)])
    b = Lattice([Params(L=L, T=T, P=0.45, seed=70 + i, start=0, replica=i) for i, (L, T) in enumerate(specs)])
    a.run(5, 1, 0)
    abi.check(abi.lib().cvf_batch_run(b._h, 5, 1, 0))
    for r in range(2):
        assert np.array_equal(a.get_config(r), b.get_config(r))
    a.run_sampled(6, 1, 0, 2)
    n = C.c_longlong()
    abi.check(abi.lib().cvf_sample_count(a._h, 1, C.byref(n)))
    buf = (abi.Sample * n.value)()
    got = C.c_longlong()
    abi.check(abi.lib().cvf_sample_stream(a._h, 1, buf, n.value, C.byref(got)))
    want = a.samples(1)
    assert got.value == len(want) == 3
    for k in range(3):
        assert (buf[k].n_hb2, buf[k].n_sigma, buf[k].r_cell, buf[k].volume) == tuple(want[k].tolist())
    a.close()
    b.close()


SMALL = [(6, 0.6, 0.0), (16, 0.9, 0.6), (24, 0.75, 0.3), (12, 0.55, 0.45), (8, 0.7, 0.45)]


def test_cluster_chunks_match_grouped_chains(engine_lib):
    """An ungrouped batch whose lattices all hold at most 2^14 cells runs each chunk of plain
    steps as one thread-block cluster per replica, with the volume moves on a side branch; a
    grouped batch runs the per-phase kernels. Both leave the same lattices, counters and volume
    chains, across chunks of several sweeps and a sampled run between them."""
    outs = []
    for groups in (1, 2):
        lat = Lattice([Params(L=L, T=T, P=P, seed=500 + i, start=0, replica=i) for i, (L, T, P) in enumerate(SMALL)])
        lat.replica_groups = groups
        lat.run(37, 1, 0)
        lat.run(5, 2, 0)
        lat.run_sampled(6, 1, 0, 3)
        lat.run(33, 1, 0)
        outs.append([(lat.get_config(r), lat.state(r), lat.samples(r)) for r in range(len(SMALL))])
        lat.close()
    for r, (a, b) in enumerate(zip(*outs)):
        assert np.array_equal(a[0], b[0]), r
        assert a[1][0] == b[1][0] and a[1][1] == b[1][1] and list(a[1][3]) == list(b[1][3]), r
        assert len(a[2]) == len(b[2]) and all(x == y for x, y in zip(a[2], b[2])), r
