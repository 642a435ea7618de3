"""The allocation-free cluster-statistics entry point (cvf_cluster_stats_noalloc).

Callers that cannot call cudaMalloc -- code running during CUDA graph capture, processes whose
device memory belongs to another allocator or a capped pool -- use this entry point: its work
space is a fixed array inside the library. These tests check it against the allocating entry
point (cvf_cluster_stats) on calls in a row, so stale contents of the shared array from an
earlier call would show up in a later one (a smaller lattice after a larger one included), that
an out-of-range label is reported, that the int32 wrap of s*s matches the oracle on a lattice
with a spanning cluster, and that sizes beyond the fixed limit are refused.
"""
import ctypes as C
import os

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params


@pytest.mark.parametrize("L", [56, 1000, 1200000, 2147483646])
def test_noalloc_rejects_sizes_beyond_limit(engine_lib, L):
    # validated before any CUDA call and before 6 L^3 is formed, so this runs without a GPU
    rc = engine_lib.cvf_cluster_stats_noalloc(C.c_void_p(16), L, C.c_void_p(16), None)
    assert rc == -1
    assert b"exceed" in engine_lib.cvf_last_error_string()


def test_noalloc_rejects_bad_arguments(engine_lib):
    assert engine_lib.cvf_cluster_stats_noalloc(None, 16, C.c_void_p(16), None) == -1
    assert engine_lib.cvf_cluster_stats_noalloc(C.c_void_p(16), 15, C.c_void_p(16), None) == -1
    assert engine_lib.cvf_cluster_stats_noalloc(C.c_void_p(16), -4, C.c_void_p(16), None) == -1


def _noalloc(engine_lib, labels, L):
    import torch

    stream = torch.cuda.current_stream()
    d_lab = torch.from_numpy(np.ascontiguousarray(labels, dtype=np.int32)).to("cuda")
    d_out = torch.full((7,), -7, dtype=torch.int64, device="cuda")
    rc = engine_lib.cvf_cluster_stats_noalloc(C.c_void_p(d_lab.data_ptr()), L, C.c_void_p(d_out.data_ptr()),
                                              C.c_void_p(stream.cuda_stream))
    assert rc == 0, engine_lib.cvf_last_error_string()
    stream.synchronize()
    return d_out.cpu().numpy().tolist()


def _as_list(cs):
    return [cs.largest, cs.second, cs.n_percolating, cs.n_clusters, cs.sum_size, cs.sum_size2, cs.sum_size2_wrap32]


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_in_a_row(engine_lib):
    """L = 16 twice, then L = 8: the smaller call after the larger ones must not see their
    sizes, candidates or coverage bitmaps."""
    big = Lattice(Params(L=16, T=0.6, P=0.45, seed=20261203, start=0))
    small = Lattice(Params(L=8, T=0.3, P=0.45, seed=5, start=2))
    for call, (lat, L) in enumerate([(big, 16), (big, 16), (small, 8)]):
        lat.run(2 + call, 1, 1)  # Swendsen-Wang steps produce fresh labels
        want = lat.cluster_stats()
        got = _noalloc(engine_lib, lat.labels(), L)
        assert got == _as_list(want), (call, got)
        assert want.n_clusters > 1


@pytest.mark.gpu
def test_noalloc_reports_out_of_range_label(engine_lib):
    lat = Lattice(Params(L=8, T=0.6, P=0.45, seed=11, start=0))
    lat.run(1, 0, 1)
    labels = lat.labels()
    labels[17] = labels.size  # 6N: one past the last site
    got = _noalloc(engine_lib, labels, 8)
    assert got[3] == -1
    # the next call on valid labels is unaffected
    assert _noalloc(engine_lib, lat.labels(), 8) == _as_list(lat.cluster_stats())


@pytest.mark.gpu
def test_noalloc_wrapped_size_squares_match_oracle(engine_lib, oracle_mod):
    """L = 48 ordered start at T = 0.1: one cluster of about 658 k sites, so the reference's int32
    accumulation of s*s wraps; the labels of the engine's Swendsen-Wang step give the oracle's
    statistics through the allocation-free entry point."""
    L = 48
    lat = Lattice(Params(L=L, T=0.1, P=0.45, seed=777, start=2))
    ora = oracle_mod.Oracle(L, 0.1, 0.45, 777, 6.0, 0, 2, threads=os.cpu_count() or 1)
    lat.run(1, 0, 1)
    ora.step(0, 1)
    want = ora.cluster_stats()
    assert want.largest > 46341 and want.sum_size2_wrap32 != want.sum_size2
    assert _noalloc(engine_lib, lat.labels(), L) == _as_list(want)
