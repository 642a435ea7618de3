"""The allocation-free cluster-statistics entry point (cvf_cluster_stats_noalloc).

Callers that cannot call cudaMalloc -- code running during CUDA graph capture, processes whose
device memory belongs to another allocator or a capped pool -- use this entry point: its work
space is a fixed array inside the library. These tests check it against the allocating entry
point (cvf_cluster_stats) on two calls in a row, so stale contents of the shared array from the
first call would show up in the second, and that sizes beyond the fixed limit are refused.
"""
import ctypes as C

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from cvfbulkwater_gb300.engine import Lattice, Params


def test_noalloc_rejects_sizes_beyond_limit(engine_lib):
    # validated before any CUDA call, so this runs without a GPU
    rc = engine_lib.cvf_cluster_stats_noalloc(C.c_void_p(16), 56, C.c_void_p(16), None)
    assert rc == -1
    assert b"exceed" in engine_lib.cvf_last_error_string()
    assert engine_lib.cvf_cluster_stats_noalloc(None, 16, C.c_void_p(16), None) == -1


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice(engine_lib):
    import torch

    lat = Lattice(Params(L=16, T=0.6, P=0.45, seed=20261203, start=0))
    stream = torch.cuda.current_stream()
    for call in range(2):
        lat.run(2 + call, 1, 1)  # Swendsen-Wang steps produce fresh labels
        labels = lat.labels()
        want = lat.cluster_stats()
        d_lab = torch.from_numpy(labels).to("cuda")
        d_out = torch.full((7,), -7, dtype=torch.int64, device="cuda")
        rc = engine_lib.cvf_cluster_stats_noalloc(C.c_void_p(d_lab.data_ptr()), 16, C.c_void_p(d_out.data_ptr()),
                                                  C.c_void_p(stream.cuda_stream))
        assert rc == 0, engine_lib.cvf_last_error_string()
        stream.synchronize()
        got = d_out.cpu().numpy().tolist()
        assert got == [want.largest, want.second, want.n_percolating, want.n_clusters, want.sum_size,
                       want.sum_size2, want.sum_size2_wrap32], (call, got)
        assert want.n_clusters > 1
