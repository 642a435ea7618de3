"""bench.py's multi-process path on CPU: two gloo ranks (127.0.0.1) agree on the barrier and the
max-over-ranks time, and each rank steps its own replica (independent lattices, no collective)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    got = d.max(float(10 + r))
    params = bench.replica_params(r)
    d.close()
    q.put((r, got, params.seed, params.replica, params.L))


@pytest.mark.timeout(120)
def test_two_rank_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=90) for _ in range(2))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [x[1] for x in res] == [11.0, 11.0]           # max over ranks
    assert [x[2] - res[0][2] for x in res] == [0, 1]      # seed + rank
    assert [x[3] for x in res] == [0, 1]                  # replica id = rank
    assert all(x[4] == 256 for x in res)
