"""Configuration transfers in both modes: kernels reading and writing the caller's cells12 array in host memory
(io_mode 1, GPUs with pageable-memory access) and host packing with a copy (io_mode 0).
Lattices, read-back cells12 arrays and error reports must be identical, for power-of-two and
other edges, aligned and unaligned caller arrays."""
import numpy as np
import pytest

from cvfbulkwater_gb300.abi import CvfError
from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def capable():
    lat = Lattice(Params(L=4, T=0.8, P=0.45, seed=1, start=0))
    ok = lat.io_mode == 1
    lat.close()
    return ok


def random_config(L, seed):
    """A valid cells12 array: run a few steps on the engine from a disordered start."""
    lat = Lattice(Params(L=L, T=0.75, P=0.3, seed=seed, start=0))
    lat.io_mode = 0
    lat.run(3, 1, 0)
    cfg = lat.get_config()
    lat.close()
    return cfg


@pytest.fixture(scope="module")
def io_capable(engine_lib):
    if not capable():
        pytest.skip("GPU cannot access pageable host memory")
    return True


@pytest.mark.parametrize("L", [4, 6, 10, 16, 24, 64])
def test_modes_round_trip(io_capable, L):
    cfg = random_config(L, 100 + L)
    outs = {}
    for set_mode in (0, 1):
        for get_mode in (0, 1):
            lat = Lattice(Params(L=L, T=0.75, P=0.3, seed=7, start=1))
            lat.io_mode = set_mode
            lat.set_config(cfg)
            lat.io_mode = get_mode
            got = lat.get_config()
            assert np.array_equal(got, cfg), (set_mode, get_mode)
            lat.run(2, 1, 0)
            outs[(set_mode, get_mode)] = lat.get_config()
            lat.close()
    first = outs[(0, 0)]
    for k, v in outs.items():
        assert np.array_equal(v, first), k


def test_unaligned_caller_arrays(io_capable):
    L = 8
    cfg = random_config(L, 5)
    N = L ** 3
    raw = np.zeros(N * 12 + 1, dtype=np.int32)
    view = raw[1:].reshape(N, 12)  # 4-byte offset: not 16-byte aligned
    view[...] = cfg
    assert view.ctypes.data % 16 != 0
    lat = Lattice(Params(L=L, T=0.75, P=0.3, seed=7, start=1))
    lat.io_mode = 1
    lat.set_config(view)
    raw2 = np.zeros(N * 12 + 1, dtype=np.int32)
    out = raw2[1:].reshape(N, 12)
    lat.get_config(out=out)
    assert np.array_equal(out, cfg)


@pytest.mark.parametrize("field,value", [(2, 6), (5, -1), (8, 2), (11, -3)])
def test_invalid_values_same_error_and_lattice_unchanged(io_capable, field, value):
    L = 6
    cfg = random_config(L, 11)
    bad = cfg.copy()
    bad[37, field] = value
    bad[150, 0] = 9  # a later bad cell: the first one is reported
    msgs = []
    for mode in (0, 1):
        lat = Lattice(Params(L=L, T=0.75, P=0.3, seed=7, start=1))
        lat.io_mode = mode
        lat.set_config(cfg)
        with pytest.raises(CvfError) as ei:
            lat.set_config(bad)
        msgs.append((ei.value.code, str(ei.value)))
        assert np.array_equal(lat.get_config(), cfg), mode
        lat.close()
    assert msgs[0] == msgs[1]
    assert "line 37" in msgs[1][1]
