"""The reference's own host arrays as the transfer format: s[arm*N + cell] and
active_bond[arm*N + cell], one byte each (GW:1135-1137 copy them to the device, GW:1298 copies s
back). cvf_set_arms / cvf_get_arms must agree with the cells12 path value for value, load a
state the oracle then continues bit for bit, reject bad values without touching the lattice, and
give the same results through the host path (io mode 0), from unaligned arrays and in the
nhb<=4 mode."""
import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def _to_arms(c12):
    """cells12 (N, 12) -> (s, active_bond), arm-major."""
    return np.ascontiguousarray(c12[:, :6].T.reshape(-1).astype(np.uint8)), \
        np.ascontiguousarray(c12[:, 6:].T.reshape(-1).astype(np.uint8))


@pytest.mark.parametrize("io_mode", [1, 0])
def test_arms_round_trip_and_parity(engine_lib, oracle_mod, io_mode):
    L = 16
    ora = oracle_mod.Oracle(L, 0.7, 0.45, 321, 6.0, 0, 0)
    ora.step(1, 0)
    s, ab = _to_arms(ora.get_config())
    eng = Lattice(Params(L=L, T=0.7, P=0.45, seed=321, start=1))
    if io_mode == 0 or abi.lib().cvf_set_io_mode(eng._h, 1) != 0:
        assert abi.lib().cvf_set_io_mode(eng._h, 0) == 0
    eng.set_arms(s, ab)
    r, v, _, ctr = ora.state()
    eng.set_state(r, v, ctr)
    assert np.array_equal(eng.get_config(), ora.get_config())
    gs, gab = eng.get_arms()
    assert np.array_equal(gs, s) and np.array_equal(gab, ab)
    eng.run(3, 1, 0)
    for _ in range(3):
        ora.step(1, 0)
    s2, ab2 = eng.get_arms()
    want_s, want_ab = _to_arms(ora.get_config())
    assert np.array_equal(s2, want_s) and np.array_equal(ab2, want_ab)
    # a bad sigma is rejected and leaves the lattice as it was
    bad = s2.copy()
    bad[5 * L ** 3 + 17] = 6
    before = eng.get_config()
    rc = abi.lib().cvf_set_arms(eng._h, 0, bad.ctypes.data, ab2.ctypes.data, bad.size)
    assert rc == -5 and b"cell 17" in engine_lib.cvf_last_error_string()
    assert np.array_equal(eng.get_config(), before)
    eng.close()


@pytest.mark.parametrize("L,shift", [(12, 0), (12, 4), (12, 1), (6, 0)])
def test_arms_access_widths(engine_lib, oracle_mod, L, shift):
    """16-byte rows (aligned arrays, N a multiple of 16), 4-byte rows (4-byte aligned, or N = 216)
    and single bytes (arrays one byte past a word boundary) give the same lattice."""
    ora = oracle_mod.Oracle(L, 0.7, 0.45, 55 + L, 6.0, 0, 0)
    s, ab = _to_arms(ora.get_config())
    bs = np.zeros(s.size + 16, dtype=np.uint8)
    bab = np.zeros(ab.size + 16, dtype=np.uint8)
    off = (-bs.ctypes.data) % 16 + shift
    offb = (-bab.ctypes.data) % 16 + shift
    bs[off:off + s.size] = s
    bab[offb:offb + ab.size] = ab
    eng = Lattice(Params(L=L, T=0.7, P=0.45, seed=55 + L, start=1))
    assert abi.lib().cvf_set_arms(eng._h, 0, bs.ctypes.data + off, bab.ctypes.data + offb, s.size) == 0
    assert np.array_equal(eng.get_config(), ora.get_config())
    bs[:] = 9
    bab[:] = 9
    assert abi.lib().cvf_get_arms(eng._h, 0, bs.ctypes.data + off, bab.ctypes.data + offb, s.size) == 0
    assert np.array_equal(bs[off:off + s.size], s) and np.array_equal(bab[offb:offb + ab.size], ab)
    assert (bs[:off] == 9).all() and (bs[off + s.size:] == 9).all()  # nothing written outside
    eng.close()


def test_arms_nhb_mode(engine_lib, oracle_mod):
    L = 12
    # Flag_chessboard = 0 keeps eta as given
    ora = oracle_mod.Oracle(L, 0.7, 0.45, 56, 6.0, 0, 0, flag_chessboard=0)
    eng = Lattice(Params(L=L, T=0.7, P=0.45, seed=56, start=1, flag_chessboard=0))
    c12 = ora.get_config()
    c12[::7, 6] = 0
    ora.set_config(c12)
    eng.set_arms(*_to_arms(c12))
    assert np.array_equal(eng.get_config(), ora.get_config())
    eng.run(2, 1, 0)
    ora.step(1, 0)
    ora.step(1, 0)
    assert np.array_equal(eng.get_arms()[0], _to_arms(ora.get_config())[0])
    eng.close()


def test_arms_batch_replica_and_sizes(engine_lib, oracle_mod):
    """A batch replica takes its own arrays; a wrong size is CVF_EINVAL."""
    specs = [(8, 0.7), (12, 0.6)]
    eng = Lattice([Params(L=L, T=T, P=0.45, seed=600 + i, start=1, replica=i) for i, (L, T) in enumerate(specs)])
    ora = oracle_mod.Oracle(12, 0.6, 0.45, 601, 6.0, 1, 0)
    s, ab = _to_arms(ora.get_config())
    eng.set_arms(s, ab, r=1)
    assert np.array_equal(eng.get_config(1), ora.get_config())
    got = eng.get_arms(1)
    assert np.array_equal(got[0], s) and np.array_equal(got[1], ab)
    assert abi.lib().cvf_set_arms(eng._h, 1, s.ctypes.data, ab.ctypes.data, s.size - 1) == -1
    assert abi.lib().cvf_get_arms(eng._h, 0, s.ctypes.data, ab.ctypes.data, s.size) == -1  # replica 0 is L=8
    eng.close()
