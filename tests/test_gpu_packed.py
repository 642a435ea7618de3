"""Packed-state export and import (cvf_get_packed / cvf_set_packed).

The packed state is the engine's device layout (colour-split sigma words, then the even- and
odd-origin cube states): 4.25 bytes per cell against the 48 of the config.out order. A state
saved with cvf_get_packed and cvf_get_state and loaded into a fresh handle resumes the chain
exactly; invalid values are refused without touching the lattice.
"""
import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu


def decode_sigma(buf, L):
    """sigma[cell, arm] from a packed buffer (cell = x + L*(y + L*z))."""
    H, N = L // 2, L ** 3
    words = buf[: 4 * N].view(np.uint32)
    col = [words[: N // 2], words[N // 2:]]
    x, y, z = np.meshgrid(np.arange(L), np.arange(L), np.arange(L), indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    cell = x + L * (y + L * z)
    c = (x + y + z) & 1
    idx = (x >> 1) + H * (y + L * z)
    w = np.where(c == 0, col[0][idx], col[1][idx])
    out = np.zeros((N, 6), dtype=np.int64)
    for a in range(6):
        out[cell, a] = (w >> (3 * a)) & 7
    return out


@pytest.mark.parametrize("L", [8, 12, 64])
def test_packed_round_trip_resumes_exactly(engine_lib, L):
    a = Lattice(Params(L=L, T=0.7, P=0.45, seed=77, start=0))
    a.run(6, 1, 1)
    buf = a.get_packed()
    assert buf.size == 4 * L ** 3 + 2 * (L // 2) ** 3
    cfg = a.get_config()
    assert np.array_equal(decode_sigma(buf, L), cfg[:, :6])
    st = a.state()
    b = Lattice(Params(L=L, T=0.7, P=0.45, seed=77, start=1))
    b.set_packed(buf)
    b.set_state(st[0], st[1], st[3])
    assert np.array_equal(b.get_config(), cfg)
    a.run(5, 1, 0)
    b.run(5, 1, 0)
    assert np.array_equal(a.get_config(), b.get_config())
    assert np.array_equal(a.get_packed(), b.get_packed())
    oa, ob = a.observables(), b.observables()
    assert (oa.n_hb2, oa.n_sigma, oa.r_cell) == (ob.n_hb2, ob.n_sigma, ob.r_cell)


def test_packed_rejects_invalid_values(engine_lib):
    L = 8
    a = Lattice(Params(L=L, T=0.7, P=0.45, seed=5, start=0))
    good = a.get_packed()
    cfg = a.get_config()
    bad = good.copy()
    words = bad[: 4 * L ** 3].view(np.uint32)
    words[13] = (words[13] & ~np.uint32(7 << 9)) | np.uint32(6 << 9)  # sigma_3 = 6
    with pytest.raises(abi.CvfError, match="word 13"):
        a.set_packed(bad)
    bad = good.copy()
    bad[: 4 * L ** 3].view(np.uint32)[3] |= np.uint32(1 << 20)  # a bit above the six fields
    with pytest.raises(abi.CvfError, match="word 3"):
        a.set_packed(bad)
    bad = good.copy()
    bad[4 * L ** 3 + 5] = 9  # an even-origin cube state out of range
    with pytest.raises(abi.CvfError, match="cube byte 5"):
        a.set_packed(bad)
    with pytest.raises(abi.CvfError):
        a.set_packed(good[:-1])
    assert np.array_equal(a.get_config(), cfg)  # nothing was loaded
    a.set_packed(good)  # every sigma 0..5 (5 included) and cube state 0..8 loads
    assert np.array_equal(a.get_config(), cfg)
