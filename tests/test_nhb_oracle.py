"""Flag_chessboard = 0 (the nhb<=4 compatibility mode) in the oracle, CPU checks.

The bond count of every cell must stay equal to the number of its arms that agree with the arm
they face (every eta is 1 and the updates move both counts by the same step, GW:2006-2007), and
the reported N_hb must be the reference's typewriter-order count with the cap NHBMAX = 4
(GW:2064-2099), restated here independently in Python on small lattices."""
import numpy as np
import pytest

from oracle import oracle as O


def matched_counts(cfg, L):
    """Arms of every cell agreeing with the arm they face (cell = x + L*(y + L*z))."""
    s = cfg[:, :6].reshape(L, L, L, 6)  # [z, y, x, arm]
    m = np.zeros((L, L, L), dtype=np.int64)
    for a, (axis, step) in enumerate([(2, 1), (2, -1), (1, 1), (1, -1), (0, 1), (0, -1)]):
        nb = np.roll(s[..., a ^ 1], -step, axis=axis)
        m += s[..., a] == nb
    return m.reshape(-1)


def typewriter_hb2(cfg, L):
    """GW:2064-2099 as written: cells in index order, bonds x+, y+, z+, both counts below 4."""
    N = L ** 3
    s = cfg[:, :6]
    cnt = [0] * N
    hb2 = 0
    for i in range(N):
        x, y, z = i % L, (i // L) % L, i // (L * L)
        for d, nb in enumerate([(x + 1) % L + L * (y + L * z), x + L * ((y + 1) % L + L * z),
                                x + L * (y + L * ((z + 1) % L))]):
            if s[i, 2 * d] == s[nb, 2 * d + 1] and cnt[i] < 4 and cnt[nb] < 4:
                cnt[i] += 1
                cnt[nb] += 1
                hb2 += 2
    return hb2


@pytest.fixture(scope="module")
def om(oracle_mod):
    return oracle_mod


@pytest.mark.parametrize("L,start,T", [(4, 0, 0.6), (6, 0, 0.3), (4, 2, 0.5), (8, 0, 0.45)])
def test_bond_counts_follow_the_lattice(om, L, start, T):
    o = om.Oracle(L, T, 0.45, 77 + L, start=start, flag_chessboard=0)
    for _ in range(6):
        o.step(1, 0)
        cfg = o.get_config()
        assert (cfg[:, 6:] == 1).all()
        assert np.array_equal(o.nhb().astype(np.int64), matched_counts(cfg, L))


@pytest.mark.parametrize("L,start,T", [(4, 2, 0.3), (4, 0, 0.3), (6, 0, 0.25), (6, 2, 0.5)])
def test_greedy_bond_count(om, L, start, T):
    o = om.Oracle(L, T, 0.45, 5 + L, start=start, flag_chessboard=0)
    for k in range(4):
        cfg = o.get_config()
        got = o.measure().n_hb2
        assert got == typewriter_hb2(cfg, L)
        m = matched_counts(cfg, L)
        if (m < 5).all():
            assert got == m.sum()  # nothing to refuse: every matched bond counts
        else:
            assert got <= m.sum()
        o.step(1, 0)


def test_ordered_start_refuses_bonds(om):
    # every arm of every cell agrees: the cap of 4 must refuse bonds
    o = om.Oracle(4, 0.5, 0.45, 3, start=2, flag_chessboard=0)
    cfg = o.get_config()
    assert (matched_counts(cfg, 4) == 6).all()
    got = o.measure().n_hb2
    assert got == typewriter_hb2(cfg, 4) and got < 6 * 64


def test_config_eta_kept_and_counted(om):
    L = 4
    rng = np.random.default_rng(9)
    cfg = np.zeros((L ** 3, 12), dtype=np.int32)
    cfg[:, :6] = rng.integers(0, 6, (L ** 3, 6))
    cfg[:, 6:] = rng.integers(0, 2, (L ** 3, 6))
    o = om.Oracle(L, 0.6, 0.45, 1, start=1, flag_chessboard=0)
    o.set_config(cfg)
    assert np.array_equal(o.get_config(), cfg)
    s = cfg[:, :6].reshape(L, L, L, 6)
    e = cfg[:, 6:].reshape(L, L, L, 6)
    want = np.zeros((L, L, L), dtype=np.int64)
    for a, (axis, step) in enumerate([(2, 1), (2, -1), (1, 1), (1, -1), (0, 1), (0, -1)]):
        want += e[..., a] * (s[..., a] == np.roll(s[..., a ^ 1], -step, axis=axis))
    assert np.array_equal(o.nhb().astype(np.int64), want.reshape(-1))
