"""The oracle's Wolff step (GW:2199-2357) pinned two ways, on the CPU.

1. An independent pure-Python restatement of one Wolff step on a small lattice -- pokes with a
   seed site and a shift in 1..5, clusters as connected components of the poke's bond graph
   (each bond its own Philox uniform), every site of a cluster shifted -- gives the oracle's
   lattice and statistics exactly.
2. Equilibrium: Wolff steps (with the cube and volume moves) sample the same NPT ensemble as
   Metropolis sweeps: the mean energy and volume per cell of the two chains agree within two
   combined standard errors (20 blocks of 1000 steps each, after 1000 steps), L=8, T=0.815,
   P=0.45 (the reference's sample run).
"""
import numpy as np

ST_POKE, ST_SHIFT, ST_BOND = 0x0A, 0x0B, 0x20


def _below(n, words, c0, c1, kind, key, replica, philox):
    thr = ((1 << 32) - n) % n
    for w in words:
        m = int(w) * n
        if (m & 0xffffffff) >= thr:
            return m >> 32
    for k in range(256):
        r = philox([c0, c1, 0x1000 | (kind << 8) | k, replica], key)
        m = int(r[0]) * n
        if (m & 0xffffffff) >= thr:
            return m >> 32
    return m >> 32


def _wolff_step_python(sig, eta, L, jeff, thr_sw, key, replica, P0, philox):
    """sig, eta: [6, N] arrays (arm, cell); returns the new sig, pokes, total, largest, P."""
    N = L ** 3
    NS = 6 * N
    sig = sig.copy()

    def cell_xyz(c):
        return c % L, (c // L) % L, c // (L * L)

    def nb(c, a):
        x, y, z = cell_xyz(c)
        d = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)][a]
        return (x + d[0]) % L + L * (((y + d[1]) % L) + L * ((z + d[2]) % L))

    pairs = [(a, b) for a in range(5) for b in range(a + 1, 6)]

    def link(owner, l, P):
        r = philox([owner, P & 0xffffffff, (ST_BOND + (l >> 2)) | ((P >> 32) << 8), replica], key)
        return int(r[l & 3]) < thr_sw[0 if l < 3 else 1]

    done, pokes, largest, P = 0, 0, 0, P0
    while done < NS:
        r = philox([P & 0xffffffff, P >> 32, ST_POKE, replica], key)
        seed = _below(NS, r[:3], P & 0xffffffff, P >> 32, ST_POKE, key, replica, philox)
        shift = 1 + _below(5, r[3:], P & 0xffffffff, P >> 32, ST_SHIFT, key, replica, philox)
        # all bonds of the poke, then the seed's component by union-find
        parent = list(range(NS))

        def find(a):
            while parent[a] != a:
                parent[a] = parent[parent[a]]
                a = parent[a]
            return a

        for c in range(N):
            for i, (a, b) in enumerate(pairs):
                if sig[a, c] == sig[b, c] and link(c, 3 + i, P):
                    parent[find(a * N + c)] = find(b * N + c)
            for d in range(3):
                o = nb(c, 2 * d)
                same = sig[2 * d, c] == sig[2 * d + 1, o]
                cond = (eta[2 * d, c] and same) if jeff > 0 else ((not same) if jeff < 0 else False)
                if cond and link(c, d, P):
                    parent[find(2 * d * N + c)] = find((2 * d + 1) * N + o)
        root = find(seed)
        members = [s for s in range(NS) if find(s) == root]
        for s in members:
            sig[s // N, s % N] = (sig[s // N, s % N] + shift) % 6
        done += len(members)
        pokes += 1
        largest = max(largest, len(members))
        P += 1
    return sig, pokes, done, largest, P


def test_oracle_wolff_equals_python_restatement(oracle_mod):
    L, T, P, seed = 4, 0.7, 0.45, 12345
    o = oracle_mod.Oracle(L, T, P, seed, 6.0, 3, 0)
    o.step(1, 0)  # a cube move, a volume move and a sweep first
    cfg = o.get_config()
    sig = cfg[:, :6].T.astype(np.int64)
    eta = cfg[:, 6:].T.astype(np.int64)
    _, _, sw = o.thresholds()
    key = [seed & 0xffffffff, seed >> 32]
    jeff = np.float32(0.5) - np.float32(P) * np.float32(0.6)
    want, pokes, total, largest, Pn = _wolff_step_python(sig, eta, L, float(jeff), [int(t) for t in sw], key, 3, 0,
                                                         oracle_mod.philox)
    o.wolff_step()
    got = o.get_config()[:, :6].T
    assert np.array_equal(got, want)
    assert o.wolff_stats() == (pokes, total, largest, Pn)


def _means(o, nmet, ncl, burn, n):
    for _ in range(burn):
        o.step(nmet, ncl)
    e = np.empty(n)
    v = np.empty(n)
    for i in range(n):
        o.step(nmet, ncl)
        m = o.measure()
        e[i] = m.energy
        v[i] = m.v_total
    return e, v


def _mean_err(x, blocks=20):
    b = x[: len(x) // blocks * blocks].reshape(blocks, -1).mean(axis=1)
    return b.mean(), b.std(ddof=1) / np.sqrt(blocks)


def test_wolff_samples_the_metropolis_ensemble(oracle_mod):
    L, T, P = 8, 0.815, 0.45
    met = oracle_mod.Oracle(L, T, P, 11, 6.0, 0, 0)
    wol = oracle_mod.Oracle(L, T, P, 11, 6.0, 0, 0)
    wol.set_wolff(True)
    e1, v1 = _means(met, 1, 0, 1000, 20000)
    e2, v2 = _means(wol, 0, 1, 1000, 20000)
    for a, b in ((e1, e2), (v1, v2)):
        (m1, s1), (m2, s2) = _mean_err(a), _mean_err(b)
        z = (m1 - m2) / np.hypot(s1, s2)
        assert abs(z) < 2.0, (m1, s1, m2, s2, z)
