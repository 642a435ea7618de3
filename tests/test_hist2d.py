"""Binned 2-D histogram reweighting oracle (oracle/hist2d.py), CPU checks. Its parity with the
reference's F90 is unpinned (no Fortran compiler here, no simulation archive); these tests check
the restatement's own invariants: bin layout formulas, unit-normalised reweighted grids, and the
Binder limit 1 - <m^4>/(3<m^2>^2) -> 2/3 for distributions narrow around a nonzero value."""
import math

import numpy as np

from oracle.hist2d import H2D


def synthetic(n=3000, seed=0):
    rng = np.random.default_rng(seed)
    That = np.array([0.72, 0.74, 0.76, 0.78])
    h, rho, run = [], [], []
    for j, t in enumerate(That):
        h.append(-1.2 + (t - 0.72) * 2 + 0.02 * rng.standard_normal(n))
        rho.append(0.62 - (t - 0.72) * 0.5 + 0.005 * rng.standard_normal(n))
        run.append(np.full(n, j))
    return np.concatenate(h), np.concatenate(rho), np.concatenate(run), That, np.full(4, 0.45)


def test_bin_layout():
    h, rho, run, That, Phat = synthetic()
    o = H2D(h, rho, run, That, Phat, 8, 0.2)
    n_bin = int(math.sqrt(3000) / 2) + 20
    assert o.nb == int(n_bin * 10 * 0.2)
    assert np.isclose(o.hsum.sum() * o.dE * o.dD, 4.0)  # four runs, each normalised to 1


def test_reweighted_grid_and_binder_limits():
    h, rho, run, That, Phat = synthetic()
    o = H2D(h, rho, run, That, Phat, 8, 0.2)
    g, mask = o.reweighted(0.75, 0.45)
    assert np.isclose(g.sum() * o.dE * o.dD, 1.0)
    be, br = o.binder_e_rho(g, mask)
    assert abs(be - 2 / 3) < 1e-4 and abs(br - 2 / 3) < 1e-4
    x, q, a1, media = o.mixed(g, 0.3)
    w = np.gradient(x)
    assert np.isclose((q * w).sum(), 1.0, atol=0.05)
    assert abs(H2D.binder_mixed(x, q, a1, media) - 2 / 3) < 1e-3
