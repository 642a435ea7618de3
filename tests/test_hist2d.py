"""Binned 2-D histogram reweighting oracle (oracle/hist2d.py), CPU checks. Its parity with the
reference's F90 is unpinned (no Fortran compiler here, no simulation archive); these tests check
the restatement's own invariants: bin layout formulas, unit-normalised reweighted grids, the
Binder limit 1 - <m^4>/(3<m^2>^2) -> 2/3 for distributions narrow around a nonzero value, and the
Ising comparisons' known answers (the 3-D fit has unit norm and variance, a histogram equal to
it scores 0). The library's host-side Ising comparison (cvf_h2d_ising) must equal the oracle's;
it needs no GPU."""
import math

import numpy as np
import pytest

from oracle import hist2d as O
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
    # relative widths ~0.01 put the cumulants within a few 1e-4 of the narrow limit 2/3
    assert abs(be - 2 / 3) < 3e-4 and abs(br - 2 / 3) < 3e-4
    x, q, a1, media = o.mixed(g, 0.3)
    w = np.gradient(x)
    assert np.isclose((q * w).sum(), 1.0, atol=0.05)
    assert abs(H2D.binder_mixed(x, q, a1, media) - 2 / 3) < 1e-3


def test_f90_literals_are_single_precision():
    # Ts = 140.5678 assigned to a real*8 from a default-kind literal
    assert O.TS == 140.56779479980469 and O.TS != 140.5678
    assert O.VIS == 7.5


def test_ising_fits_known_answers():
    z = np.linspace(-8, 8, 160001)
    i3 = np.array([O.ising3d(v) for v in z])
    dz = z[1] - z[0]
    assert abs(i3.sum() * dz - 1) < 1e-6 and abs((z * z * i3).sum() * dz - 1) < 1e-6
    p2, p3 = O.ising_peaks()
    # the 3-D search stops once the two probes differ by less than 1e-6 (F90:1211), short of the top
    assert p3 <= max(i3) and p3 == pytest.approx(max(i3), rel=1e-4)
    assert p2 == pytest.approx(max(O.ising2d(v) for v in np.linspace(0.1, 2, 20001)), rel=1e-6)
    # a histogram equal to the 3-D fit: no Liu-Panagiotopoulos distance, no KL divergence
    x = np.linspace(-3, 3, 61)
    q = np.array([O.ising3d(v) for v in x])
    liu2, liu3, kl2, kl3, zero, height = O.confront(x, q)
    assert liu3 == 0.0 and kl3 == 0.0 and liu2 > 0
    assert zero == pytest.approx(x[30] ** 2 + 0.0, abs=1e-12)  # the minimum in (-1, 1) sits at 0
    assert height < 0.01


def test_library_ising_compare_equals_oracle(engine_lib):
    from cvfbulkwater_gb300.analysis import ising_compare
    rng = np.random.default_rng(3)
    for B in (1.0, 1.07):
        x = np.sort(rng.uniform(-2.5, 2.5, 48))
        q = np.abs(rng.normal(0.3, 0.2, 48))
        q[5] = 0.0
        got = ising_compare(x, q, B)
        want = O.confront(B * x, q)
        assert list(got.values()) == pytest.approx(list(want), rel=1e-12, abs=1e-15)
    # no bin in (-1, 1), nothing on one side: the F90's fallback values
    got = ising_compare(np.array([1.5, 2.0, 2.5]), np.array([0.2, 0.5, 0.1]))
    assert got["zero"] == 1e3 and got["height"] == 1e3
