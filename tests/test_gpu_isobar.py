"""Statistical pin on the reference's processed results: the density of the L=32 lattice along the
isobar P=0.45 (PROCESSED_DATA/CVF_isobars.tar.gz, L32_P0.45_density.dat: rho = N/<V> with its
error) is reproduced by the engine at T = 0.78, 0.80 and 0.82 within 2 combined standard errors
(blocking), from disordered starts run as one batch of replicas."""
import math
import os

import numpy as np
import pytest

from cvfbulkwater_gb300.engine import Lattice, Params

GOLD = os.path.join(os.path.dirname(__file__), "golden")
pytestmark = pytest.mark.gpu


def test_isobar_density(engine_lib):
    table = {round(t, 2): (rho, err) for t, rho, err in np.loadtxt(os.path.join(GOLD, "isobar_P0.45_density.txt"))}
    temps = [0.78, 0.80, 0.82]
    L, N = 32, 32 ** 3
    lat = Lattice([Params(L=L, T=t, P=0.45, seed=777 + i, start=0, replica=i) for i, t in enumerate(temps)])
    lat.run(6000, 1, 0)
    lat.run_sampled(40000, 1, 0, 10)
    for r, t in enumerate(temps):
        v = np.array([lat.sample_observables(s, r).v_total for s in lat.samples(r)])
        rho = N / v.mean()
        b = v.reshape(20, -1).mean(1)
        err = N * (b.std(ddof=1) / math.sqrt(20)) / v.mean() ** 2
        want, want_err = table[t]
        z = (rho - want) / math.hypot(err, want_err)
        assert abs(z) < 2.0, (t, rho, want, err, want_err, z)
    lat.close()
