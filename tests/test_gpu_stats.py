"""Run statistics on the GPU (the awk stage of the reference's isobar analysis,
TA/script_analisi.sh:35) against the oracle's restatement on the same samples: the per-sample
data.out columns come from the host's cvf_sample_observables, the sums from oracle/isobar.py.
Means agree to 1e-12 relative, variances to 1e-12 of <x^2> (the sums run in another order)."""
import numpy as np
import pytest

from cvfbulkwater_gb300 import analysis
from cvfbulkwater_gb300.engine import Lattice, Params
from oracle import isobar as I

pytestmark = pytest.mark.gpu


def host_columns(lat, r):
    rows = []
    for s in lat.samples(r):
        o = lat.sample_observables(s, r)
        rows.append([o.energy, o.enthalpy, o.v_total, o.n_hb, o.m, o.r_cell])
    return np.array(rows)


def assert_stats_equal(got, cols):
    mean, var, n = I.run_stats(cols)
    assert got["n"] == n
    sq = np.mean(cols * cols, axis=0)
    for k in range(6):
        assert abs(got["mean"][k] - mean[k]) <= 1e-12 * max(abs(mean[k]), 1e-300), (k, got["mean"][k], mean[k])
        assert abs(got["var"][k] - var[k]) <= 1e-12 * sq[k] + 1e-300, (k, got["var"][k], var[k])


def test_run_statistics_match_oracle(engine_lib):
    specs = [(8, 0.70, 0.45), (12, 0.80, 0.10), (16, 0.65, 0.60)]
    lat = Lattice([Params(L=L, T=T, P=P, seed=31 + i, start=0, replica=i) for i, (L, T, P) in enumerate(specs)])
    lat.run(200, 1, 0)
    lat.run_sampled(3000, 1, 0, 3)
    rows = lat.run_statistics()
    assert len(rows) == 3
    for r, (L, T, P) in enumerate(specs):
        got = rows[r]
        assert got["L"] == L and got["T"] == pytest.approx(T) and got["P"] == pytest.approx(P)
        cols = host_columns(lat, r)
        assert len(cols) == 1000
        assert_stats_equal(got, cols)
        point = analysis.isobar_point(got)
        want = I.isobar_point(L, got["T"], np.array(got["mean"]), np.array(got["var"]), got["n"])
        for k in want:
            assert point[k] == float(want[k])
        si = analysis.to_si(point, got["P"])
        assert si["T_K"] == pytest.approx(got["T"] * I.TS + I.TI)


def test_run_statistics_capacity_and_empty(engine_lib):
    from cvfbulkwater_gb300.abi import CvfError
    lat = Lattice([Params(L=8, T=0.75, P=0.45, seed=5, start=0, replica=0, sample_capacity=10),
                   Params(L=8, T=0.75, P=0.45, seed=6, start=0, replica=1)])
    rows = lat.run_statistics()
    assert rows[0]["n"] == 0 and rows[1]["n"] == 0
    lat.run_sampled(10, 1, 0, 1)
    rows = lat.run_statistics()
    assert rows[0]["n"] == 10 and rows[1]["n"] == 10
    assert_stats_equal(rows[0], host_columns(lat, 0))
    assert_stats_equal(rows[1], host_columns(lat, 1))
    assert lat.run_statistics() == rows  # fixed summation order
    lat.run_sampled(5, 1, 0, 1)  # replica 0 is full now
    with pytest.raises(CvfError) as ei:
        lat.run_statistics()
    assert "replica 0" in str(ei.value) and "overflowed" in str(ei.value)
