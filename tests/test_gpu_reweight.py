"""FP64 reweighting forward and adjoint kernels (cvf_reweight_forward / cvf_reweight_adjoint).

Checked against the numpy restatement in oracle/reweight.py, against central finite differences of
the forward kernel, against the fluctuation identities (C_P = beta^2 var(H), K_T = beta var(V)/<V>)
and, physically, against direct simulations: samples of five runs along the isobar P = 0.45
reweighted to a temperature between them reproduce a run made at that temperature.
"""
import ctypes as C
import math

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from oracle import reweight as RW

pytestmark = pytest.mark.gpu
IDS = {name: i for i, name in enumerate(RW.OBS)}


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def gpu_forward(samples, run_of, runs, f, theta, obs, n_cells, n_iter=300, tol=1e-10):
    s = np.ascontiguousarray(samples, dtype=np.float64)
    ro = np.ascontiguousarray(run_of, dtype=np.int32)
    rr = np.ascontiguousarray(runs, dtype=np.float64)
    ff = np.array(f, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    ids = np.array([IDS[o] for o in obs], dtype=np.int32)
    out = np.zeros(len(obs) + 1)
    rc = abi.lib().cvf_reweight_forward(0, P(s), P(ro), len(s), P(rr), len(rr), P(ff), n_iter, tol, n_cells, P(th),
                                        P(ids), len(ids), P(out))
    abi.check(rc)
    return out[:-1], out[-1], ff


def gpu_adjoint(samples, run_of, runs, f, theta, obs, n_cells, g):
    s = np.ascontiguousarray(samples, dtype=np.float64)
    ro = np.ascontiguousarray(run_of, dtype=np.int32)
    rr = np.ascontiguousarray(runs, dtype=np.float64)
    ff = np.array(f, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    ids = np.array([IDS[o] for o in obs], dtype=np.int32)
    gg = np.asarray(g, dtype=np.float64)
    out = np.zeros(5)
    abi.check(abi.lib().cvf_reweight_adjoint(0, P(s), P(ro), len(s), P(rr), len(rr), P(ff), n_cells, P(th), P(ids),
                                             len(ids), P(gg), P(out)))
    return out


def synthetic(seed=7):
    """Four overlapping runs of a toy (E, V, N_hb, N_s) model; the estimator is defined for any samples."""
    rng = np.random.default_rng(seed)
    runs = np.array([[1.40, 0.40], [1.35, 0.45], [1.30, 0.45], [1.25, 0.50]])
    rows, run_of = [], []
    for j, (b, p) in enumerate(runs):
        n = 3000 + 500 * j
        nhb = rng.normal(900 - 40 * j, 12, n)
        ns = rng.normal(1400 - 30 * j, 15, n)
        E = -2000 - 0.5 * nhb - 0.08 * ns + rng.normal(0, 6, n)
        V = 560 + 0.6 * nhb * 0.1 + rng.normal(0, 3, n) + 10 * j
        rows.append(np.stack([E, V, nhb, ns], 1))
        run_of += [j] * n
    return np.concatenate(rows), np.array(run_of), runs


def test_forward_matches_numpy(engine_lib):
    s, ro, runs = synthetic()
    f_ref = RW.wham(s, ro, runs, n_iter=2000, tol=1e-12)
    theta = [1.32, 0.46, 0.0, 0.0, 0.0]
    obs = RW.OBS
    got, logz, f = gpu_forward(s, ro, runs, np.zeros(4), theta, obs, 512.0, n_iter=2000, tol=1e-12)
    assert np.allclose(f, f_ref, atol=1e-8)
    want, logz_ref = RW.forward(s, ro, runs, f_ref, theta, obs, 512.0)
    assert np.allclose(got, want, rtol=1e-9, atol=0)
    assert logz == pytest.approx(logz_ref, rel=1e-10)


def test_far_start_underflow_recovers(engine_lib):
    """A start far from the solution makes whole runs' WHAM sums underflow to zero; the log-space
    sums must carry the iteration to the same free energies (none NaN)."""
    s, ro, runs = synthetic(5)
    f_ref = RW.wham(s, ro, runs, n_iter=3000, tol=1e-12)
    far = np.array([0.0, 900.0, -800.0, 1500.0])
    _, _, f = gpu_forward(s, ro, runs, far, [1.32, 0.46, 0, 0, 0], ["E"], 512.0, n_iter=3000, tol=1e-12)
    assert np.all(np.isfinite(f)) and np.allclose(f, f_ref, atol=1e-7)
    # the oracle's log-space update from the same start agrees too
    assert np.allclose(RW.wham(s, ro, runs, f0=far, n_iter=3000, tol=1e-12), f_ref, atol=1e-7)


def test_adjoint_matches_numpy_and_finite_differences(engine_lib):
    s, ro, runs = synthetic(11)
    f = RW.wham(s, ro, runs, n_iter=2000, tol=1e-12)
    theta = np.array([1.33, 0.44, 0.01, -0.005, 0.02])
    obs = ["E", "V", "H", "RHO", "NHB"]
    g = np.array([0.3, -1.2, 0.7, 50.0, 0.1])
    adj = gpu_adjoint(s, ro, runs, f, theta, obs, 512.0, g)
    ref = RW.gradient(s, ro, runs, f, theta, obs, 512.0, g)
    assert np.allclose(adj, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())
    for q, h in enumerate([1e-5, 1e-5, 1e-5, 1e-5, 1e-5]):
        tp, tm = theta.copy(), theta.copy()
        tp[q] += h
        tm[q] -= h
        yp, _, _ = gpu_forward(s, ro, runs, f, tp, obs, 512.0, n_iter=0)
        ym, _, _ = gpu_forward(s, ro, runs, f, tm, obs, 512.0, n_iter=0)
        fd = float(g @ (yp - ym)) / (2 * h)
        assert fd == pytest.approx(adj[q], rel=2e-5, abs=1e-7 * np.abs(adj).max())


def test_fluctuation_identities(engine_lib):
    s, ro, runs = synthetic(3)
    f = RW.wham(s, ro, runs, n_iter=2000, tol=1e-12)
    theta = [1.31, 0.45, 0.0, 0.0, 0.0]
    (mH, mH2, mV, mV2), _, _ = gpu_forward(s, ro, runs, f, theta, ["H", "H2", "V", "V2"], 512.0, n_iter=0)
    dH_dbeta = gpu_adjoint(s, ro, runs, f, theta, ["H"], 512.0, [1.0])[0]
    dV_dP = gpu_adjoint(s, ro, runs, f, theta, ["V"], 512.0, [1.0])[1]
    assert -dH_dbeta == pytest.approx(mH2 - mH * mH, rel=1e-6)          # C_P T^2 = var(H)
    assert -dV_dP == pytest.approx(theta[0] * (mV2 - mV * mV), rel=1e-6)  # K_T <V> T = var(V)


def test_rejects_bad_arguments(engine_lib):
    s, ro, runs = synthetic()
    bad = ro.copy()
    bad[0] = 9
    with pytest.raises(abi.CvfError):
        gpu_forward(s, bad, runs, np.zeros(4), [1.3, 0.45, 0, 0, 0], ["E"], 512.0)


def engine_samples(L, temps, P, steps, eq, interval, seed):
    from cvfbulkwater_gb300.engine import Lattice, Params
    lat = Lattice([Params(L=L, T=t, P=P, seed=seed + i, start=0, replica=i) for i, t in enumerate(temps)])
    lat.run(eq, 1, 0)
    lat.run_sampled(steps, 1, 0, interval)
    out, run_of = [], []
    for r in range(len(temps)):
        for smp in lat.samples(r):
            o = lat.sample_observables(smp, r)
            out.append([o.energy, o.v_total, o.n_hb, float(o.n_sigma)])
            run_of.append(r)
    lat.close()
    return np.array(out), np.array(run_of)


def block_err(x, nb=20):
    b = np.asarray(x)[: len(x) // nb * nb].reshape(nb, -1).mean(1)
    return b.std(ddof=1) / math.sqrt(nb)


def jackknife_reweighted(s, ro, runs, f, theta, obs, n_cells, nb=10):
    """Jackknife covariance of reweighted means over nb blocks of every run's samples (WHAM
    refined from f on each subsample)."""
    idx = [np.flatnonzero(ro == j) for j in range(len(runs))]
    vals = []
    for k in range(nb):
        keep = np.concatenate([ix[np.arange(len(ix)) // (len(ix) // nb) != k] for ix in idx])
        m, _, _ = gpu_forward(s[keep], ro[keep], runs, f.copy(), theta, obs, n_cells, n_iter=200, tol=1e-9)
        vals.append(m)
    dev = np.asarray(vals) - np.mean(vals, 0)
    return (nb - 1) / nb * dev.T @ dev


def block_cov(x, nb=20):
    """Covariance of the means of the columns of x from nb blocks."""
    b = np.asarray(x)[: len(x) // nb * nb].reshape(nb, -1, x.shape[1]).mean(1)
    return np.cov(b, rowvar=False, ddof=1) / nb


def test_reweighting_reproduces_direct_simulation(engine_lib):
    """Samples of five runs reweighted to T = 0.75 against a direct run there. E and V are
    strongly correlated, so they are tested together: chi^2 of the difference of (E, V) under the
    combined covariance (20-block covariance of the direct run's means plus the jackknife
    covariance of the reweighted means over 10 blocks of every run) below the 95 % point of
    chi^2 with 2 degrees of freedom (5.991)."""
    L, P_, N = 8, 0.45, 512
    temps = [0.70, 0.72, 0.74, 0.76, 0.78]
    s, ro = engine_samples(L, temps, P_, 40000, 4000, 10, 9100)
    runs = np.array([[1.0 / float(np.float32(t)), float(np.float32(P_))] for t in temps])
    theta = [1.0 / 0.75, float(np.float32(P_)), 0, 0, 0]
    mean, _, f = gpu_forward(s, ro, runs, np.zeros(5), theta, ["E", "V"], float(N), n_iter=500, tol=1e-9)
    cov = jackknife_reweighted(s, ro, runs, f, theta, ["E", "V"], float(N))
    d, _ = engine_samples(L, [0.75], P_, 40000, 4000, 10, 9200)
    cov = cov + block_cov(d[:, :2])
    diff = np.asarray(mean[:2]) - d[:, :2].mean(0)
    chi2 = float(diff @ np.linalg.solve(cov, diff))
    assert chi2 < 5.991, (mean[:2], d[:, :2].mean(0), np.sqrt(np.diag(cov)), chi2)
    # adjoint response vs finite differences of the reweighted curve at T = 0.75 +/- 0.005
    beta = 1.0 / 0.75
    th = [beta, float(np.float32(P_)), 0, 0, 0]
    dH_dbeta = gpu_adjoint(s, ro, runs, f, th, ["H"], float(N), [1.0])[0]
    cp_adj = -beta * beta * dH_dbeta / N  # C_P = dH/dT per cell
    hp, _, _ = gpu_forward(s, ro, runs, f, [1 / 0.755, th[1], 0, 0, 0], ["H"], float(N), n_iter=0)
    hm, _, _ = gpu_forward(s, ro, runs, f, [1 / 0.745, th[1], 0, 0, 0], ["H"], float(N), n_iter=0)
    cp_fd = (hp[0] - hm[0]) / 0.01 / N
    assert cp_adj == pytest.approx(cp_fd, rel=2e-3)
