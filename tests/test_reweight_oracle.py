"""The numpy reweighting restatement (oracle/reweight.py) is self-consistent: one run reweighted to
its own state point gives the plain sample mean, and its analytic gradient matches finite
differences. No GPU needed."""
import numpy as np

from oracle import reweight as RW


def test_single_run_reweights_to_sample_mean():
    rng = np.random.default_rng(0)
    s = np.stack([rng.normal(-100, 3, 500), rng.normal(50, 1, 500), rng.normal(40, 2, 500), rng.normal(60, 2, 500)], 1)
    ro = np.zeros(500, dtype=int)
    runs = np.array([[1.2, 0.3]])
    f = RW.wham(s, ro, runs)
    got, _ = RW.forward(s, ro, runs, f, [1.2, 0.3, 0, 0, 0], ["E", "V", "NHB"], 100.0)
    assert np.allclose(got, s[:, :3].mean(0), rtol=1e-12)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    runs = np.array([[1.3, 0.4], [1.25, 0.45]])
    s = np.concatenate([np.stack([rng.normal(-100 + 5 * j, 3, 400), rng.normal(50 + j, 1, 400),
                                  rng.normal(40, 2, 400), rng.normal(60, 2, 400)], 1) for j in range(2)])
    ro = np.repeat([0, 1], 400)
    f = RW.wham(s, ro, runs, n_iter=1000, tol=1e-13)
    th = np.array([1.27, 0.42, 0.01, 0.02, 0.03])
    obs = ["E", "H", "RHO", "VH"]
    g = np.array([1.0, -0.5, 20.0, 0.001])
    an = RW.gradient(s, ro, runs, f, th, obs, 100.0, g)
    for q in range(5):
        tp, tm = th.copy(), th.copy()
        tp[q] += 1e-6
        tm[q] -= 1e-6
        fd = (g @ RW.forward(s, ro, runs, f, tp, obs, 100.0)[0] - g @ RW.forward(s, ro, runs, f, tm, obs, 100.0)[0]) / 2e-6
        assert abs(fd - an[q]) <= 1e-5 * max(1.0, abs(an[q]))
