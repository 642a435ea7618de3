"""FP64 numpy restatement of the engine's multiple-histogram reweighting (test infrastructure only).

The reference reweights binned (E, rho) histograms (HistogramReweighting/histogram_reweighting_
mixed_paramSI_norm_x.f90): self-consistent constants iterated up to `step` times with a 1e-7
convergence check (F90:450-473) and, per target (T, P), log P = log H - LSE_j[...] with terms more
than 10 e-folds below the maximum dropped (Calcula_Histograma, F90:1003-1124). The engine applies
the same Ferrenberg-Swendsen equations per sample (no bins, no truncation):

    D_k   = sum_j n_j exp(f_j - beta_j (E_k + P_j V_k)),      f_j = -log Z_j, f_0 = 0
    f_i  <- f_i - log sum_k exp(f_i - beta_i (E_k + P_i V_k) - log D_k)
    w_k   = exp(-beta (E'_k + P V'_k)) / D_k,  E' = E - dJ_hb N_hb - dJ_s N_s,  V' = V + dv_hb N_hb

This module restates those equations with numpy (and the response functions as covariances) so
the GPU kernels can be checked; it also provides the reference's binned form for comparison.
"""
from __future__ import annotations

import numpy as np

E, V, NHB, NSIG = 0, 1, 2, 3
OBS = ["E", "V", "NHB", "NSIG", "H", "RHO", "H2", "V2", "VH"]


def lse(a, axis=None):
    m = np.max(a, axis=axis, keepdims=True)
    out = m + np.log(np.sum(np.exp(a - m), axis=axis, keepdims=True))
    return np.squeeze(out, axis=axis) if axis is not None else float(out.ravel()[0])


def log_d(samples, run_of, runs, f):
    n_runs = len(runs)
    logn = np.log(np.bincount(run_of, minlength=n_runs).astype(np.float64))
    b, p = runs[:, 0], runs[:, 1]
    t = logn[None, :] + f[None, :] - b[None, :] * (samples[:, E:E + 1] + p[None, :] * samples[:, V:V + 1])
    return lse(t, axis=1)


def ti_start(samples, run_of, runs):
    """Starting f: d f = <E> d beta + <V> d(beta P) integrated by trapezoids between consecutive
    runs in (beta, beta P) order, relative to run 0 (the engine's start when given zeros)."""
    nr = len(runs)
    c = np.bincount(run_of, minlength=nr).astype(np.float64)
    se = np.bincount(run_of, weights=samples[:, E], minlength=nr) / c
    sv = np.bincount(run_of, weights=samples[:, V], minlength=nr) / c
    order = sorted(range(nr), key=lambda i: (runs[i, 0], runs[i, 0] * runs[i, 1]))
    f = np.zeros(nr)
    for a, b in zip(order[:-1], order[1:]):
        db = runs[b, 0] - runs[a, 0]
        dbp = runs[b, 0] * runs[b, 1] - runs[a, 0] * runs[a, 1]
        f[b] = f[a] + 0.5 * (se[a] + se[b]) * db + 0.5 * (sv[a] + sv[b]) * dbp
    return f - f[0]


def wham(samples, run_of, runs, f0=None, n_iter=300, tol=1e-7):
    """Self-consistent f_j = -log Z_j (F90:450-473 restated per sample)."""
    runs = np.asarray(runs, dtype=np.float64)
    f = np.zeros(len(runs)) if f0 is None else np.array(f0, dtype=np.float64)
    if n_iter > 0 and not np.any(f):
        f = ti_start(samples, np.asarray(run_of), runs)
    b, p = runs[:, 0], runs[:, 1]
    for _ in range(n_iter):
        ld = log_d(samples, run_of, runs, f)
        u = f[None, :] - b[None, :] * (samples[:, E:E + 1] + p[None, :] * samples[:, V:V + 1]) - ld[:, None]
        nf = f - lse(u, axis=0).ravel()  # in log space: no run's sum underflows to 0
        nf -= nf[0]
        change = np.max(np.abs(nf - f))
        f = nf
        if change < tol:
            break
    return f


def primed(samples, theta):
    beta, P, djhb, djs, dvhb = theta
    Ep = samples[:, E] - djhb * samples[:, NHB] - djs * samples[:, NSIG]
    Vp = samples[:, V] + dvhb * samples[:, NHB]
    return Ep, Vp


def obs_values(samples, theta, n_cells):
    Ep, Vp = primed(samples, theta)
    H = Ep + theta[1] * Vp
    return {"E": Ep, "V": Vp, "NHB": samples[:, NHB], "NSIG": samples[:, NSIG], "H": H,
            "RHO": n_cells / Vp, "H2": H * H, "V2": Vp * Vp, "VH": Vp * H}


def forward(samples, run_of, runs, f, theta, obs, n_cells):
    runs = np.asarray(runs, dtype=np.float64)
    ld = log_d(samples, run_of, runs, np.asarray(f, dtype=np.float64))
    Ep, Vp = primed(samples, theta)
    lw = -theta[0] * (Ep + theta[1] * Vp) - ld
    logz = lse(lw)
    w = np.exp(lw - logz)
    vals = obs_values(samples, theta, n_cells)
    return np.array([np.sum(w * vals[o]) for o in obs]), logz


def gradient(samples, run_of, runs, f, theta, obs, n_cells, g):
    """sum_m g_m d<A_m>/d theta, theta = (beta, P, dJ_hb, dJ_s, dv_hb), as covariances."""
    runs = np.asarray(runs, dtype=np.float64)
    ld = log_d(samples, run_of, runs, np.asarray(f, dtype=np.float64))
    beta, P = theta[0], theta[1]
    Ep, Vp = primed(samples, theta)
    H = Ep + P * Vp
    lw = -beta * H - ld
    w = np.exp(lw - lse(lw))
    vals = obs_values(samples, theta, n_cells)
    nh, ns = samples[:, NHB], samples[:, NSIG]
    dlw = np.stack([-H, -beta * Vp, beta * nh, beta * ns, -beta * P * nh])
    zero = np.zeros_like(H)
    dE = [zero, zero, -nh, -ns, zero]
    dV = [zero, zero, zero, zero, nh]
    dH = [dE[q] + P * dV[q] + (Vp if q == 1 else 0.0) for q in range(5)]
    grads = {"E": dE, "V": dV, "NHB": [zero] * 5, "NSIG": [zero] * 5, "H": dH,
             "RHO": [-n_cells * dV[q] / (Vp * Vp) for q in range(5)],
             "H2": [2 * H * dH[q] for q in range(5)], "V2": [2 * Vp * dV[q] for q in range(5)],
             "VH": [dV[q] * H + Vp * dH[q] for q in range(5)]}
    out = np.zeros(5)
    for gm, o in zip(g, obs):
        a = vals[o]
        ma = np.sum(w * a)
        for q in range(5):
            out[q] += gm * (np.sum(w * grads[o][q]) + np.sum(w * a * dlw[q]) - ma * np.sum(w * dlw[q]))
    return out
