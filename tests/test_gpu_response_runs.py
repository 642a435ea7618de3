"""Adjoint response functions against finite differences of independent runs.

The reference obtains alpha_P, C_P and K_T by finite differences of the means of separate runs
(CVF_ThermodynamicAnalysis/AlphaPderivate.c:111-134, CPderivate.c:105-124, KTderivate.c:346-445).
Here five engine runs at (T0, P0), (T0 -/+ 0.005, P0) and (T0, P0 -/+ 0.005) give those central
differences with 20-block errors; the hand-written adjoint kernel (cvf_reweight_adjoint) gives the
same derivatives from the fluctuations of the central run alone. They must agree within 2
combined standard errors; the adjoint's error is the jackknife over the same 20 blocks of the
fluctuation formula that the adjoint equals (C_P = beta^2 var(H) / N, alpha_P = beta^2 cov(V, H)
/ <V>, K_T = beta var(V) / <V>).
"""
import ctypes as C
import math

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from cvfbulkwater_gb300.engine import Lattice, Params

pytestmark = pytest.mark.gpu

L, N = 16, 16 ** 3
T0, P0, D = 0.75, 0.45, 0.005
NB = 20


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _adjoint(samples, beta, p, obs_id):
    """d <obs> / d (beta, P) of the single run `samples` (n x 4: E, V, N_hb, N_sigma)."""
    s = np.ascontiguousarray(samples, dtype=np.float64)
    ro = np.zeros(len(s), dtype=np.int32)
    runs = np.array([[beta, p]], dtype=np.float64)
    f = np.zeros(1)
    th = np.array([beta, p, 0.0, 0.0, 0.0])
    ids = np.array([obs_id], dtype=np.int32)
    g = np.ones(1)
    out = np.zeros(5)
    abi.check(abi.lib().cvf_reweight_adjoint(0, _ptr(s), _ptr(ro), len(s), _ptr(runs), 1, _ptr(f), float(N), _ptr(th),
                                             _ptr(ids), 1, _ptr(g), _ptr(out)))
    return out[:2]


def _blocks(x):
    x = np.asarray(x)[: len(x) // NB * NB]
    return x.reshape(NB, -1)


def _mean_err(x):
    b = _blocks(x).mean(1)
    return b.mean(), b.std(ddof=1) / math.sqrt(NB)


def _jackknife(f, *cols):
    bl = [_blocks(c) for c in cols]
    vals = []
    for k in range(NB):
        keep = [np.delete(b, k, axis=0).ravel() for b in bl]
        vals.append(f(*keep))
    vals = np.asarray(vals)
    return math.sqrt((NB - 1) / NB * ((vals - vals.mean()) ** 2).sum())


def test_adjoint_matches_finite_differences_of_independent_runs(engine_lib):
    pts = [(T0, P0), (T0 - D, P0), (T0 + D, P0), (T0, P0 - D), (T0, P0 + D)]
    lat = Lattice([Params(L=L, T=t, P=p, seed=5150 + i, start=0, replica=i, sample_capacity=40000)
                   for i, (t, p) in enumerate(pts)])
    lat.run(20000, 1, 0)
    lat.run_sampled(300000, 1, 0, 10)
    runs = []
    for r in range(len(pts)):
        smp = lat.samples(r)
        obs = [lat.sample_observables(s, r) for s in smp]
        runs.append({"E": np.array([o.energy for o in obs]), "V": np.array([o.v_total for o in obs]),
                     "H": np.array([o.enthalpy for o in obs]), "NHB": np.array([o.n_hb for o in obs]),
                     "NS": smp["n_sigma"].astype(np.float64)})
    lat.close()
    # the engine reads T and P as float (GW:298-304): differences and beta use those values
    Tf = [float(np.float32(t)) for t, _ in pts]
    Pf = [float(np.float32(p)) for _, p in pts]
    dT, dP = Tf[2] - Tf[1], Pf[4] - Pf[3]
    beta, p0 = 1.0 / Tf[0], Pf[0]
    c = runs[0]
    mV0 = c["V"].mean()

    # finite differences of the run means (per cell for C_P)
    (Hm, eHm), (Hp, eHp) = _mean_err(runs[1]["H"]), _mean_err(runs[2]["H"])
    (Vm, eVm), (Vp, eVp) = _mean_err(runs[1]["V"]), _mean_err(runs[2]["V"])
    (Wm, eWm), (Wp, eWp) = _mean_err(runs[3]["V"]), _mean_err(runs[4]["V"])
    fd = {"C_P": ((Hp - Hm) / dT / N, math.hypot(eHp, eHm) / dT / N),
          "alpha_P": ((Vp - Vm) / dT / mV0, math.hypot(eVp, eVm) / dT / mV0),
          "K_T": (-(Wp - Wm) / dP / mV0, math.hypot(eWp, eWm) / dP / mV0)}

    # adjoint of the central run's reweighted means at its own (beta, P)
    smp = np.stack([c["E"], c["V"], c["NHB"], c["NS"]], 1)
    dH = _adjoint(smp, beta, p0, 4)   # d<H>/d(beta, P)
    dV = _adjoint(smp, beta, p0, 1)   # d<V>/d(beta, P)
    adj = {"C_P": -beta * beta * dH[0] / N, "alpha_P": -beta * beta * dV[0] / mV0, "K_T": -dV[1] / mV0}
    err = {"C_P": _jackknife(lambda h: beta * beta * h.var() / N, c["H"]),
           "alpha_P": _jackknife(lambda v, h: beta * beta * np.cov(v, h, bias=True)[0, 1] / v.mean(), c["V"], c["H"]),
           "K_T": _jackknife(lambda v: beta * v.var() / v.mean(), c["V"])}
    # the adjoint is the fluctuation formula of the same samples
    H, V = c["H"], c["V"]
    assert adj["C_P"] == pytest.approx(beta * beta * H.var() / N, rel=1e-6)
    assert adj["K_T"] == pytest.approx(beta * V.var() / V.mean(), rel=1e-6)
    for k in ("C_P", "alpha_P", "K_T"):
        val, e = fd[k]
        z = (adj[k] - val) / math.hypot(e, err[k])
        assert abs(z) < 2.0, (k, adj[k], val, e, err[k], z)
        assert e < 0.5 * abs(val), (k, val, e)  # the runs resolve the derivative
