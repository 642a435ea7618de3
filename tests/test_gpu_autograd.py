"""The reweighting kernels behind torch.autograd.Function (test harness only).

forward(theta) calls cvf_reweight_forward, backward(g) calls the hand-written adjoint
cvf_reweight_adjoint. Autograd through theta = (1/T, P, dJ_hb, dJ_s, dv_hb) then gives the response
functions directly -- alpha_P = (1/V) dV/dT, K_T = -(1/V) dV/dP, C_P = dH/dT per cell -- which
replace the finite differences of CVF_ThermodynamicAnalysis/{AlphaP,KT,CP}derivate.c; they are
checked against the fluctuation formulas (TA/calculadora.sh:39,42) and finite differences, and
d<rho>/d(J_hb, J_s, v_hb) against finite differences of the forward kernel.
"""
import ctypes as C

import numpy as np
import pytest

from cvfbulkwater_gb300 import abi
from oracle import reweight as RW

pytestmark = pytest.mark.gpu
IDS = {name: i for i, name in enumerate(RW.OBS)}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Reweighted:
    """Holds the sample stream of several runs and their converged free energies."""

    def __init__(self, samples, run_of, runs, n_cells, obs):
        self.s = np.ascontiguousarray(samples, dtype=np.float64)
        self.ro = np.ascontiguousarray(run_of, dtype=np.int32)
        self.runs = np.ascontiguousarray(runs, dtype=np.float64)
        self.n_cells = float(n_cells)
        self.obs = list(obs)
        self.ids = np.array([IDS[o] for o in obs], dtype=np.int32)
        self.f = np.zeros(len(runs))
        self.forward(np.array([runs[0, 0], runs[0, 1], 0, 0, 0]), n_iter=1000)

    def forward(self, theta, n_iter=0):
        out = np.zeros(len(self.obs) + 1)
        th = np.ascontiguousarray(theta, dtype=np.float64)
        abi.check(abi.lib().cvf_reweight_forward(0, _p(self.s), _p(self.ro), len(self.s), _p(self.runs),
                                                 len(self.runs), _p(self.f), n_iter, 1e-10, self.n_cells, _p(th),
                                                 _p(self.ids), len(self.ids), _p(out)))
        return out[:-1]

    def adjoint(self, theta, g):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        gg = np.ascontiguousarray(g, dtype=np.float64)
        out = np.zeros(5)
        abi.check(abi.lib().cvf_reweight_adjoint(0, _p(self.s), _p(self.ro), len(self.s), _p(self.runs),
                                                 len(self.runs), _p(self.f), self.n_cells, _p(th), _p(self.ids),
                                                 len(self.ids), _p(gg), _p(out)))
        return out


def make_function(rw):
    import torch

    class ReweightFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            ctx.save_for_backward(theta)
            return torch.from_numpy(rw.forward(theta.detach().cpu().numpy()))

        @staticmethod
        def backward(ctx, g):
            (theta,) = ctx.saved_tensors
            return torch.from_numpy(rw.adjoint(theta.detach().cpu().numpy(), g.detach().cpu().numpy()))

    return ReweightFn.apply


@pytest.fixture(scope="module")
def runs_l8(engine_lib):
    from cvfbulkwater_gb300.engine import Lattice, Params
    temps = [0.72, 0.74, 0.76, 0.78]
    P = 0.45
    lat = Lattice([Params(L=8, T=t, P=P, seed=5150 + i, start=0, replica=i) for i, t in enumerate(temps)])
    lat.run(3000, 1, 0)
    lat.run_sampled(30000, 1, 0, 10)
    rows, run_of = [], []
    for r in range(len(temps)):
        for smp in lat.samples(r):
            o = lat.sample_observables(smp, r)
            rows.append([o.energy, o.v_total, o.n_hb, float(o.n_sigma)])
            run_of.append(r)
    lat.close()
    runs = np.array([[1.0 / float(np.float32(t)), float(np.float32(P))] for t in temps])
    return np.array(rows), np.array(run_of), runs


def test_response_functions_by_autograd(runs_l8):
    import torch
    s, ro, runs = runs_l8
    N = 512.0
    obs = ["V", "H", "RHO", "V2", "H2", "VH"]
    rw = Reweighted(s, ro, runs, N, obs)
    fn = make_function(rw)
    T = torch.tensor(0.75, dtype=torch.float64, requires_grad=True)
    P = torch.tensor(float(np.float32(0.45)), dtype=torch.float64, requires_grad=True)
    d = torch.zeros(3, dtype=torch.float64, requires_grad=True)
    y = fn(torch.cat([(1.0 / T).reshape(1), P.reshape(1), d]))
    V, H, rho, V2, H2, VH = y
    dV_dT, dV_dP = torch.autograd.grad(V, (T, P), retain_graph=True)
    (dH_dT,) = torch.autograd.grad(H, (T,), retain_graph=True)
    drho = torch.autograd.grad(rho, (d,))[0].numpy()
    t, v = 0.75, V.item()
    alpha_p = dV_dT.item() / v
    k_t = -dV_dP.item() / v
    c_p = dH_dT.item() / N
    # fluctuation formulas on the same reweighted distribution
    assert alpha_p == pytest.approx((VH.item() - v * H.item()) / (t * t * v), rel=1e-6)
    assert k_t == pytest.approx((V2.item() - v * v) / (t * v), rel=1e-6)
    assert c_p == pytest.approx((H2.item() - H.item() ** 2) / (t * t * N), rel=1e-6)
    assert k_t > 0 and c_p > 0
    # finite differences of the reweighted curve, T and P +/- 0.005
    th = lambda tt, pp: np.array([1.0 / tt, pp, 0, 0, 0])  # noqa: E731
    vp, vm = rw.forward(th(0.755, P.item()))[0], rw.forward(th(0.745, P.item()))[0]
    assert alpha_p == pytest.approx((vp - vm) / 0.01 / v, rel=5e-3, abs=1e-6)
    vp, vm = rw.forward(th(0.75, P.item() + 0.005))[0], rw.forward(th(0.75, P.item() - 0.005))[0]
    assert k_t == pytest.approx(-(vp - vm) / 0.01 / v, rel=5e-3)
    # d<rho>/d(J_hb, J_s, v_hb) against finite differences of the forward kernel
    for q in range(3):
        tp, tm = th(0.75, P.item()), th(0.75, P.item())
        tp[2 + q] += 1e-4
        tm[2 + q] -= 1e-4
        fd = (rw.forward(tp)[2] - rw.forward(tm)[2]) / 2e-4
        assert drho[q] == pytest.approx(fd, rel=1e-3, abs=1e-9)
