"""CPU restatement of the binned 2-D (E, rho) histogram reweighting of the reference's
HistogramReweighting/histogram_reweighting_mixed_paramSI_norm_x.f90 ("F90"). Test infrastructure
only: it checks the engine's cvf_h2d_* functions; nothing in the library calls it.

Parity unpinned: no Fortran compiler exists here and the simulation archive the program reads
is not in the reference checkout, so this restatement is checked only against itself and the
engine (and against the closed-form Binder limits in the tests).

  setup          F90:81-88 (unit conversions), F90:155-300 (SI conversion of every sample, ranges,
                 n_bin = int(sqrt(real(max samples))/2), 20 empty bins added, n_bin2D, the per-run
                 2-D histograms normalised by in-range count x bin area), F90:135 (log of the
                 sample counts in single precision)
  log_P          Calcula_Histograma F90:1003-1124 (log-sum-exp over runs with the 10 e-fold
                 truncation, log_Z over bins with the same truncation)
  wham           F90:398-425 (Jacobi iteration of the constants, normalised to run 1; error
                 unless the last step changed every constant by at most 1e-7)
  reweighted     F90:737-757 (grid exp(log_P - log_Z) normalised to unit integral)
  binder_e_rho   binder_energy_density F90:2610-2662
  mixed          Calcula_Histograma_Rotado_normX F90:1383-1620 (rotation F90:1126-1146, binning,
                 zero mean and unit variance, the sine map with b = 1.53, normalised again)
  binder_mixed   binder F90:2580-2608
"""
from __future__ import annotations

import math

import numpy as np

TS, TI = 140.5678, 185.4676
PS, PI = 4694.59, -2111.5552
RHOS, RHOI = 1527.3, -23.1017
HS, HI = 11.272132, 9.028914


class H2D:
    def __init__(self, h, rho, run_of, That, Phat, L, bin_factor):
        h, rho, run_of = np.asarray(h, float), np.asarray(rho, float), np.asarray(run_of)
        self.That, self.Phat = np.asarray(That, float), np.asarray(Phat, float)
        self.L, self.N = L, L * L * L
        R = len(self.That)
        self.Tk = self.That * TS + TI
        self.Pbar = self.Phat * PS + PI
        dens = RHOS * rho + RHOI
        E = HS * h + HI * self.That[run_of] - 1.8 * self.Pbar[run_of] / dens
        self.medidas = np.bincount(run_of, minlength=R)
        self.log_medidas = np.log(self.medidas.astype(np.float32)).astype(np.float64)
        Emin, Emax, Dmin, Dmax = E.min(), E.max(), dens.min(), dens.max()
        n_bin = int(np.sqrt(np.float32(self.medidas.max())) / np.float32(2.0))
        rE, rD = Emax - Emin, Dmax - Dmin
        tE, tD = rE / n_bin, rD / n_bin
        n_bin += 20
        rE, rD = rE + 20 * tE, rD + 20 * tD
        Emin, Dmin = Emin - 10 * tE, Dmin - 10 * tD
        nb = int(n_bin * 10 * bin_factor)
        self.nb, self.Emin, self.Dmin = nb, Emin, Dmin
        self.dE, self.dD = rE / nb, rD / nb
        iE = ((E - Emin) / self.dE).astype(np.int64)
        iD = ((dens - Dmin) / self.dD).astype(np.int64)
        ok = (iE >= 0) & (iE < nb) & (iD >= 0) & (iD < nb)
        hs = np.zeros((nb, nb))
        for j in range(R):
            sel = ok & (run_of == j)
            cnt = np.zeros((nb, nb))
            np.add.at(cnt, (iE[sel], iD[sel]), 1.0)
            norma = sel.sum() * self.dE * self.dD
            hs += cnt / norma  # F90:1018-1021 adds the runs in order
        self.hsum = hs
        self.ctes = np.zeros(R)
        i = np.arange(nb)
        self.Ec = Emin + (i + 0.5) * self.dE
        self.Dc = Dmin + (i + 0.5) * self.dD

    def log_P(self, temp, pres, ctes=None):
        """F90:1003-1124 at temp [K], pres [bar] -> (log_P, mask of non-empty bins, log_Z)."""
        ctes = self.ctes if ctes is None else ctes
        beta1, pres1 = 1000.0 / (0.2293 * temp), pres * 100.0
        E = self.Ec[:, None] * self.N
        V = (0.018 / self.Dc[None, :]) * self.N
        mask = self.hsum != 0
        R = len(ctes)
        args = np.empty((R,) + self.hsum.shape)
        for j in range(R):
            bj = 1000.0 / (0.2293 * self.Tk[j])
            pj = self.Pbar[j] * 100.0
            args[j] = beta1 * (E + pres1 * V) - bj * (E + pj * V) - ctes[j] + self.log_medidas[j]
        flag = (np.abs(args) > 10).any(axis=0)
        with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
            plain = np.log(np.exp(args).sum(axis=0))
            mx = args.max(axis=0)
            keep = (mx[None] - args) < 10
            s = np.where(keep, np.exp(args - mx[None]), 0.0).sum(axis=0)
            trunc = np.where(s != 0, np.log(s), 0.0) + mx
            xx = np.where(flag, trunc, plain)
            lp = np.where(mask, np.log(np.where(mask, self.hsum, 1.0)) - xx, 0.0)
        m = lp[mask].max()
        kept = mask & ((m - lp) < 10)
        z = np.exp(lp[kept] - m).sum()
        log_Z = (math.log(z) if z != 0 else 0.0) + m
        return lp, mask, log_Z

    def wham(self, steps):
        R = len(self.That)
        ctes, ctes2 = np.zeros(R), np.zeros(R)
        for _ in range(steps):
            ctes = ctes2.copy()
            new = np.array([self.log_P(self.Tk[k], self.Pbar[k], ctes)[2] for k in range(R)])
            ctes2 = new - new[0]
        if np.any(np.abs(ctes - ctes2) > 1e-7):
            raise RuntimeError("constants did not converge")
        self.ctes = ctes2
        return ctes2

    def reweighted(self, T_hat, P_hat):
        lp, mask, log_Z = self.log_P(T_hat * TS + TI, P_hat * PS + PI)
        g = np.zeros_like(lp)
        g[mask] = np.exp(lp[mask] - log_Z)
        g[mask] = g[mask] / (g.sum() * self.dE * self.dD)
        return g, mask

    def binder_e_rho(self, g, mask):
        he = np.where(mask, g, 0).sum(axis=1)
        hr = np.where(mask, g, 0).sum(axis=0)
        norma = np.where(mask, g, 0).sum()
        he, hr = he / norma, hr / norma
        e2 = self.Ec * self.Ec
        r2 = self.Dc * self.Dc
        u2, u4 = (e2 * he).sum(), (e2 * e2 * he).sum()
        v2, v4 = (r2 * hr).sum(), (r2 * r2 * hr).sum()
        return 1.0 - u4 / (3.0 * u2 * u2), 1.0 - v4 / (3.0 * v2 * v2)

    def mixed(self, g, alpha):
        """Rotado_normX: (x, q, a1, media) of the mixed parameter at angle alpha."""
        pos = g > 0
        X = self.Ec[:, None] * math.sin(alpha) + self.Dc[None, :] * math.cos(alpha)
        Xmin, Xmax = X[pos].min(), X[pos].max()
        nbm = int(np.sqrt(np.float32(self.nb * np.float32(1.0))))
        rX = Xmax - Xmin
        t = rX / nbm
        rX += 4 * t
        Xmin -= 2 * t
        t = rX / nbm
        idx = ((X - Xmin) / t).astype(np.int64)
        idx = np.where(np.abs(X - Xmin) < 1e-10, np.maximum(idx, 0), idx)
        q = np.zeros(nbm)
        np.add.at(q, idx[pos], g[pos])
        m = Xmin + (np.arange(nbm) + 0.5) * t
        q = q / (q.sum() * t)
        media = (m * q * t).sum()
        m = m - media
        p = q > 0
        norma = (q[p] * t).sum()
        var = (m[p] * m[p] * q[p] * t).sum()
        a1 = math.sqrt(norma / var)
        a2 = 1 / (norma * a1)
        m, t, q = m * a1, t * a1, q * a2
        b, pi = 1.53, 3.14159
        m = 1.0 * b * b * np.sin(pi * m / b) / (pi * pi) + 1.0 * m
        w = np.empty(nbm)
        w[0] = m[1] - m[0]
        w[1:-1] = (m[2:] - m[:-2]) / 2.0
        w[-1] = m[-1] - m[-2]
        q = q / (q * w).sum()
        m = m - (m * q * w).sum()
        p = q > 0
        norma = (q[p] * w[p]).sum()
        var = (m[p] * m[p] * q[p] * w[p]).sum()
        a1 = math.sqrt(norma / var)
        a2 = 1 / (norma * a1)
        return m * a1, q * a2, a1, media

    @staticmethod
    def binder_mixed(x, q, a1, media):
        op = x / a1 + media
        norma = q.sum()
        m2 = op * op
        u2 = (m2 * q / norma).sum()
        u4 = (m2 * m2 * q / norma).sum()
        return 1.0 - u4 / (3.0 * u2 * u2)
