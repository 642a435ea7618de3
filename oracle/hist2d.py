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
  wham           F90:446-472 (Jacobi iteration of the constants, normalised to run 1; error
                 unless the last step changed every constant by at most 1e-7)
  reweighted     F90:737-757 (grid exp(log_P - log_Z) normalised to unit integral)
  binder_e_rho   binder_energy_density F90:2610-2662
  mixed          Calcula_Histograma_Rotado_normX F90:1383-1620 (rotation F90:1126-1146, binning,
                 zero mean and unit variance, the sine map with b = 1.53, normalised again)
  binder_mixed   binder F90:2580-2608
  ising2d/3d     F90:2216-2252 (z**16 by repeated squaring, as gfortran expands it)
  ising_peaks    Ising_Peak F90:1148-1222
  confront       ConfrontIsing F90:2127-2182, ZeroTest F90:2042-2074, HeightTest F90:2076-2125
  scan           the search loop F90:732-891 (pressure outer, temperature, angle inner; B = 1)

The F90 is built with plain gfortran, so each literal it assigns to a real*8 (the unit
conversions, 1.8, 0.2293, 0.018, 1e-7, b = 1.53, pi = 3.14159, the Ising fits, 6.0/0.8, 1.14) is
the nearest single-precision value, widened: f32() below.
"""
from __future__ import annotations

import math

import numpy as np



def f32(x):
    """A default-kind Fortran literal as a real*8 value."""
    return float(np.float32(x))


TS, TI = f32(140.5678), f32(185.4676)
PS, PI = f32(4694.59), f32(-2111.5552)
RHOS, RHOI = f32(1527.3), f32(-23.1017)
HS, HI = f32(11.272132), f32(9.028914)
E18, KB, MW, CONV = f32(1.8), f32(0.2293), f32(0.018), f32(1e-7)
VIS = float(np.float32(6.0) / np.float32(0.8))


class H2D:
    def __init__(self, h, rho, run_of, That, Phat, L, bin_factor):
        h, rho, run_of = np.asarray(h, float), np.asarray(rho, float), np.asarray(run_of)
        self.That, self.Phat = np.asarray(That, float), np.asarray(Phat, float)
        self.L, self.N = L, L * L * L
        R = len(self.That)
        self.Tk = self.That * TS + TI
        self.Pbar = self.Phat * PS + PI
        dens = RHOS * rho + RHOI
        E = HS * h + HI * self.That[run_of] - E18 * self.Pbar[run_of] / dens
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
        beta1, pres1 = 1000.0 / (KB * temp), pres * 100.0
        E = self.Ec[:, None] * self.N
        V = (MW / self.Dc[None, :]) * self.N
        mask = self.hsum != 0
        R = len(ctes)
        args = np.empty((R,) + self.hsum.shape)
        for j in range(R):
            bj = 1000.0 / (KB * self.Tk[j])
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
        if np.any(np.abs(ctes - ctes2) > CONV):
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
        b, pi = f32(1.53), f32(3.14159)
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


def ising2d(z):
    a, b, c, d = f32(0.058137), f32(-2.68949), f32(-0.11235), f32(2.884162)
    z2 = z * z
    z4 = z2 * z2
    z8 = z4 * z4
    z16 = z8 * z8
    return math.exp(-(a * z16 + b * z * z + c * abs(z) + d))


def ising3d(z):
    a, c, M0, A0 = f32(0.196), f32(0.807), f32(1.141059404), f32(0.436591191)
    u = z * z / (M0 * M0) - 1
    return A0 * math.exp(-(u * u * (a * z * z / (M0 * M0) + c)))


def ising_peaks():
    peaks = []
    for k, f in enumerate((ising2d, ising3d)):
        xmin, xmax = f32(0.1), 2.0
        x1, x2 = xmin + (xmax - xmin) / 3, xmin + 2 * (xmax - xmin) / 3
        while True:
            if f(x1) > f(x2):
                xmax = x2
            elif f(x2) > f(x1):
                xmin = x1
            else:
                raise RuntimeError("equal values in the peak search")
            x1, x2 = xmin + (xmax - xmin) / 3, xmin + 2 * (xmax - xmin) / 3
            if (abs(x1 - x2) if k == 0 else abs(f(x1) - f(x2))) < f32(1e-6):
                peaks.append(f(x1) if f(x1) > f(x2) else f(x2))
                break
    return tuple(peaks)


def confront(m, q, peaks=None):
    """(liu_2D, liu_3D, kl_2D, kl_3D, zero, height) of abscissae m (already scaled by B)."""
    p2, p3 = ising_peaks() if peaks is None else peaks
    kl2 = kl3 = liu2 = liu3 = 0.0
    n_liu = 0
    for mi, h in zip(m, q):
        if h == 0:
            continue
        i2, i3 = ising2d(mi), ising3d(mi)
        if i2 > 0:
            kl2 = kl2 + (math.log(i2) - math.log(h)) * i2
        if i3 > 0:
            kl3 = kl3 + (math.log(i3) - math.log(h)) * i3
        liu2 = liu2 + math.sqrt(h) * abs(h - i2)
        liu3 = liu3 + math.sqrt(h) * abs(h - i3)
        n_liu += 1
    liu2 = liu2 / ((p2 - ising2d(0.0)) * n_liu)
    liu3 = liu3 / ((p3 - ising3d(0.0)) * n_liu)
    hmin, imin = f32(1e12), -1
    for i, (mi, h) in enumerate(zip(m, q)):
        if -1 < mi < 1 and h < hmin:
            hmin, imin = h, i
    zero = 1e3
    if imin >= 0:
        d = q[imin] - ising3d(0.0)
        zero = d * d * VIS * VIS + m[imin] * m[imin]
    h1 = h2 = -10.0
    i1 = i2 = -1
    for i, (mi, h) in enumerate(zip(m, q)):
        if mi < 0:
            if h > h1:
                h1, i1 = h, i
        elif h > h2:
            h2, i2 = h, i
    height = 1e3
    if i1 >= 0 and i2 >= 0:
        x1, x2 = f32(-1.14), f32(1.14)
        d1, d2 = q[i1] - ising3d(x1), q[i2] - ising3d(x2)
        height = d1 * d1 * VIS * VIS
        height = height + d2 * d2 * VIS * VIS
        height = height + (m[i1] - x1) * (m[i1] - x1)
        height = height + (m[i2] - x2) * (m[i2] - x2)
    return liu2, liu3, kl2, kl3, zero, height


def scan(h2d, T_hats, P_hats, S_list, B=1.0):
    """(tp_rows, rows, best) in the layout of cvf_h2d_scan."""
    peaks = ising_peaks()
    tp_rows, rows = [], []
    lo = [f32(1e12)] * 5
    best = [-1] * 5
    for P in P_hats:
        for T in T_hats:
            g, mask = h2d.reweighted(T, P)
            tp_rows.append(h2d.binder_e_rho(g, mask))
            for S in S_list:
                x, q, a1, media = h2d.mixed(g, S)
                v = (H2D.binder_mixed(x, q, a1, media),) + confront(B * x, q, peaks)
                crit = (v[1], v[2], v[5], v[6], v[5] + v[6])
                for j in range(5):
                    if lo[j] > crit[j]:
                        lo[j], best[j] = crit[j], len(rows)
                rows.append(v)
    return np.array(tp_rows), np.array(rows), best
