"""CPU restatement of the reference's multi-tau correlator (SOURCE/gpu_water3D.cu, "GW"). Test
infrastructure only: it checks the engine's device-side correlator; nothing in the library calls
it. Python floats are IEEE doubles and every operation rounds on its own, as the reference's C.

  MultiTau.__init__   GW:165-167 (32 levels, 16 channels, pairs averaged), GW:2983-3008
  MultiTau.add        GW:3010-3076 (the recursion of GW:3030 kept as written)
  MultiTau.evaluate   GW:3078-3112 with norm = 1
  correlation_text    printCorr GW:3109-3128 for one correlator ("%.0f\\t%f", f / f[0])
  max_mass            GW:1250-1272: fraction of the 6N arms in the most populated sigma value
"""
from __future__ import annotations

import numpy as np

LEVELS, P, M = 32, 16, 2


class MultiTau:
    def __init__(self):
        self.shift = [[-2e10] * P for _ in range(LEVELS)]
        self.correlation = [[0.0] * P for _ in range(LEVELS)]
        self.ncorrelation = [[0] * P for _ in range(LEVELS)]
        self.accumulator = [0.0] * LEVELS
        self.naccumulator = [0] * LEVELS
        self.insertindex = [0] * LEVELS
        self.kmax = 0
        self.accval = 0.0

    def add(self, w, k=0):
        dmin = P // M
        if k == LEVELS:
            return
        if k > self.kmax:
            self.kmax = k
        self.shift[k][self.insertindex[k]] = w
        if k == 0:
            self.accval += w
        self.accumulator[k] += w
        self.naccumulator[k] += 1
        if self.naccumulator[k] == M:
            self.add(self.accumulator[k] / M, k + 1)
            self.accumulator[k] = 0.0
            self.naccumulator[k] = 0
        ind1 = self.insertindex[k]
        sh, co, nc = self.shift[k], self.correlation[k], self.ncorrelation[k]
        if k == 0:
            ind2 = ind1
            for j in range(P):
                if sh[ind2] > -1e10:
                    co[j] += sh[ind1] * sh[ind2]
                    nc[j] += 1
                ind2 -= 1
                if ind2 < 0:
                    ind2 += P
        else:
            ind2 = ind1 - dmin
            for j in range(dmin, P):
                if ind2 < 0:
                    ind2 += P
                if sh[ind2] > -1e10:
                    co[j] += sh[ind1] * sh[ind2]
                    nc[j] += 1
                ind2 -= 1
        self.insertindex[k] += 1
        if self.insertindex[k] == P:
            self.insertindex[k] = 0

    def evaluate(self):
        dmin = P // M
        aux = (self.accval / self.ncorrelation[0][0]) * (self.accval / self.ncorrelation[0][0])
        t, f = [], []
        for i in range(P):
            if self.ncorrelation[0][i] > 0:
                t.append(float(i))
                f.append(self.correlation[0][i] / self.ncorrelation[0][i] - aux)
        for k in range(1, self.kmax):
            for i in range(dmin, P):
                if self.ncorrelation[k][i] > 0:
                    t.append(i * float(M) ** k)
                    f.append(self.correlation[k][i] / self.ncorrelation[k][i] - aux)
        return np.array(t), np.array(f)


def max_mass(cells12):
    """cells12: (N, 12) config.out rows; the six sigma columns give the 6N arms."""
    sig = np.asarray(cells12)[:, :6]
    counts = np.bincount(sig.ravel(), minlength=6)
    return float(counts.max()) / float(sig.size)


def correlation_text(t, f):
    return "".join("%.0f\t%f\n" % (t[i], f[i] / f[0]) for i in range(len(t)))
