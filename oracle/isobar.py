"""CPU restatement of the reference's isobar analysis (CVF_ThermodynamicAnalysis/ of
lcoronas/CVFBulkWater). Test infrastructure only: it checks the engine's run statistics on the
GPU and the library's host functions; nothing in the library calls it.

  run_stats      script_analisi.sh:35   mean and <x^2> - <x>^2 of data.out columns 2-7 (awk, in
                                        double precision, sums in file order)
  isobar_point   calculadora.sh:41-61   per-cell means, errors sqrt(3 var / n) / N, density,
                                        N_hb / 2N, ncoop, r_cell (error sqrt(var / n)), C_P and
                                        K_T from the fluctuations
  to_si          conversor.sh:2-12 (constants), :20 (density), :24 (enthalpy), :28 (nhb, ncoop),
                 :32 (C_P fluctuation; its third column is an empty awk field, so 0), :76 (energy
                 from enthalpy and density)
  alpha_p        AlphaPderivate.c:56-134 (order by T, central differences, one-sided at the ends,
                 error from the sample variance, the third derivative and the neighbours' errors;
                 only points 2 .. n-3 are written)
  alpha_p_text   conversor.sh:54-66 as a text pipeline: awk's %.6g output between the stages,
                 AlphaPderivate's "%lf", the x1000 conversion and the nan/inf filter
  cp_derivative  CPderivate.c:56-124 (as alpha_p without the 1/V factor; error from the third
                 derivative and the neighbours' sqrt(3 var / n))
  kt_derivative  KTderivate.c:345-563 (compresibilidad_log, error_compresibilidad_log)
  kt_text        conversor.sh:84-119 as a text pipeline: the KT_input fields as awk prints them,
                 KTderivate's per-isobar "%lf %lf %e %lf" lines, the x1000 conversion, sort -g

Pinned by tests/golden/isobars_L32*.txt (the reference's own L32_P*_density.dat,
L32_P*_density.dat.SI and L32_P*_AlphaPderivate.dat.SI for all 47 isobars, and the 47
L32_P*_KTderivate.dat.SI files, whose inputs the fixtures hold only to the 6 digits of the
density files), and where the reference checkout exists by its AlphaPderivate, CPderivate and
KTderivate programs compiled from their .c files (oracle/build_ref.py), output for output.
"""
from __future__ import annotations

import math

import numpy as np

# conversor.sh:2-12
TS, TI = 140.5678, 185.4676
PS, PI = 469.459, -211.15552
RHOS, RHOI = 1527.3, -23.1017
CPS, CPI = 4.455, 3.56843
HS, HI = 11.272132, 9.028924

COLUMNS = ("energy", "enthalpy", "volume", "n_hb", "m", "r_cell")


def run_stats(obs):
    """obs: (n, 6) data.out columns 2-7 in file order -> (mean[6], var[6], n)."""
    obs = np.asarray(obs, dtype=np.float64)
    n = len(obs)
    s = np.zeros(6)
    s2 = np.zeros(6)
    for row in obs:  # awk adds line by line
        s += row
        s2 += row * row
    mean = s / n
    return mean, s2 / n - mean * mean, n


def isobar_point(L, T, mean, var, n):
    N = float(L) * L * L
    m, v = mean, var
    err = lambda k, scale: math.sqrt(3 * v[k] / n) / scale  # noqa: E731
    return {
        "T": T,
        "energy": m[0] / N, "energy_err": err(0, N),
        "enthalpy": m[1] / N, "enthalpy_err": err(1, N),
        "volume": m[2] / N, "volume_err": err(2, N),
        "density": N / m[2], "density_err": N * math.sqrt(3 * v[2] / n) / (m[2] * m[2]),
        "nhb": m[3] / (2 * N), "nhb_err": err(3, 2 * N),
        "ncoop": m[4], "ncoop_err": math.sqrt(3 * v[4] / n),
        "rcell": m[5], "rcell_err": math.sqrt(v[5] / n),
        "cp_fluc": v[1] / (T * T * float(L) * L * L),
        "kt_fluc": v[2] / (T * m[2]),
    }


def to_si(p, P):
    T = p["T"]
    rho = p["density"] * RHOS + RHOI
    rho_err = p["density_err"] * RHOS
    h = p["enthalpy"] * HS + HI * T
    h_err = p["enthalpy_err"] * HI
    return {
        "T_K": T * TS + TI,
        "density": rho, "density_err": rho_err,
        "enthalpy": h, "enthalpy_err": h_err,
        "energy": h - 18 * (P * PS + PI) / rho,
        "energy_err": h_err - 18 * (P * PS + PI) * rho_err / (rho * rho),
        "cp_fluc": p["cp_fluc"] * CPS + CPI, "cp_fluc_err": 0.0,
        "nhb": p["nhb"], "nhb_err": p["nhb_err"], "ncoop": p["ncoop"], "ncoop_err": p["ncoop_err"],
    }


def alpha_p(T, V, V2, n):
    """AlphaPderivate.c on arrays (any order): returns the rows (T, alpha_P, error) it writes."""
    T, V, V2, n = (np.asarray(a, dtype=np.float64) for a in (T, V, V2, n))
    o = np.argsort(T, kind="stable")
    T, V, V2, n = T[o], V[o], V2[o], n[o]
    m = len(T)
    if m < 2:
        return []
    ap = np.empty(m)
    ev = np.empty(m)
    for j in range(m):
        if j == 0:
            ap[j] = (V[j + 1] - V[j]) / (T[j + 1] - T[j])
        elif j == m - 1:
            ap[j] = (V[j] - V[j - 1]) / (T[j] - T[j - 1])
        else:
            ap[j] = (V[j + 1] - V[j - 1]) / (T[j + 1] - T[j - 1])
        ap[j] *= 1.0 / V[j]
        ev[j] = math.sqrt((V2[j] / n[j]) * 3)
    rows = []
    for j in range(2, m - 2):
        dT = (T[j + 1] - T[j - 1]) / 2.0
        der = abs(V[j + 2] / 2.0 - V[j + 1] + V[j - 1] - V[j - 2] / 2.0) / (dT * dT * dT)
        der *= dT * dT / 6.0
        est = (ev[j + 1] + ev[j - 1]) / (2.0 * dT)
        e = math.sqrt(ap[j] * ap[j] * ev[j] * ev[j] / (V[j] * V[j]) + der * der / (V[j] * V[j])
                      + est * est / (V[j] * V[j]))
        rows.append((T[j], ap[j], e))
    return rows


def awk_g(x):
    """awk's print of a computed number: integers as integers, otherwise %.6g."""
    if x == int(x) and abs(x) < 1e16:
        return str(int(x))
    return "%.6g" % x


def density_si_text(T, rho, err):
    """conversor.sh:20 on one density.dat line (the fields as text) -> the three printed fields."""
    return [awk_g(float(T) * TS + TI), awk_g(float(rho) * RHOS + RHOI), awk_g(float(err) * RHOS)]


def alpha_p_text(si_lines, n=1, derivative=alpha_p):
    """conversor.sh:54-66 on one isobar's density.dat.SI lines [(T_K, rho, err) as text]; the
    sample count n cancels from the error up to the %.6g rounding. Returns the printed lines."""
    T, V, V2, N = [], [], [], []
    for t, r, e in si_lines:
        r, e = float(r), float(e)
        v = awk_g(1.0 / r)
        x = awk_g(e * e / (3 * r * r * r * r))
        T.append(float(t))
        V.append(float(v))
        V2.append(float(awk_g(float(x) * n)))
        N.append(float(n))
    out = []
    for t, a, e in derivative(T, V, V2, N):
        ts, as_, es = "%f" % t, "%f" % a, "%f" % e
        if as_ in ("-nan", "nan", "inf", "-inf") or es == "inf":
            continue
        out.append((ts, awk_g(float(as_) * 1000), awk_g(float(es) * 1000)))
    return out


def cp_derivative(T, H, H2, n):
    """CPderivate.c on arrays (any order): the rows (T, C_P, error) it writes."""
    T, H, H2, n = (np.asarray(a, dtype=np.float64) for a in (T, H, H2, n))
    o = np.argsort(T, kind="stable")
    T, H, H2, n = T[o], H[o], H2[o], n[o]
    m = len(T)
    if m < 2:
        return []
    cp = np.empty(m)
    eh = np.empty(m)
    for j in range(m):
        if j == 0:
            cp[j] = (H[j + 1] - H[j]) / (T[j + 1] - T[j])
        elif j == m - 1:
            cp[j] = (H[j] - H[j - 1]) / (T[j] - T[j - 1])
        else:
            cp[j] = (H[j + 1] - H[j - 1]) / (T[j + 1] - T[j - 1])
        eh[j] = math.sqrt((H2[j] / n[j]) * 3)
    rows = []
    for j in range(2, m - 2):
        dT = (T[j + 1] - T[j - 1]) / 2.0
        der = abs(H[j + 2] / 2.0 - H[j + 1] + H[j - 1] - H[j - 2] / 2.0) / (dT * dT * dT)
        der *= dT * dT / 6.0
        est = (eh[j + 1] + eh[j - 1]) / (2.0 * dT)
        rows.append((T[j], cp[j], math.sqrt(der * der + est * est)))
    return rows


KT_NOT_VALUE, GAS_DENS = -10.0, 500


def kt_derivative(T, P, rho, Erho):
    """KTderivate.c's K_T and its error for every point (lists), KT_NOT_VALUE where none."""
    m = len(T)

    def near(j, lo, hi):
        up = dn = -1
        Pup, Pdn = 1e12, -1e12
        for i in range(m):
            if i == j or not abs(T[i] - T[j]) < 1e-8:
                continue
            if P[i] > hi and P[i] < Pup:
                Pup, up = P[i], i
            if P[i] < lo and P[i] > Pdn:
                Pdn, dn = P[i], i
        return up, dn, Pup, Pdn

    nb = []
    for j in range(m):
        up, dn, Pup, Pdn = near(j, P[j], P[j])
        up2, dn2, Pup2, Pdn2 = near(j, Pdn, Pup)
        nb.append((up, dn, Pup, Pdn, up2, dn2, Pup2, Pdn2))
    KT, EKT = [KT_NOT_VALUE] * m, [KT_NOT_VALUE] * m
    for j in range(m):
        up, dn, Pup, Pdn = nb[j][:4]
        d, p = rho[j], P[j]
        if d < GAS_DENS or (up == -1 and dn == -1):
            continue
        if up == -1:
            if rho[dn] < GAS_DENS:
                continue
            KT[j] = (math.log(d) - math.log(rho[dn])) / (p - Pdn)
            EKT[j] = abs(Erho[j] / d + Erho[dn] / rho[dn]) / (p - Pdn)
        elif dn == -1:
            if rho[up] < GAS_DENS:
                continue
            KT[j] = (math.log(rho[up]) - math.log(d)) / (Pup - p)
            EKT[j] = abs(Erho[j] / d + Erho[up] / rho[up]) / (Pup - p)
        else:
            if rho[up] < GAS_DENS or rho[dn] < GAS_DENS:
                continue
            KT[j] = (math.log(rho[up]) - math.log(rho[dn])) / (Pup - Pdn)
            EKT[j] = abs(Erho[dn] / rho[dn] + Erho[up] / rho[up]) / (Pup - Pdn)
    for j in range(m):
        up, dn, Pup, Pdn, up2, dn2, Pup2, Pdn2 = nb[j]
        if KT[j] == KT_NOT_VALUE or EKT[j] == KT_NOT_VALUE:
            continue
        if up2 != -1 and dn2 != -1:
            if min(rho[up2], rho[up], rho[dn2], rho[dn]) < GAS_DENS:
                continue
            dP2 = (Pup2 - Pdn2) / 4.0
            der = abs(0.5 * math.log(rho[up2]) - math.log(rho[up]) + math.log(rho[dn]) - 0.5 * math.log(rho[dn2])) / (6.0 * dP2)
        elif up != -1 and dn != -1:
            if KT[up] == KT_NOT_VALUE or KT[dn] == KT_NOT_VALUE:
                continue
            der = abs(KT[dn] - 2 * KT[j] + KT[up]) / 6.0
        else:
            continue
        EKT[j] = math.sqrt(EKT[j] * EKT[j] + der * der)
    return KT, EKT


def kt_files(points, isobars, derivative=kt_derivative):
    """KTderivate.c:77-123 on the KT_input points [(T_K, P_MPa, rho, err) as text] and the isobar
    list (MPa, as text): {"%lf" of the isobar: the lines it writes to P%lf_KTderivate.dat}."""
    T = [float(t) for t, _, _, _ in points]
    P = [float(p) for _, p, _, _ in points]
    rho = [float(r) for _, _, r, _ in points]
    err = [float(e) for _, _, _, e in points]
    KT, EKT = derivative(T, P, rho, err)
    out = {}
    for iso in isobars:
        pv = float(iso)
        out["%f" % pv] = ["%f %f %e %f" % (T[k], KT[k], EKT[k], P[k]) for k in range(len(points))
                          if KT[k] != KT_NOT_VALUE and abs(P[k] - pv) < 1e-5]
    return out


def kt_text(points, isobars, derivative=kt_derivative):
    """conversor.sh:84-119: the KTderivate files of kt_files after awk '{print $1, $2*1000,
    $3*1000, $4}' and sort -g: {isobar "%lf": [(T, K_T, error, P) as printed]}."""
    out = {}
    for name, lines in kt_files(points, isobars, derivative).items():
        rows = []
        for line in lines:
            t, kt, ekt, p = line.split()
            rows.append((t, awk_g(float(kt) * 1000), awk_g(float(ekt) * 1000), p))
        rows.sort(key=lambda r: (float(r[0]), r))  # sort -g
        out[name] = rows
    return out
