// Host part of the isobar analysis: the per-run isobar point of TA/calculadora.sh, the SI units
// of TA/conversor.sh and the finite-difference alpha_P of TA/AlphaPderivate.c (reference:
// CVF_ThermodynamicAnalysis/ of lcoronas/CVFBulkWater). The run statistics they start from are
// computed on the GPU (cvf_stats.cu). All arithmetic is double precision with every operation
// rounded separately (built with -ffp-contract=off), as the reference's awk and C compute.
#include <math.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/cvf.h"

namespace cvf {
void set_last_error(const std::string& m);
}

namespace {

int iso_fail(const std::string& m) {
  cvf::set_last_error(m);
  return CVF_EINVAL;
}

// conversor.sh:2-12
constexpr double kTs = 140.5678, kTi = 185.4676;
constexpr double kPs = 469.459, kPi = -211.15552;
constexpr double kRhos = 1527.3, kRhoi = -23.1017;
constexpr double kCPs = 4.455, kCPi = 3.56843;
constexpr double kHs = 11.272132, kHi = 9.028924;

}  // namespace

extern "C" {

// calculadora.sh:41-61 on one row of L<L>_average_data.dat (columns L P T <e> var ... n).
int cvf_isobar_point_from_stats(const cvf_run_stats* s, cvf_isobar_point* o) {
  if (!s || !o) return iso_fail("null stats/out");
  if (s->n < 1) return iso_fail("run statistics without samples");
  const double N = (double)s->L * (double)s->L * (double)s->L;
  const double n = (double)s->n, T = s->T;
  const double* m = s->mean;
  const double* v = s->var;
  o->T = T;
  o->energy = m[0] / N;
  o->energy_err = sqrt(3 * v[0] / n) / N;
  o->enthalpy = m[1] / N;
  o->enthalpy_err = sqrt(3 * v[1] / n) / N;
  o->volume = m[2] / N;
  o->volume_err = sqrt(3 * v[2] / n) / N;
  o->density = N / m[2];
  o->density_err = N * sqrt(3 * v[2] / n) / (m[2] * m[2]);
  o->nhb = m[3] / (2 * N);
  o->nhb_err = sqrt(3 * v[3] / n) / (2 * N);
  o->ncoop = m[4];
  o->ncoop_err = sqrt(3 * v[4] / n);
  o->rcell = m[5];
  o->rcell_err = sqrt(v[5] / n);
  const double L = (double)s->L;
  o->cp_fluc = v[1] / (T * T * L * L * L);  // the awk expression's order of products
  o->kt_fluc = v[2] / (T * m[2]);
  return 0;
}

// conversor.sh:20 (density), :24 (enthalpy), :28 (N_hb, ncoop), :32 (C_P), :76 (energy).
int cvf_isobar_point_to_si(const cvf_isobar_point* p, double P, cvf_isobar_point_si* o) {
  if (!p || !o) return iso_fail("null point/out");
  const double T = p->T;
  o->T_K = T * kTs + kTi;
  o->density = p->density * kRhos + kRhoi;
  o->density_err = p->density_err * kRhos;
  o->enthalpy = p->enthalpy * kHs + kHi * T;
  o->enthalpy_err = p->enthalpy_err * kHi;
  const double pv = 18 * (P * kPs + kPi);
  o->energy = o->enthalpy - pv / o->density;
  o->energy_err = o->enthalpy_err - pv * o->density_err / (o->density * o->density);
  o->cp_fluc = p->cp_fluc * kCPs + kCPi;
  o->cp_fluc_err = 0.0;
  o->nhb = p->nhb;
  o->nhb_err = p->nhb_err;
  o->ncoop = p->ncoop;
  o->ncoop_err = p->ncoop_err;
  return 0;
}

// AlphaPderivate.c:56-134.
int cvf_alpha_p_derivative(const double* T, const double* V, const double* V2, const long long* n, int m,
                           double* T_out, double* ap_out, double* err_out, int* m_out) {
  if (!T || !V || !V2 || !n || !T_out || !ap_out || !err_out || !m_out || m < 0)
    return iso_fail("null array or negative count");
  *m_out = 0;
  if (m < 2) return 0;
  for (int j = 0; j < m; ++j)
    if (n[j] < 1) return iso_fail("a point without samples");
  // ascending T; equal temperatures keep their input order
  std::vector<int> o((size_t)m);
  std::iota(o.begin(), o.end(), 0);
  std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return T[a] < T[b]; });
  std::vector<double> t(m), v(m), ap(m), ev(m);
  for (int j = 0; j < m; ++j) {
    t[j] = T[o[j]];
    v[j] = V[o[j]];
  }
  for (int j = 0; j < m; ++j) {
    if (j == 0) ap[j] = (v[j + 1] - v[j]) / (t[j + 1] - t[j]);
    else if (j == m - 1) ap[j] = (v[j] - v[j - 1]) / (t[j] - t[j - 1]);
    else ap[j] = (v[j + 1] - v[j - 1]) / (t[j + 1] - t[j - 1]);
    ap[j] *= 1. / v[j];
    ev[j] = sqrt((V2[o[j]] / (double)n[o[j]]) * 3);
  }
  int k = 0;
  for (int j = 2; j < m - 2; ++j) {
    const double dT = (t[j + 1] - t[j - 1]) / 2.0;
    double der = fabs(v[j + 2] / 2.0 - v[j + 1] + v[j - 1] - v[j - 2] / 2.0) / (dT * dT * dT);
    der *= dT * dT / 6.0;
    const double est = (ev[j + 1] + ev[j - 1]) / (2.0 * dT);
    const double vv = v[j] * v[j];
    T_out[k] = t[j];
    ap_out[k] = ap[j];
    err_out[k] = sqrt(ap[j] * ap[j] * ev[j] * ev[j] / vv + der * der / vv + est * est / vv);
    ++k;
  }
  *m_out = k;
  return 0;
}

// CPderivate.c:56-124: C_P = dH/dT along an isobar by central differences (one-sided at the
// ends), the error from the third derivative and the neighbours' sqrt(3 var / n); only points
// 2 .. n-3 are written.
int cvf_cp_derivative(const double* T, const double* H, const double* H2, const long long* n, int m, double* T_out,
                      double* cp_out, double* err_out, int* m_out) {
  if (!T || !H || !H2 || !n || !T_out || !cp_out || !err_out || !m_out || m < 0)
    return iso_fail("null array or negative count");
  *m_out = 0;
  if (m < 2) return 0;
  for (int j = 0; j < m; ++j)
    if (n[j] < 1) return iso_fail("a point without samples");
  std::vector<int> o((size_t)m);
  std::iota(o.begin(), o.end(), 0);
  std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return T[a] < T[b]; });
  std::vector<double> t(m), h(m), cp(m), eh(m);
  for (int j = 0; j < m; ++j) {
    t[j] = T[o[j]];
    h[j] = H[o[j]];
  }
  for (int j = 0; j < m; ++j) {
    if (j == 0) cp[j] = (h[j + 1] - h[j]) / (t[j + 1] - t[j]);
    else if (j == m - 1) cp[j] = (h[j] - h[j - 1]) / (t[j] - t[j - 1]);
    else cp[j] = (h[j + 1] - h[j - 1]) / (t[j + 1] - t[j - 1]);
    eh[j] = sqrt((H2[o[j]] / (double)n[o[j]]) * 3);
  }
  int k = 0;
  for (int j = 2; j < m - 2; ++j) {
    const double dT = (t[j + 1] - t[j - 1]) / 2.0;
    double der = fabs(h[j + 2] / 2.0 - h[j + 1] + h[j - 1] - h[j - 2] / 2.0) / (dT * dT * dT);
    der *= dT * dT / 6.0;
    const double est = (eh[j + 1] + eh[j - 1]) / (2.0 * dT);
    T_out[k] = t[j];
    cp_out[k] = cp[j];
    err_out[k] = sqrt(der * der + est * est);
    ++k;
  }
  *m_out = k;
  return 0;
}

// KTderivate.c:345-563 (compresibilidad_log, error_compresibilidad_log): for every point, K_T =
// d ln(rho) / dP along its isotherm (points whose T agrees within 1e-8) from the nearest
// pressures above and below (one-sided at the ends), with the error from the neighbours' density
// errors plus a third-derivative term (from the second neighbours when both exist, else from the
// neighbours' K_T). Points in the gas (rho < 500), alone on their isotherm or next to a gas point
// get CVF_KT_NOT_VALUE (-10) in both outputs.
int cvf_kt_derivative(const double* T, const double* P, const double* rho, const double* Erho, int m, double* KT,
                      double* EKT) {
  if (!T || !P || !rho || !Erho || !KT || !EKT || m < 0) return iso_fail("null array or negative count");
  const double kNot = -10.0, kGas = 500;
  struct Nb {
    int up = -1, dn = -1, up2 = -1, dn2 = -1;
    double Pup = 1E12, Pdn = -1E12, Pup2 = 1E12, Pdn2 = -1E12;
  };
  std::vector<Nb> nb((size_t)m);
  for (int j = 0; j < m; ++j) {
    Nb& b = nb[j];
    for (int i = 0; i < m; ++i) {
      if (i == j || !(fabs(T[i] - T[j]) < 1E-8)) continue;
      if (P[i] > P[j] && P[i] < b.Pup) {
        b.Pup = P[i];
        b.up = i;
      }
      if (P[i] < P[j] && P[i] > b.Pdn) {
        b.Pdn = P[i];
        b.dn = i;
      }
    }
    for (int i = 0; i < m; ++i) {
      if (i == j || !(fabs(T[i] - T[j]) < 1E-8)) continue;
      if (P[i] > b.Pup && P[i] < b.Pup2) {
        b.Pup2 = P[i];
        b.up2 = i;
      }
      if (P[i] < b.Pdn && P[i] > b.Pdn2) {
        b.Pdn2 = P[i];
        b.dn2 = i;
      }
    }
  }
  for (int j = 0; j < m; ++j) {
    const Nb& b = nb[j];
    const double d = rho[j], p = P[j];
    KT[j] = EKT[j] = kNot;
    if (d < kGas || (b.up == -1 && b.dn == -1)) continue;
    if (b.up == -1) {
      if (rho[b.dn] < kGas) continue;
      KT[j] = (log(d) - log(rho[b.dn])) / (p - b.Pdn);
      EKT[j] = fabs(Erho[j] / d + Erho[b.dn] / rho[b.dn]) / (p - b.Pdn);
    } else if (b.dn == -1) {
      if (rho[b.up] < kGas) continue;
      KT[j] = (log(rho[b.up]) - log(d)) / (b.Pup - p);
      EKT[j] = fabs(Erho[j] / d + Erho[b.up] / rho[b.up]) / (b.Pup - p);
    } else {
      if (rho[b.up] < kGas || rho[b.dn] < kGas) continue;
      KT[j] = (log(rho[b.up]) - log(rho[b.dn])) / (b.Pup - b.Pdn);
      EKT[j] = fabs(Erho[b.dn] / rho[b.dn] + Erho[b.up] / rho[b.up]) / (b.Pup - b.Pdn);
    }
  }
  for (int j = 0; j < m; ++j) {
    const Nb& b = nb[j];
    if (KT[j] == kNot || EKT[j] == kNot) continue;
    double der;
    if (b.up2 != -1 && b.dn2 != -1) {
      if (rho[b.up2] < kGas || rho[b.up] < kGas || rho[b.dn2] < kGas || rho[b.dn] < kGas) continue;
      const double dP2 = (b.Pup2 - b.Pdn2) / 4.0;
      der = fabs(0.5 * log(rho[b.up2]) - log(rho[b.up]) + log(rho[b.dn]) - 0.5 * log(rho[b.dn2])) / (6.0 * dP2);
    } else if (b.up != -1 && b.dn != -1) {
      if (KT[b.up] == kNot || KT[b.dn] == kNot) continue;
      der = fabs(KT[b.dn] - 2 * KT[j] + KT[b.up]) / (6.0);
    } else {
      continue;
    }
    EKT[j] = sqrt(EKT[j] * EKT[j] + der * der);
  }
  return 0;
}

}  // extern "C"
