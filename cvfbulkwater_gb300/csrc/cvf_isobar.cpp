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

}  // extern "C"
