// Multiple-histogram (binless, per-sample) reweighting in FP64 and its hand-written adjoint.
//
// Replaces the Fortran Calcula_Histograma (HistogramReweighting/histogram_reweighting_mixed_
// paramSI_norm_x.f90:1003-1124, self-consistent constants :450-473) and the finite differences
// of CVF_ThermodynamicAnalysis/{AlphaP,CP,KT}derivate.c. With H_j(k) = E_k + P_j V_k:
//   D_k       = sum_j n_j exp(f_j - beta_j H_j(k)),            f_j = -log Z_j   (log-sum-exp)
//   f_i      <- f_i - log sum_k exp(f_i - beta_i H_i(k) - log D_k)   (each term <= -log n_i)
//   log w_k   = -beta (E'_k + P V'_k) - log D_k at the target theta = (beta, P, dJ_hb, dJ_s, dv_hb),
//               E' = E - dJ_hb N_hb - dJ_s N_s, V' = V + dv_hb N_hb
//   <A>       = sum_k A_k w_k / sum_k w_k
// The adjoint returns sum_m g_m d<A_m>/d theta = <g.dA> + <s dlogw> - <s><dlogw>, s = g.A.
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/cvf.h"

namespace cvf {

constexpr int kRwThreads = 256;
constexpr int kRwMaxRuns = 256;
constexpr int kRwMaxObs = 16;

__device__ __forceinline__ unsigned long long order_bits(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_order_bits(unsigned long long b) {
  return __longlong_as_double((long long)((b >> 63) ? (b & 0x7fffffffffffffffull) : ~b));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// log D_k for every sample and s_i = sum_k exp(f_i - beta_i H_i(k) - log D_k) for every run.
__global__ void __launch_bounds__(kRwThreads) k_rw_logD(const double* __restrict__ samp, long long n,
                                                        const double* __restrict__ runs, const double* __restrict__ logn,
                                                        const double* __restrict__ f, int nr, double* __restrict__ logD,
                                                        double* __restrict__ s_out) {
  __shared__ double s_b[kRwMaxRuns], s_p[kRwMaxRuns], s_c[kRwMaxRuns], s_acc[kRwMaxRuns];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    s_b[i] = runs[2 * i];
    s_p[i] = runs[2 * i + 1];
    s_c[i] = logn[i] + f[i];
    s_acc[i] = 0.0;
  }
  __syncthreads();
  for (long long k0 = (long long)blockIdx.x * blockDim.x; k0 < n; k0 += (long long)gridDim.x * blockDim.x) {
    long long k = k0 + threadIdx.x;
    bool ok = k < n;
    double E = 0, V = 0, ld = 0;
    if (ok) {
      E = samp[4 * k];
      V = samp[4 * k + 1];
      double m = -INFINITY;
      for (int j = 0; j < nr; ++j) m = fmax(m, s_c[j] - s_b[j] * (E + s_p[j] * V));
      double sum = 0.0;
      for (int j = 0; j < nr; ++j) sum += exp(s_c[j] - s_b[j] * (E + s_p[j] * V) - m);
      ld = m + log(sum);
      logD[k] = ld;
    }
    for (int i = 0; i < nr; ++i) {
      double u = ok ? exp(f[i] - s_b[i] * (E + s_p[i] * V) - ld) : 0.0;
      u = warp_sum(u);
      if ((threadIdx.x & 31) == 0) atomicAdd(&s_acc[i], u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) atomicAdd(&s_out[i], s_acc[i]);
}

// The same sums in log space, for runs whose sum underflowed: pass 0 takes every run's maximum
// of a_ik = f_i - beta_i H_i(k) - log D_k into mx (order bits), pass 1 adds exp(a_ik - max_i).
__global__ void __launch_bounds__(kRwThreads) k_rw_runlse(const double* __restrict__ samp, long long n,
                                                          const double* __restrict__ runs,
                                                          const double* __restrict__ f, int nr,
                                                          const double* __restrict__ logD, int pass,
                                                          unsigned long long* __restrict__ mx,
                                                          double* __restrict__ s_out) {
  __shared__ double s_b[kRwMaxRuns], s_p[kRwMaxRuns], s_f[kRwMaxRuns], s_m[kRwMaxRuns], s_acc[kRwMaxRuns];
  __shared__ unsigned long long s_mx[kRwMaxRuns];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    s_b[i] = runs[2 * i];
    s_p[i] = runs[2 * i + 1];
    s_f[i] = f[i];
    s_mx[i] = 0ull;
    s_acc[i] = 0.0;
    if (pass == 1) {
      const unsigned long long b = mx[i];
      s_m[i] = __longlong_as_double((long long)((b >> 63) ? (b & 0x7fffffffffffffffull) : ~b));
    }
  }
  __syncthreads();
  for (long long k0 = (long long)blockIdx.x * blockDim.x; k0 < n; k0 += (long long)gridDim.x * blockDim.x) {
    const long long k = k0 + threadIdx.x;
    const bool ok = k < n;
    const double E = ok ? samp[4 * k] : 0.0, V = ok ? samp[4 * k + 1] : 0.0, ld = ok ? logD[k] : 0.0;
    for (int i = 0; i < nr; ++i) {
      const double a = s_f[i] - s_b[i] * (E + s_p[i] * V) - ld;
      if (pass == 0) {
        double m = ok ? a : -INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) atomicMax(&s_mx[i], order_bits(m));
      } else {
        double u = ok ? exp(a - s_m[i]) : 0.0;
        u = warp_sum(u);
        if ((threadIdx.x & 31) == 0) atomicAdd(&s_acc[i], u);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    if (pass == 0) atomicMax(&mx[i], s_mx[i]);
    else atomicAdd(&s_out[i], s_acc[i]);
  }
}

struct Target {
  double beta, P, dJhb, dJs, dvhb, ncells;
};

__device__ __forceinline__ void primed(const double* s, const Target& t, double& E, double& V) {
  E = s[0] - t.dJhb * s[2] - t.dJs * s[3];
  V = s[1] + t.dvhb * s[2];
}

__device__ __forceinline__ double obs_value(int id, const double* s, double E, double V, const Target& t) {
  double H = E + t.P * V;
  switch (id) {
    case CVF_RW_E: return E;
    case CVF_RW_V: return V;
    case CVF_RW_NHB: return s[2];
    case CVF_RW_NSIG: return s[3];
    case CVF_RW_H: return H;
    case CVF_RW_RHO: return t.ncells / V;
    case CVF_RW_H2: return H * H;
    case CVF_RW_V2: return V * V;
    default: return V * H;  // CVF_RW_VH
  }
}

// d A / d theta for theta = (beta, P, dJ_hb, dJ_s, dv_hb) at fixed sample.
__device__ __forceinline__ void obs_grad(int id, const double* s, double E, double V, const Target& t, double* g) {
  double H = E + t.P * V;
  double dE[5] = {0, 0, -s[2], -s[3], 0};
  double dV[5] = {0, 0, 0, 0, s[2]};
  double dH[5];
  for (int p = 0; p < 5; ++p) dH[p] = dE[p] + t.P * dV[p];
  dH[1] += V;
  for (int p = 0; p < 5; ++p) {
    switch (id) {
      case CVF_RW_E: g[p] = dE[p]; break;
      case CVF_RW_V: g[p] = dV[p]; break;
      case CVF_RW_NHB:
      case CVF_RW_NSIG: g[p] = 0.0; break;
      case CVF_RW_H: g[p] = dH[p]; break;
      case CVF_RW_RHO: g[p] = -t.ncells * dV[p] / (V * V); break;
      case CVF_RW_H2: g[p] = 2.0 * H * dH[p]; break;
      case CVF_RW_V2: g[p] = 2.0 * V * dV[p]; break;
      default: g[p] = dV[p] * H + V * dH[p]; break;
    }
  }
}

__global__ void __launch_bounds__(kRwThreads) k_rw_max(const double* __restrict__ samp, long long n,
                                                       const double* __restrict__ logD, Target t,
                                                       unsigned long long* __restrict__ mx) {
  double m = -INFINITY;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double E, V;
    primed(samp + 4 * k, t, E, V);
    m = fmax(m, -t.beta * (E + t.P * V) - logD[k]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, order_bits(m));
}

// acc[0] = sum w, acc[1+m] = sum w A_m with w = exp(log w_k - max).
__global__ void __launch_bounds__(kRwThreads) k_rw_sum(const double* __restrict__ samp, long long n,
                                                       const double* __restrict__ logD, Target t,
                                                       const unsigned long long* __restrict__ mx,
                                                       const int* __restrict__ ids, int nobs, double* __restrict__ acc) {
  __shared__ double s_acc[kRwMaxObs + 1];
  __shared__ int s_ids[kRwMaxObs];
  if (threadIdx.x <= nobs) s_acc[threadIdx.x] = 0.0;
  if (threadIdx.x < nobs) s_ids[threadIdx.x] = ids[threadIdx.x];
  __syncthreads();
  const double M = from_order_bits(*mx);
  for (long long k0 = (long long)blockIdx.x * blockDim.x; k0 < n; k0 += (long long)gridDim.x * blockDim.x) {
    long long k = k0 + threadIdx.x;
    double w = 0.0, E = 0.0, V = 1.0;
    if (k < n) {
      primed(samp + 4 * k, t, E, V);
      w = exp(-t.beta * (E + t.P * V) - logD[k] - M);
    }
    double v = warp_sum(w);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s_acc[0], v);
    for (int m = 0; m < nobs; ++m) {
      double a = k < n ? w * obs_value(s_ids[m], samp + 4 * k, E, V, t) : 0.0;
      a = warp_sum(a);
      if ((threadIdx.x & 31) == 0) atomicAdd(&s_acc[1 + m], a);
    }
  }
  __syncthreads();
  if (threadIdx.x <= nobs) atomicAdd(&acc[threadIdx.x], s_acc[threadIdx.x]);
}

// acc[0..4] = sum w s dlogw, acc[5..9] = sum w dlogw, acc[10] = sum w s, acc[11..15] = sum w g.dA
__global__ void __launch_bounds__(kRwThreads) k_rw_adjoint(const double* __restrict__ samp, long long n,
                                                           const double* __restrict__ logD, Target t,
                                                           const unsigned long long* __restrict__ mx, double inv_z,
                                                           const int* __restrict__ ids, const double* __restrict__ gw,
                                                           int nobs, double* __restrict__ acc) {
  __shared__ double s_acc[16];
  __shared__ int s_ids[kRwMaxObs];
  __shared__ double s_g[kRwMaxObs];
  if (threadIdx.x < 16) s_acc[threadIdx.x] = 0.0;
  if (threadIdx.x < nobs) {
    s_ids[threadIdx.x] = ids[threadIdx.x];
    s_g[threadIdx.x] = gw[threadIdx.x];
  }
  __syncthreads();
  const double M = from_order_bits(*mx);
  for (long long k0 = (long long)blockIdx.x * blockDim.x; k0 < n; k0 += (long long)gridDim.x * blockDim.x) {
    long long k = k0 + threadIdx.x;
    double loc[16];
    for (int i = 0; i < 16; ++i) loc[i] = 0.0;
    if (k < n) {
      const double* s = samp + 4 * k;
      double E, V;
      primed(s, t, E, V);
      double H = E + t.P * V;
      double w = exp(-t.beta * H - logD[k] - M) * inv_z;
      double dl[5] = {-H, -t.beta * V, t.beta * s[2], t.beta * s[3], -t.beta * t.P * s[2]};
      double sg = 0.0, gd[5] = {0, 0, 0, 0, 0};
      for (int m = 0; m < nobs; ++m) {
        sg += s_g[m] * obs_value(s_ids[m], s, E, V, t);
        double g[5];
        obs_grad(s_ids[m], s, E, V, t, g);
        for (int p = 0; p < 5; ++p) gd[p] += s_g[m] * g[p];
      }
      for (int p = 0; p < 5; ++p) {
        loc[p] = w * sg * dl[p];
        loc[5 + p] = w * dl[p];
        loc[11 + p] = w * gd[p];
      }
      loc[10] = w * sg;
    }
    for (int i = 0; i < 16; ++i) {
      double v = warp_sum(loc[i]);
      if ((threadIdx.x & 31) == 0) atomicAdd(&s_acc[i], v);
    }
  }
  __syncthreads();
  if (threadIdx.x < 16) atomicAdd(&acc[threadIdx.x], s_acc[threadIdx.x]);
}

}  // namespace cvf

using namespace cvf;

namespace cvf {
void set_last_error(const std::string& m);
}

namespace {

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

int rw_fail(int code, const std::string& m) {
  cvf::set_last_error(m);
  return code;
}

#define RWCK(call)                                                                              \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return rw_fail(CVF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct RwSetup {
  DevBuf samp, logD, runs, logn, f, acc, mx, ids, g, runmx;
  long long n;
  int nr, grid;
};

int rw_prepare(RwSetup& S, int device, const double* samples, const int* run_of, long long n, const double* runs,
               int n_runs, const double* f, const int* obs_ids, int n_obs) {
  if (!samples || !run_of || !runs || !f || n < 1 || n_runs < 1 || n_runs > kRwMaxRuns || n_obs < 0 ||
      n_obs > kRwMaxObs)
    return rw_fail(CVF_EINVAL, "reweight: bad sizes (1 <= n_runs <= 256, n_obs <= 16)");
  for (int m = 0; m < n_obs; ++m)
    if (obs_ids[m] < 0 || obs_ids[m] > CVF_RW_VH) return rw_fail(CVF_EINVAL, "reweight: unknown observable id");
  std::vector<double> logn(n_runs, 0.0);
  std::vector<long long> cnt(n_runs, 0);
  for (long long k = 0; k < n; ++k) {
    if (run_of[k] < 0 || run_of[k] >= n_runs) return rw_fail(CVF_EINVAL, "reweight: run_of out of range");
    cnt[run_of[k]]++;
  }
  for (int i = 0; i < n_runs; ++i) {
    if (!cnt[i]) return rw_fail(CVF_EINVAL, "reweight: a run has no samples");
    logn[i] = log((double)cnt[i]);
  }
  RWCK(cudaSetDevice(device));
  S.n = n;
  S.nr = n_runs;
  int sms = 0;
  RWCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  long long blocks = (n + kRwThreads - 1) / kRwThreads;
  S.grid = (int)(blocks < 4LL * sms ? blocks : 4LL * sms);
  RWCK(cudaMalloc(&S.samp.p, (size_t)n * 4 * sizeof(double)));
  RWCK(cudaMalloc(&S.logD.p, (size_t)n * sizeof(double)));
  RWCK(cudaMalloc(&S.runs.p, (size_t)n_runs * 2 * sizeof(double)));
  RWCK(cudaMalloc(&S.logn.p, (size_t)n_runs * sizeof(double)));
  RWCK(cudaMalloc(&S.f.p, (size_t)n_runs * sizeof(double)));
  RWCK(cudaMalloc(&S.acc.p, (size_t)(kRwMaxRuns + 32) * sizeof(double)));
  RWCK(cudaMalloc(&S.runmx.p, (size_t)kRwMaxRuns * sizeof(unsigned long long)));
  RWCK(cudaMalloc(&S.mx.p, sizeof(unsigned long long)));
  RWCK(cudaMalloc(&S.ids.p, kRwMaxObs * sizeof(int)));
  RWCK(cudaMalloc(&S.g.p, kRwMaxObs * sizeof(double)));
  RWCK(cudaMemcpy(S.samp.p, samples, (size_t)n * 4 * sizeof(double), cudaMemcpyHostToDevice));
  RWCK(cudaMemcpy(S.runs.p, runs, (size_t)n_runs * 2 * sizeof(double), cudaMemcpyHostToDevice));
  RWCK(cudaMemcpy(S.logn.p, logn.data(), (size_t)n_runs * sizeof(double), cudaMemcpyHostToDevice));
  RWCK(cudaMemcpy(S.f.p, f, (size_t)n_runs * sizeof(double), cudaMemcpyHostToDevice));
  if (n_obs) RWCK(cudaMemcpy(S.ids.p, obs_ids, n_obs * sizeof(int), cudaMemcpyHostToDevice));
  return 0;
}

// One pass of log D_k (and the WHAM sums); optionally refines f in place (host array too).
int rw_pass(RwSetup& S, double* f_host, bool update, double* max_change) {
  RWCK(cudaMemset(S.acc.p, 0, S.nr * sizeof(double)));
  k_rw_logD<<<S.grid, kRwThreads>>>((const double*)S.samp.p, S.n, (const double*)S.runs.p,
                                     (const double*)S.logn.p, (const double*)S.f.p, S.nr, (double*)S.logD.p,
                                     (double*)S.acc.p);
  RWCK(cudaGetLastError());
  if (!update) return 0;
  std::vector<double> s(S.nr), logs(S.nr);
  RWCK(cudaMemcpy(s.data(), S.acc.p, S.nr * sizeof(double), cudaMemcpyDeviceToHost));
  bool under = false;
  for (int i = 0; i < S.nr; ++i) {
    under = under || !(s[i] > 0.0) || !std::isfinite(s[i]);
    logs[i] = log(s[i]);
  }
  if (under) {
    // a run far from every sample (free energies still far from converged): the same sums in
    // log space, max_i + log sum_k exp(a_ik - max_i)
    RWCK(cudaMemset(S.runmx.p, 0, S.nr * sizeof(unsigned long long)));
    RWCK(cudaMemset(S.acc.p, 0, S.nr * sizeof(double)));
    for (int pass = 0; pass < 2; ++pass)
      k_rw_runlse<<<S.grid, kRwThreads>>>((const double*)S.samp.p, S.n, (const double*)S.runs.p,
                                           (const double*)S.f.p, S.nr, (const double*)S.logD.p, pass,
                                           (unsigned long long*)S.runmx.p, (double*)S.acc.p);
    RWCK(cudaGetLastError());
    std::vector<unsigned long long> mb(S.nr);
    RWCK(cudaMemcpy(mb.data(), S.runmx.p, S.nr * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    RWCK(cudaMemcpy(s.data(), S.acc.p, S.nr * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < S.nr; ++i) {
      const unsigned long long raw = (mb[i] >> 63) ? (mb[i] & 0x7fffffffffffffffull) : ~mb[i];
      double m;
      memcpy(&m, &raw, 8);
      logs[i] = m + log(s[i]);
    }
  }
  std::vector<double> nf(S.nr);
  for (int i = 0; i < S.nr; ++i) nf[i] = f_host[i] - logs[i];
  double c = nf[0], mc = 0.0;
  for (int i = 0; i < S.nr; ++i) {
    nf[i] -= c;
    const double d = fabs(nf[i] - f_host[i]);
    mc = d > mc || d != d ? d : mc;  // a NaN change never reads as converged
    f_host[i] = nf[i];
  }
  if (!std::isfinite(mc)) return rw_fail(CVF_ELIMIT, "reweight: the free energies are not finite");
  *max_change = mc;
  RWCK(cudaMemcpy(S.f.p, f_host, S.nr * sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

int rw_target(RwSetup& S, const Target& t, int n_obs, double* acc_host) {
  unsigned long long init = 0;
  RWCK(cudaMemcpy(S.mx.p, &init, sizeof(init), cudaMemcpyHostToDevice));
  k_rw_max<<<S.grid, kRwThreads>>>((const double*)S.samp.p, S.n, (const double*)S.logD.p, t,
                                    (unsigned long long*)S.mx.p);
  RWCK(cudaMemset(S.acc.p, 0, (kRwMaxObs + 1) * sizeof(double)));
  k_rw_sum<<<S.grid, kRwThreads>>>((const double*)S.samp.p, S.n, (const double*)S.logD.p, t,
                                    (const unsigned long long*)S.mx.p, (const int*)S.ids.p, n_obs, (double*)S.acc.p);
  RWCK(cudaGetLastError());
  RWCK(cudaMemcpy(acc_host, S.acc.p, (n_obs + 1) * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

Target make_target(const double* theta, double ncells) {
  Target t;
  t.beta = theta[0];
  t.P = theta[1];
  t.dJhb = theta[2];
  t.dJs = theta[3];
  t.dvhb = theta[4];
  t.ncells = ncells;
  return t;
}

double host_max(RwSetup& S) {
  unsigned long long b = 0;
  cudaMemcpy(&b, S.mx.p, sizeof(b), cudaMemcpyDeviceToHost);
  unsigned long long raw = (b >> 63) ? (b & 0x7fffffffffffffffull) : ~b;
  double d;
  memcpy(&d, &raw, 8);
  return d;
}
}  // namespace

// Starting free energies when the caller gives none (all zero): thermodynamic integration of
// d f = <E> d beta + <V> d(beta P) between consecutive runs in (beta, beta P) order, trapezoids
// of the runs' own means, made relative to run 0. WHAM then refines them.
static void ti_start(const double* samples, const int* run_of, long long n, const double* runs, int nr, double* f) {
  std::vector<double> se(nr, 0.0), sv(nr, 0.0);
  std::vector<long long> c(nr, 0);
  for (long long k = 0; k < n; ++k) {
    se[run_of[k]] += samples[4 * k];
    sv[run_of[k]] += samples[4 * k + 1];
    c[run_of[k]]++;
  }
  std::vector<int> o(nr);
  for (int i = 0; i < nr; ++i) {
    o[i] = i;
    se[i] /= (double)c[i];
    sv[i] /= (double)c[i];
  }
  std::stable_sort(o.begin(), o.end(), [&](int a, int b) {
    const double ba = runs[2 * a], bb = runs[2 * b];
    return ba < bb || (ba == bb && ba * runs[2 * a + 1] < bb * runs[2 * b + 1]);
  });
  f[o[0]] = 0.0;
  for (int q = 1; q < nr; ++q) {
    const int a = o[q - 1], b = o[q];
    const double db = runs[2 * b] - runs[2 * a];
    const double dbp = runs[2 * b] * runs[2 * b + 1] - runs[2 * a] * runs[2 * a + 1];
    f[b] = f[a] + 0.5 * (se[a] + se[b]) * db + 0.5 * (sv[a] + sv[b]) * dbp;
  }
  const double f0 = f[0];
  for (int i = 0; i < nr; ++i) f[i] -= f0;
}

extern "C" int cvf_reweight_forward(int device, const double* samples, const int* run_of, long long n,
                                    const double* runs, int n_runs, double* f, int n_iter, double tol,
                                    double n_cells, const double* theta, const int* obs_ids, int n_obs,
                                    double* out) {
  RwSetup S;
  if (f && samples && run_of && runs && n > 0 && n_runs > 0 && n_runs <= kRwMaxRuns && n_iter > 0) {
    bool zero = true;
    for (int i = 0; i < n_runs; ++i) zero = zero && f[i] == 0.0;
    bool ok = true;
    for (long long k = 0; k < n && ok; ++k) ok = run_of[k] >= 0 && run_of[k] < n_runs;
    if (zero && ok) {
      std::vector<long long> cnt(n_runs, 0);
      for (long long k = 0; k < n; ++k) cnt[run_of[k]]++;
      for (int i = 0; i < n_runs; ++i) ok = ok && cnt[i] > 0;
      if (ok) ti_start(samples, run_of, n, runs, n_runs, f);
    }
  }
  if (int rc = rw_prepare(S, device, samples, run_of, n, runs, n_runs, f, obs_ids, n_obs)) return rc;
  for (int it = 0; it < n_iter; ++it) {
    double mc = 0.0;
    if (int rc = rw_pass(S, f, true, &mc)) return rc;
    if (mc < tol) break;
  }
  if (int rc = rw_pass(S, f, false, nullptr)) return rc;
  if (!theta || !out) return 0;
  Target t = make_target(theta, n_cells);
  double acc[kRwMaxObs + 1];
  if (int rc = rw_target(S, t, n_obs, acc)) return rc;
  double M = host_max(S);
  for (int m = 0; m < n_obs; ++m) out[m] = acc[1 + m] / acc[0];
  out[n_obs] = M + log(acc[0]);
  return 0;
}

extern "C" int cvf_reweight_adjoint(int device, const double* samples, const int* run_of, long long n,
                                    const double* runs, int n_runs, const double* f, double n_cells,
                                    const double* theta, const int* obs_ids, int n_obs, const double* g,
                                    double* grad) {
  if (!theta || !g || !grad) return rw_fail(CVF_EINVAL, "reweight_adjoint: null theta/g/grad");
  RwSetup S;
  if (int rc = rw_prepare(S, device, samples, run_of, n, runs, n_runs, f, obs_ids, n_obs)) return rc;
  if (int rc = rw_pass(S, nullptr, false, nullptr)) return rc;
  Target t = make_target(theta, n_cells);
  double acc[kRwMaxObs + 1];
  if (int rc = rw_target(S, t, n_obs, acc)) return rc;
  RWCK(cudaMemcpy(S.g.p, g, n_obs * sizeof(double), cudaMemcpyHostToDevice));
  RWCK(cudaMemset(S.acc.p, 0, 16 * sizeof(double)));
  k_rw_adjoint<<<S.grid, kRwThreads>>>((const double*)S.samp.p, S.n, (const double*)S.logD.p, t,
                                        (const unsigned long long*)S.mx.p, 1.0 / acc[0], (const int*)S.ids.p,
                                        (const double*)S.g.p, n_obs, (double*)S.acc.p);
  RWCK(cudaGetLastError());
  double a[16];
  RWCK(cudaMemcpy(a, S.acc.p, 16 * sizeof(double), cudaMemcpyDeviceToHost));
  for (int p = 0; p < 5; ++p) grad[p] = a[11 + p] + a[p] - a[10] * a[5 + p];
  return 0;
}
