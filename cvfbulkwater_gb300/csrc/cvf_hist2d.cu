// Binned 2-D (E, rho) histogram reweighting of the reference's
// HistogramReweighting/histogram_reweighting_mixed_paramSI_norm_x.f90 ("F90"): the per-run 2-D
// histograms of energy and density in SI units, the constants of the runs by the F90's own
// iteration, the reweighted distribution at any (T, P), the Binder cumulants of E, rho and of the
// mixed order parameter M = sin(a) E + cos(a) rho. The bins are reweighted on the GPU -- one
// thread per bin, all runs' log-sum-exp in registers, every target (T, P) of a WHAM step in one
// launch -- and reduced in a fixed order, so results do not depend on scheduling. The 1-D stages
// (mixed-parameter histogram of ~sqrt(n_bin2D) bins, Binder sums) run on the host.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/cvf.h"
#include "cvf_device.cuh"

namespace cvf {
void set_last_error(const std::string& m);
}

struct cvf_h2d {
  int device = 0;
  cudaStream_t s = nullptr;
  int L = 0, R = 0, nb = 0, nbm = 0;
  double N = 0, Emin = 0, Dmin = 0, dE = 0, dD = 0;
  std::vector<double> That, Phat, Tk, Pbar, log_medidas, ctes;
  double* d_hsum = nullptr;   // nb*nb: sum over runs of count / (in-range count * bin area)
  double* d_logp = nullptr;   // R*nb*nb: log P of the current targets
  double* d_run = nullptr;    // 4R: beta_j, pres_j, ctes_j, log_medidas_j
  double* d_tgt = nullptr;    // 2R: beta1, pres1 of each target
  double* d_part = nullptr;   // partial reductions
  double* d_grid = nullptr;   // nb*nb: normalised reweighted distribution
  int nblk = 0;
  std::vector<double> grid;   // host copy for the mixed parameter (filled on demand)
  std::vector<unsigned char> mask;
  bool grid_ready = false, host_grid = false;
};

namespace {

constexpr double kTs = 140.5678, kTi = 185.4676;  // F90:81-88
constexpr double kPs = 4694.59, kPi = -2111.5552;
constexpr double kRhos = 1527.3, kRhoi = -23.1017;
constexpr double kHs = 11.272132, kHi = 9.028914;
constexpr int kT = 256;

int h2d_fail(int code, const std::string& m) {
  cvf::set_last_error(m);
  return code;
}

__global__ void k_h2d_count(const int* __restrict__ cell, long long n, unsigned int* __restrict__ counts) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && cell[i] >= 0) atomicAdd(counts + cell[i], 1u);
}

// F90:1018-1021: the runs' normalised histograms added in run order.
__global__ void k_h2d_hsum(const unsigned int* __restrict__ counts, const double* __restrict__ norma, int R,
                           int nb2, double* __restrict__ hsum) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb2) return;
  double s = 0.0;
  for (int j = 0; j < R; ++j) s = __dadd_rn(s, __ddiv_rn((double)counts[(size_t)j * nb2 + b], norma[j]));
  hsum[b] = s;
}

// Calcula_Histograma F90:1003-1076 for target k (blockIdx.y) and bin b: log H - log sum_j
// exp(arg_j) with arg_j = beta1 (E + pres1 V) - beta_j (E + pres_j V) - ctes_j + log n_j, the sum
// truncated at 10 e-folds below its largest term when any |arg_j| > 10.
__global__ void k_h2d_logp(const double* __restrict__ hsum, int nb, double Emin, double dE, double Dmin, double dD,
                           double N, const double* __restrict__ run, int R, const double* __restrict__ tgt,
                           double* __restrict__ logp) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int nb2 = nb * nb, k = blockIdx.y;
  if (b >= nb2) return;
  const double h = hsum[b];
  double out = 0.0;
  if (h != 0.0) {
    const int i = b / nb, w = b - i * nb;
    const double E = __dmul_rn(__dadd_rn(Emin, __dmul_rn((double)i + 0.5, dE)), N);
    const double dens = __dadd_rn(Dmin, __dmul_rn((double)w + 0.5, dD));
    const double V = __dmul_rn(__ddiv_rn(0.018, dens), N);
    const double beta1 = tgt[2 * k], pres1 = tgt[2 * k + 1];
    const double a1 = __dmul_rn(beta1, __dadd_rn(E, __dmul_rn(pres1, V)));
    bool flag = false;
    double mx = -1e308;
    for (int j = 0; j < R; ++j) {
      const double arg = __dadd_rn(__dsub_rn(__dsub_rn(a1, __dmul_rn(run[j], __dadd_rn(E, __dmul_rn(run[R + j], V)))),
                                             run[2 * R + j]),
                                   run[3 * R + j]);
      flag = flag || fabs(arg) > 10;
      mx = arg > mx ? arg : mx;
    }
    double xx = 0.0;
    for (int j = 0; j < R; ++j) {
      const double arg = __dadd_rn(__dsub_rn(__dsub_rn(a1, __dmul_rn(run[j], __dadd_rn(E, __dmul_rn(run[R + j], V)))),
                                             run[2 * R + j]),
                                   run[3 * R + j]);
      if (!flag) xx = __dadd_rn(xx, exp(arg));
      else if (__dsub_rn(mx, arg) < 10) xx = __dadd_rn(xx, exp(__dsub_rn(arg, mx)));
    }
    if (!flag) xx = log(xx);
    else xx = __dadd_rn(xx != 0.0 ? log(xx) : 0.0, mx);
    out = __dsub_rn(log(h), xx);
  }
  logp[(size_t)k * nb2 + b] = out;
}

// Fixed-order block reductions of target k's non-empty bins: the maximum, then the sum of
// exp(logP - max) over bins less than 10 below it (F90:1078-1122).
__global__ void k_h2d_max(const double* __restrict__ hsum, const double* __restrict__ logp, int nb2, int nblk,
                          double* __restrict__ part) {
  __shared__ double s[kT];
  const int k = blockIdx.y;
  double m = -1e308;
  for (int b = blockIdx.x * kT + threadIdx.x; b < nb2; b += nblk * kT)
    if (hsum[b] != 0.0) m = fmax(m, logp[(size_t)k * nb2 + b]);
  s[threadIdx.x] = m;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)k * nblk + blockIdx.x] = s[0];
}

__global__ void k_h2d_sumexp(const double* __restrict__ hsum, const double* __restrict__ logp, int nb2, int nblk,
                             const double* __restrict__ mx, double* __restrict__ part) {
  __shared__ double s[kT];
  const int k = blockIdx.y;
  const double m = mx[k];
  double acc = 0.0;
  for (int b = blockIdx.x * kT + threadIdx.x; b < nb2; b += nblk * kT) {
    const double lp = logp[(size_t)k * nb2 + b];
    if (hsum[b] != 0.0 && __dsub_rn(m, lp) < 10) acc = __dadd_rn(acc, exp(__dsub_rn(lp, m)));
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] = __dadd_rn(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)k * nblk + blockIdx.x] = s[0];
}

// Reweighted grid exp(logP - log_Z) of target 0 (0 in empty bins) and its block partial sums.
__global__ void k_h2d_grid(const double* __restrict__ hsum, const double* __restrict__ logp, int nb2, int nblk,
                           double logz, double* __restrict__ grid, double* __restrict__ part) {
  __shared__ double s[kT];
  double acc = 0.0;
  for (int b = blockIdx.x * kT + threadIdx.x; b < nb2; b += nblk * kT) {
    const double g = hsum[b] != 0.0 ? exp(__dsub_rn(logp[b], logz)) : 0.0;
    grid[b] = g;
    acc = __dadd_rn(acc, g);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] = __dadd_rn(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// grid /= norma, then the marginals: rows (energy bins) into marg[0..nb), columns (density bins)
// into marg[nb..2nb), each summed in bin order by one thread.
__global__ void k_h2d_scale(double* __restrict__ grid, int nb2, double norma) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb2) grid[b] = __ddiv_rn(grid[b], norma);
}
__global__ void k_h2d_marginals(const double* __restrict__ hsum, const double* __restrict__ grid, int nb,
                                double* __restrict__ marg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nb) return;
  double s = 0.0;
  if (t < nb) {
    for (int w = 0; w < nb; ++w)
      if (hsum[t * nb + w] != 0.0) s = __dadd_rn(s, grid[t * nb + w]);
  } else {
    const int w = t - nb;
    for (int i = 0; i < nb; ++i)
      if (hsum[i * nb + w] != 0.0) s = __dadd_rn(s, grid[i * nb + w]);
  }
  marg[t] = s;
}

#define HK(x)                                                                          \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) return h2d_fail(CVF_ECUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

// log Z of every target currently in d_tgt (count nt) into logz[] (F90:1078-1122).
int log_z(cvf_h2d* H, int nt, std::vector<double>& logz) {
  const int nb2 = H->nb * H->nb;
  dim3 g1((nb2 + kT - 1) / kT, nt);
  k_h2d_logp<<<g1, kT, 0, H->s>>>(H->d_hsum, H->nb, H->Emin, H->dE, H->Dmin, H->dD, H->N, H->d_run, H->R, H->d_tgt,
                                  H->d_logp);
  dim3 g2(H->nblk, nt);
  k_h2d_max<<<g2, kT, 0, H->s>>>(H->d_hsum, H->d_logp, nb2, H->nblk, H->d_part);
  HK(cudaGetLastError());
  std::vector<double> part((size_t)nt * H->nblk);
  HK(cudaMemcpyAsync(part.data(), H->d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaStreamSynchronize(H->s));
  std::vector<double> mx(nt);
  for (int k = 0; k < nt; ++k) {
    double m = -1e308;
    for (int b = 0; b < H->nblk; ++b) m = std::max(m, part[(size_t)k * H->nblk + b]);
    if (m == -1e308) return h2d_fail(CVF_EINVAL, "no histogram at a requested (T, P)");
    mx[k] = m;
  }
  double* d_mx = H->d_part + (size_t)nt * H->nblk;
  HK(cudaMemcpyAsync(d_mx, mx.data(), nt * sizeof(double), cudaMemcpyHostToDevice, H->s));
  k_h2d_sumexp<<<g2, kT, 0, H->s>>>(H->d_hsum, H->d_logp, nb2, H->nblk, d_mx, H->d_part);
  HK(cudaGetLastError());
  HK(cudaMemcpyAsync(part.data(), H->d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaStreamSynchronize(H->s));
  logz.assign(nt, 0.0);
  for (int k = 0; k < nt; ++k) {
    double z = 0.0;
    for (int b = 0; b < H->nblk; ++b) z += part[(size_t)k * H->nblk + b];
    logz[k] = (z != 0.0 ? log(z) : 0.0) + mx[k];
  }
  return 0;
}

int upload_runs(cvf_h2d* H) {
  const int R = H->R;
  std::vector<double> run(4 * (size_t)R);
  for (int j = 0; j < R; ++j) {
    run[j] = 1000. / (0.2293 * H->Tk[j]);
    run[R + j] = H->Pbar[j] * 100.0;
    run[2 * R + j] = H->ctes[j];
    run[3 * R + j] = H->log_medidas[j];
  }
  HK(cudaMemcpyAsync(H->d_run, run.data(), run.size() * sizeof(double), cudaMemcpyHostToDevice, H->s));
  return 0;
}

int set_targets(cvf_h2d* H, const std::vector<double>& temp, const std::vector<double>& pres) {
  std::vector<double> t(2 * temp.size());
  for (size_t k = 0; k < temp.size(); ++k) {
    t[2 * k] = 1000. / (0.2293 * temp[k]);
    t[2 * k + 1] = pres[k] * 100.0;
  }
  HK(cudaMemcpyAsync(H->d_tgt, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, H->s));
  return 0;
}

void destroy(cvf_h2d* H) {
  if (!H) return;
  cudaSetDevice(H->device);
  if (H->s) cudaStreamSynchronize(H->s);
  for (double* p : {H->d_hsum, H->d_logp, H->d_run, H->d_tgt, H->d_part, H->d_grid})
    if (p) cudaFree(p);
  if (H->s) cudaStreamDestroy(H->s);
  delete H;
}

}  // namespace

extern "C" {

int cvf_h2d_create(int device, const double* h, const double* rho, const int* run_of, long long n, const double* That,
                   const double* Phat, int n_runs, int L, double bin_factor, int steps, cvf_h2d** out) {
  if (!h || !rho || !run_of || !That || !Phat || !out || n < 1 || n_runs < 1 || L < 1 || !(bin_factor > 0) ||
      steps < 0)
    return h2d_fail(CVF_EINVAL, "null array or bad size");
  *out = nullptr;
  for (long long i = 0; i < n; ++i)
    if (run_of[i] < 0 || run_of[i] >= n_runs) return h2d_fail(CVF_EINVAL, "run index out of range");
  cvf_h2d* H = new cvf_h2d();
  H->device = device;
  H->L = L;
  H->R = n_runs;
  H->N = (double)L * L * L;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&H->s, cudaStreamNonBlocking) != cudaSuccess) {
    destroy(H);
    return h2d_fail(CVF_ECUDA, "device or stream");
  }
  const int R = n_runs;
  H->That.assign(That, That + R);
  H->Phat.assign(Phat, Phat + R);
  H->Tk.resize(R);
  H->Pbar.resize(R);
  for (int j = 0; j < R; ++j) {
    H->Tk[j] = That[j] * kTs + kTi;  // F90:119-120
    H->Pbar[j] = Phat[j] * kPs + kPi;
  }
  // F90:155-181, 264-275: SI energy and density of every sample and their ranges
  std::vector<double> E((size_t)n), D((size_t)n);
  std::vector<long long> cnt(R, 0);
  double Emin = 0, Emax = 0, Dmin = 0, Dmax = 0;
  for (long long i = 0; i < n; ++i) {
    const int j = run_of[i];
    const double dens = kRhos * rho[i] + kRhoi;
    const double e = kHs * h[i] + kHi * That[j] - 1.8 * H->Pbar[j] / dens;
    E[i] = e;
    D[i] = dens;
    if (i == 0) {
      Emin = Emax = e;
      Dmin = Dmax = dens;
    } else {
      Emax = std::max(Emax, e);
      Emin = std::min(Emin, e);
      Dmax = std::max(Dmax, dens);
      Dmin = std::min(Dmin, dens);
    }
    ++cnt[j];
  }
  long long maxn = 0;
  H->log_medidas.resize(R);
  for (int j = 0; j < R; ++j) {
    if (cnt[j] < 1) {
      destroy(H);
      return h2d_fail(CVF_EINVAL, "a run without samples");
    }
    maxn = std::max(maxn, cnt[j]);
    H->log_medidas[j] = (double)logf((float)cnt[j]);  // log(real(medidas)): single precision (F90:135)
  }
  // F90:220-236
  int n_bin = (int)(sqrtf((float)maxn) / 2.0f);
  if (n_bin < 1) n_bin = 1;
  double rE = Emax - Emin, rD = Dmax - Dmin;
  const double tE = rE / n_bin, tD = rD / n_bin;
  n_bin += 20;
  rE += 20 * tE;
  Emin -= 10 * tE;
  rD += 20 * tD;
  Dmin -= 10 * tD;
  H->nb = (int)(n_bin * 10 * bin_factor);
  if (H->nb < 2 || (long long)H->nb * H->nb > (1LL << 31) / 2) {
    destroy(H);
    return h2d_fail(CVF_EINVAL, "bin count out of range (bin_factor)");
  }
  H->Emin = Emin;
  H->Dmin = Dmin;
  H->dE = rE / H->nb;
  H->dD = rD / H->nb;
  H->nbm = (int)sqrtf((float)H->nb * 1.0f);  // n_bin_mixed (F90:716)
  const int nb = H->nb, nb2 = nb * nb;
  // F90:264-279: bin every sample; out-of-range samples leave the run's normalisation
  std::vector<int> cell((size_t)n);
  std::vector<double> norma(R, 0.0);
  for (long long i = 0; i < n; ++i) {
    const long long ie = (long long)((E[i] - Emin) / H->dE), id = (long long)((D[i] - Dmin) / H->dD);
    if (ie >= 0 && ie < nb && id >= 0 && id < nb) {
      cell[i] = (int)((long long)run_of[i] * nb2 + ie * nb + id);
      norma[run_of[i]] += 1.0;
    } else {
      cell[i] = -1;
    }
  }
  for (int j = 0; j < R; ++j) norma[j] = norma[j] * H->dE * H->dD;
  H->nblk = std::min(1024, (nb2 + kT - 1) / kT);
  unsigned int* d_counts = nullptr;
  int* d_cell = nullptr;
  double* d_norma = nullptr;
  auto bail = [&](int code, const std::string& m) {
    if (d_counts) cudaFree(d_counts);
    if (d_cell) cudaFree(d_cell);
    if (d_norma) cudaFree(d_norma);
    destroy(H);
    return h2d_fail(code, m);
  };
  if (cudaMalloc(&d_counts, (size_t)R * nb2 * sizeof(unsigned int)) != cudaSuccess ||
      cudaMalloc(&d_cell, (size_t)n * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&d_norma, (size_t)R * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_hsum, (size_t)nb2 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_logp, (size_t)R * nb2 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_run, 4 * (size_t)R * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_tgt, 2 * (size_t)R * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_part, ((size_t)R * H->nblk + R + 2 * (size_t)nb) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_grid, (size_t)nb2 * sizeof(double)) != cudaSuccess)
    return bail(CVF_ENOMEM, "cudaMalloc");
  cudaMemsetAsync(d_counts, 0, (size_t)R * nb2 * sizeof(unsigned int), H->s);
  cudaMemcpyAsync(d_cell, cell.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, H->s);
  cudaMemcpyAsync(d_norma, norma.data(), (size_t)R * sizeof(double), cudaMemcpyHostToDevice, H->s);
  k_h2d_count<<<(unsigned)((n + kT - 1) / kT), kT, 0, H->s>>>(d_cell, n, d_counts);
  k_h2d_hsum<<<(nb2 + kT - 1) / kT, kT, 0, H->s>>>(d_counts, d_norma, R, nb2, H->d_hsum);
  cudaError_t e = cudaStreamSynchronize(H->s);
  cudaFree(d_counts);
  cudaFree(d_cell);
  cudaFree(d_norma);
  d_counts = nullptr;
  d_cell = nullptr;
  d_norma = nullptr;
  if (e != cudaSuccess) return bail(CVF_ECUDA, std::string("histograms: ") + cudaGetErrorString(e));
  // F90:398-425: Jacobi iteration of the constants, every run's log Z in one launch per step
  H->ctes.assign(R, 0.0);
  std::vector<double> ctes2(R, 0.0), logz;
  if (int rc = set_targets(H, H->Tk, H->Pbar)) return bail(rc, "targets");
  for (int st = 0; st < steps; ++st) {
    H->ctes = ctes2;
    if (int rc = upload_runs(H)) return bail(rc, "runs");
    if (int rc = log_z(H, R, logz)) {
      destroy(H);
      return rc;
    }
    for (int k = 0; k < R; ++k) ctes2[k] = logz[k] - logz[0];
  }
  for (int k = 0; k < R && steps > 0; ++k)
    if (fabs(H->ctes[k] - ctes2[k]) > 1E-07) return bail(CVF_ELIMIT, "the constants did not converge: use more steps");
  H->ctes = ctes2;
  if (int rc = upload_runs(H)) return bail(rc, "runs");
  *out = H;
  return 0;
}

int cvf_h2d_info(const cvf_h2d* H, int* n_bin2d, int* n_bin_mixed, double* Emin, double* dE, double* Dmin, double* dD,
                 double* ctes) {
  if (!H) return h2d_fail(CVF_EINVAL, "null handle");
  if (n_bin2d) *n_bin2d = H->nb;
  if (n_bin_mixed) *n_bin_mixed = H->nbm;
  if (Emin) *Emin = H->Emin;
  if (dE) *dE = H->dE;
  if (Dmin) *Dmin = H->Dmin;
  if (dD) *dD = H->dD;
  if (ctes) std::copy(H->ctes.begin(), H->ctes.end(), ctes);
  return 0;
}

// F90:737-759 with binder_energy_density F90:2610-2662.
int cvf_h2d_reweight(cvf_h2d* H, double T_hat, double P_hat, double* grid, double* binder_e, double* binder_rho) {
  if (!H) return h2d_fail(CVF_EINVAL, "null handle");
  HK(cudaSetDevice(H->device));
  std::vector<double> logz;
  if (int rc = set_targets(H, {T_hat * kTs + kTi}, {P_hat * kPs + kPi})) return rc;
  if (int rc = log_z(H, 1, logz)) return rc;
  const int nb = H->nb, nb2 = nb * nb;
  k_h2d_grid<<<H->nblk, kT, 0, H->s>>>(H->d_hsum, H->d_logp, nb2, H->nblk, logz[0], H->d_grid, H->d_part);
  HK(cudaGetLastError());
  std::vector<double> part(H->nblk);
  HK(cudaMemcpyAsync(part.data(), H->d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaStreamSynchronize(H->s));
  double norma = 0.0;
  for (double x : part) norma += x;
  norma = norma * H->dE * H->dD;
  k_h2d_scale<<<(nb2 + kT - 1) / kT, kT, 0, H->s>>>(H->d_grid, nb2, norma);
  double* d_marg = H->d_part + (size_t)H->R * H->nblk + H->R;
  k_h2d_marginals<<<(2 * nb + kT - 1) / kT, kT, 0, H->s>>>(H->d_hsum, H->d_grid, nb, d_marg);
  HK(cudaGetLastError());
  std::vector<double> marg(2 * (size_t)nb);
  HK(cudaMemcpyAsync(marg.data(), d_marg, marg.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  if (grid) HK(cudaMemcpyAsync(grid, H->d_grid, (size_t)nb2 * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaStreamSynchronize(H->s));
  H->grid_ready = true;
  H->host_grid = false;
  double tot = 0.0;
  for (int i = 0; i < nb; ++i) tot += marg[i];
  double u2 = 0, u4 = 0, v2 = 0, v4 = 0;
  for (int i = 0; i < nb; ++i) {
    const double ene = H->Emin + (i + 0.5) * H->dE, m2 = ene * ene;
    u2 += m2 * (marg[i] / tot);
    u4 += m2 * m2 * (marg[i] / tot);
    const double rho = H->Dmin + (i + 0.5) * H->dD, r2 = rho * rho;
    v2 += r2 * (marg[nb + i] / tot);
    v4 += r2 * r2 * (marg[nb + i] / tot);
  }
  if (binder_e) *binder_e = 1.0 - u4 / (3.0 * u2 * u2);
  if (binder_rho) *binder_rho = 1.0 - v4 / (3.0 * v2 * v2);
  return 0;
}

// Calcula_Histograma_Rotado_normX F90:1383-1620 and binder F90:2580-2608 on the last reweighted
// grid; x and q hold n_bin_mixed values (may be NULL).
int cvf_h2d_mixed(cvf_h2d* H, double alpha, double* x_out, double* q_out, double* binder_m) {
  if (!H || !H->grid_ready) return h2d_fail(CVF_EINVAL, "call cvf_h2d_reweight first");
  const int nb = H->nb, nbm = H->nbm;
  if (nbm < 3) return h2d_fail(CVF_EINVAL, "too few mixed-parameter bins");
  if (!H->host_grid) {
    H->grid.resize((size_t)nb * nb);
    HK(cudaSetDevice(H->device));
    HK(cudaMemcpy(H->grid.data(), H->d_grid, H->grid.size() * sizeof(double), cudaMemcpyDeviceToHost));
    H->host_grid = true;
  }
  const double sa = sin(alpha), ca = cos(alpha);
  double Xmin = 1E12, Xmax = -1E12;
  for (int i = 0; i < nb; ++i)
    for (int w = 0; w < nb; ++w)
      if (H->grid[(size_t)i * nb + w] > 0) {
        const double X = (H->Emin + (i + 0.5) * H->dE) * sa + (H->Dmin + (w + 0.5) * H->dD) * ca;
        Xmax = std::max(Xmax, X);
        Xmin = std::min(Xmin, X);
      }
  double rX = Xmax - Xmin, t = rX / nbm;
  rX = rX + 4 * t;
  Xmin = Xmin - 2 * t;
  t = rX / nbm;
  std::vector<double> q(nbm, 0.0), m(nbm);
  for (int i = 0; i < nb; ++i)
    for (int w = 0; w < nb; ++w) {
      const double g = H->grid[(size_t)i * nb + w];
      if (!(g > 0)) continue;
      const double X = (H->Emin + (i + 0.5) * H->dE) * sa + (H->Dmin + (w + 0.5) * H->dD) * ca;
      long long ix = (long long)((X - Xmin) / t);
      if (ix < 0 || ix >= nbm) {
        if (fabs(X - Xmin) < 1E-10) ix = 0;
        else return h2d_fail(CVF_EINVAL, "point outside the mixed-parameter histogram");
      }
      q[ix] += g;
    }
  for (int i = 0; i < nbm; ++i) m[i] = Xmin + (i + 0.5) * t;
  double norma = 0;
  for (int i = 0; i < nbm; ++i) norma += q[i];
  for (auto& v : q) v = v / (norma * t);
  double media = 0;
  for (int i = 0; i < nbm; ++i) media += m[i] * q[i] * t;
  for (auto& v : m) v -= media;
  norma = 0;
  double var = 0;
  for (int i = 0; i < nbm; ++i)
    if (q[i] > 0) {
      norma += q[i] * t;
      var += m[i] * m[i] * q[i] * t;
    }
  double a1 = sqrt(norma / var), a2 = 1 / (norma * a1);
  for (int i = 0; i < nbm; ++i) {
    m[i] *= a1;
    q[i] *= a2;
  }
  const double b = 1.53, alh = 1.0, bt = 1.0, pi = 3.14159;
  for (auto& v : m) v = alh * b * b * sin(pi * v / b) / (pi * pi) + bt * v;
  std::vector<double> wdt(nbm);
  wdt[0] = m[1] - m[0];
  for (int i = 1; i < nbm - 1; ++i) wdt[i] = (m[i + 1] - m[i - 1]) / 2.0;
  wdt[nbm - 1] = m[nbm - 1] - m[nbm - 2];
  norma = 0;
  for (int i = 0; i < nbm; ++i) norma += q[i] * wdt[i];
  for (auto& v : q) v /= norma;
  double media_rx = 0;
  for (int i = 0; i < nbm; ++i) media_rx += m[i] * q[i] * wdt[i];
  for (auto& v : m) v -= media_rx;
  norma = 0;
  var = 0;
  for (int i = 0; i < nbm; ++i)
    if (q[i] > 0) {
      norma += q[i] * wdt[i];
      var += m[i] * m[i] * q[i] * wdt[i];
    }
  a1 = sqrt(norma / var);
  a2 = 1 / (norma * a1);
  for (int i = 0; i < nbm; ++i) {
    m[i] *= a1;
    q[i] *= a2;
  }
  if (x_out) std::copy(m.begin(), m.end(), x_out);
  if (q_out) std::copy(q.begin(), q.end(), q_out);
  if (binder_m) {
    double nq = 0;
    for (double v : q) nq += v;
    double u2 = 0, u4 = 0;
    for (int i = 0; i < nbm; ++i) {
      const double op = m[i] / a1 + media, m2 = op * op;
      u2 += m2 * q[i] / nq;
      u4 += m2 * m2 * q[i] / nq;
    }
    *binder_m = 1.0 - u4 / (3.0 * u2 * u2);
  }
  return 0;
}

int cvf_h2d_destroy(cvf_h2d* H) {
  destroy(H);
  return 0;
}

}  // extern "C"
