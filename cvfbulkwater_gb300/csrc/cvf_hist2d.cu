// Binned 2-D (E, rho) histogram reweighting of the reference's
// HistogramReweighting/histogram_reweighting_mixed_paramSI_norm_x.f90 ("F90"): the per-run 2-D
// histograms of energy and density in SI units, the constants of the runs by the F90's own
// iteration, the reweighted distribution at any (T, P), the Binder cumulants of E, rho and of the
// mixed order parameter M = sin(a) E + cos(a) rho. The bins are reweighted on the GPU -- one
// thread per bin, all runs' log-sum-exp in registers, every target (T, P) of a WHAM step in one
// launch -- and reduced in a fixed order, so results do not depend on scheduling. The mixed
// parameter is binned on the GPU for a batch of angles at once; the 1-D stages on its
// ~sqrt(n_bin2D) bins (normalisation, sine map, Binder sums, Ising comparisons) run on the host.
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
  double* d_colpart = nullptr;  // kColChunks*nb: column sums of row chunks of the grid
  int* d_rowext = nullptr;      // 2*nb: first and last column with g > 0 of every grid row
  int nblk = 0;
  double* d_scratch = nullptr;  // mixed-parameter binning of a batch of angles
  size_t scratch_n = 0;
  bool grid_ready = false;
};

namespace {

// The F90 is built with plain gfortran, so every literal it assigns to or mixes with a real*8 is
// a default-kind (single precision) constant: the float nearest the decimal, widened.
constexpr double kTs = (double)140.5678f, kTi = (double)185.4676f;  // F90:81-88
constexpr double kPs = (double)4694.59f, kPi = (double)-2111.5552f;
constexpr double kRhos = (double)1527.3f, kRhoi = (double)-23.1017f;
constexpr double kHs = (double)11.272132f, kHi = (double)9.028914f;
constexpr double kE18 = (double)1.8f;      // F90:161, 245
constexpr double kKb = (double)0.2293f;    // F90:1013, 1042
constexpr double kMw = (double)0.018f;     // F90:1031
constexpr double kConv = (double)1E-07f;   // F90:468
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
    const double V = __dmul_rn(__ddiv_rn(kMw, dens), N);
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
// into marg[nb..2nb), each in a fixed order (empty bins hold 0 in the grid and add nothing).
__global__ void k_h2d_scale(double* __restrict__ grid, int nb2, double norma) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb2) grid[b] = __ddiv_rn(grid[b], norma);
}
constexpr int kColChunks = 32;
// One warp per row: its sum (lanes over the row, then a fixed shuffle tree) and the first and
// last column with g > 0 (nb and -1 for a row without any).
__global__ void k_h2d_rows(const double* __restrict__ grid, int nb, double* __restrict__ marg,
                           int* __restrict__ rowext) {
  const int i = blockIdx.x * (kT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= nb) return;
  const double* row = grid + (size_t)i * nb;
  double s = 0.0;
  int lo = nb, hi = -1;
  for (int w = lane; w < nb; w += 32) {
    const double g = row[w];
    s = __dadd_rn(s, g);
    if (g > 0) {
      lo = min(lo, w);
      hi = max(hi, w);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    marg[i] = s;
    rowext[2 * i] = lo;
    rowext[2 * i + 1] = hi;
  }
}
// Column sums in two passes: chunk c of the rows per thread and column, then the chunks in order.
__global__ void k_h2d_cols_part(const double* __restrict__ grid, int nb, double* __restrict__ part) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (w >= nb) return;
  const int i0 = (int)((long long)c * nb / kColChunks), i1 = (int)((long long)(c + 1) * nb / kColChunks);
  double s = 0.0;
  for (int i = i0; i < i1; ++i) s = __dadd_rn(s, grid[(size_t)i * nb + w]);
  part[(size_t)c * nb + w] = s;
}
__global__ void k_h2d_cols(const double* __restrict__ part, int nb, double* __restrict__ marg) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nb) return;
  double s = 0.0;
  for (int c = 0; c < kColChunks; ++c) s = __dadd_rn(s, part[(size_t)c * nb + w]);
  marg[nb + w] = s;
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
    run[j] = 1000. / (kKb * H->Tk[j]);
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
    t[2 * k] = 1000. / (kKb * temp[k]);
    t[2 * k + 1] = pres[k] * 100.0;
  }
  HK(cudaMemcpyAsync(H->d_tgt, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, H->s));
  return 0;
}

// ---------------------------------------------------------------- mixed order parameter
// Calcula_Histograma_Rotado_normX F90:1383-1462 on the GPU for a batch of angles: X = sin(a) E +
// cos(a) rho (Rotate, F90:1126-1138) of every bin with g > 0, its range widened by two bins on
// each side, and the sum of g per X bin. Along one energy row X is monotone in the density bin,
// so the bin index of 32 consecutive bins is monotone across a warp: a segmented warp scan adds
// the runs of equal index and the last lane of each run adds its sum to the warp's own shared
// histogram, in a fixed order, so the result does not depend on scheduling.
constexpr int kMaxAngles = 64;
constexpr int kXWarps = 8;

__device__ __forceinline__ double mixed_x(int i, int w, double Emin, double dE, double Dmin, double dD, double sa,
                                          double ca) {
  const double E = __dadd_rn(Emin, __dmul_rn((double)i + 0.5, dE));
  const double D = __dadd_rn(Dmin, __dmul_rn((double)w + 0.5, dD));
  return __dadd_rn(__dmul_rn(E, sa), __dmul_rn(D, ca));
}

// Range of X over the bins with g > 0 for angle a = blockIdx.x, then Xmin, the bin width and its
// reciprocal (F90:1418-1428) into xp[3a..3a+2]. Along a row X is monotone in the column, so its
// extremes over the row's occupied bins are at the row's first and last occupied column.
// err[0] = 1 when no bin is occupied or the width is not positive.
__global__ void k_h2d_xrange(const int* __restrict__ rowext, int nb, double Emin, double dE, double Dmin,
                             double dD, const double* __restrict__ sc, int nbm, double* __restrict__ xp,
                             int* __restrict__ err) {
  __shared__ double slo[kT], shi[kT];
  const int a = blockIdx.x;
  const double sa = sc[2 * a], ca = sc[2 * a + 1];
  double lo = INFINITY, hi = -INFINITY;
  for (int i = threadIdx.x; i < nb; i += kT) {
    const int w0 = rowext[2 * i], w1 = rowext[2 * i + 1];
    if (w1 < w0) continue;
    const double x0 = mixed_x(i, w0, Emin, dE, Dmin, dD, sa, ca), x1 = mixed_x(i, w1, Emin, dE, Dmin, dD, sa, ca);
    lo = fmin(lo, fmin(x0, x1));
    hi = fmax(hi, fmax(x0, x1));
  }
  slo[threadIdx.x] = lo;
  shi[threadIdx.x] = hi;
  __syncthreads();
  for (int st = kT / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      slo[threadIdx.x] = fmin(slo[threadIdx.x], slo[threadIdx.x + st]);
      shi[threadIdx.x] = fmax(shi[threadIdx.x], shi[threadIdx.x + st]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    lo = slo[0];
    hi = shi[0];
    double rX = __dsub_rn(hi, lo);
    double t = __ddiv_rn(rX, (double)nbm);
    rX = __dadd_rn(rX, __dmul_rn(4.0, t));
    const double Xmin = __dsub_rn(lo, __dmul_rn(2.0, t));
    t = __ddiv_rn(rX, (double)nbm);
    xp[3 * a] = Xmin;
    xp[3 * a + 1] = t;
    xp[3 * a + 2] = t > 0 ? __drcp_rn(t) : 0.0;
    if (!(t > 0) || !(lo <= hi)) atomicExch(err, 1);
  }
}

// int((X - Xmin) / t) of F90:1446 with the quotient rounded as one division: the product with
// the rounded reciprocal is within 1e-15 relative of it, so it gives the same integer part unless
// it lies within 1e-12 of an integer, where the division itself decides.
__device__ __forceinline__ double mixed_bin(double num, double t, double inv_t) {
  double q = __dmul_rn(num, inv_t);
  if (fabs(q - rint(q)) <= 1e-12 * fmax(1.0, fabs(q))) q = __ddiv_rn(num, t);
  return trunc(q);
}

__global__ void __launch_bounds__(32 * kXWarps) k_h2d_xhist(const double* __restrict__ grid,
                                                           const int* __restrict__ rowext, int nb, double Emin,
                                                           double dE, double Dmin, double dD,
                                                           const double* __restrict__ sc,
                                                           const double* __restrict__ xp, int nbm, int nwarps,
                                                           double* __restrict__ wpart, int* __restrict__ err) {
  extern __shared__ double hs[];
  const int a = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* h = hs + (size_t)warp * nbm;
  for (int k = lane; k < nbm; k += 32) h[k] = 0.0;
  __syncwarp();
  const double sa = sc[2 * a], ca = sc[2 * a + 1], Xmin = xp[3 * a], t = xp[3 * a + 1], inv_t = xp[3 * a + 2];
  const double tiny = (double)1E-10f;  // F90:1449
  const int gw = blockIdx.x * kXWarps + warp;
  const int r0 = (int)((long long)gw * nb / nwarps), r1 = (int)((long long)(gw + 1) * nb / nwarps);
  bool bad = false;
  for (int i = r0; i < r1; ++i) {
    const int wlo = rowext[2 * i], whi = rowext[2 * i + 1];
    if (whi < wlo) continue;
    const double* row = grid + (size_t)i * nb;
    const double es = __dmul_rn(__dadd_rn(Emin, __dmul_rn((double)i + 0.5, dE)), sa);
    for (int w0 = wlo; w0 <= whi; w0 += 32) {
      const int w = w0 + lane;
      const double g = w <= whi ? row[w] : 0.0;
      const double X = __dadd_rn(es, __dmul_rn(__dadd_rn(Dmin, __dmul_rn((double)w + 0.5, dD)), ca));
      const double num = __dsub_rn(X, Xmin);
      const double tq = mixed_bin(num, t, inv_t);
      const bool in = tq >= 0.0 && tq < (double)nbm;
      int key = (int)fmin(fmax(tq, 0.0), (double)(nbm - 1));
      double v = 0.0;
      if (g > 0) {
        if (in || fabs(num) < tiny) v = g;
        else bad = true;
        if (!in && fabs(num) < tiny) key = 0;
      }
      for (int d = 1; d < 32; d <<= 1) {
        const double ov = __shfl_up_sync(0xffffffffu, v, d);
        const int ok = __shfl_up_sync(0xffffffffu, key, d);
        if (lane >= d && ok == key) v = __dadd_rn(ov, v);
      }
      const int nk = __shfl_down_sync(0xffffffffu, key, 1);
      if (lane == 31 || nk != key) h[key] = __dadd_rn(h[key], v);
      __syncwarp();
    }
  }
  if (bad) atomicExch(err, 2);
  for (int k = lane; k < nbm; k += 32) wpart[((size_t)a * nwarps + gw) * nbm + k] = h[k];
}

// Sum of the warps' histograms, one warp per (bin k, angle a): lane l adds the partials of warps
// l, l + 32, ... in order, then a fixed shuffle tree: q[a][k].
__global__ void k_h2d_xsum(const double* __restrict__ wpart, int nwarps, int nbm, double* __restrict__ q) {
  const int a = blockIdx.y, k = blockIdx.x * (kT / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= nbm) return;
  double s = 0.0;
  for (int g = lane; g < nwarps; g += 32) s = __dadd_rn(s, wpart[((size_t)a * nwarps + g) * nbm + k]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
  if (lane == 0) q[(size_t)a * nbm + k] = s;
}

// Raw mixed-parameter histograms of n <= kMaxAngles angles: qraw (n x nbm) and xp (Xmin, width,
// 1 / width) of the last reweighted grid (its row extents come with it).
int bin_mixed(cvf_h2d* H, const double* alpha, int n, std::vector<double>& qraw, std::vector<double>& xp) {
  const int nb = H->nb, nbm = H->nbm;
  if (nbm < 3) return h2d_fail(CVF_EINVAL, "too few mixed-parameter bins");
  HK(cudaSetDevice(H->device));
  const int nwb = std::max(1, std::min(128, (nb + kXWarps - 1) / kXWarps)), nwarps = nwb * kXWarps;
  const size_t need = 2 * (size_t)n + 3 * (size_t)n + (size_t)n * nwarps * nbm + (size_t)n * nbm + 1;
  if (need > H->scratch_n) {
    if (H->d_scratch) cudaFree(H->d_scratch);
    H->d_scratch = nullptr;
    H->scratch_n = 0;
    HK(cudaMalloc(&H->d_scratch, need * sizeof(double)));
    H->scratch_n = need;
  }
  double* d_sc = H->d_scratch;
  double* d_xp = d_sc + 2 * (size_t)n;
  double* d_w = d_xp + 3 * (size_t)n;
  double* d_q = d_w + (size_t)n * nwarps * nbm;
  int* d_err = reinterpret_cast<int*>(d_q + (size_t)n * nbm);
  std::vector<double> sc(2 * (size_t)n);
  for (int a = 0; a < n; ++a) {
    sc[2 * a] = sin(alpha[a]);
    sc[2 * a + 1] = cos(alpha[a]);
  }
  HK(cudaMemcpyAsync(d_sc, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice, H->s));
  HK(cudaMemsetAsync(d_err, 0, sizeof(int), H->s));
  k_h2d_xrange<<<n, kT, 0, H->s>>>(H->d_rowext, nb, H->Emin, H->dE, H->Dmin, H->dD, d_sc, nbm, d_xp, d_err);
  k_h2d_xhist<<<dim3(nwb, n), 32 * kXWarps, (size_t)kXWarps * nbm * sizeof(double), H->s>>>(
      H->d_grid, H->d_rowext, nb, H->Emin, H->dE, H->Dmin, H->dD, d_sc, d_xp, nbm, nwarps, d_w, d_err);
  k_h2d_xsum<<<dim3((nbm + kT / 32 - 1) / (kT / 32), n), kT, 0, H->s>>>(d_w, nwarps, nbm, d_q);
  HK(cudaGetLastError());
  qraw.resize((size_t)n * nbm);
  xp.resize(3 * (size_t)n);
  int err = 0;
  HK(cudaMemcpyAsync(qraw.data(), d_q, qraw.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaMemcpyAsync(xp.data(), d_xp, xp.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, H->s));
  HK(cudaStreamSynchronize(H->s));
  if (err == 1) return h2d_fail(CVF_EINVAL, "no width for the mixed-parameter histogram");
  if (err == 2) return h2d_fail(CVF_EINVAL, "point outside the mixed-parameter histogram");
  return 0;
}

// F90:1478-1562: bin centres, normalisation, zero mean and unit variance, the sine map with
// b = 1.53, normalised again over the mapped bin widths. a1 and media are those binder() uses.
int mixed_1d(int nbm, double Xmin, double t, const double* qraw, std::vector<double>& m, std::vector<double>& q,
             double& a1_out, double& media_out) {
  q.assign(qraw, qraw + nbm);
  m.resize(nbm);
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
  const double b = (double)1.53f, alh = 1.0, bt = 1.0, pi = (double)3.14159f;  // F90:1544-1548
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
  a1_out = a1;
  media_out = media;
  return 0;
}

// binder F90:2580-2608: the cumulant of M = x / a1 + media.
double binder_of(const std::vector<double>& m, const std::vector<double>& q, double a1, double media) {
  double nq = 0;
  for (double v : q) nq += v;
  double u2 = 0, u4 = 0;
  for (size_t i = 0; i < m.size(); ++i) {
    const double op = m[i] / a1 + media, m2 = op * op;
    u2 += m2 * q[i] / nq;
    u4 += m2 * m2 * q[i] / nq;
  }
  return 1.0 - u4 / (3.0 * u2 * u2);
}

// ---------------------------------------------------------------- Ising comparisons
// Ising2D F90:2216-2232 (the fit of Liu and Panagiotopoulos, JCP 2010) and Ising3D F90:2234-2252
// (Tsypin, PRE 62, 2000, normalised to unit norm and variance); z**16 by repeated squaring as
// gfortran expands a constant integer power.
double ising2d(double z) {
  const double a = (double)0.058137f, b = (double)-2.68949f, c = (double)-0.11235f, d = (double)2.884162f;
  const double z2 = z * z, z4 = z2 * z2, z8 = z4 * z4, z16 = z8 * z8;
  return exp(-(a * z16 + b * z * z + c * fabs(z) + d));
}
double ising3d(double z) {
  const double a = (double)0.196f, c = (double)0.807f, M0 = (double)1.141059404f, A0 = (double)0.436591191f;
  const double u = z * z / (M0 * M0) - 1;
  return A0 * exp(-(u * u * (a * z * z / (M0 * M0) + c)));
}

// Ising_Peak F90:1148-1222: ternary searches for the maxima on [0.1, 2].
int ising_peaks(double& p2, double& p3) {
  for (int which = 0; which < 2; ++which) {
    auto f = [which](double z) { return which == 0 ? ising2d(z) : ising3d(z); };
    double xmin = (double)0.1f, xmax = 2;
    double x1 = xmin + (xmax - xmin) / 3, x2 = xmin + 2 * (xmax - xmin) / 3;
    for (int it = 0;; ++it) {
      if (it > 10000) return h2d_fail(CVF_ELIMIT, "Ising peak search did not end");
      if (f(x1) > f(x2)) {
        xmax = x2;
      } else if (f(x2) > f(x1)) {
        xmin = x1;
      } else {
        return h2d_fail(CVF_EINVAL, "Ising peak search met equal values");
      }
      x1 = xmin + (xmax - xmin) / 3;
      x2 = xmin + 2 * (xmax - xmin) / 3;
      const bool done = which == 0 ? fabs(x1 - x2) < (double)1E-06f : fabs(f(x1) - f(x2)) < (double)1E-06f;
      if (done) {
        (which == 0 ? p2 : p3) = f(x1) > f(x2) ? f(x1) : f(x2);
        break;
      }
    }
  }
  return 0;
}

// out = liu_2D, liu_3D, kl_2D, kl_3D, zero, height for abscissae m and histogram q.
void confront(const double* m, const double* q, int n, double peak2, double peak3, double* out) {
  double kl2 = 0, kl3 = 0, liu2 = 0, liu3 = 0;
  int n_liu = 0;
  for (int i = 0; i < n; ++i) {
    const double hist = q[i];
    if (hist == 0) continue;
    const double i2 = ising2d(m[i]), i3 = ising3d(m[i]);
    if (i2 > 0) kl2 = kl2 + (log(i2) - log(hist)) * i2;
    if (i3 > 0) kl3 = kl3 + (log(i3) - log(hist)) * i3;
    liu2 = liu2 + sqrt(hist) * fabs(hist - i2);
    liu3 = liu3 + sqrt(hist) * fabs(hist - i3);
    ++n_liu;
  }
  liu2 = liu2 / ((peak2 - ising2d(0.0)) * n_liu);
  liu3 = liu3 / ((peak3 - ising3d(0.0)) * n_liu);
  const double vis = (double)(6.0f / 0.8f);  // F90:2066, 2118
  // ZeroTest: the lowest bin with -1 < m < 1 against Ising3D(0); none such reads as 1E3
  double hmin = (double)1E12f, zero = 1E3;
  int imin = -1;
  for (int i = 0; i < n; ++i)
    if (m[i] > -1 && m[i] < 1 && q[i] < hmin) {
      hmin = q[i];
      imin = i;
    }
  if (imin >= 0) {
    const double d = q[imin] - ising3d(0.0);
    zero = d * d * vis * vis;
    zero = zero + m[imin] * m[imin];
  }
  // HeightTest: the highest bin on each side of 0 against the Ising3D maxima at -+1.14
  double h1 = -10, h2 = -10, height = 1E3;
  int i1 = -1, i2 = -1;
  for (int i = 0; i < n; ++i) {
    if (m[i] < 0) {
      if (q[i] > h1) {
        h1 = q[i];
        i1 = i;
      }
    } else if (q[i] > h2) {
      h2 = q[i];
      i2 = i;
    }
  }
  if (i1 >= 0 && i2 >= 0) {
    const double x1 = (double)-1.14f, x2 = (double)1.14f;
    const double d1 = q[i1] - ising3d(x1), d2 = q[i2] - ising3d(x2);
    height = d1 * d1 * vis * vis;
    height = height + d2 * d2 * vis * vis;
    height = height + (m[i1] - x1) * (m[i1] - x1);
    height = height + (m[i2] - x2) * (m[i2] - x2);
  }
  out[0] = liu2;
  out[1] = liu3;
  out[2] = kl2;
  out[3] = kl3;
  out[4] = zero;
  out[5] = height;
}

void destroy(cvf_h2d* H) {
  if (!H) return;
  cudaSetDevice(H->device);
  if (H->s) cudaStreamSynchronize(H->s);
  for (double* p : {H->d_hsum, H->d_logp, H->d_run, H->d_tgt, H->d_part, H->d_grid, H->d_scratch, H->d_colpart})
    if (p) cudaFree(p);
  if (H->d_rowext) cudaFree(H->d_rowext);
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
    const double e = kHs * h[i] + kHi * That[j] - kE18 * H->Pbar[j] / dens;
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
      cudaMalloc(&H->d_grid, (size_t)nb2 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_colpart, (size_t)kColChunks * nb * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H->d_rowext, 2 * (size_t)nb * sizeof(int)) != cudaSuccess)
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
  // F90:446-472: Jacobi iteration of the constants, every run's log Z in one launch per step
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
    if (fabs(H->ctes[k] - ctes2[k]) > kConv) return bail(CVF_ELIMIT, "the constants did not converge: use more steps");
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
  k_h2d_rows<<<(nb + kT / 32 - 1) / (kT / 32), kT, 0, H->s>>>(H->d_grid, nb, d_marg, H->d_rowext);
  k_h2d_cols_part<<<dim3((nb + kT - 1) / kT, kColChunks), kT, 0, H->s>>>(H->d_grid, nb, H->d_colpart);
  k_h2d_cols<<<(nb + kT - 1) / kT, kT, 0, H->s>>>(H->d_colpart, nb, d_marg);
  HK(cudaGetLastError());
  std::vector<double> marg(2 * (size_t)nb);
  HK(cudaMemcpyAsync(marg.data(), d_marg, marg.size() * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  if (grid) HK(cudaMemcpyAsync(grid, H->d_grid, (size_t)nb2 * sizeof(double), cudaMemcpyDeviceToHost, H->s));
  HK(cudaStreamSynchronize(H->s));
  H->grid_ready = true;
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
  return cvf_h2d_mixed_batch(H, &alpha, 1, x_out, q_out, binder_m);
}

// The same for n angles at once: the 2-D grid is binned on the GPU for every angle, the 1-D
// stages run on the host. x and q hold n x n_bin_mixed values, binder_m n (each may be NULL).
int cvf_h2d_mixed_batch(cvf_h2d* H, const double* alpha, int n, double* x_out, double* q_out, double* binder_m) {
  if (!H || !H->grid_ready) return h2d_fail(CVF_EINVAL, "call cvf_h2d_reweight first");
  if (!alpha || n < 1) return h2d_fail(CVF_EINVAL, "null or empty angle list");
  const int nbm = H->nbm;
  std::vector<double> x, q;
  double a1 = 0, media = 0;
  for (int c0 = 0; c0 < n; c0 += kMaxAngles) {
    const int c = std::min(kMaxAngles, n - c0);
    std::vector<double> qraw, xp;
    if (int rc = bin_mixed(H, alpha + c0, c, qraw, xp)) return rc;
    for (int k = 0; k < c; ++k) {
      const int a = c0 + k;
      if (int rc = mixed_1d(nbm, xp[3 * k], xp[3 * k + 1], qraw.data() + (size_t)k * nbm, x, q, a1, media)) return rc;
      if (x_out) std::copy(x.begin(), x.end(), x_out + (size_t)a * nbm);
      if (q_out) std::copy(q.begin(), q.end(), q_out + (size_t)a * nbm);
      if (binder_m) binder_m[a] = binder_of(x, q, a1, media);
    }
  }
  return 0;
}

// ConfrontIsing F90:2127-2182, ZeroTest F90:2042-2074 and HeightTest F90:2076-2125 of a mixed
// distribution whose abscissae are scaled by B (F90:807): out = liu_2D, liu_3D, kl_2D, kl_3D,
// zero, height.
int cvf_h2d_ising(const double* x, const double* q, int n_bin_mixed, double B, double* out) {
  if (!x || !q || !out || n_bin_mixed < 1) return h2d_fail(CVF_EINVAL, "null array or bad size");
  double peak2, peak3;
  if (int rc = ising_peaks(peak2, peak3)) return rc;
  std::vector<double> m(n_bin_mixed);
  for (int i = 0; i < n_bin_mixed; ++i) m[i] = B * x[i];
  confront(m.data(), q, n_bin_mixed, peak2, peak3, out);
  return 0;
}

// The F90's search loop F90:732-891: for every pressure (outer), temperature and angle S (inner)
// in the given lists (internal units), the reweighted distribution, its Binder cumulants of E and
// rho (tp_rows: n_P x n_T x 2), and per angle the Binder cumulant of the mixed parameter and the
// Ising comparisons at scale B (rows: n_P x n_T x n_S x 7: binder_m, liu_2D, liu_3D, kl_2D, kl_3D,
// zero, height). best[5] receives the row of the smallest liu_2D, liu_3D, zero, height and
// zero + height (the first one in loop order, as the F90's strict comparisons pick; -1 if none is
// below the F90's start value 1E12). Any output may be NULL.
int cvf_h2d_scan(cvf_h2d* H, const double* T_hat, int n_T, const double* P_hat, int n_P, const double* S, int n_S,
                 double B, double* tp_rows, double* rows, long long* best) {
  if (!H || !T_hat || !P_hat || !S || n_T < 1 || n_P < 1 || n_S < 1)
    return h2d_fail(CVF_EINVAL, "null or empty parameter list");
  double peak2, peak3;
  if (int rc = ising_peaks(peak2, peak3)) return rc;
  const int nbm = H->nbm;
  const double start = (double)1E12f;  // F90:725-729
  double lo[5] = {start, start, start, start, start};
  long long arg[5] = {-1, -1, -1, -1, -1};
  std::vector<double> x, q, m(nbm);
  double a1 = 0, media = 0, be = 0, br = 0;
  for (int p = 0; p < n_P; ++p)
    for (int t = 0; t < n_T; ++t) {
      if (int rc = cvf_h2d_reweight(H, T_hat[t], P_hat[p], nullptr, &be, &br)) return rc;
      const long long tp = (long long)p * n_T + t;
      if (tp_rows) {
        tp_rows[2 * tp] = be;
        tp_rows[2 * tp + 1] = br;
      }
      for (int c0 = 0; c0 < n_S; c0 += kMaxAngles) {
        const int c = std::min(kMaxAngles, n_S - c0);
        std::vector<double> qraw, xp;
        if (int rc = bin_mixed(H, S + c0, c, qraw, xp)) return rc;
        for (int k = 0; k < c; ++k) {
          if (int rc = mixed_1d(nbm, xp[3 * k], xp[3 * k + 1], qraw.data() + (size_t)k * nbm, x, q, a1, media))
            return rc;
          const long long r = tp * n_S + c0 + k;
          double v[7];
          v[0] = binder_of(x, q, a1, media);
          for (int i = 0; i < nbm; ++i) m[i] = B * x[i];
          confront(m.data(), q.data(), nbm, peak2, peak3, v + 1);
          if (rows) std::copy(v, v + 7, rows + 7 * r);
          const double crit[5] = {v[1], v[2], v[5], v[6], v[5] + v[6]};
          for (int j = 0; j < 5; ++j)
            if (lo[j] > crit[j]) {
              lo[j] = crit[j];
              arg[j] = r;
            }
        }
      }
    }
  if (best) std::copy(arg, arg + 5, best);
  return 0;
}

// Constants of the runs given directly (the F90 reads them from its Constants_L file when it
// exists and matches the runs, F90:396-440); n_runs values, made relative to run 1 as given.
int cvf_h2d_set_constants(cvf_h2d* H, const double* ctes) {
  if (!H || !ctes) return h2d_fail(CVF_EINVAL, "null handle or array");
  HK(cudaSetDevice(H->device));
  H->ctes.assign(ctes, ctes + H->R);
  H->grid_ready = false;
  return upload_runs(H);
}

int cvf_h2d_destroy(cvf_h2d* H) {
  destroy(H);
  return 0;
}

}  // extern "C"
