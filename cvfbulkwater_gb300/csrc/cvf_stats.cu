// Run statistics on the GPU from the on-device sample stream: the awk stage of
// TA/script_analisi.sh:35 (CVF_ThermodynamicAnalysis/ of lcoronas/CVFBulkWater), the mean and
// <x^2> - <x>^2 of the six data.out columns (GW:2138-2159) of every replica, without copying the
// samples to the host.
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

namespace {

constexpr int kStatThreads = 256;

// The data.out columns of one sample record, rounded operation by operation as the host's
// fill_obs computes them (energy, enthalpy, volume, N_hb, m, r_cell).
__device__ __forceinline__ void sample_columns(const ReplicaDesc& R, const SampleRec& s, double N, double* c) {
  const double nhb = __dmul_rn(0.5, (double)s.n_hb2);
  const double evdw_r = evdw(s.r_cell, R.dist, R.freq, R.n_shells, R.Rc);
  const double e = __dadd_rn(__dadd_rn(evdw_r, __dmul_rn(-(double)kJhbF, nhb)), __dmul_rn(-(double)kJsigF, (double)s.n_sigma));
  const double v = __dadd_rn(__dmul_rn(__dmul_rn(__dmul_rn(N, s.r_cell), s.r_cell), s.r_cell), __dmul_rn((double)kVhbF, nhb));
  c[0] = e;
  c[1] = __dadd_rn(e, __dmul_rn((double)R.P, v));
  c[2] = v;
  c[3] = nhb;
  c[4] = __ddiv_rn((double)s.n_sigma, __dmul_rn(N, 15.0));
  c[5] = s.r_cell;
}

// One block per replica. Thread t adds the samples t, t + 256, ... in order; a fixed tree in
// shared memory adds the 256 partial sums, so the result does not depend on scheduling.
// out[r*14 + k]: mean of column k (k < 6), variance of column k - 6 (6 <= k < 12), samples used
// (12: the stored ones), samples recorded (13: more than stored when the stream overflowed).
__global__ void __launch_bounds__(kStatThreads) k_run_stats(const ReplicaDesc* __restrict__ reps,
                                                            const ReplicaState* __restrict__ st, int nrep,
                                                            double* __restrict__ out) {
  __shared__ double s_sum[12][kStatThreads];
  const int r = blockIdx.x;
  if (r >= nrep) return;
  const ReplicaDesc& R = reps[r];
  const ReplicaState& S = st[r];
  const uint32_t n = S.samples ? (S.n_samples < S.cap_samples ? S.n_samples : S.cap_samples) : 0u;
  const double N = (double)R.L * (double)R.L * (double)R.L;
  double acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += kStatThreads) {
    double c[6];
    sample_columns(R, S.samples[i], N, c);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      acc[k] = __dadd_rn(acc[k], c[k]);
      acc[6 + k] = __dadd_rn(acc[6 + k], __dmul_rn(c[k], c[k]));
    }
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) s_sum[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = kStatThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
#pragma unroll
      for (int k = 0; k < 12; ++k) s_sum[k][threadIdx.x] = __dadd_rn(s_sum[k][threadIdx.x], s_sum[k][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) {
    const int k = threadIdx.x;
    const double nn = (double)n;
    const double mean = n ? __ddiv_rn(s_sum[k][0], nn) : 0.0;
    const double var = n ? __dsub_rn(__ddiv_rn(s_sum[6 + k][0], nn), __dmul_rn(mean, mean)) : 0.0;
    out[r * 14 + k] = mean;
    out[r * 14 + 6 + k] = var;
  }
  if (threadIdx.x == 0) {
    out[r * 14 + 12] = (double)n;
    out[r * 14 + 13] = (double)S.n_samples;
  }
}

}  // namespace

cudaError_t launch_run_stats(const BatchDev& b, double* out, cudaStream_t s) {
  k_run_stats<<<b.nrep, kStatThreads, 0, s>>>(b.reps, b.st, b.nrep, out);
  return cudaGetLastError();
}

}  // namespace cvf
