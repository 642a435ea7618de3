// Multi-tau autocorrelation of the sigma "magnetisation" on the GPU: Flag_correlation of
// SOURCE/gpu_water3D.cu ("GW"). Each production step the reference copies the whole lattice to
// the host, takes the fraction of arms in the most populated sigma value (GW:1245-1272) and adds
// it to a multi-tau correlator (GW:2983-3076). Here a histogram kernel counts the sigma values
// on the device and one thread per replica runs the correlator on device-resident state; only
// the evaluated correlation (GW:3078-3112) crosses to the host, at the end.
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

namespace {

__device__ __forceinline__ int find_rep(const int* __restrict__ blk, int nrep, int b) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(blk + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Number of zero 3-bit fields among the six fields of x.
__device__ __forceinline__ uint32_t zero_fields6(uint32_t x) {
  return 6u - (uint32_t)__popc((x | (x >> 1) | (x >> 2)) & 0x9249u);
}

// One thread per cell word (the colour-0 array, then the colour-1 array) through the one-thread-
// per-cell block table: counts of each sigma value among the word's six arms, summed per warp
// and added to the replica's hist.
__global__ void __launch_bounds__(kThreads) k_corr_hist(const ReplicaDesc* __restrict__ reps,
                                                        const int* __restrict__ blk, int nrep,
                                                        CorrState* __restrict__ corr) {
  const int r = find_rep(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t half = (uint32_t)R.L * R.L * (uint32_t)R.H;
  const uint32_t q = (uint32_t)(blockIdx.x - __ldg(blk + r)) * blockDim.x + threadIdx.x;
  uint32_t c[6] = {0, 0, 0, 0, 0, 0};
  if (q < 2 * half) {
    const uint32_t w = q < half ? R.cells[0][q] : R.cells[1][q - half];
#pragma unroll
    for (uint32_t v = 0; v < 6; ++v) c[v] = zero_fields6(w ^ (v * 0x9249u));
  }
#pragma unroll
  for (int v = 0; v < 6; ++v) c[v] = __reduce_add_sync(0xffffffffu, c[v]);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int v = 0; v < 6; ++v)
      if (c[v]) atomicAdd(&corr[r].hist[v], (unsigned long long)c[v]);
  }
}

// GW:3010-3076 for one value w entering level k0, written as a loop over the levels it reaches
// (the recursion of GW:3030 only touches deeper levels, so each level's update can finish first).
// Every product and sum is rounded on its own, as the host C code computes it.
__device__ void corr_add(CorrState& C, double w) {
  const int dmin = kCorrP / kCorrM;
  for (int k = 0; k < kCorrLevels; ++k) {
    if (k > C.kmax) C.kmax = k;
    const int ins = C.insertindex[k];
    C.shift[k][ins] = w;
    if (k == 0) C.accval = __dadd_rn(C.accval, w);
    C.accumulator[k] = __dadd_rn(C.accumulator[k], w);
    ++C.naccumulator[k];
    bool next = false;
    double wn = 0.0;
    if (C.naccumulator[k] == kCorrM) {
      wn = __ddiv_rn(C.accumulator[k], (double)kCorrM);
      next = true;
      C.accumulator[k] = 0;
      C.naccumulator[k] = 0;
    }
    if (k == 0) {
      int ind2 = ins;
      for (int j = 0; j < kCorrP; ++j) {
        if (C.shift[k][ind2] > -1e10) {
          C.correlation[k][j] = __dadd_rn(C.correlation[k][j], __dmul_rn(C.shift[k][ins], C.shift[k][ind2]));
          ++C.ncorrelation[k][j];
        }
        if (--ind2 < 0) ind2 += kCorrP;
      }
    } else {
      int ind2 = ins - dmin;
      for (int j = dmin; j < kCorrP; ++j) {
        if (ind2 < 0) ind2 += kCorrP;
        if (C.shift[k][ind2] > -1e10) {
          C.correlation[k][j] = __dadd_rn(C.correlation[k][j], __dmul_rn(C.shift[k][ins], C.shift[k][ind2]));
          ++C.ncorrelation[k][j];
        }
        --ind2;
      }
    }
    if (++C.insertindex[k] == kCorrP) C.insertindex[k] = 0;
    if (!next) return;
    w = wn;
  }
}

// One thread per replica: the most populated sigma value's share of the 6N arms (GW:1262-1270),
// then the add; clears hist for the next step.
__global__ void k_corr_add(const ReplicaDesc* __restrict__ reps, int nrep, CorrState* __restrict__ corr) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  CorrState& C = corr[r];
  const double arms = 6.0 * (double)reps[r].L * (double)reps[r].L * (double)reps[r].L;
  double max_mass = -2e10;
  for (int v = 0; v < 6; ++v) {
    const double c = (double)C.hist[v];
    if (c > max_mass) max_mass = c;
    C.hist[v] = 0;
  }
  corr_add(C, __ddiv_rn(max_mass, arms));
}

}  // namespace

cudaError_t launch_corr_step(const BatchDev& b, cudaStream_t s) {
  k_corr_hist<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.blk_cell, b.nrep, b.corr);
  k_corr_add<<<(b.nrep + 127) / 128, 128, 0, s>>>(b.reps, b.nrep, b.corr);
  return cudaGetLastError();
}

}  // namespace cvf
