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

// Bit planes of the sigma fields of two cell words: bit 3a of word a0, bit 3a+1 of word a1 hold
// bit i of arm a's sigma (i = 0, 1, 2 for p0, p1, p2); q* are the complements within the 12 bits.
struct Planes {
  uint32_t p0, p1, p2, q0, q1, q2;
};
__device__ __forceinline__ Planes planes(uint32_t a0, uint32_t a1) {
  constexpr uint32_t M = 0x9249u, M1 = M << 1, MM = M | M1;
  Planes b;
  b.p0 = (a0 & M) | ((a1 << 1) & M1);
  b.p1 = ((a0 >> 1) & M) | (a1 & M1);
  b.p2 = ((a0 >> 2) & M) | ((a1 >> 1) & M1);
  b.q0 = b.p0 ^ MM;
  b.q1 = b.p1 ^ MM;
  b.q2 = b.p2 ^ MM;
  return b;
}
// Adds the number of arms of the two words with each sigma value 0..5 to c.
__device__ __forceinline__ void count_pair(uint32_t a0, uint32_t a1, uint32_t* c) {
  const Planes b = planes(a0, a1);
  c[0] += __popc(b.q0 & b.q1 & b.q2);
  c[1] += __popc(b.p0 & b.q1 & b.q2);
  c[2] += __popc(b.q0 & b.p1 & b.q2);
  c[3] += __popc(b.p0 & b.p1 & b.q2);
  c[4] += __popc(b.q0 & b.q1 & b.p2);
  c[5] += __popc(b.p0 & b.q1 & b.p2);
}

// One thread per four consecutive cell words (one 128-bit load; the colour-0 array, then the
// colour-1 array, whose length N/2 is a multiple of 4): counts of each sigma value among their
// 24 arms, summed per warp, then per block in shared memory, and added to slot
// blockIdx.x % kCorrSlots of the replica's hist (six atomics per block, spread over the slots so
// that they do not queue on one address).
__global__ void __launch_bounds__(kThreads) k_corr_hist(const ReplicaDesc* __restrict__ reps,
                                                        const int* __restrict__ blk, int nrep,
                                                        CorrState* __restrict__ corr) {
  __shared__ uint32_t s_c[kThreads / 32][6];
  const int r = find_rep(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t half = (uint32_t)R.L * R.L * (uint32_t)R.H;
  const uint32_t q = 4u * ((uint32_t)(blockIdx.x - __ldg(blk + r)) * blockDim.x + threadIdx.x);
  uint32_t c[6] = {0, 0, 0, 0, 0, 0};
  if (q < 2 * half) {
    const uint32_t* src = q < half ? R.cells[0] + q : R.cells[1] + (q - half);
    const uint4 w = *reinterpret_cast<const uint4*>(src);
    count_pair(w.x, w.y, c);
    count_pair(w.z, w.w, c);
  }
#pragma unroll
  for (int v = 0; v < 6; ++v) c[v] = __reduce_add_sync(0xffffffffu, c[v]);
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int v = 0; v < 6; ++v) s_c[warp][v] = c[v];
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    unsigned long long t = 0;
    for (int i = 0; i < kThreads / 32; ++i) t += s_c[i][threadIdx.x];
    if (t) atomicAdd(&corr[r].hist[blockIdx.x % kCorrSlots][threadIdx.x], t);
  }
}

// GW:3010-3076 for one value w entering level 0, by one warp: the levels run in order (the
// recursion of GW:3030 only touches deeper levels, so each level's update can finish first) and
// lane j < 16 updates channel j of the level, whose partner is slot (insertindex - j) mod 16 for
// both branches of GW:3044-3066. Every lane computes the level's scalars alike and lane 0 stores
// them; every product and sum is rounded on its own, as the host C code computes it.
__device__ void corr_add_warp(CorrState& C, double w, int lane) {
  const int dmin = kCorrP / kCorrM;
  for (int k = 0; k < kCorrLevels; ++k) {
    const int ins = C.insertindex[k];
    const double acc = __dadd_rn(C.accumulator[k], w);
    const int nacc = C.naccumulator[k] + 1;
    const bool next = nacc == kCorrM;
    const double wn = __ddiv_rn(acc, (double)kCorrM);
    if (lane < kCorrP && lane >= (k == 0 ? 0 : dmin)) {
      int ind2 = ins - lane;
      if (ind2 < 0) ind2 += kCorrP;
      const double sh = ind2 == ins ? w : C.shift[k][ind2];
      if (sh > -1e10) {
        C.correlation[k][lane] = __dadd_rn(C.correlation[k][lane], __dmul_rn(w, sh));
        ++C.ncorrelation[k][lane];
      }
    }
    __syncwarp();
    if (lane == 0) {
      if (k > C.kmax) C.kmax = k;
      C.shift[k][ins] = w;
      if (k == 0) C.accval = __dadd_rn(C.accval, w);
      C.accumulator[k] = next ? 0.0 : acc;
      C.naccumulator[k] = next ? 0 : nacc;
      C.insertindex[k] = ins + 1 == kCorrP ? 0 : ins + 1;
    }
    __syncwarp();
    if (!next) return;
    w = wn;
  }
}

// One warp per replica: the slot sums of the histogram (cleared for the next step), the most
// populated sigma value's share of the 6N arms (GW:1262-1270), then the add.
__global__ void k_corr_add(const ReplicaDesc* __restrict__ reps, int nrep, CorrState* __restrict__ corr) {
  const int r = blockIdx.x, lane = threadIdx.x;
  if (r >= nrep) return;
  CorrState& C = corr[r];
  unsigned long long n[6];
#pragma unroll
  for (int v = 0; v < 6; ++v) {
    n[v] = C.hist[lane][v];  // kCorrSlots == 32: one slot per lane
    C.hist[lane][v] = 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n[v] += __shfl_xor_sync(0xffffffffu, n[v], o);
  }
  const double arms = 6.0 * (double)reps[r].L * (double)reps[r].L * (double)reps[r].L;
  double max_mass = -2e10;
  for (int v = 0; v < 6; ++v) {
    const double c = (double)n[v];
    if (c > max_mass) max_mass = c;
  }
  corr_add_warp(C, __ddiv_rn(max_mass, arms), lane);
}

}  // namespace

cudaError_t launch_corr_step(const BatchDev& b, cudaStream_t s) {
  static_assert(kCorrSlots == 32, "k_corr_add reads one slot per lane");
  k_corr_hist<<<b.nblk_cell4, kThreads, 0, s>>>(b.reps, b.blk_cell4, b.nrep, b.corr);
  k_corr_add<<<b.nrep, 32, 0, s>>>(b.reps, b.nrep, b.corr);
  return cudaGetLastError();
}

}  // namespace cvf
