// Flag_chessboard = 0 of SOURCE/gpu_water3D.cu ("GW"), the nhb<=4 compatibility mode: every eta
// is 1 (GW:721-724, or the values of input_config), no cube moves, and a hydrogen bond counts in
// the energy only while both cells hold at most NHBMAX = 4 bonds (GW:1964-2007, non-chessboard
// branch). Each cell keeps its bond count as a byte (dev_nhb of the reference), set from the
// configuration (GW:841-862) and moved with every accepted arm update.
//
// Sweep: one launch per (colour, arm): colour 0 arms 0..5, then colour 1 arms 0..5. In one launch
// every cell of the colour updates arm a against the neighbour it faces along a; those
// neighbours are all different and of the other colour, so no two threads touch the same count
// and the cells are independent. The random numbers are the checkerboard sweep's (proposal digit
// a of word 0, acceptance chunk a, the refinement block on a 16-bit tie), so the decisions are
// the same integer comparisons as the oracle's.
//
// Measurement (GW:2064-2099): the reported N_hb counts each bond in typewriter order (cell, then
// x+, y+, z+) for both cells while both hold fewer than 4 counted bonds -- a greedy matching
// whose outcome depends on the order, a problem with no known parallel solution in general (for
// a cap of 1 it is the lexicographically first maximal matching, a P-complete problem). Only a
// cell with 5 or 6 matched bonds can refuse one, so: every matched bond is counted in parallel,
// the cells with 5 or more matched bonds are marked, and a wavefront over the rows replays the
// greedy order, keeping counts for marked cells only (k_nhb_wave: 3L - 2 dependent launches).
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

namespace {

__device__ __forceinline__ int rep_of(const int* __restrict__ blk, int nrep, int b) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(blk + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct Cell {
  uint32_t x, y, z;
};

__device__ __forceinline__ Cell cell_xyz(uint32_t c, uint32_t L) {
  const uint32_t yz = c / L;
  return Cell{c - yz * L, yz % L, yz / L};
}

// The packed word of the cell at (x, y, z).
__device__ __forceinline__ uint32_t word_at(const ReplicaDesc& R, uint32_t x, uint32_t y, uint32_t z) {
  return R.cells[(x + y + z) & 1u][(x >> 1) + (uint32_t)R.H * (y + (uint32_t)R.L * z)];
}

// Neighbour of (x, y, z) along arm a: 0 x+, 1 x-, 2 y+, 3 y-, 4 z+, 5 z- (GW:1936-1962).
__device__ __forceinline__ Cell step_arm(Cell c, int a, uint32_t L) {
  const uint32_t m = L - 1;
  switch (a) {
    case 0: c.x = c.x == m ? 0 : c.x + 1; break;
    case 1: c.x = c.x == 0 ? m : c.x - 1; break;
    case 2: c.y = c.y == m ? 0 : c.y + 1; break;
    case 3: c.y = c.y == 0 ? m : c.y - 1; break;
    case 4: c.z = c.z == m ? 0 : c.z + 1; break;
    default: c.z = c.z == 0 ? m : c.z - 1; break;
  }
  return c;
}

__device__ __forceinline__ uint32_t nat(Cell c, uint32_t L) { return c.x + L * (c.y + L * c.z); }
__device__ __forceinline__ uint32_t field(uint32_t w, int a) { return (w >> (3 * a)) & 7u; }

// GW:841-862: bonds of the cell whose two arms agree, counted where eta = 1 (replica `only`, or
// every replica when only < 0).
__global__ void k_nhb_init(const ReplicaDesc* __restrict__ reps, const int* __restrict__ blk, int nrep, int only) {
  const int r = rep_of(blk, nrep, blockIdx.x);
  if (only >= 0 && r != only) return;
  const ReplicaDesc& R = reps[r];
  const uint32_t L = R.L, N = L * L * L;
  const uint32_t c = (uint32_t)(blockIdx.x - __ldg(blk + r)) * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const Cell p = cell_xyz(c, L);
  const uint32_t w = word_at(R, p.x, p.y, p.z), eta = R.eta6[c];
  uint32_t acc = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const Cell q = step_arm(p, a, L);
    acc += ((eta >> a) & 1u) * (field(w, a) == field(word_at(R, q.x, q.y, q.z), a ^ 1));
  }
  R.nhb[c] = (uint8_t)acc;
}

// One (colour, arm) pass of the sweep; thread = colour word q (N/2 per replica).
__global__ void k_nhb_sweep(const ReplicaDesc* __restrict__ reps, const ReplicaState* __restrict__ st,
                            const int* __restrict__ blk, int nrep, int colour, int a, int jsweep) {
  const int r = rep_of(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t L = R.L, H = R.H, half = L * L * H;
  const uint32_t q = (uint32_t)(blockIdx.x - __ldg(blk + r)) * blockDim.x + threadIdx.x;
  if (q >= half) return;
  const uint32_t t = st[r].cur[0] + (uint32_t)jsweep;
  const uint32_t hx = q % H, yz = q / H, y = yz % L, z = yz / L;
  const Cell p{2 * hx + ((y + z + (uint32_t)colour) & 1u), y, z};
  const uint32_t c0 = nat(p, L);
  uint32_t* own = R.cells[colour] + q;
  const uint32_t w = *own;
  const U4 rr = philox(c0, t, kStSweep, R.replica, R.key0, R.key1);
  uint32_t u = rr.x;
  if (u * 46656u < 2560u) {  // the exact draw of word 0 rejected it (p = 6e-7)
    for (uint32_t k = 0; k < 256; ++k) {
      u = philox(c0, t, retry_tag(kStSweep, k), R.replica, R.key0, R.key1).x;
      if (u * 46656u >= 2560u) break;
    }
  }
  uint32_t f = u, n = 0;
  for (int i = 0; i <= a; ++i) {
    const unsigned long long m = (unsigned long long)f * 6ull;
    n = (uint32_t)(m >> 32);
    f = (uint32_t)m;
  }
  const uint32_t o = field(w, a);
  if (n == o) return;
  const Cell pj = step_arm(p, a, L);
  const uint32_t j = nat(pj, L);
  const uint32_t nb = field(word_at(R, pj.x, pj.y, pj.z), a ^ 1);
  const int dn = (int)(n == nb) - (int)(o == nb);
  const int ni = R.nhb[c0], nj = R.nhb[j];
  const int hbn = (ni + dn <= 4) && (nj + dn <= 4) && n == nb;
  const int hbo = (ni <= 4) && (nj <= 4) && o == nb;
  uint32_t h = 0;
#pragma unroll
  for (int b = 0; b < 6; ++b) h += 1u << (4 * field(w, b));
  const int dns = (int)((h >> (4 * n)) & 15u) - (int)((h >> (4 * o)) & 15u) + 1;
  const int idx = (hbn - hbo + 1) * 11 + dns + 5;
  const unsigned long long T = R.thr_sweep[idx];
  const uint32_t word = a < 2 ? rr.y : (a < 4 ? rr.z : rr.w);
  const uint32_t hu = (a & 1) ? (word >> 16) : (word & 0xffffu);
  bool acc;
  if (hu != (uint32_t)(T >> 16)) {
    acc = hu < (uint32_t)(T >> 16);
  } else {
    const U4 rf = philox(c0, t, kStSweepRefine, R.replica, R.key0, R.key1);
    const uint32_t lw = a < 2 ? rf.x : (a < 4 ? rf.y : rf.z);
    const uint32_t lu = (a & 1) ? (lw >> 16) : (lw & 0xffffu);
    acc = (((unsigned long long)hu << 16) | lu) < T;
  }
  if (acc) {
    *own = (w & ~(7u << (3 * a))) | (n << (3 * a));
    R.nhb[c0] = (uint8_t)(ni + dn);
    R.nhb[j] = (uint8_t)(nj + dn);
  }
}

__global__ void k_nhb_begin(ReplicaState* __restrict__ st, int nrep) {
  const int r = blockIdx.x;
  if (r < nrep && threadIdx.x < 32) {
    st[r].acc_slot[0][threadIdx.x] = 0;
    st[r].acc_slot[1][threadIdx.x] = 0;
  }
}

// sum_{a<b} delta(sigma_a, sigma_b) of one cell (rotations by 1, 2, 3 arms).
__device__ __forceinline__ uint32_t zero_fields6(uint32_t x) {
  return 6u - (uint32_t)__popc((x | (x >> 1) | (x >> 2)) & 0x9249u);
}
__device__ __forceinline__ uint32_t pairs6(uint32_t w) {
  w &= 0x3ffffu;
  const uint32_t r1 = ((w >> 3) | (w << 15)) & 0x3ffffu;
  const uint32_t r2 = ((w >> 6) | (w << 12)) & 0x3ffffu;
  const uint32_t r3 = ((w >> 9) | (w << 9)) & 0x3ffffu;
  return zero_fields6(w ^ r1) + zero_fields6(w ^ r2) + (zero_fields6(w ^ r3) >> 1);
}

// Per cell: the number of its six arms that agree with the arm they face (eta plays no part,
// GW:2064-2099), marked when 5 or more; the matched forward bonds (x+, y+, z+) and the sigma
// pairs summed per block into slot block % 32.
__global__ void k_nhb_mark(const ReplicaDesc* __restrict__ reps, ReplicaState* __restrict__ st,
                           const int* __restrict__ blk, int nrep) {
  __shared__ unsigned long long s_acc[2];
  const int r = rep_of(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t L = R.L, N = L * L * L;
  const uint32_t c = (uint32_t)(blockIdx.x - __ldg(blk + r)) * blockDim.x + threadIdx.x;
  uint32_t fwd = 0, ns = 0;
  if (c < N) {
    const Cell p = cell_xyz(c, L);
    const uint32_t w = word_at(R, p.x, p.y, p.z);
    uint32_t m = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const Cell q = step_arm(p, a, L);
      const uint32_t e = field(w, a) == field(word_at(R, q.x, q.y, q.z), a ^ 1);
      m += e;
      if ((a & 1) == 0) fwd += e;
    }
    R.sat[c] = m >= 5;
    R.cnt[c] = 0;
    ns = pairs6(w);
  }
  if (threadIdx.x < 2) s_acc[threadIdx.x] = 0;
  __syncthreads();
  fwd = __reduce_add_sync(0xffffffffu, fwd);
  ns = __reduce_add_sync(0xffffffffu, ns);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], (unsigned long long)fwd);
    atomicAdd(&s_acc[1], (unsigned long long)ns);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&st[r].acc_slot[0][blockIdx.x & 31], s_acc[0]);
    atomicAdd(&st[r].acc_slot[1][blockIdx.x & 31], s_acc[1]);
  }
}

// The greedy count in typewriter order as a wavefront over rows. Row (y, z) touches the cells
// of rows (y, z), (y+1, z) and (y, z+1) (mod L). Wave t holds the rows with y + 2z = t: rows of
// one wave share no row they touch, and of two bonds that share a cell the one earlier in the
// typewriter order always lies in an earlier wave or earlier in the same row (its backward y
// bond comes from wave t-1 or, wrapped, a later wave; its backward z bond from wave t-2 or,
// wrapped, a later wave). So 3L - 2 waves, each row replayed along x, give exactly the
// sequential result. One warp per row: the lanes load the row's matched forward bonds, the
// marks and the counts of the three rows it touches into shared memory, lane 0 replays the
// row, the lanes store the counts back. Refused bonds are subtracted from the replica's slots
// (modulo 2^64, exact).
constexpr int kWaveWarps = 4;
__global__ void __launch_bounds__(32 * kWaveWarps) k_nhb_wave(const ReplicaDesc* __restrict__ reps,
                                                             ReplicaState* __restrict__ st, int nrep, int t) {
  extern __shared__ uint8_t sm[];
  const int r = blockIdx.y;
  if (r >= nrep) return;
  const ReplicaDesc& R = reps[r];
  const int L = R.L;
  if (t > 3 * L - 3) return;
  const int zlo = t <= L - 1 ? 0 : (t - L + 2) / 2, zhi = min(L - 1, t / 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int z = zlo + (int)blockIdx.x * kWaveWarps + warp;
  if (z > zhi) return;
  const int y = t - 2 * z;
  const uint32_t Lu = (uint32_t)L, yp = y + 1 == L ? 0 : y + 1, zp = z + 1 == L ? 0 : z + 1;
  uint8_t* msk = sm + (size_t)warp * 6 * L;  // bits 0..2 matched x+, y+, z+ bonds, bit 3 marked
  uint8_t* satY = msk + L;
  uint8_t* satZ = satY + L;
  uint8_t* cnt0 = satZ + L;
  uint8_t* cntY = cnt0 + L;
  uint8_t* cntZ = cntY + L;
  for (int x = lane; x < L; x += 32) {
    const uint32_t xu = (uint32_t)x, xn = x + 1 == L ? 0u : xu + 1;
    const uint32_t w = word_at(R, xu, y, z);
    uint32_t m = (uint32_t)(field(w, 0) == field(word_at(R, xn, y, z), 1)) |
                 ((uint32_t)(field(w, 2) == field(word_at(R, xu, yp, z), 3)) << 1) |
                 ((uint32_t)(field(w, 4) == field(word_at(R, xu, y, zp), 5)) << 2);
    const uint32_t c = xu + Lu * ((uint32_t)y + Lu * z), cy = xu + Lu * (yp + Lu * z), cz = xu + Lu * ((uint32_t)y + Lu * zp);
    m |= (uint32_t)R.sat[c] << 3;
    msk[x] = (uint8_t)m;
    satY[x] = R.sat[cy];
    satZ[x] = R.sat[cz];
    cnt0[x] = R.cnt[c];
    cntY[x] = R.cnt[cy];
    cntZ[x] = R.cnt[cz];
  }
  __syncwarp();
  if (lane == 0) {
    unsigned long long refused = 0;
    for (int x = 0; x < L; ++x) {
      const uint32_t m = msk[x];
      if (!(m & 7u)) continue;
      const bool si = (m >> 3) & 1u;
      for (int d = 0; d < 3; ++d) {
        if (!((m >> d) & 1u)) continue;
        const int xn = x + 1 == L ? 0 : x + 1;
        const bool sj = d == 0 ? ((msk[xn] >> 3) & 1u) : (d == 1 ? satY[x] != 0 : satZ[x] != 0);
        uint8_t* cj = d == 0 ? cnt0 + xn : (d == 1 ? cntY + x : cntZ + x);
        if ((!si || cnt0[x] < 4) && (!sj || *cj < 4)) {
          if (si) cnt0[x] = cnt0[x] + 1;
          if (sj) *cj = *cj + 1;
        } else {
          ++refused;
        }
      }
    }
    if (refused) atomicAdd(&st[r].acc_slot[0][z & 31], 0ull - refused);
  }
  __syncwarp();
  for (int x = lane; x < L; x += 32) {
    const uint32_t xu = (uint32_t)x;
    R.cnt[xu + Lu * ((uint32_t)y + Lu * z)] = cnt0[x];
    R.cnt[xu + Lu * (yp + Lu * z)] = cntY[x];
    R.cnt[xu + Lu * ((uint32_t)y + Lu * zp)] = cntZ[x];
  }
}

// The measurement record: N_hb2 = 2 (matched forward bonds - refused bonds), N_sigma.
__global__ void k_nhb_finish(ReplicaState* __restrict__ st, int nrep, int record) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  ReplicaState& S = st[r];
  unsigned long long hb = 0, ns = 0;
  for (int i = 0; i < 32; ++i) {
    hb += S.acc_slot[0][i];
    ns += S.acc_slot[1][i];
  }
  S.acc_hb2 = 2 * hb;
  S.acc_ns = ns;
  SampleRec rec;
  rec.n_hb2 = (long long)S.acc_hb2;
  rec.n_sigma = (long long)ns;
  rec.r_cell = S.r_cell;
  rec.volume = S.volume;
  S.last = rec;
  if (record && S.samples && S.n_samples < S.cap_samples) S.samples[S.n_samples] = rec;
  if (record) S.n_samples++;
}

}  // namespace

void launch_nhb_init(const BatchDev& b, int only, cudaStream_t s) {
  k_nhb_init<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.blk_cell, b.nrep, only);
}

void launch_nhb_sweep(const BatchDev& b, int jsweep, cudaStream_t s) {
  for (int colour = 0; colour < 2; ++colour)
    for (int a = 0; a < 6; ++a)
      k_nhb_sweep<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.st, b.blk_cell, b.nrep, colour, a, jsweep);
}

void launch_nhb_measure(const BatchDev& b, int record, cudaStream_t s) {
  k_nhb_begin<<<b.nrep, 32, 0, s>>>(b.st, b.nrep);
  k_nhb_mark<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.st, b.blk_cell, b.nrep);
  // rows per wave: at most L/2 + 1; one warp and 6L bytes of shared memory per row
  const int rows = b.max_L / 2 + 1;
  const dim3 grid((rows + kWaveWarps - 1) / kWaveWarps, b.nrep);
  const size_t smem = (size_t)kWaveWarps * 6 * b.max_L;
  for (int t = 0; t <= 3 * b.max_L - 3; ++t) k_nhb_wave<<<grid, 32 * kWaveWarps, smem, s>>>(b.reps, b.st, b.nrep, t);
  k_nhb_finish<<<(b.nrep + 127) / 128, 128, 0, s>>>(b.st, b.nrep, record);
}

}  // namespace cvf
