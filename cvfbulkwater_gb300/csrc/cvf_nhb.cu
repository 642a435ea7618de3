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

// Arm a of colour word q of replica R with sweep counter t.
__device__ __forceinline__ void nhb_update(const ReplicaDesc& R, uint32_t q, int colour, int a, uint32_t t) {
  const uint32_t L = R.L, H = R.H;
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

// One (colour, arm) pass of the sweep: thread = colour words q and q + N/4 of its replica (the
// N/2 words of the colour; blk is the table of N/4 threads per replica).
__global__ void k_nhb_sweep(const ReplicaDesc* __restrict__ reps, const ReplicaState* __restrict__ st,
                            const int* __restrict__ blk, int nrep, int colour, int a, int jsweep) {
  const int r = rep_of(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t quarter = (uint32_t)R.L * R.L * R.H / 2;
  const uint32_t q = (uint32_t)(blockIdx.x - __ldg(blk + r)) * blockDim.x + threadIdx.x;
  if (q >= quarter) return;
  const uint32_t t = st[r].cur[0] + (uint32_t)jsweep;
  nhb_update(R, q, colour, a, t);
  nhb_update(R, q + quarter, colour, a, t);
}

__global__ void k_nhb_begin(ReplicaState* __restrict__ st, int nrep) {
  const int r = blockIdx.x;
  if (r < nrep && threadIdx.x < 32) {
    st[r].acc_slot[0][threadIdx.x] = 0;
    st[r].acc_slot[1][threadIdx.x] = 0;
  }
}

// Per cell: which of its six arms agree with the arm they face (eta plays no part,
// GW:2064-2099), stored as the matched forward bonds (bits 0..2: x+, y+, z+) and a mark (bit 3)
// when 5 or more agree; the matched forward bonds and the sigma pairs summed per block into slot
// block % 32.
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
    uint32_t m = 0, bits = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const Cell q = step_arm(p, a, L);
      const uint32_t e = field(w, a) == field(word_at(R, q.x, q.y, q.z), a ^ 1);
      m += e;
      if ((a & 1) == 0) bits |= e << (a >> 1);
    }
    fwd = __popc(bits);
    R.sat[c] = (uint8_t)(bits | (uint32_t)(m >= 5) << 3);
    R.cnt[c] = 0;
    ns = sigma_pairs(w);
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

// One cell's turn in the greedy count (GW:2064-2099): its x+, y+ and z+ bonds in that order.
// m: bits 0..2 the matched bonds, bit 3 the cell is marked; own: its count so far (including the
// x bond from the cell before it); nx/y/z: mark and count of the cell at the other end. Returns
// what the x+ bond adds to the next cell's count (1 when accepted and that cell is marked).
__device__ __forceinline__ uint32_t nhb_turn(uint32_t m, uint32_t& own, uint32_t nx_sat, uint32_t nx_cnt,
                                             uint32_t y_sat, uint32_t& y_cnt, uint32_t z_sat,
                                             uint32_t& z_cnt, uint32_t& refused) {
  const uint32_t si = (m >> 3) & 1u;
  uint32_t out = 0;
  if (m & 1u) {
    if ((!si || own < 4) && (!nx_sat || nx_cnt < 4)) {
      own += si;
      out = nx_sat;
    } else {
      ++refused;
    }
  }
  if (m & 2u) {
    if ((!si || own < 4) && (!y_sat || y_cnt < 4)) {
      own += si;
      y_cnt += y_sat;
    } else {
      ++refused;
    }
  }
  if (m & 4u) {
    if ((!si || own < 4) && (!z_sat || z_cnt < 4)) {
      own += si;
      z_cnt += z_sat;
    } else {
      ++refused;
    }
  }
  return out;
}

// The greedy count in typewriter order as a wavefront over rows. Row (y, z) touches the cells
// of rows (y, z), (y+1, z) and (y, z+1) (mod L). Wave t holds the rows with y + 2z = t: rows of
// one wave share no row they touch, and of two bonds that share a cell the one earlier in the
// typewriter order always lies in an earlier wave or earlier in the same row (its backward y
// bond comes from wave t-1 or, wrapped, a later wave; its backward z bond from wave t-2 or,
// wrapped, a later wave). So 3L - 2 waves, each row replayed along x, give exactly the
// sequential result. One warp per row: the lanes load the row's matched forward bonds, the
// marks and the counts of the three rows it touches into shared memory, replay the row, and
// store the counts back. Refused bonds are subtracted from the replica's slots (modulo 2^64,
// exact).
//
// Along the row only the x bonds chain the cells: what cell x's x+ bond adds to cell x+1's count
// (0 or 1) is a function of what cell x-1's added to cell x's, and the y and z partners are
// distinct cells. So each lane takes ceil(L/32) consecutive cells, evaluates that function for
// both inputs over its cells, a warp scan composes the functions (exclusive, from 0 at x = 0),
// and each lane replays its cells with the true input. The wrapped bond of x = L-1 meets cell 0
// after cell 0's own turn, whose outcome does not depend on the chain.
constexpr int kWaveWarps = 4;
__global__ void __launch_bounds__(32 * kWaveWarps) k_nhb_wave(const ReplicaDesc* __restrict__ reps,
                                                             ReplicaState* __restrict__ st, int nrep, int t) {
  extern __shared__ uint8_t sm[];
  pdl_trigger();
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
  // the warp's six rows of L bytes in shared memory, indexed from sm itself: bits 0..2 matched
  // x+, y+, z+ bonds and bit 3 the mark of row (y, z); the marks of rows (y+1, z) and (y, z+1);
  // the counts of the three rows
  const int bM = warp * 6 * L, bSY = bM + L, bSZ = bSY + L, bC0 = bSZ + L, bCY = bC0 + L, bCZ = bCY + L;
  const uint8_t* __restrict__ gsat = R.sat;
  uint8_t* __restrict__ gcnt = R.cnt;
  const uint32_t o0 = Lu * ((uint32_t)y + Lu * z), oY = Lu * (yp + Lu * z), oZ = Lu * ((uint32_t)y + Lu * zp);
  pdl_wait();
#pragma unroll 4
  for (int x = lane; x < L; x += 32) {
    const uint8_t m = gsat[o0 + x], sy = gsat[oY + x], sz = gsat[oZ + x];
    const uint8_t c0v = __ldcg(gcnt + o0 + x), cyv = __ldcg(gcnt + oY + x), czv = __ldcg(gcnt + oZ + x);
    sm[bM + x] = m;
    sm[bSY + x] = sy >> 3;
    sm[bSZ + x] = sz >> 3;
    sm[bC0 + x] = c0v;
    sm[bCY + x] = cyv;
    sm[bCZ + x] = czv;
  }
  __syncwarp();
  const int per = (L + 31) >> 5;
  const int x0 = min(L, lane * per), x1 = min(L, x0 + per);
  uint32_t refused = 0, scratch = 0;
  // cell 0 after its own turn, which the wrapped bond of x = L-1 meets
  uint32_t c0 = sm[bC0];
  if (L > 1) {
    uint32_t yc = sm[bCY], zc = sm[bCZ];
    nhb_turn(sm[bM], c0, sm[bM + 1] >> 3, sm[bC0 + 1], sm[bSY], yc, sm[bSZ], zc, scratch);
  }
  // the count of cell x1 before the chain reaches it (lane + 1 overwrites it in the replay)
  const uint32_t next_init = x1 < L ? sm[bC0 + x1] : c0;
  // this lane's cells as a function of the input, both inputs side by side: bit i = output for
  // input i
  uint32_t cur0 = 0, cur1 = 1;
  for (int x = x0; x < x1; ++x) {
    const bool last = x + 1 == L;
    const uint32_t m = sm[bM + x], nsat = sm[bM + (last ? 0 : x + 1)] >> 3, ncnt = last ? c0 : sm[bC0 + x + 1];
    const uint32_t sy = sm[bSY + x], sz = sm[bSZ + x], cy = sm[bCY + x], cz = sm[bCZ + x], cc = sm[bC0 + x];
    uint32_t own0 = cc + cur0, own1 = cc + cur1, y0 = cy, y1 = cy, z0 = cz, z1 = cz;
    cur0 = nhb_turn(m, own0, nsat, ncnt, sy, y0, sz, z0, scratch);
    cur1 = nhb_turn(m, own1, nsat, ncnt, sy, y1, sz, z1, scratch);
  }
  uint32_t f = x0 == x1 ? 2u : (cur0 | (cur1 << 1));  // no cells: the identity
  // inclusive scan of the composition (earlier lanes' function applied first)
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t g = __shfl_up_sync(0xffffffffu, f, off);
    if (lane >= off) f = ((f >> (g & 1u)) & 1u) | (((f >> ((g >> 1) & 1u)) & 1u) << 1);
  }
  const uint32_t before = __shfl_up_sync(0xffffffffu, f, 1);
  uint32_t cur = lane == 0 ? 0u : (before & 1u);
  __syncwarp();
  for (int x = x0; x < x1; ++x) {
    uint32_t own = sm[bC0 + x] + cur, yc = sm[bCY + x], zc = sm[bCZ + x];
    const bool last = x + 1 == L;
    const uint32_t nc = last ? c0 : (x + 1 == x1 ? next_init : sm[bC0 + x + 1]);
    cur = nhb_turn(sm[bM + x], own, sm[bM + (last ? 0 : x + 1)] >> 3, nc, sm[bSY + x], yc, sm[bSZ + x], zc,
                   refused);
    sm[bC0 + x] = (uint8_t)own;
    sm[bCY + x] = (uint8_t)yc;
    sm[bCZ + x] = (uint8_t)zc;
  }
  const uint32_t wrap = __shfl_sync(0xffffffffu, cur, (L - 1) / per);
  if (lane == 0 && L > 1) sm[bC0] = (uint8_t)(sm[bC0] + wrap);
  refused = __reduce_add_sync(0xffffffffu, refused);
  if (lane == 0 && refused) atomicAdd(&st[r].acc_slot[0][z & 31], 0ull - (unsigned long long)refused);
  __syncwarp();
  for (int x = lane; x < L; x += 32) {
    gcnt[o0 + x] = sm[bC0 + x];
    gcnt[oY + x] = sm[bCY + x];
    gcnt[oZ + x] = sm[bCZ + x];
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
      k_nhb_sweep<<<b.nblk_cell4, kThreads, 0, s>>>(b.reps, b.st, b.blk_cell4, b.nrep, colour, a, jsweep);
}

void launch_nhb_measure(const BatchDev& b, int record, cudaStream_t s) {
  k_nhb_begin<<<b.nrep, 32, 0, s>>>(b.st, b.nrep);
  k_nhb_mark<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.st, b.blk_cell, b.nrep);
  // rows per wave: at most L/2 + 1; one warp and 6L bytes of shared memory per row
  const int rows = b.max_L / 2 + 1;
  const dim3 grid((rows + kWaveWarps - 1) / kWaveWarps, b.nrep);
  const size_t smem = (size_t)kWaveWarps * 6 * b.max_L;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(32 * kWaveWarps);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  for (int t = 0; t <= 3 * b.max_L - 3; ++t) {
    cfg.numAttrs = t > 0 && b.pdl ? 1 : 0;  // each wave a programmatic dependent of the one before
    cudaLaunchKernelEx(&cfg, k_nhb_wave, (const ReplicaDesc*)b.reps, b.st, b.nrep, t);
  }
  k_nhb_finish<<<(b.nrep + 127) / 128, 128, 0, s>>>(b.st, b.nrep, record);
}

}  // namespace cvf
