// Monte Carlo kernels of the GB300 CVF engine: lattice initialisation, the NPT volume move,
// the eta cube ("chessboard") move, the checkerboard sigma sweep and the exact int64
// observable reductions. Reference: SOURCE/gpu_water3D.cu ("GW") of lcoronas/CVFBulkWater.
//
// The sweep is integer-issue bound (one Philox4x32-10 block and six table-driven Metropolis
// decisions per cell), so its hot path is branch-free: every arm is decided with 16-bit
// uniforms against a shared-memory threshold table, and the two rare events -- a proposal word
// rejected by the exact uniform draw (p = 6e-7) and a 16-bit tie that needs the low half of the
// uniform (p ~ 2^-16 per arm) -- leave the hot path for out-of-line exact code.
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

__constant__ uint32_t c_state_active[9];
__constant__ uint8_t c_eta_table[72];  // [state*8 + vertex offset] -> 6-bit eta mask

void init_sw_device_tables();
static unsigned long long g_tables_ready = 0;  // bit d: tables copied to device d

// Copies the cube tables to the current device's constant memory (once per device).
void init_device_tables() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && ((g_tables_ready >> dev) & 1ull)) return;
  uint32_t act[9];
  uint8_t eta[72];
  for (int s = 0; s < 9; ++s) {
    act[s] = state_active(s);
    for (int p = 0; p < 8; ++p) eta[s * 8 + p] = (uint8_t)cube_eta_bits(s, p);
  }
  cudaMemcpyToSymbol(c_state_active, act, sizeof(act));
  cudaMemcpyToSymbol(c_eta_table, eta, sizeof(eta));
  init_sw_device_tables();
  if (dev < 64) g_tables_ready |= 1ull << dev;
}

// Block -> replica through the prefix table blk[0..nrep] (blk[0] = 0).
__device__ __forceinline__ int find_replica(const int* __restrict__ blk, int nrep, int b) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(blk + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// n / d and n % d; shift >= 0 means d = 2^shift.
__device__ __forceinline__ void divmod32(uint32_t n, uint32_t d, int shift, uint32_t& q, uint32_t& r) {
  if (shift >= 0) {
    q = n >> shift;
    r = n & (d - 1u);
  } else {
    q = n / d;
    r = n - q * d;
  }
}

// Block vb of the cube table -> (cube parity, cube index): a replica's cube blocks are split in
// two equal halves, the first for the cubes with all-even origins, the second for all-odd
// origins, so the parity is uniform inside a block.
__device__ __forceinline__ bool cube_of(const int* __restrict__ blk, int r, int vb, int H, uint32_t& par,
                                        uint32_t& qi) {
  const int b0 = __ldg(blk + r), half = (__ldg(blk + r + 1) - b0) >> 1;
  const int lb = vb - b0;
  par = lb >= half;
  qi = (uint32_t)(lb - (int)par * half) * blockDim.x + threadIdx.x;
  return qi < (uint32_t)H * H * H;
}

__device__ __forceinline__ uint32_t cell_word_index(int x, int y, int z, int L, int H) {
  return (uint32_t)(x >> 1) + (uint32_t)H * ((uint32_t)y + (uint32_t)L * (uint32_t)z);
}

// ------------------------------------------------------------------ measurement slots
// Block sum of the per-thread counts into slot vb % 32 of replica state S (all threads of the
// block call it; s_acc is the block's two-word scratch).
__device__ __forceinline__ void measure_accumulate(ReplicaState& S, int vb, uint32_t hb2, uint32_t ns,
                                                   unsigned long long* s_acc) {
  if (threadIdx.x < 2) s_acc[threadIdx.x] = 0;
  __syncthreads();
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    hb2 += __shfl_xor_sync(0xffffffffu, hb2, o);
    ns += __shfl_xor_sync(0xffffffffu, ns, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], (unsigned long long)hb2);
    atomicAdd(&s_acc[1], (unsigned long long)ns);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&S.acc_slot[0][vb & 31], s_acc[0]);
    atomicAdd(&S.acc_slot[1][vb & 31], s_acc[1]);
  }
}

__device__ __forceinline__ void measure_zero(ReplicaState& S) {
  for (int i = 0; i < 32; ++i) {
    S.acc_slot[0][i] = 0;
    S.acc_slot[1][i] = 0;
  }
}

// Sums the slots into the replica's last measurement and appends it to the sample stream when
// record is set.
__device__ __forceinline__ void measure_finish(ReplicaState& S, int record) {
  unsigned long long hb2 = 0, ns = 0;
  for (int i = 0; i < 32; ++i) {
    hb2 += S.acc_slot[0][i];
    ns += S.acc_slot[1][i];
  }
  S.acc_hb2 = hb2;
  S.acc_ns = ns;
  SampleRec rec;
  rec.n_hb2 = (long long)hb2;
  rec.n_sigma = (long long)ns;
  rec.r_cell = S.r_cell;
  rec.volume = S.volume;
  S.last = rec;
  if (record && S.samples && S.n_samples < S.cap_samples) S.samples[S.n_samples] = rec;
  if (record) S.n_samples++;
}

// ------------------------------------------------------------------ initialisation
// GW:812-825: disordered start draws each sigma uniformly, ordered start one common value.
__global__ void k_init_sigma(const ReplicaDesc* __restrict__ reps, const int* __restrict__ blk, int nrep) {
  int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int start = R.start;
  const int L = R.L, H = R.H;
  uint32_t c = (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  uint32_t N = (uint32_t)L * L * L;
  if (c >= N) return;
  uint32_t x, yz, y, z;
  divmod32(c, L, R.lgL, yz, x);
  divmod32(yz, L, R.lgL, z, y);
  uint32_t w = 0;
  if (start == 2) {
    U4 q = philox(0, 0, kStInitOrder, R.replica, R.key0, R.key1);
    uint32_t v;
    if (!lemire_try(q.x, 6, v) && !lemire_try(q.y, 6, v) && !lemire_try(q.z, 6, v) && !lemire_try(q.w, 6, v))
      v = lemire_retry(6, 0, 0, kStInitOrder, R.replica, R.key0, R.key1);
    for (int a = 0; a < 6; ++a) w |= v << (3 * a);
  } else if (start == 0) {
    U4 q = philox(c, 0, kStInitSigma, R.replica, R.key0, R.key1);
    uint32_t d;
    if (!lemire_try(q.x, 46656u, d) && !lemire_try(q.y, 46656u, d) && !lemire_try(q.z, 46656u, d) &&
        !lemire_try(q.w, 46656u, d))
      d = lemire_retry(46656u, c, 0, kStInitSigma, R.replica, R.key0, R.key1);
    for (int a = 0; a < 6; ++a) {
      w |= (d % 6u) << (3 * a);
      d /= 6u;
    }
  }
  R.cells[(x + y + z) & 1][cell_word_index(x, y, z, L, H)] = w;
}

// GW:3259-3312: every cube starts in a uniformly drawn state.
__global__ void k_init_cubes(const ReplicaDesc* __restrict__ reps, const int* __restrict__ blk, int nrep) {
  int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int L = R.L, H = R.H;
  uint32_t par, qi;
  if (!cube_of(blk, r, blockIdx.x, H, par, qi)) return;
  uint32_t a, bc, b, c;
  divmod32(qi, H, R.lgH, bc, a);
  divmod32(bc, H, R.lgH, c, b);
  uint32_t x0 = 2 * a + par, y0 = 2 * b + par, z0 = 2 * c + par;
  uint32_t cid = x0 + (uint32_t)L * (y0 + (uint32_t)L * z0);
  U4 w = philox(cid, 0, kStInitCube, R.replica, R.key0, R.key1);
  uint32_t st;
  if (!lemire_try(w.x, 9, st) && !lemire_try(w.y, 9, st) && !lemire_try(w.z, 9, st) && !lemire_try(w.w, 9, st))
    st = lemire_retry(9, cid, 0, kStInitCube, R.replica, R.key0, R.key1);
  R.cubes[par][qi] = (uint8_t)st;
}

// ------------------------------------------------------------------ step begin: move counters
// One thread per replica: snapshot the move counters that this step's kernels use.
__global__ void k_step_begin(ReplicaState* __restrict__ st, int nrep, int nmet, int ncl, int do_cube,
                             int do_volume, int zero_slots) {
  pdl_trigger();
  pdl_wait();
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  ReplicaState& S = st[r];
  if (zero_slots) measure_zero(S);
  S.cur[0] = S.ctr[0];
  S.ctr[0] += (uint32_t)nmet;
  S.cur[1] = S.ctr[1];
  S.ctr[1] += (uint32_t)do_cube;
  if (do_volume) {  // otherwise a side branch may be moving the volume counter
    S.cur[2] = S.ctr[2];
    S.ctr[2] += 1u;
  }
  S.cur[3] = S.ctr[3];
  S.ctr[3] += (uint32_t)ncl;
}

// The counters after a chunk of `steps` steps whose kernels took them as offsets from ctr (step
// i: cube ctr[1] + i, volume ctr[2] + i, sweep j ctr[0] + i*nmet + j, SW step j ctr[3] + i*ncl +
// j): ctr advanced and cur left as the last step's k_step_begin would leave them. One launch per
// chunk instead of one k_step_begin per step.
__global__ void k_chunk_end(ReplicaState* __restrict__ st, int nrep, int steps, int nmet, int ncl, int do_volume) {
  pdl_trigger();
  pdl_wait();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  ReplicaState& S = st[r];
  const uint32_t last = (uint32_t)(steps - 1);
  S.cur[0] = S.ctr[0] + last * (uint32_t)nmet;
  S.ctr[0] += (uint32_t)(steps * nmet);
  S.cur[1] = S.ctr[1] + last;
  S.ctr[1] += (uint32_t)steps;
  if (do_volume) {  // otherwise the side branch moves the volume counter
    S.cur[2] = S.ctr[2] + last;
    S.ctr[2] += (uint32_t)steps;
  }
  S.cur[3] = S.ctr[3] + last * (uint32_t)ncl;
  S.ctr[3] += (uint32_t)(steps * ncl);
}

// ------------------------------------------------------------------ volume move (one warp)
// NPT volume move of GW:1740-1781 in FP64, every operation rounded separately. The shell terms
// of E_vdW(r') are computed by the 32 lanes and summed by lane 0 in shell order, which is the
// reference's sequential sum.
__device__ void volume_move_warp(const ReplicaDesc& R, ReplicaState& S, uint32_t t) {
  __shared__ double s_term[kMaxShells];
  __shared__ double s_trial;
  const int lane = threadIdx.x & 31;
  U4 q = philox(0, t, kStVolume, R.replica, R.key0, R.key1);
  const double r0 = S.r_cell;
  if (lane == 0) {
    double u1 = u53(q.x, q.y);
    double trial = CVF_DADD(r0, CVF_DMUL(0.01 * 2, CVF_DSUB(u1, 0.5)));
    for (uint32_t k = 1; trial < 0.0 && k < 64; ++k) {
      U4 qq = philox(k, t, kStVolume, R.replica, R.key0, R.key1);
      u1 = u53(qq.x, qq.y);
      trial = CVF_DADD(r0, CVF_DMUL(0.01 * 2, CVF_DSUB(u1, 0.5)));
    }
    s_trial = trial;
  }
  __syncwarp();
  const double trial = s_trial;
  const double shift = R.vdw_shift;  // the same expression, evaluated once on the host
  for (int i = lane; i < R.n_shells; i += 32) {
    double rd = CVF_DMUL(trial, (double)R.dist[i]);
    double term;
    if (rd < (double)R.Rc) {
      double u = 1.0 / rd;
      u = CVF_DMUL(CVF_DMUL(u, u), u);
      double a6 = CVF_DMUL(u, u);
      double a12 = CVF_DMUL(a6, a6);
      term = CVF_DMUL((double)R.freq[i], CVF_DSUB(CVF_DSUB(a12, a6), shift));
    } else {
      term = __longlong_as_double(0x7FF8000000000001ll);  // NaN marks a shell beyond the cut-off
    }
    s_term[i] = term;
  }
  __syncwarp();
  if (lane != 0) return;
  double tE = 0.0;
  for (int i = 0; i < R.n_shells; ++i) {
    double term = s_term[i];
    if (term == term) tE = CVF_DADD(tE, term);
  }
  const double Ld = (double)R.L;
  double tV = CVF_DMUL(CVF_DMUL(CVF_DMUL(CVF_DMUL(CVF_DMUL(trial, trial), trial), Ld), Ld), Ld);
  double dV = CVF_DSUB(tV, S.volume);
  float Nf = (float)((long long)R.L * R.L * R.L);
  double NT = (double)__fmul_rn(Nf, R.T);
  double dE = CVF_DSUB(CVF_DSUB(tE, S.e_vdw), CVF_DMUL(NT, own_log(tV / S.volume)));
  double u2 = u53(q.z, q.w);
  double arg = CVF_DMUL(-R.beta, CVF_DADD(dE, CVF_DMUL((double)R.P, dV)));
  // own_exp(arg) >= 1 > u2 for arg >= 0 (the last Horner step adds a non-negative product to
  // 1.0, or the power of two is at least 2), so the exponential is needed only below zero
  if (arg >= 0.0 || u2 < own_exp(arg)) {
    S.r_cell = trial;
    S.volume = tV;
    S.e_vdw = tE;
  }
}

// The volume moves of `steps` consecutive steps of replica blockIdx.x (one warp), with the volume
// counters ctr[2], ctr[2] + 1, ...; the counter advances by `steps` at the end. The volume chain
// reads and writes only r_cell, volume and e_vdw, which the cube moves and sweeps neither read
// nor write (the acceptance of sigma and eta moves does not depend on the volume), so a chunk's
// volume moves can run beside its other kernels.
__global__ void __launch_bounds__(32) k_volume_chain(const ReplicaDesc* __restrict__ reps,
                                                    ReplicaState* __restrict__ st, int nrep, int steps) {
  const int r = blockIdx.x;
  if (r >= nrep) return;
  ReplicaState& S = st[r];
  const uint32_t t0 = S.ctr[2];
  for (int i = 0; i < steps; ++i) {
    volume_move_warp(reps[r], S, t0 + (uint32_t)i);
    __syncwarp();
  }
  if (threadIdx.x == 0) S.ctr[2] = t0 + (uint32_t)steps;
}

// ------------------------------------------------------------------ vector access helpers
template <int V>
struct VecLoad;
template <>
struct VecLoad<1> {
  static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* w) { w[0] = *p; }
  static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* w) { *p = w[0]; }
};
template <>
struct VecLoad<2> {
  static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* w) {
    uint2 t = *reinterpret_cast<const uint2*>(p);
    w[0] = t.x;
    w[1] = t.y;
  }
  static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* w) {
    *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
  }
};
template <>
struct VecLoad<4> {
  static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* w) {
    uint4 t = *reinterpret_cast<const uint4*>(p);
    w[0] = t.x;
    w[1] = t.y;
    w[2] = t.z;
    w[3] = t.w;
  }
  static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* w) {
    *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
  }
};
template <>
struct VecLoad<8> {
  static __device__ __forceinline__ void ld(const uint32_t* p, uint32_t* w) {
    VecLoad<4>::ld(p, w);
    VecLoad<4>::ld(p + 4, w + 4);
  }
  static __device__ __forceinline__ void st(uint32_t* p, const uint32_t* w) {
    VecLoad<4>::st(p, w);
    VecLoad<4>::st(p + 4, w + 4);
  }
};
template <int V>
struct Log2V;
template <>
struct Log2V<8> {
  static constexpr int v = 3;
};
template <>
struct Log2V<1> {
  static constexpr int v = 0;
};
template <>
struct Log2V<2> {
  static constexpr int v = 1;
};
template <>
struct Log2V<4> {
  static constexpr int v = 2;
};

// ------------------------------------------------------------------ cube move (+ volume blocks)
// Warp-private copy of the cube tables (a warp reads 9 distinct words at most, so the random
// lookups of its 32 cubes neither serialise like divergent constant-bank reads nor conflict).
//   act[s]  12-bit mask of the cube edges that carry eta = 1 in state s
//   thr[i]  acceptance threshold of dN_hb = i - 4 (U < thr, thr in [0, 2^32])
struct CubeTables {
  unsigned long long thr[9];
  uint32_t act[9];
};

__device__ __forceinline__ void fill_cube_tables(const ReplicaDesc& R, CubeTables* ct, int lane) {
  if (lane < 9) {
    ct->thr[lane] = R.thr_cube[lane];
    ct->act[lane] = c_state_active[lane];
  }
}

// The accepted raw proposal word of a cube group when words 0 and 3 both fell in the rejected
// range of the exact draw in [0, 9^4) (p ~ 1.3e-6 each).
__device__ __noinline__ uint32_t cube_proposal_retry(uint32_t gid, uint32_t t, const ReplicaDesc* R) {
  uint32_t w = 0;
  for (uint32_t k = 0; k < 256; ++k) {
    w = philox(gid, t, retry_tag(kStCube, k), R->replica, R->key0, R->key1).x;
    if (w * 6561u >= 5476u) return w;
  }
  return w;
}

// Acceptance of cube kk of a group when the high half hu of its uniform tied with T >> 16: the
// low half from the group's refinement block.
__device__ __noinline__ bool cube_accept_exact(uint32_t gid, uint32_t t, uint32_t kk, uint32_t hu,
                                               unsigned long long T, const ReplicaDesc* R) {
  const U4 rf = philox(gid, t, kStCubeRefine, R->replica, R->key0, R->key1);
  const uint32_t word = kk < 2 ? rf.y : rf.z;
  const uint32_t lo = (kk & 1) ? (word >> 16) : (word & 0xffffu);
  return ((((unsigned long long)hu) << 16) | lo) < T;
}

// GW:3374-3466. One thread per VC consecutive cubes along x of one parity (both parities in one
// launch: cubes share no edge and sigma is frozen, so all cube decisions are independent). The
// parity of the block's index among the replica's blocks in the table blk (blk_cubev) is the
// cubes' parity, even origins (2a,2b,2c) or odd origins (2a+1,2b+1,2c+1), and block pairs 2i,
// 2i+1 take the same chunk of each: the two reads of every cell (one per cube containing it)
// come close together, the second from L2. Vertex p = dx | dy<<1 | dz<<2 of
// cube (a,b,c) has colour (parity + popc(p)) & 1 and word (x>>1) + H*(y + L*z), which is a for
// every vertex except dx = 1 of an odd cube (a + 1, wrapping at the row end): the VC cubes read
// each vertex row with one VC-word access, the odd dx = 1 rows with one more word. Their VC state
// bytes are one aligned word, written back when a state changed. t is the cube-move counter of
// the step. Plain (coherent) loads: the persistent step kernel reads cells that other blocks
// wrote earlier in the same launch.
template <int VC>
__device__ __forceinline__ void cube_move_v(const ReplicaDesc& R, const CubeTables* ct, const int* __restrict__ blk,
                                            int r, int vb, uint32_t t) {
  const uint32_t L = R.L, H = R.H, cpr = H / VC;
  const int lb = vb - __ldg(blk + r);
  const uint32_t par = (uint32_t)lb & 1u;
  const uint32_t qi = (uint32_t)(lb >> 1) * blockDim.x + threadIdx.x;
  if (qi >= cpr * H * H) return;
  uint32_t seg, bc, b, c;
  divmod32(qi, cpr, R.lgH >= 0 ? R.lgH - Log2V<VC>::v : -1, bc, seg);
  divmod32(bc, H, R.lgH, c, b);
  const uint32_t a0 = seg * VC;
  const uint32_t y0 = 2 * b + par, z0 = 2 * c + par;
  const uint32_t y1 = y0 + 1 == L ? 0 : y0 + 1, z1 = z0 + 1 == L ? 0 : z0 + 1;
  // one Philox block per group of four cubes along x (the thread's VC cubes lie in one group):
  // words 0, 3 give the four proposals as base-9 digits of an exact uniform in [0, 9^4), words
  // 1, 2 the high halves of the four acceptance uniforms. Drawn before the vertex words are
  // loaded, so the rare retry call holds few live registers.
  const uint32_t kk0 = a0 & 3u;
  const uint32_t gid = 2 * (a0 - kk0) + par + L * (y0 + L * z0);
  const U4 rr = philox(gid, t, kStCube, R.replica, R.key0, R.key1);
  uint32_t u = rr.x;
  if (u * 6561u < 5476u) u = rr.w;
  if (u * 6561u < 5476u) u = cube_proposal_retry(gid, t, &R);
  uint32_t dig[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const unsigned long long m = (unsigned long long)u * 9ull;
    dig[j] = (uint32_t)(m >> 32);
    u = (uint32_t)m;
  }
  const uint32_t rows[4] = {H * (y0 + L * z0), H * (y1 + L * z0), H * (y0 + L * z1), H * (y1 + L * z1)};
  const uint32_t anext = a0 + VC == H ? 0 : a0 + VC;
  uint32_t w[8][VC];
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const uint32_t* arr = R.cells[(par + (uint32_t)__popc(p)) & 1u] + rows[p >> 1];
    VecLoad<VC>::ld(arr + a0, w[p]);
    if ((p & 1) && par) {  // x = 2a + 2: words a0+1 .. a0+VC
      const uint32_t nxt = arr[anext];
#pragma unroll
      for (int k = 0; k < VC; ++k) w[p][k] = k + 1 < VC ? w[p][k + 1] : nxt;
    }
  }
  uint8_t* cs = R.cubes[par] + a0 + H * bc;
  uint32_t st[VC];
  uint32_t packed;
  if (VC == 4) packed = *reinterpret_cast<const uint32_t*>(cs);
  else if (VC == 2) packed = *reinterpret_cast<const uint16_t*>(cs);
  else packed = *cs;
#pragma unroll
  for (int k = 0; k < VC; ++k) st[k] = (packed >> (8 * k)) & 0xffu;
  // decisions from the 16-bit high halves; a tie (p ~ 2^-16 per cube) is settled after the loop,
  // once the vertex words are dead
  uint32_t nwk[VC];
  int dhk[VC];
  uint32_t acc_mask = 0, tie_mask = 0;
#pragma unroll
  for (int k = 0; k < VC; ++k) {
    // edge e along d from p0 to p1: sigma_{2d}(p0) == sigma_{2d+1}(p1), compared in place by
    // shifting the start word one field up
    uint32_t D = 0;
#pragma unroll
    for (int e = 0; e < 12; ++e) {
      const int d = edge_dir(e), p0 = edge_start(e), p1 = p0 | (1 << d);
      const uint32_t x = ((w[p0][k] << 3) ^ w[p1][k]) & (7u << (6 * d + 3));
      D |= (x == 0u ? 1u : 0u) << e;
    }
    const uint32_t kk = VC == 4 ? (uint32_t)k : kk0 + (uint32_t)k;
    const uint32_t nw = VC == 4 ? dig[k] : (kk == 0 ? dig[0] : (kk == 1 ? dig[1] : (kk == 2 ? dig[2] : dig[3])));
    const int dhb = __popc(ct->act[nw] & D) - __popc(ct->act[st[k]] & D);
    const uint32_t word = kk < 2 ? rr.y : rr.z;
    const uint32_t hu = (kk & 1) ? (word >> 16) : (word & 0xffffu);
    const uint32_t th = (uint32_t)(ct->thr[dhb + 4] >> 16);
    acc_mask |= (hu < th ? 1u : 0u) << k;
    tie_mask |= (hu == th ? 1u : 0u) << k;
    nwk[k] = nw;
    dhk[k] = dhb;
  }
  if (tie_mask) {
#pragma unroll
    for (int k = 0; k < VC; ++k)
      if ((tie_mask >> k) & 1u) {
        const uint32_t kk = VC == 4 ? (uint32_t)k : kk0 + (uint32_t)k;
        const uint32_t word = kk < 2 ? rr.y : rr.z;
        const uint32_t hu = (kk & 1) ? (word >> 16) : (word & 0xffffu);
        if (cube_accept_exact(gid, t, kk, hu, ct->thr[dhk[k] + 4], &R)) acc_mask |= 1u << k;
      }
  }
  bool changed = false;
#pragma unroll
  for (int k = 0; k < VC; ++k) {
    if (((acc_mask >> k) & 1u) && nwk[k] != st[k]) {
      st[k] = nwk[k];
      changed = true;
    }
  }
  if (changed) {
    uint32_t out = 0;
#pragma unroll
    for (int k = 0; k < VC; ++k) out |= st[k] << (8 * k);
    if (VC == 4) *reinterpret_cast<uint32_t*>(cs) = out;
    else if (VC == 2) *reinterpret_cast<uint16_t*>(cs) = (uint16_t)out;
    else *cs = (uint8_t)out;
  }
}

__device__ __forceinline__ void cube_move(const ReplicaDesc& R, const CubeTables* ct, const int* __restrict__ blk,
                                          int r, int vb, uint32_t t) {
  if (R.cvec == 4) cube_move_v<4>(R, ct, blk, r, vb, t);
  else if (R.cvec == 2) cube_move_v<2>(R, ct, blk, r, vb, t);
  else cube_move_v<1>(R, ct, blk, r, vb, t);
}

// The volume move of replica b for the first nvol blocks b (one warp each: scheduled first, they
// run beside the cube blocks), then the cube moves of every replica, both with the counters of the
// current step.
__global__ void __launch_bounds__(kThreads, 4) k_cube_volume(const ReplicaDesc* __restrict__ reps,
                                                          ReplicaState* __restrict__ st,
                                                          const int* __restrict__ blk, int nrep, int nvol,
                                                          int soff) {
  pdl_trigger();
  if ((int)blockIdx.x < nvol) {
    pdl_wait();
    const int r = blockIdx.x;
    if (threadIdx.x < 32 && r < nrep)
      volume_move_warp(reps[r], st[r], soff < 0 ? st[r].cur[2] : st[r].ctr[2] + (uint32_t)soff);
    return;
  }
  __shared__ CubeTables s_ct[kThreads / 32];
  const int vb = (int)blockIdx.x - nvol;
  const int r = find_replica(blk, nrep, vb);
  const ReplicaDesc& R = reps[r];
  CubeTables* ct = s_ct + (threadIdx.x >> 5);
  fill_cube_tables(R, ct, threadIdx.x & 31);
  __syncwarp();
  pdl_wait();
  cube_move(R, ct, blk, r, vb, soff < 0 ? st[r].cur[1] : st[r].ctr[1] + (uint32_t)soff);
}

// ------------------------------------------------------------------ checkerboard sweep
// Thread -> (row segment, y, z) of a replica's colour array: q = hc + (H/V) * row. Rows run by y
// then z (row = y + L*z), or with R.lgty >= 0 in tiles of TY = 2^lgty rows in y: row = yi + TY*(z
// + L*yt), y = TY*yt + yi, so the consecutive threads of a block cover TY rows in y and several
// planes in z. The order only places work on threads; every cell's update is the same.
template <int V>
__device__ __forceinline__ bool segment_of(const ReplicaDesc& R, uint32_t q, int& hc, int& y, int& z) {
  const uint32_t L = R.L, cpr = R.H / V;
  if (q >= cpr * L * L) return false;
  uint32_t row, hh, zz, yy;
  divmod32(q, cpr, R.lgH >= 0 ? R.lgH - Log2V<V>::v : -1, row, hh);
  if (R.lgty < 0) {
    divmod32(row, L, R.lgL, zz, yy);
  } else {
    uint32_t yt;
    divmod32(row >> R.lgty, L, R.lgL, yt, zz);
    yy = (yt << R.lgty) + (row & ((1u << R.lgty) - 1u));
  }
  hc = (int)hh;
  y = (int)yy;
  z = (int)zz;
  return true;
}

// Loads the V own words of a thread's row segment, the other colour's words around them and
// the eta masks of the V cells. Shared by the sweep and the measurement.
template <int V>
struct CellBlock {
  uint32_t own[V], xp[V], xm[V], yp[V], ym[V], zp[V], zm[V];
  uint32_t eta[V];
  uint32_t* own_ptr;
  int x0, y, z, s;

  static __device__ __forceinline__ void ld_bytes(const uint8_t* a, uint32_t* b) {
    if (V == 8) {
      const uint2 t = *reinterpret_cast<const uint2*>(a);
      b[0] = t.x;
      b[1] = t.y;
    } else if (V == 4) {
      b[0] = *reinterpret_cast<const uint32_t*>(a);
    } else if (V == 2) {
      b[0] = *reinterpret_cast<const uint16_t*>(a);
    } else {
      b[0] = *a;
    }
  }
  static __device__ __forceinline__ uint32_t byte_of(const uint32_t* b, int k) {
    return (b[k >> 2] >> (8 * (k & 3))) & 0xffu;
  }

  // The segment's words, the other colour's words around them and the eta masks of its cells
  // (s_eta: cube state x vertex offset -> mask).
  __device__ __forceinline__ void load(const ReplicaDesc& R, int colour, int hc, int y_, int z_,
                                       const uint8_t* s_eta) {
    const int L = R.L, H = R.H;
    y = y_;
    z = z_;
    s = (y + z + colour) & 1;
    const int h0 = hc * V;
    x0 = 2 * h0 + s;
    const uint32_t* oth = R.cells[colour ^ 1];
    const int yp1 = y + 1 == L ? 0 : y + 1, ym1 = y == 0 ? L - 1 : y - 1;
    const int zp1 = z + 1 == L ? 0 : z + 1, zm1 = z == 0 ? L - 1 : z - 1;
    const uint32_t row = (uint32_t)H * ((uint32_t)y + (uint32_t)L * z);
    own_ptr = R.cells[colour] + row + h0;
    VecLoad<V>::ld(own_ptr, own);
    uint32_t mid[V];
    VecLoad<V>::ld(oth + row + h0, mid);
    VecLoad<V>::ld(oth + (uint32_t)H * ((uint32_t)yp1 + (uint32_t)L * z) + h0, yp);
    VecLoad<V>::ld(oth + (uint32_t)H * ((uint32_t)ym1 + (uint32_t)L * z) + h0, ym);
    VecLoad<V>::ld(oth + (uint32_t)H * ((uint32_t)y + (uint32_t)L * zp1) + h0, zp);
    VecLoad<V>::ld(oth + (uint32_t)H * ((uint32_t)y + (uint32_t)L * zm1) + h0, zm);
    // x neighbours: s == 0 -> x+ at h, x- at h-1; s == 1 -> x+ at h+1, x- at h
    const uint32_t extra = oth[row + (s == 0 ? (h0 == 0 ? H - 1 : h0 - 1) : (h0 + V == H ? 0 : h0 + V))];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      if (s == 0) {
        xp[k] = mid[k];
        xm[k] = k > 0 ? mid[k - 1] : extra;
      } else {
        xm[k] = mid[k];
        xp[k] = k + 1 < V ? mid[k + 1] : extra;
      }
    }
    // eta from the even cube (x>>1, y>>1, z>>1) and the odd cube containing the cell: cell k
    // lies in even cube h0 + k and odd cube h0 + k (s = 1) or h0 + k - 1 (s = 0)
    const int yo = (y & 1) ? y : ym1, zo = (z & 1) ? z : zm1;
    const uint32_t erow = (uint32_t)H * ((uint32_t)(y >> 1) + (uint32_t)H * (z >> 1));
    const uint32_t orow = (uint32_t)H * ((uint32_t)(yo >> 1) + (uint32_t)H * (zo >> 1));
    const int p = s | ((y & 1) << 1) | ((z & 1) << 2);
    // the states of the V even cubes over the segment and of the V odd cubes from its start (one
    // V-byte load each: rows and segments start at multiples of V), and the odd cube before it
    uint32_t ce[(V + 3) / 4], co[(V + 3) / 4];
    ld_bytes(R.cubes[0] + erow + h0, ce);
    ld_bytes(R.cubes[1] + orow + h0, co);
    const uint32_t co_prev = R.cubes[1][orow + (h0 == 0 ? H - 1 : h0 - 1)];
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const uint32_t se = byte_of(ce, k);
      const uint32_t so = s ? byte_of(co, k) : (k == 0 ? co_prev : byte_of(co, k - 1));
      eta[k] = (uint32_t)s_eta[se * 8 + p] | (uint32_t)s_eta[so * 8 + (p ^ 7)];
    }
  }
};

__device__ __forceinline__ uint32_t neighbour_sigmas(uint32_t xp, uint32_t xm, uint32_t yp, uint32_t ym,
                                                     uint32_t zp, uint32_t zm) {
  // arm a faces sigma_{a^1} of the neighbour along a (GW:1936-1962)
  // the three "+" neighbours give a field one place up of where it goes, the three "-" ones a
  // field one place down: two masked selections and two shifts
  const uint32_t up = (xp & 0x38u) | (yp & 0xe00u) | (zp & 0x38000u);
  const uint32_t dn = (xm & 0x7u) | (ym & 0x1c0u) | (zm & 0x7000u);
  return (up >> 3) | (dn << 3);
}

__device__ __forceinline__ uint32_t sigma_histogram(uint32_t w) {
  uint32_t h = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a) h += 1u << (4 * ((w >> (3 * a)) & 7u));
  return h;
}

// Proposal word after the exact uniform draw rejected word 0 of the sweep block (p = 6e-7).
__device__ __noinline__ uint32_t sweep_proposal_retry(uint32_t c0, uint32_t t, uint32_t rep, uint32_t k0,
                                                      uint32_t k1) {
  uint32_t w = 0;
  for (uint32_t k = 0; k < 256; ++k) {
    w = philox(c0, t, retry_tag(kStSweep, k), rep, k0, k1).x;
    if (w * 46656u >= 2560u) return w;
  }
  return w;
}

// Exact update of one cell with the full 32-bit uniforms (high halves from the sweep block,
// low halves from the refinement block). Taken only when a 16-bit comparison tied. Returns the
// new word.
__device__ __noinline__ uint32_t sweep_cell_exact(uint32_t w, uint32_t nbe, uint32_t u, uint32_t a1, uint32_t a2,
                                                  uint32_t a3, uint32_t c0, uint32_t t, const ReplicaDesc* R) {
  const U4 rf = philox(c0, t, kStSweepRefine, R->replica, R->key0, R->key1);
  uint32_t h = sigma_histogram(w);
  uint32_t f = u;
  for (int a = 0; a < 6; ++a) {
    unsigned long long m = (unsigned long long)f * 6ull;
    const uint32_t n = (uint32_t)(m >> 32);
    f = (uint32_t)m;
    const uint32_t o = (w >> (3 * a)) & 7u;
    if (n == o) continue;
    const uint32_t nb = (nbe >> (3 * a)) & 7u;  // 7 where eta_a = 0: never equal to a sigma
    const int dhb = (int)(n == nb) - (int)(o == nb);
    const int dns = (int)((h >> (4 * n)) & 15u) - (int)((h >> (4 * o)) & 15u) + 1;
    const unsigned long long T = R->thr_sweep[(dhb + 1) * 11 + dns + 5];
    const uint32_t hw = a < 2 ? a1 : (a < 4 ? a2 : a3);
    const uint32_t lw = a < 2 ? rf.x : (a < 4 ? rf.y : rf.z);
    const uint32_t sh = 16 * (a & 1);
    const unsigned long long U = ((unsigned long long)((hw >> sh) & 0xffffu) << 16) | ((lw >> sh) & 0xffffu);
    if (U < T) {
      w = (w & ~(7u << (3 * a))) | (n << (3 * a));
      h += (1u << (4 * n)) - (1u << (4 * o));
    }
  }
  return w;
}

// Byte select: byte i of the result is byte ((sel >> 4i) & 7) of the eight bytes {hi:lo}. Every
// selector nibble used here is below 8 (no sign replication).
__device__ __forceinline__ uint32_t prmt(uint32_t lo, uint32_t hi, uint32_t sel) {
  uint32_t r;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(sel));
  return r;
}

// Warp-private shared-memory tables (no block barrier: each warp fills and reads its own copy).
// The measurement needs the eta tables only; the sweep adds its decision tables.
//   nbmask  per 6-bit eta mask, the value 7 in the 3-bit field of every arm with eta = 0
//   eta     cube state x vertex offset -> 6-bit eta mask
struct EtaTables {
  uint32_t nbmask[64];
  uint8_t eta[72];
};
// Histograms are eight bytes {hi:lo} holding 4x the count of each sigma value 0..5 (bytes 6, 7
// zero). The sweep tables index with at most 8 distinct entries of 8 bytes or a 33-word array, so
// a warp's random lookups never conflict in a shared-memory bank, except dcnt and cnt2 (36 live
// entries each).
//   cnt[v]   4 at byte v (v = 0..5), zero for v = 6, 7: one arm of value v
//   nbw[v]   44 at byte v (v = 0..5), zero for v = 6, 7 (7 marks an arm with eta = 0)
//   dcnt[i]  cnt[i >> 3] - cnt[i & 7] per 32-bit word (wrapping): the histogram change of an arm
//            going from value i & 7 to value i >> 3, one lookup and two adds where cnt takes two
//            lookups and four adds (the 8-cell sweep: L=256 step 205.8 -> 202.2 us; the kernels
//            at the 64-register bound spill with it and keep cnt)
//   cnt2[i]  cnt[i >> 3] + cnt[i & 7]: the histogram of two adjacent arms (6-bit field of the
//            word), three lookups for the cell's starting histogram instead of six (278 thread
//            instructions per cell of the 8-cell sweep instead of 284; colour launch at L=256
//            85.1 -> 84.0 us)
//   tv[i]    2*(T_i >> 16) + ((T_i & 0xffff) != 0) - 1 for the threshold T_i of entry
//            i = 11*dN_hb + (h_new - h_old) + 17
struct SweepTables {
  uint2 cnt[8];
  uint2 nbw[8];
  uint2 dcnt[64];
  uint2 cnt2[64];
  uint32_t tv[33];
  EtaTables et;
};

__device__ __forceinline__ uint2 count_bytes(uint32_t v, uint32_t b) {
  return v < 4 ? make_uint2(b << (8 * v), 0u) : (v < 6 ? make_uint2(0u, b << (8 * (v - 4))) : make_uint2(0u, 0u));
}

__device__ __forceinline__ void fill_eta_tables(const ReplicaDesc& R, EtaTables* et, int lane) {
  et->nbmask[lane] = R.nbmask[lane];
  et->nbmask[32 + lane] = R.nbmask[32 + lane];
  if (lane < 18) reinterpret_cast<uint32_t*>(et->eta)[lane] = reinterpret_cast<const uint32_t*>(R.eta_tab)[lane];
}

__device__ __forceinline__ const EtaTables* warp_eta_tables(const ReplicaDesc& R, EtaTables* all) {
  EtaTables* et = all + (threadIdx.x >> 5);
  fill_eta_tables(R, et, threadIdx.x & 31);
  __syncwarp();
  return et;
}

__device__ __forceinline__ void fill_sweep_tables(const ReplicaDesc& R, SweepTables* wt, uint32_t lane) {
  fill_eta_tables(R, &wt->et, lane);
  wt->tv[lane] = R.tv[lane];
  if (lane == 0) wt->tv[32] = R.tv[32];
  if (lane < 8) {
    wt->cnt[lane] = count_bytes(lane, 4u);
    wt->nbw[lane] = count_bytes(lane, 44u);
  }
  for (uint32_t i = lane; i < 64; i += 32) {
    const uint2 n = count_bytes(i >> 3, 4u), o = count_bytes(i & 7u, 4u);
    wt->dcnt[i] = make_uint2(n.x - o.x, n.y - o.y);
    wt->cnt2[i] = make_uint2(n.x + o.x, n.y + o.y);
  }
}

__device__ __forceinline__ const SweepTables* warp_sweep_tables(const ReplicaDesc& R, SweepTables* all) {
  SweepTables* wt = all + (threadIdx.x >> 5);
  fill_sweep_tables(R, wt, threadIdx.x & 31);
  __syncwarp();
  return wt;
}

// One block-wide copy of the sweep tables of replica R (every block of the plain sweep kernels
// serves one replica), filled by the first threads of the block; the caller synchronises the
// block after it. A copy at a fixed shared-memory address lets the table reads of the decision
// loop use constant offsets.
__device__ __forceinline__ void fill_block_sweep_tables(const ReplicaDesc& R, SweepTables* t) {
  const int i = threadIdx.x;
  if (i < 64) t->et.nbmask[i] = R.nbmask[i];
  if (i < 18) reinterpret_cast<uint32_t*>(t->et.eta)[i] = reinterpret_cast<const uint32_t*>(R.eta_tab)[i];
  if (i < 33) t->tv[i] = R.tv[i];
  if (i < 8) {
    t->cnt[i] = count_bytes((uint32_t)i, 4u);
    t->nbw[i] = count_bytes((uint32_t)i, 44u);
  }
  if (i < 64) {
    const uint2 n = count_bytes((uint32_t)i >> 3, 4u), o = count_bytes((uint32_t)i & 7u, 4u);
    t->dcnt[i] = make_uint2(n.x - o.x, n.y - o.y);
    t->cnt2[i] = make_uint2(n.x + o.x, n.y + o.y);
  }
}

// Metropolis update of the six arms of one cell, arms in order 0..5 (GW:1964-2007 energy change,
// chessboard branch). Proposal of arm a: the a-th most significant base-6 digit of the uniform
// word u (the high word of u*6 in a multiply chain). The threshold entry is
// i = 11*dN_hb + (h_new - h_old) + 17, with h the count of the cell's arms per sigma value and
// dN_hb = [new == nb] - [old == nb] for the facing neighbour value nb (7 where eta_a = 0). Both
// terms come from byte selects on G = 4h + 44*[v == nb]: the selector v + 0x7770 picks byte v
// with zeros above it, so G[new] - G[old] + 68 is the byte offset 4i into tv. The proposal's
// selector is the high word of u*6 + (0x7770 << 32).
// With d = tv - 2*hu for the 16-bit high half hu of the acceptance uniform, accept is d >= 1; a
// tie d == 0 needs the low half. A tie makes the product of d over the six arms zero; a product
// that wraps to zero without a tie only sends the cell through the exact path as well, which
// decides every arm from the full 32-bit uniforms. A proposal equal to the old
// value lands on entry 17 (dN = 0), which always accepts and changes nothing.
// An accepted arm adds (new - old) << 3a to the word (the difference of the two selectors) and
// its histogram change to h, except after the last arm, whose histogram nothing reads.
template <bool kFold, bool kDelta>
__device__ __forceinline__ uint32_t update_cell(uint32_t w, uint32_t nbe, const U4& rr,
                                                uint32_t c0, uint32_t t, const ReplicaDesc& R, const SweepTables* wt) {
  // a proposal word in the rejected range of the exact draw (p = 6e-7): with kFold it sends the
  // cell through the exact path, which draws the retry word, and the fast path's decisions are
  // discarded (one rare-path test per cell instead of two); otherwise the retry word is drawn
  // first (the measuring and persistent kernels keep within their registers so)
  uint32_t u = rr.x;
  bool reject = u * 46656u < 2560u;
  if (!kFold && reject) {
    u = sweep_proposal_retry(c0, t, R.replica, R.key0, R.key1);
    reject = false;
  }
  const uint32_t w0 = w;
  uint32_t hx = 0, hy = 0;
#pragma unroll
  for (int a = 0; a < 6; a += 2) {
    const uint2 c = wt->cnt2[(w0 >> (3 * a)) & 63u];
    hx += c.x;
    hy += c.y;
  }
  const char* tvb = reinterpret_cast<const char*>(wt->tv) + 68;
  uint32_t f = u, tprod = 1u;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const unsigned long long m = (unsigned long long)f * 6ull + (0x7770ull << 32);
    const uint32_t sn = (uint32_t)(m >> 32);
    f = (uint32_t)m;
    const uint32_t osel = ((w0 >> (3 * a)) & 7u) | 0x7770u;  // the old value's selector
    const uint2 e = wt->nbw[(nbe >> (3 * a)) & 7u];
    const uint32_t gx = hx + e.x, gy = hy + e.y;
    const int off = (int)(prmt(gx, gy, sn) - prmt(gx, gy, osel));
    const uint32_t tv = *reinterpret_cast<const uint32_t*>(tvb + off);
    const uint32_t word = a < 2 ? rr.y : (a < 4 ? rr.z : rr.w);
    const uint32_t hu = (a & 1) ? (word >> 16) : (word & 0xffffu);
    const int d = (int)(tv - 2u * hu);
    tprod *= (uint32_t)d;
    const uint32_t dv = sn - osel;  // new - old: the word changes by dv << 3a (one predicated multiply-add)
    if (a == 5) {
      // the histogram is not read after the last arm
      asm("{\n\t.reg .pred p;\n\tsetp.ge.s32 p, %1, 1;\n\t@p mad.lo.u32 %0, %2, %3, %0;\n\t}"
          : "+r"(w)
          : "r"(d), "r"(dv), "r"(1u << (3 * a)));
    } else if (kDelta) {
      // one lookup of the histogram change of the pair (new, old): entry 8 * new + old
      const uint2 dc = wt->dcnt[8u * sn + osel - 9u * 0x7770u];
      asm("{\n\t.reg .pred p;\n\tsetp.ge.s32 p, %3, 1;\n\t@p mad.lo.u32 %0, %4, %7, %0;\n\t@p add.u32 %1, %1, %5;"
          "\n\t@p add.u32 %2, %2, %6;\n\t}"
          : "+r"(w), "+r"(hx), "+r"(hy)
          : "r"(d), "r"(dv), "r"(dc.x), "r"(dc.y), "r"(1u << (3 * a)));
    } else {
      const uint2 cn = wt->cnt[sn - 0x7770u], co = wt->cnt[osel - 0x7770u];
      asm("{\n\t.reg .pred p;\n\tsetp.ge.s32 p, %3, 1;\n\t@p mad.lo.u32 %0, %4, %9, %0;\n\t@p add.u32 %1, %1, %5;"
          "\n\t@p sub.u32 %1, %1, %6;\n\t@p add.u32 %2, %2, %7;\n\t@p sub.u32 %2, %2, %8;\n\t}"
          : "+r"(w), "+r"(hx), "+r"(hy)
          : "r"(d), "r"(dv), "r"(cn.x), "r"(co.x), "r"(cn.y), "r"(co.y), "r"(1u << (3 * a)));
    }
  }
  if (tprod == 0u || reject) {
    const uint32_t ue = reject ? sweep_proposal_retry(c0, t, R.replica, R.key0, R.key1) : u;
    w = sweep_cell_exact(w0, nbe, ue, rr.y, rr.z, rr.w, c0, t, &R);
  }
  return w;
}

// One colour of the checkerboard sweep: every cell with (x+y+z)&1 == colour updates its six
// arms; its six neighbours have the other colour and stay frozen. Thread = V consecutive
// colour cells of one row, read and written with 128-bit accesses when V = 4.
// Resident blocks per SM the register allocation must allow: 4 (64 registers) for tiles up to 4
// cells, 3 (80 registers, no spills) for the 8-cell tile.
template <int V>
struct SweepMinBlocks {
  static constexpr int v = V >= 8 ? 3 : 4;
};
// Row segment q (V cells) of one colour of replica R with sweep counter t. With kMeasure (the
// colour-1 sweep of a recorded step) it also adds the segment's share of the measurement of
// GW:2014-2160 to hb2 and ns after the update: every bond has exactly one colour-1 end, so the
// colour-1 cells count all bonds (delta of the facing sigmas times the bond's eta, twice), and
// each colour-1 cell adds the sigma pairs of itself and of the colour-0 cell with the same word
// index (the x-neighbour the segment loads anyway).
template <int V, bool kMeasure, bool kFold = false, bool kDelta = false>
__device__ __forceinline__ void sweep_segment(const ReplicaDesc& R, const SweepTables* wt, uint32_t q, int colour,
                                              uint32_t t, uint32_t& hb2, uint32_t& ns) {
  int hc, y, z;
  if (!segment_of<V>(R, q, hc, y, z)) return;
  // nbe: the facing neighbour sigmas with 7 in the field of every arm whose eta is 0 -- all that
  // the decisions and the measurement need of the neighbours and of eta
  uint32_t out[V], nbe[V];
  uint32_t* own_ptr;
  int x0;
  {
    CellBlock<V> cb;
    cb.load(R, colour, hc, y, z, wt->et.eta);
#pragma unroll
    for (int k = 0; k < V; ++k) {
      nbe[k] = neighbour_sigmas(cb.xp[k], cb.xm[k], cb.yp[k], cb.ym[k], cb.zp[k], cb.zm[k]) |
               wt->et.nbmask[~cb.eta[k] & 63u];
      out[k] = cb.own[k];
      if (kMeasure) ns += sigma_pairs(cb.s == 0 ? cb.xp[k] : cb.xm[k]);
    }
    own_ptr = cb.own_ptr;
    x0 = cb.x0;
  }
  const uint32_t L = R.L;
  const uint32_t cbase = L * ((uint32_t)y + L * (uint32_t)z) + (uint32_t)x0;
  const PhiloxKeys rk = philox_keys(R.key0, R.key1);
#pragma unroll
  for (int k = 0; k < V; ++k) {
    const uint32_t c0 = cbase + 2u * k;
    const U4 rr = philox_rk(c0, t, kStSweep, R.replica, rk);
    out[k] = update_cell<kFold, kDelta>(out[k], nbe[k], rr, c0, t, R, wt);
  }
  VecLoad<V>::st(own_ptr, out);
  if (kMeasure) {
#pragma unroll
    for (int k = 0; k < V; ++k) {
      const uint32_t x = out[k] ^ nbe[k];  // a field of 7 (eta = 0) never matches
      const uint32_t eqm = ~(x | (x >> 1) | (x >> 2)) & 0x9249u;
      hb2 += 2u * (uint32_t)__popc(eqm);
      ns += sigma_pairs(out[k]);
    }
  }
}

template <int V>
__global__ void __launch_bounds__(kThreads, SweepMinBlocks<V>::v) k_sweep(const ReplicaDesc* __restrict__ reps,
                                                    ReplicaState* __restrict__ st,
                                                    const int* __restrict__ blk, int nrep, int colour, int jsweep,
                                                    int from_ctr) {
  pdl_trigger();
  __shared__ SweepTables s_tab;
  const int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  fill_block_sweep_tables(R, &s_tab);
  __syncthreads();
  pdl_wait();
  uint32_t hb2 = 0, ns = 0;
  sweep_segment<V, false, true, V == 8>(R, &s_tab, (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x, colour,
                                        (from_ctr ? st[r].ctr[0] : st[r].cur[0]) + (uint32_t)jsweep, hb2, ns);
}

// A chunk of Metropolis-only steps of a small replica on one thread-block cluster of kClusterCtas
// blocks (cluster c = replica c): each block takes every kClusterCtas-th cube block (one cube per
// thread with cube1 and the table of one thread per cube, else the replica's cube tile and its
// table) and row segment (V cells per thread) of the replica, and a cluster barrier (release / acquire, so the cells and cube states
// written before it are seen after it) separates the cube moves and the two colours of every
// sweep. The step counters are those the per-phase kernels get from k_step_begin: cube move
// ctr[1] + s, sweep j of step s ctr[0] + s * nmet + j; block 0 advances them after the last step.
// The volume moves run on a side branch (k_volume_chain). The same cells, draws and decisions as
// the per-phase kernels, with kClusterCtas blocks instead of one launch per phase: a step of
// an L=16 lattice is a few microseconds of work spread over launches of a few blocks.
constexpr int kClusterCtas = 8;

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int V>
__global__ void __launch_bounds__(kThreads) k_chunk_cluster(const ReplicaDesc* __restrict__ reps,
                                                            ReplicaState* __restrict__ st,
                                                            const int* __restrict__ blk_cube, int cube1,
                                                            int nrep, int steps, int nmet) {
  __shared__ SweepTables s_tab;
  __shared__ CubeTables s_ct[kThreads / 32];
  uint32_t rank;
  asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
  const int r = (int)(blockIdx.x / kClusterCtas);
  const bool live = r < nrep;  // every block of the cluster reaches every barrier
  const ReplicaDesc& R = reps[live ? r : 0];
  const SweepTables* wt = &s_tab;
  fill_block_sweep_tables(R, &s_tab);
  CubeTables* ct = s_ct + (threadIdx.x >> 5);
  fill_cube_tables(R, ct, threadIdx.x & 31);
  __syncthreads();
  ReplicaState& S = st[live ? r : 0];
  const uint32_t c0 = S.ctr[0], c1 = S.ctr[1];
  const uint32_t nseg = (uint32_t)(R.H / V) * (uint32_t)R.L * (uint32_t)R.L;
  const int vb0 = __ldg(blk_cube + (live ? r : 0)), vb1 = __ldg(blk_cube + (live ? r : 0) + 1);
  uint32_t hb2 = 0, ns = 0;
  cluster_barrier();  // every block has read the counters before block 0 moves them
  for (int s = 0; s < steps; ++s) {
    if (live)
      for (int vb = vb0 + (int)rank; vb < vb1; vb += kClusterCtas)
        if (cube1) cube_move_v<1>(R, ct, blk_cube, r, vb, c1 + (uint32_t)s);
        else cube_move(R, ct, blk_cube, r, vb, c1 + (uint32_t)s);
    cluster_barrier();
    for (int j = 0; j < nmet; ++j) {
      const uint32_t t = c0 + (uint32_t)(s * nmet + j);
      for (int colour = 0; colour < 2; ++colour) {
        if (live)
          for (uint32_t q = rank * kThreads + threadIdx.x; q < nseg; q += kClusterCtas * kThreads)
            sweep_segment<V, false, true>(R, wt, q, colour, t, hb2, ns);
        cluster_barrier();
      }
    }
  }
  if (live && rank == 0 && threadIdx.x == 0 && steps > 0) {
    // the counters as the last step's k_step_begin leaves them (the volume counter belongs to
    // the volume branch)
    S.cur[0] = c0 + (uint32_t)((steps - 1) * nmet);
    S.ctr[0] = c0 + (uint32_t)(steps * nmet);
    S.cur[1] = c1 + (uint32_t)(steps - 1);
    S.ctr[1] = c1 + (uint32_t)steps;
    S.cur[3] = S.ctr[3];
  }
}

// Colour-1 sweep of a recorded step fused with its measurement: the counts go to the slots
// that k_step_begin zeroed, k_measure_end sums them after the step.
template <int V>
__global__ void __launch_bounds__(kThreads, SweepMinBlocks<V>::v) k_sweep_measure(
    const ReplicaDesc* __restrict__ reps, ReplicaState* __restrict__ st, const int* __restrict__ blk, int nrep,
    int jsweep) {
  pdl_trigger();
  __shared__ SweepTables s_tab;
  __shared__ unsigned long long s_acc[2];
  const int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  fill_block_sweep_tables(R, &s_tab);
  __syncthreads();
  pdl_wait();
  uint32_t hb2 = 0, ns = 0;
  sweep_segment<V, true, true, V == 8>(R, &s_tab, (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x, 1,
                         st[r].cur[0] + (uint32_t)jsweep, hb2, ns);
  measure_accumulate(st[r], blockIdx.x, hb2, ns, s_acc);
}

// ------------------------------------------------------------------ measurement
// GW:2014-2160: N_hb2 = sum over bonds of delta * (eta_i + eta_j), counted from the colour-0
// end of every bond (each bond joins the two colours); N_sigma over cells of both colours.
// Counts of the V-cell colour-0 segment q of replica R, added to hb2 and ns.
template <int V>
__device__ __forceinline__ void measure_segment(const ReplicaDesc& R, const EtaTables* et, uint32_t q, uint32_t& hb2,
                                                uint32_t& ns) {
  int hc, y, z;
  if (!segment_of<V>(R, q, hc, y, z)) return;
  const int L = R.L, H = R.H;
  CellBlock<V> cb;
  cb.load(R, 0, hc, y, z, et->eta);
  uint32_t w1[V];
  VecLoad<V>::ld(R.cells[1] + (uint32_t)H * ((uint32_t)y + (uint32_t)L * z) + hc * V, w1);
#pragma unroll
  for (int k = 0; k < V; ++k) {
    const uint32_t w = cb.own[k];
    const uint32_t nbs = neighbour_sigmas(cb.xp[k], cb.xm[k], cb.yp[k], cb.ym[k], cb.zp[k], cb.zm[k]);
    // bonds whose two arm sigmas agree, restricted to eta = 1 (bit 3a per arm)
    const uint32_t x = w ^ nbs;
    const uint32_t eqm = ~(x | (x >> 1) | (x >> 2)) & et->nbmask[cb.eta[k] & 63u] & 0x9249u;
    hb2 += 2u * (uint32_t)__popc(eqm);
    ns += sigma_pairs(w) + sigma_pairs(w1[k]);
  }
}

template <int V>
__global__ void __launch_bounds__(kThreads) k_measure(const ReplicaDesc* __restrict__ reps,
                                                      ReplicaState* __restrict__ st,
                                                      const int* __restrict__ blk, int nrep) {
  __shared__ unsigned long long s_acc[2];
  __shared__ EtaTables s_tab[kThreads / 32];
  const int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const EtaTables* et = warp_eta_tables(R, s_tab);
  uint32_t hb2 = 0, ns = 0;
  measure_segment<V>(R, et, (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x, hb2, ns);
  measure_accumulate(st[r], blockIdx.x, hb2, ns, s_acc);
}

__global__ void k_measure_begin(ReplicaState* __restrict__ st, int nrep) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrep) measure_zero(st[r]);
}

// host_out (mapped page-locked host memory, one record per replica) also receives the records.
__global__ void k_measure_end(ReplicaState* __restrict__ st, int nrep, int record, SampleRec* host_out) {
  pdl_trigger();
  pdl_wait();
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrep) {
    measure_finish(st[r], record);
    if (host_out) {
      host_out[r] = st[r].last;
      __threadfence_system();
    }
  }
}

// ------------------------------------------------------------------ persistent step kernel
// The persistent kernel separates its phases with grid_barrier (every block of the cooperative
// launch is resident; a wait gives up after b.barrier_polls looks, error code 3 of replica 0).
//
// Per-warp tables of the persistent kernel: the sweep and cube tables of one replica, reloaded
// when the warp moves to a block of another replica.
struct StepTables {
  SweepTables sw;
  CubeTables cube;
};

__device__ __forceinline__ void ensure_tables(const ReplicaDesc* reps, int r, StepTables* wt, int& held) {
  if (held == r) return;
  __syncwarp();
  const uint32_t lane = threadIdx.x & 31;
  fill_sweep_tables(reps[r], &wt->sw, lane);
  fill_cube_tables(reps[r], &wt->cube, lane);
  __syncwarp();
  if (lane == 0) held = r;
  __syncwarp();
}

// Dynamic dealing of a phase's n blocks: tickets come from one counter that grows through the
// launch; every block takes tickets until one lies past the phase's range, so the counter ends
// each phase at base + n + gridDim.x and the next phase's base is known to every block.
struct Dealer {
  unsigned int base;
  int slot;
};

template <typename F>
__device__ __forceinline__ void deal(GridSync* gs, Dealer& d, int n, int* s_vb, F&& work) {
  if (threadIdx.x == 0) s_vb[d.slot] = (int)(atomicAdd(&gs->ticket, 1u) - d.base);
  __syncthreads();
  for (;;) {
    const int vb = s_vb[d.slot];
    if (vb >= n) break;
    if (threadIdx.x == 0) s_vb[d.slot ^ 1] = (int)(atomicAdd(&gs->ticket, 1u) - d.base);
    work(vb);
    __syncthreads();
    d.slot ^= 1;
  }
  d.base += (unsigned int)n + gridDim.x;
}

// nsteps Metropolis steps of every replica in one cooperative launch. Each phase (cube moves with
// one volume block per replica, then every sweep colour, then the measurement of a recorded
// step) deals the blocks of its per-phase table (blk_cubev, blk_sweep) to the resident blocks
// through tickets, and a grid barrier closes the phase. Step s uses the counters the per-phase
// kernels get from k_step_begin: sweep ctr[0] + s*nmet + j, cube ctr[1] + s, volume
// ctr[2] + s; the counters advance once, after the last step. With interval > 0 a measurement
// follows every step s with s % interval == 0; its slots are zeroed by the volume warp at the
// start of the step and summed into the sample stream by the same warp at the start of the
// next step (before that step's volume move), or after the last barrier.
template <int V>
__global__ void __launch_bounds__(kThreads, SweepMinBlocks<V>::v) k_run(BatchDev b, int nsteps, int nmet,
                                                                         int interval) {
  __shared__ StepTables s_tab[kThreads / 32];
  __shared__ unsigned long long s_acc[2];
  __shared__ int s_held[kThreads / 32];
  __shared__ int s_vb[2];
  if ((threadIdx.x & 31) == 0) s_held[threadIdx.x >> 5] = -1;
  __syncwarp();
  Dealer d{0u, 0};
  const int pps = 2 + 2 * nmet;  // phases per step: cube/volume, 2 per sweep, measurement
  for (int ph = 0; ph < nsteps * pps; ++ph) {
    const int s = ph / pps, k = ph - s * pps;
    if (k == 0) {
      const bool rec = interval > 0 && s % interval == 0;
      const bool prev_rec = interval > 0 && s > 0 && (s - 1) % interval == 0;
      deal(b.gsync, d, b.nblk_cubev + b.nrep, s_vb, [&](int vb) {
        if (vb < b.nblk_cubev) {
          const int r = find_replica(b.blk_cubev, b.nrep, vb);
          StepTables* wt = s_tab + (threadIdx.x >> 5);
          ensure_tables(b.reps, r, wt, s_held[threadIdx.x >> 5]);
          cube_move(b.reps[r], &wt->cube, b.blk_cubev, r, vb, b.st[r].ctr[1] + (uint32_t)s);
        } else if (threadIdx.x < 32) {
          const int r = vb - b.nblk_cubev;
          ReplicaState& S = b.st[r];
          if (threadIdx.x == 0) {
            if (prev_rec) measure_finish(S, 1);
            if (rec) measure_zero(S);
          }
          __syncwarp();
          volume_move_warp(b.reps[r], S, S.ctr[2] + (uint32_t)s);
        }
      });
    } else if (k < pps - 1) {
      const int colour = (k - 1) & 1;
      const uint32_t toff = (uint32_t)(s * nmet + ((k - 1) >> 1));
      deal(b.gsync, d, b.nblk_sweep, s_vb, [&](int vb) {
        const int r = find_replica(b.blk_sweep, b.nrep, vb);
        StepTables* wt = s_tab + (threadIdx.x >> 5);
        ensure_tables(b.reps, r, wt, s_held[threadIdx.x >> 5]);
        uint32_t hb2 = 0, ns = 0;
        sweep_segment<V, false>(b.reps[r], &wt->sw, (uint32_t)(vb - b.blk_sweep[r]) * blockDim.x + threadIdx.x,
                                colour, b.st[r].ctr[0] + toff, hb2, ns);
      });
    } else {
      if (!(interval > 0 && s % interval == 0)) continue;  // no measurement after this step
      deal(b.gsync, d, b.nblk_sweep, s_vb, [&](int vb) {
        const int r = find_replica(b.blk_sweep, b.nrep, vb);
        StepTables* wt = s_tab + (threadIdx.x >> 5);
        ensure_tables(b.reps, r, wt, s_held[threadIdx.x >> 5]);
        uint32_t hb2 = 0, ns = 0;
        measure_segment<V>(b.reps[r], &wt->sw.et, (uint32_t)(vb - b.blk_sweep[r]) * blockDim.x + threadIdx.x, hb2,
                           ns);
        measure_accumulate(b.st[r], vb, hb2, ns, s_acc);
      });
    }
    if (!grid_barrier(b.gsync, b.st, b.barrier_polls)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) b.gsync->ticket = 0u;  // every ticket of the launch is taken
  const bool last_rec = interval > 0 && (nsteps - 1) % interval == 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < b.nrep; r += gridDim.x * blockDim.x) {
    ReplicaState& S = b.st[r];
    if (last_rec) measure_finish(S, 1);
    S.cur[0] = S.ctr[0] + (uint32_t)((nsteps - 1) * nmet);
    S.ctr[0] += (uint32_t)(nsteps * nmet);
    S.cur[1] = S.ctr[1] + (uint32_t)(nsteps - 1);
    S.ctr[1] += (uint32_t)nsteps;
    S.cur[2] = S.ctr[2] + (uint32_t)(nsteps - 1);
    S.ctr[2] += (uint32_t)nsteps;
    S.cur[3] = S.ctr[3];
  }
}

// ------------------------------------------------------------------ launchers
static inline dim3 grid1(int n) { return dim3((unsigned)((n + kThreads - 1) / kThreads)); }

void launch_init_lattice(const BatchDev& b, cudaStream_t s) {
  k_init_sigma<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.blk_cell, b.nrep);
  k_init_cubes<<<b.nblk_cube, kThreads, 0, s>>>(b.reps, b.blk_cube, b.nrep);
}

cudaError_t launch_chunk_cluster(const BatchDev& b, int steps, int nmet, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(b.nrep * kClusterCtas));
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // the phases are short and latency-bound: the fewest cells (cubes) per thread that still cover
  // the largest replica in one pass of the cluster's threads
  const long long pass = (long long)kClusterCtas * kThreads, L = b.max_L, H = L / 2;
  int v = 1;
  while (v < b.vec && (H / v) * L * L > pass) v *= 2;
  const int cube1 = 2 * ((H * H * H + kThreads - 1) / kThreads) <= kClusterCtas;
  const int* blk = cube1 ? b.blk_cube : b.blk_cubev;
  switch (v) {
    case 8: return cudaLaunchKernelEx(&cfg, k_chunk_cluster<8>, (const ReplicaDesc*)b.reps, b.st, blk, cube1, b.nrep, steps, nmet);
    case 4: return cudaLaunchKernelEx(&cfg, k_chunk_cluster<4>, (const ReplicaDesc*)b.reps, b.st, blk, cube1, b.nrep, steps, nmet);
    case 2: return cudaLaunchKernelEx(&cfg, k_chunk_cluster<2>, (const ReplicaDesc*)b.reps, b.st, blk, cube1, b.nrep, steps, nmet);
    default: return cudaLaunchKernelEx(&cfg, k_chunk_cluster<1>, (const ReplicaDesc*)b.reps, b.st, blk, cube1, b.nrep, steps, nmet);
  }
}

void launch_volume_chain(const BatchDev& b, int steps, cudaStream_t s) {
  k_volume_chain<<<b.nrep, 32, 0, s>>>(b.reps, b.st, b.nrep, steps);
}

void launch_step_begin(const BatchDev& b, int nmet, int ncl, int do_cube, int do_volume, cudaStream_t s,
                       int zero_slots) {
  launch_pdl(k_step_begin, grid1(b.nrep), s, b.pdl, b.st, b.nrep, nmet, ncl, do_cube, do_volume, zero_slots);
}

void launch_sweep_measure(const BatchDev& b, int jsweep, cudaStream_t s) {
  const dim3 g((unsigned)b.nblk_sweep);
  switch (b.vec) {
    case 8: launch_pdl(k_sweep_measure<8>, g, s, b.pdl, b.reps, b.st, b.blk_sweep, b.nrep, jsweep); break;
    case 4: launch_pdl(k_sweep_measure<4>, g, s, b.pdl, b.reps, b.st, b.blk_sweep, b.nrep, jsweep); break;
    case 2: launch_pdl(k_sweep_measure<2>, g, s, b.pdl, b.reps, b.st, b.blk_sweep, b.nrep, jsweep); break;
    default: launch_pdl(k_sweep_measure<1>, g, s, b.pdl, b.reps, b.st, b.blk_sweep, b.nrep, jsweep); break;
  }
}

void launch_measure_end(const BatchDev& b, int record, cudaStream_t s, SampleRec* host_out) {
  launch_pdl(k_measure_end, grid1(b.nrep), s, b.pdl, b.st, b.nrep, record, host_out);
}

void launch_cube_volume(const BatchDev& b, int do_cubes, int do_volume, cudaStream_t s, int soff) {
  const int cube_blocks = do_cubes ? b.nblk_cubev : 0;
  const int vol_blocks = do_volume ? b.nrep : 0;
  if (cube_blocks + vol_blocks == 0) return;
  const dim3 grid((unsigned)(cube_blocks + vol_blocks));
  launch_pdl(k_cube_volume, grid, s, b.pdl, b.reps, b.st, b.blk_cubev, b.nrep, vol_blocks, soff);
}

void launch_chunk_end(const BatchDev& b, int steps, int nmet, int ncl, int do_volume, cudaStream_t s) {
  launch_pdl(k_chunk_end, dim3((unsigned)((b.nrep + kThreads - 1) / kThreads)), s, b.pdl, b.st, b.nrep, steps, nmet,
             ncl, do_volume);
}

void launch_sweep(const BatchDev& b, int colour, int jsweep, cudaStream_t s, int from_ctr) {
  const dim3 g((unsigned)b.nblk_sweep);
  const int* blk = b.blk_sweep;
  switch (b.vec) {
    case 8: launch_pdl(k_sweep<8>, g, s, b.pdl, b.reps, b.st, blk, b.nrep, colour, jsweep, from_ctr); break;
    case 4: launch_pdl(k_sweep<4>, g, s, b.pdl, b.reps, b.st, blk, b.nrep, colour, jsweep, from_ctr); break;
    case 2: launch_pdl(k_sweep<2>, g, s, b.pdl, b.reps, b.st, blk, b.nrep, colour, jsweep, from_ctr); break;
    default: launch_pdl(k_sweep<1>, g, s, b.pdl, b.reps, b.st, blk, b.nrep, colour, jsweep, from_ctr); break;
  }
}

// Replica host_r's last measurement, with its current r_cell and volume (a state set since the
// measurement changed them, not the cells), written to host_out: page-locked host memory mapped
// for the device.
__global__ void k_last_read(const ReplicaState* __restrict__ st, SampleRec* host_out, int host_r) {
  pdl_trigger();
  pdl_wait();
  if (threadIdx.x != 0) return;
  const ReplicaState& S = st[host_r];
  SampleRec rec = S.last;
  rec.r_cell = S.r_cell;
  rec.volume = S.volume;
  *host_out = rec;
  __threadfence_system();
}

void launch_last_read(const BatchDev& b, cudaStream_t s, SampleRec* host_out, int host_r) {
  launch_pdl(k_last_read, dim3(1u), s, b.pdl, b.st, host_out, host_r);
}

void launch_measure(const BatchDev& b, int record, cudaStream_t s) {
  k_measure_begin<<<grid1(b.nrep), kThreads, 0, s>>>(b.st, b.nrep);
  switch (b.vec) {
    case 8: k_measure<8><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
    case 4: k_measure<4><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
    case 2: k_measure<2><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
    default: k_measure<1><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
  }
  k_measure_end<<<grid1(b.nrep), kThreads, 0, s>>>(b.st, b.nrep, record, nullptr);
}

template <int V>
static cudaError_t launch_run_v(const BatchDev& b, int nsteps, int nmet, int interval, cudaStream_t s) {
  int dev = 0, nsm = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_run<V>, kThreads, 0);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  const int work = b.nblk_sweep > b.nblk_cubev + b.nrep ? b.nblk_sweep : b.nblk_cubev + b.nrep;
  const int grid = nsm * per < work ? nsm * per : work;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_run<V>, b, nsteps, nmet, interval);
}

cudaError_t launch_run(const BatchDev& b, int nsteps, int nmet, int interval, cudaStream_t s) {
  if (nsteps <= 0) return cudaSuccess;
  switch (b.vec) {
    case 8: return launch_run_v<8>(b, nsteps, nmet, interval, s);
    case 4: return launch_run_v<4>(b, nsteps, nmet, interval, s);
    case 2: return launch_run_v<2>(b, nsteps, nmet, interval, s);
    default: return launch_run_v<1>(b, nsteps, nmet, interval, s);
  }
}

}  // namespace cvf
