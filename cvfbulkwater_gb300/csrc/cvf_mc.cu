// Monte Carlo kernels of the GB300 CVF engine: lattice initialisation, the NPT volume move,
// the eta cube ("chessboard") move, the checkerboard sigma sweep and the exact int64
// observable reductions. Reference: SOURCE/gpu_water3D.cu ("GW") of lcoronas/CVFBulkWater.
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

__constant__ uint32_t c_state_active[9];
__constant__ uint8_t c_eta_table[72];  // [state*8 + vertex offset] -> 6-bit eta mask
__constant__ int c_edge_dir[12];
__constant__ int c_edge_start[12];

void init_sw_device_tables();
static unsigned long long g_tables_ready = 0;  // bit d: tables copied to device d

// Copies the cube tables to the current device's constant memory (once per device).
void init_device_tables() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && ((g_tables_ready >> dev) & 1ull)) return;
  uint32_t act[9];
  uint8_t eta[72];
  int dir[12], st[12];
  for (int s = 0; s < 9; ++s) {
    act[s] = state_active(s);
    for (int p = 0; p < 8; ++p) eta[s * 8 + p] = (uint8_t)cube_eta_bits(s, p);
  }
  for (int e = 0; e < 12; ++e) {
    dir[e] = edge_dir(e);
    st[e] = edge_start(e);
  }
  cudaMemcpyToSymbol(c_state_active, act, sizeof(act));
  cudaMemcpyToSymbol(c_eta_table, eta, sizeof(eta));
  cudaMemcpyToSymbol(c_edge_dir, dir, sizeof(dir));
  cudaMemcpyToSymbol(c_edge_start, st, sizeof(st));
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

__device__ __forceinline__ uint32_t cell_word_index(int x, int y, int z, int L, int H) {
  return (uint32_t)(x >> 1) + (uint32_t)H * ((uint32_t)y + (uint32_t)L * (uint32_t)z);
}

// ------------------------------------------------------------------ initialisation
// GW:812-825: disordered start draws each sigma uniformly, ordered start one common value.
__global__ void k_init_sigma(const ReplicaDesc* __restrict__ reps, const int* __restrict__ blk, int nrep) {
  int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int start = R.start;
  const int L = R.L, H = R.H;
  long long c = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  long long N = (long long)L * L * L;
  if (c >= N) return;
  int x = (int)(c % L), y = (int)((c / L) % L), z = (int)(c / ((long long)L * L));
  uint32_t w = 0;
  if (start == 2) {
    U4 q = philox(0, 0, kStInitOrder, R.replica, R.key0, R.key1);
    uint32_t v;
    if (!lemire_try(q.x, 6, v) && !lemire_try(q.y, 6, v) && !lemire_try(q.z, 6, v) && !lemire_try(q.w, 6, v))
      v = lemire_retry(6, 0, 0, kStInitOrder, R.replica, R.key0, R.key1);
    for (int a = 0; a < 6; ++a) w |= v << (3 * a);
  } else if (start == 0) {
    U4 q = philox((uint32_t)c, 0, kStInitSigma, R.replica, R.key0, R.key1);
    uint32_t d;
    if (!lemire_try(q.x, 46656u, d) && !lemire_try(q.y, 46656u, d) && !lemire_try(q.z, 46656u, d) &&
        !lemire_try(q.w, 46656u, d))
      d = lemire_retry(46656u, (uint32_t)c, 0, kStInitSigma, R.replica, R.key0, R.key1);
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
  long long q = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  long long H3 = (long long)H * H * H;
  if (q >= 2 * H3) return;
  int par = q >= H3;
  long long qi = q - par * H3;
  int a = (int)(qi % H), b = (int)((qi / H) % H), c = (int)(qi / ((long long)H * H));
  int x0 = 2 * a + par, y0 = 2 * b + par, z0 = 2 * c + par;
  uint32_t cid = (uint32_t)x0 + (uint32_t)L * ((uint32_t)y0 + (uint32_t)L * (uint32_t)z0);
  U4 w = philox(cid, 0, kStInitCube, R.replica, R.key0, R.key1);
  uint32_t st;
  if (!lemire_try(w.x, 9, st) && !lemire_try(w.y, 9, st) && !lemire_try(w.z, 9, st) && !lemire_try(w.w, 9, st))
    st = lemire_retry(9, cid, 0, kStInitCube, R.replica, R.key0, R.key1);
  R.cubes[par][qi] = (uint8_t)st;
}

// ------------------------------------------------------------------ step begin: volume move
// One thread per replica. Snapshots the move counters used by this step's kernels and performs
// the NPT volume move of GW:1740-1781 in FP64 with every operation rounded separately.
__global__ void k_step_begin(const ReplicaDesc* __restrict__ reps, ReplicaState* __restrict__ st, int nrep,
                             int nmet, int ncl, int do_cube) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  const ReplicaDesc& R = reps[r];
  ReplicaState& S = st[r];
  S.cur[0] = S.ctr[0];
  S.ctr[0] += (uint32_t)nmet;
  S.cur[1] = S.ctr[1];
  S.ctr[1] += (uint32_t)do_cube;
  S.cur[3] = S.ctr[3];
  S.ctr[3] += (uint32_t)ncl;
  uint32_t t = S.ctr[2]++;
  S.cur[2] = t;

  U4 q = philox(0, t, kStVolume, R.replica, R.key0, R.key1);
  double r0 = S.r_cell;
  double u1 = u53(q.x, q.y);
  double trial = CVF_DADD(r0, CVF_DMUL(0.01 * 2, CVF_DSUB(u1, 0.5)));
  for (uint32_t k = 1; trial < 0.0 && k < 64; ++k) {
    U4 qq = philox(k, t, kStVolume, R.replica, R.key0, R.key1);
    u1 = u53(qq.x, qq.y);
    trial = CVF_DADD(r0, CVF_DMUL(0.01 * 2, CVF_DSUB(u1, 0.5)));
  }
  const double Ld = (double)R.L;
  double tV = CVF_DMUL(CVF_DMUL(CVF_DMUL(CVF_DMUL(CVF_DMUL(trial, trial), trial), Ld), Ld), Ld);
  double dV = CVF_DSUB(tV, S.volume);
  double tE = evdw(trial, R.dist, R.freq, R.n_shells, R.Rc);
  float Nf = (float)((long long)R.L * R.L * R.L);
  double NT = (double)__fmul_rn(Nf, R.T);
  double dE = CVF_DSUB(CVF_DSUB(tE, S.e_vdw), CVF_DMUL(NT, own_log(tV / S.volume)));
  double u2 = u53(q.z, q.w);
  double arg = CVF_DMUL(-R.beta, CVF_DADD(dE, CVF_DMUL((double)R.P, dV)));
  if (u2 < own_exp(arg)) {
    S.r_cell = trial;
    S.volume = tV;
    S.e_vdw = tE;
  }
}

// ------------------------------------------------------------------ cube move
// GW:3374-3466. One thread per cube (both parities in one launch: cubes share no edge and
// sigma is frozen, so all cube decisions are independent). Writes only the cube's state byte.
__global__ void __launch_bounds__(kThreads) k_cube_move(const ReplicaDesc* __restrict__ reps,
                                                        const ReplicaState* __restrict__ st,
                                                        const int* __restrict__ blk, int nrep) {
  int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int L = R.L, H = R.H;
  long long q = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  long long H3 = (long long)H * H * H;
  if (q >= 2 * H3) return;
  int par = q >= H3;
  long long qi = q - par * H3;
  int a = (int)(qi % H), b = (int)((qi / H) % H), c = (int)(qi / ((long long)H * H));
  int x0 = 2 * a + par, y0 = 2 * b + par, z0 = 2 * c + par;
  int x1 = x0 + 1 == L ? 0 : x0 + 1, y1 = y0 + 1 == L ? 0 : y0 + 1, z1 = z0 + 1 == L ? 0 : z0 + 1;
  uint32_t w[8];
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    int x = (p & 1) ? x1 : x0, y = (p & 2) ? y1 : y0, z = (p & 4) ? z1 : z0;
    w[p] = __ldg(R.cells[(x + y + z) & 1] + cell_word_index(x, y, z, L, H));
  }
  uint32_t D = 0;  // edges whose two arm sigmas agree
#pragma unroll
  for (int e = 0; e < 12; ++e) {
    const int d = edge_dir(e), p0 = edge_start(e), p1 = p0 | (1 << d);
    uint32_t s0 = (w[p0] >> (6 * d)) & 7u, s1 = (w[p1] >> (6 * d + 3)) & 7u;
    D |= (uint32_t)(s0 == s1) << e;
  }
  uint32_t cid = (uint32_t)x0 + (uint32_t)L * ((uint32_t)y0 + (uint32_t)L * (uint32_t)z0);
  uint32_t t = st[r].cur[1];
  U4 rr = philox(cid, t, kStCube, R.replica, R.key0, R.key1);
  uint32_t nw;
  if (!lemire_try(rr.x, 9, nw) && !lemire_try(rr.z, 9, nw) && !lemire_try(rr.w, 9, nw))
    nw = lemire_retry(9, cid, t, kStCube, R.replica, R.key0, R.key1);
  uint8_t* cs = R.cubes[par] + qi;
  uint32_t old = *cs;
  int dhb = __popc(c_state_active[nw] & D) - __popc(c_state_active[old] & D);
  if ((unsigned long long)rr.y < R.thr_cube[dhb + 4] && nw != old) *cs = (uint8_t)nw;
}

// ------------------------------------------------------------------ checkerboard sweep
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

// Loads the V own words of a thread's row segment, the other colour's words around them and
// the eta masks of the V cells. Shared by the sweep and the measurement.
template <int V>
struct CellBlock {
  uint32_t own[V], xp[V], xm[V], yp[V], ym[V], zp[V], zm[V];
  uint32_t eta[V];
  uint32_t* own_ptr;
  int x0, y, z, s;

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
    const size_t row = (size_t)H * ((size_t)y + (size_t)L * z);
    own_ptr = R.cells[colour] + row + h0;
    VecLoad<V>::ld(own_ptr, own);
    uint32_t mid[V];
    VecLoad<V>::ld(oth + row + h0, mid);
    VecLoad<V>::ld(oth + (size_t)H * ((size_t)yp1 + (size_t)L * z) + h0, yp);
    VecLoad<V>::ld(oth + (size_t)H * ((size_t)ym1 + (size_t)L * z) + h0, ym);
    VecLoad<V>::ld(oth + (size_t)H * ((size_t)y + (size_t)L * zp1) + h0, zp);
    VecLoad<V>::ld(oth + (size_t)H * ((size_t)y + (size_t)L * zm1) + h0, zm);
    // x neighbours: s == 0 -> x+ at h, x- at h-1; s == 1 -> x+ at h+1, x- at h
    uint32_t extra;
    if (s == 0) extra = oth[row + (h0 == 0 ? H - 1 : h0 - 1)];
    else extra = oth[row + (h0 + V == H ? 0 : h0 + V)];
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
    // eta from the even cube (x>>1, y>>1, z>>1) and the odd cube containing the cell
    const int yo = (y & 1) ? y : ym1, zo = (z & 1) ? z : zm1;
    const size_t erow = (size_t)H * ((size_t)(y >> 1) + (size_t)H * (z >> 1));
    const size_t orow = (size_t)H * ((size_t)(yo >> 1) + (size_t)H * (zo >> 1));
    const int p = s | ((y & 1) << 1) | ((z & 1) << 2);
#pragma unroll
    for (int k = 0; k < V; ++k) {
      int ae = h0 + k;
      int ao = s ? ae : (ae == 0 ? H - 1 : ae - 1);
      uint32_t se = __ldg(R.cubes[0] + erow + ae);
      uint32_t so = __ldg(R.cubes[1] + orow + ao);
      eta[k] = (uint32_t)s_eta[se * 8 + p] | (uint32_t)s_eta[so * 8 + (p ^ 7)];
    }
  }
};

__device__ __forceinline__ uint32_t neighbour_sigmas(uint32_t xp, uint32_t xm, uint32_t yp, uint32_t ym,
                                                     uint32_t zp, uint32_t zm) {
  // arm a faces sigma_{a^1} of the neighbour along a (GW:1936-1962)
  return ((xp >> 3) & 7u) | ((xm & 7u) << 3) | (((yp >> 9) & 7u) << 6) | (((ym >> 6) & 7u) << 9) |
         (((zp >> 15) & 7u) << 12) | (((zm >> 12) & 7u) << 15);
}

__device__ __forceinline__ uint32_t sigma_histogram(uint32_t w) {
  uint32_t h = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a) h += 1u << (4 * ((w >> (3 * a)) & 7u));
  return h;
}

// Metropolis update of the six arms of one cell (GW:1964-2007 energy change, chessboard branch),
// arms in order 0..5, all decisions integer.
__device__ __forceinline__ uint32_t update_cell(uint32_t w, uint32_t nbs, uint32_t eta, uint32_t c0,
                                                uint32_t t, const ReplicaDesc& R, const uint32_t* s_thi,
                                                const uint16_t* s_tlo) {
  U4 rr = philox(c0, t, kStSweep, R.replica, R.key0, R.key1);
  uint32_t d;
  if (!lemire_try(rr.x, 46656u, d)) d = lemire_retry(46656u, c0, t, kStSweep, R.replica, R.key0, R.key1);
  uint32_t h = sigma_histogram(w);
  bool have_rf = false;
  U4 rf = {0, 0, 0, 0};
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    uint32_t n = d % 6u;
    d /= 6u;
    uint32_t o = (w >> (3 * a)) & 7u;
    if (n != o) {
      uint32_t nb = (nbs >> (3 * a)) & 7u;
      int dhb = ((eta >> a) & 1u) ? ((int)(n == nb) - (int)(o == nb)) : 0;
      int dns = (int)((h >> (4 * n)) & 15u) - (int)((h >> (4 * o)) & 15u) + 1;
      int idx = (dhb + 1) * 11 + dns + 5;
      uint32_t thi = s_thi[idx];
      uint32_t word = a < 2 ? rr.y : (a < 4 ? rr.z : rr.w);
      uint32_t hu = (word >> (16 * (a & 1))) & 0xffffu;
      bool acc = hu < thi;
      if (hu == thi) {
        uint32_t tlo = s_tlo[idx];
        if (tlo) {
          if (!have_rf) {
            rf = philox(c0, t, kStSweepRefine, R.replica, R.key0, R.key1);
            have_rf = true;
          }
          uint32_t rw = a < 2 ? rf.x : (a < 4 ? rf.y : rf.z);
          acc = ((rw >> (16 * (a & 1))) & 0xffffu) < tlo;
        }
      }
      if (acc) {
        w = (w & ~(7u << (3 * a))) | (n << (3 * a));
        h += (1u << (4 * n)) - (1u << (4 * o));
      }
    }
  }
  return w;
}

__device__ __forceinline__ void load_sweep_tables(const ReplicaDesc& R, uint32_t* s_thi, uint16_t* s_tlo,
                                                  uint8_t* s_eta) {
  for (int i = threadIdx.x; i < 33; i += blockDim.x) {
    unsigned long long T = R.thr_sweep[i];
    s_thi[i] = (uint32_t)(T >> 16);
    s_tlo[i] = (uint16_t)(T & 0xffffu);
  }
  for (int i = threadIdx.x; i < 72; i += blockDim.x) s_eta[i] = c_eta_table[i];
}

// One colour of the checkerboard sweep: every cell with (x+y+z)&1 == colour updates its six
// arms; its six neighbours have the other colour and stay frozen. Thread = V consecutive
// colour cells of one row, read and written with 128-bit accesses when V = 4.
template <int V>
__global__ void __launch_bounds__(kThreads) k_sweep(const ReplicaDesc* __restrict__ reps,
                                                    const ReplicaState* __restrict__ st,
                                                    const int* __restrict__ blk, int nrep, int colour, int jsweep) {
  __shared__ uint32_t s_thi[33];
  __shared__ uint16_t s_tlo[33];
  __shared__ uint8_t s_eta[72];
  const int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  load_sweep_tables(R, s_thi, s_tlo, s_eta);
  __syncthreads();
  const int L = R.L, H = R.H;
  const int cpr = H / V;
  long long q = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  if (q >= (long long)cpr * L * L) return;
  int hc = (int)(q % cpr);
  long long row = q / cpr;
  int y = (int)(row % L), z = (int)(row / L);
  CellBlock<V> cb;
  cb.load(R, colour, hc, y, z, s_eta);
  const uint32_t t = st[r].cur[0] + (uint32_t)jsweep;
  const uint32_t cbase = (uint32_t)L * ((uint32_t)y + (uint32_t)L * (uint32_t)z);
  uint32_t out[V];
#pragma unroll
  for (int k = 0; k < V; ++k) {
    uint32_t c0 = (uint32_t)(cb.x0 + 2 * k) + cbase;
    uint32_t nbs = neighbour_sigmas(cb.xp[k], cb.xm[k], cb.yp[k], cb.ym[k], cb.zp[k], cb.zm[k]);
    out[k] = update_cell(cb.own[k], nbs, cb.eta[k], c0, t, R, s_thi, s_tlo);
  }
  VecLoad<V>::st(cb.own_ptr, out);
}

// ------------------------------------------------------------------ measurement
__device__ __forceinline__ uint32_t pairs_from_hist(uint32_t h) {
  uint32_t p = 0;
#pragma unroll
  for (int v = 0; v < 6; ++v) {
    uint32_t c = (h >> (4 * v)) & 15u;
    p += c * (c - 1) / 2;
  }
  return p;
}

// GW:2014-2160: N_hb2 = sum over bonds of delta * (eta_i + eta_j), counted from the colour-0
// end of every bond (each bond joins the two colours); N_sigma over cells of both colours.
template <int V>
__global__ void __launch_bounds__(kThreads) k_measure(const ReplicaDesc* __restrict__ reps,
                                                      ReplicaState* __restrict__ st,
                                                      const int* __restrict__ blk, int nrep) {
  __shared__ uint32_t s_thi[33];
  __shared__ uint16_t s_tlo[33];
  __shared__ uint8_t s_eta[72];
  __shared__ unsigned long long s_acc[2];
  const int r = find_replica(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  load_sweep_tables(R, s_thi, s_tlo, s_eta);
  if (threadIdx.x < 2) s_acc[threadIdx.x] = 0;
  __syncthreads();
  const int L = R.L, H = R.H;
  const int cpr = H / V;
  long long q = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  uint32_t hb2 = 0, ns = 0;
  if (q < (long long)cpr * L * L) {
    int hc = (int)(q % cpr);
    long long row = q / cpr;
    int y = (int)(row % L), z = (int)(row / L);
    CellBlock<V> cb;
    cb.load(R, 0, hc, y, z, s_eta);
    uint32_t w1[V];
    VecLoad<V>::ld(R.cells[1] + (size_t)H * ((size_t)y + (size_t)L * z) + hc * V, w1);
#pragma unroll
    for (int k = 0; k < V; ++k) {
      uint32_t w = cb.own[k];
      uint32_t nbs = neighbour_sigmas(cb.xp[k], cb.xm[k], cb.yp[k], cb.ym[k], cb.zp[k], cb.zm[k]);
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        uint32_t same = ((w >> (3 * a)) & 7u) == ((nbs >> (3 * a)) & 7u);
        hb2 += same * 2u * ((cb.eta[k] >> a) & 1u);
      }
      ns += pairs_from_hist(sigma_histogram(w)) + pairs_from_hist(sigma_histogram(w1[k]));
    }
  }
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
    atomicAdd(&st[r].acc_hb2, s_acc[0]);
    atomicAdd(&st[r].acc_ns, s_acc[1]);
  }
}

__global__ void k_measure_begin(ReplicaState* __restrict__ st, int nrep) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  st[r].acc_hb2 = 0;
  st[r].acc_ns = 0;
}

__global__ void k_measure_end(ReplicaState* __restrict__ st, int nrep, int record) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  ReplicaState& S = st[r];
  SampleRec rec;
  rec.n_hb2 = (long long)S.acc_hb2;
  rec.n_sigma = (long long)S.acc_ns;
  rec.r_cell = S.r_cell;
  rec.volume = S.volume;
  S.last = rec;
  if (record && S.samples && S.n_samples < S.cap_samples) S.samples[S.n_samples] = rec;
  if (record) S.n_samples++;
}

// ------------------------------------------------------------------ launchers
static inline dim3 grid1(int n) { return dim3((unsigned)((n + kThreads - 1) / kThreads)); }

void launch_init_lattice(const BatchDev& b, cudaStream_t s) {
  k_init_sigma<<<b.nblk_cell, kThreads, 0, s>>>(b.reps, b.blk_cell, b.nrep);
  k_init_cubes<<<b.nblk_cube, kThreads, 0, s>>>(b.reps, b.blk_cube, b.nrep);
}

void launch_step_begin(const BatchDev& b, int nmet, int ncl, int do_cube, cudaStream_t s) {
  k_step_begin<<<grid1(b.nrep), kThreads, 0, s>>>(b.reps, b.st, b.nrep, nmet, ncl, do_cube);
}

void launch_cube_move(const BatchDev& b, cudaStream_t s) {
  k_cube_move<<<b.nblk_cube, kThreads, 0, s>>>(b.reps, b.st, b.blk_cube, b.nrep);
}

void launch_sweep(const BatchDev& b, int colour, int jsweep, cudaStream_t s) {
  switch (b.vec) {
    case 4: k_sweep<4><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep, colour, jsweep); break;
    case 2: k_sweep<2><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep, colour, jsweep); break;
    default: k_sweep<1><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep, colour, jsweep); break;
  }
}

void launch_measure(const BatchDev& b, int record, cudaStream_t s) {
  k_measure_begin<<<grid1(b.nrep), kThreads, 0, s>>>(b.st, b.nrep);
  switch (b.vec) {
    case 4: k_measure<4><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
    case 2: k_measure<2><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
    default: k_measure<1><<<b.nblk_sweep, kThreads, 0, s>>>(b.reps, b.st, b.blk_sweep, b.nrep); break;
  }
  k_measure_end<<<grid1(b.nrep), kThreads, 0, s>>>(b.st, b.nrep, record);
}

}  // namespace cvf
