// Cluster steps (Swendsen-Wang and Wolff) and cluster statistics of the GB300 CVF engine.
//
// Reference: SOURCE/gpu_water3D.cu ("GW") GW:2365-2542 (bond activation, min-label scans until
// nothing changes, cluster shift), GW:2199-2357 (the CPU Wolff step of the WOLFF build) and
// GW:2677-2780 (cluster statistics on the host).
// Here the labelling is a lock-free union-find over the 6N arm sites (site = arm*N + cell):
// parents only ever point to smaller site ids, roots are hooked under smaller roots with
// atomicMin, so each component's root is its minimum site id -- the same canonical label the
// reference's min-label propagation converges to, independent of thread scheduling.
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

// eta table of this translation unit ([state*8 + vertex offset] -> 6-bit eta mask); constant
// memory is per translation unit without relocatable device code.
static __constant__ uint8_t c_eta_table[72];

// In-cell components of every intra-cell bond mask: entry m (bit e set when the e-th pair (a, b),
// a < b in row-major order, is bonded) holds in 3-bit field a the smallest arm of arm a's
// component.
static __device__ uint32_t g_incell_lab[1 << 15];

static uint32_t incell_components(uint32_t m) {
  int root[6] = {0, 1, 2, 3, 4, 5};
  int e = 0;
  for (int a = 0; a < 5; ++a)
    for (int b = a + 1; b < 6; ++b, ++e) {
      if (!((m >> e) & 1u)) continue;
      const int ra = root[a], rb = root[b], lo = ra < rb ? ra : rb, hi = ra < rb ? rb : ra;
      for (int k = 0; k < 6; ++k)
        if (root[k] == hi) root[k] = lo;
    }
  uint32_t lab = 0;
  for (int k = 0; k < 6; ++k) lab |= (uint32_t)root[k] << (3 * k);
  return lab;
}

void init_sw_device_tables() {
  uint8_t eta[72];
  for (int s = 0; s < 9; ++s)
    for (int p = 0; p < 8; ++p) eta[s * 8 + p] = (uint8_t)cube_eta_bits(s, p);
  cudaMemcpyToSymbol(c_eta_table, eta, sizeof(eta));
  static uint32_t lab[1 << 15];
  for (uint32_t m = 0; m < (1u << 15); ++m) lab[m] = incell_components(m);
  cudaMemcpyToSymbol(g_incell_lab, lab, sizeof(lab));
}

__device__ __forceinline__ int find_replica_sw(const int* __restrict__ blk, int nrep, int b) {
  int lo = 0, hi = nrep - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(blk + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void cell_xyz(const ReplicaDesc& R, uint32_t c, int& x, int& y, int& z) {
  const uint32_t L = R.L;
  uint32_t q, rem;
  if (R.lgL >= 0) {
    x = (int)(c & (L - 1));
    q = c >> R.lgL;
    y = (int)(q & (L - 1));
    z = (int)(q >> R.lgL);
  } else {
    q = c / L;
    rem = c - q * L;
    x = (int)rem;
    z = (int)(q / L);
    y = (int)(q - (uint32_t)z * L);
  }
}

__device__ __forceinline__ uint32_t word_at(const ReplicaDesc& R, int x, int y, int z) {
  return R.cells[(x + y + z) & 1][(uint32_t)(x >> 1) + (uint32_t)R.H * ((uint32_t)y + (uint32_t)R.L * (uint32_t)z)];
}

// eta of the cell's six arms: from its two cubes, or (Flag_chessboard = 0) as stored.
__device__ __forceinline__ uint32_t eta_of_cell(const ReplicaDesc& R, int x, int y, int z) {
  const int L = R.L, H = R.H;
  if (R.eta6) return R.eta6[(size_t)x + (size_t)L * ((size_t)y + (size_t)L * z)];
  const int xo = (x & 1) ? x : (x == 0 ? L - 1 : x - 1);
  const int yo = (y & 1) ? y : (y == 0 ? L - 1 : y - 1);
  const int zo = (z & 1) ? z : (z == 0 ? L - 1 : z - 1);
  const int p = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
  uint32_t se = R.cubes[0][(size_t)(x >> 1) + (size_t)H * ((size_t)(y >> 1) + (size_t)H * (z >> 1))];
  uint32_t so = R.cubes[1][(size_t)(xo >> 1) + (size_t)H * ((size_t)(yo >> 1) + (size_t)H * (zo >> 1))];
  return (uint32_t)c_eta_table[se * 8 + p] | (uint32_t)c_eta_table[so * 8 + (p ^ 7)];
}

// ---------------------------------------------------------------- bonds + in-cell components
// Random numbers of a cell per SW step: three Philox blocks (kStSwBond + 0..2, words 0..11).
// Link l (0..17) is decided by the 32-bit uniform U whose high half is half (l & 1) of word
// l >> 1; the low half, at the same position of the refinement blocks kStSwBondRefine + 0..2, is
// drawn only when the high half equals T >> 16 (p ~ 2^-16 per link): U < T with T in [0, 2^32].
// Words 9 and 10 (then the retry streams of kStSwFlip) give an exact uniform in [0, 6^6) whose
// base-6 digits, most significant first, are the shifts of the clusters rooted at the cell's arm
// sites 0..5 (GW:2531-2542 draws one shift per cluster).
__device__ __noinline__ bool sw_link_exact(uint32_t c, uint32_t t, int l, uint32_t hi, unsigned long long T,
                                           const ReplicaDesc* R) {
  const U4 rf = philox(c, t, kStSwBondRefine + (uint32_t)(l >> 3), R->replica, R->key0, R->key1);
  const int k = (l >> 1) & 3;
  const uint32_t word = k == 0 ? rf.x : (k == 1 ? rf.y : (k == 2 ? rf.z : rf.w));
  const uint32_t lo = (word >> (16 * (l & 1))) & 0xffffu;
  return ((((unsigned long long)hi) << 16) | lo) < T;
}

// The accepted raw word of the shift digits when words 9 and 10 both fell in the rejected range.
__device__ __noinline__ uint32_t sw_flip_retry(uint32_t c, uint32_t t, const ReplicaDesc* R) {
  uint32_t w = 0;
  for (uint32_t k = 0; k < 256; ++k) {
    w = philox(c, t, retry_tag(kStSwFlip, k), R->replica, R->key0, R->key1).x;
    if (w * 46656u >= 2560u) return w;
  }
  return w;
}

// Exact bond mask of a cell whose fast decision met a tie (a 16-bit high half equal to T >> 16,
// p ~ 2^-16 per link): the bond blocks drawn again and every link decided from its full 32-bit
// uniform. eq has bit l set when link l's sigma (and eta) condition holds. Returns the 18-bit
// bond mask.
__device__ __noinline__ uint32_t sw_links_exact(uint32_t c, uint32_t t, uint32_t eq, const ReplicaDesc* R) {
  uint32_t bonds = 0;
  for (int l = 0; l < 18; ++l) {
    if (!((eq >> l) & 1u)) continue;
    const unsigned long long T = R->thr_sw[l < 3 ? 0 : 1];
    const U4 q = philox(c, t, kStSwBond + (uint32_t)(l >> 3), R->replica, R->key0, R->key1);
    const int k = (l >> 1) & 3;
    const uint32_t word = k == 0 ? q.x : (k == 1 ? q.y : (k == 2 ? q.z : q.w));
    const uint32_t hi = (word >> (16 * (l & 1))) & 0xffffu;
    bool b;
    if ((unsigned long long)hi != (T >> 16)) b = hi < (uint32_t)(T >> 16);
    else b = sw_link_exact(c, t, l, hi, T, R);
    bonds |= (uint32_t)b << l;
  }
  return bonds;
}

// GW:2383-2438: links 0..2 are the x+, y+, z+ hydrogen-bond links of the cell, links 3..17 the
// intra-cell pairs (a<b) in row-major order. The sigma conditions of the 15 pairs come from three
// whole-word comparisons (each arm against the arm 1, 2 and 3 places further round), and every
// link is decided from its 16-bit high half; a tie sends the cell through sw_links_exact. Besides
// the in-cell labels the kernel stores, per cell, the bond bits of its three hydrogen-bond links
// and the in-cell root (smallest arm of its in-cell component) of every arm, for the union and
// the finish.
__global__ void __launch_bounds__(kThreads) k_sw_local(const ReplicaDesc* __restrict__ reps,
                                                       ReplicaState* __restrict__ st,
                                                       const int* __restrict__ blk, int nrep, int jsw,
                                                       int worklist, int from_ctr) {
  pdl_trigger();
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int L = R.L;
  const uint32_t N = (uint32_t)L * L * L;
  const uint32_t c = (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  if (c >= N) return;
  int x, y, z;
  cell_xyz(R, c, x, y, z);
  pdl_wait();
  const uint32_t t = (from_ctr ? st[r].ctr[3] : st[r].cur[3]) + (uint32_t)jsw;
  const uint32_t w = word_at(R, x, y, z);
  const PhiloxKeys rk = philox_keys(R.key0, R.key1);
  uint32_t rw[12];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const U4 q = philox_rk((uint32_t)c, t, kStSwBond + j, R.replica, rk);
    rw[4 * j] = q.x;
    rw[4 * j + 1] = q.y;
    rw[4 * j + 2] = q.z;
    rw[4 * j + 3] = q.w;
  }
  // eq: bit l set when the sigma (and eta) condition of link l holds
  uint32_t eq = 0;
  if (R.Jeff != 0.0) {
    const uint32_t eta = eta_of_cell(R, x, y, z);
    const int xn = x + 1 == L ? 0 : x + 1, yn = y + 1 == L ? 0 : y + 1, zn = z + 1 == L ? 0 : z + 1;
    const uint32_t wn[3] = {word_at(R, xn, y, z), word_at(R, x, yn, z), word_at(R, x, y, zn)};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const bool same = ((w >> (6 * d)) & 7u) == ((wn[d] >> (6 * d + 3)) & 7u);
      const bool cond = R.Jeff > 0.0 ? (((eta >> (2 * d)) & 1u) && same) : !same;
      eq |= (uint32_t)cond << d;
    }
  }
  {
    // e[k] bit 3a: sigma_a == sigma_{(a+k) mod 6}
    const uint32_t w18 = w & 0x3ffffu;
    uint32_t e[4];
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
      const uint32_t rot = ((w18 >> (3 * k)) | (w18 << (18 - 3 * k))) & 0x3ffffu;
      const uint32_t xx = w18 ^ rot;
      e[k] = ~(xx | (xx >> 1) | (xx >> 2)) & 0x9249u;
    }
    int l = 3;
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int b = a + 1; b < 6; ++b, ++l) {
        // pairs 4 and 5 apart are the pairs (b, a) 2 and 1 apart going on round
        const int k = b - a;
        const uint32_t bit = k <= 3 ? (e[k] >> (3 * a)) & 1u : (e[6 - k] >> (3 * b)) & 1u;
        eq |= bit << l;
      }
  }
  // fast decisions from the 16-bit high halves: link l (half l & 1 of word l >> 1) bonds when its
  // condition holds and its half is below th = T >> 16 (T in [0, 2^32], so th in [0, 65536]);
  // the odd half compares the whole word with th * 65536 - 1, and a link class with th = 0 (never
  // bonds) leaves eq. Any half equal to th (65536 counted as 0xffff) sends the cell through the
  // exact path, which decides the links whose condition holds from their 32-bit uniforms: a
  // zero-halfword test of the word xor the two thresholds per word.
  const uint32_t thb = (uint32_t)(R.thr_sw[0] >> 16), ts = (uint32_t)(R.thr_sw[1] >> 16);
  const uint32_t ub = thb >= 65536u ? 0xffffffffu : (thb << 16) - 1u;
  const uint32_t us = ts >= 65536u ? 0xffffffffu : (ts << 16) - 1u;
  const uint32_t cb = thb < 0xffffu ? thb : 0xffffu, cs = ts < 0xffffu ? ts : 0xffffu;
  if (thb == 0u) eq &= ~7u;
  if (ts == 0u) eq &= 7u;
  uint32_t lt = 0, tz = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const uint32_t w = rw[k];
    const uint32_t th0 = 2 * k < 3 ? thb : ts, u1 = 2 * k + 1 < 3 ? ub : us;
    asm("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %1, %2;\n\t@p or.b32 %0, %0, %4;"
        "\n\tsetp.le.u32 p, %3, %5;\n\t@p or.b32 %0, %0, %6;\n\t}"
        : "+r"(lt)
        : "r"(w & 0xffffu), "r"(th0), "r"(w), "r"(1u << (2 * k)), "r"(u1), "r"(1u << (2 * k + 1)));
    const uint32_t x = w ^ (((2 * k + 1 < 3 ? cb : cs) << 16) | (2 * k < 3 ? cb : cs));
    tz |= (x - 0x00010001u) & ~x;
  }
  uint32_t bonds = eq & lt;
  if (tz & 0x80008000u) bonds = sw_links_exact(c, t, eq, &R);
  const uint32_t bm = bonds >> 3;  // intra-cell bonds: bit l-3 for link l = 3..17
  // shift digits of the clusters rooted at this cell's arm sites
  uint32_t u = rw[9];
  if (u * 46656u < 2560u) u = rw[10];
  if (u * 46656u < 2560u) u = sw_flip_retry(c, t, &R);
  uint32_t fw = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const unsigned long long m = (unsigned long long)u * 6ull;
    fw |= (uint32_t)(m >> 32) << (3 * a);
    u = (uint32_t)m;
  }
  R.flip[c] = fw;
  // in-cell components: lab holds 3 bits per arm, the smallest arm of its component
  const uint32_t lab = __ldg(g_incell_lab + bm);
  R.cellsw[c] = (bonds & 7u) | (lab << 3);
  if (worklist) {
    // cells with a hydrogen-bond link go to the replica's worklist (one atomic per warp)
    const unsigned act = __activemask();
    const unsigned linked = __ballot_sync(act, (bonds & 7u) != 0u);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (linked && lane == __ffs(linked) - 1) base = atomicAdd(&st[r].swq, (uint32_t)__popc(linked));
    base = __shfl_sync(act, base, __ffs(linked ? linked : 1u) - 1);
    if ((linked >> lane) & 1u) R.swlist[base + __popc(linked & ((1u << lane) - 1u))] = c;
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) R.label[a * N + c] = (int32_t)(((lab >> (3 * a)) & 7u) * N + c);
}

// ---------------------------------------------------------------- union-find
__device__ __forceinline__ int32_t uf_find(int32_t* p, int32_t x) {
  // Path halving. Parents only decrease and stay inside the component, so stale reads only
  // cost extra iterations; the walk ends at the root (at most x steps).
  for (int it = 0; it < (1 << 30); ++it) {
    int32_t px = __ldcg(p + x);
    if (px == x) return x;
    int32_t ppx = __ldcg(p + px);
    if (ppx != px) p[x] = ppx;
    x = ppx;
  }
  return x;
}

// Hooks the larger of the two roots under the smaller; gives up (false) after max_iters attempts.
__device__ __forceinline__ bool uf_unite(int32_t* p, int32_t a, int32_t b, uint32_t max_iters) {
  for (uint32_t it = 0; it < max_iters; ++it) {
    a = uf_find(p, a);
    b = uf_find(p, b);
    if (a == b) return true;
    if (a > b) {
      int32_t tmp = a;
      a = b;
      b = tmp;
    }
    int32_t old = atomicMin(p + b, a);
    if (old == b) return true;
    b = old;
  }
  return false;
}

// The worklist of the cells with a hydrogen-bond link, spread over the replica's threads (one
// thread per four cells of the lattice): a link joins the in-cell
// component of the cell's arm 2d with the in-cell component of the neighbour's arm 2d+1, so the
// union starts from the two in-cell roots (recorded by k_sw_local) rather than from the arm sites.
__global__ void __launch_bounds__(kThreads) k_sw_union(const ReplicaDesc* __restrict__ reps,
                                                       ReplicaState* __restrict__ st,
                                                       const int* __restrict__ blk, int nrep) {
  pdl_trigger();
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t L = R.L;
  const uint32_t N = L * L * L;
  const uint32_t nth = (uint32_t)(blk[r + 1] - blk[r]) * blockDim.x;
  const uint32_t t0 = (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  pdl_wait();
  const uint32_t n = st[r].swq;
  for (uint32_t i = t0; i < n; i += nth) {
    const uint32_t c = R.swlist[i];
    const uint32_t sw = R.cellsw[c];
    const uint32_t hb = sw & 7u;
    int xi, yi, zi;
    cell_xyz(R, c, xi, yi, zi);
    const uint32_t x = xi, y = yi, z = zi;
    const uint32_t nb[3] = {(x + 1 == L ? 0 : x + 1) + L * (y + L * z), x + L * ((y + 1 == L ? 0 : y + 1) + L * z),
                            x + L * (y + L * (z + 1 == L ? 0 : z + 1))};
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if ((hb >> d) & 1u) {
        const uint32_t ra = (sw >> (3 + 6 * d)) & 7u;                          // in-cell root of arm 2d
        const uint32_t rb = (R.cellsw[nb[d]] >> (3 + 3 * (2 * d + 1))) & 7u;  // of the neighbour's arm 2d+1
        if (!uf_unite(R.label, (int32_t)(ra * N + c), (int32_t)(rb * N + nb[d]), R.union_iters)) st[r].err = 1;
      }
  }
}

// The same unions with one thread per cell (cells without a hydrogen-bond link return at once),
// for lattices small enough that the worklist's few threads would leave SMs idle.
__global__ void __launch_bounds__(kThreads) k_sw_union_cells(const ReplicaDesc* __restrict__ reps,
                                                             ReplicaState* __restrict__ st,
                                                             const int* __restrict__ blk, int nrep) {
  pdl_trigger();
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const uint32_t L = R.L;
  const uint32_t N = L * L * L;
  const uint32_t c = (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  if (c >= N) return;
  pdl_wait();
  const uint32_t sw = R.cellsw[c];
  const uint32_t hb = sw & 7u;
  if (!hb) return;
  int xi, yi, zi;
  cell_xyz(R, c, xi, yi, zi);
  const uint32_t x = xi, y = yi, z = zi;
  const uint32_t nb[3] = {(x + 1 == L ? 0 : x + 1) + L * (y + L * z), x + L * ((y + 1 == L ? 0 : y + 1) + L * z),
                          x + L * (y + L * (z + 1 == L ? 0 : z + 1))};
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if ((hb >> d) & 1u) {
      const uint32_t ra = (sw >> (3 + 6 * d)) & 7u;
      const uint32_t rb = (R.cellsw[nb[d]] >> (3 + 3 * (2 * d + 1))) & 7u;
      if (!uf_unite(R.label, (int32_t)(ra * N + c), (int32_t)(rb * N + nb[d]), R.union_iters)) st[r].err = 1;
    }
}

// Compression, cluster shift and update in one pass, one thread per cell. An in-cell component
// none of whose arms carries a hydrogen-bond link (the cell's own x+, y+, z+ links, or the links
// of its x-, y-, z- neighbours into it) is a whole cluster: its root is its smallest arm site,
// which k_sw_local already stored as the label of every arm in it. Each of the other components
// walks once, from its in-cell root to the cluster's root (the minimum site id of the cluster),
// which becomes the label of each of its arms. Each
// cluster's shift is digit a of the shift word that k_sw_local drew for cell c, for the root site
// a*N + c (GW:2531-2542 gives every cluster one uniform shift in 0..5); sigma is shifted by it.
__global__ void __launch_bounds__(kThreads) k_sw_finish(const ReplicaDesc* __restrict__ reps,
                                                        ReplicaState* __restrict__ st,
                                                        const int* __restrict__ blk, int nrep, int jsw) {
  pdl_trigger();
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int L = R.L;
  const uint32_t N = (uint32_t)L * L * L;
  const uint32_t c = (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  if (c >= N) return;
  int x, y, z;
  cell_xyz(R, c, x, y, z);
  const uint32_t cxm = (uint32_t)(x == 0 ? L - 1 : x - 1) + (uint32_t)L * ((uint32_t)y + (uint32_t)L * (uint32_t)z);
  const uint32_t cym = (uint32_t)x + (uint32_t)L * ((uint32_t)(y == 0 ? L - 1 : y - 1) + (uint32_t)L * (uint32_t)z);
  const uint32_t czm = (uint32_t)x + (uint32_t)L * ((uint32_t)y + (uint32_t)L * (uint32_t)(z == 0 ? L - 1 : z - 1));
  pdl_wait();
  if (c == 0) st[r].swq = 0;  // the union has used the worklist; the next SW step refills it
  const uint32_t sw = R.cellsw[c];
  const uint32_t lab = sw >> 3;
  // arms with a hydrogen-bond link: 0, 2, 4 from this cell's links, 1, 3, 5 from the neighbours'
  const uint32_t ext = (sw & 1u) | ((R.cellsw[cxm] & 1u) << 1) | ((sw & 2u) << 1) | ((R.cellsw[cym] & 2u) << 2) |
                       ((sw & 4u) << 2) | ((R.cellsw[czm] & 4u) << 3);
  // in-cell roots of the components that some link reaches, as a 6-bit mask
  uint32_t ext_root = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a)
    if ((ext >> a) & 1u) ext_root |= 1u << ((lab >> (3 * a)) & 7u);
  uint32_t* wp = R.cells[(x + y + z) & 1] + (uint32_t)(x >> 1) + (uint32_t)R.H * ((uint32_t)y + (uint32_t)L * (uint32_t)z);
  const uint32_t w = *wp;
  const uint32_t own_flip = R.flip[c];
  uint32_t out = 0;
  if (ext_root == 0) {
    // no link reaches the cell: every cluster is an in-cell component, rooted here
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const uint32_t m = (lab >> (3 * a)) & 7u;
      uint32_t v = ((w >> (3 * a)) & 7u) + ((own_flip >> (3 * m)) & 7u);
      v = v >= 6u ? v - 6u : v;
      out |= v << (3 * a);
    }
    *wp = out;
    return;
  }
  // one walk per in-cell component that a link reaches: its root (stored as the label of each of
  // its arms) and the root's shift digit, which replaces field m of the cell's shift word
  uint32_t shw = own_flip;
  uint32_t todo = ext_root;
  while (todo) {
    const uint32_t m = (uint32_t)__ffs(todo) - 1u;
    todo &= todo - 1u;
    int32_t root = (int32_t)(m * N + c);
    for (int it = 0; it < (1 << 30); ++it) {
      const int32_t px = __ldcg(R.label + root);
      if (px == root) break;
      root = px;
    }
#pragma unroll
    for (int a = 0; a < 6; ++a)
      if (((lab >> (3 * a)) & 7u) == m) R.label[a * N + c] = root;
    uint32_t rc = (uint32_t)root, ra = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k)
      if (rc >= N) {
        rc -= N;
        ++ra;
      }
    const uint32_t fw = rc == c ? own_flip : R.flip[rc];
    shw = (shw & ~(7u << (3 * m))) | (((fw >> (3 * ra)) & 7u) << (3 * m));
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    const uint32_t m = (lab >> (3 * a)) & 7u;
    uint32_t v = ((w >> (3 * a)) & 7u) + ((shw >> (3 * m)) & 7u);
    if (v >= 6u) v -= 6u;
    out |= v << (3 * a);
  }
  *wp = out;
}

// ---------------------------------------------------------------- Wolff cluster step
// GW:2199-2357 (cluster_step, cluster_poke, add_to_cluster, update_cluster): pokes until the
// flipped clusters add up to 6N sites. Poke P takes a seed site in [0, 6N) and a shift in 1..5,
// grows the seed's cluster over the bonds of the Swendsen-Wang step and shifts every site of it.
// Here every bond has its own uniform per poke, so the cluster is the seed's connected component
// of the poke's bond graph, whatever order it is searched in, and pokes can be grown in parallel:
// a batch grows one poke per warp of a cooperative grid from the same lattice, marks per site the
// first poke of the batch that changes it, and commits the pokes before the first one that
// examined (read) a site an earlier poke of the batch changes -- exactly the lattice that pokes
// applied one after another give. A poke whose cluster outgrows its warp (kWolffQ sites) is grown
// by the whole grid when it heads a batch.
//   poke P: block kStWolffPoke at (lo P, hi P): words 0-2 an exact draw of the seed site, word 3
//           an exact draw in [0, 5) (then the retry streams), shift = 1 + it
//   bond:   link l of owner cell c (the Swendsen-Wang numbering: 0-2 the x+, y+, z+ hydrogen-bond
//           links of c, 3-17 the intra-cell pairs) in poke P: U < T with U word l & 3 of block
//           kStWolffBond + l/4 at (c, lo P, tag | hi P << 8)
constexpr int kWolffQ = 128;   // cluster sites one warp grows
constexpr int kWolffH = 256;   // slots of its hash set of cluster sites (2 kWolffQ; hs_insert
                               // takes the top 8 bits of a multiplicative hash)
static_assert(kWolffH == 256 && kWolffH >= 2 * kWolffQ, "hs_insert hashes to 8 bits");
constexpr int kChgNone = 0x7f7f7f7f;  // chg of a site no poke of the batch changes

struct WolffWarp {
  uint32_t q[kWolffQ];
  uint32_t hs[kWolffH];
};

__device__ __forceinline__ uint32_t* word_ptr(const ReplicaDesc& R, uint32_t c) {
  int x, y, z;
  cell_xyz(R, c, x, y, z);
  return R.cells[(x + y + z) & 1] + (uint32_t)(x >> 1) + (uint32_t)R.H * ((uint32_t)y + (uint32_t)R.L * (uint32_t)z);
}

// Neighbour of cell c along arm a (0 x+, 1 x-, 2 y+, 3 y-, 4 z+, 5 z-).
__device__ __forceinline__ uint32_t nb_cell(const ReplicaDesc& R, uint32_t c, int a) {
  int x, y, z;
  cell_xyz(R, c, x, y, z);
  const int L = R.L;
  switch (a) {
    case 0: x = x + 1 == L ? 0 : x + 1; break;
    case 1: x = x == 0 ? L - 1 : x - 1; break;
    case 2: y = y + 1 == L ? 0 : y + 1; break;
    case 3: y = y == 0 ? L - 1 : y - 1; break;
    case 4: z = z + 1 == L ? 0 : z + 1; break;
    default: z = z == 0 ? L - 1 : z - 1; break;
  }
  return (uint32_t)x + (uint32_t)L * ((uint32_t)y + (uint32_t)L * (uint32_t)z);
}

__device__ __forceinline__ bool wolff_link(const ReplicaDesc& R, uint32_t owner, int l, unsigned long long P) {
  const U4 r = philox(owner, (uint32_t)P, (kStWolffBond + (uint32_t)(l >> 2)) | ((uint32_t)(P >> 32) << 8), R.replica,
                      R.key0, R.key1);
  const uint32_t u = (l & 3) == 0 ? r.x : ((l & 3) == 1 ? r.y : ((l & 3) == 2 ? r.z : r.w));
  return (unsigned long long)u < R.thr_sw[l < 3 ? 0 : 1];
}

// Seed site and shift of poke P.
__device__ __forceinline__ void wolff_poke(const ReplicaDesc& R, unsigned long long P, uint32_t NS, uint32_t& seed,
                                           uint32_t& shift) {
  const uint32_t lo = (uint32_t)P, hi = (uint32_t)(P >> 32);
  const U4 r = philox(lo, hi, kStWolffPoke, R.replica, R.key0, R.key1);
  if (!lemire_try(r.x, NS, seed) && !lemire_try(r.y, NS, seed) && !lemire_try(r.z, NS, seed))
    seed = lemire_retry(NS, lo, hi, kStWolffPoke, R.replica, R.key0, R.key1);
  uint32_t d;
  if (!lemire_try(r.w, 5u, d)) d = lemire_retry(5u, lo, hi, kStWolffShift, R.replica, R.key0, R.key1);
  shift = 1u + d;
}

// The sites bonded to site (a, c) in poke P: up to five intra-cell arms and the facing arm of the
// neighbour; out[k] = site or 0xffffffff. Cell words are read through L2 (other blocks change
// them between batches). Returns the hydrogen-bond partner's cell (examined either way).
__device__ __forceinline__ uint32_t wolff_bonds(const ReplicaDesc& R, uint32_t site, unsigned long long P, uint32_t N,
                                                uint32_t out[6]) {
  const uint32_t a = site / N, c = site - a * N;
  const uint32_t w = __ldcg(word_ptr(R, c));
  const uint32_t sa = (w >> (3 * a)) & 7u;
#pragma unroll
  for (int b = 0; b < 6; ++b) {
    out[b] = 0xffffffffu;
    if ((uint32_t)b == a || ((w >> (3 * b)) & 7u) != sa) continue;
    const int lo = (uint32_t)b < a ? b : (int)a, hi = (uint32_t)b < a ? (int)a : b;
    const int l = 3 + (lo == 0 ? 0 : lo == 1 ? 5 : lo == 2 ? 9 : lo == 3 ? 12 : 14) + (hi - lo - 1);
    if (wolff_link(R, c, l, P)) out[b] = (uint32_t)b * N + c;
  }
  const int d = (int)a >> 1;
  const uint32_t nbc = nb_cell(R, c, (int)a);
  const uint32_t owner = (a & 1u) ? nbc : c;
  const uint32_t pa = a ^ 1u;  // the facing arm
  out[a] = 0xffffffffu;
  if (R.Jeff != 0.0) {
    const uint32_t sb = (__ldcg(word_ptr(R, nbc)) >> (3 * pa)) & 7u;
    int x, y, z;
    cell_xyz(R, c, x, y, z);
    const bool cond = R.Jeff > 0.0 ? (((eta_of_cell(R, x, y, z) >> a) & 1u) && sb == sa) : sb != sa;
    if (cond && wolff_link(R, owner, d, P)) out[a] = pa * N + nbc;
  }
  return nbc;
}

// Inserts site into the warp's hash set; true when it was not there.
__device__ __forceinline__ bool hs_insert(uint32_t* hs, uint32_t site) {
  uint32_t h = (site * 2654435761u) >> 24;  // top 8 bits: kWolffH = 256 slots
  for (int k = 0; k < kWolffH; ++k) {
    const uint32_t old = atomicCAS(hs + h, 0xffffffffu, site);
    if (old == 0xffffffffu) return true;
    if (old == site) return false;
    h = (h + 1u) & (kWolffH - 1);
  }
  return false;
}

// Shifts site by sh (mod 6) in place: an atomic add of the field's change, so that sites of one
// cell word updated by different threads compose.
__device__ __forceinline__ void wolff_shift(const ReplicaDesc& R, uint32_t site, uint32_t N, uint32_t sh) {
  const uint32_t a = site / N, c = site - a * N;
  uint32_t* p = word_ptr(R, c);
  const uint32_t v = (__ldcg(p) >> (3 * a)) & 7u;
  uint32_t nv = v + sh;
  if (nv >= 6u) nv -= 6u;
  atomicAdd(p, (nv - v) << (3 * a));
}

__global__ void __launch_bounds__(kWolffThreads) k_wolff(const ReplicaDesc* __restrict__ reps,
                                                         ReplicaState* __restrict__ st, int r, WolffDev W,
                                                         GridSync* gs, unsigned int polls) {
  __shared__ WolffWarp s_w[kWolffThreads / 32];
  __shared__ int s_commit, s_big, s_first;
  __shared__ long long s_sum, s_max, s_take;
  __shared__ long long s_wsum[kWolffThreads / 32], s_wmax[kWolffThreads / 32];
  const ReplicaDesc& R = reps[r];
  ReplicaState& S = st[r];
  const uint32_t N = (uint32_t)R.L * R.L * R.L, NS = 6u * N;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * (kWolffThreads / 32) + wib;  // the warp's poke within a batch
  const unsigned int nthr = gridDim.x * blockDim.x, tid = blockIdx.x * blockDim.x + threadIdx.x;
  WolffWarp& ww = s_w[wib];
  volatile WolffLoop* lp = W.loop;
  if (tid == 0) {
    lp->p0 = S.wpoke;
    lp->done = lp->pokes = lp->maxs = 0;
    lp->big = 0;
  }
  if (!grid_barrier(gs, st, polls)) return;
  for (int batch = 0;; ++batch) {
    // the loop state as the previous batch left it (block 0 changes it only after every block
    // has passed the batch's second barrier)
    const long long done0 = lp->done;
    if (done0 >= (long long)NS) break;
    const unsigned long long p0 = lp->p0;
    if (!lp->big) {
      // grow: one poke per warp
      for (int i = lane; i < kWolffH; i += 32) ww.hs[i] = 0xffffffffu;
      __syncwarp();
      uint32_t seed = 0, shift = 0;
      const unsigned long long P = p0 + (unsigned long long)gw;
      if (lane == 0) {
        wolff_poke(R, P, NS, seed, shift);
        hs_insert(ww.hs, seed);
        ww.q[0] = seed;
      }
      shift = __shfl_sync(0xffffffffu, shift, 0);
      __syncwarp();
      int n = 1, head = 0;
      bool over = false;
      while (head < n && !over) {
        const int end = n;
        for (int base = head; base < end && !over; base += 32) {
          const int i = base + lane;
          uint32_t nb[6];
          if (i < end) {
            wolff_bonds(R, ww.q[i], P, N, nb);
          } else {
#pragma unroll
            for (int k = 0; k < 6; ++k) nb[k] = 0xffffffffu;
          }
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            const bool fresh = nb[k] != 0xffffffffu && hs_insert(ww.hs, nb[k]);
            const unsigned m = __ballot_sync(0xffffffffu, fresh);
            const int pos = n + __popc(m & ((1u << lane) - 1u));
            if (fresh && pos < kWolffQ) ww.q[pos] = nb[k];
            n += __popc(m);
            if (n > kWolffQ) over = true;
          }
          __syncwarp();
        }
        head = end;
      }
      const int size = over ? kWolffQ : n;
      // mark the sites this poke changes, then (after the barrier) look for an earlier poke of the
      // batch that changes a site this one examined: the six arms of each cluster site's cell and
      // the facing arm of its hydrogen-bond partner
      for (int i = lane; i < size; i += 32) atomicMin(W.chg + ww.q[i], gw);
      if (!grid_barrier(gs, st, polls)) return;
      bool conflict = false;
      for (int i = lane; i < size && !over; i += 32) {
        const uint32_t site = ww.q[i], a = site / N, c = site - a * N;
#pragma unroll
        for (uint32_t b = 0; b < 6; ++b)
          if (__ldcg(W.chg + b * N + c) < gw) conflict = true;
        if (__ldcg(W.chg + (a ^ 1u) * N + nb_cell(R, c, (int)a)) < gw) conflict = true;
      }
      conflict = __any_sync(0xffffffffu, conflict);
      if (lane == 0) {
        W.size[gw] = n;
        W.flag[gw] = (over ? 2 : 0) | (conflict ? 1 : 0);
      }
      if (!grid_barrier(gs, st, polls)) return;
      // commit: the pokes before the first flagged one, up to the one that completes 6N sites;
      // every block computes the same answer, a round of kWolffThreads pokes at a time (the
      // loads of a round in parallel, a block scan of the sizes)
      {
        const long long rem = (long long)NS - done0;
        long long cum = 0, mx = 0;
        int commit = W.B;
        for (int base = 0; base < W.B; base += kWolffThreads) {
          const int w = base + (int)threadIdx.x;
          const bool in = w < W.B;
          const int f = in ? __ldcg(W.flag + w) : 0;
          const long long sz = in ? __ldcg(W.size + w) : 0;
          long long incl = sz;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
          }
          if (lane == 31) s_wsum[wib] = incl;
          if (threadIdx.x == 0) s_first = 0x7fffffff;
          __syncthreads();
          long long off = 0, tot = 0;
#pragma unroll
          for (int k = 0; k < kWolffThreads / 32; ++k) {
            off += k < wib ? s_wsum[k] : 0;
            tot += s_wsum[k];
          }
          incl += off;  // inclusive prefix of the round's sizes
          // 2w: stop before poke w (flagged); 2w + 1: stop after it (it completes 6N sites)
          if (in && f != 0) atomicMin(&s_first, 2 * w);
          if (in && f == 0 && cum + incl >= rem) atomicMin(&s_first, 2 * w + 1);
          __syncthreads();
          const int fs = s_first;
          const int stop = fs == 0x7fffffff ? base + kWolffThreads : (fs >> 1) + (fs & 1);  // pokes taken so far
          const bool taken = in && w < stop;
          if (taken && w == stop - 1) s_take = incl;
          long long m = taken ? sz : 0;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const long long t = __shfl_xor_sync(0xffffffffu, m, o);
            m = t > m ? t : m;
          }
          if (lane == 0) s_wmax[wib] = m;
          __syncthreads();
          long long rm = 0;
#pragma unroll
          for (int k = 0; k < kWolffThreads / 32; ++k) rm = s_wmax[k] > rm ? s_wmax[k] : rm;
          mx = rm > mx ? rm : mx;
          if (fs != 0x7fffffff || base + kWolffThreads >= W.B) {
            commit = stop < W.B ? stop : W.B;
            cum += stop > base ? (fs != 0x7fffffff ? s_take : tot) : 0;
            break;
          }
          cum += tot;
          __syncthreads();  // s_wsum and s_wmax are rewritten by the next round
        }
        if (threadIdx.x == 0) {
          s_commit = commit;
          s_sum = cum;
          s_max = mx;
          s_big = commit == 0;  // the first poke outgrew its warp
        }
      }
      __syncthreads();
      const int commit = s_commit;
      if (gw < commit)
        for (int i = lane; i < n; i += 32) wolff_shift(R, ww.q[i], N, shift);
      for (int i = lane; i < size; i += 32) W.chg[ww.q[i]] = kChgNone;
      if (tid == 0) {
        lp->p0 = p0 + (unsigned long long)commit;
        lp->done = done0 + s_sum;
        lp->pokes = lp->pokes + commit;
        if (s_max > lp->maxs) lp->maxs = s_max;
        lp->big = s_big;
      }
      if (!grid_barrier(gs, st, polls)) return;
    } else {
      // the batch's first poke outgrew its warp: the whole grid grows it, a level at a time
      uint32_t seed = 0, shift = 0;
      wolff_poke(R, p0, NS, seed, shift);
      if (tid == 0) {
        W.q[0] = seed;
        atomicOr(W.mark + (seed >> 5), 1u << (seed & 31));
        lp->tail = 1;
        lp->level1 = 1;
      }
      if (!grid_barrier(gs, st, polls)) return;
      unsigned int l0 = 0, l1 = lp->level1;
      while (l0 < l1) {
        for (unsigned int i = l0 + tid; i < l1; i += nthr) {
          uint32_t nb[6];
          wolff_bonds(R, __ldcg(W.q + i), p0, N, nb);
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            if (nb[k] == 0xffffffffu) continue;
            const uint32_t bit = 1u << (nb[k] & 31);
            if (atomicOr(W.mark + (nb[k] >> 5), bit) & bit) continue;
            W.q[atomicAdd((unsigned int*)&lp->tail, 1u)] = nb[k];
          }
        }
        if (!grid_barrier(gs, st, polls)) return;
        if (tid == 0) lp->level1 = lp->tail;
        if (!grid_barrier(gs, st, polls)) return;
        l0 = l1;
        l1 = lp->level1;
      }
      for (unsigned int i = tid; i < l1; i += nthr) {
        const uint32_t site = __ldcg(W.q + i);
        wolff_shift(R, site, N, shift);
        W.mark[site >> 5] = 0u;
      }
      if (!grid_barrier(gs, st, polls)) return;
      if (tid == 0) {
        lp->p0 = p0 + 1ull;
        lp->done = done0 + (long long)l1;
        lp->pokes = lp->pokes + 1;
        if ((long long)l1 > lp->maxs) lp->maxs = (long long)l1;
        lp->big = 0;
      }
      if (!grid_barrier(gs, st, polls)) return;
    }
  }
  if (tid == 0) {
    S.wpoke = lp->p0;
    S.w_pokes = lp->pokes;
    S.w_sum = lp->done;
    S.w_max = lp->maxs;
  }
}

int wolff_blocks_per_sm() {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_wolff, kWolffThreads, 0) != cudaSuccess) return 0;
  return per;
}

cudaError_t launch_wolff_step(const BatchDev& b, cudaStream_t s) {
  for (int r = 0; r < b.nrep; ++r) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)b.wdev.grid);
    cfg.blockDim = dim3(kWolffThreads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_wolff, (const ReplicaDesc*)b.reps, b.st, r, b.wdev, b.gsync,
                                       b.barrier_polls);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------- cluster statistics
__global__ void __launch_bounds__(kThreads) k_cs_count(const ReplicaDesc* __restrict__ reps,
                                                       const int* __restrict__ blk, int nrep) {
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const long long NS = 6LL * R.L * R.L * R.L;
  long long s = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  if (s >= NS) return;
  int32_t lab = R.label[s];
  unsigned peers = __match_any_sync(__activemask(), lab);
  if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) atomicAdd(R.csize + lab, __popc(peers));
}

__device__ __forceinline__ void top2_merge(unsigned long long& a1, unsigned long long& a2, unsigned long long b1,
                                           unsigned long long b2) {
  if (b1 > a1) {
    a2 = a1 > b2 ? a1 : b2;
    a1 = b1;
  } else {
    a2 = a2 > b1 ? a2 : b1;
  }
}

// Per label slot: cluster count, sums of s and s^2 (exact and with the reference's 32-bit wrap of
// s*s, GW:2697), block top-2 sizes into blocktop, percolation candidates (size >= 2L, GW:2702).
__global__ void __launch_bounds__(kThreads) k_cs_reduce(const ReplicaDesc* __restrict__ reps,
                                                        ReplicaState* __restrict__ st,
                                                        const int* __restrict__ blk, int nrep,
                                                        unsigned long long* __restrict__ blocktop) {
  __shared__ unsigned long long s_red[3];
  __shared__ unsigned long long s_top[kThreads / 32][2];
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int L = R.L;
  const long long NS = 6LL * L * L * L;
  long long s = (long long)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  if (threadIdx.x < 3) s_red[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long ncl = 0, sum2 = 0, sum2w = 0, t1 = 0, t2 = 0;
  if (s < NS) {
    long long sz = R.csize[s];
    if (sz > 0) {
      ncl = 1;
      sum2 = (unsigned long long)(sz * sz);
      sum2w = (unsigned long long)(long long)(int32_t)(uint32_t)((unsigned long long)sz * (unsigned long long)sz);
      t1 = (unsigned long long)sz;
      int k = -1;
      if (sz >= 2LL * L) {
        k = atomicAdd(&st[r].ncand, 1);
        if (k >= R.max_cand) {
          k = -1;
          st[r].err = 2;
        }
      }
      R.cand[s] = k;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ncl += __shfl_xor_sync(0xffffffffu, ncl, o);
    sum2 += __shfl_xor_sync(0xffffffffu, sum2, o);
    sum2w += __shfl_xor_sync(0xffffffffu, sum2w, o);
    unsigned long long b1 = __shfl_xor_sync(0xffffffffu, t1, o), b2 = __shfl_xor_sync(0xffffffffu, t2, o);
    top2_merge(t1, t2, b1, b2);
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_red[0], ncl);
    atomicAdd(&s_red[1], sum2);
    atomicAdd(&s_red[2], sum2w);
    s_top[warp][0] = t1;
    s_top[warp][1] = t2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a1 = 0, a2 = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) top2_merge(a1, a2, s_top[w][0], s_top[w][1]);
    blocktop[2 * (long long)blockIdx.x] = a1;
    blocktop[2 * (long long)blockIdx.x + 1] = a2;
    atomicAdd(&st[r].ncl, s_red[0]);
    atomicAdd(&st[r].sum2, s_red[1]);
    atomicAdd(&st[r].sum2w, s_red[2]);
  }
}

// Coordinate coverage of candidate clusters (GW:2723-2780): bit x of axis 0, y of axis 1,
// z of axis 2, OR-reduced across lanes that hit the same word before the atomic.
__global__ void __launch_bounds__(kThreads) k_cs_cover(const ReplicaDesc* __restrict__ reps,
                                                       const int* __restrict__ blk, int nrep) {
  const int r = find_replica_sw(blk, nrep, blockIdx.x);
  const ReplicaDesc& R = reps[r];
  const int L = R.L;
  const uint32_t N = (uint32_t)L * L * L;
  const uint32_t s = (uint32_t)(blockIdx.x - blk[r]) * blockDim.x + threadIdx.x;
  int k = -1;
  int coord[3] = {0, 0, 0};
  if (s < 6 * N) {
    k = R.cand[R.label[s]];
    cell_xyz(R, s % N, coord[0], coord[1], coord[2]);
  }
  const unsigned active = __ballot_sync(0xffffffffu, k >= 0);
  if (k < 0) return;
  const int W = (L + 31) >> 5;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    long long word = ((long long)k * 3 + ax) * W + (coord[ax] >> 5);
    unsigned grp = __match_any_sync(active, word);
    unsigned bits = __reduce_or_sync(grp, 1u << (coord[ax] & 31));
    if ((threadIdx.x & 31) == (unsigned)(__ffs(grp) - 1)) atomicOr(R.cover + word, bits);
  }
}

// One block per replica: merge the block top-2 values, count candidates that cover every x,
// every y or every z coordinate, and emit the statistics record.
__global__ void __launch_bounds__(kThreads) k_cs_final(const ReplicaDesc* __restrict__ reps,
                                                       ReplicaState* __restrict__ st,
                                                       const int* __restrict__ blk, int nrep,
                                                       const unsigned long long* __restrict__ blocktop,
                                                       int record) {
  __shared__ unsigned long long s_top[kThreads][2];
  __shared__ unsigned long long s_perc;
  const int r = blockIdx.x;
  if (r >= nrep) return;
  const ReplicaDesc& R = reps[r];
  ReplicaState& S = st[r];
  const int L = R.L;
  const int W = (L + 31) >> 5;
  unsigned long long a1 = 0, a2 = 0;
  for (int b = blk[r] + threadIdx.x; b < blk[r + 1]; b += blockDim.x)
    top2_merge(a1, a2, blocktop[2 * (long long)b], blocktop[2 * (long long)b + 1]);
  s_top[threadIdx.x][0] = a1;
  s_top[threadIdx.x][1] = a2;
  if (threadIdx.x == 0) s_perc = 0;
  __syncthreads();
  int ncand = S.ncand < R.max_cand ? S.ncand : R.max_cand;
  unsigned long long perc = 0;
  for (int k = threadIdx.x; k < ncand; k += blockDim.x) {
    bool any = false;
    for (int ax = 0; ax < 3 && !any; ++ax) {
      bool full = true;
      for (int j = 0; j < W && full; ++j) {
        int bits = L - 32 * j;
        uint32_t want = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
        full = (R.cover[((long long)k * 3 + ax) * W + j] & want) == want;
      }
      any = full;
    }
    perc += any;
  }
  atomicAdd(&s_perc, perc);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m1 = 0, m2 = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) top2_merge(m1, m2, s_top[i][0], s_top[i][1]);
    CStatsRec rec;
    rec.largest = (long long)m1;
    rec.second = (long long)m2;
    rec.n_percolating = (long long)s_perc;
    rec.n_clusters = (long long)S.ncl;
    rec.sum_size = 6LL * L * L * L;
    rec.sum_size2 = (long long)S.sum2;
    rec.sum_size2_wrap32 = (long long)S.sum2w;
    S.last_cstats = rec;
    if (record && S.cstats && S.n_cstats < S.cap_cstats) S.cstats[S.n_cstats] = rec;
    if (record) S.n_cstats++;
  }
}

__global__ void k_cs_begin(ReplicaState* __restrict__ st, int nrep) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  st[r].ncl = 0;
  st[r].sum2 = 0;
  st[r].sum2w = 0;
  st[r].ncand = 0;
}

// ---------------------------------------------------------------- launchers
// Lattices of 2^20 cells or more (L >= 102) unite over the worklist; smaller ones with one thread
// per cell, whose bonded threads spread over every SM (L=64 step 38 us with the worklist against
// 34 us per cell; L=128 125-127 us against 129-133 us).
void launch_sw_step(const BatchDev& b, int jsw, cudaStream_t s, int from_ctr) {
  const dim3 g((unsigned)b.nblk_cell);
  const int wl = (long long)b.max_L * b.max_L * b.max_L >= (1ll << 20);
  launch_pdl(k_sw_local, g, s, b.pdl, b.reps, b.st, b.blk_cell, b.nrep, jsw, wl, from_ctr);
  if (wl) launch_pdl(k_sw_union, dim3((unsigned)b.nblk_cell4), s, b.pdl, b.reps, b.st, b.blk_cell4, b.nrep);
  else launch_pdl(k_sw_union_cells, g, s, b.pdl, b.reps, b.st, b.blk_cell, b.nrep);
  launch_pdl(k_sw_finish, g, s, b.pdl, b.reps, b.st, b.blk_cell, b.nrep, jsw);
}

// Needs csize zeroed and cover zeroed by the caller (memset nodes); blocktop sized 2*nblk_site.
void launch_cluster_stats_impl(const BatchDev& b, unsigned long long* blocktop, int record, cudaStream_t s) {
  k_cs_begin<<<(b.nrep + kThreads - 1) / kThreads, kThreads, 0, s>>>(b.st, b.nrep);
  k_cs_count<<<b.nblk_site, kThreads, 0, s>>>(b.reps, b.blk_site, b.nrep);
  k_cs_reduce<<<b.nblk_site, kThreads, 0, s>>>(b.reps, b.st, b.blk_site, b.nrep, blocktop);
  k_cs_cover<<<b.nblk_site, kThreads, 0, s>>>(b.reps, b.blk_site, b.nrep);
  k_cs_final<<<b.nrep, kThreads, 0, s>>>(b.reps, b.st, b.blk_site, b.nrep, blocktop, record);
}

}  // namespace cvf
