// Configuration upload kernels that read the caller's cells12 array (the config.out order of
// GW:1296-1305 and GW:730-811: six sigma values then six eta values per cell, cell =
// x + L*(y + L*z)) where it lies in host memory. They serve GPUs that access pageable host memory
// coherently through the host page tables (NVLink-C2C on GB300): the 48 bytes per cell cross the
// link once, and no host thread packs the lattice.
#include "cvf_device.cuh"
#include "cvf_spec.cuh"

namespace cvf {

__device__ __forceinline__ void cell_xyz(uint32_t c, uint32_t L, int lgL, uint32_t& x, uint32_t& y, uint32_t& z) {
  if (lgL >= 0) {
    x = c & (L - 1);
    y = (c >> lgL) & (L - 1);
    z = c >> (2 * lgL);
  } else {
    const uint32_t yz = c / L;
    x = c - yz * L;
    z = yz / L;
    y = yz - z * L;
  }
}

// One thread per cell: checks sigma in [0,5] and eta in {0,1} (GW:776-790), packs sigma into the
// colour-split word and the six eta bits into eta6[c]; the smallest offending cell goes to *bad.
// kVec (a 16-byte aligned array): the block's 256 cells (12 KB) are read with fully coalesced
// 16-byte loads into shared memory first, so every line of host memory crosses the link once.
constexpr int kCfgCells = 256;  // cells per block = threads per block
template <bool kVec>
__global__ void __launch_bounds__(kCfgCells) k_pack_cells(const int* __restrict__ c12, uint32_t L, uint32_t H, int lgL,
                                                          uint32_t N, uint32_t* __restrict__ cells0,
                                                          uint32_t* __restrict__ cells1, uint8_t* __restrict__ eta6,
                                                          unsigned long long* bad) {
  __shared__ int4 s_in[3 * kCfgCells];
  const uint32_t c0 = blockIdx.x * kCfgCells, c = c0 + threadIdx.x;
  int v[12];
  if (kVec) {
    const uint32_t n4 = 3u * min((uint32_t)kCfgCells, N - c0);
    const int4* src = reinterpret_cast<const int4*>(c12) + 3ull * c0;
    for (uint32_t i = threadIdx.x; i < n4; i += kCfgCells) s_in[i] = src[i];
    __syncthreads();
    if (c >= N) return;
    const int4 a = s_in[3 * threadIdx.x], b = s_in[3 * threadIdx.x + 1], d = s_in[3 * threadIdx.x + 2];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    v[8] = d.x; v[9] = d.y; v[10] = d.z; v[11] = d.w;
  } else {
    if (c >= N) return;
#pragma unroll
    for (int i = 0; i < 12; ++i) v[i] = c12[12ull * c + i];
  }
  uint32_t w = 0, e = 0;
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    ok = ok && (uint32_t)v[a] <= 5u && (uint32_t)v[6 + a] <= 1u;
    w |= ((uint32_t)v[a] & 7u) << (3 * a);
    e |= ((uint32_t)v[6 + a] & 1u) << a;
  }
  if (!ok) {
    atomicMin(bad, (unsigned long long)c);
    return;
  }
  uint32_t x, y, z;
  cell_xyz(c, L, lgL, x, y, z);
  ((x + y + z) & 1u ? cells1 : cells0)[(x >> 1) + H * (y + L * z)] = w;
  eta6[c] = (uint8_t)e;
}

// The reverse for cvf_get_config: one thread per cell builds its twelve values (sigma from the
// colour-split word, eta from the even and the odd cube containing the cell, as the host unpack
// does) in shared memory, then the block writes its 12 KB to the caller's 16-byte aligned array
// with fully coalesced 16-byte stores.
__global__ void __launch_bounds__(kCfgCells) k_unpack_cells(const uint32_t* __restrict__ cells0,
                                                            const uint32_t* __restrict__ cells1,
                                                            const uint8_t* __restrict__ ce,
                                                            const uint8_t* __restrict__ co, uint32_t L, uint32_t H,
                                                            int lgL, uint32_t N, int* __restrict__ c12) {
  __shared__ int4 s_out[3 * kCfgCells];
  __shared__ uint8_t s_tab[72];
  if (threadIdx.x < 72) s_tab[threadIdx.x] = (uint8_t)cube_eta_bits(threadIdx.x >> 3, threadIdx.x & 7);
  __syncthreads();
  const uint32_t c0 = blockIdx.x * kCfgCells, c = c0 + threadIdx.x;
  if (c < N) {
    uint32_t x, y, z;
    cell_xyz(c, L, lgL, x, y, z);
    const uint32_t w = ((x + y + z) & 1u ? cells1 : cells0)[(x >> 1) + H * (y + L * z)];
    const uint32_t xo = (x & 1u) ? x : (x == 0 ? L - 1 : x - 1);
    const uint32_t yo = (y & 1u) ? y : (y == 0 ? L - 1 : y - 1);
    const uint32_t zo = (z & 1u) ? z : (z == 0 ? L - 1 : z - 1);
    const uint32_t p = (x & 1u) | ((y & 1u) << 1) | ((z & 1u) << 2);
    const uint32_t se = ce[(x >> 1) + H * ((y >> 1) + H * (z >> 1))];
    const uint32_t so = co[(xo >> 1) + H * ((yo >> 1) + H * (zo >> 1))];
    const uint32_t eta = (uint32_t)s_tab[se * 8 + p] | (uint32_t)s_tab[so * 8 + (p ^ 7u)];
    int v[12];
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      v[a] = (int)((w >> (3 * a)) & 7u);
      v[6 + a] = (int)((eta >> a) & 1u);
    }
    s_out[3 * threadIdx.x] = make_int4(v[0], v[1], v[2], v[3]);
    s_out[3 * threadIdx.x + 1] = make_int4(v[4], v[5], v[6], v[7]);
    s_out[3 * threadIdx.x + 2] = make_int4(v[8], v[9], v[10], v[11]);
  }
  __syncthreads();
  const uint32_t n4 = 3u * min((uint32_t)kCfgCells, N - c0);
  int4* dst = reinterpret_cast<int4*>(c12) + 3ull * c0;
  for (uint32_t i = threadIdx.x; i < n4; i += kCfgCells) dst[i] = s_out[i];
}

// One thread per cube: the cube state from the eta of its vertices with the decision tree of
// GW:3330-3369 (vertices v1 = origin, v2 x+1, v3 y+1, v6 y+1 z+1, v7 x+1 z+1, v8 x+1 y+1). Even
// origins (2a,2b,2c) first, then odd origins (2a+1,2b+1,2c+1).
__global__ void k_pack_cubes(const uint8_t* __restrict__ eta6, uint32_t L, uint32_t H, uint8_t* __restrict__ ce,
                             uint8_t* __restrict__ co) {
  const uint32_t H3 = H * H * H;
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 2 * H3) return;
  const uint32_t par = q >= H3, qi = q - par * H3;
  const uint32_t a = qi % H, b = (qi / H) % H, c = qi / (H * H);
  const uint32_t x = 2 * a + par, y = 2 * b + par, z = 2 * c + par;
  const uint32_t xp = x + 1 == L ? 0 : x + 1, yp = y + 1 == L ? 0 : y + 1, zp = z + 1 == L ? 0 : z + 1;
  auto eta = [&](int arm, uint32_t xx, uint32_t yy, uint32_t zz) -> uint32_t {
    return (eta6[xx + L * (yy + L * zz)] >> arm) & 1u;
  };
  uint32_t st;
  if (eta(0, x, y, z) == 0) {
    if (eta(0, x, yp, zp) == 0) st = 2;
    else if (eta(4, x, yp, z) == 0) st = 3;
    else st = 8;
  } else if (eta(2, x, y, z) == 0) {
    if (eta(4, xp, y, z) == 0) st = 4;
    else if (eta(2, xp, y, zp) == 0) st = 5;
    else st = 7;
  } else {
    if (eta(0, x, yp, z) == 0) st = 0;
    else if (eta(4, xp, yp, z) == 0) st = 1;
    else st = 6;
  }
  (par ? co : ce)[qi] = (uint8_t)st;
}

static inline unsigned grid_of(unsigned long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// The reference's own host arrays (GW:1135-1137, GW:1298): s[arm*N + cell] and
// active_bond[arm*N + cell], one byte each, 12 bytes per cell. One thread per G consecutive cells
// reads (or writes) G bytes of each of the twelve arm rows at once: G = 16 (16-byte accesses, a
// warp covers 512 contiguous bytes of every row) when both arrays are 16-byte aligned and N is a
// multiple of 16, else G = 4 (4-byte accesses when 4-byte aligned, else single bytes).
template <int G, bool kWide>
struct ArmRow;
template <>
struct ArmRow<16, true> {
  static __device__ __forceinline__ void ld(const uint8_t* p, uint32_t q, uint32_t* v) {
    const uint4 t = reinterpret_cast<const uint4*>(p)[q];
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static __device__ __forceinline__ void st(uint8_t* p, uint32_t q, const uint32_t* v) {
    reinterpret_cast<uint4*>(p)[q] = make_uint4(v[0], v[1], v[2], v[3]);
  }
};
template <>
struct ArmRow<4, true> {
  static __device__ __forceinline__ void ld(const uint8_t* p, uint32_t q, uint32_t* v) {
    v[0] = reinterpret_cast<const uint32_t*>(p)[q];
  }
  static __device__ __forceinline__ void st(uint8_t* p, uint32_t q, const uint32_t* v) {
    reinterpret_cast<uint32_t*>(p)[q] = v[0];
  }
};
template <>
struct ArmRow<4, false> {
  static __device__ __forceinline__ void ld(const uint8_t* p, uint32_t q, uint32_t* v) {
    v[0] = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) v[0] |= (uint32_t)p[4 * q + k] << (8 * k);
  }
  static __device__ __forceinline__ void st(uint8_t* p, uint32_t q, const uint32_t* v) {
#pragma unroll
    for (int k = 0; k < 4; ++k) p[4 * q + k] = (uint8_t)(v[0] >> (8 * k));
  }
};

template <int G, bool kWide>
__global__ void __launch_bounds__(kThreads) k_pack_arms(const uint8_t* __restrict__ s, const uint8_t* __restrict__ ab,
                                                        uint32_t L, uint32_t H, int lgL, uint32_t N,
                                                        uint32_t* __restrict__ cells0, uint32_t* __restrict__ cells1,
                                                        uint8_t* __restrict__ eta6, unsigned long long* bad) {
  constexpr int W = G / 4;  // 32-bit words per row segment
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x, c0 = G * q;
  if (c0 >= N) return;
  uint32_t sv[6][W], ev[6][W];
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    ArmRow<G, kWide>::ld(s + (size_t)a * N, q, sv[a]);
    ArmRow<G, kWide>::ld(ab + (size_t)a * N, q, ev[a]);
  }
#pragma unroll
  for (int k = 0; k < G; ++k) {
    uint32_t w = 0, e = 0;
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const uint32_t sg = (sv[a][k >> 2] >> (8 * (k & 3))) & 0xffu, et = (ev[a][k >> 2] >> (8 * (k & 3))) & 0xffu;
      ok = ok && sg <= 5u && et <= 1u;
      w |= (sg & 7u) << (3 * a);
      e |= (et & 1u) << a;
    }
    const uint32_t c = c0 + k;
    if (!ok) {
      atomicMin(bad, (unsigned long long)c);
      continue;
    }
    uint32_t x, y, z;
    cell_xyz(c, L, lgL, x, y, z);
    ((x + y + z) & 1u ? cells1 : cells0)[(x >> 1) + H * (y + L * z)] = w;
    eta6[c] = (uint8_t)e;
  }
}

// The reverse: sigma from the colour-split words, eta from the two cubes of each cell.
template <int G, bool kWide>
__global__ void __launch_bounds__(kThreads) k_unpack_arms(const uint32_t* __restrict__ cells0,
                                                          const uint32_t* __restrict__ cells1,
                                                          const uint8_t* __restrict__ ce, const uint8_t* __restrict__ co,
                                                          uint32_t L, uint32_t H, int lgL, uint32_t N,
                                                          uint8_t* __restrict__ s, uint8_t* __restrict__ ab) {
  constexpr int W = G / 4;
  __shared__ uint8_t s_tab[72];
  if (threadIdx.x < 72) s_tab[threadIdx.x] = (uint8_t)cube_eta_bits(threadIdx.x >> 3, threadIdx.x & 7);
  __syncthreads();
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x, c0 = G * q;
  if (c0 >= N) return;
  uint32_t sv[6][W], ev[6][W];
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int i = 0; i < W; ++i) sv[a][i] = ev[a][i] = 0;
#pragma unroll
  for (int k = 0; k < G; ++k) {
    uint32_t x, y, z;
    cell_xyz(c0 + k, L, lgL, x, y, z);
    const uint32_t w = ((x + y + z) & 1u ? cells1 : cells0)[(x >> 1) + H * (y + L * z)];
    const uint32_t xo = (x & 1u) ? x : (x == 0 ? L - 1 : x - 1);
    const uint32_t yo = (y & 1u) ? y : (y == 0 ? L - 1 : y - 1);
    const uint32_t zo = (z & 1u) ? z : (z == 0 ? L - 1 : z - 1);
    const uint32_t p = (x & 1u) | ((y & 1u) << 1) | ((z & 1u) << 2);
    const uint32_t se = ce[(x >> 1) + H * ((y >> 1) + H * (z >> 1))];
    const uint32_t so = co[(xo >> 1) + H * ((yo >> 1) + H * (zo >> 1))];
    const uint32_t eta = (uint32_t)s_tab[se * 8 + p] | (uint32_t)s_tab[so * 8 + (p ^ 7u)];
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      sv[a][k >> 2] |= ((w >> (3 * a)) & 7u) << (8 * (k & 3));
      ev[a][k >> 2] |= ((eta >> a) & 1u) << (8 * (k & 3));
    }
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    ArmRow<G, kWide>::st(s + (size_t)a * N, q, sv[a]);
    ArmRow<G, kWide>::st(ab + (size_t)a * N, q, ev[a]);
  }
}

// Validation of a packed state (cvf_set_packed) already copied to the device: words words[0..nw)
// must hold six sigma fields in 0..5 and zero bits 18..31, bytes cubes[0..ncb) cube states 0..8.
// The smallest offending index goes to *bad (words first, then cube bytes at nw + i).
__global__ void k_check_packed(const uint32_t* __restrict__ words, unsigned long long nw,
                               const uint8_t* __restrict__ cubes, unsigned long long ncb, unsigned long long* bad) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = true;
  if (i < nw) {
    const uint32_t w = words[i];
    // a 3-bit field is above 5 (6 or 7) when its bits 2 and 1 are both set
    ok = (w >> 18) == 0u && (w & (w << 1) & 0x24924u) == 0u;
  } else if (i < nw + ncb) {
    ok = cubes[i - nw] < 9u;
  }
  if (!ok) atomicMin(bad, i);
}

cudaError_t launch_check_packed(const uint32_t* words, unsigned long long nw, const uint8_t* cubes,
                                unsigned long long ncb, unsigned long long* bad, cudaStream_t s) {
  const unsigned long long n = nw + ncb;
  k_check_packed<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(words, nw, cubes, ncb, bad);
  return cudaGetLastError();
}

cudaError_t launch_pack_config(const ReplicaDesc& R, const int* c12, uint32_t* cells0, uint32_t* cells1, uint8_t* eta6,
                               uint8_t* ce, uint8_t* co, unsigned long long* bad, cudaStream_t s) {
  const uint32_t L = (uint32_t)R.L, H = (uint32_t)R.H, N = L * L * L;
  const bool vec = ((uintptr_t)c12 & 15u) == 0;
  static_assert(kCfgCells == kThreads, "one cell per thread");
  if (vec) k_pack_cells<true><<<grid_of(N), kCfgCells, 0, s>>>(c12, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  else k_pack_cells<false><<<grid_of(N), kCfgCells, 0, s>>>(c12, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  k_pack_cubes<<<grid_of(2ull * H * H * H), kThreads, 0, s>>>(eta6, L, H, ce, co);
  return cudaGetLastError();
}

cudaError_t launch_pack_arms(const ReplicaDesc& R, const uint8_t* sg, const uint8_t* ab, uint32_t* cells0,
                             uint32_t* cells1, uint8_t* eta6, uint8_t* ce, uint8_t* co, unsigned long long* bad,
                             cudaStream_t s) {
  const uint32_t L = (uint32_t)R.L, H = (uint32_t)R.H, N = L * L * L;  // N is a multiple of 8
  const uintptr_t al = (uintptr_t)sg | (uintptr_t)ab;
  if ((al & 15u) == 0 && N % 16 == 0)
    k_pack_arms<16, true><<<grid_of(N / 16), kThreads, 0, s>>>(sg, ab, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  else if ((al & 3u) == 0)
    k_pack_arms<4, true><<<grid_of(N / 4), kThreads, 0, s>>>(sg, ab, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  else
    k_pack_arms<4, false><<<grid_of(N / 4), kThreads, 0, s>>>(sg, ab, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  k_pack_cubes<<<grid_of(2ull * H * H * H), kThreads, 0, s>>>(eta6, L, H, ce, co);
  return cudaGetLastError();
}

cudaError_t launch_unpack_arms(const ReplicaDesc& R, uint8_t* sg, uint8_t* ab, cudaStream_t s) {
  const uint32_t L = (uint32_t)R.L, H = (uint32_t)R.H, N = L * L * L;
  const uintptr_t al = (uintptr_t)sg | (uintptr_t)ab;
  if ((al & 15u) == 0 && N % 16 == 0)
    k_unpack_arms<16, true><<<grid_of(N / 16), kThreads, 0, s>>>(R.cells[0], R.cells[1], R.cubes[0], R.cubes[1], L, H, R.lgL, N, sg, ab);
  else if ((al & 3u) == 0)
    k_unpack_arms<4, true><<<grid_of(N / 4), kThreads, 0, s>>>(R.cells[0], R.cells[1], R.cubes[0], R.cubes[1], L, H, R.lgL, N, sg, ab);
  else
    k_unpack_arms<4, false><<<grid_of(N / 4), kThreads, 0, s>>>(R.cells[0], R.cells[1], R.cubes[0], R.cubes[1], L, H, R.lgL, N, sg, ab);
  return cudaGetLastError();
}

cudaError_t launch_unpack_config(const ReplicaDesc& R, int* c12, cudaStream_t s) {
  const uint32_t L = (uint32_t)R.L, H = (uint32_t)R.H, N = L * L * L;
  if (((uintptr_t)c12 & 15u) != 0) return cudaErrorInvalidValue;
  k_unpack_cells<<<grid_of(N), kCfgCells, 0, s>>>(R.cells[0], R.cells[1], R.cubes[0], R.cubes[1], L, H, R.lgL, N, c12);
  return cudaGetLastError();
}

}  // namespace cvf
