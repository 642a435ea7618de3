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
template <bool kVec>
__global__ void k_pack_cells(const int* __restrict__ c12, uint32_t L, uint32_t H, int lgL, uint32_t N,
                             uint32_t* __restrict__ cells0, uint32_t* __restrict__ cells1, uint8_t* __restrict__ eta6,
                             unsigned long long* bad) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  int v[12];
  if (kVec) {
    const int4* p = reinterpret_cast<const int4*>(c12) + 3ull * c;
    const int4 a = p[0], b = p[1], d = p[2];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    v[8] = d.x; v[9] = d.y; v[10] = d.z; v[11] = d.w;
  } else {
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

cudaError_t launch_pack_config(const ReplicaDesc& R, const int* c12, uint32_t* cells0, uint32_t* cells1, uint8_t* eta6,
                               uint8_t* ce, uint8_t* co, unsigned long long* bad, cudaStream_t s) {
  const uint32_t L = (uint32_t)R.L, H = (uint32_t)R.H, N = L * L * L;
  const bool vec = ((uintptr_t)c12 & 15u) == 0;
  if (vec) k_pack_cells<true><<<grid_of(N), kThreads, 0, s>>>(c12, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  else k_pack_cells<false><<<grid_of(N), kThreads, 0, s>>>(c12, L, H, R.lgL, N, cells0, cells1, eta6, bad);
  k_pack_cubes<<<grid_of(2ull * H * H * H), kThreads, 0, s>>>(eta6, L, H, ce, co);
  return cudaGetLastError();
}

}  // namespace cvf
