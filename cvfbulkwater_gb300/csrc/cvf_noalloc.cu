// Cluster statistics of a caller-owned device label array without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is being captured
// (an allocation would break the capture), processes whose device memory is fully reserved by
// another allocator or capped by a memory pool, and embedding hosts that forbid the library to
// grow its footprint after start-up. This variant of the cluster-statistics kernels (cvf_sw.cu)
// takes its work space from a fixed array in the library's own device memory instead: the
// array below exists on every GPU that loads the library, from load until process exit.
//
// Limits and sharing: at most CVF_NOALLOC_MAX_SITES = 6 L^3 label sites (even L <= 54). Every
// call uses the same array and leaves its contents behind; each call clears what must start at
// zero, but two calls whose kernels overlap on the GPU (different streams, no ordering) race on
// it and give wrong results. The first call on a device looks up the array's device address
// (cudaGetSymbolAddress); make that first call before any stream capture.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/cvf.h"

namespace cvf {
void set_last_error(const std::string& m);
}

namespace {

constexpr int kNaThreads = 256;
constexpr long long kNaMaxSites = CVF_NOALLOC_MAX_SITES;
constexpr int kNaMaxL = 54;                       // largest even L with 6 L^3 <= kNaMaxSites
static_assert(6LL * kNaMaxL * kNaMaxL * kNaMaxL <= kNaMaxSites, "scratch limit");
constexpr int kNaMaxCand = 3 * kNaMaxL * kNaMaxL;  // clusters of size >= 2L: at most 6N / 2L
constexpr int kNaMaxW = (kNaMaxL + 31) / 32;
constexpr int kNaMaxBlocks = (int)((kNaMaxSites + kNaThreads - 1) / kNaThreads);

// Byte offsets of the parts of the scratch array.
constexpr size_t kOffSize = 0;                                              // int32[max sites]
constexpr size_t kOffCand = kOffSize + 4 * (size_t)kNaMaxSites;             // int32[max sites]
constexpr size_t kOffCover = kOffCand + 4 * (size_t)kNaMaxSites;            // uint32[cand*3*W]
constexpr size_t kOffTop = kOffCover + 4 * (size_t)kNaMaxCand * 3 * kNaMaxW;  // u64[2*blocks]
constexpr size_t kOffCnt = kOffTop + 16 * (size_t)kNaMaxBlocks;             // u64[4] counters
constexpr size_t kScratchBytes = kOffCnt + 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct NaPtrs {
  int32_t* size;
  int32_t* cand;
  uint32_t* cover;
  unsigned long long* top;
  unsigned long long* cnt;  // [0] clusters, [1] sum s^2, [2] sum wrap32(s^2), [3] low 32 bits: candidates; bit 63: bad label
};

__global__ void k_na_count(const int32_t* __restrict__ labels, int nsites, NaPtrs p) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsites) return;
  const int32_t lab = labels[s];
  if (lab < 0 || lab >= nsites) {
    atomicOr(p.cnt + 3, 1ull << 63);
    return;
  }
  const unsigned peers = __match_any_sync(__activemask(), lab);
  if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) atomicAdd(p.size + lab, __popc(peers));
}

__device__ __forceinline__ void na_top2(unsigned long long& a1, unsigned long long& a2, unsigned long long b1,
                                        unsigned long long b2) {
  if (b1 > a1) {
    a2 = a1 > b2 ? a1 : b2;
    a1 = b1;
  } else {
    a2 = a2 > b1 ? a2 : b1;
  }
}

__global__ void k_na_reduce(int nsites, int L, NaPtrs p) {
  __shared__ unsigned long long s_red[3];
  __shared__ unsigned long long s_top[kNaThreads / 32][2];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (threadIdx.x < 3) s_red[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long ncl = 0, sum2 = 0, sum2w = 0, t1 = 0, t2 = 0;
  if (s < nsites) {
    const long long sz = p.size[s];
    if (sz > 0) {
      ncl = 1;
      sum2 = (unsigned long long)(sz * sz);
      sum2w = (unsigned long long)(long long)(int32_t)(uint32_t)((unsigned long long)sz * (unsigned long long)sz);
      t1 = (unsigned long long)sz;
      int k = -1;
      if (sz >= 2LL * L) {
        k = (int)(atomicAdd(p.cnt + 3, 1ull) & 0xffffffffull);
        if (k >= kNaMaxCand) k = -1;  // cannot happen: at most 6N / 2L <= kNaMaxCand candidates
      }
      p.cand[s] = k;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ncl += __shfl_xor_sync(0xffffffffu, ncl, o);
    sum2 += __shfl_xor_sync(0xffffffffu, sum2, o);
    sum2w += __shfl_xor_sync(0xffffffffu, sum2w, o);
    const unsigned long long b1 = __shfl_xor_sync(0xffffffffu, t1, o), b2 = __shfl_xor_sync(0xffffffffu, t2, o);
    na_top2(t1, t2, b1, b2);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_red[0], ncl);
    atomicAdd(&s_red[1], sum2);
    atomicAdd(&s_red[2], sum2w);
    s_top[threadIdx.x >> 5][0] = t1;
    s_top[threadIdx.x >> 5][1] = t2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a1 = 0, a2 = 0;
    for (int w = 0; w < kNaThreads / 32; ++w) na_top2(a1, a2, s_top[w][0], s_top[w][1]);
    p.top[2 * blockIdx.x] = a1;
    p.top[2 * blockIdx.x + 1] = a2;
    atomicAdd(p.cnt + 0, s_red[0]);
    atomicAdd(p.cnt + 1, s_red[1]);
    atomicAdd(p.cnt + 2, s_red[2]);
  }
}

__global__ void k_na_cover(const int32_t* __restrict__ labels, int nsites, int L, NaPtrs p) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int N = nsites / 6;
  int k = -1, coord[3] = {0, 0, 0};
  if (s < nsites) {
    const int32_t lab = labels[s];
    if (lab >= 0 && lab < nsites) k = p.cand[lab];
    const int c = s % N;
    coord[0] = c % L;
    coord[1] = (c / L) % L;
    coord[2] = c / (L * L);
  }
  const unsigned active = __ballot_sync(0xffffffffu, k >= 0);
  if (k < 0) return;
  const int W = (L + 31) >> 5;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const int word = (k * 3 + ax) * W + (coord[ax] >> 5);
    const unsigned grp = __match_any_sync(active, word);
    const unsigned bits = __reduce_or_sync(grp, 1u << (coord[ax] & 31));
    if ((threadIdx.x & 31) == (unsigned)(__ffs(grp) - 1)) atomicOr(p.cover + word, bits);
  }
}

__global__ void k_na_final(int nsites, int L, int nblocks, NaPtrs p, long long* __restrict__ out7) {
  __shared__ unsigned long long s_top[kNaThreads][2];
  __shared__ unsigned long long s_perc;
  unsigned long long a1 = 0, a2 = 0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) na_top2(a1, a2, p.top[2 * b], p.top[2 * b + 1]);
  s_top[threadIdx.x][0] = a1;
  s_top[threadIdx.x][1] = a2;
  if (threadIdx.x == 0) s_perc = 0;
  __syncthreads();
  const int W = (L + 31) >> 5;
  const unsigned long long c3 = p.cnt[3];
  int ncand = (int)(c3 & 0xffffffffull);
  if (ncand > kNaMaxCand) ncand = kNaMaxCand;
  unsigned long long perc = 0;
  for (int k = threadIdx.x; k < ncand; k += blockDim.x) {
    bool any = false;
    for (int ax = 0; ax < 3 && !any; ++ax) {
      bool full = true;
      for (int j = 0; j < W && full; ++j) {
        const int bits = L - 32 * j;
        const uint32_t want = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
        full = (p.cover[(k * 3 + ax) * W + j] & want) == want;
      }
      any = full;
    }
    perc += any;
  }
  atomicAdd(&s_perc, perc);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m1 = 0, m2 = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) na_top2(m1, m2, s_top[i][0], s_top[i][1]);
    const bool bad = (c3 >> 63) != 0;
    out7[0] = (long long)m1;
    out7[1] = (long long)m2;
    out7[2] = (long long)s_perc;
    out7[3] = bad ? -1 : (long long)p.cnt[0];
    out7[4] = (long long)nsites;
    out7[5] = (long long)p.cnt[1];
    out7[6] = (long long)p.cnt[2];
  }
}

// Device address of g_noalloc_scratch per device ordinal. Several host threads may make their
// first call on a device at once; they look up the same address, and the atomic slot makes
// their concurrent stores and loads well defined.
std::atomic<void*> g_scratch_addr[64];

int na_fail(int code, const std::string& m) {
  cvf::set_last_error(m);
  return code;
}

}  // namespace

extern "C" int cvf_cluster_stats_noalloc(const int* labels, int L, long long* out7, void* stream) {
  if (!labels || !out7) return na_fail(CVF_EINVAL, "cluster_stats_noalloc: null labels or out7");
  if (L < 4 || (L & 1)) return na_fail(CVF_EINVAL, "cluster_stats_noalloc: L must be even and >= 4");
  // L is bounded before 6 L^3 is formed, so no product can overflow
  if (L > kNaMaxL)
    return na_fail(CVF_EINVAL, "cluster_stats_noalloc: L = " + std::to_string(L) +
                                   ": its 6*L^3 label sites exceed the fixed scratch limit of " +
                                   std::to_string(kNaMaxSites) + " (even L <= 54)");
  const long long nsites = 6LL * L * L * L;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(CVF_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return na_fail(CVF_EINVAL, "cluster_stats_noalloc: device ordinal >= 64");
  void* addr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess || !addr)
      return na_fail(CVF_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[dev].store(addr, std::memory_order_release);
  }
  unsigned char* base = (unsigned char*)addr;
  NaPtrs p;
  p.size = (int32_t*)(base + kOffSize);
  p.cand = (int32_t*)(base + kOffCand);
  p.cover = (uint32_t*)(base + kOffCover);
  p.top = (unsigned long long*)(base + kOffTop);
  p.cnt = (unsigned long long*)(base + kOffCnt);
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)nsites;
  const int nblocks = (n + kNaThreads - 1) / kNaThreads;
  const int W = (L + 31) / 32;
  const size_t cover_bytes = (size_t)(3 * L * L) * 3 * W * sizeof(uint32_t);
  // clear the parts that accumulate: sizes, coverage bitmaps, counters
  if ((e = cudaMemsetAsync(p.size, 0, (size_t)n * sizeof(int32_t), s)) != cudaSuccess ||
      (e = cudaMemsetAsync(p.cover, 0, cover_bytes, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(p.cnt, 0, 4 * sizeof(unsigned long long), s)) != cudaSuccess)
    return na_fail(CVF_ECUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  k_na_count<<<nblocks, kNaThreads, 0, s>>>(labels, n, p);
  k_na_reduce<<<nblocks, kNaThreads, 0, s>>>(n, L, p);
  k_na_cover<<<nblocks, kNaThreads, 0, s>>>(labels, n, L, p);
  k_na_final<<<1, kNaThreads, 0, s>>>(n, L, nblocks, p, out7);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(CVF_ECUDA, std::string("cluster_stats_noalloc launch: ") + cudaGetErrorString(e));
  return 0;
}
