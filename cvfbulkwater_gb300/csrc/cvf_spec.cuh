// Engine specification shared by host and device code of the GB300 CVF engine.
//
// Everything a Monte Carlo decision depends on is defined here once, as integer arithmetic
// or as explicitly ordered FP64 operations, so that the CUDA kernels, the host driver and the
// CPU oracle (an independent restatement in oracle/cvf_oracle.c) agree bit for bit.
//
// Model: Coronas-Vilanova-Franzese water on an L^3 periodic simple-cubic lattice
// (reference SOURCE/gpu_water3D.cu, "GW" below). Each cell has six arms a = 0..5
// (0 x+, 1 x-, 2 y+, 3 y-, 4 z+, 5 z-), a q=6 Potts variable sigma_a per arm and a bond
// availability eta_a per arm. eta is owned by 2x2x2 cubes in one of nine "two-factor"
// states (GW:3180-3466, SOURCE/chessboard.h:155-208).
//
// Packed cell word (one uint32 per cell): bits 3a..3a+2 hold sigma_a, bits 18..31 are zero.
// eta is not stored per cell: it is derived from the states of the two cubes that contain
// the cell, so a cube move writes one byte per cube and the sweep never races on eta.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CVF_HD __host__ __device__ __forceinline__
#else
#define CVF_HD inline
#endif

// FP64 operations that must not be contracted into FMA on either side.
#if defined(__CUDA_ARCH__)
#define CVF_DMUL(a, b) __dmul_rn((a), (b))
#define CVF_DADD(a, b) __dadd_rn((a), (b))
#define CVF_DSUB(a, b) __dsub_rn((a), (b))
#else
#define CVF_DMUL(a, b) ((a) * (b))
#define CVF_DADD(a, b) ((a) + (b))
#define CVF_DSUB(a, b) ((a) - (b))
#endif

namespace cvf {

// ----------------------------------------------------------------- model constants
// Float literals as in GW:57-64; promoted to double where the reference promotes them.
constexpr float kJhbF = 0.5f;
constexpr float kJsigF = 0.08f;
constexpr float kVhbF = 0.6f;
constexpr int kArms = 6;
constexpr int kQ = 6;
constexpr double kRcell0 = 1.0001;  // GW:150
constexpr int kMaxShells = 512;

// ----------------------------------------------------------------- random streams
// Philox4x32-10 (Salmon et al., SC'11). key = seed, counter = (site, move counter, tag, replica).
enum : uint32_t {
  kStSweep = 0x01u,        // per cell per sweep: w0 proposals, w1..w3 accept high halves
  kStSweepRefine = 0x02u,  // per cell per sweep, drawn only on a high-half tie
  kStCube = 0x03u,         // per 4 cubes along x per cube move: w0,w3 proposals, w1,w2 accept high halves
  kStVolume = 0x04u,       // per volume move: (w0,w1) trial, (w2,w3) accept
  kStSwFlip = 0x05u,       // retry streams of the cluster-shift digits (words 9, 10 of the bond blocks)
  kStInitSigma = 0x06u,
  kStInitCube = 0x07u,
  kStInitOrder = 0x08u,
  kStCubeRefine = 0x09u,   // per 4 cubes per cube move, drawn only on a high-half tie
  kStSwBond = 0x10u,       // + 0..2: 12 words per cell per SW step: 18 link high halves, shift digits
  kStSwBondRefine = 0x18u, // + 0..2: the links' low halves, drawn only on a high-half tie
  kStWolffPoke = 0x0Au,    // per Wolff poke P at counter (lo P, hi P): w0..w2 seed site, w3 shift
  kStWolffShift = 0x0Bu,   // retry kind of the Wolff shift draw
  kStWolffBond = 0x20u,    // + l/4: link l of an owner cell in poke P, counter (cell, lo P, tag | hi P << 8)
};
CVF_HD uint32_t retry_tag(uint32_t kind, uint32_t k) { return 0x1000u | (kind << 8) | k; }

struct U4 {
  uint32_t x, y, z, w;
};

CVF_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umulhi(a, b);
#else
  uint64_t p = (uint64_t)a * b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

CVF_HD U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return U4{c0, c1, c2, c3};
}

// The same block with the key schedule computed once by the caller: rk[2r], rk[2r+1] are the two
// key words of round r. A kernel that draws several blocks with one key (every cell of a launch
// uses the replica's seed) computes the schedule once instead of once per block.
struct PhiloxKeys {
  uint32_t k[20];
};
CVF_HD PhiloxKeys philox_keys(uint32_t k0, uint32_t k1) {
  PhiloxKeys p;
  for (int r = 0; r < 10; ++r) {
    p.k[2 * r] = k0;
    p.k[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return p;
}
CVF_HD U4 philox_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const PhiloxKeys& rk) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c2, hi1, lo1);
    uint32_t n0 = hi1 ^ c1 ^ rk.k[2 * r];
    uint32_t n2 = hi0 ^ c3 ^ rk.k[2 * r + 1];
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  return U4{c0, c1, c2, c3};
}

// Lemire multiply-shift: value in [0,n) and whether the word lies in the exact (unbiased) range.
CVF_HD bool lemire_try(uint32_t w, uint32_t n, uint32_t& out) {
  uint64_t m = (uint64_t)w * n;
  out = (uint32_t)(m >> 32);
  return (uint32_t)m >= (uint32_t)(0u - n) % n;
}

// Slow path after the first words were rejected: word 0 of retry streams 0..255.
CVF_HD uint32_t lemire_retry(uint32_t n, uint32_t c0, uint32_t c1, uint32_t kind, uint32_t c3,
                             uint32_t k0, uint32_t k1) {
  uint32_t out = 0;
  for (uint32_t k = 0; k < 256; ++k) {
    U4 r = philox(c0, c1, retry_tag(kind, k), c3, k0, k1);
    if (lemire_try(r.x, n, out)) return out;
  }
  return out;
}

// 53-bit uniform double in [0,1) from two words.
CVF_HD double u53(uint32_t lo, uint32_t hi) {
  uint64_t b = ((((uint64_t)hi) << 32) | lo) >> 11;
  return (double)b * (1.0 / 9007199254740992.0);
}

// Acceptance threshold for probability p: U < T with U a uniform 32-bit integer, T in [0, 2^32].
inline uint64_t threshold_from_p(double p) {
  if (p >= 1.0) return 1ull << 32;
  if (!(p > 0.0)) return 0;
  double t = __builtin_floor(p * 4294967296.0 + 0.5);
  if (t >= 4294967296.0) return 1ull << 32;
  return (uint64_t)t;
}

// ----------------------------------------------------------------- cube geometry
// Vertex offsets as bits dx | dy<<1 | dz<<2. Edge e of a cube runs along kEdgeDir[e] from the
// vertex kEdgeStart[e]; the numbering and the nine states follow SOURCE/chessboard.h:21-53 and
// :155-208 so that the eta -> state decision tree of GW:3314-3371 maps identically.
// Packed as 2-bit (direction) and 3-bit (start offset) fields so device code can fold them.
constexpr uint32_t kEdgeDirBits = 0x9049a4u;              // e -> bits 2e..2e+1
constexpr unsigned long long kEdgeStartBits = 0x774891200ull;  // e -> bits 3e..3e+2
CVF_HD constexpr int edge_dir(int e) { return (int)((kEdgeDirBits >> (2 * e)) & 3u); }
CVF_HD constexpr int edge_start(int e) { return (int)((kEdgeStartBits >> (3 * e)) & 7ull); }
// Active-edge masks of the nine states (bit e set = edge e carries eta = 1), i.e. all edges
// except the four inactive ones listed per solution in SOURCE/chessboard.h:155-208.
CVF_HD constexpr uint32_t state_active(int s) {
  return s == 0 ? 0xdb3u : s == 1 ? 0x7d3u : s == 2 ? 0xcbeu : s == 3 ? 0x6deu : s == 4 ? 0x775u
       : s == 5 ? 0xb6du : s == 6 ? 0xbcbu : s == 7 ? 0xcedu : 0xb3eu;
}

// eta bits (6-bit arm mask) that a cube in state s gives to its vertex at offset p.
// A vertex with offset bit d = 0 is the start of the cube's d-edge (arm 2d), else its end
// (arm 2d+1).
CVF_HD uint32_t cube_eta_bits(int s, int p) {
  uint32_t m = 0;
  for (int d = 0; d < 3; ++d) {
    int start = p & ~(1 << d);
    int e = 0;
    for (int k = 0; k < 12; ++k)
      if (edge_dir(k) == d && edge_start(k) == start) e = k;
    if ((state_active(s) >> e) & 1u) m |= 1u << (2 * d + ((p >> d) & 1));
  }
  return m;
}

// ----------------------------------------------------------------- own FP64 exp / log
// exp: k = round(x/ln2), r = x - k ln2 in two parts (high part with 32 zero low mantissa bits),
// Taylor series of e^r to r^13 in Horner form, times 2^k built from the exponent bits.
// log: x = m 2^e with m in [1/sqrt2, sqrt2), log m = 2 atanh(s), s = (m-1)/(m+1), odd series
// to s^25. Every operation is rounded separately so host and device agree bit for bit.
CVF_HD double bits_to_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  __builtin_memcpy(&d, &b, 8);
  return d;
#endif
}
CVF_HD uint64_t double_to_bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  __builtin_memcpy(&b, &d, 8);
  return b;
#endif
}

CVF_HD double own_exp(double x) {
  const double kLn2Hi = 0.6931467056274414;
  const double kLn2Lo = 4.7493250390316726e-07;
  const double kInvLn2 = 1.4426950408889634;
  if (x != x) return x;
  if (x > 709.78) return bits_to_double(0x7FF0000000000000ull);
  if (x < -708.3) return 0.0;
  double kd = __builtin_floor(CVF_DADD(CVF_DMUL(x, kInvLn2), 0.5));
  double r = CVF_DSUB(CVF_DSUB(x, CVF_DMUL(kd, kLn2Hi)), CVF_DMUL(kd, kLn2Lo));
  const double c[14] = {1.6059043836821613e-10, 2.08767569878681e-09, 2.505210838544172e-08,
                        2.755731922398589e-07,  2.7557319223985893e-06, 2.48015873015873e-05,
                        0.0001984126984126984,  0.001388888888888889,  0.008333333333333333,
                        0.041666666666666664,   0.16666666666666666,   0.5,
                        1.0,                    1.0};
  double p = c[0];
  for (int i = 1; i < 14; ++i) p = CVF_DADD(CVF_DMUL(p, r), c[i]);
  int k = (int)kd;
  return CVF_DMUL(p, bits_to_double((uint64_t)(k + 1023) << 52));
}

CVF_HD double own_log(double x) {
  const double kLn2Hi = 0.6931467056274414;
  const double kLn2Lo = 4.7493250390316726e-07;
  if (x != x) return x;
  if (x < 0.0) return bits_to_double(0x7FF8000000000000ull);
  if (x == 0.0) return bits_to_double(0xFFF0000000000000ull);
  if (x > 1.7976931348623157e308) return x;
  uint64_t b = double_to_bits(x);
  int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) {
    b = double_to_bits(CVF_DMUL(x, 18014398509481984.0));
    e = (int)((b >> 52) & 0x7ff) - 54;
  }
  double m = bits_to_double((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  e -= 1023;
  if (m > 1.4142135623730951) {
    m = CVF_DMUL(m, 0.5);
    e += 1;
  }
  double s = CVF_DSUB(m, 1.0) / CVF_DADD(m, 1.0);
  double z = CVF_DMUL(s, s);
  const double c[13] = {0.04,
                        0.043478260869565216,
                        0.047619047619047616,
                        0.05263157894736842,
                        0.058823529411764705,
                        0.06666666666666667,
                        0.07692307692307693,
                        0.09090909090909091,
                        0.1111111111111111,
                        0.14285714285714285,
                        0.2,
                        0.3333333333333333,
                        1.0};
  double q = c[0];
  for (int i = 1; i < 13; ++i) q = CVF_DADD(CVF_DMUL(q, z), c[i]);
  double lm = CVF_DMUL(CVF_DMUL(2.0, s), q);
  double ed = (double)e;
  return CVF_DADD(CVF_DMUL(ed, kLn2Hi), CVF_DADD(CVF_DMUL(ed, kLn2Lo), lm));
}

// van der Waals lattice energy E(r) = sum_i f_i [(r d_i)^-12 - (r d_i)^-6 - shift], GW:1784-1805.
// The cut-off shift (1/Rc)^12 - (1/Rc)^6 of E_vdW (GW:1790-1794).
CVF_HD double vdw_shift(float Rc) {
  double tmp = 1.0 / (double)Rc;
  tmp = CVF_DMUL(CVF_DMUL(tmp, tmp), tmp);
  const double att = CVF_DMUL(tmp, tmp);
  const double rep = CVF_DMUL(att, att);
  return CVF_DSUB(rep, att);
}

CVF_HD double evdw(double r, const float* dist, const int* freq, int n, float Rc) {
  const double shift = vdw_shift(Rc);
  double tmp, att, rep;
  double ret = 0.0;
  for (int i = 0; i < n; ++i) {
    double rd = CVF_DMUL(r, (double)dist[i]);
    if (rd < (double)Rc) {
      tmp = 1.0 / rd;
      tmp = CVF_DMUL(CVF_DMUL(tmp, tmp), tmp);
      att = CVF_DMUL(tmp, tmp);
      rep = CVF_DMUL(att, att);
      ret = CVF_DADD(ret, CVF_DMUL((double)freq[i], CVF_DSUB(CVF_DSUB(rep, att), shift)));
    }
  }
  return ret;
}

}  // namespace cvf
