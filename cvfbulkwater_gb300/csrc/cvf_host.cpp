// Host-side helpers of the engine (no GPU). Compiled with -ffp-contract=off: the acceptance
// tables and FP64 observables must round the same way as the CPU oracle.
#include "cvf_host.h"

#include <math.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>
#include <sys/mman.h>
#include <unistd.h>

#include "cvf_spec.cuh"

namespace cvf {

void compute_shells(int L, float Rc, std::vector<float>& dist, std::vector<int>& freq) {
  dist.clear();
  freq.clear();
  const long long N = (long long)L * L * L;
  for (long long j = 1; j < N; ++j) {
    int dx = (int)(j % L), dy = (int)((j / L) % L), dz = (int)(j / ((long long)L * L));
    if (dx > L / 2) dx = L - dx;
    if (dy > L / 2) dy = L - dy;
    if (dz > L / 2) dz = L - dz;
    float d = (float)sqrt((double)(dx * dx + dy * dy + dz * dz));
    if (!(d < Rc)) continue;
    size_t k = 0;
    for (; k < dist.size(); ++k)
      if (dist[k] == d) break;
    if (k == dist.size()) {
      dist.push_back(d);
      freq.push_back(1);
    } else {
      freq[k]++;
    }
  }
  for (size_t k = 0; k < freq.size(); ++k) freq[k] = (freq[k] / 2) * (int)N;
}

Thresholds make_thresholds(float T, float P) {
  Thresholds t;
  t.beta = 1. / T;
  float jeff_f = kJhbF - P * kVhbF;
  t.Jeff = (double)jeff_f;
  const double Js = (double)kJsigF;
  for (int dhb = -1; dhb <= 1; ++dhb)
    for (int dns = -5; dns <= 5; ++dns) {
      double dE = -t.Jeff * (double)dhb - Js * (double)dns;
      t.sweep[(dhb + 1) * 11 + dns + 5] = threshold_from_p(exp(-t.beta * dE));
    }
  for (int dhb = -4; dhb <= 4; ++dhb) {
    double dE = -t.Jeff * (double)dhb - Js * 0.0;
    t.cube[dhb + 4] = threshold_from_p(exp(-t.beta * dE));
  }
  // GW:992-993
  t.sw[0] = threshold_from_p(1.0 - exp(-t.beta * fabs(t.Jeff)));
  t.sw[1] = threshold_from_p(1.0 - exp(-t.beta * fabs(Js)));
  return t;
}

double host_evdw(double r, const std::vector<float>& dist, const std::vector<int>& freq, float Rc) {
  return evdw(r, dist.data(), freq.data(), (int)dist.size(), Rc);
}

void fill_obs(cvf_obs* o, long long n_hb2, long long n_sigma, double r_cell, double volume, double e_vdw,
              long long N, float P) {
  o->n_hb2 = n_hb2;
  o->n_sigma = n_sigma;
  o->r_cell = r_cell;
  o->volume = volume;
  o->e_vdw = e_vdw;
  o->n_hb = 0.5 * (double)n_hb2;
  o->energy = (e_vdw + (-(double)kJhbF) * o->n_hb) + (-(double)kJsigF) * (double)n_sigma;
  o->v_total = (double)N * r_cell * r_cell * r_cell + (double)kVhbF * o->n_hb;
  o->enthalpy = o->energy + (double)P * o->v_total;
  o->m = (double)n_sigma / ((double)N * 15.0);
}

void fill_cstats(cvf_cstats* c) {
  if (c->n_clusters > 0) {
    c->mean = (double)c->sum_size / (double)c->n_clusters;
    c->variance = (double)c->sum_size2 / (double)c->n_clusters - c->mean * c->mean;
    float n = (float)c->n_clusters;
    float avg = (float)c->sum_size / n;
    float avg2 = (float)c->sum_size2_wrap32 / n;
    avg2 -= avg * avg;
    c->mean_ref = avg;
    c->variance_ref = avg2;
  } else {
    c->mean = c->variance = 0.0;
    c->mean_ref = c->variance_ref = 0.0f;
  }
}

static inline size_t word_index(int L, int x, int y, int z) {
  const int H = L / 2;
  return (size_t)(x >> 1) + (size_t)H * ((size_t)y + (size_t)L * z);
}

// Runs body(begin, end) over [0, n) split across up to 16 host threads; `work` is the total
// amount of work (elements touched), below 2^16 of which the call stays on the calling thread.
template <class F>
static void parallel_for(long long n, long long work, F body) {
  unsigned hw = std::thread::hardware_concurrency();
  int nt = (int)std::min<unsigned>(hw ? hw : 1u, 16u);
  if (work < (1 << 16) || nt <= 1 || n < 2) {
    body(0LL, n);
    return;
  }
  std::vector<std::thread> th;
  long long chunk = (n + nt - 1) / nt;
  for (int i = 0; i < nt; ++i) {
    long long b = i * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { body(b, e); });
  }
  for (auto& t : th) t.join();
}

void touch_pages(void* p, size_t bytes) {
  if (!bytes) return;
  long ps = sysconf(_SC_PAGESIZE);
  if (ps <= 0) ps = 4096;
  const uintptr_t lo = (uintptr_t)p & ~((uintptr_t)ps - 1), hi = (uintptr_t)p + bytes;
  const long long n = (long long)((hi - lo + ps - 1) / ps);
  std::vector<unsigned char> in(n, 0);
  if (mincore((void*)lo, hi - lo, in.data()) != 0) std::fill(in.begin(), in.end(), 0);
  long long missing = 0;
  for (unsigned char v : in) missing += (v & 1) ? 0 : 1;
  if (!missing) return;
  parallel_for(n, missing * 64, [&](long long b, long long e) {
    for (long long k = b; k < e; ++k) {
      if (in[k] & 1) continue;
      // the first byte of the page that lies inside the range
      const uintptr_t a = std::max(lo + (uintptr_t)k * ps, (uintptr_t)p);
      *reinterpret_cast<volatile char*>(a) = 0;
    }
  });
}

std::string config_value_error(const int* c12, long long c) {
  for (int a = 0; a < 6; ++a) {
    int s = c12[c * 12 + a], e = c12[c * 12 + 6 + a];
    if (s < 0 || s > 5) return "Unexpected value for spin (" + std::to_string(s) + ") appeared in line " + std::to_string(c);
    if (e < 0 || e > 1)
      return "Unexpected value for active_bond (" + std::to_string(e) + ") appeared in line " + std::to_string(c);
  }
  return "invalid cell " + std::to_string(c);
}

bool pack_config(int L, const int* c12, uint32_t* cells0, uint32_t* cells1, uint8_t* ce, uint8_t* co,
                 std::string& err) {
  const int H = L / 2;
  const long long N = (long long)L * L * L;
  // first offending cell, if any (smallest index wins, as in a sequential reader)
  std::atomic<long long> bad{N};
  parallel_for((long long)L * L, N, [&](long long b, long long e) {
    for (long long row = b; row < e; ++row) {
      const int y = (int)(row % L), z = (int)(row / L);
      const long long c_row = row * L;
      uint32_t* dst[2] = {cells0 + (size_t)H * row, cells1 + (size_t)H * row};
      for (int x = 0; x < L; ++x) {
        const int* v = c12 + (c_row + x) * 12;
        uint32_t w = 0;
        bool ok = true;
        for (int a = 0; a < 6; ++a) {
          ok = ok && v[a] >= 0 && v[a] <= 5 && v[6 + a] >= 0 && v[6 + a] <= 1;
          w |= (uint32_t)(v[a] & 7) << (3 * a);
        }
        if (!ok) {
          long long c = c_row + x, cur = bad.load();
          while (c < cur && !bad.compare_exchange_weak(cur, c)) {
          }
          return;
        }
        dst[(x + y + z) & 1][x >> 1] = w;
      }
    }
  });
  if (bad.load() < N) {
    err = config_value_error(c12, bad.load());
    return false;
  }
  auto eta = [&](int arm, int x, int y, int z) -> int {
    return c12[((long long)x + (long long)L * (y + (long long)L * z)) * 12 + 6 + arm];
  };
  // cube states from eta with the decision tree of GW:3330-3369 (vertices v1 = origin, v2 x+1,
  // v3 y+1, v6 y+1 z+1, v7 x+1 z+1, v8 x+1 y+1)
  parallel_for(2LL * H, N / 4, [&](long long b, long long e) {
    for (long long pc = b; pc < e; ++pc) {
      int par = (int)(pc / H), c = (int)(pc % H);
      for (int bb = 0; bb < H; ++bb)
        for (int a = 0; a < H; ++a) {
          int x = 2 * a + par, y = 2 * bb + par, z = 2 * c + par;
          int xp = x + 1 == L ? 0 : x + 1, yp = y + 1 == L ? 0 : y + 1, zp = z + 1 == L ? 0 : z + 1;
          int st;
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
          (par ? co : ce)[(size_t)a + (size_t)H * ((size_t)bb + (size_t)H * c)] = (uint8_t)st;
        }
    }
  });
  return true;
}

void unpack_config(int L, const uint32_t* cells0, const uint32_t* cells1, const uint8_t* ce, const uint8_t* co,
                   int* c12) {
  const int H = L / 2;
  uint8_t tab[72];
  for (int s = 0; s < 9; ++s)
    for (int p = 0; p < 8; ++p) tab[s * 8 + p] = (uint8_t)cube_eta_bits(s, p);
  parallel_for((long long)L * L, (long long)L * L * L, [&](long long b, long long e) {
    for (long long row = b; row < e; ++row) {
      const int y = (int)(row % L), z = (int)(row / L);
      const int yo = (y & 1) ? y : (y + L - 1) % L, zo = (z & 1) ? z : (z + L - 1) % L;
      const uint32_t* src[2] = {cells0 + (size_t)H * row, cells1 + (size_t)H * row};
      const uint8_t* erow = ce + (size_t)H * ((size_t)(y >> 1) + (size_t)H * (z >> 1));
      const uint8_t* orow = co + (size_t)H * ((size_t)(yo >> 1) + (size_t)H * (zo >> 1));
      int* out = c12 + row * L * 12;
      for (int x = 0; x < L; ++x) {
        const uint32_t w = src[(x + y + z) & 1][x >> 1];
        const int xo = (x & 1) ? x : (x + L - 1) % L;
        const int p = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
        const uint32_t eta = (uint32_t)tab[erow[x >> 1] * 8 + p] | (uint32_t)tab[orow[xo >> 1] * 8 + (p ^ 7)];
        int* v = out + 12 * x;
        for (int a = 0; a < 6; ++a) {
          v[a] = (int)((w >> (3 * a)) & 7u);
          v[6 + a] = (int)((eta >> a) & 1u);
        }
      }
    }
  });
}

}  // namespace cvf
