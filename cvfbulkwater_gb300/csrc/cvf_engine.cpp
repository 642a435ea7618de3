// Host engine behind the C ABI of include/cvf.h: owns device memory, builds the per-replica
// descriptors, captures Monte Carlo steps into CUDA graphs and replays them.
// There is no CPU fallback: every Monte Carlo move runs in the kernels of cvf_mc.cu / cvf_sw.cu.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/cvf.h"
#include "cvf_device.cuh"
#include "cvf_host.h"
#include "cvf_spec.cuh"

using namespace cvf;

static thread_local std::string g_err;

namespace cvf {
void set_last_error(const std::string& m) { g_err = m; }
}  // namespace cvf

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return fail(CVF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct ReplicaHost {
  cvf_params p;
  int L, H;
  long long N;
  std::vector<float> dist;
  std::vector<int> freq;
  Thresholds thr;
  ReplicaDesc desc;
};

struct cvf_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<ReplicaHost> reps;
  BatchDev b{};
  std::vector<void*> allocs;
  bool sw_alloc = false;
  bool sw_done = false;
  unsigned long long* blocktop = nullptr;
  std::map<std::tuple<int, int, int, int>, cudaGraphExec_t> graphs;
  // 0 (default): one launch per phase (step begin, cube + volume, each sweep colour,
  // measurement) in a captured graph; 1: Metropolis-only steps run as one persistent
  // cooperative launch per graph.
  int launch_mode = 0;
  void* staging = nullptr;  // pinned host buffer for configuration transfers (lazily allocated)
  SampleRec* rec_pin = nullptr;  // mapped page-locked landing place of the records cvf_observables
  SampleRec* rec_dev = nullptr;  // reads (one per replica), and its device address
  // the measured last step of the last run wrote every replica's record into rec_pin
  bool host_rec_valid = false;
  size_t staging_bytes = 0;
  // cvf_set_config / cvf_get_config: 1 = kernels read and pack, or unpack and write, the
  // caller's array in host memory (the GPU accesses pageable memory through the host page
  // tables), 0 = host packing and unpacking + copies.
  int io_mode = 0;
  bool io_capable = false;
  void* io_scratch = nullptr;  // device: packed cells, eta bytes and cube states of one replica
  size_t io_scratch_bytes = 0;
  unsigned long long* io_bad = nullptr;  // device: smallest invalid cell of a device-side pack
  double* stats = nullptr;               // device: 14 doubles per replica for cvf_run_statistics
  bool corr_on = false;                  // every captured step feeds the replicas' correlators
  // Replica groups: Metropolis-only steps of a batch are captured as one chain of per-phase
  // kernels per group of consecutive replicas, on parallel branches of the graph, so that one
  // group's blocks fill the tails of another group's kernels. 0 = automatic.
  int group_setting = 0;
  // Flag_chessboard = 0 for every replica: the nhb<=4 compatibility mode (no cube moves, bond
  // counts per cell, per-arm sweep launches, greedy bond count in the measurement)
  bool nhb_mode = false;
  // Every replica's last record (st.last) holds the measurement of its current cells:
  // cvf_observables then reads it instead of measuring the lattice. A Metropolis-only run that
  // follows cvf_observables measures its last step, so the read after it finds it there.
  bool last_valid = false;
  bool obs_since_run = false;
  cudaGraphExec_t nhb_read = nullptr;  // Flag_chessboard = 0: the read's 3L + 1 launches, captured once
  struct Group {
    BatchDev b;
    cudaStream_t s = nullptr;
    cudaEvent_t done = nullptr;
    int r0 = 0, r1 = 0;
  };
  std::vector<Group> groups;
  int groups_vec = 0;
  cudaEvent_t fork = nullptr;
  cudaStream_t vstream = nullptr;  // side branch of a chunk's volume moves
  cudaEvent_t vfork = nullptr, vdone = nullptr;
};

// Drops every cached graph (kernel arguments such as the block tables change).
static void drop_graphs(cvf_handle* h) {
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
  h->graphs.clear();
  if (h->nhb_read) cudaGraphExecDestroy(h->nhb_read);
  h->nhb_read = nullptr;
}

// A correlator in its initial state (GW:2983-3008): empty channels hold -2e10.
static CorrState corr_initial() {
  CorrState c;
  memset(&c, 0, sizeof(c));
  for (int k = 0; k < kCorrLevels; ++k)
    for (int i = 0; i < kCorrP; ++i) c.shift[k][i] = -2E10;
  return c;
}

// Device scratch for a device-side pack of one replica (freed with the handle).
static int ensure_io_scratch(cvf_handle* h, const ReplicaHost& R) {
  const size_t need = (size_t)R.N * 4 + (size_t)R.N + 2 * (size_t)R.H * R.H * R.H + 256;
  if (!h->io_bad) {
    cudaError_t e = cudaMalloc(&h->io_bad, sizeof(unsigned long long));
    if (e != cudaSuccess) return fail(CVF_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  if (h->io_scratch_bytes >= need) return 0;
  if (h->io_scratch) cudaFree(h->io_scratch);
  h->io_scratch = nullptr;
  h->io_scratch_bytes = 0;
  cudaError_t e = cudaMalloc(&h->io_scratch, need);
  if (e != cudaSuccess) return fail(CVF_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->io_scratch_bytes = need;
  return 0;
}

// Pinned host staging for one replica's packed lattice (N words) and cube states (2 (L/2)^3 B).
static int ensure_staging(cvf_handle* h, const ReplicaHost& R) {
  size_t need = (size_t)R.N * 4 + 2 * (size_t)R.H * R.H * R.H;
  if (h->staging_bytes >= need) return 0;
  if (h->staging) cudaFreeHost(h->staging);
  h->staging = nullptr;
  h->staging_bytes = 0;
  cudaError_t e = cudaHostAlloc(&h->staging, need, cudaHostAllocDefault);
  if (e != cudaSuccess) return fail(CVF_ENOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  h->staging_bytes = need;
  return 0;
}

static int dev_alloc(cvf_handle* h, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) return fail(CVF_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->allocs.push_back(*p);
  return 0;
}

static int upload_descs(cvf_handle* h) {
  std::vector<ReplicaDesc> d;
  for (auto& r : h->reps) d.push_back(r.desc);
  CK(cudaMemcpy(h->b.reps, d.data(), d.size() * sizeof(ReplicaDesc), cudaMemcpyHostToDevice));
  return 0;
}

static int fill_tables(cvf_handle* h, int r0, int r1, int vec, BatchDev& b);

static int build_tables(cvf_handle* h, int force_vec = 0) {
  const int n = (int)h->reps.size();
  int vec = 4;
  if (const char* ev = getenv("CVF_SWEEP_VEC")) {
    int v = atoi(ev);
    if (v == 1 || v == 2 || v == 4 || v == 8) vec = v;
  }
  if (force_vec) vec = force_vec;
  for (auto& r : h->reps) {
    while (vec > 1 && r.H % vec) vec >>= 1;
  }
  h->b.vec = vec;
  return fill_tables(h, 0, n, vec, h->b);
}

// Block prefix tables of replicas [r0, r1) (a new device allocation) into b.
static int fill_tables(cvf_handle* h, int r0, int r1, int vec, BatchDev& b) {
  const int n = r1 - r0;
  std::vector<int> ts(n + 1), tc(n + 1), tcv(n + 1), tl(n + 1), tsi(n + 1), ts4(n + 1), tl4(n + 1);
  ts[0] = tc[0] = tcv[0] = tl[0] = tsi[0] = ts4[0] = tl4[0] = 0;
  auto blocks = [](long long threads) { return (int)((threads + kThreads - 1) / kThreads); };
  for (int i = 0; i < n; ++i) {
    const auto& r = h->reps[r0 + i];
    long long L = r.L, H = r.H;
    ts[i + 1] = ts[i] + blocks((H / vec) * L * L);
    tc[i + 1] = tc[i] + 2 * blocks(H * H * H);  // even-origin cubes, then odd-origin cubes
    tcv[i + 1] = tcv[i] + 2 * blocks(H * H * H / r.desc.cvec);
    tl[i + 1] = tl[i] + blocks(r.N);
    tsi[i + 1] = tsi[i] + blocks(6 * r.N);
    ts4[i + 1] = ts4[i] + blocks(6 * r.N / 4);
    tl4[i + 1] = tl4[i] + blocks(r.N / 4);
  }
  int* d;
  if (int rc = dev_alloc(h, (void**)&d, sizeof(int) * 7 * (n + 1))) return rc;
  std::vector<int> all;
  all.insert(all.end(), ts.begin(), ts.end());
  all.insert(all.end(), tc.begin(), tc.end());
  all.insert(all.end(), tl.begin(), tl.end());
  all.insert(all.end(), tsi.begin(), tsi.end());
  all.insert(all.end(), ts4.begin(), ts4.end());
  all.insert(all.end(), tcv.begin(), tcv.end());
  all.insert(all.end(), tl4.begin(), tl4.end());
  CK(cudaMemcpy(d, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
  b.blk_sweep = d;
  b.blk_cube = d + (n + 1);
  b.blk_cell = d + 2 * (n + 1);
  b.blk_site = d + 3 * (n + 1);
  b.blk_site4 = d + 4 * (n + 1);
  b.blk_cubev = d + 5 * (n + 1);
  b.blk_cell4 = d + 6 * (n + 1);
  b.nblk_cell4 = tl4[n];
  b.nblk_cubev = tcv[n];
  b.nblk_site4 = ts4[n];
  b.nblk_sweep = ts[n];
  b.nblk_cube = tc[n];
  b.nblk_cell = tl[n];
  b.nblk_site = tsi[n];
  b.max_L = 0;
  for (int i = r0; i < r1; ++i) b.max_L = std::max(b.max_L, h->reps[i].L);
  b.pdl = 1;
  return 0;
}

// Number of replica groups in effect: the setting, or automatically 4 for batches of 8 or more
// replicas, 2 for 2..7, never more than the replicas.
static int group_count(const cvf_handle* h) {
  const int n = (int)h->reps.size();
  int g = h->group_setting > 0 ? h->group_setting : (n >= 8 ? 4 : (n >= 2 ? 2 : 1));
  return g < n ? g : n;
}

// (Re)builds the group views: consecutive replicas cut where the running cell count crosses
// multiples of total / G, each group with its own block tables, stream and completion event.
static int build_groups(cvf_handle* h) {
  const int G = group_count(h);
  const int n = (int)h->reps.size();
  if (G <= 1) {
    h->groups.clear();
    return 0;
  }
  if ((int)h->groups.size() != G || h->groups_vec != h->b.vec) {
    long long total = 0;
    for (auto& r : h->reps) total += r.N;
    std::vector<int> cut{0};
    long long acc = 0;
    for (int i = 0; i < n && (int)cut.size() < G; ++i) {
      acc += h->reps[i].N;
      const long long target = total * (long long)cut.size() / G;
      if (acc >= target && i + 1 < n && n - (i + 1) >= G - (int)cut.size()) cut.push_back(i + 1);
    }
    cut.push_back(n);
    for (auto& g : h->groups) {
      if (g.s) cudaStreamDestroy(g.s);
      if (g.done) cudaEventDestroy(g.done);
    }
    h->groups.assign(cut.size() - 1, cvf_handle::Group());
    for (size_t k = 0; k + 1 < cut.size(); ++k) {
      auto& g = h->groups[k];
      g.r0 = cut[k];
      g.r1 = cut[k + 1];
      g.b = h->b;
      if (int rc = fill_tables(h, g.r0, g.r1, h->b.vec, g.b)) return rc;
      g.b.pdl = 0;  // the groups' chains run side by side
      g.b.reps = h->b.reps + g.r0;
      g.b.st = h->b.st + g.r0;
      g.b.nrep = g.r1 - g.r0;
      CK(cudaStreamCreateWithFlags(&g.s, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
    }
    if (!h->fork) CK(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
    h->groups_vec = h->b.vec;
  }
  for (auto& g : h->groups) g.b.corr = h->b.corr ? h->b.corr + g.r0 : nullptr;
  return 0;
}

// Scratch of the Wolff step (sized for the largest replica; one replica's step runs at a time).
static int ensure_wolff(cvf_handle* h) {
  if (h->b.wdev.loop) return 0;
  long long nmax = 0;
  for (auto& r : h->reps) nmax = std::max(nmax, r.N);
  int nsm = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device));
  // one block per SM (two fit), so that a kernel on a side branch (the volume chain) never keeps
  // the cooperative grid from being resident; 16 warps per block, one poke each (152 blocks of
  // 512 threads: L=64 step 59 -> 57 ms, L=128 204 -> 189 ms against 304 blocks of 256)
  const int fit = wolff_blocks_per_sm();
  if (fit < 1) return fail(CVF_ECUDA, "the Wolff kernel does not fit on an SM");
  WolffDev& w = h->b.wdev;
  w.grid = nsm;
  w.B = w.grid * (kWolffThreads / 32);
  if (int rc = dev_alloc(h, (void**)&w.chg, (size_t)(6 * nmax) * sizeof(int))) return rc;
  if (int rc = dev_alloc(h, (void**)&w.q, (size_t)(6 * nmax) * sizeof(uint32_t))) return rc;
  if (int rc = dev_alloc(h, (void**)&w.mark, (size_t)((6 * nmax + 31) / 32) * sizeof(uint32_t))) return rc;
  if (int rc = dev_alloc(h, (void**)&w.size, (size_t)w.B * sizeof(int))) return rc;
  if (int rc = dev_alloc(h, (void**)&w.flag, (size_t)w.B * sizeof(int))) return rc;
  if (int rc = dev_alloc(h, (void**)&w.loop, sizeof(WolffLoop))) return rc;
  CK(cudaMemset(w.chg, 0x7f, (size_t)(6 * nmax) * sizeof(int)));  // no poke changes any site
  CK(cudaMemset(w.mark, 0, (size_t)((6 * nmax + 31) / 32) * sizeof(uint32_t)));
  CK(cudaMemset(w.loop, 0, sizeof(WolffLoop)));
  drop_graphs(h);
  return 0;
}

static int ensure_sw(cvf_handle* h) {
  if (h->sw_alloc) return 0;
  for (auto& r : h->reps) {
    size_t NS = (size_t)(6 * r.N);
    int W = (r.L + 31) / 32;
    r.desc.max_cand = 3 * r.L * r.L;  // at most 6N / 2L clusters of size >= 2L
    if (int rc = dev_alloc(h, (void**)&r.desc.label, NS * sizeof(int32_t))) return rc;
    if (int rc = dev_alloc(h, (void**)&r.desc.cellsw, (size_t)r.N * sizeof(uint32_t))) return rc;
    if (int rc = dev_alloc(h, (void**)&r.desc.flip, (size_t)r.N * sizeof(uint32_t))) return rc;
    if (int rc = dev_alloc(h, (void**)&r.desc.swlist, (size_t)r.N * sizeof(uint32_t))) return rc;
    if (int rc = dev_alloc(h, (void**)&r.desc.csize, NS * sizeof(int32_t))) return rc;
    if (int rc = dev_alloc(h, (void**)&r.desc.cand, NS * sizeof(int32_t))) return rc;
    if (int rc = dev_alloc(h, (void**)&r.desc.cover, (size_t)r.desc.max_cand * 3 * W * sizeof(uint32_t))) return rc;
    CK(cudaMemset(r.desc.label, 0, NS * sizeof(int32_t)));
  }
  if (int rc = dev_alloc(h, (void**)&h->blocktop, (size_t)h->b.nblk_site * 2 * sizeof(unsigned long long))) return rc;
  h->sw_alloc = true;
  drop_graphs(h);
  return upload_descs(h);
}

// Cluster step j (of the step's ncl): a Wolff step when the handle's cluster steps are Wolff
// steps, else a Swendsen-Wang step.
static void launch_cluster_step(const BatchDev& b, int jsw, cudaStream_t s, int from_ctr = 0) {
  if (b.wolff) launch_wolff_step(b, s);
  else launch_sw_step(b, jsw, s, from_ctr);
}

// volume: the step's volume move in the cube kernel (false when a side branch runs the chunk's
// volume moves).
// The mapped page-locked records of cvf_observables (one per replica), allocated once.
static int ensure_rec(cvf_handle* h) {
  if (h->rec_pin) return 0;
  const size_t bytes = h->reps.size() * sizeof(SampleRec);
  cudaError_t e = cudaHostAlloc((void**)&h->rec_pin, bytes, cudaHostAllocMapped);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&h->rec_dev, h->rec_pin, 0);
  if (e != cudaSuccess) {
    if (h->rec_pin) cudaFreeHost(h->rec_pin);
    h->rec_pin = nullptr;
    h->rec_dev = nullptr;
    return fail(CVF_ENOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  }
  return 0;
}

static void enqueue_step(cvf_handle* h, int nmet, int ncl, bool volume = true) {
  launch_step_begin(h->b, nmet, ncl, 1, volume ? 1 : 0, h->stream);
  launch_cube_volume(h->b, 1, volume ? 1 : 0, h->stream);
  for (int j = 0; j < nmet; ++j) {
    launch_sweep(h->b, 0, j, h->stream);
    launch_sweep(h->b, 1, j, h->stream);
  }
  for (int j = 0; j < ncl; ++j) launch_cluster_step(h->b, j, h->stream);
}

// Step i of a chunk without records: the kernels take their counters as offsets from ctr (cube
// ctr[1] + i, volume ctr[2] + i, sweep j ctr[0] + i*nmet + j, SW step j ctr[3] + i*ncl + j), and
// one launch_chunk_end after the chunk advances the counters, instead of one k_step_begin per step.
static void enqueue_step_at(const BatchDev& b, cudaStream_t s, int nmet, int ncl, bool volume, int i) {
  launch_cube_volume(b, 1, volume ? 1 : 0, s, i);
  for (int j = 0; j < nmet; ++j) {
    launch_sweep(b, 0, i * nmet + j, s, 1);
    launch_sweep(b, 1, i * nmet + j, s, 1);
  }
  for (int j = 0; j < ncl; ++j) launch_cluster_step(b, i * ncl + j, s, 1);
}

// A Metropolis-only step followed by a recorded measurement: the measurement rides on the last
// colour-1 sweep (slots zeroed by the step's begin kernel), then the slots are summed into the
// last record (appended to the sample stream when keep is set; also written to host_out, mapped
// page-locked memory with one record per replica, when that is given).
static void enqueue_recorded_metropolis_step(cvf_handle* h, int nmet, int keep = 1, SampleRec* host_out = nullptr) {
  launch_step_begin(h->b, nmet, 0, 1, 1, h->stream, 1);
  launch_cube_volume(h->b, 1, 1, h->stream);
  for (int j = 0; j < nmet; ++j) {
    launch_sweep(h->b, 0, j, h->stream);
    if (j + 1 < nmet) launch_sweep(h->b, 1, j, h->stream);
    else launch_sweep_measure(h->b, j, h->stream);
  }
  launch_measure_end(h->b, keep, h->stream, host_out);
}

// One Metropolis-only step of the replicas of view b on stream s, with the recorded measurement
// when record is set (appended to the sample stream when keep is set) and the correlator step
// when corr is set.
static void enqueue_metropolis_on(const BatchDev& b, cudaStream_t s, int nmet, bool record, bool corr, int keep = 1) {
  if (record && nmet > 0) {
    launch_step_begin(b, nmet, 0, 1, 1, s, 1);
    launch_cube_volume(b, 1, 1, s);
    for (int j = 0; j < nmet; ++j) {
      launch_sweep(b, 0, j, s);
      if (j + 1 < nmet) launch_sweep(b, 1, j, s);
      else launch_sweep_measure(b, j, s);
    }
    launch_measure_end(b, keep, s);
  } else {
    launch_step_begin(b, nmet, 0, 1, 1, s);
    launch_cube_volume(b, 1, 1, s);
    for (int j = 0; j < nmet; ++j) {
      launch_sweep(b, 0, j, s);
      launch_sweep(b, 1, j, s);
    }
    if (record) launch_measure(b, keep, s);
  }
  if (corr) launch_corr_step(b, s);
}

static void enqueue_cstats(cvf_handle* h, int record) {
  for (auto& r : h->reps) {
    cudaMemsetAsync(r.desc.csize, 0, (size_t)(6 * r.N) * sizeof(int32_t), h->stream);
    int W = (r.L + 31) / 32;
    cudaMemsetAsync(r.desc.cover, 0, (size_t)r.desc.max_cand * 3 * W * sizeof(uint32_t), h->stream);
  }
  launch_cluster_stats_impl(h->b, h->blocktop, record, h->stream);
}

// Graph of `steps` MC steps; when record is set, step i is followed by a recorded measurement (and
// cluster statistics when ncl > 0) for every i with i % rec_every == 0 (rec_every = 0: the first
// step only), so one graph can hold several intervals of a sampled run. record = 2: the
// measurement of Metropolis-only steps is kept as the replicas' last record only (no sample)
// and, outside replica groups, also written to the mapped records that cvf_observables reads.
static int get_graph(cvf_handle* h, int steps, int nmet, int ncl, int record, cudaGraphExec_t* out,
                     int rec_every = 0) {
  if (!record) rec_every = 0;
  const auto rec_at = [&](int i) { return record && (rec_every > 0 ? i % rec_every == 0 : i == 0); };
  auto key = std::make_tuple(steps, nmet, ncl, record | (rec_every << 2));
  auto it = h->graphs.find(key);
  if (it != h->graphs.end()) {
    *out = it->second;
    return 0;
  }
  if (record == 2)
    if (int rc = ensure_rec(h)) return rc;  // the graph holds the records' device address
  cudaGraph_t g;
  if (h->launch_mode == 1 && ncl == 0 && !h->corr_on && !h->nhb_mode && record != 2) {
    // one persistent launch; a driver that cannot capture a cooperative launch leaves the
    // handle on the per-phase kernels
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t el = launch_run(h->b, steps, nmet, record ? (rec_every > 0 ? rec_every : steps) : 0, h->stream);
    cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    cudaGraphExec_t ex = nullptr;
    if (el == cudaSuccess && ec == cudaSuccess) {
      cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      if (ei == cudaSuccess) {
        h->graphs[key] = ex;
        *out = ex;
        return 0;
      }
    } else if (ec == cudaSuccess) {
      cudaGraphDestroy(g);
    }
    cudaGetLastError();
    h->launch_mode = 0;
  }
  if (ncl == 0 && group_count(h) > 1 && !h->nhb_mode) {
    if (int rc = build_groups(h)) return rc;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    CK(cudaEventRecord(h->fork, h->stream));
    for (auto& gr : h->groups) CK(cudaStreamWaitEvent(gr.s, h->fork, 0));
    for (auto& gr : h->groups) {
      if (record) {
        for (int i = 0; i < steps; ++i) enqueue_metropolis_on(gr.b, gr.s, nmet, rec_at(i), h->corr_on, record == 1);
      } else {
        for (int i = 0; i < steps; ++i) {
          enqueue_step_at(gr.b, gr.s, nmet, 0, true, i);
          if (h->corr_on) launch_corr_step(gr.b, gr.s);
        }
        launch_chunk_end(gr.b, steps, nmet, 0, 1, gr.s);
      }
    }
    for (auto& gr : h->groups) {
      CK(cudaEventRecord(gr.done, gr.s));
      CK(cudaStreamWaitEvent(h->stream, gr.done, 0));
    }
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaGraphExec_t ex;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(CVF_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    h->graphs[key] = ex;
    *out = ex;
    return 0;
  }
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < steps && h->nhb_mode; ++i) {
    // Flag_chessboard = 0: volume move, nmet per-arm sweeps, ncl SW steps, no cube move
    // (GW:1348-1384, GW:1480-1555); the SW steps leave the bond counts as they are, as the
    // reference's cluster update does (GW:2531-2542)
    launch_step_begin(h->b, nmet, ncl, 0, 1, h->stream);
    launch_cube_volume(h->b, 0, 1, h->stream);
    for (int j = 0; j < nmet; ++j) launch_nhb_sweep(h->b, j, h->stream);
    for (int j = 0; j < ncl; ++j) launch_cluster_step(h->b, j, h->stream);
    if (rec_at(i)) {
      launch_nhb_measure(h->b, 1, h->stream);
      if (ncl > 0 && !h->b.wolff) enqueue_cstats(h, 1);
    }
    if (h->corr_on) launch_corr_step(h->b, h->stream);
  }
  // a chunk without records of a handle up to 2^22 cells runs its volume moves on a side branch,
  // beside the cube moves and sweeps, and joins it at the end: there the one-warp FP64 volume
  // move (about 15 us) outlasts the cube moves it otherwise runs beside (L=16 step 16.1 -> 9.8
  // us); on larger lattices the cube moves hide it and the branch only adds its fork and join
  long long cells = 0;
  for (const auto& r : h->reps) cells += r.N;
  const bool side = !h->nhb_mode && !record && steps > 0 && cells <= (1ll << 22);
  if (side) {
    if (!h->vstream) CK(cudaStreamCreateWithFlags(&h->vstream, cudaStreamNonBlocking));
    if (!h->vfork) CK(cudaEventCreateWithFlags(&h->vfork, cudaEventDisableTiming));
    if (!h->vdone) CK(cudaEventCreateWithFlags(&h->vdone, cudaEventDisableTiming));
    CK(cudaEventRecord(h->vfork, h->stream));
    CK(cudaStreamWaitEvent(h->vstream, h->vfork, 0));
    launch_volume_chain(h->b, steps, h->vstream);
    CK(cudaEventRecord(h->vdone, h->vstream));
  }
  // small lattices (every replica up to 2^14 cells, L <= 24): the chunk's cube moves and sweeps
  // as one launch of a thread-block cluster per replica (L=16 step 9.8 -> 8.4 us; at L=32 the
  // eight blocks are too few: 14.4 against 11.4 us per phase)
  int max_cells = 0;
  for (const auto& r : h->reps) max_cells = std::max(max_cells, (int)r.N);
  bool clustered = false;
  if (side && ncl == 0 && nmet > 0 && !h->corr_on && max_cells <= (1 << 14)) {
    clustered = launch_chunk_cluster(h->b, steps, nmet, h->stream) == cudaSuccess;
    if (!clustered) cudaGetLastError();
  }
  // chunks without records take their counters as offsets (one end kernel per chunk)
  const bool offsets = !record && !h->nhb_mode && !clustered && steps > 0;
  for (int i = 0; i < steps && offsets; ++i) {
    enqueue_step_at(h->b, h->stream, nmet, ncl, !side, i);
    if (h->corr_on) launch_corr_step(h->b, h->stream);
  }
  if (offsets) launch_chunk_end(h->b, steps, nmet, ncl, side ? 0 : 1, h->stream);
  for (int i = 0; i < steps && !h->nhb_mode && !clustered && !offsets; ++i) {
    if (side) {
      enqueue_step(h, nmet, ncl, false);
    } else if (rec_at(i) && ncl == 0 && nmet > 0) {
      enqueue_recorded_metropolis_step(h, nmet, record == 1, record == 2 ? h->rec_dev : nullptr);
    } else {
      enqueue_step(h, nmet, ncl);
      if (rec_at(i)) {
        launch_measure(h->b, 1, h->stream);
        if (ncl > 0 && !h->b.wolff) enqueue_cstats(h, 1);
      }
    }
    if (h->corr_on) launch_corr_step(h->b, h->stream);  // after the step's measurement, as GW:1245
  }
  if (side) CK(cudaStreamWaitEvent(h->stream, h->vdone, 0));
  CK(cudaStreamEndCapture(h->stream, &g));
  cudaGraphExec_t ex;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(CVF_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  h->graphs[key] = ex;
  *out = ex;
  return 0;
}

static int check_rep(const cvf_handle* h, int r) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  if (r < 0 || r >= (int)h->reps.size()) return fail(CVF_EINVAL, "replica index out of range");
  return 0;
}

static int read_state(cvf_handle* h, int r, ReplicaState* out) {
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(out, h->b.st + r, sizeof(ReplicaState), cudaMemcpyDeviceToHost));
  return 0;
}

static int check_err(cvf_handle* h) {
  CK(cudaStreamSynchronize(h->stream));
  for (int r = 0; r < (int)h->reps.size(); ++r) {
    int err = 0;
    CK(cudaMemcpy(&err, (char*)(h->b.st + r) + offsetof(ReplicaState, err), sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
      if (err == 3) {
        // the barrier state is stale, and so is the scratch of a Wolff step that stopped midway
        cudaMemset(h->b.gsync, 0, sizeof(GridSync));
        WolffDev& w = h->b.wdev;
        if (w.loop) {
          long long nmax = 0;
          for (auto& rr : h->reps) nmax = std::max(nmax, rr.N);
          cudaMemset(w.chg, 0x7f, (size_t)(6 * nmax) * sizeof(int));
          cudaMemset(w.mark, 0, (size_t)((6 * nmax + 31) / 32) * sizeof(uint32_t));
          cudaMemset(w.loop, 0, sizeof(WolffLoop));
        }
      }
      return fail(CVF_ELIMIT, "device loop limit reached (code " + std::to_string(err) + ") in replica " + std::to_string(r));
    }
  }
  return 0;
}

extern "C" {

const char* cvf_last_error_string(void) { return g_err.c_str(); }
const char* cvf_version(void) { return "cvfbulkwater_gb300 0.1 (sm_103a)"; }

int cvf_batch_create(const cvf_params* params, int n, cvf_handle** out) {
  if (!params || !out || n < 1) return fail(CVF_EINVAL, "null params/out or n_replicas < 1");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    const cvf_params& p = params[i];
    if (p.L < 4 || (p.L & 1)) return fail(CVF_EINVAL, "L must be even and >= 4");
    // L is bounded first so that 6 L^3 is formed without overflow (largest even L: 710)
    if (p.L > 1024 || (long long)p.L * p.L * p.L * 6 >= (1LL << 31))
      return fail(CVF_EINVAL, "L too large (6 L^3 must fit int32)");
    if (p.flag_chessboard != 0 && p.flag_chessboard != 1) return fail(CVF_EINVAL, "Flag_chessboard must be 0 or 1");
    if (p.flag_chessboard != params[0].flag_chessboard)
      return fail(CVF_EINVAL, "all replicas of a handle share Flag_chessboard");
    if (!(p.T > 0.0f)) return fail(CVF_EINVAL, "T must be > 0");
    if (!(p.R_cutoff > 0.0f)) return fail(CVF_EINVAL, "R_cutoff must be > 0");
    if (p.start < 0 || p.start > 2) return fail(CVF_EINVAL, "Flag_config must be 0, 1 or 2");
    if (p.device != params[0].device) return fail(CVF_EINVAL, "all replicas of a handle share one device");
  }
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (params[0].device < 0 || params[0].device >= ndev)
    return fail(CVF_EINVAL, "Device_ID " + std::to_string(params[0].device) + " out of range (" + std::to_string(ndev) + " devices)");
  CK(cudaSetDevice(params[0].device));
  init_device_tables();
  cvf_handle* h = new cvf_handle();
  h->device = params[0].device;
  h->nhb_mode = params[0].flag_chessboard == 0;
  {
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->device) == cudaSuccess && pageable) {
      h->io_capable = true;
      h->io_mode = 1;
    }
  }
  auto bail = [&](int rc) {
    cvf_destroy(h);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(CVF_ECUDA, "cudaStreamCreate failed"));
  h->reps.resize(n);
  std::vector<ReplicaState> st(n);
  for (int i = 0; i < n; ++i) {
    ReplicaHost& r = h->reps[i];
    r.p = params[i];
    r.L = r.p.L;
    r.H = r.L / 2;
    r.N = (long long)r.L * r.L * r.L;
    compute_shells(r.L, r.p.R_cutoff, r.dist, r.freq);
    if ((int)r.dist.size() > kMaxShells) return bail(fail(CVF_EINVAL, "too many vdW shells"));
    r.thr = make_thresholds(r.p.T, r.p.P);
    ReplicaDesc& d = r.desc;
    memset(&d, 0, sizeof(d));
    size_t half_cells = (size_t)(r.N / 2), ncubes = (size_t)r.H * r.H * r.H;
    int rc;
    if ((rc = dev_alloc(h, (void**)&d.cells[0], half_cells * 4)) || (rc = dev_alloc(h, (void**)&d.cells[1], half_cells * 4)) ||
        (rc = dev_alloc(h, (void**)&d.cubes[0], ncubes)) || (rc = dev_alloc(h, (void**)&d.cubes[1], ncubes)))
      return bail(rc);
    if (h->nhb_mode) {
      const size_t nc = (size_t)r.N;
      if ((rc = dev_alloc(h, (void**)&d.eta6, nc)) || (rc = dev_alloc(h, (void**)&d.nhb, nc)) ||
          (rc = dev_alloc(h, (void**)&d.sat, nc)) || (rc = dev_alloc(h, (void**)&d.cnt, nc)))
        return bail(rc);
      if (cudaMemset(d.eta6, 63, nc) != cudaSuccess) return bail(fail(CVF_ECUDA, "eta reset failed"));  // GW:721-724
    }
    float* dd;
    int* df;
    if ((rc = dev_alloc(h, (void**)&dd, kMaxShells * sizeof(float))) || (rc = dev_alloc(h, (void**)&df, kMaxShells * sizeof(int))))
      return bail(rc);
    cudaMemcpy(dd, r.dist.data(), r.dist.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(df, r.freq.data(), r.freq.size() * sizeof(int), cudaMemcpyHostToDevice);
    d.dist = dd;
    d.freq = df;
    d.n_shells = (int)r.dist.size();
    d.L = r.L;
    d.H = r.H;
    auto lg = [](int v) { return (v & (v - 1)) ? -1 : __builtin_ctz((unsigned)v); };
    d.lgL = lg(r.L);
    d.lgH = lg(r.H);
    d.start = r.p.start;
    d.cvec = r.H % 4 == 0 ? 4 : (r.H % 2 == 0 ? 2 : 1);
    d.lgty = -1;
    d.key0 = (uint32_t)((unsigned long long)r.p.seed & 0xffffffffu);
    d.key1 = (uint32_t)((unsigned long long)r.p.seed >> 32);
    d.replica = r.p.replica;
    d.T = r.p.T;
    d.P = r.p.P;
    d.Rc = r.p.R_cutoff;
    d.vdw_shift = vdw_shift(d.Rc);
    d.beta = r.thr.beta;
    d.Jeff = r.thr.Jeff;
    memcpy(d.thr_sweep, r.thr.sweep, sizeof(d.thr_sweep));
    for (int i = 0; i < 33; ++i)
      d.tv[i] = 2u * (uint32_t)(r.thr.sweep[i] >> 16) + ((r.thr.sweep[i] & 0xffffull) != 0) - 1u;
    for (int m = 0; m < 64; ++m) {
      uint32_t v = 0;
      for (int a = 0; a < 6; ++a)
        if ((m >> a) & 1) v |= 7u << (3 * a);
      d.nbmask[m] = v;
    }
    for (int st = 0; st < 9; ++st)
      for (int pp = 0; pp < 8; ++pp) d.eta_tab[st * 8 + pp] = (uint8_t)cube_eta_bits(st, pp);
    memcpy(d.thr_cube, r.thr.cube, sizeof(d.thr_cube));
    memcpy(d.thr_sw, r.thr.sw, sizeof(d.thr_sw));
    d.union_iters = kUnionIters;
    ReplicaState& s = st[i];
    memset(&s, 0, sizeof(s));
    s.r_cell = kRcell0;
    s.volume = (double)r.N * s.r_cell * s.r_cell * s.r_cell;  // GW:481
    s.e_vdw = host_evdw(s.r_cell, r.dist, r.freq, r.p.R_cutoff);
    s.cap_samples = (uint32_t)(r.p.sample_capacity > 0 ? r.p.sample_capacity : 65536);
    s.cap_cstats = s.cap_samples;
    if ((rc = dev_alloc(h, (void**)&s.samples, s.cap_samples * sizeof(SampleRec))) ||
        (rc = dev_alloc(h, (void**)&s.cstats, s.cap_cstats * sizeof(CStatsRec))))
      return bail(rc);
  }
  h->b.nrep = n;
  h->b.barrier_polls = kBarrierPolls;
  int rc;
  if ((rc = dev_alloc(h, (void**)&h->b.reps, n * sizeof(ReplicaDesc))) ||
      (rc = dev_alloc(h, (void**)&h->b.st, n * sizeof(ReplicaState))) ||
      (rc = dev_alloc(h, (void**)&h->b.gsync, sizeof(GridSync))))
    return bail(rc);
  if (cudaMemset(h->b.gsync, 0, sizeof(GridSync)) != cudaSuccess) return bail(fail(CVF_ECUDA, "barrier reset failed"));
  if (cudaMemcpy(h->b.st, st.data(), n * sizeof(ReplicaState), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(CVF_ECUDA, "state upload failed"));
  if ((rc = upload_descs(h)) || (rc = build_tables(h))) return bail(rc);
  // start 1 leaves sigma at zero until cvf_set_config; cubes always start random (GW:700-708)
  launch_init_lattice(h->b, h->stream);
  if (h->nhb_mode) launch_nhb_init(h->b, -1, h->stream);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return bail(fail(CVF_ECUDA, std::string("init: ") + cudaGetErrorString(e)));
  *out = h;
  return 0;
}

int cvf_create(const cvf_params* params, cvf_handle** out) { return cvf_batch_create(params, 1, out); }

int cvf_destroy(cvf_handle* h) {
  if (!h) return 0;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  for (auto& g : h->groups) {
    if (g.s) cudaStreamDestroy(g.s);
    if (g.done) cudaEventDestroy(g.done);
  }
  if (h->fork) cudaEventDestroy(h->fork);
  if (h->vfork) cudaEventDestroy(h->vfork);
  if (h->vdone) cudaEventDestroy(h->vdone);
  if (h->vstream) cudaStreamDestroy(h->vstream);
  for (void* p : h->allocs) cudaFree(p);
  if (h->io_scratch) cudaFree(h->io_scratch);
  if (h->io_bad) cudaFree(h->io_bad);
  if (h->staging) cudaFreeHost(h->staging);
  if (h->rec_pin) cudaFreeHost(h->rec_pin);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return 0;
}

int cvf_num_replicas(const cvf_handle* h) { return h ? (int)h->reps.size() : 0; }

int cvf_set_config(cvf_handle* h, int r, const int* c12, long long n_cells) {
  if (int rc = check_rep(h, r)) return rc;
  h->last_valid = false;
  h->host_rec_valid = false;
  ReplicaHost& R = h->reps[r];
  if (!c12 || n_cells != R.N) return fail(CVF_EINVAL, "cells12 must hold 12 ints for each of the N cells");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  const size_t half = (size_t)(R.N / 2), nc = (size_t)R.H * R.H * R.H;
  if (h->io_mode == 1 && !h->nhb_mode) {
    // pack on the GPU straight from the caller's array into scratch; the lattice changes only
    // when every value is valid
    if (int rc = ensure_io_scratch(h, R)) return rc;
    uint32_t* d0 = (uint32_t*)h->io_scratch;
    uint32_t* d1 = d0 + half;
    uint8_t* eta6 = (uint8_t*)(d1 + half);
    uint8_t* dce = eta6 + R.N;
    uint8_t* dco = dce + nc;
    unsigned long long bad = (unsigned long long)R.N;
    CK(cudaMemcpyAsync(h->io_bad, &bad, sizeof(bad), cudaMemcpyHostToDevice, h->stream));
    CK(launch_pack_config(R.desc, c12, d0, d1, eta6, dce, dco, h->io_bad, h->stream));
    CK(cudaMemcpyAsync(&bad, h->io_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (bad < (unsigned long long)R.N) return fail(CVF_ECONFIG, config_value_error(c12, (long long)bad));
    CK(cudaMemcpyAsync(R.desc.cells[0], d0, half * 4, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(R.desc.cells[1], d1, half * 4, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(R.desc.cubes[0], dce, nc, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(R.desc.cubes[1], dco, nc, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
  }
  if (int rc = ensure_staging(h, R)) return rc;
  uint32_t* c0 = (uint32_t*)h->staging;
  uint32_t* c1 = c0 + half;
  uint8_t* ce = (uint8_t*)(c1 + half);
  uint8_t* co = ce + nc;
  std::string err;
  if (!pack_config(R.L, c12, c0, c1, ce, co, err)) return fail(CVF_ECONFIG, err);
  CK(cudaMemcpyAsync(R.desc.cells[0], c0, half * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cells[1], c1, half * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cubes[0], ce, nc, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cubes[1], co, nc, cudaMemcpyHostToDevice, h->stream));
  if (h->nhb_mode) {
    // Flag_chessboard = 0 keeps the file's eta (GW:751-756) and counts the bonds from it
    // (GW:841-862); the cube states stay unused
    std::vector<uint8_t> e6((size_t)R.N);
    for (long long c = 0; c < R.N; ++c) {
      uint32_t e = 0;
      for (int a = 0; a < 6; ++a) e |= (uint32_t)(c12[c * 12 + 6 + a] & 1) << a;
      e6[c] = (uint8_t)e;
    }
    CK(cudaMemcpyAsync(R.desc.eta6, e6.data(), e6.size(), cudaMemcpyHostToDevice, h->stream));
    launch_nhb_init(h->b, r, h->stream);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(h->stream));  // the staging buffer is reused by the next call
  return 0;
}

int cvf_get_config(cvf_handle* h, int r, int* c12, long long n_cells) {
  if (int rc = check_rep(h, r)) return rc;
  ReplicaHost& R = h->reps[r];
  if (!c12 || n_cells != R.N) return fail(CVF_EINVAL, "cells12 must hold 12 ints for each of the N cells");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  if (h->io_mode == 1 && !h->nhb_mode && ((uintptr_t)c12 & 15u) == 0) {
    // the GPU writes the caller's array in place, block by block with coalesced 16-byte stores,
    // into pages that host threads have made present first
    touch_pages(c12, (size_t)R.N * 12 * sizeof(int));
    CK(launch_unpack_config(R.desc, c12, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
  }
  if (int rc = ensure_staging(h, R)) return rc;
  const size_t half = (size_t)(R.N / 2), nc = (size_t)R.H * R.H * R.H;
  uint32_t* c0 = (uint32_t*)h->staging;
  uint32_t* c1 = c0 + half;
  uint8_t* ce = (uint8_t*)(c1 + half);
  uint8_t* co = ce + nc;
  CK(cudaMemcpyAsync(c0, R.desc.cells[0], half * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(c1, R.desc.cells[1], half * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(ce, R.desc.cubes[0], nc, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(co, R.desc.cubes[1], nc, cudaMemcpyDeviceToHost, h->stream));
  std::vector<uint8_t> e6;
  if (h->nhb_mode) {
    e6.resize((size_t)R.N);
    CK(cudaMemcpyAsync(e6.data(), R.desc.eta6, e6.size(), cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  unpack_config(R.L, c0, c1, ce, co, c12);
  if (h->nhb_mode)  // Flag_chessboard = 0: eta as read (GW:1296-1305 writes active_bond)
    for (long long c = 0; c < R.N; ++c)
      for (int a = 0; a < 6; ++a) c12[c * 12 + 6 + a] = (e6[c] >> a) & 1;
  return 0;
}

// The reference's host arrays s[arm*N + cell] and active_bond[arm*N + cell] (GW:1135-1137 copies
// them to the device, GW:1298 copies s back): checked and packed on the GPU where they lie in host
// memory, or through the cells12 path.
static std::string arms_value_error(const uint8_t* sg, const uint8_t* ab, long long N, long long c) {
  for (int a = 0; a < 6; ++a) {
    const int v = sg[a * N + c], e = ab[a * N + c];
    if (v > 5) return "Unexpected value for spin (" + std::to_string(v) + ") appeared in cell " + std::to_string(c);
    if (e > 1) return "Unexpected value for active_bond (" + std::to_string(e) + ") appeared in cell " + std::to_string(c);
  }
  return "invalid cell " + std::to_string(c);
}

int cvf_set_arms(cvf_handle* h, int r, const unsigned char* sg, const unsigned char* ab, long long n_sites) {
  if (int rc = check_rep(h, r)) return rc;
  ReplicaHost& R = h->reps[r];
  if (!sg || !ab || n_sites != 6 * R.N) return fail(CVF_EINVAL, "s and active_bond must hold 6 N bytes each");
  if (h->io_mode != 1 || h->nhb_mode) {
    std::vector<int> c12((size_t)R.N * 12);
    for (long long c = 0; c < R.N; ++c)
      for (int a = 0; a < 6; ++a) {
        if (sg[a * R.N + c] > 5 || ab[a * R.N + c] > 1) return fail(CVF_ECONFIG, arms_value_error(sg, ab, R.N, c));
        c12[(size_t)c * 12 + a] = sg[a * R.N + c];
        c12[(size_t)c * 12 + 6 + a] = ab[a * R.N + c];
      }
    return cvf_set_config(h, r, c12.data(), R.N);
  }
  h->last_valid = false;
  h->host_rec_valid = false;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  if (int rc = ensure_io_scratch(h, R)) return rc;
  const size_t half = (size_t)(R.N / 2), nc = (size_t)R.H * R.H * R.H;
  uint32_t* d0 = (uint32_t*)h->io_scratch;
  uint32_t* d1 = d0 + half;
  uint8_t* eta6 = (uint8_t*)(d1 + half);
  uint8_t* dce = eta6 + R.N;
  uint8_t* dco = dce + nc;
  unsigned long long bad = (unsigned long long)R.N;
  CK(cudaMemcpyAsync(h->io_bad, &bad, sizeof(bad), cudaMemcpyHostToDevice, h->stream));
  CK(launch_pack_arms(R.desc, sg, ab, d0, d1, eta6, dce, dco, h->io_bad, h->stream));
  CK(cudaMemcpyAsync(&bad, h->io_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (bad < (unsigned long long)R.N) return fail(CVF_ECONFIG, arms_value_error(sg, ab, R.N, (long long)bad));
  CK(cudaMemcpyAsync(R.desc.cells[0], d0, half * 4, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cells[1], d1, half * 4, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cubes[0], dce, nc, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cubes[1], dco, nc, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int cvf_get_arms(cvf_handle* h, int r, unsigned char* sg, unsigned char* ab, long long n_sites) {
  if (int rc = check_rep(h, r)) return rc;
  ReplicaHost& R = h->reps[r];
  if (!sg || !ab || n_sites != 6 * R.N) return fail(CVF_EINVAL, "s and active_bond must hold 6 N bytes each");
  if (h->io_mode != 1 || h->nhb_mode) {
    std::vector<int> c12((size_t)R.N * 12);
    if (int rc = cvf_get_config(h, r, c12.data(), R.N)) return rc;
    for (long long c = 0; c < R.N; ++c)
      for (int a = 0; a < 6; ++a) {
        sg[a * R.N + c] = (unsigned char)c12[(size_t)c * 12 + a];
        ab[a * R.N + c] = (unsigned char)c12[(size_t)c * 12 + 6 + a];
      }
    return 0;
  }
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  // the GPU writes the caller's arrays in place, into pages host threads have made present first
  touch_pages(sg, (size_t)(6 * R.N));
  touch_pages(ab, (size_t)(6 * R.N));
  CK(launch_unpack_arms(R.desc, sg, ab, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

// Packed state of one replica: the colour-0 words, the colour-1 words, the even-origin cube
// states, the odd-origin cube states, exactly as the replica holds them on the device.
static long long packed_bytes(const ReplicaHost& R) { return 4 * R.N + 2LL * R.H * R.H * R.H; }

int cvf_packed_size(const cvf_handle* h, int r, long long* bytes) {
  if (int rc = check_rep(h, r)) return rc;
  if (!bytes) return fail(CVF_EINVAL, "null bytes");
  *bytes = packed_bytes(h->reps[r]);
  return 0;
}

int cvf_get_packed(cvf_handle* h, int r, void* buf, long long bytes) {
  if (int rc = check_rep(h, r)) return rc;
  if (h->nhb_mode) return fail(CVF_EINVAL, "the packed state holds cube states: Flag_chessboard = 1 only");
  ReplicaHost& R = h->reps[r];
  if (!buf || bytes != packed_bytes(R)) return fail(CVF_EINVAL, "packed buffer must hold 4 N + 2 (L/2)^3 bytes");
  CK(cudaSetDevice(h->device));
  const size_t half = (size_t)(R.N / 2), nc = (size_t)R.H * R.H * R.H;
  uint8_t* p = (uint8_t*)buf;
  CK(cudaMemcpyAsync(p, R.desc.cells[0], half * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(p + half * 4, R.desc.cells[1], half * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(p + half * 8, R.desc.cubes[0], nc, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(p + half * 8 + nc, R.desc.cubes[1], nc, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int cvf_set_packed(cvf_handle* h, int r, const void* buf, long long bytes) {
  if (int rc = check_rep(h, r)) return rc;
  if (h->nhb_mode) return fail(CVF_EINVAL, "the packed state holds cube states: Flag_chessboard = 1 only");
  ReplicaHost& R = h->reps[r];
  if (!buf || bytes != packed_bytes(R)) return fail(CVF_EINVAL, "packed buffer must hold 4 N + 2 (L/2)^3 bytes");
  h->last_valid = false;
  h->host_rec_valid = false;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  // copied and checked in scratch first: the lattice changes only when every value is valid
  if (int rc = ensure_io_scratch(h, R)) return rc;
  const size_t half = (size_t)(R.N / 2), nc = (size_t)R.H * R.H * R.H;
  uint8_t* d = (uint8_t*)h->io_scratch;
  CK(cudaMemcpyAsync(d, buf, (size_t)bytes, cudaMemcpyHostToDevice, h->stream));
  const unsigned long long nw = 2 * half, ncb = 2 * nc;
  unsigned long long bad = nw + ncb;
  CK(cudaMemcpyAsync(h->io_bad, &bad, sizeof(bad), cudaMemcpyHostToDevice, h->stream));
  CK(launch_check_packed((const uint32_t*)d, nw, d + 4 * nw, ncb, h->io_bad, h->stream));
  CK(cudaMemcpyAsync(&bad, h->io_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (bad < nw)
    return fail(CVF_ECONFIG, "packed state: word " + std::to_string(bad) + " holds a sigma above 5 or bits above 17");
  if (bad < nw + ncb)
    return fail(CVF_ECONFIG, "packed state: cube byte " + std::to_string(bad - nw) + " is not a state 0..8");
  CK(cudaMemcpyAsync(R.desc.cells[0], d, half * 4, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cells[1], d + half * 4, half * 4, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cubes[0], d + half * 8, nc, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(R.desc.cubes[1], d + half * 8 + nc, nc, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int cvf_set_distances(cvf_handle* h, int r, const float* dist, const int* freq, int n) {
  if (int rc = check_rep(h, r)) return rc;
  if (!dist || !freq || n < 0 || n > kMaxShells) return fail(CVF_EINVAL, "bad distances table");
  ReplicaHost& R = h->reps[r];
  R.dist.assign(dist, dist + n);
  R.freq.assign(freq, freq + n);
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy((void*)R.desc.dist, dist, n * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy((void*)R.desc.freq, freq, n * sizeof(int), cudaMemcpyHostToDevice));
  R.desc.n_shells = n;
  if (int rc = upload_descs(h)) return rc;
  // E_vdW follows the new table (GW:1128 computes it after the table is read)
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  s.e_vdw = host_evdw(s.r_cell, R.dist, R.freq, R.p.R_cutoff);
  CK(cudaMemcpy((char*)(h->b.st + r) + offsetof(ReplicaState, e_vdw), &s.e_vdw, sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

int cvf_get_distances(const cvf_handle* h, int r, float* dist, int* freq, int cap, int* n) {
  if (int rc = check_rep(h, r)) return rc;
  const ReplicaHost& R = h->reps[r];
  int k = (int)R.dist.size();
  if (n) *n = k;
  if (cap < k || !dist || !freq) return fail(CVF_EINVAL, "capacity too small");
  std::copy(R.dist.begin(), R.dist.end(), dist);
  std::copy(R.freq.begin(), R.freq.end(), freq);
  return 0;
}

static int run_impl(cvf_handle* h, int n_steps, int nmet, int ncl, int interval) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  if (n_steps < 0 || nmet < 0 || ncl < 0) return fail(CVF_EINVAL, "negative step counts");
  const bool want_last = h->obs_since_run;
  h->obs_since_run = false;
  CK(cudaSetDevice(h->device));
  if (ncl > 0) {
    if (int rc = h->b.wolff ? ensure_wolff(h) : ensure_sw(h)) return rc;
  }
  if (n_steps == 0) return 0;
  h->last_valid = false;
  h->host_rec_valid = false;
  const int chunk_plain = 32;
  if (interval <= 0) {
    // a Metropolis-only run right after cvf_observables measures its last step (on the step's
    // last colour-1 sweep), and the next cvf_observables reads that record
    const bool last = want_last && ncl == 0 && nmet > 0 && !h->nhb_mode;
    const int plain = last ? n_steps - 1 : n_steps;
    int full = plain / chunk_plain, rem = plain % chunk_plain;
    cudaGraphExec_t g;
    if (full) {
      if (int rc = get_graph(h, chunk_plain, nmet, ncl, 0, &g)) return rc;
      for (int i = 0; i < full; ++i) CK(cudaGraphLaunch(g, h->stream));
    }
    if (rem) {
      if (int rc = get_graph(h, rem, nmet, ncl, 0, &g)) return rc;
      CK(cudaGraphLaunch(g, h->stream));
    }
    if (last) {
      if (int rc = get_graph(h, 1, nmet, 0, 2, &g)) return rc;
      CK(cudaGraphLaunch(g, h->stream));
      h->last_valid = true;
      h->host_rec_valid = group_count(h) <= 1;  // the per-phase capture writes the mapped records
    }
  } else {
    // graphs of m intervals (about 32 steps) while enough steps remain, then single intervals,
    // then the remainder: each graph launch costs a few microseconds on the device
    const int m = interval >= chunk_plain ? 1 : chunk_plain / interval;
    int left = n_steps;
    cudaGraphExec_t g;
    if (m > 1 && left >= m * interval) {
      if (int rc = get_graph(h, m * interval, nmet, ncl, 1, &g, interval)) return rc;
      for (; left >= m * interval; left -= m * interval) CK(cudaGraphLaunch(g, h->stream));
    }
    if (left >= interval) {
      if (int rc = get_graph(h, interval, nmet, ncl, 1, &g)) return rc;
      for (; left >= interval; left -= interval) CK(cudaGraphLaunch(g, h->stream));
    }
    if (left) {
      if (int rc = get_graph(h, left, nmet, ncl, 1, &g)) return rc;
      CK(cudaGraphLaunch(g, h->stream));
    }
    // the run's last step was recorded when it sits on the interval grid
    h->last_valid = !h->nhb_mode && (n_steps - 1) % interval == 0;
  }
  if (ncl > 0 && !h->b.wolff) h->sw_done = true;
  CK(cudaGetLastError());
  return 0;
}

int cvf_run_steps(cvf_handle* h, int n_steps, int nmet, int ncl) { return run_impl(h, n_steps, nmet, ncl, 0); }

int cvf_batch_run(cvf_handle* h, int n_steps, int nmet, int ncl) { return run_impl(h, n_steps, nmet, ncl, 0); }

int cvf_run_sampled(cvf_handle* h, int n_steps, int nmet, int ncl, int interval) {
  if (interval < 1) return fail(CVF_EINVAL, "interval must be >= 1");
  return run_impl(h, n_steps, nmet, ncl, interval);
}

int cvf_synchronize(cvf_handle* h) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  CK(cudaSetDevice(h->device));
  return check_err(h);
}

int cvf_observables(cvf_handle* h, int r, cvf_obs* out) {
  if (int rc = check_rep(h, r)) return rc;
  if (!out) return fail(CVF_EINVAL, "null out");
  CK(cudaSetDevice(h->device));
  h->obs_since_run = true;
  if (int rc = ensure_rec(h)) return rc;
  bool landed = false;  // the record already written to rec_pin[r] by a kernel
  if (h->last_valid && h->host_rec_valid) {
    // the run's measured last step wrote every replica's record into the mapped buffer
    landed = true;
  } else if (h->last_valid) {
    // the record is current: the read kernel writes it, with the replica's current r_cell and
    // volume, straight into the mapped page-locked buffer
    launch_last_read(h->b, h->stream, h->rec_dev + r, r);
    landed = true;
  } else if (h->nhb_mode) {
    if (!h->nhb_read) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      launch_nhb_measure(h->b, 0, h->stream);
      CK(cudaStreamEndCapture(h->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&h->nhb_read, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        h->nhb_read = nullptr;
        return fail(CVF_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      }
    }
    CK(cudaGraphLaunch(h->nhb_read, h->stream));
  } else {
    launch_measure(h->b, 0, h->stream);
    h->last_valid = true;
  }
  // only the 32-byte measurement record crosses to the host, into page-locked memory
  if (!landed)
    CK(cudaMemcpyAsync(h->rec_pin + r, (char*)(h->b.st + r) + offsetof(ReplicaState, last), sizeof(SampleRec),
                       cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const SampleRec last = h->rec_pin[r];
  const ReplicaHost& R = h->reps[r];
  fill_obs(out, last.n_hb2, last.n_sigma, last.r_cell, last.volume,
           host_evdw(last.r_cell, R.dist, R.freq, R.p.R_cutoff), R.N, R.p.P);
  return 0;
}

static void degenerate_cstats(const ReplicaHost& R, cvf_cstats* c) {
  long long NS = 6 * R.N;
  c->largest = NS;
  c->second = 0;
  c->n_percolating = 1;
  c->n_clusters = 1;
  c->sum_size = NS;
  c->sum_size2 = NS * NS;
  c->sum_size2_wrap32 = (long long)(int32_t)(uint32_t)((unsigned long long)NS * (unsigned long long)NS);
  fill_cstats(c);
}

static void from_rec(const CStatsRec& x, cvf_cstats* c) {
  c->largest = x.largest;
  c->second = x.second;
  c->n_percolating = x.n_percolating;
  c->n_clusters = x.n_clusters;
  c->sum_size = x.sum_size;
  c->sum_size2 = x.sum_size2;
  c->sum_size2_wrap32 = x.sum_size2_wrap32;
  fill_cstats(c);
}

int cvf_set_cluster_algorithm(cvf_handle* h, int algorithm) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  if (algorithm != CVF_CLUSTER_SW && algorithm != CVF_CLUSTER_WOLFF) return fail(CVF_EINVAL, "unknown cluster algorithm");
  CK(cudaSetDevice(h->device));
  const int w = algorithm == CVF_CLUSTER_WOLFF ? 1 : 0;
  if (w == h->b.wolff) return 0;
  if (w)
    if (int rc = ensure_wolff(h)) return rc;
  h->b.wolff = w;
  drop_graphs(h);
  return 0;
}

int cvf_wolff_stats(cvf_handle* h, int r, long long* out4) {
  if (int rc = check_rep(h, r)) return rc;
  if (!out4) return fail(CVF_EINVAL, "null out");
  CK(cudaSetDevice(h->device));
  if (int rc = check_err(h)) return rc;
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  out4[0] = s.w_pokes;
  out4[1] = s.w_sum;
  out4[2] = s.w_max;
  out4[3] = (long long)s.wpoke;
  return 0;
}

int cvf_set_wolff_counter(cvf_handle* h, int r, unsigned long long pokes) {
  if (int rc = check_rep(h, r)) return rc;
  CK(cudaSetDevice(h->device));
  if (int rc = check_err(h)) return rc;
  CK(cudaMemcpy((char*)(h->b.st + r) + offsetof(ReplicaState, wpoke), &pokes, sizeof(pokes), cudaMemcpyHostToDevice));
  return 0;
}

int cvf_cluster_stats(cvf_handle* h, int r, cvf_cstats* out) {
  if (int rc = check_rep(h, r)) return rc;
  if (!out) return fail(CVF_EINVAL, "null out");
  if (!h->sw_done) {
    degenerate_cstats(h->reps[r], out);
    return 0;
  }
  CK(cudaSetDevice(h->device));
  enqueue_cstats(h, 0);
  if (int rc = check_err(h)) return rc;
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  from_rec(s.last_cstats, out);
  return 0;
}

int cvf_get_labels(cvf_handle* h, int r, int* labels, long long n) {
  if (int rc = check_rep(h, r)) return rc;
  const ReplicaHost& R = h->reps[r];
  if (!labels || n != 6 * R.N) return fail(CVF_EINVAL, "labels must hold 6N ints");
  if (!h->sw_alloc) {
    memset(labels, 0, (size_t)n * sizeof(int));
    return 0;
  }
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(labels, R.desc.label, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost));
  return 0;
}

int cvf_sample_count(cvf_handle* h, int r, long long* count) {
  if (int rc = check_rep(h, r)) return rc;
  CK(cudaSetDevice(h->device));
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  *count = s.n_samples;
  return 0;
}

int cvf_get_samples(cvf_handle* h, int r, cvf_sample* out, long long max, long long* n_out) {
  if (int rc = check_rep(h, r)) return rc;
  CK(cudaSetDevice(h->device));
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  long long n = std::min<long long>(std::min<long long>(s.n_samples, s.cap_samples), max);
  static_assert(sizeof(cvf_sample) == sizeof(SampleRec), "sample layout");
  if (n > 0) CK(cudaMemcpy(out, s.samples, (size_t)n * sizeof(SampleRec), cudaMemcpyDeviceToHost));
  if (n_out) *n_out = n;
  if (s.n_samples > s.cap_samples) return fail(CVF_ELIMIT, "sample stream overflowed its capacity");
  return 0;
}

int cvf_sample_stream(cvf_handle* h, int r, cvf_sample* out, long long max, long long* n_out) {
  return cvf_get_samples(h, r, out, max, n_out);
}

int cvf_get_cstats_stream(cvf_handle* h, int r, cvf_cstats* out, long long max, long long* n_out) {
  if (int rc = check_rep(h, r)) return rc;
  CK(cudaSetDevice(h->device));
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  long long n = std::min<long long>(std::min<long long>(s.n_cstats, s.cap_cstats), max);
  std::vector<CStatsRec> tmp((size_t)std::max<long long>(n, 0));
  if (n > 0) CK(cudaMemcpy(tmp.data(), s.cstats, (size_t)n * sizeof(CStatsRec), cudaMemcpyDeviceToHost));
  for (long long i = 0; i < n; ++i) from_rec(tmp[(size_t)i], out + i);
  if (n_out) *n_out = n;
  return 0;
}

int cvf_clear_samples(cvf_handle* h) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  uint32_t zero = 0;
  for (int r = 0; r < (int)h->reps.size(); ++r) {
    CK(cudaMemcpy((char*)(h->b.st + r) + offsetof(ReplicaState, n_samples), &zero, 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy((char*)(h->b.st + r) + offsetof(ReplicaState, n_cstats), &zero, 4, cudaMemcpyHostToDevice));
  }
  return 0;
}

int cvf_sample_observables(const cvf_handle* h, int r, const cvf_sample* s, cvf_obs* out) {
  if (int rc = check_rep(h, r)) return rc;
  const ReplicaHost& R = h->reps[r];
  fill_obs(out, s->n_hb2, s->n_sigma, s->r_cell, s->volume, host_evdw(s->r_cell, R.dist, R.freq, R.p.R_cutoff), R.N,
           R.p.P);
  return 0;
}

int cvf_get_state(cvf_handle* h, int r, cvf_state* out) {
  if (int rc = check_rep(h, r)) return rc;
  CK(cudaSetDevice(h->device));
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  out->r_cell = s.r_cell;
  out->volume = s.volume;
  out->e_vdw = s.e_vdw;
  for (int i = 0; i < 4; ++i) out->counters[i] = s.ctr[i];
  return 0;
}

int cvf_set_state(cvf_handle* h, int r, const cvf_state* in) {
  if (int rc = check_rep(h, r)) return rc;
  CK(cudaSetDevice(h->device));
  ReplicaState s;
  if (int rc = read_state(h, r, &s)) return rc;
  const ReplicaHost& R = h->reps[r];
  s.r_cell = in->r_cell;
  s.volume = in->volume;
  s.e_vdw = host_evdw(in->r_cell, R.dist, R.freq, R.p.R_cutoff);
  for (int i = 0; i < 4; ++i) s.ctr[i] = in->counters[i];
  CK(cudaMemcpy(h->b.st + r, &s, sizeof(ReplicaState), cudaMemcpyHostToDevice));
  h->host_rec_valid = false;  // the mapped records hold the old r_cell and volume
  return 0;
}

static void set_row_tile(cvf_handle* h, int lgty) {
  for (auto& r : h->reps) r.desc.lgty = (lgty >= 0 && (1 << lgty) < r.L && r.L % (1 << lgty) == 0) ? lgty : -1;
}

// Device copies of every replica's lattice, cube states and scalar state, restored after timing.
struct StateBackup {
  std::vector<void*> bufs;
  void* st = nullptr;
  ~StateBackup() {
    for (void* p : bufs) cudaFree(p);
    if (st) cudaFree(st);
  }
};

static int backup_state(cvf_handle* h, StateBackup& b, bool cubes_and_scalars) {
  for (auto& r : h->reps) {
    const size_t half = (size_t)(r.N / 2) * sizeof(uint32_t), nc = (size_t)r.H * r.H * r.H;
    const size_t bytes = 2 * half + (cubes_and_scalars ? 2 * nc : 0);
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(CVF_ENOMEM, "autotune: cannot allocate the state backup");
    b.bufs.push_back(p);
    CK(cudaMemcpyAsync(p, r.desc.cells[0], half, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync((char*)p + half, r.desc.cells[1], half, cudaMemcpyDeviceToDevice, h->stream));
    if (cubes_and_scalars) {
      CK(cudaMemcpyAsync((char*)p + 2 * half, r.desc.cubes[0], nc, cudaMemcpyDeviceToDevice, h->stream));
      CK(cudaMemcpyAsync((char*)p + 2 * half + nc, r.desc.cubes[1], nc, cudaMemcpyDeviceToDevice, h->stream));
    }
  }
  if (cubes_and_scalars) {
    const size_t sb = h->reps.size() * sizeof(ReplicaState);
    if (cudaMalloc(&b.st, sb) != cudaSuccess) return fail(CVF_ENOMEM, "autotune: cannot allocate the state backup");
    CK(cudaMemcpyAsync(b.st, h->b.st, sb, cudaMemcpyDeviceToDevice, h->stream));
  }
  return 0;
}

static int restore_state(cvf_handle* h, const StateBackup& b) {
  for (size_t i = 0; i < h->reps.size(); ++i) {
    auto& r = h->reps[i];
    const size_t half = (size_t)(r.N / 2) * sizeof(uint32_t), nc = (size_t)r.H * r.H * r.H;
    char* p = (char*)b.bufs[i];
    CK(cudaMemcpyAsync(r.desc.cells[0], p, half, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(r.desc.cells[1], p + half, half, cudaMemcpyDeviceToDevice, h->stream));
    if (b.st) {
      CK(cudaMemcpyAsync(r.desc.cubes[0], p + 2 * half, nc, cudaMemcpyDeviceToDevice, h->stream));
      CK(cudaMemcpyAsync(r.desc.cubes[1], p + 2 * half + nc, nc, cudaMemcpyDeviceToDevice, h->stream));
    }
  }
  if (b.st) CK(cudaMemcpyAsync(h->b.st, b.st, h->reps.size() * sizeof(ReplicaState), cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return 0;
}

int cvf_autotune(cvf_handle* h, int* vec_out) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  h->last_valid = false;
  h->host_rec_valid = false;
  if (h->nhb_mode) {  // the per-arm sweep of Flag_chessboard = 0 has no tile to choose
    if (vec_out) *vec_out = h->b.vec;
    return 0;
  }
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  std::vector<int> vecs;
  for (int v : {8, 4, 2, 1}) {
    bool ok = true;
    for (auto& r : h->reps) ok = ok && (r.H % v == 0);
    if (ok) vecs.push_back(v);
  }
  // row tiles: plain order (-1) and patches of 8, 4 or 2 rows in y where they differ from it
  std::vector<int> tys{-1};
  for (int lg : {3, 2, 1}) {
    bool ok = true;
    for (auto& r : h->reps) ok = ok && (1 << lg) < r.L && r.L % (1 << lg) == 0;
    if (ok) tys.push_back(lg);
  }
  // save every lattice; the timing sweeps are undone afterwards
  StateBackup saved;
  if (int rc = backup_state(h, saved, false)) return rc;
  // block tables of every tile (block counts depend on the tile)
  std::vector<BatchDev> tabs;
  for (int v : vecs) {
    if (int rc = build_tables(h, v)) return rc;
    tabs.push_back(h->b);
  }
  struct Cand {
    size_t tab;
    int lgty;
    float ms;
  };
  std::vector<Cand> cands;
  for (size_t i = 0; i < vecs.size(); ++i)
    for (int lg : tys) cands.push_back({i, lg, 1e30f});
  // three interleaved rounds, the best time of each candidate: tiles within a few per cent of
  // each other are not told apart by one timing taken after another
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int round = 0; round < 3; ++round) {
    for (auto& c : cands) {
      set_row_tile(h, c.lgty);
      if (int rc = upload_descs(h)) return rc;
      const BatchDev& tb = tabs[c.tab];
      launch_sweep(tb, 0, 0, h->stream);  // warm-up
      launch_sweep(tb, 1, 0, h->stream);
      cudaEventRecord(e0, h->stream);
      for (int i = 0; i < 5; ++i) {
        launch_sweep(tb, 0, i, h->stream);
        launch_sweep(tb, 1, i, h->stream);
      }
      cudaEventRecord(e1, h->stream);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      c.ms = std::min(c.ms, ms);
    }
  }
  size_t bi = 0;
  for (size_t c = 1; c < cands.size(); ++c)
    if (cands[c].ms < cands[bi].ms) bi = c;
  set_row_tile(h, cands[bi].lgty);
  if (int rc = upload_descs(h)) return rc;
  if (int rc = restore_state(h, saved)) return rc;
  // the sweep blocks depend on the tile: keep the chosen tables and drop captured graphs
  drop_graphs(h);
  h->b = tabs[cands[bi].tab];
  // a batch of replicas also chooses its launch mode: 16 Metropolis steps of each mode from the
  // same saved state (lattice, cube states, r_cell, volume, counters), the faster kept
  if (h->reps.size() > 1 && !h->corr_on) {
    StateBackup full;
    if (int rc = backup_state(h, full, true)) return rc;
    float best_ms = 1e30f;
    int best_mode = h->launch_mode;
    for (int mode : {0, 1}) {
      drop_graphs(h);
      h->launch_mode = mode;
      if (int rc = cvf_run_steps(h, 16, 1, 0)) return rc;  // captures the graph, warms up
      if (h->launch_mode != mode) continue;                  // the cooperative capture fell back
      float ms = 1e30f;
      for (int round = 0; round < 2; ++round) {
        cudaEventRecord(e0, h->stream);
        if (int rc = cvf_run_steps(h, 16, 1, 0)) return rc;
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float m = 0.f;
        cudaEventElapsedTime(&m, e0, e1);
        ms = std::min(ms, m);
      }
      if (int rc = check_err(h)) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best_mode = mode;
      }
    }
    drop_graphs(h);
    h->launch_mode = best_mode;
    h->last_valid = false;
    h->host_rec_valid = false;
    if (int rc = restore_state(h, full)) return rc;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (vec_out) *vec_out = vecs.empty() ? h->b.vec : vecs[cands[bi].tab];
  return 0;
}

int cvf_set_row_tile(cvf_handle* h, int lgty) {
  if (!h || lgty < -1 || lgty > 8) return fail(CVF_EINVAL, "row tile must be -1 (plain) or log2 of 2..256 rows");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  set_row_tile(h, lgty);
  drop_graphs(h);
  return upload_descs(h);
}

int cvf_get_tuning(const cvf_handle* h, int* tile, int* lgty, int* launch_mode) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  if (tile) *tile = h->b.vec;
  if (lgty) *lgty = h->reps.empty() ? -1 : h->reps[0].desc.lgty;
  if (launch_mode) *launch_mode = h->launch_mode;
  return 0;
}

int cvf_set_sweep_tile(cvf_handle* h, int vec, int* vec_out) {
  if (!h || !(vec == 1 || vec == 2 || vec == 4 || vec == 8)) return fail(CVF_EINVAL, "tile must be 1, 2, 4 or 8");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  drop_graphs(h);
  if (int rc = build_tables(h, vec)) return rc;
  if (vec_out) *vec_out = h->b.vec;
  return 0;
}

int cvf_get_stream(cvf_handle* h, void** stream) {
  if (!h || !stream) return fail(CVF_EINVAL, "null handle/out");
  *stream = (void*)h->stream;
  return 0;
}

int cvf_profile_launch(cvf_handle* h, int kind, int n) {
  if (!h || n < 0 || kind < 0 || kind > 3) return fail(CVF_EINVAL, "bad profile request");
  h->last_valid = false;
  h->host_rec_valid = false;
  if (h->nhb_mode) return fail(CVF_EINVAL, "kernel profiling covers the Flag_chessboard = 1 kernels");
  CK(cudaSetDevice(h->device));
  for (int i = 0; i < n; ++i) {
    switch (kind) {
      case 0:
        launch_sweep(h->b, 0, i, h->stream);
        launch_sweep(h->b, 1, i, h->stream);
        break;
      case 1:
        launch_step_begin(h->b, 0, 0, 1, 0, h->stream);
        launch_cube_volume(h->b, 1, 0, h->stream);
        break;
      case 2:
        launch_step_begin(h->b, 0, 0, 0, 1, h->stream);
        launch_cube_volume(h->b, 0, 1, h->stream);
        break;
      default: launch_measure(h->b, 0, h->stream); break;
    }
  }
  CK(cudaGetLastError());
  return 0;
}

int cvf_set_launch_mode(cvf_handle* h, int mode) {
  if (!h || mode < 0 || mode > 1) return fail(CVF_EINVAL, "launch mode must be 0 or 1");
  if (mode == h->launch_mode) return 0;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  drop_graphs(h);
  h->launch_mode = mode;
  return 0;
}

int cvf_set_io_mode(cvf_handle* h, int mode) {
  if (!h || mode < 0 || mode > 1) return fail(CVF_EINVAL, "io mode must be 0 or 1");
  if (mode == 1 && !h->io_capable)
    return fail(CVF_EINVAL, "this GPU cannot access pageable host memory (cudaDevAttrPageableMemoryAccess = 0)");
  h->io_mode = mode;
  return 0;
}

int cvf_get_io_mode(const cvf_handle* h, int* mode) {
  if (!h || !mode) return fail(CVF_EINVAL, "null handle/out");
  *mode = h->io_mode;
  return 0;
}

int cvf_set_wait_limits(cvf_handle* h, long long barrier_polls, long long union_iters) {
  if (!h) return fail(CVF_EINVAL, "null handle");
  const unsigned int polls = barrier_polls < 0 ? kBarrierPolls
                             : (unsigned int)std::min<long long>(barrier_polls, (long long)kBarrierPolls);
  const uint32_t iters = union_iters < 0 ? kUnionIters
                         : (uint32_t)std::min<long long>(union_iters, (long long)kUnionIters);
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  for (auto& r : h->reps) r.desc.union_iters = iters;
  if (int rc = upload_descs(h)) return rc;
  // the persistent kernel takes the bound as a by-value argument of its captured launch
  h->b.barrier_polls = polls;
  for (auto& g : h->groups) g.b.barrier_polls = polls;
  drop_graphs(h);
  return 0;
}

int cvf_get_launch_mode(const cvf_handle* h, int* mode) {
  if (!h || !mode) return fail(CVF_EINVAL, "null handle/out");
  *mode = h->launch_mode;
  return 0;
}

int cvf_set_replica_groups(cvf_handle* h, int groups) {
  if (!h || groups < 0) return fail(CVF_EINVAL, "groups must be >= 0 (0 = automatic)");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  h->group_setting = groups;
  drop_graphs(h);
  return 0;
}

int cvf_get_replica_groups(const cvf_handle* h, int* groups) {
  if (!h || !groups) return fail(CVF_EINVAL, "null handle/out");
  *groups = group_count(h);
  return 0;
}

int cvf_set_correlation(cvf_handle* h, int enable) {
  if (!h || enable < 0 || enable > 1) return fail(CVF_EINVAL, "enable must be 0 or 1");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  const int n = (int)h->reps.size();
  if (enable) {
    if (!h->b.corr) {
      if (int rc = dev_alloc(h, (void**)&h->b.corr, (size_t)n * sizeof(CorrState))) return rc;
    }
    std::vector<CorrState> init((size_t)n, corr_initial());
    CK(cudaMemcpy(h->b.corr, init.data(), init.size() * sizeof(CorrState), cudaMemcpyHostToDevice));
  }
  h->corr_on = enable != 0;
  drop_graphs(h);
  return 0;
}

// GW:3078-3112 (evaluate with norm = 1) on a copy of the replica's correlator.
int cvf_get_correlation(cvf_handle* h, int r, double* t, double* f, int cap, int* n_out) {
  if (int rc = check_rep(h, r)) return rc;
  if (!t || !f || !n_out || cap < 0) return fail(CVF_EINVAL, "null arrays/count");
  if (!h->b.corr) return fail(CVF_EINVAL, "the correlation was never enabled (cvf_set_correlation)");
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  CorrState C;
  CK(cudaMemcpy(&C, h->b.corr + r, sizeof(C), cudaMemcpyDeviceToHost));
  const int dmin = kCorrP / kCorrM;
  double aux = 0;
  if (C.ncorrelation[0][0] > 0) aux = (C.accval / C.ncorrelation[0][0]) * (C.accval / C.ncorrelation[0][0]);
  int im = 0;
  auto put = [&](double tt, double ff) {
    if (im < cap) {
      t[im] = tt;
      f[im] = ff;
    }
    ++im;
  };
  for (int i = 0; i < kCorrP; ++i)
    if (C.ncorrelation[0][i] > 0) put((double)i, C.correlation[0][i] / C.ncorrelation[0][i] - aux);
  for (int k = 1; k < C.kmax; ++k)
    for (int i = dmin; i < kCorrP; ++i)
      if (C.ncorrelation[k][i] > 0) put(i * pow((double)kCorrM, k), C.correlation[k][i] / C.ncorrelation[k][i] - aux);
  *n_out = im;
  if (im > cap) return fail(CVF_EINVAL, "capacity too small for the correlation points");
  return 0;
}

int cvf_run_statistics(cvf_handle* h, cvf_run_stats* out, int n_out) {
  if (!h || !out) return fail(CVF_EINVAL, "null handle/out");
  const int n = (int)h->reps.size();
  if (n_out < n) return fail(CVF_EINVAL, "out must hold one row per replica");
  CK(cudaSetDevice(h->device));
  if (!h->stats) {
    if (int rc = dev_alloc(h, (void**)&h->stats, (size_t)n * 14 * sizeof(double))) return rc;
  }
  CK(launch_run_stats(h->b, h->stats, h->stream));
  std::vector<double> v((size_t)n * 14);
  CK(cudaMemcpyAsync(v.data(), h->stats, v.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int r = 0; r < n; ++r) {
    cvf_run_stats& o = out[r];
    o.L = h->reps[r].L;
    o.P = (double)h->reps[r].p.P;
    o.T = (double)h->reps[r].p.T;
    for (int k = 0; k < 6; ++k) {
      o.mean[k] = v[r * 14 + k];
      o.var[k] = v[r * 14 + 6 + k];
    }
    o.n = (long long)v[r * 14 + 12];
  }
  for (int r = 0; r < n; ++r)
    if (v[r * 14 + 13] > v[r * 14 + 12])
      return fail(CVF_ELIMIT, "sample stream of replica " + std::to_string(r) +
                                  " overflowed its capacity: statistics of the stored samples only");
  return 0;
}

int cvf_get_thresholds(const cvf_handle* h, int r, unsigned long long* out) {
  if (int rc = check_rep(h, r)) return rc;
  const Thresholds& t = h->reps[r].thr;
  memcpy(out, t.sweep, sizeof(t.sweep));
  memcpy(out + 33, t.cube, sizeof(t.cube));
  memcpy(out + 42, t.sw, sizeof(t.sw));
  return 0;
}

}  // extern "C"
