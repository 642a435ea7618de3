// Device-side data structures of the GB300 CVF engine and the launch entry points that the
// host engine (cvf_engine.cpp) calls. One ReplicaDesc per lattice (a plain run is a batch of
// one replica); kernels map blocks to replicas through a prefix table of block counts.
//
// HBM layout of one replica with edge L (N = L^3, H = L/2):
//   cells[c]  : uint32[H*L*L]  colour-c cells ((x+y+z)&1 == c), word (x>>1) + H*(y + L*z),
//                              bits 3a..3a+2 = sigma_a
//   cubes[0]  : uint8[H^3]     states of the cubes with all-even origins (2a,2b,2c),
//                              index a + H*(b + H*c)
//   cubes[1]  : uint8[H^3]     states of the cubes with all-odd origins (2a+1,2b+1,2c+1)
//   label     : int32[6N]      Swendsen-Wang site labels, site = arm*N + x + L*(y + L*z)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cvf {

struct ReplicaDesc {
  uint32_t* cells[2];
  uint8_t* cubes[2];
  // Swendsen-Wang work arrays (null until the first SW step)
  int32_t* label;     // 6N parents / labels
  uint32_t* cellsw;   // N: bits 0..2 = active x+, y+, z+ cluster bonds; bits 3+3a..5+3a = the
                      // smallest arm of arm a's in-cell component (its in-cell root)
  uint32_t* flip;     // N: bits 3a..3a+2 = shift of the cluster whose root is arm site a of the cell
  uint32_t* swlist;   // N: cells with a hydrogen-bond link in the current SW step (ReplicaState.swq of them)
  int32_t* csize;     // 6N: cluster sizes by root
  int32_t* cand;      // 6N: percolation candidate id by root (-1 none)
  uint32_t* cover;    // max_cand * 3 * W: coordinate coverage bitmaps
  int max_cand;       // capacity of cover
  uint32_t union_iters;  // attempts of one Swendsen-Wang union before it gives up (error code 1)
  // Flag_chessboard = 0 (null otherwise): eta of every cell as 6 bits, the bond count of every
  // cell, and the greedy measurement's work arrays (per cell: bits 0..2 its matched x+, y+, z+
  // bonds and bit 3 set when 5 or more of its arms are matched; the counts of those cells);
  // cells indexed x + L*(y + L*z)
  uint8_t* eta6;
  uint8_t* nhb;
  uint8_t* sat;
  uint8_t* cnt;
  // vdW shells (device copies)
  const float* dist;
  const int* freq;
  int n_shells;
  int L, H;
  int lgL, lgH;       // log2 of L and H when they are powers of two, else -1
  int start;          // Flag_config of the replica (0 disordered, 1 from file, 2 ordered)
  int cvec;           // consecutive cubes per thread in the cube move: 4, 2 or 1 (divides H)
  int lgty;           // sweep row order: -1 rows by y then z; else tiles of 2^lgty rows in y, the
                      // tiles' rows by z (a block covers a patch of y and z rows); set by autotune
  uint32_t key0, key1, replica;
  float T, P, Rc;
  double vdw_shift;   // vdw_shift(Rc), computed once on the host
  double beta, Jeff;
  unsigned long long thr_sweep[33];  // U < T, T in [0, 2^32]; index (dN_hb+1)*11 + dN_s+5
  // Sweep fast-path tables, read through L1 by the kernels:
  //   tv[i] = 2*(T_i >> 16) + ((T_i & 0xffff) != 0) - 1 for the same index i (modulo 2^32);
  //   eta_tab[s*8 + p] = eta bits a cube in state s gives its vertex at offset p;
  //   nbmask[m] = 7 in every 3-bit field a whose bit a of the 6-bit mask m is set.
  uint32_t tv[33];
  uint32_t nbmask[64];
  uint8_t eta_tab[72];
  unsigned long long thr_cube[9];    // index dN_hb+4
  unsigned long long thr_sw[2];      // hydrogen-bond link, intra-cell link
};

// One measurement: exact integer counts plus the volume degree of freedom.
struct SampleRec {
  long long n_hb2;    // sum over bonds of delta*(eta_i + eta_j) = 2 N_hb
  long long n_sigma;  // sum over cells of sum_{a<b} delta(sigma_a, sigma_b)
  double r_cell;
  double volume;
};

// Cluster statistics of the last SW labelling (GW:2677-2780), exact integers.
struct CStatsRec {
  long long largest, second, n_percolating, n_clusters;
  long long sum_size, sum_size2, sum_size2_wrap32;
};

struct ReplicaState {
  double r_cell, volume, e_vdw;
  uint32_t ctr[4];  // next move counters: sweep, cube, volume, SW
  uint32_t cur[4];  // counters used by the moves of the current step
  unsigned long long acc_hb2, acc_ns;
  unsigned long long acc_slot[2][32];  // measurement partial sums, slot = block % 32
  unsigned long long top2[2];
  unsigned long long ncl, sum2, sum2w, nperc;
  int ncand;
  int err;  // nonzero: a bounded loop gave up (1 SW union, 2 candidate overflow, 3 grid barrier)
  uint32_t swq;  // entries of the replica's SW worklist (k_sw_local appends, k_sw_finish clears)
  uint32_t n_samples, n_cstats;
  uint32_t cap_samples, cap_cstats;
  SampleRec* samples;   // device sample stream
  CStatsRec* cstats;    // device cluster-statistics stream
  SampleRec last;
  CStatsRec last_cstats;
  // Wolff cluster steps: the poke counter (the random streams of poke P) and the last step's
  // pokes, summed cluster sizes and largest cluster
  unsigned long long wpoke;
  long long w_pokes, w_sum, w_max;
};

// Multi-tau correlator of one replica (GW:165-181, GW:2983-3128): kCorrLevels levels of kCorrP
// channels, kCorrM values averaged into the next level. It correlates, step by step, the
// fraction of arms in the most populated sigma value (GW:1245-1272); hist collects the counts of
// the step being added.
constexpr int kCorrLevels = 32, kCorrP = 16, kCorrM = 2;
constexpr int kCorrSlots = 32;
struct CorrState {
  double shift[kCorrLevels][kCorrP];
  double correlation[kCorrLevels][kCorrP];
  long long ncorrelation[kCorrLevels][kCorrP];
  double accumulator[kCorrLevels];
  int naccumulator[kCorrLevels];
  int insertindex[kCorrLevels];
  int kmax;
  int pad;
  double accval;
  unsigned long long hist[kCorrSlots][6];  // per-block sums spread over slots (block % kCorrSlots)
};

// Grid barrier state of the persistent step kernel (zeroed at creation and after an error).
struct GridSync {
  unsigned int count;  // blocks arrived at the current barrier
  unsigned int gen;    // barrier generation
  int err;             // nonzero: a barrier wait gave up
  unsigned int ticket; // block tickets handed out in the current launch
};

// Scratch of the Wolff step kernel (one replica at a time; sized for the largest replica) and
// its loop state. A batch is one poke per warp of the cooperative grid of kWolffThreads-thread
// blocks.
constexpr int kWolffThreads = 512;
struct WolffLoop {
  unsigned long long p0;  // first poke of the current batch
  long long done, pokes, maxs;  // sites flipped, pokes and largest cluster of the step so far
  int commit;             // pokes of the batch committed (the prefix before the first conflict)
  int big;                // the batch's first poke outgrew its warp: the whole grid grows it
  unsigned int tail, level0, level1;  // global queue of the grid-wide growth
};
struct WolffDev {
  int* chg;            // [6N] per site: smallest poke of the batch whose cluster changes it
  uint32_t* q;         // [6N] sites of a cluster grown by the whole grid
  uint32_t* mark;      // [6N/32] bitmask of those sites
  int* size;           // [B] cluster size per poke of the batch
  int* flag;           // [B] 1: examines a cell an earlier poke changes, 2: outgrew its warp
  WolffLoop* loop;
  int B;               // pokes per batch (warps of the grid)
  int grid;            // blocks of the cooperative launch
};

// ------------------------------------------------------------- launch entry points
struct BatchDev {
  ReplicaDesc* reps;    // device array [nrep]
  ReplicaState* st;     // device array [nrep]
  int nrep;
  int vec;              // cells per thread in the sweep (1, 2, 4 or 8; divides every H)
  int* blk_sweep;       // device prefix tables (nrep+1) of blocks per replica
  int* blk_cube;        // one thread per cube (initialisation)
  int* blk_cubev;       // one thread per cvec consecutive cubes (cube move)
  int* blk_cell;        // one thread per cell
  int* blk_site;        // one thread per arm site (6N)
  int* blk_site4;       // one thread per 4 arm sites
  int* blk_cell4;       // one thread per 4 cell words
  int nblk_sweep, nblk_cube, nblk_cubev, nblk_cell, nblk_site, nblk_site4, nblk_cell4;
  int max_L;            // largest edge among the replicas
  int pdl;              // launch the step's kernels as programmatic dependents (launch_pdl)
  GridSync* gsync;      // device barrier state of the persistent step kernel
  unsigned int barrier_polls;  // polls of one grid-barrier wait before it gives up (error code 3)
  CorrState* corr;      // device array [nrep] of correlators (null until enabled)
  int wolff;            // cluster steps are Wolff steps (GW:2199-2357) instead of Swendsen-Wang
  WolffDev wdev;        // its scratch (allocated when enabled)
};

constexpr int kThreads = 256;
// Default bounds of the device waits: a grid-barrier wait polls at most kBarrierPolls times
// (with a short sleep between polls, about a second in all), a union gives up after
// kUnionIters attempts. cvf_set_wait_limits lowers them for tests of the error path.
constexpr unsigned int kBarrierPolls = 1u << 24;
constexpr unsigned int kUnionIters = 1u << 24;

void launch_init_lattice(const BatchDev& b, cudaStream_t s);
void init_device_tables();
// Snapshot of this step's move counters; zero_slots also clears the measurement slots of a
// step whose measurement is fused into its last colour-1 sweep.
void launch_step_begin(const BatchDev& b, int nmet, int ncl, int do_cube, int do_volume, cudaStream_t s,
                       int zero_slots = 0);
// Cube moves of all replicas (do_cubes) and, in extra blocks of the same launch, their volume
// moves (do_volume): the two moves are independent, so the volume move hides under the cubes.
// soff >= 0: the step is step soff of a chunk whose kernels take their counters as offsets from
// ctr (no k_step_begin; launch_chunk_end after the chunk); soff < 0: the counters of cur.
void launch_cube_volume(const BatchDev& b, int do_cubes, int do_volume, cudaStream_t s, int soff = -1);
void launch_chunk_end(const BatchDev& b, int steps, int nmet, int ncl, int do_volume, cudaStream_t s);
void launch_volume_chain(const BatchDev& b, int steps, cudaStream_t s);
cudaError_t launch_chunk_cluster(const BatchDev& b, int steps, int nmet, cudaStream_t s);
// jsweep: the sweep's offset from cur[0], or with from_ctr from ctr[0] (step i, sweep j of a chunk:
// i * nmet + j).
void launch_sweep(const BatchDev& b, int colour, int jsweep, cudaStream_t s, int from_ctr = 0);
// Replica host_r's last record with its current r_cell and volume into host_out (mapped
// page-locked host memory).
void launch_last_read(const BatchDev& b, cudaStream_t s, SampleRec* host_out, int host_r);
void launch_measure(const BatchDev& b, int record, cudaStream_t s);
// Colour-1 sweep jsweep fused with the measurement of the step (slots zeroed by the step's
// launch_step_begin), and the summation of the slots into the replica's record.
void launch_sweep_measure(const BatchDev& b, int jsweep, cudaStream_t s);
void launch_measure_end(const BatchDev& b, int record, cudaStream_t s, SampleRec* host_out = nullptr);
// Persistent cooperative launch of nsteps Metropolis steps (cube + volume move, nmet sweeps) of
// every replica, with a recorded measurement after every step s with s % interval == 0 when
// interval > 0. Same lattice, counters and samples as the per-phase kernels.
cudaError_t launch_run(const BatchDev& b, int nsteps, int nmet, int interval, cudaStream_t s);
void launch_sw_step(const BatchDev& b, int jsw, cudaStream_t s, int from_ctr = 0);
// One Wolff cluster step of every replica (one cooperative launch per replica): pokes until the
// flipped clusters add up to 6N sites.
cudaError_t launch_wolff_step(const BatchDev& b, cudaStream_t s);
// Blocks per SM of the Wolff kernel (the cooperative grid is this times the SM count).
int wolff_blocks_per_sm();
// Flag_chessboard = 0: bond counts from the lattice and eta6 (GW:841-862; one replica, or all for
// only_replica < 0), one Metropolis sweep
// (12 launches: colour 0 arms 0..5, colour 1 arms 0..5) and the measurement with the greedy
// bond count of GW:2064-2099 into the replicas' last record (appended to the sample stream when
// record is set).
void launch_nhb_init(const BatchDev& b, int only_replica, cudaStream_t s);
void launch_nhb_sweep(const BatchDev& b, int jsweep, cudaStream_t s);
void launch_nhb_measure(const BatchDev& b, int record, cudaStream_t s);
// One correlator step of every replica: the sigma histogram of the lattice, then the add of the
// most-populated fraction to the replica's correlator (b.corr must be allocated).
cudaError_t launch_corr_step(const BatchDev& b, cudaStream_t s);
// Run statistics of every replica from its sample stream: out[r*14 + k] = mean of data.out
// column k (k < 6: energy, enthalpy, volume, N_hb, m, r_cell), variance of column k - 6
// (6 <= k < 12), number of stored samples used (k = 12), number recorded (k = 13).
cudaError_t launch_run_stats(const BatchDev& b, double* out, cudaStream_t s);
// Configuration upload read in place from host memory (the GPU must access pageable host
// memory): pack the caller's cells12 array into cells0/cells1/ce/co (scratch buffers of the
// replica's sizes; eta6 holds N bytes; *bad must start at N and receives the smallest invalid
// cell).
cudaError_t launch_pack_config(const ReplicaDesc& R, const int* c12, uint32_t* cells0, uint32_t* cells1, uint8_t* eta6,
                               uint8_t* ce, uint8_t* co, unsigned long long* bad, cudaStream_t s);
// cvf_get_config on the GPU: the replica's lattice written as cells12 straight into the caller's
// 16-byte aligned array in host memory (pageable-memory access); cudaErrorInvalidValue if the
// array is not aligned.
cudaError_t launch_unpack_config(const ReplicaDesc& R, int* c12, cudaStream_t s);
// The same from / to the reference's host arrays s[arm*N + cell] and active_bond[arm*N + cell]
// (one byte each) where they lie in host memory; *bad as for launch_pack_config.
cudaError_t launch_pack_arms(const ReplicaDesc& R, const uint8_t* s, const uint8_t* active_bond, uint32_t* cells0,
                             uint32_t* cells1, uint8_t* eta6, uint8_t* ce, uint8_t* co, unsigned long long* bad,
                             cudaStream_t st);
cudaError_t launch_unpack_arms(const ReplicaDesc& R, uint8_t* s, uint8_t* active_bond, cudaStream_t st);
// Checks a packed state on the device (sigma fields in 0..5 with bits 18..31 zero in the nw
// words, cube states 0..8 in the ncb bytes); *bad must start at nw + ncb and receives the smallest
// offending index (cube byte i at nw + i).
cudaError_t launch_check_packed(const uint32_t* words, unsigned long long nw, const uint8_t* cubes,
                                unsigned long long ncb, unsigned long long* bad, cudaStream_t s);
void launch_cluster_stats_impl(const BatchDev& b, unsigned long long* blocktop, int record, cudaStream_t s);

#ifdef __CUDACC__
// Programmatic dependent launch: kernels of a chain are launched so that the next one may start
// while the previous drains (launch_pdl). Each lets its dependents launch as soon as its own
// blocks have started (pdl_trigger), and waits for the previous kernel's completion and memory
// (pdl_wait) before it touches the state that kernel writes; what it does before the wait reads
// only the descriptors and tables, which no kernel writes. Without a programmatic predecessor
// the wait returns at once.
// Bit 2 of every 3-bit field of x (18 bits) set where the field is not zero: adding 3 to the
// field's low two bits carries into bit 2 unless they are zero (no carry leaves the field).
__device__ __forceinline__ uint32_t nonzero_fields(uint32_t x) {
  return (((x & 0x1b6dbu) + 0x1b6dbu) | x) & 0x24924u;
}

// sum_{a<b} delta(sigma_a, sigma_b) of one cell: with Z_k the number of arms a equal to arm
// (a+k) mod 6, every unordered pair is counted by Z_k and Z_{6-k}, so the sum is
// Z_1 + Z_2 + Z_3/2, and Z_3/2 counts arms 0..2 against 3..5. The rotations by 3k bits are
// windows of the word repeated above itself (w * (1 + 2^18), 18 + 14 bits).
__device__ __forceinline__ uint32_t sigma_pairs(uint32_t w) {
  w &= 0x3ffffu;
  const uint32_t ww = w * 0x40001u;
  const uint32_t x1 = (w ^ (ww >> 3)) & 0x3ffffu, x2 = (w ^ (ww >> 6)) & 0x3ffffu, x3 = (w ^ (ww >> 9)) & 0x1ffu;
  return 15u - (uint32_t)(__popc(nonzero_fields(x1)) + __popc(nonzero_fields(x2)) + __popc(nonzero_fields(x3)));
}

__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// With pdl = 0 (chains captured on parallel branches, where blocks waiting early would hold SM
// slots that the other branches' kernels could use) the launch is an ordinary one.
template <typename... P, typename... A>
static inline void launch_pdl(void (*kernel)(P...), dim3 grid, cudaStream_t s, int pdl, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, ((P)args)...);
}

// Grid-wide barrier of a cooperative (co-resident) launch: the last block to arrive bumps the
// generation word the others poll. A wait gives up after max_polls looks (with a short sleep
// between them, so the default bound is about a second), sets gs->err and the replica's error
// code 3, and every block then leaves; returns false once any block has given up.
static __device__ __noinline__ bool grid_barrier(GridSync* gs, ReplicaState* st0, unsigned int max_polls) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &gs->gen;
    volatile int* err = &gs->err;
    const unsigned int g = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(&gs->count, 1u) == gridDim.x - 1) {
      atomicExch(&gs->count, 0u);
      __threadfence();
      atomicAdd(&gs->gen, 1u);
    } else {
      // the bound is checked before each look at the generation word, so a bound of 0 makes
      // every block that has to wait give up
      for (unsigned int polls = 0;; ++polls) {
        if (*err != 0 || polls >= max_polls) {
          ok = 0;
          break;
        }
        if (*gen != g) break;
        __nanosleep(64);
      }
      if (!ok && atomicExch(&gs->err, 1) == 0) atomicExch(&st0->err, 3);
    }
    __threadfence();
    s_ok = ok && *err == 0;
  }
  __syncthreads();
  return s_ok != 0;
}
#endif

}  // namespace cvf
