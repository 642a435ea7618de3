/*
 * CPU oracle for the CVF bulk-water NPT Monte Carlo step (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference program SOURCE/gpu_water3D.cu of
 * lcoronas/CVFBulkWater, written in the reference's own data layout (one byte per
 * arm variable, struct-of-arrays by arm: s[arm*N + cell], eta[arm*N + cell]) and
 * driven by the engine's counter-based Philox4x32-10 random streams, so that the
 * GPU engine must reproduce its lattice, labels and integer counts bit for bit.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it,
 * and only as the checker or as the timed CPU baseline.  The GPU product never links it.
 *
 * Parity pins: Philox known-answer vectors (Salmon et al., SC'11 / Random123), the
 * reference's SOURCE/distances file (exact), SOURCE/input_config (chessboard invariants
 * and round trip) and the statistics of SOURCE/data.out (L=32, T=0.815, P=0.45).
 */
#ifndef CVF_ORACLE_H
#define CVF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle oracle_t;

typedef struct {
    int64_t n_hb2;     /* sum over bonds of delta*(eta_i + eta_j): twice N_hb (GW:2037-2063) */
    int64_t n_sigma;   /* sum over cells of sum_{a<b} delta(s_a, s_b) (GW:2101-2103) */
    double r_cell, volume, e_vdw;
    double n_hb, energy, enthalpy, v_total, m;
} oracle_obs_t;

typedef struct {
    int64_t largest, second, n_percolating, n_clusters;
    int64_t sum_size, sum_size2, sum_size2_wrap32;
} oracle_cstats_t;

/* Philox4x32-10 block: out[4] = philox(ctr = {c0,c1,c2,c3}, key = {k0,k1}). */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Own FP64 exp/log (Cody-Waite reduction + Taylor / atanh series), used by the volume move. */
double oracle_exp(double x);
double oracle_log(double x);

/* vdW shell table (GW:865-932, distance_PBC GW:1323-1337): distinct minimum-image
 * distances d < Rc from cell 0 in first-encounter order, freq = (count/2)*N.
 * Returns the number of shells (<= cap). */
int oracle_distances(int L, float Rc, float* dist, int* freq, int cap);

/* start: 0 random, 1 caller sets config, 2 ordered (GW:730-833). */
oracle_t* oracle_create(int L, float T, float P, int64_t seed, float Rc, uint32_t replica, int start);
/* flag_chessboard = 0: the nhb<=4 mode (every eta 1, no cube moves, bond counts per cell). */
oracle_t* oracle_create_mode(int L, float T, float P, int64_t seed, float Rc, uint32_t replica, int start,
                             int flag_chessboard);
/* Flag_chessboard = 0: the per-cell bond counts that drive the dynamics (N bytes). */
void oracle_get_nhb(const oracle_t* o, uint8_t* nhb);
void oracle_destroy(oracle_t* o);
void oracle_set_threads(oracle_t* o, int n_threads);

/* 12 ints per cell (config.out order, GW:1296-1305). set_config infers cube states from
 * eta with the reference's decision tree (GW:3314-3371) and rewrites eta from them. */
int oracle_set_config(oracle_t* o, const int32_t* cells12, int64_t n_cells);
int oracle_get_config(const oracle_t* o, int32_t* cells12, int64_t n_cells);
void oracle_get_cubes(const oracle_t* o, uint8_t* even_states, uint8_t* odd_states);

/* Moves. Each advances its own counter. */
void oracle_cube_move(oracle_t* o);
void oracle_volume_move(oracle_t* o);
void oracle_sweep(oracle_t* o);
void oracle_sw_step(oracle_t* o);
/* One Wolff cluster step (GW:2199-2357): pokes until their clusters add up to 6N sites. */
void oracle_wolff_step(oracle_t* o);
/* Cluster steps of oracle_step are Wolff steps when on (default: Swendsen-Wang). */
void oracle_set_wolff(oracle_t* o, int on);
/* The last Wolff step: pokes, summed cluster sizes, largest cluster; then the poke counter. */
void oracle_wolff_stats(const oracle_t* o, int64_t out[4]);
/* One MC step in the reference's order (GW:1346-1733): cube move, volume move,
 * n_metropolis sweeps, n_cluster Swendsen-Wang steps. */
void oracle_step(oracle_t* o, int n_metropolis, int n_cluster);

void oracle_measure(const oracle_t* o, oracle_obs_t* out);
void oracle_cluster_stats(const oracle_t* o, oracle_cstats_t* out);
/* 6N labels (site = arm*N + cell), canonical minimum site id; all zero before any SW step. */
void oracle_get_labels(const oracle_t* o, int32_t* labels);

void oracle_get_state(const oracle_t* o, double* r_cell, double* volume, double* e_vdw, uint32_t counters[4]);
void oracle_set_state(oracle_t* o, double r_cell, double volume, const uint32_t counters[4]);
/* thresholds: sweep[33] (idx (dhb+1)*11+dns+5), cube[9] (idx dhb+4), sw[2] (hb, sigma). Values in [0, 2^32]. */
void oracle_get_thresholds(const oracle_t* o, uint64_t* sweep33, uint64_t* cube9, uint64_t* sw2);
double oracle_evdw(const oracle_t* o, double r);

#ifdef __cplusplus
}
#endif
#endif
