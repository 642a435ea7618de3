/*
 * cvf.h -- C ABI of the GB300 engine for the Coronas-Vilanova-Franzese (CVF) bulk-water
 * lattice model (NPT Monte Carlo), a drop-in for the hot path of SOURCE/gpu_water3D.cu of
 * lcoronas/CVFBulkWater ("GW" below).
 *
 * The reference has no library API: its boundary is the executable contract of gpu_water3D
 * (input_data / input_config / distances in, data.out / cluster.out / config.out / water3D.log
 * out) and, inside it, the seam MonteCarlo_Step() (GW:52-53, GW:1346-1733). Each entry point
 * below names the reference code it replaces. Plain C types only; the library allocates and
 * owns all device memory; callers pass host buffers with explicit sizes.
 *
 * Conventions
 *  - Every function returns 0 on success or a negative CVF_E* code; cvf_last_error_string()
 *    describes the last failure of the calling thread.
 *  - A handle holds one or more replicas (independent lattices) on one GPU and one CUDA stream.
 *    A handle is not thread-safe; different handles may be used concurrently.
 *  - Cells are numbered cell = x + L*(y + L*z); arms a = 0..5 are x+, x-, y+, y-, z+, z-
 *    (GW:1936-1962). Arm sites for cluster labels are site = a*N + cell.
 *  - "cells12" arrays hold 12 ints per cell in config.out order: sigma_0..sigma_5 then
 *    eta_0..eta_5 (GW:1296-1305).
 */
#ifndef CVF_H
#define CVF_H

#ifdef __cplusplus
extern "C" {
#endif

#define CVF_OK 0
#define CVF_EINVAL -1     /* invalid argument (sizes, ranges, unsupported flag) */
#define CVF_ECUDA -2      /* CUDA runtime error */
#define CVF_ELIMIT -3     /* a bounded device loop gave up (error word set by a kernel) */
#define CVF_ENOMEM -4     /* device allocation failed */
#define CVF_ECONFIG -5    /* malformed configuration (cells12 values out of range) */

typedef struct cvf_handle cvf_handle;

/* Run parameters of one replica. Mirrors the 14 lines of input_data (GW:293-386) that the
 * hot path consumes, plus the lattice edge that the reference fixes at compile time (GW:35-37). */
typedef struct cvf_params {
  int L;                 /* lattice edge: even, >= 4 */
  float T;               /* temperature, internal units (read as float, GW:304) */
  float P;               /* pressure, internal units (read as float, GW:298) */
  long long seed;        /* Philox key (GW:310 reads it as %ld) */
  float R_cutoff;        /* vdW cut-off radius in lattice units (GW:352) */
  int start;             /* Flag_config: 0 disordered, 1 caller loads cells12, 2 ordered (GW:730-833) */
  int flag_chessboard;   /* 1: eta moves by 2x2x2 cubes (GW:639-724). 0: the nhb<=4 compatibility
                            mode (GW:721-724, GW:1964-2007, GW:2064-2099): eta fixed (all 1, or
                            as set by cvf_set_config), no cube move; SW steps leave the bond
                            counts as they are, as in the reference. All replicas of a handle
                            share the value. */
  unsigned int replica;  /* replica id, counter word 3 of every Philox draw */
  int device;            /* CUDA device ordinal (Device_ID, GW:457-468) */
  int sample_capacity;   /* samples kept on the device per replica; 0 selects 65536 */
} cvf_params;

/* One measurement (GW:2014-2160). Integer counts are exact. */
typedef struct cvf_obs {
  long long n_hb2;       /* sum over bonds of delta*(eta_i+eta_j) = 2*N_hb */
  long long n_sigma;     /* sum over cells of sum_{a<b} delta(sigma_a, sigma_b) */
  double r_cell;         /* lattice spacing */
  double volume;         /* N r^3 tracked by the volume move */
  double e_vdw;          /* vdW lattice energy at r_cell */
  double n_hb;           /* n_hb2 / 2 (data.out column 5) */
  double energy;         /* e = E_vdW - J_hb N_hb - J_sigma N_sigma (column 2) */
  double enthalpy;       /* h = e + P v (column 3) */
  double v_total;        /* v = N r^3 + v_hb N_hb (column 4) */
  double m;              /* N_sigma / (15 N) (column 6) */
} cvf_obs;

/* Cluster statistics of the last Swendsen-Wang labelling (GW:2677-2780). */
typedef struct cvf_cstats {
  long long largest, second, n_percolating, n_clusters;
  long long sum_size;          /* always 6N */
  long long sum_size2;         /* exact sum of s^2 */
  long long sum_size2_wrap32;  /* sum of s*s wrapped to int32 as in GW:2697 */
  double mean;                 /* sum_size / n_clusters */
  double variance;             /* exact sum_size2/n - mean^2 */
  float mean_ref;              /* cluster.out column 5, the reference's float formula */
  float variance_ref;          /* cluster.out column 6, incl. the int32 wrap of s*s */
} cvf_cstats;

/* One recorded sample of the device sample stream. */
typedef struct cvf_sample {
  long long n_hb2, n_sigma;
  double r_cell, volume;
} cvf_sample;

/* Mutable scalar state (for exact checkpoint/resume; the reference restarts r_cell at
 * 1.0001 and loses its RNG state, GW:150). counters: sweep, cube, volume, SW moves done. */
typedef struct cvf_state {
  double r_cell, volume, e_vdw;
  unsigned int counters[4];
} cvf_state;

const char* cvf_last_error_string(void);
const char* cvf_version(void);

/* Replaces main()'s set-up GW:440-1170 for one lattice. */
int cvf_create(const cvf_params* params, cvf_handle** out);
/* n independent replicas (own L, T, P, seed, replica id) stepped together in one set of
 * launches captured in a CUDA graph. No reference counterpart: the reference runs one lattice
 * per process. */
int cvf_batch_create(const cvf_params* params, int n_replicas, cvf_handle** out);
int cvf_destroy(cvf_handle* h);
int cvf_num_replicas(const cvf_handle* h);

/* Replaces the input_config reader GW:730-811 and gpu_Chessboard_set_state GW:3314-3371:
 * cube states are inferred from eta with the reference's decision tree and every eta is
 * rewritten from them (what the reference's first cube move does). */
int cvf_set_config(cvf_handle* h, int replica, const int* cells12, long long n_cells);
/* Replaces the config.out writer GW:1296-1305. */
int cvf_get_config(cvf_handle* h, int replica, int* cells12, long long n_cells);
/* The reference's own host arrays: s[arm*N + cell] (sigma 0..5) and active_bond[arm*N + cell]
 * (eta 0/1), one byte each, 6N bytes per array (replaces the cudaMemcpy of s and active_bond to
 * dev_s / dev_active_bond, GW:1135-1137, and of dev_s back to s, GW:1298). Same checks and
 * cube-state inference as cvf_set_config (CVF_ECONFIG names the first bad cell; the lattice is
 * then unchanged); cvf_get_arms writes eta as the cubes give it. 12 bytes per cell cross the
 * host link instead of the 48 of cells12. */
int cvf_set_arms(cvf_handle* h, int replica, const unsigned char* s, const unsigned char* active_bond,
                 long long n_sites);
int cvf_get_arms(cvf_handle* h, int replica, unsigned char* s, unsigned char* active_bond, long long n_sites);

/* Packed state of a replica, for checkpoint and resume without the text format: the engine's own
 * device layout, 4 N + 2 (L/2)^3 bytes (about 4.25 bytes per cell against the 48 of cells12):
 *   bytes [0, 2N):          the N/2 colour-0 words ((x+y+z) even), word (x>>1) + (L/2)*(y + L*z),
 *                           bits 3a..3a+2 = sigma_a (arm a), bits 18..31 zero;
 *   bytes [2N, 4N):         the N/2 colour-1 words, the same layout;
 *   then (L/2)^3 bytes:     states 0..8 of the cubes with even origins (2i, 2j, 2k), index
 *                           i + (L/2)*(j + (L/2)*k);
 *   then (L/2)^3 bytes:     the cubes with odd origins (2i+1, 2j+1, 2k+1), the same index.
 * eta of every arm follows from the two cube states (the cube numbering of SOURCE/chessboard.h).
 * cvf_set_packed checks every value (CVF_ECONFIG, lattice unchanged) before it loads the state;
 * with cvf_set_state it resumes a chain exactly. Flag_chessboard = 1 only. No reference
 * counterpart (the reference's only state file is config.out, GW:1296-1305). */
int cvf_packed_size(const cvf_handle* h, int replica, long long* bytes);
int cvf_get_packed(cvf_handle* h, int replica, void* buf, long long bytes);
int cvf_set_packed(cvf_handle* h, int replica, const void* buf, long long bytes);

/* vdW shell table (GW:865-989). The library computes it at create (Flag_distances=0);
 * set_distances loads a table read from a distances file (Flag_distances=1). */
int cvf_set_distances(cvf_handle* h, int replica, const float* dist, const int* freq, int n);
int cvf_get_distances(const cvf_handle* h, int replica, float* dist, int* freq, int cap, int* n);

/* Replaces n_steps calls of MonteCarlo_Step (GW:1346-1733) for every replica: one cube move,
 * one volume move, n_metropolis checkerboard sweeps, n_cluster Swendsen-Wang steps per step. */
int cvf_run_steps(cvf_handle* h, int n_steps, int n_metropolis, int n_cluster);
/* The same for a handle made by cvf_batch_create (every replica steps; one graph per chunk). */
int cvf_batch_run(cvf_handle* h, int n_steps, int n_metropolis, int n_cluster);
/* The production loop GW:1204-1244: after step i (0-based within the call) with
 * i % interval == 0, a sample (and, when n_cluster > 0, a cluster-statistics record) is
 * appended on the device. No host synchronisation inside. */
int cvf_run_sampled(cvf_handle* h, int n_steps, int n_metropolis, int n_cluster, int interval);
int cvf_synchronize(cvf_handle* h);

/* Replaces measure() GW:2014-2160 for the current configuration. A Metropolis-only
 * cvf_run_steps that follows a cvf_observables call measures its last step on the way, so the
 * next call reads that record (synchronising with the stream) instead of measuring again. */
int cvf_observables(cvf_handle* h, int replica, cvf_obs* out);
/* Replaces print_cluster_statistics() GW:2677-2721 for the current labels. Before any SW step
 * the labels are all zero (one cluster of 6N sites), as in the reference's cluster.out. */
int cvf_cluster_stats(cvf_handle* h, int replica, cvf_cstats* out);
/* 6N canonical labels (minimum site id of the cluster), site = arm*N + cell (GW:2365-2529). */
int cvf_get_labels(cvf_handle* h, int replica, int* labels, long long n_sites);

/* Device sample stream: number of samples recorded since the last clear, and a copy. */
int cvf_sample_count(cvf_handle* h, int replica, long long* count);
int cvf_get_samples(cvf_handle* h, int replica, cvf_sample* out, long long max, long long* n_out);
/* cvf_get_samples under the name of the sample-stream export: the (N_hb2, N_sigma, r_cell, V)
 * records, from which cvf_sample_observables gives E, V, N_hb and N_sigma. */
int cvf_sample_stream(cvf_handle* h, int replica, cvf_sample* out, long long max, long long* n_out);
int cvf_get_cstats_stream(cvf_handle* h, int replica, cvf_cstats* out, long long max, long long* n_out);
int cvf_clear_samples(cvf_handle* h);
/* Observables of one sample (host FP64 formulas of GW:2138-2159). */
int cvf_sample_observables(const cvf_handle* h, int replica, const cvf_sample* s, cvf_obs* out);

int cvf_get_state(cvf_handle* h, int replica, cvf_state* out);
int cvf_set_state(cvf_handle* h, int replica, const cvf_state* in);

/* Acceptance thresholds of a replica (U < T with U a uniform 32-bit integer):
 * out[0..32] sweep, index (dN_hb+1)*11 + dN_sigma+5; out[33..41] cube, index dN_hb+4;
 * out[42] SW hydrogen-bond link; out[43] SW intra-cell link. */
int cvf_get_thresholds(const cvf_handle* h, int replica, unsigned long long* out44);

/* ---- File formats of the executable contract (host only, no GPU needed) ---- */

/* The 14 positional "name value" lines of input_data (GW:293-386), plus an optional 15th line
 * "Lattice_Size L" (the reference fixes L = 32 at compile time, GW:35-37; default 32). */
typedef struct cvf_input {
  float P, T;
  long long seed;
  int metropolis_steps, cluster_steps, equilibrium_steps, sampling_steps, sampling_interval;
  float R_cutoff;
  int flag_config, flag_distances, flag_correlation, flag_chessboard, device_id;
  int L;
} cvf_input;
/* Returns 0, or CVF_EINVAL with the reference's message (e.g. "Error [Pressure]: Can't read
 * input file") in cvf_last_error_string(). */
int cvf_read_input_data(const char* path, cvf_input* out);
/* input_config reader with the reference's checks (GW:730-800): 12 ints per line, sigma in
 * 0..5, eta in 0..1, exactly n_cells rows. */
int cvf_read_config_file(const char* path, int* cells12, long long n_cells);
/* config.out writer (GW:1296-1305). */
int cvf_write_config_file(const char* path, const int* cells12, long long n_cells);
/* distances file writer / reader (GW:917-985): header "L L L", then "%f %d" per shell. */
int cvf_write_distances_file(const char* path, int L, const float* dist, const int* freq, int n);
int cvf_read_distances_file(const char* path, int L, float* dist, int* freq, int cap, int* n);
/* One data.out line (GW:2159) and one cluster.out line (GW:2717-2718), NUL-terminated, with the
 * trailing newline. Return the length or CVF_EINVAL if cap is too small. */
int cvf_format_data_line(char* buf, int cap, int t, const cvf_obs* o);
int cvf_format_cluster_line(char* buf, int cap, int t, const cvf_cstats* c);

/* ---------------------------------------------------------------- 2-D histogram reweighting
 * Binned (E, rho) histogram reweighting of HistogramReweighting/
 * histogram_reweighting_mixed_paramSI_norm_x.f90 ("F90") on the GPU. Inputs per sample: the
 * enthalpy per cell h = H/N and the density rho = N/V in internal units (F90:160-165) and its run;
 * per run the internal T and P. The F90's literals are single precision (plain gfortran), and so
 * are its constants here. cvf_h2d_create converts every sample to SI energy (kJ/mol) and density
 * (kg/m^3) (F90:155-181), bins them as the F90 does (F90:220-279; n_bin2D scales with bin_factor)
 * and runs `steps` iterations of the F90's constants (F90:446-472), failing with CVF_ELIMIT when
 * they have not converged to 1e-7; cvf_h2d_set_constants takes them as given instead (the F90's
 * Constants_L file, F90:380-440). cvf_h2d_reweight gives the normalised distribution on the
 * n_bin2D x n_bin2D grid at (T, P) (internal units; grid may be NULL) and the Binder cumulants of
 * E and rho (F90:737-759, F90:2610-2662); cvf_h2d_mixed then the distribution of the mixed order
 * parameter at angle alpha, M = sin(alpha) E + cos(alpha) rho, normalised and mapped as the F90
 * does (F90:1383-1620; n_bin_mixed points, x and q may be NULL) and its Binder cumulant
 * (F90:2580-2608); cvf_h2d_mixed_batch the same for n angles (x, q: n x n_bin_mixed).
 * cvf_h2d_ising compares a mixed distribution, abscissae scaled by B, with the 2-D and 3-D Ising
 * order-parameter distributions (ConfrontIsing, ZeroTest, HeightTest, F90:2042-2254): out[6] =
 * liu_2D, liu_3D, kl_2D, kl_3D, zero, height. cvf_h2d_scan runs the F90's search (F90:732-891)
 * over the given pressures (outer), temperatures and angles (inner): tp_rows n_P x n_T x
 * {binder_e, binder_rho}; rows n_P x n_T x n_S x {binder_m, liu_2D, liu_3D, kl_2D, kl_3D, zero,
 * height}; best[5] the row of the smallest liu_2D, liu_3D, zero, height, zero + height (-1: none). */
typedef struct cvf_h2d cvf_h2d;
int cvf_h2d_create(int device, const double* h, const double* rho, const int* run_of, long long n, const double* That,
                   const double* Phat, int n_runs, int L, double bin_factor, int steps, cvf_h2d** out);
int cvf_h2d_info(const cvf_h2d* H, int* n_bin2d, int* n_bin_mixed, double* Emin, double* dE, double* Dmin, double* dD,
                 double* ctes);
int cvf_h2d_set_constants(cvf_h2d* H, const double* ctes);
int cvf_h2d_reweight(cvf_h2d* H, double T_hat, double P_hat, double* grid, double* binder_e, double* binder_rho);
int cvf_h2d_mixed(cvf_h2d* H, double alpha, double* x, double* q, double* binder_m);
int cvf_h2d_mixed_batch(cvf_h2d* H, const double* alpha, int n, double* x, double* q, double* binder_m);
int cvf_h2d_ising(const double* x, const double* q, int n_bin_mixed, double B, double* out);
int cvf_h2d_scan(cvf_h2d* H, const double* T_hat, int n_T, const double* P_hat, int n_P, const double* S, int n_S,
                 double B, double* tp_rows, double* rows, long long* best);
int cvf_h2d_destroy(cvf_h2d* H);

/* Multi-tau autocorrelation (Flag_correlation = 1; GW:1245-1313, GW:2983-3128). Enabling (1)
 * resets every replica's correlator; from then on every step of cvf_run_steps /
 * cvf_run_sampled adds, per replica, the fraction of arms in the most populated sigma value
 * (counted on the GPU) to a correlator of 32 levels x 16 channels that averages pairs into the
 * next level, kept on the device. 0 stops adding (the state stays readable). Steps run with
 * launch mode 1 fall back to per-phase launches while the correlation is on.
 * cvf_get_correlation evaluates replica r's correlator as the reference does at the end of a
 * run (GW:3078-3112, mean squared subtracted): n_out points (t, f), up to cap of them written;
 * correlation.dat prints t and f / f[0]. No other reference counterpart. */
int cvf_set_correlation(cvf_handle* h, int enable);
int cvf_get_correlation(cvf_handle* h, int r, double* t, double* f, int cap, int* n_out);

/* Cluster algorithm of the n_cluster steps of cvf_run_steps / cvf_run_sampled (replaces the
 * compile-time choice GW:195-213 #define WOLFF vs GW:214 #define SWENDSEN_WANG):
 *   CVF_CLUSTER_SW (default): one Swendsen-Wang step (GW:2365-2542);
 *   CVF_CLUSTER_WOLFF: one Wolff step, cluster_step() GW:2199-2357: pokes (a random seed site
 *   and a shift in 1..5) until the flipped clusters add up to 6N sites, over the Swendsen-Wang
 *   bonds. Wolff steps leave no labels: cvf_cluster_stats then reports the all-singleton
 *   statistics of a handle without Swendsen-Wang steps, and cvf_wolff_stats the step's own
 *   figures. */
#define CVF_CLUSTER_SW 0
#define CVF_CLUSTER_WOLFF 1
int cvf_set_cluster_algorithm(cvf_handle* h, int algorithm);
/* The last Wolff step of replica r (GW:2205-2222 num_clusters, cumm_cluster_size,
 * tmp_max_cluster_size): out4 = {pokes, summed cluster sizes, largest cluster, poke counter}.
 * The poke counter numbers the Wolff random streams; cvf_set_wolff_counter restores it when a
 * run resumes from a checkpoint. */
int cvf_wolff_stats(cvf_handle* h, int r, long long* out4);
int cvf_set_wolff_counter(cvf_handle* h, int r, unsigned long long pokes);

/* ---------------------------------------------------------------- isobar analysis
 * The reference's thermodynamic analysis (CVF_ThermodynamicAnalysis/) on the engine's results.
 *
 * Run statistics (replaces the awk stage of TA/script_analisi.sh:35): for every replica of the
 * handle, the mean and the variance <x^2> - <x>^2 of the six data.out columns (GW:2138-2159:
 * energy, enthalpy, volume, N_hb, m = N_sigma/(15N), r_cell) over the samples recorded so far,
 * computed on the GPU from the on-device sample stream; only the statistics cross to the host.
 * out holds n_out >= number of replicas rows. When a replica recorded more samples than its
 * capacity, every row still holds the statistics of the stored (first) samples and the call
 * returns CVF_ELIMIT, as cvf_get_samples does. */
typedef struct cvf_run_stats {
  int L;
  double P, T;
  double mean[6]; /* energy, enthalpy, volume, n_hb, m, r_cell */
  double var[6];  /* <x^2> - <x>^2, the formula of the reference's awk stage */
  long long n;    /* samples */
} cvf_run_stats;
int cvf_run_statistics(cvf_handle* h, cvf_run_stats* out, int n_out);

/* One isobar point per run (TA/calculadora.sh:41-61): per-cell means and errors
 * sqrt(3 var / n) / N (the factor 3 is the reference's fixed 1 + 2 tau / dt), density N / <V>,
 * N_hb / 2N, the cooperative fraction m, r_cell with error sqrt(var / n), and the fluctuation
 * estimates C_P = var(H) / (T^2 N) and K_T = var(V) / (T <V>). */
typedef struct cvf_isobar_point {
  double T;
  double energy, energy_err, enthalpy, enthalpy_err, volume, volume_err, density, density_err;
  double nhb, nhb_err, ncoop, ncoop_err, rcell, rcell_err;
  double cp_fluc, kt_fluc;
} cvf_isobar_point;
int cvf_isobar_point_from_stats(const cvf_run_stats* s, cvf_isobar_point* out);

/* SI units of an isobar point at pressure P (internal units), TA/conversor.sh: T in K
 * (conversor.sh:2-3,20), density in kg/m^3 (:6-7,20), enthalpy in kJ/mol as h*Hs + Hi*T with
 * error err*Hi (:11-12,24, kept as the reference writes it), energy E = H - 18 (P Ps + Pi) / rho
 * with the reference's error expression (:76), C_P = cp*CPs + CPi (:8-9,32; the reference's
 * error column is empty, 0), N_hb and m unchanged (:28). */
typedef struct cvf_isobar_point_si {
  double T_K, density, density_err, enthalpy, enthalpy_err, energy, energy_err, cp_fluc, cp_fluc_err;
  double nhb, nhb_err, ncoop, ncoop_err;
} cvf_isobar_point_si;
int cvf_isobar_point_to_si(const cvf_isobar_point* p, double P, cvf_isobar_point_si* out);

/* Thermal expansion alpha_P = (1/V) dV/dT along an isobar by finite differences
 * (TA/AlphaPderivate.c:56-134): the m points (T, V, variance of V, samples) in any order are
 * sorted by T; central differences inside, one-sided at the ends; the error combines the
 * sample error sqrt(3 var / n), the third-derivative term and the neighbours' errors. Like the
 * reference, only the points 2 .. m-3 of the sorted list are returned (m_out = max(m - 4, 0));
 * the outputs hold m entries. The differentiable reweighting (cvf_reweight_*) gives alpha_P,
 * K_T and C_P without finite differences. */
int cvf_alpha_p_derivative(const double* T, const double* V, const double* V2, const long long* n, int m,
                           double* T_out, double* ap_out, double* err_out, int* m_out);
/* CPderivate.c:56-124: C_P = dH/dT of one isobar (H = <H>/N, H2 = var(H)/N^2, n samples per
 * point, any order); writes the points 2 .. m-3 of the T-sorted isobar as the reference does. */
int cvf_cp_derivative(const double* T, const double* H, const double* H2, const long long* n, int m, double* T_out,
                      double* cp_out, double* err_out, int* m_out);
/* KTderivate.c:345-563: K_T = d ln(rho) / dP along isotherms for m points (T in K, P in MPa, rho
 * and its error in kg/m^3, any order), KT and EKT per point, -10 where the reference gives no
 * value (gas, rho < 500; a point alone on its isotherm; a gas neighbour). */
int cvf_kt_derivative(const double* T, const double* P, const double* rho, const double* Erho, int m, double* KT,
                      double* EKT);

/* Autotuner: times the checkerboard sweep kernel on this handle's replicas for every supported
 * cells-per-thread tile (1, 2, 4 or 8 consecutive colour cells: 32-, 64-, 128- or 2x128-bit
 * accesses) and every row order (rows by y then z, or patches of 8, 4 or 2 rows in y across
 * several z planes per block) and keeps the fastest pair; a batch of several replicas then times
 * 16 Metropolis steps in each launch mode (cvf_set_launch_mode) and keeps the faster. The lattices
 * (and for the mode choice the cube states, r_cell, volume and counters) are saved before and
 * restored after, so the Markov chains are unchanged (the tile and row order only change the
 * thread mapping, never the result). vec_out may be NULL; cvf_get_tuning reports all three
 * choices. No reference counterpart. */
int cvf_autotune(cvf_handle* h, int* vec_out);
/* Row order of the sweep set by hand: -1 rows by y then z, k >= 1 patches of 2^k rows in y (used
 * where 2^k divides L and is below it). cvf_get_tuning: the tile, the row order and the launch
 * mode in effect (any pointer may be NULL). No reference counterpart. */
int cvf_set_row_tile(cvf_handle* h, int lg_rows);
int cvf_get_tuning(const cvf_handle* h, int* tile, int* lg_rows, int* launch_mode);
/* Sets the sweep tile by hand (1, 2, 4 or 8 cells per thread; reduced to the largest that divides
 * every replica's L/2), as the autotuner would. The environment variable CVF_SWEEP_VEC gives the
 * tile a new handle starts with (default 4). Returns the tile in effect through vec_out (may be
 * NULL). No reference counterpart. */
int cvf_set_sweep_tile(cvf_handle* h, int vec, int* vec_out);

/* Launch mode of Metropolis-only steps (n_cluster == 0). 0 (default): a captured CUDA graph per
 * chunk of steps with one kernel per phase (cube + volume moves, each sweep colour, the recorded
 * measurements). 1: each captured chunk is one persistent cooperative kernel that runs every
 * phase of every step of every replica, dealing blocks through tickets, with grid barriers
 * between the phases. Both give the same lattices, counters and samples bit for bit; steps with
 * Swendsen-Wang moves always use per-phase launches. If the CUDA driver cannot capture the
 * cooperative launch, the handle falls back to mode 0 (cvf_get_launch_mode then reports 0). A
 * barrier wait that gives up (about a second) ends the launch and reports CVF_ELIMIT with code 3
 * at the next cvf_synchronize. No reference counterpart (the reference launches one kernel per
 * arm and parity). */
int cvf_set_launch_mode(cvf_handle* h, int mode);
int cvf_get_launch_mode(const cvf_handle* h, int* mode);

/* Bounds of the handle's device waits, for tests of the error path: a grid-barrier wait of the
 * persistent launch (mode 1) polls at most barrier_polls times, one Swendsen-Wang union gives up
 * after union_iters attempts; either sets the replica's error word and the kernel returns, and
 * the next cvf_synchronize reports CVF_ELIMIT (code 3 and code 1). A value < 0 restores the
 * default (2^24 each, about a second of barrier polling; values above it are clamped to it). The
 * state of the replicas after a wait gave up is not a Markov chain state any more: discard the
 * handle. Replaces the reference's unbounded host-polled convergence loop (GW:1480-1555), which
 * has no bound to set. */
int cvf_set_wait_limits(cvf_handle* h, long long barrier_polls, long long union_iters);

/* Replica groups of a batch (0 = automatic: 4 groups for 8 or more replicas, 2 for 2 to 7).
 * Metropolis-only steps of a batch are captured as one chain of per-phase kernels per group of
 * consecutive replicas (groups of about equal cell counts), on parallel branches of the CUDA
 * graph, so that the blocks of one group fill the tails of another group's kernels. The results
 * do not depend on the grouping. cvf_get_replica_groups reports the count in effect. No
 * reference counterpart. */
int cvf_set_replica_groups(cvf_handle* h, int groups);
int cvf_get_replica_groups(const cvf_handle* h, int* groups);

/* Transfer mode of cvf_set_config and cvf_get_config. 1: kernels read and pack, or unpack and
 * write, the caller's cells12 array where it lies in host memory (the GPU accesses pageable host
 * memory through the host page tables, as over NVLink-C2C on GB300); the default when the device
 * reports cudaDevAttrPageableMemoryAccess. cvf_get_config first has host threads touch the
 * array's pages that are not resident, and uses the mode only for a 16-byte aligned array. 0:
 * host threads pack into pinned memory and unpack from it, with one copy each way (the only mode
 * on other systems; cvf_set_io_mode(h, 1) then fails with CVF_EINVAL). Both modes give the same
 * lattice and array and the same error for an invalid value (the lattice is left unchanged).
 * No reference counterpart. */
int cvf_set_io_mode(cvf_handle* h, int mode);
int cvf_get_io_mode(const cvf_handle* h, int* mode);

/* The CUDA stream (a cudaStream_t passed as void*) on which all work of the handle is ordered,
 * for callers that time or order their own work around the engine. No reference counterpart. */
int cvf_get_stream(cvf_handle* h, void** stream);
/* Profiling hook: enqueue n launches of one kernel kind outside any graph on the handle's stream:
 * kind 0 = one checkerboard sweep (two launches, colour 0 then 1; sweep i of the call draws the
 * random stream of sweep (last step's first sweep + i), so repeated calls reuse streams),
 * 1 = cube move, 2 = volume move, 3 = measurement. For timing only. No reference counterpart. */
int cvf_profile_launch(cvf_handle* h, int kind, int n);

/* Cluster statistics (as cvf_cluster_stats) of a caller-owned device array of 6*L^3 labels,
 * without allocating any device memory. No counterpart in the reference.
 * For callers that cannot call cudaMalloc: code running while a CUDA graph is captured, processes
 * whose device memory is reserved by another allocator or capped by a pool, hosts that forbid a
 * library to grow its footprint after start-up. The work space is a fixed array inside the
 * library (about 8.6 MB on every GPU that loads it, held until the process exits).
 *   labels: device pointer, site = arm*N + cell, each label a site id in [0, 6N);
 *   out7:   device pointer to 7 long longs: largest, second, n_percolating, n_clusters,
 *           sum_size, sum_size2, sum_size2_wrap32 (n_clusters = -1 if a label is out of range);
 *   stream: cudaStream_t passed as void* (NULL = legacy default stream); nothing synchronises.
 * Limit: 6*L^3 <= CVF_NOALLOC_MAX_SITES (even L <= 54); larger L returns CVF_EINVAL.
 * All calls share the array: calls whose work overlaps on the GPU race and give wrong results.
 * The first call on a device looks up the array's address; make it before any stream capture. */
#define CVF_NOALLOC_MAX_SITES 1048576
int cvf_cluster_stats_noalloc(const int* labels, int L, long long* out7, void* stream);

/* Histogram reweighting (replaces the Fortran Calcula_Histograma F90:1003-1124 and the finite
 * differences of CVF_ThermodynamicAnalysis/{AlphaP,CP,KT}derivate.c).
 *   samples: n rows of (E, V, N_hb, N_sigma) in internal units, grouped by run;
 *   run_of:  run index of each row; runs: n_runs rows of (beta, P) of the simulations;
 *   f:       in/out dimensionless free energies -log Z_j (n_runs), refined by n_iter WHAM
 *            iterations on the device when n_iter > 0 (all zeros in: started from thermodynamic
 *            integration of <E> d beta + <V> d(beta P) between consecutive runs);
 *   theta:   target (beta, P, dJ_hb, dJ_sigma, dv_hb): weights exp(-beta (E' + P V')) with
 *            E' = E - dJ_hb N_hb - dJ_sigma N_sigma and V' = V + dv_hb N_hb;
 *   out:     n_obs reweighted means of the columns (E, V, N_hb, N_sigma, H = E + P V, rho = N/V,
 *            E^2, V^2, H^2, V*H, ...) selected by obs_ids (see cvf_reweight_obs ids below),
 *            and log Z(theta) in out[n_obs].
 * cvf_reweight_adjoint returns grad_theta[5] = sum_m g[m] d out[m] / d theta. */
#define CVF_RW_E 0
#define CVF_RW_V 1
#define CVF_RW_NHB 2
#define CVF_RW_NSIG 3
#define CVF_RW_H 4
#define CVF_RW_RHO 5
#define CVF_RW_H2 6
#define CVF_RW_V2 7
#define CVF_RW_VH 8
int cvf_reweight_forward(int device, const double* samples, const int* run_of, long long n, const double* runs,
                         int n_runs, double* f, int n_iter, double tol, double n_cells, const double* theta,
                         const int* obs_ids, int n_obs, double* out);
int cvf_reweight_adjoint(int device, const double* samples, const int* run_of, long long n, const double* runs,
                         int n_runs, const double* f, double n_cells, const double* theta, const int* obs_ids,
                         int n_obs, const double* g, double* grad_theta);

#ifdef __cplusplus
}
#endif
#endif
