// gpu_water3D -- drop-in replacement of the reference executable SOURCE/gpu_water3D.
//
// Same invocation (no arguments; the current directory holds the files), same inputs
// (input_data, input_config when Flag_config=1, distances when Flag_distances=1) and outputs
// (data.out, cluster.out, config.out, water3D.log, distances when Flag_distances=0) as
// main() of SOURCE/gpu_water3D.cu (GW:279-1321). The Monte Carlo work runs in the engine behind
// include/cvf.h. Extensions: an optional 15th input_data line "Lattice_Size L" or "-L L" on the
// command line (the reference fixes L = 32 at compile time).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/cvf.h"

static void die(const char* what) {
  fprintf(stderr, "%s\n", what ? what : "error");
  exit(1);
}

static void check(int rc) {
  if (rc) die(cvf_last_error_string());
}

int main(int argc, char** argv) {
  cvf_input in;
  if (cvf_read_input_data("input_data", &in)) die(cvf_last_error_string());
  for (int i = 1; i + 1 < argc; ++i)
    if (!strcmp(argv[i], "-L")) in.L = atoi(argv[i + 1]);
  const int L = in.L;
  const long long N = (long long)L * L * L;
  if (in.sampling_interval < 1) die("Error[Sampling_Interval]: must be >= 1");

  FILE* odata = fopen("data.out", "w");
  if (!odata) die("Can't create output file");
  FILE* log = fopen("water3D.log", "w");
  if (!log) die("Can't create log file");
  // header as GW:447-509
  fprintf(log, "++++ Welcome to water3D log file ++++\n");
  fprintf(log, "RNG allocated memory: %d MB\n", 0);
  fprintf(log, " ++++++++++++++++++++++++++++++++++++++++++\n");
  fprintf(log, "Source file: %s\n", "cvfbulkwater_gb300 gpu_water3D");
  fprintf(log, " 3D water model, %d x %d x %d lattice, N = %lld, P = %1.2f, T = %1.2f\n", L, L, L, N, in.P, in.T);
  fprintf(log, " J_hb = %1.2f, J_sigma = %1.2f, v_HB = %1.2f\n", 0.5f, 0.08f, 0.6f);
  fprintf(log, " Flag configuration = %d\n", in.flag_config);
  fprintf(log, " Monte Carlo Step: %d Metropolis + %d Cluster\n", in.metropolis_steps, in.cluster_steps);
  fprintf(log, " Metropolis: Parallel GPU algorithm\n");
  fprintf(log, " Cluster: Swendsen-Wang Parallel GPU algorithm\n");
  fprintf(log, " Device = %d\n", in.device_id);
  fprintf(log, " %d equilibration, %d updates/measurement, %d updates\n", in.equilibrium_steps, in.sampling_interval,
          in.sampling_steps);
  fprintf(log, " Output file %s\n", "data.out");
  fprintf(log, " Random seed %lld\n", in.seed);

  cvf_params p;
  memset(&p, 0, sizeof(p));
  p.L = L;
  p.T = in.T;
  p.P = in.P;
  p.seed = in.seed;
  p.R_cutoff = in.R_cutoff;
  p.start = in.flag_config;
  p.flag_chessboard = in.flag_chessboard;
  p.replica = 0;
  p.device = in.device_id;
  p.sample_capacity = 1 << 16;
  if (in.flag_config < 0 || in.flag_config > 2) {
    fprintf(stderr, "Error: Wrong value for flag_config = %d\n", in.flag_config);
    fprintf(stderr, "Flag_config=0  Initial spins completely disordered\n");
    fprintf(stderr, "Flag_config=1  Initial spins read from file\n");
    fprintf(stderr, "Flag_config=2  Initial spins completely ordered (T=0)\n");
    exit(1);
  }
  cvf_handle* h = nullptr;
  check(cvf_create(&p, &h));
  fprintf(log, "Starting Chessboard\n");
  std::vector<int> cells((size_t)N * 12);
  if (in.flag_config == 1) {
    check(cvf_read_config_file("input_config", cells.data(), N));
    check(cvf_set_config(h, 0, cells.data(), N));
  }
  std::vector<float> dist(512);
  std::vector<int> freq(512);
  int nsh = 0;
  if (in.flag_distances == 0) {
    check(cvf_get_distances(h, 0, dist.data(), freq.data(), 512, &nsh));
    check(cvf_write_distances_file("distances", L, dist.data(), freq.data(), nsh));
  } else {
    check(cvf_read_distances_file("distances", L, dist.data(), freq.data(), 512, &nsh));
    check(cvf_set_distances(h, 0, dist.data(), freq.data(), nsh));
  }
  FILE* logsize = fopen("cluster.out", "w");
  if (!logsize) die("Can't open input file");

  // equilibration, GW:1176-1194
  check(cvf_run_steps(h, in.equilibrium_steps, in.metropolis_steps, in.cluster_steps));
  // every production step feeds the correlator (GW:1245-1272)
  if (in.flag_correlation == 1) check(cvf_set_correlation(h, 1));

  // production, GW:1204-1275: a sample after every step i with i % N_MEASURE == 0
  double E = 0, E2 = 0, M = 0, M2 = 0;
  const int interval = in.sampling_interval;
  const long long per_chunk = (long long)interval * 16384;
  std::vector<cvf_sample> smp;
  std::vector<cvf_cstats> cst;
  char line[256];
  long long done = 0;
  while (done < in.sampling_steps) {
    long long steps = in.sampling_steps - done;
    if (steps > per_chunk) steps = per_chunk;
    check(cvf_clear_samples(h));
    check(cvf_run_sampled(h, (int)steps, in.metropolis_steps, in.cluster_steps, interval));
    long long n = 0;
    check(cvf_sample_count(h, 0, &n));
    smp.resize((size_t)n);
    check(cvf_get_samples(h, 0, smp.data(), n, &n));
    if (in.cluster_steps > 0) {
      cst.resize((size_t)n);
      long long m = 0;
      check(cvf_get_cstats_stream(h, 0, cst.data(), n, &m));
    } else {
      cst.assign((size_t)n, cvf_cstats());
      cvf_cstats c;
      check(cvf_cluster_stats(h, 0, &c));  // no SW step: one cluster of 6N sites (labels zero)
      for (auto& x : cst) x = c;
    }
    for (long long i = 0; i < n; ++i) {
      int t = (int)(done + i * interval);
      cvf_obs o;
      check(cvf_sample_observables(h, 0, &smp[(size_t)i], &o));
      if (cvf_format_cluster_line(line, sizeof(line), t, &cst[(size_t)i]) > 0) fputs(line, logsize);
      if (cvf_format_data_line(line, sizeof(line), t, &o) > 0) fputs(line, odata);
      E += o.energy;
      E2 += o.energy * o.energy;
      M += o.m;
      M2 += o.m * o.m;
    }
    done += steps;
  }
  fclose(odata);
  fclose(logsize);
  // GW:1277-1293
  const double nm = in.sampling_steps * 1. / interval;
  M /= nm;
  M2 /= nm;
  E /= nm;
  E2 /= nm;
  fprintf(log, "Magnetization:\t%1.6lf\t+/-\t%1.6lf\n", M, sqrt(M2 - M * M));
  fprintf(log, "Energy:\t\t%1.6lf\t+/-\t%1.6lf\n", E, sqrt(E2 - E * E));
  check(cvf_get_config(h, 0, cells.data(), N));
  check(cvf_write_config_file("config.out", cells.data(), N));
  if (in.flag_correlation == 1) {  // GW:1307-1313, printCorr GW:3109-3128
    std::vector<double> ct(32 * 16), cf(32 * 16);
    int nc = 0;
    check(cvf_get_correlation(h, 0, ct.data(), cf.data(), (int)ct.size(), &nc));
    FILE* fc = fopen("correlation.dat", "w");
    if (!fc) die("Can't create correlation.dat");
    for (int i = 0; i < nc; ++i) fprintf(fc, "%.0f\t%f\n", ct[i], cf[i] / cf[0]);
    fclose(fc);
  }
  // the union-find labelling needs one pass per SW step; -1 when no SW step ran (GW:1557-1559)
  fprintf(log, "Max_SW_scans = %d\n", in.cluster_steps > 0 ? 1 : -1);
  fprintf(log, " ** simulation done\n");
  fclose(log);
  check(cvf_synchronize(h));
  cvf_destroy(h);
  return 0;
}
