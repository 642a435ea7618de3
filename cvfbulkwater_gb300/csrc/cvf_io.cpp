// File formats of the gpu_water3D executable contract (host only): input_data, input_config /
// config.out, the distances table, and the data.out / cluster.out line formats.
// Reference: SOURCE/gpu_water3D.cu ("GW").
#include <stdio.h>
#include <string.h>

#include <string>

#include "../../include/cvf.h"

namespace cvf {
void set_last_error(const std::string& m);
}

static int io_fail(const std::string& m) {
  cvf::set_last_error(m);
  return CVF_EINVAL;
}

extern "C" {

// GW:293-386: each line is read with fscanf("%s <value>"); the name is not checked.
int cvf_read_input_data(const char* path, cvf_input* in) {
  if (!path || !in) return io_fail("null path/out");
  FILE* f = fopen(path, "r");
  if (!f) return io_fail("Can't open input file");
  char name[256];
  memset(in, 0, sizeof(*in));
  struct Item {
    const char* label;
    char kind;  // f float, d int, l long long
    void* dst;
  } items[] = {
      {"Pressure", 'f', &in->P},
      {"Temperature", 'f', &in->T},
      {"Seed", 'l', &in->seed},
      {"Metropolis_Steps", 'd', &in->metropolis_steps},
      {"Cluster_Steps", 'd', &in->cluster_steps},
      {"Equilibration_Steps", 'd', &in->equilibrium_steps},
      {"Sampling_Steps", 'd', &in->sampling_steps},
      {"Sampling_Interval", 'd', &in->sampling_interval},
      {"R_cutoff", 'f', &in->R_cutoff},
      {"Flag_config", 'd', &in->flag_config},
      {"Flag_distances", 'd', &in->flag_distances},
      {"Flag_correlation", 'd', &in->flag_correlation},
      {"Flag_chessboard", 'd', &in->flag_chessboard},
      {"Device_ID", 'd', &in->device_id},
  };
  for (auto& it : items) {
    int ok = 0;
    if (it.kind == 'f') ok = fscanf(f, "%255s %f", name, (float*)it.dst);
    else if (it.kind == 'l') ok = fscanf(f, "%255s %lld", name, (long long*)it.dst);
    else ok = fscanf(f, "%255s %d", name, (int*)it.dst);
    if (ok != 2) {
      fclose(f);
      // the reference's messages (GW:301-382); Pressure uses "Error [Pressure]"
      if (!strcmp(it.label, "Pressure")) return io_fail("Error [Pressure]: Can't read input file");
      if (!strcmp(it.label, "Temperature")) return io_fail("Error [Temperature]: Can't read input file");
      return io_fail(std::string("Error[") + it.label + "]: Can't read input file");
    }
  }
  in->L = 32;
  int L = 0;
  if (fscanf(f, "%255s %d", name, &L) == 2 && !strcmp(name, "Lattice_Size")) in->L = L;
  fclose(f);
  return 0;
}

// GW:730-800
int cvf_read_config_file(const char* path, int* c12, long long n) {
  if (!path || !c12 || n < 1) return io_fail("null path/out");
  FILE* f = fopen(path, "r");
  if (!f) return io_fail("Can't open the initial configuration file");
  int v[12];
  long long i = 0;
  while (fscanf(f, "%d %d %d %d %d %d %d %d %d %d %d %d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &v[7],
                &v[8], &v[9], &v[10], &v[11]) == 12) {
    if (i >= n) {
      fclose(f);
      return io_fail("Initial configuration file error: There are more rows than cells in the file");
    }
    for (int j = 0; j < 6; ++j) {
      if (v[j] < 0 || v[j] > 5) {
        fclose(f);
        return io_fail("Initial configuration file error: Unexpected value for spin (" + std::to_string(v[j]) +
                       ") appeared in line " + std::to_string(i));
      }
      if (v[6 + j] < 0 || v[6 + j] > 1) {
        fclose(f);
        return io_fail("Initial configuration file error: Unexpected value for active_bond (" +
                       std::to_string(v[6 + j]) + ") appeared in line " + std::to_string(i));
      }
    }
    memcpy(c12 + 12 * i, v, sizeof(v));
    ++i;
  }
  fclose(f);
  if (i < n) return io_fail("Initial configuration file error: Unexpected ending. Can't fill the spin array");
  return 0;
}

// GW:1296-1305
int cvf_write_config_file(const char* path, const int* c, long long n) {
  if (!path || !c) return io_fail("null path/in");
  FILE* f = fopen(path, "w");
  if (!f) return io_fail("Can't create config file");
  for (long long i = 0; i < n; ++i) {
    const int* v = c + 12 * i;
    fprintf(f, "%d %d %d %d %d %d ", v[0], v[1], v[2], v[3], v[4], v[5]);
    fprintf(f, "%d %d %d %d %d %d\n", v[6], v[7], v[8], v[9], v[10], v[11]);
  }
  fclose(f);
  return 0;
}

// GW:917-932
int cvf_write_distances_file(const char* path, int L, const float* d, const int* fr, int n) {
  if (!path || (!d && n) || (!fr && n)) return io_fail("null path/in");
  FILE* f = fopen(path, "w");
  if (!f) return io_fail("Can't create distances file");
  fprintf(f, "%d %d %d\n", L, L, L);
  for (int i = 0; i < n; ++i) fprintf(f, "%f %d\n", d[i], fr[i]);
  fclose(f);
  return 0;
}

// GW:934-985
int cvf_read_distances_file(const char* path, int L, float* d, int* fr, int cap, int* n) {
  if (!path || !d || !fr || !n) return io_fail("null path/out");
  FILE* f = fopen(path, "r");
  if (!f) return io_fail("Can't open distances file");
  int lx, ly, lz;
  if (fscanf(f, "%d %d %d", &lx, &ly, &lz) != 3) {
    fclose(f);
    return io_fail("Error: Can't read distances file");
  }
  if (lx != L || ly != L || lz != L) {
    fclose(f);
    return io_fail(lx != L ? "Error: Distances file. X rank mismatch"
                           : (ly != L ? "Error: Distances file. Y rank mismatch" : "Error: Distances file. Z rank mismatch"));
  }
  int k = 0;
  float dv;
  int fv;
  while (fscanf(f, "%f %d", &dv, &fv) == 2) {
    if (k >= cap) {
      fclose(f);
      return io_fail("distances file holds more shells than the buffer");
    }
    d[k] = dv;
    fr[k] = fv;
    ++k;
  }
  fclose(f);
  *n = k;
  return 0;
}

// GW:2159
int cvf_format_data_line(char* buf, int cap, int t, const cvf_obs* o) {
  if (!buf || !o) return io_fail("null buffer/obs");
  int k = snprintf(buf, (size_t)cap, "%d %1.7e %1.7e %1.7e %1.7e %1.7e %1.7e\n", t, o->energy, o->enthalpy, o->v_total,
                   o->n_hb, o->m, o->r_cell);
  if (k < 0 || k >= cap) return io_fail("buffer too small");
  return k;
}

// GW:2717-2718: average and variance are the reference's float expressions.
int cvf_format_cluster_line(char* buf, int cap, int t, const cvf_cstats* c) {
  if (!buf || !c) return io_fail("null buffer/stats");
  int k = snprintf(buf, (size_t)cap, "%d %d %d %d %f %f %d\n", t, (int)c->largest, (int)c->second,
                   (int)c->n_percolating, (double)c->mean_ref, (double)c->variance_ref, (int)c->n_clusters);
  if (k < 0 || k >= cap) return io_fail("buffer too small");
  return k;
}

}  // extern "C"
