// Host-side pieces of the engine that need no GPU: parameter checks, the vdW shell table,
// acceptance thresholds, packing of config.out-style cells to the colour-split device layout,
// and the eta <-> cube-state conversions. Shared by the engine and the gpu_water3D driver.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cvf.h"

namespace cvf {

// GW:865-932 with distance_PBC GW:1323-1337: distinct minimum-image distances d < Rc from cell 0
// in first-encounter order (x fastest), freq = (count/2)*N.
void compute_shells(int L, float Rc, std::vector<float>& dist, std::vector<int>& freq);

struct Thresholds {
  unsigned long long sweep[33], cube[9], sw[2];
  double beta, Jeff;
};
// beta = 1/T (GW:388); Jeff = J_hb - P v_hb evaluated in float as in GW:391; tables in FP64.
Thresholds make_thresholds(float T, float P);

double host_evdw(double r, const std::vector<float>& dist, const std::vector<int>& freq, float Rc);

// data.out formulas of GW:2138-2159 from exact counts.
void fill_obs(cvf_obs* o, long long n_hb2, long long n_sigma, double r_cell, double volume, double e_vdw,
              long long N, float P);
void fill_cstats(cvf_cstats* c);

// cells12 (config.out order) -> colour-split words (cells0/cells1: N/2 words each) and cube
// states (cubes_even/cubes_odd: (L/2)^3 bytes each); returns false on a value out of range.
// eta is read with the decision tree of GW:3314-3371. Threaded over rows of the lattice.
bool pack_config(int L, const int* cells12, uint32_t* cells0, uint32_t* cells1, uint8_t* cubes_even,
                 uint8_t* cubes_odd, std::string& err);
// The reader's message (GW:776-790) for the first invalid value of cell c.
std::string config_value_error(const int* c12, long long c);
// Writes a zero into every page of [p, p + bytes) that is not resident (mincore), from host
// threads, so that the pages exist before a GPU writes the range (a GPU's first write to a
// pageable page faults far more slowly than a host thread's).
void touch_pages(void* p, size_t bytes);
void unpack_config(int L, const uint32_t* cells0, const uint32_t* cells1, const uint8_t* cubes_even,
                   const uint8_t* cubes_odd, int* cells12);

}  // namespace cvf
