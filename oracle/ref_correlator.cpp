// Test harness (not part of the library): drives the reference's own multi-tau correlator,
// initialize / add / evaluate of SOURCE/gpu_water3D.cu (GW:2983-3107), compiled from that file
// where it lies by oracle/build_ref.py, so that oracle/correlator.py is checked against the
// reference's code. Only the structure layout (GW:170-181) and the allocation of GW:1096-1116
// are restated here, to call those functions.
#include <stdlib.h>
#include <string.h>

struct correlator {
  double** shift;
  double** correlation;
  long int** ncorrelation;
  double* accumulator;
  int* naccumulator;
  int* insertindex;
  double* t;
  double* f;
  int npcorr;
  int kmax;
  double accval;
};

void initialize(int N, correlator mol[]);
void add(correlator mol[], int i, double w, int k);
void evaluate(correlator mol[], int N, int norm);

namespace {
constexpr int kLevels = 32, kP = 16;  // numcorrelators, p (GW:165-166)
}

// Adds w[0..n) at level 0, evaluates with norm = 1; writes up to cap points, returns npcorr.
extern "C" int ref_corr_run(const double* w, int n, double* t, double* f, int cap) {
  correlator c;
  c.shift = (double**)malloc(sizeof(double*) * kLevels);
  c.correlation = (double**)malloc(sizeof(double*) * kLevels);
  c.ncorrelation = (long int**)malloc(sizeof(long int*) * kLevels);
  for (int j = 0; j < kLevels; ++j) {
    c.shift[j] = (double*)calloc(kP, sizeof(double));
    c.correlation[j] = (double*)calloc(kP, sizeof(double));
    c.ncorrelation[j] = (long int*)calloc(kP, sizeof(long int));
  }
  c.accumulator = (double*)calloc(kLevels, sizeof(double));
  c.naccumulator = (int*)calloc(kLevels, sizeof(int));
  c.insertindex = (int*)calloc(kLevels, sizeof(int));
  c.t = (double*)calloc(kLevels * kP, sizeof(double));
  c.f = (double*)calloc(kLevels * kP, sizeof(double));
  initialize(1, &c);
  for (int i = 0; i < n; ++i) add(&c, 0, w[i], 0);
  evaluate(&c, 1, 1);
  const int np = c.npcorr;
  for (int i = 0; i < np && i < cap; ++i) {
    t[i] = c.t[i];
    f[i] = c.f[i];
  }
  for (int j = 0; j < kLevels; ++j) {
    free(c.shift[j]);
    free(c.correlation[j]);
    free(c.ncorrelation[j]);
  }
  free(c.shift);
  free(c.correlation);
  free(c.ncorrelation);
  free(c.accumulator);
  free(c.naccumulator);
  free(c.insertindex);
  free(c.t);
  free(c.f);
  return np;
}
