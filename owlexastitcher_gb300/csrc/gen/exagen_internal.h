// exagen_internal.h -- the generator's result object and host-side field
// set-up, shared by the CPU generator (exagen.cpp) and the GPU generator
// (exagen_gpu.cu).
#pragma once

#include <string>
#include <vector>

#include "../../../include/exastitch_gen.h"
#include "exagen_field.h"

namespace exagen {

// the seeded parameter stream of the field (splitmix64)
struct Stream {
  uint64_t s;
  explicit Stream(uint64_t seed) : s(seed) {}
  double next01()
  {
    s += 0x9e3779b97f4a7c15ull;
    return (double)(mix64(s) >> 11) * (1.0 / 9007199254740992.0);
  }
  double uniform(double a, double b) { return a + (b - a) * next01(); }
};

// The field's parameters and tables on the host.  setup() draws the
// Gaussians and fills the noise lattices; the cloud mapping range and the
// per-level Gaussian tables are filled by the generator that runs.
struct Field {
  int kind = EXA_FIELD_GAUSSIANS;
  int K = 0;
  std::vector<double> cx, cy, cz, sx, sy, sz, amp;
  double noiseAmp = 0.1;
  int octaves = 4;
  uint64_t seed = 0;
  double extent[3] = {1, 1, 1};
  double cloudLo = 0.0, cloudHi = 1.0;
  std::vector<std::vector<float>> latTab;
  std::vector<int> latN;
  std::vector<std::vector<double>> gtab[3];  // per axis, per level

  void setup(const exa_gen_params &P);
  double gauss1(int k, int axis, double p) const
  {
    const double c = axis == 0 ? cx[k] : axis == 1 ? cy[k] : cz[k];
    const double s = axis == 0 ? sx[k] : axis == 1 ? sy[k] : sz[k];
    const double t = (p - c) / s;
    return gen_exp(-0.5 * t * t);
  }
  // row i of axis a at level L: the factors of the level's cell centres
  void gaussRow(int a, int L, int64_t i, double *out) const
  {
    for (int k = 0; k < K; ++k)
      out[k] = gauss1(k, a, cell_center(L, i) / extent[a]) * (a == 0 ? amp[k] : 1.0);
  }
  // view with host pointers (Gaussian tables only where they were built)
  FieldView view() const;
  // unit-cube coordinates, direct sum over the Gaussians
  double evalUnit(double x, double y, double z) const;
};

int numThreadsOf(const exa_gen_params *p);
void setLastError(const std::string &msg);
void checkParams(const exa_gen_params *p);

} // namespace exagen

struct exa_gen_result {
  exa_gen_params params;
  exagen::Field field;
  std::vector<exa_vec4f> vertices;
  std::vector<int32_t> indices;
  std::vector<exa_gridlet> gridlets;
  std::vector<float> gridletScalars;
  std::vector<int32_t> amrCells;
  std::vector<float> amrScalars;
  exa_gen_stats stats;
};
