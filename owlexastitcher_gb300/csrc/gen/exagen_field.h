// exagen_field.h -- the generator's analytic field, shared word for word by
// the CPU generator (exagen.cpp) and the GPU generator (exagen_gpu.cu), so
// that both evaluate the same binary64 operations in the same order (both
// build without contracted multiply-adds).  The two transcendental calls of
// the field go through gen_exp, written here, because the C library's and
// CUDA's exp need not agree in the last bit, and a one-bit difference can
// flip a refinement decision.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define GEN_HD __host__ __device__ inline
#else
#define GEN_HD inline
#endif

namespace exagen {

constexpr int kMaxLevels = 16;
constexpr int kMaxOctaves = 16;

GEN_HD uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// e^x.  Cody and Waite's argument reduction (W. J. Cody, W. Waite, "Software
// Manual for the Elementary Functions", 1980): x = k ln2 + r with k =
// round(x / ln2) and ln2 split into a 32-bit head (so k * head is exact for
// |k| < 2^21) and the binary64 nearest to the remainder; then the Taylor
// series of e^r to r^13 / 13! (|r| <= 0.35: truncation below 2e-17
// relative) by Horner's rule, scaled by 2^k.  About 1-2 ulp.
GEN_HD double gen_exp(double x)
{
  if (x != x) return x;
  if (x > 709.8) return INFINITY;
  if (x < -745.2) return 0.0;
  const double kLn2Head = 0x1.62e42feep-1;        // ln 2 to 32 bits
  const double kLn2Tail = 0x1.a39ef35793c76p-33;  // ln 2 - kLn2Head
  const double kd = floor(x * 0x1.71547652b82fep0 + 0.5);  // x / ln 2, rounded
  const double r = (x - kd * kLn2Head) - kd * kLn2Tail;
  double p = 1.0 / 6227020800.0;  // 1/13!
  p = p * r + 1.0 / 479001600.0;
  p = p * r + 1.0 / 39916800.0;
  p = p * r + 1.0 / 3628800.0;
  p = p * r + 1.0 / 362880.0;
  p = p * r + 1.0 / 40320.0;
  p = p * r + 1.0 / 5040.0;
  p = p * r + 1.0 / 720.0;
  p = p * r + 1.0 / 120.0;
  p = p * r + 1.0 / 24.0;
  p = p * r + 1.0 / 6.0;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  return ldexp(p, (int)kd);
}

// Everything an evaluation of the field reads.  Pointers are host or
// device arrays, as the evaluating side needs.
struct FieldView {
  int kind;                // EXA_FIELD_*
  int K;                   // Gaussians
  int octaves;
  uint64_t seed;
  double noiseAmp;
  double extent[3];        // finest units per axis
  double cloudLo, cloudHi; // cloud mapping clamp((exp(3 fbm) - lo) / (hi - lo), 0, 1)
  const float *lat[kMaxOctaves];  // per octave: m^3 lattice values of the unit cube
  int latN[kMaxOctaves];
  // per axis and level: n * K factors exp(-0.5 ((c_i - c_k) / s_k)^2), times
  // amp_k on x, for the cell centres c_i of that level
  const double *gtab[3][kMaxLevels];
};

// hashed lattice value in [-1, 1), rounded to binary32
GEN_HD double lattice(const FieldView &F, int64_t i, int64_t j, int64_t k, int o)
{
  uint64_t h = mix64(F.seed ^ 0x243f6a8885a308d3ull);
  h = mix64(h ^ (uint64_t)(i * 73856093ll));
  h = mix64(h ^ (uint64_t)(j * 19349663ll));
  h = mix64(h ^ (uint64_t)(k * 83492791ll));
  h = mix64(h ^ (uint64_t)o);
  return (double)(float)((double)(h >> 11) * (2.0 / 9007199254740992.0) - 1.0);
}

GEN_HD double lattice_fast(const FieldView &F, int64_t i, int64_t j, int64_t k, int o)
{
  const int m = F.latN[o];
  if (i >= 0 && j >= 0 && k >= 0 && i < m && j < m && k < m)
    return (double)F.lat[o][((size_t)k * m + j) * m + i];
  return lattice(F, i, j, k, o);
}

// value noise: hashed lattice values, smoothstep-weighted trilinear
GEN_HD double vnoise(const FieldView &F, double x, double y, double z, int o)
{
  const double fx = floor(x), fy = floor(y), fz = floor(z);
  const int64_t i = (int64_t)fx, j = (int64_t)fy, k = (int64_t)fz;
  double tx = x - fx, ty = y - fy, tz = z - fz;
  tx = tx * tx * (3 - 2 * tx);
  ty = ty * ty * (3 - 2 * ty);
  tz = tz * tz * (3 - 2 * tz);
  double c[2][2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) c[a][b][d] = lattice_fast(F, i + d, j + b, k + a, o);
  const double x00 = c[0][0][0] + tx * (c[0][0][1] - c[0][0][0]);
  const double x01 = c[0][1][0] + tx * (c[0][1][1] - c[0][1][0]);
  const double x10 = c[1][0][0] + tx * (c[1][0][1] - c[1][0][0]);
  const double x11 = c[1][1][0] + tx * (c[1][1][1] - c[1][1][0]);
  const double y0 = x00 + ty * (x01 - x00), y1 = x10 + ty * (x11 - x10);
  return y0 + tz * (y1 - y0);
}

// octave sum normalised by the sum of weights 0.5^o; base frequency f0
GEN_HD double octave_noise(const FieldView &F, double x, double y, double z, double f0, int n)
{
  double sum = 0, wsum = 0, w = 1, f = f0;
  for (int o = 0; o < n; ++o) {
    sum += w * vnoise(F, x * f, y * f, z * f, o);
    wsum += w;
    w *= 0.5;
    f *= 2.0;
  }
  return sum / wsum;
}

GEN_HD double cloud_raw(const FieldView &F, double x, double y, double z)
{
  return gen_exp(3.0 * octave_noise(F, x, y, z, 2.0, F.octaves));
}

GEN_HD double cloud_map(const FieldView &F, double raw)
{
  const double v = (raw - F.cloudLo) / (F.cloudHi - F.cloudLo);
  return v < 0 ? 0 : (v > 1 ? 1 : v);
}

GEN_HD double cell_center(int L, int64_t i) { return ((double)i + 0.5) * (double)(1ll << L); }

// the field at the centre of level-L cell (i, j, k)
GEN_HD double eval_cell(const FieldView &F, int L, int64_t i, int64_t j, int64_t k)
{
  const double x = cell_center(L, i) / F.extent[0], y = cell_center(L, j) / F.extent[1],
               z = cell_center(L, k) / F.extent[2];
  if (F.kind != 0) return cloud_map(F, cloud_raw(F, x, y, z));
  const double *gx = F.gtab[0][L] + (size_t)i * F.K;
  const double *gy = F.gtab[1][L] + (size_t)j * F.K;
  const double *gz = F.gtab[2][L] + (size_t)k * F.K;
  double g = 0;
  for (int q = 0; q < F.K; ++q) g += gx[q] * gy[q] * gz[q];
  return g + F.noiseAmp * octave_noise(F, x, y, z, 4.0, F.octaves);
}

// refinement test of a level-L cell with value v: Gaussians |v| > t max|f|;
// cloud: deeper levels need denser cloud (thresholds t, 2t, 4t, ...)
GEN_HD bool refine_crit(int kind, double v, int L, int Lroot, double threshold, double maxAbs)
{
  if (kind == 0) return fabs(v) > threshold * maxAbs;
  return v > threshold * ldexp(1.0, Lroot - L);
}

} // namespace exagen
