/*
 * surrogate.c -- CPU restatement of the learned field (hash-grid encoding +
 * MLP) for checking the CUDA kernels in owlexastitcher_gb300/csrc/
 * exa_surrogate.cu{,h}.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h): used by tests/ as the checker,
 * never by the product library.
 *
 * The encoding (cell, weights, hash, feature sums) is restated in binary32
 * with the CUDA code's operation order, so the features are bit-identical;
 * the FP16 inference table and the BF16 rounding points are emulated with
 * round-to-nearest-even conversions.  The MLP products are summed in
 * binary64 (the tensor cores' FP32 accumulation order is not specified), and
 * the backward pass is binary64 throughout, applying the same BF16 rounding
 * of the MMA operands as the forward definition.
 *
 * The encoding follows Mueller et al. 2022, "Instant neural graphics
 * primitives with a multiresolution hash encoding" (spatial hash with
 * primes 1, 2654435761, 805459861; dense indexing where a level's grid
 * fits the table).  No reference file covers it: the learned field has no
 * counterpart in owlExaStitcher.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle.h"

#define OS_LEVELS 16
#define OS_IN 32
#define OS_HID 64
#define OS_PARAMS (OS_HID * OS_IN + OS_HID * OS_HID + OS_HID)

/* 1: no BF16 / binary16 rounding in os_forward / os_gradients (the
 * backward's chain rule can then be checked by finite differences) */
static int g_exact = 0;
void os_set_exact(int on) { g_exact = on; }

static float clamp01(float v) { return v < 0.f ? 0.f : (v > 1.f ? 1.f : (v == v ? v : 0.f)); }

/* float -> bf16 -> float, round to nearest even (NaN kept quiet) */
float os_bf16(float f)
{
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) {
    u = (u | 0x00400000u) & 0xffff0000u;
  } else {
    const uint32_t lsb = (u >> 16) & 1u;
    u = (u + 0x7fffu + lsb) & 0xffff0000u;
  }
  float r;
  memcpy(&r, &u, 4);
  return r;
}

/* float -> IEEE binary16 -> float, round to nearest even: the value is
 * rounded to the binary16 grid (11 significant bits, quantum 2^-24 in the
 * subnormal range) with nearbyint in the default rounding mode */
float os_half(float f)
{
  if (f != f) return f;
  const double a = fabs((double)f);
  if (a >= 65520.0) return f > 0.f ? INFINITY : -INFINITY;
  double q;
  if (a < 6.103515625e-05) {
    q = 5.9604644775390625e-08; /* 2^-24 */
  } else {
    int e;
    frexp(a, &e); /* a = m 2^e, m in [0.5, 1) */
    q = ldexp(1.0, e - 11);
  }
  return (float)(nearbyint((double)f / q) * q);
}

static float rb(float f) { return g_exact ? f : os_bf16(f); }
static float rh(float f) { return g_exact ? f : os_half(f); }

void os_geom_init(os_geom *g, int log2T, int baseRes, float growth, const float lo[3], const float hi[3], float vmin,
                  float vmax)
{
  memset(g, 0, sizeof(*g));
  g->log2T = log2T;
  const uint64_t T = 1ull << log2T;
  for (int l = 0; l < OS_LEVELS; ++l) {
    int r = (int)floor((double)baseRes * pow((double)growth, (double)l));
    if (r < 1) r = 1;
    g->res[l] = r;
    const uint64_t side = (uint64_t)r + 1;
    if (side * side * side <= T) g->denseMask |= 1u << l;
  }
  for (int a = 0; a < 3; ++a) {
    const float e = hi[a] - lo[a];
    g->lo[a] = lo[a];
    g->inv[a] = 1.f / (e > 1e-30f ? e : 1e-30f);
  }
  if (!(vmin <= vmax)) { vmin = 0.f; vmax = 1.f; }
  g->vmin = vmin;
  g->vrange = vmax > vmin ? vmax - vmin : 1.f;
}

static void corners(const os_geom *g, int l, const float x[3], uint32_t idx[8], float w[8])
{
  const int r = g->res[l];
  int c[3];
  float f[3];
  for (int a = 0; a < 3; ++a) {
    const float p = x[a] * (float)r;
    int ci = (int)floorf(p);
    ci = ci < 0 ? 0 : (ci > r - 1 ? r - 1 : ci);
    c[a] = ci;
    f[a] = clamp01(p - (float)ci);
  }
  const int dense = (g->denseMask >> l) & 1u;
  for (int k = 0; k < 8; ++k) {
    const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
    const float wx = dx ? f[0] : 1.f - f[0];
    const float wy = dy ? f[1] : 1.f - f[1];
    const float wz = dz ? f[2] : 1.f - f[2];
    w[k] = (wx * wy) * wz;
    const uint32_t X = (uint32_t)(c[0] + dx), Y = (uint32_t)(c[1] + dy), Z = (uint32_t)(c[2] + dz);
    if (dense) {
      const uint32_t side = (uint32_t)r + 1u;
      idx[k] = X + side * (Y + side * Z);
    } else {
      idx[k] = (X * 1u ^ Y * 2654435761u ^ Z * 805459861u) & ((1u << g->log2T) - 1u);
    }
  }
}

static void normalize(const os_geom *g, const float pos[3], float x[3])
{
  for (int a = 0; a < 3; ++a) x[a] = clamp01((pos[a] - g->lo[a]) * g->inv[a]);
}

/* features of one position; half != 0 reads the table through binary16 */
void os_encode(const os_geom *g, const float *table, const float pos[3], int half, float feat[OS_IN])
{
  float x[3];
  normalize(g, pos, x);
  const size_t T = (size_t)1 << g->log2T;
  for (int l = 0; l < OS_LEVELS; ++l) {
    uint32_t idx[8];
    float w[8];
    corners(g, l, x, idx, w);
    float f0 = 0.f, f1 = 0.f;
    for (int k = 0; k < 8; ++k) {
      const float *e = table + 2 * ((size_t)l * T + idx[k]);
      const float e0 = half ? rh(e[0]) : e[0], e1 = half ? rh(e[1]) : e[1];
      f0 += w[k] * e0;
      f1 += w[k] * e1;
    }
    feat[2 * l] = f0;
    feat[2 * l + 1] = f1;
  }
}

/* forward of one input row; keeps the BF16 activations for the backward */
static double mlp_forward(const float *w, const float feat[OS_IN], float a0[OS_IN], float h1[OS_HID], float h2[OS_HID])
{
  const float *W1 = w, *W2 = w + OS_HID * OS_IN, *w3 = w + OS_HID * OS_IN + OS_HID * OS_HID;
  for (int i = 0; i < OS_IN; ++i) a0[i] = rb(feat[i]);
  for (int j = 0; j < OS_HID; ++j) {
    double z = 0.0;
    for (int i = 0; i < OS_IN; ++i) z += (double)rb(W1[j * OS_IN + i]) * (double)a0[i];
    const float zf = (float)z;
    h1[j] = rb(zf > 0.f ? zf : 0.f);
  }
  for (int j = 0; j < OS_HID; ++j) {
    double z = 0.0;
    for (int i = 0; i < OS_HID; ++i) z += (double)rb(W2[j * OS_HID + i]) * (double)h1[i];
    const float zf = (float)z;
    h2[j] = rb(zf > 0.f ? zf : 0.f);
  }
  double y = 0.0;
  for (int j = 0; j < OS_HID; ++j) y += (double)h2[j] * (double)rb(w3[j]);
  return y;
}

/* normalised outputs y of n positions (inference path: binary16 table) */
void os_forward(const os_geom *g, const float *w, const float *table, const float *pos, int64_t n, double *y)
{
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    float feat[OS_IN], a0[OS_IN], h1[OS_HID], h2[OS_HID];
    os_encode(g, table, pos + 3 * i, 1, feat);
    y[i] = mlp_forward(w, feat, a0, h1, h2);
  }
}

/* Gradients of L = (1/n) sum over valid pairs of (y - target)^2 with the
 * training path's forward (FP32 master table).  gW: OS_PARAMS doubles,
 * gTable: 2 * 16 * T doubles (both zeroed here).  Returns L. */
double os_gradients(const os_geom *g, const float *w, const float *table, const float *pairs, int n, double *gW,
                    double *gTable)
{
  const float *W1 = w, *W2 = w + OS_HID * OS_IN, *w3 = w + OS_HID * OS_IN + OS_HID * OS_HID;
  const size_t T = (size_t)1 << g->log2T;
  memset(gW, 0, sizeof(double) * OS_PARAMS);
  if (gTable) memset(gTable, 0, sizeof(double) * 2 * OS_LEVELS * T);
  double loss = 0.0;
  const float invRange = 1.f / g->vrange;
  for (int s = 0; s < n; ++s) {
    const float *pr = pairs + 4 * (size_t)s;
    const float v = pr[3];
    if (!(v == v)) continue;
    const float target = (v - g->vmin) * invRange;
    float feat[OS_IN], a0[OS_IN], h1[OS_HID], h2[OS_HID];
    os_encode(g, table, pr, 0, feat);
    const double y = mlp_forward(w, feat, a0, h1, h2);
    const double diff = y - (double)target;
    loss += diff * diff;
    const double gr = 2.0 * diff / (double)n;
    double d2[OS_HID], e1[OS_HID], d1[OS_HID], din[OS_IN];
    for (int j = 0; j < OS_HID; ++j) {
      gW[OS_HID * OS_IN + OS_HID * OS_HID + j] += gr * (double)h2[j];
      d2[j] = h2[j] > 0.f ? (double)rb((float)(gr * (double)rb(w3[j]))) : 0.0;
    }
    for (int i = 0; i < OS_HID; ++i) {
      double z = 0.0;
      for (int j = 0; j < OS_HID; ++j) z += d2[j] * (double)rb(W2[j * OS_HID + i]);
      e1[i] = z;
      d1[i] = h1[i] > 0.f ? (double)rb((float)z) : 0.0;
    }
    for (int j = 0; j < OS_HID; ++j)
      for (int i = 0; i < OS_HID; ++i) gW[OS_HID * OS_IN + j * OS_HID + i] += d2[j] * (double)h1[i];
    for (int j = 0; j < OS_HID; ++j)
      for (int i = 0; i < OS_IN; ++i) gW[j * OS_IN + i] += d1[j] * (double)a0[i];
    for (int i = 0; i < OS_IN; ++i) {
      double z = 0.0;
      for (int j = 0; j < OS_HID; ++j) z += d1[j] * (double)rb(W1[j * OS_IN + i]);
      din[i] = z;
    }
    (void)e1;
    if (gTable) {
      float x[3];
      normalize(g, pr, x);
      for (int l = 0; l < OS_LEVELS; ++l) {
        uint32_t idx[8];
        float wk[8];
        corners(g, l, x, idx, wk);
        for (int k = 0; k < 8; ++k) {
          double *e = gTable + 2 * ((size_t)l * T + idx[k]);
          e[0] += (double)wk[k] * din[2 * l];
          e[1] += (double)wk[k] * din[2 * l + 1];
        }
      }
    }
  }
  return loss / (double)n;
}
