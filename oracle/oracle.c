/*
 * oracle.c -- CPU restatement of the owlExaStitcher ExaStitch rendering path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only tests/, the
 * smoke check and bench.py's CPU-baseline leg load this library.
 *
 * Built with -ffp-contract=off; every float expression is written in the
 * operation order of the reference line it cites (file:line relative to the
 * owlExaStitcher tree), with float literals so nothing is promoted to double.
 * Third-party helpers the reference takes from OWL (not vendored in the
 * reference tree) are defined here as plain textbook operations:
 *   dot(a,b) = a.x*b.x + a.y*b.y + a.z*b.z, cross = the usual determinant
 *   rows, length = sqrtf(dot), normalize(v) = v * (1.f/sqrtf(dot(v,v))),
 *   min/max = (a<b?a:b)/(a>b?a:b), box contains/overlaps inclusive,
 *   rcp(x) = 1.f/x, xfmPoint(A,p) = (p.x*vx + p.y*vy + p.z*vz) + A.p,
 *   make_rgba = 8 bits per channel, min(255,max(0,int(c*256))).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef exa_vec3f v3;
typedef exa_vec4f v4;
typedef exa_vec3i v3i;

/* ================================================================== */
/* small vector helpers (textbook definitions, see header comment)     */
/* ================================================================== */
static inline v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, v3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 div3(v3 a, v3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 muls(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline v3 smul(float s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b)
{
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float fmin_t(float a, float b) { return a < b ? a : b; }
static inline float fmax_t(float a, float b) { return a > b ? a : b; }
static inline v3 min3(v3 a, v3 b) { return mk3(fmin_t(a.x, b.x), fmin_t(a.y, b.y), fmin_t(a.z, b.z)); }
static inline v3 max3(v3 a, v3 b) { return mk3(fmax_t(a.x, b.x), fmax_t(a.y, b.y), fmax_t(a.z, b.z)); }
static inline float rmin3(v3 a) { return fmin_t(a.x, fmin_t(a.y, a.z)); }
static inline float rmax3(v3 a) { return fmax_t(a.x, fmax_t(a.y, a.z)); }
static inline float len3(v3 a) { return sqrtf(dot3(a, a)); }
static inline v3 norm3(v3 a) { return muls(a, 1.f / sqrtf(dot3(a, a))); }
static inline v3 xyz(v4 a) { return mk3(a.x, a.y, a.z); }
static inline int imin_t(int a, int b) { return a < b ? a : b; }
static inline int imax_t(int a, int b) { return a > b ? a : b; }
static inline int iclamp(int v, int lo, int hi) { return imin_t(imax_t(v, lo), hi); }

/* owl LinearSpace3f * vec3f: b.x*vx + b.y*vy + b.z*vz */
static inline v3 xfm_vector(const exa_affine3f *A, v3 v)
{
  return add3(add3(smul(v.x, A->l.vx), smul(v.y, A->l.vy)), smul(v.z, A->l.vz));
}
static inline v3 xfm_point(const exa_affine3f *A, v3 p)
{
  return add3(xfm_vector(A, p), A->p);
}

/* ================================================================== */
/* project-defined math                                                */
/* ================================================================== */

/* splitmix64 finaliser (Steele, Lea, Flood 2014; Vigna's constants) */
uint64_t oc_mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* Natural log for positive normal floats: x = m*2^e with m in
 * [sqrt(1/2), sqrt(2)); log(m) = 2*atanh(s), s = (m-1)/(m+1), by its
 * Taylor series through s^9; log(2) split in a 16-bit head and a tail. */
float oc_log(float x)
{
  const uint32_t bits = f2u(x);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  float m = u2f((bits & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421354f) { m = m * 0.5f; e = e + 1; }
  const float s  = (m - 1.f) / (m + 1.f);
  const float s2 = s * s;
  const float p  = s2 * (0.333333343f + s2 * (0.200000003f + s2 * (0.142857149f + s2 * 0.111111112f)));
  const float lm = 2.f * s + (2.f * s) * p;
  const float fe = (float)e;
  return fe * 0.693145752f + (fe * 1.42860677e-06f + lm);
}

/* sin and cos of 2*pi*u: quadrant from round(4u), remainder angle
 * theta in [-pi/4, pi/4], Taylor series through theta^9 / theta^8. */
void oc_sincos_turns(float u, float *s, float *c)
{
  const float u4 = u * 4.f;
  const float q  = floorf(u4 + 0.5f);
  const float r  = u4 - q;
  const float t  = r * 1.57079637f;
  const float t2 = t * t;
  const float sp = t + (t * t2) * (-0.166666672f + t2 * (0.00833333377f + t2 * (-0.000198412701f + t2 * 2.75573188e-06f)));
  const float cp = 1.f + t2 * (-0.5f + t2 * (0.0416666679f + t2 * (-0.00138888892f + t2 * 2.48015876e-05f)));
  const int qi = ((int)q) & 3;
  if (qi == 0)      { *s = sp;  *c = cp;  }
  else if (qi == 1) { *s = cp;  *c = -sp; }
  else if (qi == 2) { *s = -sp; *c = -cp; }
  else              { *s = -cp; *c = sp;  }
}

/* Counter-based stream: one key per (pixel, accumulation frame, batch
 * frame, sample); the n-th draw is mix64(key + n*golden) >> 40 scaled by
 * 2^-24.  Stands in for owl::common::LCG<4> (deviceCode.cu:41,1278), whose
 * one stream per pixel runs through all of the pixel's samples; keying by
 * sample makes every camera sample an independent unit of work. */
void oc_rng_init(oc_rng *r, uint32_t pixelID, uint32_t accumID, uint32_t frameID, uint32_t sampleID)
{
  r->key = oc_mix64((((uint64_t)pixelID << 32) | (uint64_t)accumID) ^
                    oc_mix64((((uint64_t)frameID << 32) | (uint64_t)sampleID) + 0x5851f42d4c957f2dull));
  r->counter = 0;
}

float oc_rng_next(oc_rng *r)
{
  r->counter += 1;
  const uint64_t z = oc_mix64(r->key + r->counter * 0x9e3779b97f4a7c15ull);
  return (float)(uint32_t)(z >> 40) * 5.96046448e-08f;
}

/* ================================================================== */
/* Gridlet.h:30-98                                                     */
/* ================================================================== */
static inline float lerpf_(float a, float b, float x) /* common.h:64-68 */
{
  return (1.f - x) * a + x * b;
}

int oc_intersect_gridlet(float *value, int *cellID, v3 pos,
                         const exa_gridlet *g, const float *scalars)
{
  /* getBounds, Gridlet.h:31-36 */
  const float cw = (float)(1 << g->level);
  const v3 lo = muls(mk3((float)g->lower.x + 0.5f, (float)g->lower.y + 0.5f,
                         (float)g->lower.z + 0.5f), cw);
  const v3 hi = muls(mk3(((float)g->lower.x + (float)g->dims.x) + 0.5f,
                         ((float)g->lower.y + (float)g->dims.y) + 0.5f,
                         ((float)g->lower.z + (float)g->dims.z) + 0.5f), cw);
  /* Gridlet.h:48 contains() */
  if (!(lo.x <= pos.x && lo.y <= pos.y && lo.z <= pos.z &&
        pos.x <= hi.x && pos.y <= hi.y && pos.z <= hi.z))
    return 0;
  const int nx = g->dims.x + 1, ny = g->dims.y + 1, nz = g->dims.z + 1;
  const float lw = (float)(1 << g->level);
  const v3 p = mk3((pos.x - lo.x) / lw, (pos.y - lo.y) / lw, (pos.z - lo.z) / lw);
  const int ix = (int)p.x, iy = (int)p.y, iz = (int)p.z;
  const int ax = imin_t(ix + 1, nx - 1), ay = imin_t(iy + 1, ny - 1), az = imin_t(iz + 1, nz - 1);
#define LIN(x, y, z) ((z) * ny * nx + (y) * nx + (x))
  const float *S = scalars + g->begin;
  const float f1 = S[LIN(ix, iy, iz)], f2 = S[LIN(ax, iy, iz)];
  const float f3 = S[LIN(ix, ay, iz)], f4 = S[LIN(ax, ay, iz)];
  const float f5 = S[LIN(ix, iy, az)], f6 = S[LIN(ax, iy, az)];
  const float f7 = S[LIN(ix, ay, az)], f8 = S[LIN(ax, ay, az)];
#undef LIN
  if (isnan(f1) || isnan(f2) || isnan(f3) || isnan(f4) ||
      isnan(f5) || isnan(f6) || isnan(f7) || isnan(f8))
    return 0;
  const v3 frac = mk3(p.x - (float)ix, p.y - (float)iy, p.z - (float)iz);
  const float f12 = lerpf_(f1, f2, frac.x);
  const float f56 = lerpf_(f5, f6, frac.x);
  const float f34 = lerpf_(f3, f4, frac.x);
  const float f78 = lerpf_(f7, f8, frac.x);
  const float f1234 = lerpf_(f12, f34, frac.y);
  const float f5678 = lerpf_(f56, f78, frac.y);
  *value = lerpf_(f1234, f5678, frac.z);
  *cellID = iz * g->dims.y * g->dims.x + iy * g->dims.x + ix;
  return 1;
}

/* ================================================================== */
/* Plane.h:23-99                                                       */
/* ================================================================== */
typedef struct { v3 N; float d; } plane_t;
static inline plane_t make_plane(v3 a, v3 b, v3 c) /* Plane.h:32-38 */
{
  plane_t p;
  p.N = cross3(sub3(b, a), sub3(c, a));
  p.d = dot3(a, p.N);
  return p;
}
static inline float plane_eval(plane_t p, v3 v) { return dot3(v, p.N) - p.d; }

int oc_intersect_tet(float *value, v3 P, v4 a, v4 b, v4 c, v4 d)
{
  const v3 va = sub3(xyz(a), P), vb = sub3(xyz(b), P);
  const v3 vc = sub3(xyz(c), P), vd = sub3(xyz(d), P);
  const plane_t pa = make_plane(vb, vd, vc);
  const plane_t pb = make_plane(va, vc, vd);
  const plane_t pc = make_plane(va, vd, vb);
  const plane_t pd = make_plane(va, vb, vc);
  const v3 zero = mk3(0.f, 0.f, 0.f);
  const float fa = plane_eval(pa, zero) / plane_eval(pa, va);
  if (fa < 0.f || fa > 1.f) return 0;
  /* Plane.h:89,92,95 test fa > 1 (not fb/fc/fd); kept as written */
  const float fb = plane_eval(pb, zero) / plane_eval(pb, vb);
  if (fb < 0.f || fa > 1.f) return 0;
  const float fc = plane_eval(pc, zero) / plane_eval(pc, vc);
  if (fc < 0.f || fa > 1.f) return 0;
  const float fd = plane_eval(pd, zero) / plane_eval(pd, vd);
  if (fd < 0.f || fa > 1.f) return 0;
  *value = fa * a.w + fb * b.w + fc * c.w + fd * d.w;
  return 1;
}

/* ================================================================== */
/* UElems.h:40-464 (Newton inversion of the trilinear-type maps)       */
/* ================================================================== */
static inline float det3(v3 x, v3 y, v3 z) { return dot3(x, cross3(y, z)); }

static void pyr_fns(const float *pc, float *sf) /* UElems.h:46-60 */
{
  const float rm = 1.f - pc[0], sm = 1.f - pc[1], tm = 1.f - pc[2];
  sf[0] = rm * sm * tm;
  sf[1] = pc[0] * sm * tm;
  sf[2] = pc[0] * pc[1] * tm;
  sf[3] = rm * pc[1] * tm;
  sf[4] = pc[2];
}
static void pyr_derivs(const float *pc, float *d) /* UElems.h:62-86 */
{
  d[0] = -(pc[1] - 1.f) * (pc[2] - 1.f);
  d[1] = (pc[1] - 1.f) * (pc[2] - 1.f);
  d[2] = pc[1] - pc[1] * pc[2];
  d[3] = pc[1] * (pc[2] - 1.f);
  d[4] = 0.f;
  d[5] = -(pc[0] - 1.f) * (pc[2] - 1.f);
  d[6] = pc[0] * (pc[2] - 1.f);
  d[7] = pc[0] - pc[0] * pc[2];
  d[8] = (pc[0] - 1.f) * (pc[2] - 1.f);
  d[9] = 0.f;
  d[10] = -(pc[0] - 1.f) * (pc[1] - 1.f);
  d[11] = pc[0] * (pc[1] - 1.f);
  d[12] = -pc[0] * pc[1];
  d[13] = (pc[0] - 1.f) * pc[1];
  d[14] = 1.f;
}
static void wedge_fns(const float *pc, float *sf) /* UElems.h:180-189 */
{
  sf[0] = (1.f - pc[0] - pc[1]) * (1.f - pc[2]);
  sf[1] = pc[0] * (1.f - pc[2]);
  sf[2] = pc[1] * (1.f - pc[2]);
  sf[3] = (1.f - pc[0] - pc[1]) * pc[2];
  sf[4] = pc[0] * pc[2];
  sf[5] = pc[1] * pc[2];
}
static void wedge_derivs(const float *pc, float *d) /* UElems.h:191-217 */
{
  d[0] = -1.f + pc[2];
  d[1] = 1.f - pc[2];
  d[2] = 0.f;
  d[3] = -pc[2];
  d[4] = pc[2];
  d[5] = 0.f;
  d[6] = -1.f + pc[2];
  d[7] = 0.f;
  d[8] = 1.f - pc[2];
  d[9] = -pc[2];
  d[10] = 0.f;
  d[11] = pc[2];
  d[12] = -1.f + pc[0] + pc[1];
  d[13] = -pc[0];
  d[14] = -pc[1];
  d[15] = 1.f - pc[0] - pc[1];
  d[16] = pc[0];
  d[17] = pc[1];
}
static void hex_fns(const float *pc, float *sf) /* UElems.h:313-330 */
{
  const float rm = 1.f - pc[0], sm = 1.f - pc[1], tm = 1.f - pc[2];
  sf[0] = rm * sm * tm;
  sf[1] = pc[0] * sm * tm;
  sf[2] = pc[0] * pc[1] * tm;
  sf[3] = rm * pc[1] * tm;
  sf[4] = rm * sm * pc[2];
  sf[5] = pc[0] * sm * pc[2];
  sf[6] = pc[0] * pc[1] * pc[2];
  sf[7] = rm * pc[1] * pc[2];
}
static void hex_derivs(const float *pc, float *d) /* UElems.h:332-370 */
{
  const float rm = 1.f - pc[0], sm = 1.f - pc[1], tm = 1.f - pc[2];
  d[0] = -sm * tm;
  d[1] = sm * tm;
  d[2] = pc[1] * tm;
  d[3] = -pc[1] * tm;
  d[4] = -sm * pc[2];
  d[5] = sm * pc[2];
  d[6] = pc[1] * pc[2];
  d[7] = -pc[1] * pc[2];
  d[8] = -rm * tm;
  d[9] = -pc[0] * tm;
  d[10] = pc[0] * tm;
  d[11] = rm * tm;
  d[12] = -rm * pc[2];
  d[13] = -pc[0] * pc[2];
  d[14] = pc[0] * pc[2];
  d[15] = rm * pc[2];
  d[16] = -rm * sm;
  d[17] = -pc[0] * sm;
  d[18] = -pc[0] * pc[1];
  d[19] = -rm * pc[1];
  d[20] = rm * sm;
  d[21] = pc[0] * sm;
  d[22] = pc[0] * pc[1];
  d[23] = rm * pc[1];
}

/* shared Newton loop of intersectPyrEXT / WedgeEXT / HexEXT
 * (UElems.h:98-176, 229-309, 384-463); NV vertices; kind 1 = wedge */
static int newton_elem(float *value, v3 P, const v4 *V, int NV,
                       void (*fns)(const float *, float *),
                       void (*derivs)(const float *, float *), int isWedge)
{
  float pc[3] = {0.5f, 0.5f, 0.5f};
  float d[24];
  float w[8];
  int converged = 0;
  for (int it = 0; !converged && it < 10; it++) {
    fns(pc, w);
    derivs(pc, d);
    v3 fcol = mk3(0.f, 0.f, 0.f), rcol = fcol, scol = fcol, tcol = fcol;
    for (int i = 0; i < NV; ++i) {
      const v3 pt = xyz(V[i]);
      fcol = add3(fcol, muls(pt, w[i]));
      rcol = add3(rcol, muls(pt, d[i]));
      scol = add3(scol, muls(pt, d[i + NV]));
      tcol = add3(tcol, muls(pt, d[i + 2 * NV]));
    }
    fcol = sub3(fcol, P);
    const float dd = det3(rcol, scol, tcol);
    if (fabsf(dd) < 1e-6f) return 0;
    const float d0 = det3(fcol, scol, tcol) / dd;
    const float d1 = det3(rcol, fcol, tcol) / dd;
    const float d2 = det3(rcol, scol, fcol) / dd;
    pc[0] = pc[0] - d0;
    pc[1] = pc[1] - d1;
    pc[2] = pc[2] - d2;
    /* UElems.h:147-154: the 1e-4 / 1e6 literals are double constants;
     * the comparisons therefore run in double, as written there */
    if (((double)fabsf(d0) < 1e-4) & ((double)fabsf(d1) < 1e-4) &
        ((double)fabsf(d2) < 1e-4)) {
      converged = 1;
    } else if (((double)fabsf(pc[0]) > 1e6) | ((double)fabsf(pc[1]) > 1e6) |
               ((double)fabsf(pc[2]) > 1e6)) {
      return 0;
    }
  }
  if (!converged) return 0;
  /* UElems.h:161-162: 0.f - 1e-6 and 1.f + 1e-6 are double expressions
   * stored into float */
  const float lower = (float)(0.0 - 1e-6);
  const float upper = (float)(1.0 + 1e-6);
  int inside = pc[0] >= lower && pc[0] <= upper && pc[1] >= lower &&
               pc[1] <= upper && pc[2] >= lower && pc[2] <= upper;
  if (isWedge) inside = inside && (pc[0] + pc[1] <= upper);
  if (!inside) return 0;
  float val = 0.f;
  for (int i = 0; i < NV; i++) val += w[i] * V[i].w;
  *value = val;
  return 1;
}

int oc_intersect_pyr(float *value, v3 P, const v4 *v)
{
  return newton_elem(value, P, v, 5, pyr_fns, pyr_derivs, 0);
}
int oc_intersect_wedge(float *value, v3 P, const v4 *v)
{
  return newton_elem(value, P, v, 6, wedge_fns, wedge_derivs, 1);
}
int oc_intersect_hex(float *value, v3 P, const v4 *v)
{
  return newton_elem(value, P, v, 8, hex_fns, hex_derivs, 0);
}

/* sampler/programs/ExaStitchSampler.cu:133-161: vertex count selects the
 * element type (4 tet, 5 pyramid, 6 wedge, 8 hex) */
int oc_intersect_elem(float *value, v3 P, const int32_t *idx, const v4 *vertices)
{
  v4 v[8];
  int nv = 0;
  for (int i = 0; i < 8; ++i)
    if (idx[i] >= 0) { nv++; v[i] = vertices[idx[i]]; }
  if (nv == 4) return oc_intersect_tet(value, P, v[0], v[1], v[2], v[3]);
  if (nv == 5) return oc_intersect_pyr(value, P, v);
  if (nv == 6) return oc_intersect_wedge(value, P, v);
  if (nv == 8) return oc_intersect_hex(value, P, v);
  return 0;
}

/* Grid.cuh:51-59 */
v3i oc_project_on_grid(v3 V, v3i dims, exa_box3f b)
{
  const v3 V01 = div3(sub3(V, b.lower), sub3(b.upper, b.lower));
  v3i r;
  r.x = iclamp((int)(V01.x * (float)dims.x), 0, dims.x - 1);
  r.y = iclamp((int)(V01.y * (float)dims.y), 0, dims.y - 1);
  r.z = iclamp((int)(V01.z * (float)dims.z), 0, dims.z - 1);
  return r;
}

/* ================================================================== */
/* field container + uniform-grid point-location accel                 */
/* ================================================================== */
struct oc_field {
  const v4 *vertices; uint64_t numVertices;
  const int32_t *indices; uint64_t numElems;
  const exa_gridlet *gridlets; uint64_t numGridlets;
  const float *scalars; uint64_t numScalars;
  const float *gridletMaxOps, *elemMaxOps;
  /* accel: uniform grid over the union of primitive bounds; each cell
   * lists every primitive whose closed AABB touches it (gridlets first,
   * then elements, each in ascending index) */
  exa_box3f gb; v3i gd; v3 cs;
  uint32_t *cellBegin; /* gd.x*gd.y*gd.z + 1 */
  int32_t *items;      /* >= 0: gridlet id; < 0: -(elem id) - 1 */
  /* AMR cells (oc_field_set_amr): the field is their tent-basis
   * reconstruction; cells are looked up by (level, z, y, x) keys sorted
   * ascending, lattice boxes per level as the GPU builds them */
  const int32_t *amrCells; uint64_t numAmr;
  const float *amrScalars;
  uint64_t *amrKeys; uint32_t *amrOrder;
  int amrLevels;
  int amrHas[16], amrLo[16][3], amrN[16][3];
  /* ExaBricks (oc_field_set_bricks): bricks, their scalars, the active
   * brick regions built here; the uniform grid above then lists regions */
  const exa_brick *bricks; uint64_t numBricks;
  const float *brickScalars;
  exa_abr *abrs; uint64_t numAbrs;
  int32_t *leafList; uint64_t leafListSize, leafListCap;
  /* surface mesh, traced where lp->meshBVH != 0 */
  const exa_vec3f *meshVertices;
  const exa_vec3i *meshIndices;
  uint64_t numTris;
};

static exa_box3f gridlet_bounds(const exa_gridlet *g)
{
  const float cw = (float)(1 << g->level);
  exa_box3f b;
  b.lower = muls(mk3((float)g->lower.x + 0.5f, (float)g->lower.y + 0.5f,
                     (float)g->lower.z + 0.5f), cw);
  b.upper = muls(mk3(((float)g->lower.x + (float)g->dims.x) + 0.5f,
                     ((float)g->lower.y + (float)g->dims.y) + 0.5f,
                     ((float)g->lower.z + (float)g->dims.z) + 0.5f), cw);
  return b;
}

static exa_box3f elem_bounds(const oc_field *f, uint64_t e)
{
  exa_box3f b;
  b.lower = mk3(INFINITY, INFINITY, INFINITY);
  b.upper = mk3(-INFINITY, -INFINITY, -INFINITY);
  for (int i = 0; i < 8; ++i) {
    const int idx = f->indices[e * 8 + i];
    if (idx < 0) break;
    const v3 p = xyz(f->vertices[idx]);
    b.lower = min3(b.lower, p);
    b.upper = max3(b.upper, p);
  }
  return b;
}

static void cell_range(const oc_field *f, exa_box3f b, v3i *lo, v3i *hi)
{
  lo->x = iclamp((int)floorf((b.lower.x - f->gb.lower.x) / f->cs.x), 0, f->gd.x - 1);
  lo->y = iclamp((int)floorf((b.lower.y - f->gb.lower.y) / f->cs.y), 0, f->gd.y - 1);
  lo->z = iclamp((int)floorf((b.lower.z - f->gb.lower.z) / f->cs.z), 0, f->gd.z - 1);
  hi->x = iclamp((int)floorf((b.upper.x - f->gb.lower.x) / f->cs.x), 0, f->gd.x - 1);
  hi->y = iclamp((int)floorf((b.upper.y - f->gb.lower.y) / f->cs.y), 0, f->gd.y - 1);
  hi->z = iclamp((int)floorf((b.upper.z - f->gb.lower.z) / f->cs.z), 0, f->gd.z - 1);
}

oc_field *oc_field_create(const v4 *vertices, uint64_t numVertices,
                          const int32_t *indices, uint64_t numElems,
                          const exa_gridlet *gridlets, uint64_t numGridlets,
                          const float *scalars, uint64_t numScalars)
{
  oc_field *f = (oc_field *)calloc(1, sizeof(oc_field));
  f->vertices = vertices; f->numVertices = numVertices;
  f->indices = indices; f->numElems = numElems;
  f->gridlets = gridlets; f->numGridlets = numGridlets;
  f->scalars = scalars; f->numScalars = numScalars;
  exa_box3f all;
  all.lower = mk3(INFINITY, INFINITY, INFINITY);
  all.upper = mk3(-INFINITY, -INFINITY, -INFINITY);
  double vol = 0.0;
  for (uint64_t g = 0; g < numGridlets; ++g) {
    const exa_box3f b = gridlet_bounds(&gridlets[g]);
    all.lower = min3(all.lower, b.lower); all.upper = max3(all.upper, b.upper);
  }
  for (uint64_t e = 0; e < numElems; ++e) {
    const exa_box3f b = elem_bounds(f, e);
    all.lower = min3(all.lower, b.lower); all.upper = max3(all.upper, b.upper);
    vol += (double)(b.upper.x - b.lower.x) * (b.upper.y - b.lower.y) * (b.upper.z - b.lower.z);
  }
  if (numGridlets + numElems == 0) {
    all.lower = mk3(0.f, 0.f, 0.f); all.upper = mk3(1.f, 1.f, 1.f);
  }
  f->gb = all;
  /* cell size: about the mean element extent, at most 256 cells per axis */
  const v3 ext = sub3(all.upper, all.lower);
  const double maxExt = fmax(fmax(ext.x, ext.y), ext.z);
  double cellW = numElems ? cbrt(vol / (double)numElems) * 2.0 : maxExt / 32.0;
  if (cellW < maxExt / 256.0) cellW = maxExt / 256.0;
  if (cellW <= 0.0) cellW = 1.0;
  f->gd.x = imax_t(1, (int)ceil(ext.x / cellW));
  f->gd.y = imax_t(1, (int)ceil(ext.y / cellW));
  f->gd.z = imax_t(1, (int)ceil(ext.z / cellW));
  f->cs = mk3(fmax_t(ext.x, 1e-30f) / (float)f->gd.x, fmax_t(ext.y, 1e-30f) / (float)f->gd.y,
              fmax_t(ext.z, 1e-30f) / (float)f->gd.z);
  const uint64_t nc = (uint64_t)f->gd.x * f->gd.y * f->gd.z;
  f->cellBegin = (uint32_t *)calloc(nc + 1, sizeof(uint32_t));
  /* two passes: count, then fill */
  for (int pass = 0; pass < 2; ++pass) {
    uint32_t *cursor = NULL;
    if (pass == 1) {
      uint64_t acc = 0;
      for (uint64_t c = 0; c < nc; ++c) { const uint32_t k = f->cellBegin[c]; f->cellBegin[c] = (uint32_t)acc; acc += k; }
      f->cellBegin[nc] = (uint32_t)acc;
      f->items = (int32_t *)malloc((acc ? acc : 1) * sizeof(int32_t));
      cursor = (uint32_t *)malloc(nc * sizeof(uint32_t));
      memcpy(cursor, f->cellBegin, nc * sizeof(uint32_t));
    }
    for (uint64_t k = 0; k < numGridlets + numElems; ++k) {
      exa_box3f b = k < numGridlets ? gridlet_bounds(&gridlets[k]) : elem_bounds(f, k - numGridlets);
      v3i lo, hi;
      cell_range(f, b, &lo, &hi);
      for (int z = lo.z; z <= hi.z; ++z)
        for (int y = lo.y; y <= hi.y; ++y)
          for (int x = lo.x; x <= hi.x; ++x) {
            const uint64_t c = ((uint64_t)z * f->gd.y + y) * f->gd.x + x;
            if (pass == 0) f->cellBegin[c]++;
            else f->items[cursor[c]++] = k < numGridlets ? (int32_t)k : -(int32_t)(k - numGridlets) - 1;
          }
    }
    free(cursor);
  }
  return f;
}

void oc_field_destroy(oc_field *f)
{
  if (!f) return;
  free(f->abrs);
  free(f->leafList);
  free(f->amrKeys);
  free(f->amrOrder);
  free(f->cellBegin);
  free(f->items);
  free(f);
}

/* ------------------------------------------------ AMR cells
 * AMRCellSampler (sampler/AMRCellSampler.h:66-84, programs/
 * AMRCellSampler.cu:26-69): every cell whose support [pos - w/2,
 * pos + w + w/2] holds the point (inclusive) adds its scalar with the tent
 * weight prod(1 - |p - c| / (size / 2)); the sample is the weighted mean,
 * absent when the weights sum to 0.  Summation order (OptiX's is
 * unspecified): levels ascending, then cells in z, y, x order. */
static uint64_t amr_key(int level, int64_t x, int64_t y, int64_t z)
{
  return ((uint64_t)level << 60) | ((uint64_t)z << 40) | ((uint64_t)y << 20) | (uint64_t)x;
}

static const uint64_t *g_sort_keys;
static int amr_cmp(const void *a, const void *b)
{
  const uint64_t ka = g_sort_keys[*(const uint32_t *)a], kb = g_sort_keys[*(const uint32_t *)b];
  return ka < kb ? -1 : (ka > kb ? 1 : 0);
}

int oc_field_set_amr(oc_field *f, const int32_t *cells, uint64_t n, const float *scalars, uint64_t numScalars)
{
  if (numScalars < n) return 1;
  f->amrCells = cells;
  f->numAmr = n;
  f->amrScalars = scalars;
  f->amrLevels = 0;
  memset(f->amrHas, 0, sizeof(f->amrHas));
  int hi[16][3];
  for (uint64_t i = 0; i < n; ++i) {
    const int L = cells[i * 4 + 3];
    if (L < 0 || L > 15) return 2;
    for (int a = 0; a < 3; ++a) {
      const int q = cells[i * 4 + a] >> L;
      if (cells[i * 4 + a] & ((1 << L) - 1)) return 3;
      if (!f->amrHas[L] || q < f->amrLo[L][a]) f->amrLo[L][a] = q;
      if (!f->amrHas[L] || q > hi[L][a]) hi[L][a] = q;
    }
    f->amrHas[L] = 1;
    if (L + 1 > f->amrLevels) f->amrLevels = L + 1;
  }
  for (int L = 0; L < 16; ++L)
    for (int a = 0; a < 3; ++a) f->amrN[L][a] = f->amrHas[L] ? hi[L][a] - f->amrLo[L][a] + 1 : 0;
  free(f->amrKeys);
  free(f->amrOrder);
  f->amrKeys = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
  f->amrOrder = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
  uint64_t *k = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
  for (uint64_t i = 0; i < n; ++i) {
    const int L = cells[i * 4 + 3];
    const int64_t x = (cells[i * 4] >> L) - f->amrLo[L][0], y = (cells[i * 4 + 1] >> L) - f->amrLo[L][1],
                  z = (cells[i * 4 + 2] >> L) - f->amrLo[L][2];
    if (x >= (1 << 20) || y >= (1 << 20) || z >= (1 << 20)) { free(k); return 4; }
    k[i] = amr_key(L, x, y, z);
    f->amrOrder[i] = (uint32_t)i;
  }
  g_sort_keys = k;
  qsort(f->amrOrder, n, sizeof(uint32_t), amr_cmp);
  for (uint64_t i = 0; i < n; ++i) f->amrKeys[i] = k[f->amrOrder[i]];
  free(k);
  for (uint64_t i = 1; i < n; ++i)
    if (f->amrKeys[i] == f->amrKeys[i - 1]) return 5; /* duplicate cell */
  return 0;
}

/* model cell index of level-L lattice cell (x, y, z), or -1 */
static int64_t amr_find(const oc_field *f, int L, int x, int y, int z)
{
  const int64_t lx = x - f->amrLo[L][0], ly = y - f->amrLo[L][1], lz = z - f->amrLo[L][2];
  if (lx < 0 || ly < 0 || lz < 0 || lx >= f->amrN[L][0] || ly >= f->amrN[L][1] || lz >= f->amrN[L][2]) return -1;
  const uint64_t key = amr_key(L, lx, ly, lz);
  uint64_t lo = 0, hi = f->numAmr;
  while (lo < hi) {
    const uint64_t m = (lo + hi) / 2;
    if (f->amrKeys[m] < key) lo = m + 1; else hi = m;
  }
  return lo < f->numAmr && f->amrKeys[lo] == key ? (int64_t)f->amrOrder[lo] : -1;
}

static exa_sample amr_sample(const oc_field *f, v3 pos)
{
  float sumW = 0.f, sumWV = 0.f;
  const float P[3] = {pos.x, pos.y, pos.z};
  for (int L = 0; L < f->amrLevels; ++L) {
    if (!f->amrHas[L]) continue;
    const int w = 1 << L;
    const float half = (float)w * .5f;
    int cand[3][3], nc[3] = {0, 0, 0};
    int any = 1;
    for (int a = 0; a < 3 && any; ++a) {
      nc[a] = 0;
      const float q = floorf(P[a] / (float)w);
      if (!(q >= (float)f->amrLo[L][a] - 2.f && q <= (float)(f->amrLo[L][a] + f->amrN[L][a]) + 1.f)) { any = 0; break; }
      const int b = (int)q;
      for (int i = b - 1; i <= b + 1; ++i) {
        if (i < f->amrLo[L][a] || i >= f->amrLo[L][a] + f->amrN[L][a]) continue;
        const float lower = (float)(i * w) - half, upper = (float)(i * w + w) + half;
        if (lower <= P[a] && P[a] <= upper) cand[a][nc[a]++] = i;
      }
      any = nc[a] > 0;
    }
    if (!any) continue;
    for (int kz = 0; kz < nc[2]; ++kz)
      for (int ky = 0; ky < nc[1]; ++ky)
        for (int kx = 0; kx < nc[0]; ++kx) {
          const int id[3] = {cand[0][kx], cand[1][ky], cand[2][kz]};
          const int64_t c = amr_find(f, L, id[0], id[1], id[2]);
          if (c < 0) continue;
          float wgt = 1.f;
          for (int a = 0; a < 3; ++a) {
            const float lower = (float)(id[a] * w) - half, upper = (float)(id[a] * w + w) + half;
            const float center = (lower + upper) / 2.f, size = upper - lower;
            wgt = wgt * (1.f - fabsf(P[a] - center) / (size * .5f));
          }
          const float scalar = f->amrScalars[c];
          sumW += wgt;
          sumWV += scalar * wgt;
        }
  }
  exa_sample s = {-1, -1, 0.f};
  if (sumW > 0.f) { s.primID = 0; s.value = sumWV / sumW; }
  return s;
}

/* ------------------------------------------------ ExaBricks
 * ABRs::buildFrom / buildRec / addLeaf / computeValueRange (model/ABRs.cpp)
 * and ExaBrickSampler's sample() in the grid + DDA traversal mode
 * (sampler/ExaBrickSampler.h:113-239).  Split choice: the primitive face
 * closest to the domain centre per axis, the widest axis first (ties: the
 * lowest axis); the upper half is recursed into first; a region lists its
 * bricks in ascending id order.  Sampling takes the lowest-index region
 * whose closed domain holds the point (OptiX's order is unspecified). */
static inline int64_t lookup_cell(const oc_field *f, v3 p);

typedef struct { float lo[3], hi[3]; int id; } bprim;

static void abr_add_leaf(oc_field *f, const bprim *p, size_t n, const float *lo, const float *hi)
{
  for (int a = 0; a < 3; ++a)
    if (lo[a] >= hi[a]) return;
  if (!n) return;
  int *ids = (int *)malloc(n * sizeof(int));
  for (size_t i = 0; i < n; ++i) ids[i] = p[i].id;
  /* ascending unique ids (std::set) */
  for (size_t i = 1; i < n; ++i) {
    const int v = ids[i];
    size_t j = i;
    while (j > 0 && ids[j - 1] > v) { ids[j] = ids[j - 1]; --j; }
    ids[j] = v;
  }
  size_t u = 0;
  for (size_t i = 0; i < n; ++i)
    if (i == 0 || ids[i] != ids[i - 1]) ids[u++] = ids[i];
  if (f->leafListSize + u > f->leafListCap) {
    f->leafListCap = (f->leafListSize + u) * 2 + 16;
    f->leafList = (int32_t *)realloc(f->leafList, f->leafListCap * sizeof(int32_t));
  }
  exa_abr r;
  memset(&r, 0, sizeof(r));
  r.domain.lower = mk3(lo[0], lo[1], lo[2]);
  r.domain.upper = mk3(hi[0], hi[1], hi[2]);
  r.leafListBegin = (int32_t)f->leafListSize;
  r.leafListSize = (int32_t)u;
  for (size_t i = 0; i < u; ++i) f->leafList[f->leafListSize++] = ids[i];
  free(ids);
  f->abrs = (exa_abr *)realloc(f->abrs, (f->numAbrs + 1) * sizeof(exa_abr));
  f->abrs[f->numAbrs++] = r;
}

static void abr_build_rec(oc_field *f, bprim *p, size_t n, const float *lo, const float *hi)
{
  if (!n) { free(p); return; }
  for (int a = 0; a < 3; ++a)
    if (hi[a] == lo[a]) { free(p); return; }
  float tgt[3], bestPos[3], bestDist[3], span[3];
  for (int a = 0; a < 3; ++a) {
    tgt[a] = (lo[a] + hi[a]) * 0.5f;
    bestPos[a] = lo[a];
    span[a] = hi[a] - lo[a];
    bestDist[a] = span[a];
  }
  for (size_t i = 0; i < n; ++i)
    for (int dim = 0; dim < 3; ++dim)
      for (int side = 0; side < 2; ++side) {
        const float pos = side ? p[i].lo[dim] : p[i].hi[dim];
        if (pos <= lo[dim] || pos >= hi[dim]) continue;
        const float dist = fabsf(tgt[dim] - pos);
        if (dist < bestDist[dim]) { bestPos[dim] = pos; bestDist[dim] = dist; }
      }
  const int widest = (span[0] >= span[1] && span[0] >= span[2]) ? 0 : (span[1] >= span[2] ? 1 : 2);
  int splitDim = -1;
  float splitPos = 0.f;
  for (int i = 0; i < 3; ++i) {
    const int dim = (widest + i) % 3;
    if (bestPos[dim] <= lo[dim] || bestPos[dim] >= hi[dim]) continue;
    splitDim = dim;
    splitPos = bestPos[dim];
    break;
  }
  if (splitDim < 0) { abr_add_leaf(f, p, n, lo, hi); free(p); return; }
  float lhi[3] = {hi[0], hi[1], hi[2]}, rlo[3] = {lo[0], lo[1], lo[2]};
  lhi[splitDim] = splitPos;
  rlo[splitDim] = splitPos;
  bprim *pl = (bprim *)malloc(n * sizeof(bprim)), *pr = (bprim *)malloc(n * sizeof(bprim));
  size_t nl = 0, nr = 0;
  for (size_t i = 0; i < n; ++i) {
    bprim cl, cr;
    int okl = 1, okr = 1;
    for (int a = 0; a < 3; ++a) {
      cl.lo[a] = fmax_t(p[i].lo[a], lo[a]); cl.hi[a] = fmin_t(p[i].hi[a], lhi[a]);
      cr.lo[a] = fmax_t(p[i].lo[a], rlo[a]); cr.hi[a] = fmin_t(p[i].hi[a], hi[a]);
      okl = okl && cl.lo[a] < cl.hi[a];
      okr = okr && cr.lo[a] < cr.hi[a];
    }
    cl.id = cr.id = p[i].id;
    if (okl) pl[nl++] = cl;
    if (okr) pr[nr++] = cr;
  }
  free(p);
  abr_build_rec(f, pr, nr, rlo, hi);
  abr_build_rec(f, pl, nl, lo, lhi);
}

static void abr_value_range(exa_abr *r, const exa_brick *bricks, const float *scalars, const int32_t *leafList)
{
  r->valueRange.lower = 1e30f;
  r->valueRange.upper = -1e30f;
  const float dlo[3] = {r->domain.lower.x, r->domain.lower.y, r->domain.lower.z};
  const float dhi[3] = {r->domain.upper.x, r->domain.upper.y, r->domain.upper.z};
  for (int i = 0; i < r->leafListSize; ++i) {
    const exa_brick *b = &bricks[leafList[r->leafListBegin + i]];
    const float cw = (float)(1 << b->level);
    const int lower[3] = {b->lower.x, b->lower.y, b->lower.z}, size[3] = {b->size.x, b->size.y, b->size.z};
    for (int iz = 0; iz < size[2]; ++iz) {
      const float pz = (float)lower[2] + ((float)iz + .5f) * cw;
      if (!((pz - cw) <= dhi[2] && (pz + cw) >= dlo[2])) continue;
      for (int iy = 0; iy < size[1]; ++iy) {
        const float py = (float)lower[1] + ((float)iy + .5f) * cw;
        if (!((py - cw) <= dhi[1] && (py + cw) >= dlo[1])) continue;
        for (int ix = 0; ix < size[0]; ++ix) {
          const float px = (float)lower[0] + ((float)ix + .5f) * cw;
          if (!((px - cw) <= dhi[0] && (px + cw) >= dlo[0])) continue;
          const float v = scalars[(size_t)b->begin + ix + (size_t)size[0] * iy + (size_t)size[0] * size[1] * iz];
          if (v < r->valueRange.lower) r->valueRange.lower = v;
          if (r->valueRange.upper < v) r->valueRange.upper = v;
        }
      }
    }
  }
}

int oc_field_set_bricks(oc_field *f, const exa_brick *bricks, uint64_t nb, const float *scalars, uint64_t ns)
{
  for (uint64_t i = 0; i < nb; ++i) {
    if (bricks[i].level < 0 || bricks[i].level > 30) return 1;
    if (bricks[i].size.x < 1 || bricks[i].size.y < 1 || bricks[i].size.z < 1) return 2;
    if ((uint64_t)bricks[i].begin + (uint64_t)bricks[i].size.x * bricks[i].size.y * bricks[i].size.z > ns) return 3;
  }
  f->bricks = bricks; f->numBricks = nb; f->brickScalars = scalars;
  free(f->abrs); free(f->leafList);
  f->abrs = NULL; f->numAbrs = 0; f->leafList = NULL; f->leafListSize = f->leafListCap = 0;
  bprim *p = (bprim *)malloc((nb ? nb : 1) * sizeof(bprim));
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint64_t i = 0; i < nb; ++i) {
    const float cw = (float)(1 << bricks[i].level);
    const int lower[3] = {bricks[i].lower.x, bricks[i].lower.y, bricks[i].lower.z};
    const int size[3] = {bricks[i].size.x, bricks[i].size.y, bricks[i].size.z};
    for (int a = 0; a < 3; ++a) {
      p[i].lo[a] = (float)lower[a] - 0.5f * cw;                 /* ExaBrick::getDomain */
      p[i].hi[a] = (float)lower[a] + ((float)size[a] + 0.5f) * cw;
      lo[a] = fmin_t(lo[a], p[i].lo[a]);
      hi[a] = fmax_t(hi[a], p[i].hi[a]);
    }
    p[i].id = (int)i;
  }
  abr_build_rec(f, p, nb, lo, hi);
  for (uint64_t i = 0; i < f->numAbrs; ++i) {
    exa_abr *r = &f->abrs[i];
    int finest = 1 << 30;
    for (int k = 0; k < r->leafListSize; ++k) finest = imin_t(finest, bricks[f->leafList[r->leafListBegin + k]].level);
    r->finestLevelCellWidth = (float)(1 << finest);
    abr_value_range(r, bricks, scalars, f->leafList);
  }
  /* the uniform grid lists regions (closed boxes) in ascending index */
  free(f->cellBegin); free(f->items);
  exa_box3f all;
  all.lower = mk3(lo[0], lo[1], lo[2]);
  all.upper = mk3(hi[0], hi[1], hi[2]);
  if (!nb) { all.lower = mk3(0.f, 0.f, 0.f); all.upper = mk3(1.f, 1.f, 1.f); }
  f->gb = all;
  const v3 ext = sub3(all.upper, all.lower);
  const double maxExt = fmax(fmax(ext.x, ext.y), ext.z);
  double cellW = maxExt / fmin(256.0, fmax(4.0, 2.0 * cbrt((double)f->numAbrs)));
  if (cellW <= 0.0) cellW = 1.0;
  f->gd.x = imax_t(1, (int)ceil(ext.x / cellW));
  f->gd.y = imax_t(1, (int)ceil(ext.y / cellW));
  f->gd.z = imax_t(1, (int)ceil(ext.z / cellW));
  f->cs = mk3(fmax_t(ext.x, 1e-30f) / (float)f->gd.x, fmax_t(ext.y, 1e-30f) / (float)f->gd.y,
              fmax_t(ext.z, 1e-30f) / (float)f->gd.z);
  const uint64_t nc = (uint64_t)f->gd.x * f->gd.y * f->gd.z;
  f->cellBegin = (uint32_t *)calloc(nc + 1, sizeof(uint32_t));
  f->items = NULL;
  for (int pass = 0; pass < 2; ++pass) {
    uint32_t *cursor = NULL;
    if (pass == 1) {
      uint64_t acc = 0;
      for (uint64_t c = 0; c < nc; ++c) { const uint32_t k = f->cellBegin[c]; f->cellBegin[c] = (uint32_t)acc; acc += k; }
      f->cellBegin[nc] = (uint32_t)acc;
      f->items = (int32_t *)malloc((acc ? acc : 1) * sizeof(int32_t));
      cursor = (uint32_t *)malloc(nc * sizeof(uint32_t));
      memcpy(cursor, f->cellBegin, nc * sizeof(uint32_t));
    }
    for (uint64_t k = 0; k < f->numAbrs; ++k) {
      v3i a, b;
      cell_range(f, f->abrs[k].domain, &a, &b);
      for (int z = a.z; z <= b.z; ++z)
        for (int y = a.y; y <= b.y; ++y)
          for (int x = a.x; x <= b.x; ++x) {
            const uint64_t c = ((uint64_t)z * f->gd.y + y) * f->gd.x + x;
            if (pass == 0) f->cellBegin[c]++;
            else f->items[cursor[c]++] = (int32_t)k;
          }
    }
    free(cursor);
  }
  return 0;
}

void oc_field_abrs(const oc_field *f, const exa_abr **abrs, uint64_t *numAbrs, const int32_t **leafList,
                   uint64_t *leafListSize)
{
  *abrs = f->abrs; *numAbrs = f->numAbrs; *leafList = f->leafList; *leafListSize = f->leafListSize;
}

/* addBasisFunctions (sampler/ExaBrickSampler.h:113-200) */
static void add_basis(const oc_field *f, int brickID, v3 pos, float *sumWV, float *sumW)
{
  const exa_brick *b = &f->bricks[brickID];
  const float cw = (float)(1 << b->level);
  const float lx = (pos.x - (float)b->lower.x) / cw - .5f;
  const float ly = (pos.y - (float)b->lower.y) / cw - .5f;
  const float lz = (pos.z - (float)b->lower.z) / cw - .5f;
  const int ilx = imax_t(-1, (int)floorf(lx)), ily = imax_t(-1, (int)floorf(ly)), ilz = imax_t(-1, (int)floorf(lz));
  const int ihx = ilx + 1, ihy = ily + 1, ihz = ilz + 1;
  const float fx = lx - (float)ilx, fy = ly - (float)ily, fz = lz - (float)ilz;
  const float nx = 1.f - fx, ny = 1.f - fy, nz = 1.f - fz;
  const float *S = f->brickScalars + b->begin;
  const int sx = b->size.x, sy = b->size.y, sz = b->size.z;
#define OC_ADD(x, y, z, w) do { const float wt = (w); const float sc = S[(x) + (y) * sx + (z) * sx * sy]; \
    *sumW += wt; *sumWV += wt * sc; } while (0)
  if (ilz >= 0 && ilz < sz) {
    if (ily >= 0 && ily < sy) {
      if (ilx >= 0 && ilx < sx) OC_ADD(ilx, ily, ilz, nz * ny * nx);
      if (ihx < sx) OC_ADD(ihx, ily, ilz, nz * ny * fx);
    }
    if (ihy < sy) {
      if (ilx >= 0 && ilx < sx) OC_ADD(ilx, ihy, ilz, nz * fy * nx);
      if (ihx < sx) OC_ADD(ihx, ihy, ilz, nz * fy * fx);
    }
  }
  if (ihz < sz) {
    if (ily >= 0 && ily < sy) {
      if (ilx >= 0 && ilx < sx) OC_ADD(ilx, ily, ihz, fz * ny * nx);
      if (ihx < sx) OC_ADD(ihx, ily, ihz, fz * ny * fx);
    }
    if (ihy < sy) {
      if (ilx >= 0 && ilx < sx) OC_ADD(ilx, ihy, ihz, fz * fy * nx);
      if (ihx < sx) OC_ADD(ihx, ihy, ihz, fz * fy * fx);
    }
  }
#undef OC_ADD
}

static exa_sample brick_sample(const oc_field *f, v3 pos)
{
  exa_sample s = {0, -1, 0.f};
  const int64_t c = lookup_cell(f, pos);
  if (c < 0) return s;
  int best = -1;
  for (uint32_t i = f->cellBegin[c]; i < f->cellBegin[c + 1]; ++i) {
    const exa_abr *r = &f->abrs[f->items[i]];
    if (r->domain.lower.x <= pos.x && r->domain.lower.y <= pos.y && r->domain.lower.z <= pos.z &&
        pos.x <= r->domain.upper.x && pos.y <= r->domain.upper.y && pos.z <= r->domain.upper.z) {
      best = f->items[i];
      break;
    }
  }
  if (best < 0) return s;
  const exa_abr *r = &f->abrs[best];
  float sumWV = 0.f, sumW = 0.f;
  for (int i = 0; i < r->leafListSize; ++i) add_basis(f, f->leafList[r->leafListBegin + i], pos, &sumWV, &sumW);
  if (sumW > 0.f) s.value = sumWV / sumW;
  return s;
}

void oc_field_set_mesh(oc_field *f, const exa_vec3f *vertices, const exa_vec3i *indices, uint64_t numTris)
{
  f->meshVertices = vertices;
  f->meshIndices = indices;
  f->numTris = numTris;
}

void oc_field_set_prim_opacities(oc_field *f, const float *g, const float *e)
{
  f->gridletMaxOps = g;
  f->elemMaxOps = e;
}

/* model/ExaStitchModel.cpp:78-109 and 224-245 */
void oc_field_bounds(const oc_field *f, exa_box3f *cb, exa_range1f *vr)
{
  exa_box3f b;
  b.lower = mk3(INFINITY, INFINITY, INFINITY);
  b.upper = mk3(-INFINITY, -INFINITY, -INFINITY);
  exa_range1f r = {1e30f, -1e30f};
  for (uint64_t e = 0; e < f->numElems; ++e)
    for (int j = 0; j < 8; ++j) {
      const int idx = f->indices[e * 8 + j];
      if (idx < 0) continue;
      const v4 v = f->vertices[idx];
      b.lower = min3(b.lower, xyz(v)); b.upper = max3(b.upper, xyz(v));
      /* std::min(lower, w): NaN never replaces the running value */
      if (v.w < r.lower) r.lower = v.w;
      if (r.upper < v.w) r.upper = v.w;
    }
  for (uint64_t g = 0; g < f->numGridlets; ++g) {
    const exa_gridlet *gl = &f->gridlets[g];
    const uint64_t n = (uint64_t)(gl->dims.x + 1) * (gl->dims.y + 1) * (gl->dims.z + 1);
    for (uint64_t i = 0; i < n; ++i) {
      const float s = f->scalars[gl->begin + i];
      if (s < r.lower) r.lower = s;
      if (r.upper < s) r.upper = s;
    }
    const exa_box3f gb = gridlet_bounds(gl);
    b.lower = min3(b.lower, gb.lower); b.upper = max3(b.upper, gb.lower);
    b.lower = min3(b.lower, gb.upper); b.upper = max3(b.upper, gb.upper);
  }
  /* ExaBrickModel::init (ExaBrickModel.cpp:157-166): bricks' bounds, the
   * regions' value ranges */
  for (uint64_t i = 0; i < f->numBricks; ++i) {
    const exa_brick *bk = &f->bricks[i];
    const int w = 1 << bk->level;
    const v3 lo = mk3((float)bk->lower.x, (float)bk->lower.y, (float)bk->lower.z);
    const v3 hi = mk3((float)(bk->lower.x + bk->size.x * w), (float)(bk->lower.y + bk->size.y * w),
                      (float)(bk->lower.z + bk->size.z * w));
    b.lower = min3(b.lower, lo); b.upper = max3(b.upper, lo);
    b.lower = min3(b.lower, hi); b.upper = max3(b.upper, hi);
  }
  for (uint64_t i = 0; i < f->numAbrs && f->numBricks; ++i) {
    r.lower = fminf(r.lower, f->abrs[i].valueRange.lower);
    r.upper = fmaxf(r.upper, f->abrs[i].valueRange.upper);
  }
  /* AMRCellModel::load (AMRCellModel.cpp:56-64) */
  for (uint64_t i = 0; i < f->numAmr; ++i) {
    const int32_t *c = &f->amrCells[i * 4];
    const int w = 1 << c[3];
    const v3 lo = mk3((float)c[0], (float)c[1], (float)c[2]);
    const v3 hi = mk3((float)(c[0] + w), (float)(c[1] + w), (float)(c[2] + w));
    b.lower = min3(b.lower, lo); b.upper = max3(b.upper, lo);
    b.lower = min3(b.lower, hi); b.upper = max3(b.upper, hi);
    const float s = f->amrScalars[i];
    if (s < r.lower) r.lower = s;
    if (r.upper < s) r.upper = s;
  }
  *cb = b;
  *vr = r;
}

static inline int gridlet_visible(const oc_field *f, int g, int cull)
{
  return !(cull && f->gridletMaxOps && f->gridletMaxOps[g] == 0.f);
}
static inline int elem_visible(const oc_field *f, int e, int cull)
{
  return !(cull && f->elemMaxOps && f->elemMaxOps[e] == 0.f);
}

/* an element is a candidate only where its bounding box (the box of its
 * vertices, StitchGeomBounds_Impl in programs/ExaStitchSampler.cu:73-92)
 * holds the point, inclusively: OptiX calls the intersection program only
 * for primitives whose box the query ray meets, and the element tests'
 * tolerances (UElems.h) accept points just outside an element */
static inline int elem_box_contains(const oc_field *f, int e, v3 p)
{
  const int32_t *I = &f->indices[(uint64_t)e * 8];
  v3 lo = mk3(INFINITY, INFINITY, INFINITY), hi = mk3(-INFINITY, -INFINITY, -INFINITY);
  for (int i = 0; i < 8 && I[i] >= 0; ++i) {
    const v4 v = f->vertices[I[i]];
    lo = mk3(fmin_t(lo.x, v.x), fmin_t(lo.y, v.y), fmin_t(lo.z, v.z));
    hi = mk3(fmax_t(hi.x, v.x), fmax_t(hi.y, v.y), fmax_t(hi.z, v.z));
  }
  return p.x >= lo.x && p.y >= lo.y && p.z >= lo.z && p.x <= hi.x && p.y <= hi.y && p.z <= hi.z;
}

static inline int64_t lookup_cell(const oc_field *f, v3 p)
{
  if (!(p.x >= f->gb.lower.x && p.y >= f->gb.lower.y && p.z >= f->gb.lower.z &&
        p.x <= f->gb.upper.x && p.y <= f->gb.upper.y && p.z <= f->gb.upper.z))
    return -1;
  const int x = iclamp((int)floorf((p.x - f->gb.lower.x) / f->cs.x), 0, f->gd.x - 1);
  const int y = iclamp((int)floorf((p.y - f->gb.lower.y) / f->cs.y), 0, f->gd.y - 1);
  const int z = iclamp((int)floorf((p.z - f->gb.lower.z) / f->cs.z), 0, f->gd.z - 1);
  return ((int64_t)z * f->gd.y + y) * f->gd.x + x;
}

/* sample() (sampler/ExaStitchSampler.h:128-140) with the OptiX query
 * replaced by the canonical rule: lowest-index containing gridlet, else
 * lowest-index containing element; primitives with max opacity 0 are
 * invisible when culling (programs/ExaStitchSampler.cu:35-41,81-83). */
exa_sample oc_sample(const oc_field *f, v3 pos, int cull)
{
  if (f->numAmr) return amr_sample(f, pos);
  if (f->numBricks) return brick_sample(f, pos);
  exa_sample s = {-1, -1, 0.f};
  const int64_t c = lookup_cell(f, pos);
  if (c < 0) return s;
  int bestG = -1, bestE = -1;
  float gv = 0.f, ev = 0.f;
  int gc = -1;
  for (uint32_t i = f->cellBegin[c]; i < f->cellBegin[c + 1]; ++i) {
    const int32_t it = f->items[i];
    if (it >= 0) {
      if (bestG >= 0 && it >= bestG) continue;
      if (!gridlet_visible(f, it, cull)) continue;
      float v; int cid;
      if (oc_intersect_gridlet(&v, &cid, pos, &f->gridlets[it], f->scalars)) {
        bestG = it; gv = v; gc = cid;
      }
    } else if (bestG < 0) {
      const int e = -it - 1;
      if (bestE >= 0 && e >= bestE) continue;
      if (!elem_visible(f, e, cull) || !elem_box_contains(f, e, pos)) continue;
      float v;
      if (oc_intersect_elem(&v, pos, &f->indices[(uint64_t)e * 8], f->vertices)) {
        bestE = e; ev = v;
      }
    }
  }
  if (bestG >= 0) { s.primID = bestG; s.cellID = gc; s.value = gv; }
  else if (bestE >= 0) { s.primID = bestE; s.cellID = -1; s.value = ev; }
  return s;
}

void oc_sample_points(const oc_field *f, const v3 *pos, uint64_t n,
                      exa_sample *out, int cull, int nthreads)
{
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4096)
#endif
  for (int64_t i = 0; i < (int64_t)n; ++i) out[i] = oc_sample(f, pos[i], cull);
}

int oc_sample_all(const oc_field *f, v3 pos, int cull, int maxOut, int *kinds,
                  int *ids, float *values)
{
  int n = 0;
  for (uint64_t g = 0; g < f->numGridlets && n < maxOut; ++g) {
    if (!gridlet_visible(f, (int)g, cull)) continue;
    float v; int cid;
    if (oc_intersect_gridlet(&v, &cid, pos, &f->gridlets[g], f->scalars)) {
      kinds[n] = 0; ids[n] = (int)g; values[n] = v; n++;
    }
  }
  for (uint64_t e = 0; e < f->numElems && n < maxOut; ++e) {
    if (!elem_visible(f, (int)e, cull) || !elem_box_contains(f, (int)e, pos)) continue;
    float v;
    if (oc_intersect_elem(&v, pos, &f->indices[e * 8], f->vertices)) {
      kinds[n] = 1; ids[n] = (int)e; values[n] = v; n++;
    }
  }
  return n;
}

/* ================================================================== */
/* majorants: Grid.cu:43-246, 687-719; sampler/ExaStitchSampler.cu     */
/* ================================================================== */
static inline void update_mc(exa_range1f *vr, v3i id, v3i dims, exa_range1f r)
{
  /* Grid.cu:43-50: atomicMin/atomicMax (order independent) */
  exa_range1f *m = &vr[((size_t)id.z * dims.y + id.y) * dims.x + id.x];
  if (r.lower < m->lower) m->lower = r.lower;
  if (r.upper > m->upper) m->upper = r.upper;
}

void oc_build_majorants(const oc_field *f, v3i dims, exa_box3f wb, exa_range1f *vr)
{
  const size_t numMCs = (size_t)dims.x * dims.y * dims.z;
  for (size_t i = 0; i < numMCs; ++i) { vr[i].lower = 1e30f; vr[i].upper = -1e30f; } /* Grid.cu:61-70 */
  /* ExaBrick cells: the cell box grown by half a cell (Grid.cu:399-430) */
  for (uint64_t bi = 0; bi < f->numBricks; ++bi) {
    const exa_brick *b = &f->bricks[bi];
    const int w = 1 << b->level;
    const float half = (float)w * .5f;
    for (int z = 0; z < b->size.z; ++z)
      for (int y = 0; y < b->size.y; ++y)
        for (int x = 0; x < b->size.x; ++x) {
          const float value = f->brickScalars[(size_t)b->begin + x + (size_t)b->size.x * (y + (size_t)b->size.y * z)];
          if (isnan(value)) continue;
          const int lx = b->lower.x + x * w, ly = b->lower.y + y * w, lz = b->lower.z + z * w;
          const v3 lo3 = mk3((float)lx - half, (float)ly - half, (float)lz - half);
          const v3 hi3 = mk3((float)(lx + w) + half, (float)(ly + w) + half, (float)(lz + w) + half);
          const v3i lo = oc_project_on_grid(lo3, dims, wb), hi = oc_project_on_grid(hi3, dims, wb);
          const exa_range1f r = {value, value};
          for (int mz = lo.z; mz <= hi.z; ++mz)
            for (int my = lo.y; my <= hi.y; ++my)
              for (int mx = lo.x; mx <= hi.x; ++mx) { v3i id = {mx, my, mz}; update_mc(vr, id, dims, r); }
        }
  }
  /* AMR cells: the cell's support projected onto the grid (Grid.cu:248-285) */
  for (uint64_t i = 0; i < f->numAmr; ++i) {
    const int32_t *c = &f->amrCells[i * 4];
    const float value = f->amrScalars[i];
    if (isnan(value)) continue;
    const int w = 1 << c[3];
    const float half = (float)w * .5f;
    const v3 lo3 = mk3((float)c[0] - half, (float)c[1] - half, (float)c[2] - half);
    const v3 hi3 = mk3((float)(c[0] + w) + half, (float)(c[1] + w) + half, (float)(c[2] + w) + half);
    const v3i lo = oc_project_on_grid(lo3, dims, wb), hi = oc_project_on_grid(hi3, dims, wb);
    const exa_range1f r = {value, value};
    for (int z = lo.z; z <= hi.z; ++z)
      for (int y = lo.y; y <= hi.y; ++y)
        for (int x = lo.x; x <= hi.x; ++x) { v3i id = {x, y, z}; update_mc(vr, id, dims, r); }
  }
  /* elements: buildGrid<8> (Grid.cu:73-117) */
  for (uint64_t e = 0; e < f->numElems; ++e) {
    const int32_t *I = &f->indices[e * 8];
    exa_box3f cb;
    cb.lower = mk3(INFINITY, INFINITY, INFINITY);
    cb.upper = mk3(-INFINITY, -INFINITY, -INFINITY);
    exa_range1f r = {1e30f, -1e30f};
    int any = 0;
    for (int i = 0; i < 8; ++i) {
      if (I[i] < 0) break;
      const v4 V = f->vertices[I[i]];
      if (!isnan(V.w)) {
        cb.lower = min3(cb.lower, xyz(V)); cb.upper = max3(cb.upper, xyz(V));
        r.lower = fminf(r.lower, V.w); r.upper = fmaxf(r.upper, V.w);
        any = 1;
      }
    }
    if (!any) continue; /* empty box: the reference's loop adds nothing */
    const v3i lo = oc_project_on_grid(cb.lower, dims, wb);
    const v3i hi = oc_project_on_grid(cb.upper, dims, wb);
    for (int z = lo.z; z <= hi.z; ++z)
      for (int y = lo.y; y <= hi.y; ++y)
        for (int x = lo.x; x <= hi.x; ++x) { v3i id = {x, y, z}; update_mc(vr, id, dims, r); }
  }
  /* gridlets: buildGrid (Grid.cu:134-246), one (gridlet, cell) at a time */
  const v3 mcSize = div3(sub3(wb.upper, wb.lower), mk3((float)dims.x, (float)dims.y, (float)dims.z));
  for (uint64_t g = 0; g < f->numGridlets; ++g) {
    const exa_gridlet *gl = &f->gridlets[g];
    const exa_box3f gb = gridlet_bounds(gl);
    const v3i lo = oc_project_on_grid(gb.lower, dims, wb);
    const v3i hi = oc_project_on_grid(gb.upper, dims, wb);
    const int nx = gl->dims.x + 1, ny = gl->dims.y + 1;
    const float cw = (float)(1 << gl->level);
    const float *S = f->scalars + gl->begin;
    for (int z = 0; z < gl->dims.z; ++z)
      for (int y = 0; y < gl->dims.y; ++y)
        for (int x = 0; x < gl->dims.x; ++x) {
          exa_box3f cellB;
          cellB.lower = add3(muls(mk3((float)(gl->lower.x + x), (float)(gl->lower.y + y), (float)(gl->lower.z + z)), cw),
                             mk3(0.5f * cw, 0.5f * cw, 0.5f * cw));
          cellB.upper = add3(muls(mk3((float)(gl->lower.x + x + 1), (float)(gl->lower.y + y + 1), (float)(gl->lower.z + z + 1)), cw),
                             mk3(0.5f * cw, 0.5f * cw, 0.5f * cw));
          float fv[8];
          fv[0] = S[(z * ny + y) * nx + x];
          fv[1] = S[(z * ny + y) * nx + x + 1];
          fv[2] = S[(z * ny + y + 1) * nx + x];
          fv[3] = S[(z * ny + y + 1) * nx + x + 1];
          fv[4] = S[((z + 1) * ny + y) * nx + x];
          fv[5] = S[((z + 1) * ny + y) * nx + x + 1];
          fv[6] = S[((z + 1) * ny + y + 1) * nx + x];
          fv[7] = S[((z + 1) * ny + y + 1) * nx + x + 1];
          exa_range1f cr = {1e30f, -1e30f};
          for (int k = 0; k < 8; ++k)
            if (!isnan(fv[k])) { cr.lower = fminf(cr.lower, fv[k]); cr.upper = fmaxf(cr.upper, fv[k]); }
          for (int mz = lo.z; mz <= hi.z; ++mz)
            for (int my = lo.y; my <= hi.y; ++my)
              for (int mx = lo.x; mx <= hi.x; ++mx) {
                exa_box3f mb;
                mb.lower = add3(wb.lower, mul3(mk3((float)mx, (float)my, (float)mz), mcSize));
                mb.upper = add3(wb.lower, mul3(mk3((float)(mx + 1), (float)(my + 1), (float)(mz + 1)), mcSize));
                /* box3f::overlaps, inclusive */
                if (mb.lower.x <= cellB.upper.x && mb.lower.y <= cellB.upper.y && mb.lower.z <= cellB.upper.z &&
                    cellB.lower.x <= mb.upper.x && cellB.lower.y <= mb.upper.y && cellB.lower.z <= mb.upper.z) {
                  v3i id = {mx, my, mz};
                  update_mc(vr, id, dims, cr);
                }
              }
        }
  }
}

/* the entries the linear transfer-function filter (EXA_TF_FILTER_LINEAR)
 * can blend for normalised values in [l, u]: floor(l*N - 0.5) ..
 * floor(u*N - 0.5) + 1, clipped to the table; 0 when none is inside it */
static int tf_linear_span(float l, float u, int n, int *lo, int *hi)
{
  const float N = (float)n;
  const float a = floorf(l * N - 0.5f), b = floorf(u * N - 0.5f) + 1.f;
  if (!(b >= 0.f) || !(a <= N - 1.f)) return 0;
  *lo = a < 0.f ? 0 : (int)a;
  *hi = b > N - 1.f ? n - 1 : (int)b;
  return 1;
}

/* Grid.cu:687-719 (== computeGridletMaxOpacitiesGPU,
 * sampler/ExaStitchSampler.cu:144-176); under the linear filter the span
 * of tf_linear_span */
static float range_max_opacity(exa_range1f vr, const v4 *cm, int n, exa_range1f xf, int filter)
{
  if (vr.upper < vr.lower) return 0.f;
  vr.lower -= xf.lower;
  vr.lower /= xf.upper - xf.lower;
  vr.upper -= xf.lower;
  vr.upper /= xf.upper - xf.lower;
  int lo, hi;
  if (filter == EXA_TF_FILTER_LINEAR) {
    if (!tf_linear_span(vr.lower, vr.upper, n, &lo, &hi)) return 0.f;
  } else {
    lo = iclamp((int)(vr.lower * (float)(n - 1)), 0, n - 1);
    hi = iclamp((int)(vr.upper * (float)(n - 1)) + 1, 0, n - 1);
  }
  float m = 0.f;
  for (int i = lo; i <= hi; ++i) m = fmaxf(m, cm[i].w);
  return m;
}

void oc_compute_max_opacities(const exa_range1f *r, uint64_t n, const v4 *cm,
                              int nc, exa_range1f xf, int filter, float *out)
{
  for (uint64_t i = 0; i < n; ++i) out[i] = range_max_opacity(r[i], cm, nc, xf, filter);
}

/* sampler/ExaStitchSampler.cu:52-142: min/max over the non-NaN corners of
 * every cell == over every non-NaN scalar of the gridlet */
void oc_gridlet_value_ranges(const oc_field *f, exa_range1f *out)
{
  for (uint64_t g = 0; g < f->numGridlets; ++g) {
    const exa_gridlet *gl = &f->gridlets[g];
    exa_range1f r = {1e30f, -1e30f};
    const uint64_t n = (uint64_t)(gl->dims.x + 1) * (gl->dims.y + 1) * (gl->dims.z + 1);
    if (gl->dims.x > 0 && gl->dims.y > 0 && gl->dims.z > 0)
      for (uint64_t i = 0; i < n; ++i) {
        const float s = f->scalars[gl->begin + i];
        if (!isnan(s)) { r.lower = fminf(r.lower, s); r.upper = fmaxf(r.upper, s); }
      }
    out[g] = r;
  }
}

/* sampler/ExaStitchSampler.cu:178-227 (computeUmeshMaxOpacitiesGPU<8>) */
void oc_elem_max_opacities(const oc_field *f, const v4 *cm, int nc,
                           exa_range1f xf, int filter, float *out)
{
  for (uint64_t e = 0; e < f->numElems; ++e) {
    exa_range1f r = {1e30f, -1e30f};
    for (int i = 0; i < 8; ++i) {
      const int idx = f->indices[e * 8 + i];
      if (idx < 0) continue;
      const float w = f->vertices[idx].w;
      r.lower = fmin_t(r.lower, w);
      r.upper = fmax_t(r.upper, w);
    }
    out[e] = range_max_opacity(r, cm, nc, xf, filter);
  }
}

/* ================================================================== */
/* rendering (deviceCode.cu)                                           */
/* ================================================================== */
typedef struct { v3 org, dir; float tmin, tmax; } ray_t;

enum { BOUNDARY = 0, SCATTERING = 1 };

#define OC_TRACK_CAP (1 << 22)

typedef struct {
  const oc_field *f;
  const exa_launch_params *lp;
  uint32_t err;
  int px, py, width, height;  /* the pixel being rendered (Teaser shade mode) */
  uint64_t work;              /* heat map: DDA cells of the walks, march positions */
} rctx;

/* one channel of the linear filter: the blend of the two entries, limited
 * to their range */
static float tf_lerp(float p, float q, float a)
{
  const float r = (1.f - a) * p + a * q;
  return fminf(fmaxf(r, fminf(p, q)), fmaxf(p, q));
}

/* EXA_TF_FILTER_LINEAR: deviceCode.cu:331-332 (tex2D of the texture that
 * OWLRenderer.cpp:659-707 sets up: normalised coordinates, linear
 * filtering, border address mode with a zero border colour; at y = .5 of a
 * one-row texture only row 0 has weight) in binary32: xB = f*N - 0.5,
 * i = floor(xB), a = xB - i, (1-a)*T[i] + a*T[i+1] */
static v4 lookup_tf_linear(const v4 *T, int n, float f)
{
  v4 z = {0.f, 0.f, 0.f, 0.f};
  const float xB = f * (float)n - 0.5f;
  if (!(xB >= -1.f && xB < (float)n)) return z;
  const float fi = floorf(xB);
  const int i = (int)fi;
  const float a = xB - fi;
  const v4 p = i >= 0 ? T[i] : z;
  const v4 q = i + 1 < n ? T[i + 1] : z;
  v4 r = {tf_lerp(p.x, q.x, a), tf_lerp(p.y, q.y, a), tf_lerp(p.z, q.z, a), tf_lerp(p.w, q.w, a)};
  return r;
}

/* deviceCode.cu:320-341: the buffer variant, or the texture variant under
 * EXA_TF_FILTER_LINEAR */
static v4 lookup_tf(const exa_launch_params *lp, float f)
{
  const exa_range1f d = lp->transferFunc.domain;
  v4 zero = {0.f, 0.f, 0.f, 0.f};
  if (d.lower >= d.upper) return zero;
  f -= d.lower;
  f /= (d.upper - d.lower);
  if (lp->transferFunc.numValues == 0) return zero;
  if (lp->ext.tfFilter == EXA_TF_FILTER_LINEAR)
    return lookup_tf_linear(lp->transferFunc.values, lp->transferFunc.numValues, f);
  /* min(1, f) in std::min's operand order, as fminf also gives it: a NaN
   * value (an element with collapsed vertices passes its inside tests with
   * NaN weights) clamps to 1, the last entry, and no NaN reaches the
   * conversion to int */
  f = fmax_t(0.f, f < 1.f ? f : 1.f);
  const int i = imin_t(lp->transferFunc.numValues - 1, (int)(f * (float)lp->transferFunc.numValues));
  return lp->transferFunc.values[i];
}

/* the transfer-function lookup of lp (filter, domain, table) at value f */
void oc_lookup_tf(const exa_launch_params *lp, float f, exa_vec4f *out)
{
  const v4 r = lookup_tf(lp, f);
  out->x = r.x; out->y = r.y; out->z = r.z; out->w = r.w;
}

/* sampler/Sampler.h:105-122 */
static int box_test(ray_t r, exa_box3f b, float *t0, float *t1)
{
  const v3 lo = div3(sub3(b.lower, r.org), r.dir);
  const v3 hi = div3(sub3(b.upper, r.org), r.dir);
  const v3 nr = min3(lo, hi), fr = max3(lo, hi);
  *t0 = fmax_t(r.tmin, rmax3(nr));
  *t1 = fmin_t(r.tmax, rmin3(fr));
  return *t0 < *t1;
}

/* clip planes after the box test (deviceCode.cu:53-60 intersect; :882-893,
 * 1010-1021, 1097-1106, 1143-1154, 1229-1240): a front-facing plane moves
 * t0 forward, a back-facing one t1 back; a ray parallel to a plane gets
 * FLT_MAX with backFace false, which moves t0 to FLT_MAX */
static void clip_planes(const exa_launch_params *lp, ray_t r, float *t0, float *t1)
{
  for (int i = 0; i < EXA_CLIP_PLANES_MAX; ++i) {
    if (!lp->clipPlanes[i].enabled) continue;
    const v3 N = lp->clipPlanes[i].N;
    const float sd = dot3(N, r.dir);
    int backFace = 0;
    float pt = 3.40282347e+38f;
    if (sd != 0.f) {
      backFace = sd > 0.f;
      pt = (lp->clipPlanes[i].d - dot3(N, r.org)) / sd;
    }
    if (pt > *t0 && !backFace) *t0 = fmax_t(*t0, pt);
    if (pt < *t1 && backFace) *t1 = fmin_t(pt, *t1);
  }
}

/* sampler/ExaStitchSampler.h:108-126 */
static exa_sample test_sample(const oc_field *f, v3 pos, int primID)
{
  exa_sample s = {-1, -1, 0.f};
  if (primID < 0) return s;
  if (oc_intersect_gridlet(&s.value, &s.cellID, pos, &f->gridlets[primID], f->scalars))
    s.primID = primID;
  return s;
}

/* deviceCode.cu:625-651 (Default and Gridlets shade modes) */
static v4 classify(const rctx *c, exa_sample s)
{
  v4 xf = lookup_tf(c->lp, s.value);
  if (c->lp->shadeMode == EXA_SHADE_MODE_GRIDLETS) {
    if (s.cellID == -1) { xf.x = 1.f; xf.y = 0.f; xf.z = 0.f; }
    else {
      const exa_gridlet *g = &c->f->gridlets[s.primID];
      const int ix = s.cellID % g->dims.x;
      const int iy = s.cellID / g->dims.x % g->dims.y;
      const int iz = s.cellID / (g->dims.x * g->dims.y);
      int col = (ix % 2 == iy % 2);
      col = (iz % 2 == 0) ? col : !col;
      if (col == 0) { xf.x = 1.f; xf.y = 1.f; xf.z = 1.f; }
      else { xf.x = 0.f; xf.y = 0.f; xf.z = 0.7f; }
    }
  } else if (c->lp->shadeMode == EXA_SHADE_MODE_TEASER) {
    /* deviceCode.cu:652-695: the TF colour and the checker colour blended
     * across a screen-space diagonal band */
    v3 rgb2;
    if (s.cellID == -1) rgb2 = mk3(1.f, 0.f, 0.f);
    else {
      const exa_gridlet *g = &c->f->gridlets[s.primID];
      const int ix = s.cellID % g->dims.x;
      const int iy = s.cellID / g->dims.x % g->dims.y;
      const int iz = s.cellID / (g->dims.x * g->dims.y);
      int col = (ix % 2 == iy % 2);
      col = (iz % 2 == 0) ? col : !col;
      rgb2 = col == 0 ? mk3(1.f, 1.f, 1.f) : mk3(0.f, 0.f, .7f);
    }
    const v3 rgb1 = mk3(xf.x, xf.y, xf.z);
    const float u = (float)c->px / (float)c->width, v = (float)c->py / (float)c->height;
    const float A = .6f - .4f, B = .4f - .6f;
    const float C1 = A * .4f + B * .6f, C2 = A * .6f + B * .4f, C = A * u + B * v;
    if (C <= C1) { xf.x = rgb1.x; xf.y = rgb1.y; xf.z = rgb1.z; }
    else if (C >= C2) { xf.x = rgb2.x; xf.y = rgb2.y; xf.z = rgb2.z; }
    else {
      xf.x = (rgb1.x * (C2 - C) + rgb2.x * (C - C1)) / (C2 - C1);
      xf.y = (rgb1.y * (C2 - C) + rgb2.y * (C - C1)) / (C2 - C1);
      xf.z = (rgb1.z * (C2 - C) + rgb2.z * (C - C1)) / (C2 - C1);
    }
  }
  return xf;
}

/* dda3 (DDA.h:26-113) as a stepper: init = the prologue (:34-70), the
 * current cell is (leaf, t0, t1), next() = the tie-advancing step
 * (:352-375); next returns 0 when a stop index is reached. */
typedef struct {
  v3 tnext, dist;
  v3i cell, step, stop, dims;
  float t0, tmax;
} oc_dda;

static void dda_init(oc_dda *d, v3 org, v3 dir, float tmin, float tmax, v3i dims, exa_box3f mb)
{
  const v3 rcp = mk3(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
  const v3 lo = mul3(sub3(mb.lower, org), rcp);
  const v3 hi = mul3(sub3(mb.upper, org), rcp);
  const v3 tnear = min3(lo, hi), tfar = max3(lo, hi);
  d->dims = dims;
  d->cell = oc_project_on_grid(org, dims, mb);
  d->dist = div3(sub3(tfar, tnear), mk3((float)dims.x, (float)dims.y, (float)dims.z));
  d->step.x = dir.x > 0.f ? 1 : -1; d->step.y = dir.y > 0.f ? 1 : -1; d->step.z = dir.z > 0.f ? 1 : -1;
  d->stop.x = dir.x > 0.f ? dims.x : -1; d->stop.y = dir.y > 0.f ? dims.y : -1; d->stop.z = dir.z > 0.f ? dims.z : -1;
  d->tnext.x = dir.x > 0.f ? tnear.x + (float)(d->cell.x + 1) * d->dist.x : tnear.x + (float)(dims.x - d->cell.x) * d->dist.x;
  d->tnext.y = dir.y > 0.f ? tnear.y + (float)(d->cell.y + 1) * d->dist.y : tnear.y + (float)(dims.y - d->cell.y) * d->dist.y;
  d->tnext.z = dir.z > 0.f ? tnear.z + (float)(d->cell.z + 1) * d->dist.z : tnear.z + (float)(dims.z - d->cell.z) * d->dist.z;
  /* a direction component of 0 (or one whose reciprocal overflows) gives a
   * NaN crossing, on which DDA.h's loop never advances: that axis is never
   * crossed, so its next crossing is at +inf (other rays are unaffected) */
  if (isnan(d->tnext.x)) d->tnext.x = INFINITY;
  if (isnan(d->tnext.y)) d->tnext.y = INFINITY;
  if (isnan(d->tnext.z)) d->tnext.z = INFINITY;
  d->t0 = fmax_t(tmin, 0.f);
  d->tmax = tmax;
}
static inline float dda_t1(const oc_dda *d) { return fmin_t(rmin3(d->tnext), d->tmax); }
static inline int dda_leaf(const oc_dda *d) { return (d->cell.z * d->dims.y + d->cell.y) * d->dims.x + d->cell.x; }
static int dda_next(oc_dda *d)
{
  const float t1 = dda_t1(d);
  const float tc = rmin3(d->tnext);
  if (d->tnext.x == tc) { d->tnext.x += d->dist.x; d->cell.x += d->step.x; if (d->cell.x == d->stop.x) return 0; }
  if (d->tnext.y == tc) { d->tnext.y += d->dist.y; d->cell.y += d->step.y; if (d->cell.y == d->stop.y) return 0; }
  if (d->tnext.z == tc) { d->tnext.z += d->dist.z; d->cell.z += d->step.z; if (d->cell.z == d->stop.z) return 0; }
  d->t0 = t1;
  return 1;
}

int oc_dda3(exa_vec3f org, exa_vec3f dir, float tmin, float tmax, exa_vec3i dims,
            exa_box3f box, int maxCells, long long *ids, float *t0s, float *t1s)
{
  oc_dda d;
  int n = 0;
  dda_init(&d, org, dir, tmin, tmax, dims, box);
  while (n < maxCells) {
    ids[n] = dda_leaf(&d); t0s[n] = d.t0; t1s[n] = dda_t1(&d);
    n++;
    if (n >= maxCells || !dda_next(&d)) break;
  }
  return n;
}

/* sampleInteraction (deviceCode.cu:699-854) with dda3 (DDA.h:26-113)
 * inlined; shadow = ratio tracking (:785-839), else Woodcock (:726-783).
 * Returns the collision type; *pos in world space. */
static int sample_interaction(rctx *c, ray_t ray, int shadow, v3 *posOut,
                              float *TrOut, v4 *xfOut, oc_rng *rng, float *tHit)
{
  const exa_launch_params *lp = c->lp;
  const oc_field *f = c->f;
  ray.org = xfm_point(&lp->voxelSpaceTransform, ray.org);
  ray.dir = xfm_vector(&lp->voxelSpaceTransform, ray.dir);
  const float dt_scale = len3(ray.dir);
  ray.dir = norm3(ray.dir);
  ray.tmin = ray.tmin * dt_scale;
  ray.tmax = ray.tmax * dt_scale;

  int type = BOUNDARY;
  float Tr = 1.f;
  v3 pos = mk3(0.f, 0.f, 0.f);
  v4 xf = *xfOut;
  const float scale = lp->transferFunc.opacityScale;
  const int cull = lp->ext.cullTransparentPrims;

  oc_dda dda;
  dda_init(&dda, ray.org, ray.dir, ray.tmin, ray.tmax, lp->majorantGrid.dims, lp->majorantGrid.bounds);
  const v3i dims = lp->majorantGrid.dims;
  const int cellCap = lp->ext.ddaCellCap > 0 ? lp->ext.ddaCellCap : dims.x + dims.y + dims.z + 3;
  int ncells = 0;
  int done = 0;
  while (!done) {
    if (++ncells > cellCap) { c->err |= EXA_DEVERR_DDA_CAP; break; }
    const float t1 = dda_t1(&dda);
    const int leafID = dda_leaf(&dda);
    if (lp->ext.stepCounters) ((unsigned long long *)lp->ext.stepCounters)[3]++;
    /* ---- woodcockFunc / ratioTrackingFunc body ---- */
    {
      const float majorant = lp->maxOpacities[leafID];
      float t = dda.t0;
      int primID = -1;
      int steps = 0;
      while (1) {
        if (majorant <= 0.f) break;
        if (++steps > (lp->ext.trackStepCap > 0 ? lp->ext.trackStepCap : OC_TRACK_CAP)) {
          c->err |= EXA_DEVERR_TRACK_CAP;
          done = 1;
          break;
        }
        t -= oc_log(1.f - oc_rng_next(rng)) / (majorant * scale);
        if (t >= t1) break;
        pos = add3(ray.org, muls(ray.dir, t));
        exa_sample s = test_sample(f, pos, primID);
        if (s.primID < 0) s = oc_sample(f, pos, cull);
        if (lp->ext.stepCounters) {
          unsigned long long *sc = (unsigned long long *)lp->ext.stepCounters;
          sc[0]++;
          if (s.primID >= 0) sc[s.cellID != -1 ? 1 : 2]++;
        }
        if (s.primID < 0) continue;
        if (s.cellID != -1) primID = s.primID;
        xf = classify(c, s);
        const float sigmaT = xf.w;
        if (!shadow) {
          const float u = oc_rng_next(rng);
          if (sigmaT * scale >= u * majorant) {
            Tr = 0.f; type = SCATTERING; done = 1;
            if (tHit) *tHit = t;
            break;
          }
        } else {
          Tr *= 1.f - (sigmaT * scale) / majorant;
          if (Tr <= 0.f) { type = SCATTERING; done = 1; break; }
        }
      }
    }
    if (done) break;
    if (!dda_next(&dda)) break;
  }
  c->work += (uint64_t)ncells;
  *posOut = xfm_point(&lp->ext.voxelSpaceTransformInv, pos);
  *TrOut = Tr;
  *xfOut = xf;
  return type;
}

/* Surface meshes (MeshGeomCH, deviceCode.cu:306-318): the closest hit by
 * brute force over all triangles -- the smallest t in [0, tmax], the lowest
 * triangle index among equal t.  Triangle test: Moeller and Trumbore 1997,
 * no back-face culling; Ng = normalize(cross(b - a, c - a)), kd = 0.8. */
typedef struct { int prim; float t; v3 Ng; } mesh_hit;

static int tri_intersect(v3 org, v3 dir, v3 a, v3 b, v3 c, float tmax, float *t)
{
  const v3 e1 = sub3(b, a), e2 = sub3(c, a);
  const v3 p = cross3(dir, e2);
  const float det = dot3(e1, p);
  if (!(det != 0.f)) return 0;
  const float inv = 1.f / det;
  const v3 s = sub3(org, a);
  const float u = dot3(s, p) * inv;
  if (!(u >= 0.f && u <= 1.f)) return 0;
  const v3 q = cross3(s, e1);
  const float v = dot3(dir, q) * inv;
  if (!(v >= 0.f && u + v <= 1.f)) return 0;
  *t = dot3(e2, q) * inv;
  return *t >= 0.f && *t <= tmax;
}

static v3 mesh_vertex(const oc_field *f, int32_t i)
{
  const exa_vec3f v = f->meshVertices[i];
  return mk3(v.x, v.y, v.z);
}

static mesh_hit mesh_trace(const oc_field *f, v3 org, v3 dir, float tmax)
{
  mesh_hit h = {-1, tmax, {0.f, 0.f, 0.f}};
  float best = tmax;
  for (uint64_t k = 0; k < f->numTris; ++k) {
    const exa_vec3i id = f->meshIndices[k];
    float t;
    if (tri_intersect(org, dir, mesh_vertex(f, id.x), mesh_vertex(f, id.y), mesh_vertex(f, id.z), best, &t) &&
        (h.prim < 0 || t < best)) {
      best = t;
      h.prim = (int)k;
    }
  }
  if (h.prim >= 0) {
    const exa_vec3i id = f->meshIndices[h.prim];
    const v3 a = mesh_vertex(f, id.x), b = mesh_vertex(f, id.y), c = mesh_vertex(f, id.z);
    h.t = best;
    h.Ng = norm3(cross3(sub3(b, a), sub3(c, a)));
  }
  return h;
}

/* the surface test of the integrators: trace when the launch has a mesh,
 * clip ray.tmax at the hit (deviceCode.cu:1032-1039) */
static mesh_hit mesh_clip(rctx *c, ray_t *ray)
{
  mesh_hit h = {-1, 0.f, {0.f, 0.f, 0.f}};
  if (!c->lp->meshBVH) return h;
  h = mesh_trace(c->f, ray->org, ray->dir, ray->tmax);
  if (h.prim >= 0) ray->tmax = fmin_t(ray->tmax, h.t);
  return h;
}

/* sampleLight (deviceCode.cu:856-926); directional lights are an
 * extension: lights[i].pos is the direction towards the light, no
 * distance falloff */
static v3 sample_light(rctx *c, v3 pos, oc_rng *rng, int numLights, float *trOut)
{
  const exa_launch_params *lp = c->lp;
  int which = (int)(oc_rng_next(rng) * (float)numLights);
  if (which == numLights) which = 0;
  ray_t ray;
  float Tr, t00 = 1e30f, t11 = -1e30f;
  v3 np; v4 xf = {0.f, 0.f, 0.f, 0.f};
  ray.org = pos;
  ray.tmin = 0.f;
  if (lp->ext.lightType[which] == EXA_LIGHT_DIRECTIONAL) {
    ray.dir = norm3(lp->lights[which].pos);
    ray.tmax = 1e30f;
    box_test(ray, lp->worldSpaceBounds, &t00, &t11);
    clip_planes(lp, ray, &t00, &t11);
    ray.tmax = t11;
    const mesh_hit mh = mesh_clip(c, &ray);
    const int ct = sample_interaction(c, ray, 1, &np, &Tr, &xf, rng, NULL);
    if (trOut) *trOut = Tr;
    const float I = ct == BOUNDARY && mh.prim >= 0 ? fmaxf(0.f, dot3(mh.Ng, ray.dir)) * Tr * lp->lights[which].intensity
                                                   : Tr * lp->lights[which].intensity;
    return mk3(I, I, I);
  }
  v3 lightDir = sub3(lp->lights[which].pos, pos);
  const float ld = len3(xfm_vector(&lp->lightSpaceTransform, lightDir));
  const float ldWorld = len3(lightDir);
  lightDir = norm3(lightDir);
  ray.dir = lightDir;
  ray.tmax = ldWorld;
  box_test(ray, lp->worldSpaceBounds, &t00, &t11);
  clip_planes(lp, ray, &t00, &t11);
  ray.tmax = t11;
  const mesh_hit mh = mesh_clip(c, &ray);
  const int ct = sample_interaction(c, ray, 1, &np, &Tr, &xf, rng, NULL);
  if (trOut) *trOut = Tr;
  /* a shadow ray that reached a surface: max(0, N.l) (:921-925) */
  const float I = ct == BOUNDARY && mh.prim >= 0
                      ? fmaxf(0.f, dot3(mh.Ng, lightDir)) * Tr / (ld * ld) * lp->lights[which].intensity
                      : Tr / (ld * ld) * lp->lights[which].intensity;
  return mk3(I, I, I);
}

/* make_orthonormal_basis (deviceCode.cu:144-149) */
static void onb(v3 *u, v3 *v, v3 w)
{
  *v = fabsf(w.x) > fabsf(w.y) ? norm3(mk3(-w.z, 0.f, w.x)) : norm3(mk3(0.f, w.z, -w.y));
  *u = cross3(*v, w);
}

/* lambertianSample (deviceCode.cu:932-951): cosine-weighted about N; the
 * draws in order u1, u2; 2 pi u2 by the turn-based sine/cosine */
static v3 lambertian_sample(v3 N, oc_rng *rng)
{
  v3 u, v;
  onb(&u, &v, N);
  const float u1 = oc_rng_next(rng);
  const float u2 = oc_rng_next(rng);
  const float r = sqrtf(u1);
  float sn, cs;
  oc_sincos_turns(u2, &sn, &cs);
  const v3 sp = mk3(r * cs, r * sn, sqrtf(1.f - u1));
  return norm3(add3(add3(smul(sp.x, u), smul(sp.y, v)), smul(sp.z, N)));
}

/* henyeyGreensteinSample (deviceCode.cu:965-985); direction only */
static v3 hg_sample(v3 wo, float g, oc_rng *rng)
{
  const int gnz = fabsf(g) >= 1.19209290e-07f;
  const float u1 = oc_rng_next(rng);
  const float u2 = oc_rng_next(rng);
  const float a = gnz ? (1.f - g * g) / (1.f - g + 2.f * g * u1) : 0.f;
  const float cost = gnz ? (1.f + g * g - a * a) / (2.f * g) : 1.f - 2.f * u1;
  const float sint = sqrtf(fmaxf(0.f, 1.f - cost * cost));
  float sphi, cphi;
  oc_sincos_turns(u2, &sphi, &cphi);
  v3 u, v;
  onb(&u, &v, wo);
  const v3 mw = mk3(-wo.x, -wo.y, -wo.z);
  return add3(add3(muls(u, sint * cphi), muls(v, sint * sphi)), muls(mw, cost));
}

static int num_lights(const exa_launch_params *lp)
{
  int n = 0;
  for (int i = 0; i < EXA_LIGHTS_MAX; ++i) if (lp->lights[i].on) n++;
  return n;
}

/* pathTracingIntegrate (deviceCode.cu:991-1120) */
static v4 path_trace(rctx *c, ray_t ray, oc_rng *rng, v4 bg, int numLights,
                     float *tHit, float *trOut)
{
  const exa_launch_params *lp = c->lp;
  v3 throughput = mk3(1.f, 1.f, 1.f), Ld = mk3(0.f, 0.f, 0.f);
  unsigned bounce = 0;
  float t0 = 1e30f, t1 = -1e30f;
  const unsigned maxB = (unsigned)lp->ext.maxBounces;
  if (box_test(ray, lp->worldSpaceBounds, &t0, &t1)) {
    clip_planes(lp, ray, &t0, &t1);
    ray.org = add3(ray.org, muls(ray.dir, t0));
    t1 -= t0;
    while (1) {
      float Tr; v3 pos; v4 xf = {0.f, 0.f, 0.f, 0.f};
      ray.tmax = t1;
      const mesh_hit mh = mesh_clip(c, &ray);
      const int ct = sample_interaction(c, ray, 0, &pos, &Tr, &xf, rng, bounce == 0 ? tHit : NULL);
      const int surface = ct == BOUNDARY && mh.prim >= 0;
      if (ct == BOUNDARY && !surface) break;
      if (bounce++ >= maxB) { throughput = mk3(0.f, 0.f, 0.f); break; }
      v3 albedo;
      if (surface) {
        /* just past the surface (eps 1, :1056-1058), kd 0.8 */
        pos = add3(add3(ray.org, muls(ray.dir, mh.t)), muls(norm3(ray.dir), 1.f));
        albedo = mk3(.8f, .8f, .8f);
      } else {
        albedo = lp->ext.albedo < 0.f ? xyz(xf) : mk3(lp->ext.albedo, lp->ext.albedo, lp->ext.albedo);
      }
      throughput = mul3(throughput, albedo);
      const float P = rmax3(throughput);
      if (P < 0.2f) {
        if (oc_rng_next(rng) > P) { throughput = mk3(0.f, 0.f, 0.f); break; }
        throughput = div3(throughput, mk3(P, P, P));
      }
      throughput = add3(throughput, mk3(0.f, 0.f, 0.f)); /* += Le (always 0) */
      if (numLights > 0) Ld = add3(Ld, mul3(throughput, sample_light(c, pos, rng, numLights, bounce == 1 ? trOut : NULL)));
      v3 sd;
      if (surface) {
        /* Lambertian BRDF, then 16 units off the surface (:1084-1087) */
        sd = lambertian_sample(mh.Ng, rng);
        throughput = muls(throughput, fmaxf(0.f, dot3(sd, mh.Ng)));
        pos = add3(pos, smul(16.f, norm3(sd)));
      } else {
        const v3 wo = mk3(-ray.dir.x, -ray.dir.y, -ray.dir.z);
        sd = hg_sample(wo, lp->ext.hgG, rng);
      }
      ray.org = pos;
      ray.dir = sd;
      box_test(ray, lp->worldSpaceBounds, &t0, &t1);
      clip_planes(lp, ray, &t0, &t1);
    }
  }
  if (numLights == 0) Ld = mk3(1.f, 1.f, 1.f);
  const v3 L = mul3(Ld, throughput);
  v4 color = {L.x, L.y, L.z, 1.f};
  return bounce ? color : bg;
}

/* directLightingIntegrate (deviceCode.cu:1126-1207) */
static v4 direct_light(rctx *c, ray_t ray, oc_rng *rng, v4 bg, int numLights,
                       float *tHit, float *trOut)
{
  const exa_launch_params *lp = c->lp;
  v3 throughput = mk3(1.f, 1.f, 1.f);
  float t0 = 1e30f, t1 = -1e30f;
  if (!box_test(ray, lp->worldSpaceBounds, &t0, &t1)) return bg;
  clip_planes(lp, ray, &t0, &t1);
  ray.org = add3(ray.org, muls(ray.dir, t0));
  t1 -= t0;
  ray.tmax = t1;
  const mesh_hit mh = mesh_clip(c, &ray);
  float Tr; v3 pos; v4 xf = {0.f, 0.f, 0.f, 0.f};
  const int ct = sample_interaction(c, ray, 0, &pos, &Tr, &xf, rng, tHit);
  const int surface = ct == BOUNDARY && mh.prim >= 0;
  if (ct == BOUNDARY && !surface) return bg;
  v3 albedo;
  if (surface) {
    pos = add3(add3(ray.org, muls(ray.dir, mh.t)), muls(norm3(ray.dir), 1.f));
    albedo = mk3(.8f, .8f, .8f);
  } else {
    albedo = lp->ext.albedo < 0.f ? xyz(xf) : mk3(lp->ext.albedo, lp->ext.albedo, lp->ext.albedo);
  }
  if (numLights > 0) {
    throughput = mul3(throughput, mul3(albedo, sample_light(c, pos, rng, numLights, trOut)));
  } else {
    throughput = mul3(throughput, albedo);
    /* surfaces without lights: a headlight (:1196-1198) */
    if (surface) throughput = muls(throughput, fmaxf(0.f, dot3(mk3(-ray.dir.x, -ray.dir.y, -ray.dir.z), mh.Ng)));
  }
  v4 color = {throughput.x, throughput.y, throughput.z, 1.f};
  return color;
}

/* rayMarchingIntegrate + integrateDVR (deviceCode.cu:348-398, 1213-1260):
 * TF samples at spacing render.dt from the jittered first sample of
 * firstSampleT (:104-112), composited front to back, early exit at opacity
 * 0.99, over the background (over(), :151-154).  The shading normal is
 * g / |g + 1e-4| with the gradient g left at 0 (its computation is
 * commented out in the reference), so each light adds cd * 0. */
#define OC_MARCH_CAP (1ll << 24)
static v4 ray_march(rctx *c, ray_t ray, oc_rng *rng, v4 bg, int numLights)
{
  const exa_launch_params *lp = c->lp;
  v4 color = bg;
  float t0 = 1e30f, t1 = -1e30f;
  if (!box_test(ray, lp->worldSpaceBounds, &t0, &t1)) return color;
  clip_planes(lp, ray, &t0, &t1);
  if (lp->meshBVH) {
    /* a surface ends the march, shaded by a headlight (:1243-1251) */
    const mesh_hit mh = mesh_trace(c->f, ray.org, ray.dir, ray.tmax);
    if (mh.prim >= 0) {
      t1 = fmin_t(t1, mh.t);
      const float cs = fmaxf(0.f, dot3(mk3(-ray.dir.x, -ray.dir.y, -ray.dir.z), mh.Ng));
      color.x = cs; color.y = cs; color.z = cs; color.w = cs;
    }
  }
  const float ils = oc_rng_next(rng);
  const v3 org = xfm_point(&lp->voxelSpaceTransform, ray.org);
  const v3 vd = norm3(xfm_vector(&lp->voxelSpaceTransform, ray.dir));
  const float dt = lp->render.dt;
  const float numSegsf = floorf((t0 - dt * ils) / dt);
  float t = dt * (ils + numSegsf);
  if (t < t0) t += dt;
  const v3 g = mk3(0.f, 0.f, 0.f);
  const v3 N = muls(g, 1.f / len3(add3(g, mk3(1e-4f, 1e-4f, 1e-4f))));
  const int cull = lp->ext.cullTransparentPrims != 0;
  v4 acc = {0.f, 0.f, 0.f, 0.f};
  for (long long k = 0; t <= t1; t += dt, ++k) {
    if (k >= OC_MARCH_CAP) { c->err |= EXA_DEVERR_TRACK_CAP; break; }
    c->work++;
    const v3 pos = add3(org, muls(vd, t));
    const exa_sample smp = oc_sample(c->f, pos, cull);
    if (smp.primID < 0) continue;
    const v4 xf = lookup_tf(lp, smp.value);
    const v3 cd = mk3(xf.x, xf.y, xf.z);
    v3 shaded = smul(.1f, cd);
    if (numLights == 0) shaded = cd;
    for (int l = 0; l < numLights; ++l) {
      const v3 lv = sub3(lp->lights[l].pos, pos);
      const v3 L = norm3(lv);
      const float ld = len3(lv);
      shaded = add3(shaded, muls(cd, (.9f * dot3(N, L)) / (ld * ld) * lp->lights[l].intensity));
    }
    const float a = (1.f - acc.w) * xf.w;
    acc.x += a * shaded.x;
    acc.y += a * shaded.y;
    acc.z += a * shaded.z;
    acc.w += a * 1.f;
    if (acc.w >= 0.99f) break;
  }
  const float r = 1.f - acc.w;
  v4 out = {acc.x + r * color.x, acc.y + r * color.y, acc.z + r * color.z, acc.w + r * color.w};
  return out;
}

/* __saturatef: clamp to [0, 1], NaN to 0 */
static inline float sat_f(float x) { return x > 0.f ? (x < 1.f ? x : 1.f) : 0.f; }

static inline uint32_t make_8bit(float f)
{
  return (uint32_t)imin_t(255, imax_t(0, (int)(f * 256.f)));
}

/* renderFrame_Impl (deviceCode.cu:1268-1345) for one pixel */
static void render_pixel(rctx *c, int width, int height, int px, int py)
{
  const exa_launch_params *lp = c->lp;
  const int pixelID = px + width * py;
  /* backGroundColor, deviceCode.cu:43-50 */
  const float tb = (float)py / (float)height;
  const v4 bg = {(1.f - tb) * 1.f + tb * 0.5f, (1.f - tb) * 1.f + tb * 0.7f, (1.f - tb) * 1.f + tb * 1.f, 1.f};
  const int numLights = num_lights(lp);
  oc_rng rng;
  v4 acc = {0.f, 0.f, 0.f, 0.f};
  float tHit = -1.f, trv = -1.f;
  for (int s = 0; s < lp->render.spp; ++s) {
    oc_rng_init(&rng, (uint32_t)pixelID, (uint32_t)lp->accumID, lp->ext.frameID, (uint32_t)s);
    const float rx = oc_rng_next(&rng);
    const float ry = oc_rng_next(&rng);
    float sx = (float)px + rx, sy = (float)py + ry;
    if (lp->subImage.active) {  /* deviceCode.cu:1286-1294 */
      const float W = (float)width, H = (float)height;
      sx = sx / W; sy = sy / H;
      sx = (1.f - sx) * lp->subImage.value.lower.x + sx * lp->subImage.value.upper.x;
      sy = (1.f - sy) * lp->subImage.value.lower.y + sy * lp->subImage.value.upper.y;
      sx *= W; sy *= H;
    }
    /* generateRay, deviceCode.cu:88-101 */
    v3 dir = add3(add3(lp->camera.dir_00, smul(sx, lp->camera.dir_du)), smul(sy, lp->camera.dir_dv));
    dir = norm3(dir);
    if (fabsf(dir.x) < 1e-5f) dir.x = 1e-5f;
    if (fabsf(dir.y) < 1e-5f) dir.y = 1e-5f;
    if (fabsf(dir.z) < 1e-5f) dir.z = 1e-5f;
    ray_t ray; ray.org = lp->camera.org; ray.dir = dir; ray.tmin = 0.f; ray.tmax = 1e10f;
    v4 col;
    if (lp->integrator == EXA_PATH_TRACING_INTEGRATOR)
      col = path_trace(c, ray, &rng, bg, numLights, s == 0 ? &tHit : NULL, s == 0 ? &trv : NULL);
    else if (lp->integrator == EXA_RAY_MARCHING_INTEGRATOR)
      col = ray_march(c, ray, &rng, bg, numLights);
    else
      col = direct_light(c, ray, &rng, bg, numLights, s == 0 ? &tHit : NULL, s == 0 ? &trv : NULL);
    acc.x += col.x; acc.y += col.y; acc.z += col.z; acc.w += col.w;
  }
  if (lp->render.heatMapEnabled) {
    /* deviceCode.cu:1323-1327 with the pixel's work in place of its clock
     * cycles; temperature_to_rgb / hue_to_rgb (:155-170) */
    const float t = (float)c->work * (lp->render.heatMapScale / (float)lp->render.spp);
    const float K = 4.0f / 6.0f;
    const float hue = K - K * t, v = .5f + 0.5f * t;
    const float sh = sat_f(hue) * 6.0f;
    const float r = sat_f(fabsf(sh - 3.f) - 1.0f), g = sat_f(2.0f - fabsf(sh - 2.0f)), b = sat_f(2.0f - fabsf(sh - 4.0f));
    acc.x = v * r + (1.f - .5f) * acc.x;
    acc.y = v * g + (1.f - .5f) * acc.y;
    acc.z = v * b + (1.f - .5f) * acc.z;
    acc.w = .5f + (1.f - .5f) * acc.w;
  }
  if (lp->accumID > 0 && lp->accumBuffer) {
    const v4 o = lp->accumBuffer[pixelID];
    acc.x += o.x; acc.y += o.y; acc.z += o.z; acc.w += o.w;
  }
  if (lp->accumBuffer) lp->accumBuffer[pixelID] = acc;
  const float inv = 1.f / (float)(lp->accumID + 1);
  acc.x *= inv; acc.y *= inv; acc.z *= inv; acc.w *= inv;
  if (lp->subImage.selecting) {  /* deviceCode.cu:1337-1342 */
    const int lx = imin_t(imax_t((int)(lp->subImage.selection.lower.x * (float)width), 0), width - 1);
    const int ly = imin_t(imax_t((int)(lp->subImage.selection.lower.y * (float)height), 0), height - 1);
    const int hx = imin_t(imax_t((int)(lp->subImage.selection.upper.x * (float)width), 0), width - 1);
    const int hy = imin_t(imax_t((int)(lp->subImage.selection.upper.y * (float)height), 0), height - 1);
    if (((px == lx || px == hx) && py >= ly && py <= hy) || ((py == ly || py == hy) && px >= lx && px <= hx)) {
      acc.x = 1.f - acc.x; acc.y = 1.f - acc.y; acc.z = 1.f - acc.z; acc.w = 1.f - acc.w;
    }
  }
  const float is = 1.f / (float)lp->render.spp;
  const uint32_t rgba = make_8bit(acc.x * is) | (make_8bit(acc.y * is) << 8) |
                        (make_8bit(acc.z * is) << 16) | (make_8bit(acc.w * is) << 24);
  if (lp->fbPointer) lp->fbPointer[pixelID] = rgba;
  if (lp->ext.traceT) lp->ext.traceT[pixelID] = tHit;
  if (lp->ext.traceTr) lp->ext.traceTr[pixelID] = trv;
}

uint32_t oc_render(const oc_field *f, const exa_launch_params *lp, int width,
                   int height, int64_t pb, int64_t pe, int nthreads)
{
  uint32_t err = 0;
  if (pe > (int64_t)width * height) pe = (int64_t)width * height;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) reduction(| : err)
#endif
  for (int64_t p = pb; p < pe; ++p) {
    rctx c = {f, lp, 0, (int)(p % width), (int)(p / width), width, height, 0};
    render_pixel(&c, width, height, (int)(p % width), (int)(p / width));
    err |= c.err;
  }
  return err;
}

/* ================================================================== */
/* binary64 converged reference: direct lighting with ratio tracking    */
/* ================================================================== */
typedef struct { double x, y, z; } d3;
static inline d3 dk(double x, double y, double z) { d3 r = {x, y, z}; return r; }

static double d_sample_value(const oc_field *f, d3 p, int cull, int *hit)
{
  /* the field itself is fp32 data: locate in float, interpolate there */
  v3 pf = mk3((float)p.x, (float)p.y, (float)p.z);
  exa_sample s = oc_sample(f, pf, cull);
  *hit = s.primID >= 0;
  return s.value;
}

static double d_lookup_alpha(const exa_launch_params *lp, double v, double rgb[3])
{
  const exa_range1f d = lp->transferFunc.domain;
  if (d.lower >= d.upper || lp->transferFunc.numValues == 0) { rgb[0] = rgb[1] = rgb[2] = 0; return 0; }
  double fv = (v - d.lower) / ((double)d.upper - d.lower);
  if (lp->ext.tfFilter == EXA_TF_FILTER_LINEAR) {
    /* the linear filter of lookup_tf_linear in binary64 */
    const int n = lp->transferFunc.numValues;
    const double xB = fv * n - 0.5;
    rgb[0] = rgb[1] = rgb[2] = 0;
    if (!(xB >= -1.0 && xB < n)) return 0;
    const double fi = floor(xB), a = xB - fi;
    const int i = (int)fi;
    const v4 z = {0.f, 0.f, 0.f, 0.f};
    const v4 p = i >= 0 ? lp->transferFunc.values[i] : z;
    const v4 q = i + 1 < n ? lp->transferFunc.values[i + 1] : z;
    rgb[0] = (1 - a) * p.x + a * q.x;
    rgb[1] = (1 - a) * p.y + a * q.y;
    rgb[2] = (1 - a) * p.z + a * q.z;
    return (1 - a) * p.w + a * q.w;
  }
  if (fv < 0) fv = 0;
  if (!(fv < 1)) fv = 1; /* NaN as well, as the binary32 lookup clamps it */
  int i = (int)(fv * lp->transferFunc.numValues);
  if (i > lp->transferFunc.numValues - 1) i = lp->transferFunc.numValues - 1;
  const v4 c = lp->transferFunc.values[i];
  rgb[0] = c.x; rgb[1] = c.y; rgb[2] = c.z;
  return c.w;
}

/* expected transmittance by ratio tracking in binary64 over the same
 * majorant grid (walked densely in fixed steps of the majorant cell) */
static double d_transmittance(const oc_field *f, const exa_launch_params *lp,
                              d3 o, d3 dir, double tmax, uint64_t *rs)
{
  /* uniform majorant = global max opacity * scale, classic ratio tracking */
  const int cull = lp->ext.cullTransparentPrims;
  const double scale = lp->transferFunc.opacityScale;
  double maj = 0;
  const int64_t nmc = (int64_t)lp->majorantGrid.dims.x * lp->majorantGrid.dims.y * lp->majorantGrid.dims.z;
  for (int64_t i = 0; i < nmc; ++i) if (lp->maxOpacities[i] > maj) maj = lp->maxOpacities[i];
  maj *= scale;
  if (maj <= 0) return 1.0;
  double Tr = 1.0, t = 0.0;
  for (int k = 0; k < OC_TRACK_CAP; ++k) {
    *rs = oc_mix64(*rs + 0x9e3779b97f4a7c15ull);
    const double u = ((*rs >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    t -= log(u) / maj;
    if (t >= tmax) break;
    int hit;
    const double v = d_sample_value(f, dk(o.x + dir.x * t, o.y + dir.y * t, o.z + dir.z * t), cull, &hit);
    if (!hit) continue;
    double rgb[3];
    const double a = d_lookup_alpha(lp, v, rgb) * scale;
    Tr *= 1.0 - a / maj;
  }
  return Tr;
}

/* ---- binary64 path tracing (the expectation of pathTracingIntegrate,
 * deviceCode.cu:991-1120, with the launch parameters' albedo, HG g and
 * bounce limit): independent random numbers, every quantity in binary64,
 * tracking through the majorant grid by a binary64 DDA (Amanatides and Woo
 * 1987) -- delta tracking for free flights and ratio tracking for shadow
 * rays, both unbiased for any majorant that bounds the extinction, as the
 * max opacities do.  No surface meshes and no clip planes. */
static double d_rand(uint64_t *rs)
{
  *rs = oc_mix64(*rs + 0x9e3779b97f4a7c15ull);
  return ((*rs >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* boxTest (sampler/Sampler.h:105-122) in binary64 */
static int d_box(d3 o, d3 dir, double tmin, double tmax, const exa_box3f *b, double *t0, double *t1)
{
  const double lo[3] = {b->lower.x, b->lower.y, b->lower.z}, hi[3] = {b->upper.x, b->upper.y, b->upper.z};
  const double oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
  double a0 = tmin, a1 = tmax;
  for (int a = 0; a < 3; ++a) {
    double ta = (lo[a] - oo[a]) / dd[a], tb = (hi[a] - oo[a]) / dd[a];
    if (ta > tb) { const double tt = ta; ta = tb; tb = tt; }
    if (ta > a0) a0 = ta;
    if (tb < a1) a1 = tb;
  }
  *t0 = a0;
  *t1 = a1;
  return a0 < a1;
}

/* tracking along o + t dir for t in [0, tmax] through the majorant grid.
 * shadow = 0: delta tracking, returns 1 at a collision (*tHit, rgb, alpha);
 * shadow = 1: ratio tracking, *Tr the transmittance estimate */
static int d_track(const oc_field *f, const exa_launch_params *lp, d3 o, d3 dir, double tmax, int shadow,
                   uint64_t *rs, double *tHit, double rgb[3], double *Tr)
{
  const int cull = lp->ext.cullTransparentPrims;
  const double scale = lp->transferFunc.opacityScale;
  const v3i D = lp->majorantGrid.dims;
  const exa_box3f B = lp->majorantGrid.bounds;
  *Tr = 1.0;
  double tin, tout;
  if (!d_box(o, dir, 0.0, tmax, &B, &tin, &tout)) return 0;
  const double lo[3] = {B.lower.x, B.lower.y, B.lower.z};
  const double cs[3] = {((double)B.upper.x - B.lower.x) / D.x, ((double)B.upper.y - B.lower.y) / D.y,
                        ((double)B.upper.z - B.lower.z) / D.z};
  const double oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
  const int n[3] = {D.x, D.y, D.z};
  int cell[3], step[3];
  double tnext[3], tdelta[3];
  const double tm = 0.5 * (tin + tout);  /* locate the first cell mid-way into it */
  for (int a = 0; a < 3; ++a) {
    const double pe = oo[a] + dd[a] * tin;
    int c = (int)floor((pe - lo[a]) / cs[a]);
    if (dd[a] == 0.0) c = (int)floor((oo[a] + dd[a] * tm - lo[a]) / cs[a]);
    cell[a] = c < 0 ? 0 : (c >= n[a] ? n[a] - 1 : c);
    step[a] = dd[a] > 0 ? 1 : -1;
    if (dd[a] == 0.0) { tnext[a] = INFINITY; tdelta[a] = INFINITY; continue; }
    const double bound = lo[a] + (cell[a] + (dd[a] > 0 ? 1 : 0)) * cs[a];
    tnext[a] = (bound - oo[a]) / dd[a];
    tdelta[a] = cs[a] / fabs(dd[a]);
  }
  double t = tin;
  for (int guard = 0; guard < n[0] + n[1] + n[2] + 8; ++guard) {
    double t1 = tnext[0] < tnext[1] ? tnext[0] : tnext[1];
    if (tnext[2] < t1) t1 = tnext[2];
    if (tout < t1) t1 = tout;
    const double maj = lp->maxOpacities[((int64_t)cell[2] * n[1] + cell[1]) * n[0] + cell[0]] * scale;
    if (maj > 0) {
      double tt = t;
      for (int k = 0; k < OC_TRACK_CAP; ++k) {
        tt -= log(d_rand(rs)) / maj;
        if (tt >= t1) break;
        int hit;
        double c3[3];
        const double v = d_sample_value(f, dk(o.x + dir.x * tt, o.y + dir.y * tt, o.z + dir.z * tt), cull, &hit);
        if (!hit) continue;
        const double a = d_lookup_alpha(lp, v, c3) * scale;
        if (!shadow) {
          if (a >= d_rand(rs) * maj) {
            *tHit = tt;
            rgb[0] = c3[0]; rgb[1] = c3[1]; rgb[2] = c3[2];
            return 1;
          }
        } else {
          *Tr *= 1.0 - a / maj;
        }
      }
    }
    if (t1 >= tout) return 0;
    t = t1;
    int ax = 0;
    if (tnext[1] < tnext[ax]) ax = 1;
    if (tnext[2] < tnext[ax]) ax = 2;
    cell[ax] += step[ax];
    if (cell[ax] < 0 || cell[ax] >= n[ax]) return 0;
    tnext[ax] += tdelta[ax];
  }
  return 0;
}

/* the light sample of sampleLight (deviceCode.cu:856-926) in expectation
 * over the uniformly chosen light: mean of intensity x transmittance (x
 * 1/d^2 for point lights, d in light space) */
static double d_light(const oc_field *f, const exa_launch_params *lp, d3 pos, int numLights, uint64_t *rs)
{
  double L = 0.0;
  for (int li = 0; li < EXA_LIGHTS_MAX; ++li) {
    if (!lp->lights[li].on) continue;
    d3 ldir;
    double tmax = 1e30, fall = 1.0;
    if (lp->ext.lightType[li] == EXA_LIGHT_DIRECTIONAL) {
      ldir = dk(lp->lights[li].pos.x, lp->lights[li].pos.y, lp->lights[li].pos.z);
    } else {
      ldir = dk(lp->lights[li].pos.x - pos.x, lp->lights[li].pos.y - pos.y, lp->lights[li].pos.z - pos.z);
      const exa_affine3f *T = &lp->lightSpaceTransform;
      const d3 lv = dk(T->l.vx.x * ldir.x + T->l.vy.x * ldir.y + T->l.vz.x * ldir.z,
                       T->l.vx.y * ldir.x + T->l.vy.y * ldir.y + T->l.vz.y * ldir.z,
                       T->l.vx.z * ldir.x + T->l.vy.z * ldir.y + T->l.vz.z * ldir.z);
      fall = 1.0 / (lv.x * lv.x + lv.y * lv.y + lv.z * lv.z);
      tmax = sqrt(ldir.x * ldir.x + ldir.y * ldir.y + ldir.z * ldir.z);
    }
    const double nl = sqrt(ldir.x * ldir.x + ldir.y * ldir.y + ldir.z * ldir.z);
    ldir = dk(ldir.x / nl, ldir.y / nl, ldir.z / nl);
    double t0, t1, Tr = 1.0, th, c3[3];
    if (d_box(pos, ldir, 0.0, tmax, &lp->worldSpaceBounds, &t0, &t1)) d_track(f, lp, pos, ldir, t1, 1, rs, &th, c3, &Tr);
    L += Tr * fall * lp->lights[li].intensity;
  }
  return L / numLights;
}

/* henyeyGreensteinSample (deviceCode.cu:965-985) in binary64 */
static d3 d_hg(d3 wo, double g, uint64_t *rs)
{
  const double u1 = d_rand(rs), u2 = d_rand(rs);
  double cost;
  if (fabs(g) >= 1.19209290e-07) {
    const double a = (1 - g * g) / (1 - g + 2 * g * u1);
    cost = (1 + g * g - a * a) / (2 * g);
  } else {
    cost = 1 - 2 * u1;
  }
  const double sint = sqrt(fmax(0.0, 1 - cost * cost));
  const double phi = 2 * 3.14159265358979323846 * u2;
  d3 v = fabs(wo.x) > fabs(wo.y) ? dk(-wo.z, 0, wo.x) : dk(0, wo.z, -wo.y);
  const double vn = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
  v = dk(v.x / vn, v.y / vn, v.z / vn);
  const d3 u = dk(v.y * wo.z - v.z * wo.y, v.z * wo.x - v.x * wo.z, v.x * wo.y - v.y * wo.x);
  const double a = sint * cos(phi), b = sint * sin(phi);
  return dk(u.x * a + v.x * b - wo.x * cost, u.y * a + v.y * b - wo.y * cost, u.z * a + v.z * b - wo.z * cost);
}

static void d_path_trace(const oc_field *f, const exa_launch_params *lp, d3 o, d3 dir, int numLights,
                         const double bg[3], uint64_t *rs, double out[3])
{
  double thr[3] = {1, 1, 1}, Ld[3] = {0, 0, 0};
  unsigned bounce = 0;
  const unsigned maxB = (unsigned)lp->ext.maxBounces;
  double t0, t1;
  if (d_box(o, dir, 0.0, 1e30, &lp->worldSpaceBounds, &t0, &t1)) {
    o = dk(o.x + dir.x * t0, o.y + dir.y * t0, o.z + dir.z * t0);
    t1 -= t0;
    while (1) {
      double th, rgb[3], Tr;
      if (!d_track(f, lp, o, dir, t1, 0, rs, &th, rgb, &Tr)) break;
      if (bounce++ >= maxB) { thr[0] = thr[1] = thr[2] = 0; break; }
      const d3 pos = dk(o.x + dir.x * th, o.y + dir.y * th, o.z + dir.z * th);
      for (int k = 0; k < 3; ++k) thr[k] *= lp->ext.albedo < 0.f ? rgb[k] : (double)lp->ext.albedo;
      double P = thr[0] > thr[1] ? thr[0] : thr[1];
      if (thr[2] > P) P = thr[2];
      if (P < 0.2) {
        if (d_rand(rs) > P) { thr[0] = thr[1] = thr[2] = 0; break; }
        for (int k = 0; k < 3; ++k) thr[k] /= P;
      }
      if (numLights > 0) {
        const double L = d_light(f, lp, pos, numLights, rs);
        for (int k = 0; k < 3; ++k) Ld[k] += thr[k] * L;
      }
      dir = d_hg(dk(-dir.x, -dir.y, -dir.z), lp->ext.hgG, rs);
      o = pos;
      /* the next segment keeps the previous segment's end as its limit
       * (boxTest with ray.tmax = t1, deviceCode.cu:1029, 1107) */
      double n0, n1;
      d_box(o, dir, 0.0, t1, &lp->worldSpaceBounds, &n0, &n1);
      t1 = n1;
    }
  }
  if (numLights == 0) Ld[0] = Ld[1] = Ld[2] = 1;
  if (!bounce) { out[0] = bg[0]; out[1] = bg[1]; out[2] = bg[2]; return; }
  for (int k = 0; k < 3; ++k) out[k] = Ld[k] * thr[k];
}

void oc_render_f64(const oc_field *f, const exa_launch_params *lp, int width,
                   int height, int64_t pb, int64_t pe, double *out, int nthreads)
{
  if (pe > (int64_t)width * height) pe = (int64_t)width * height;
  const int numLights = num_lights(lp);
  const int cull = lp->ext.cullTransparentPrims;
  const double scale = lp->transferFunc.opacityScale;
  double maj = 0;
  const int64_t nmc = (int64_t)lp->majorantGrid.dims.x * lp->majorantGrid.dims.y * lp->majorantGrid.dims.z;
  for (int64_t i = 0; i < nmc; ++i) if (lp->maxOpacities[i] > maj) maj = lp->maxOpacities[i];
  maj *= scale;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t p = pb; p < pe; ++p) {
    const int px = (int)(p % width), py = (int)(p / width);
    uint64_t rs = oc_mix64(((uint64_t)p << 20) ^ 0x1234567ull ^ ((uint64_t)lp->accumID << 50));
    const double tb = (double)py / height;
    const double bg[3] = {(1 - tb) + tb * 0.5, (1 - tb) + tb * 0.7, 1.0};
    double acc[3] = {0, 0, 0};
    for (int s = 0; s < lp->render.spp; ++s) {
      rs = oc_mix64(rs + 1);
      const double rx = ((rs >> 11) + 0.5) / 9007199254740992.0;
      rs = oc_mix64(rs + 1);
      const double ry = ((rs >> 11) + 0.5) / 9007199254740992.0;
      d3 dir = dk(lp->camera.dir_00.x + (px + rx) * lp->camera.dir_du.x + (py + ry) * lp->camera.dir_dv.x,
                  lp->camera.dir_00.y + (px + rx) * lp->camera.dir_du.y + (py + ry) * lp->camera.dir_dv.y,
                  lp->camera.dir_00.z + (px + rx) * lp->camera.dir_du.z + (py + ry) * lp->camera.dir_dv.z);
      const double dl = sqrt(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
      dir = dk(dir.x / dl, dir.y / dl, dir.z / dl);
      const d3 o = dk(lp->camera.org.x, lp->camera.org.y, lp->camera.org.z);
      if (lp->integrator == EXA_PATH_TRACING_INTEGRATOR) {
        double c3[3];
        d_path_trace(f, lp, o, dir, numLights, bg, &rs, c3);
        acc[0] += c3[0]; acc[1] += c3[1]; acc[2] += c3[2];
        continue;
      }
      /* box test against world bounds (identity voxel transform assumed
       * by the caller for this reference) */
      double t0 = 0, t1 = 1e10;
      const double bl[3] = {lp->worldSpaceBounds.lower.x, lp->worldSpaceBounds.lower.y, lp->worldSpaceBounds.lower.z};
      const double bu[3] = {lp->worldSpaceBounds.upper.x, lp->worldSpaceBounds.upper.y, lp->worldSpaceBounds.upper.z};
      const double oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
      for (int a = 0; a < 3; ++a) {
        double ta = (bl[a] - oo[a]) / dd[a], tb2 = (bu[a] - oo[a]) / dd[a];
        if (ta > tb2) { double tt = ta; ta = tb2; tb2 = tt; }
        if (ta > t0) t0 = ta;
        if (tb2 < t1) t1 = tb2;
      }
      if (!(t0 < t1) || maj <= 0) { acc[0] += bg[0]; acc[1] += bg[1]; acc[2] += bg[2]; continue; }
      /* delta tracking for the free-flight distance under the global
       * majorant, unbiased; the shadow ray uses ratio tracking */
      double t = t0;
      int scattered = 0;
      double rgb[3] = {0, 0, 0};
      for (int k = 0; k < OC_TRACK_CAP; ++k) {
        rs = oc_mix64(rs + 1);
        const double u = ((rs >> 11) + 0.5) / 9007199254740992.0;
        t -= log(u) / maj;
        if (t >= t1) break;
        int hit;
        const d3 pp = dk(o.x + dir.x * t, o.y + dir.y * t, o.z + dir.z * t);
        const double v = d_sample_value(f, pp, cull, &hit);
        if (!hit) continue;
        const double a = d_lookup_alpha(lp, v, rgb) * scale;
        rs = oc_mix64(rs + 1);
        const double u2 = ((rs >> 11) + 0.5) / 9007199254740992.0;
        if (a >= u2 * maj) { scattered = 1; break; }
      }
      if (!scattered) { acc[0] += bg[0]; acc[1] += bg[1]; acc[2] += bg[2]; continue; }
      const d3 pos = dk(o.x + dir.x * t, o.y + dir.y * t, o.z + dir.z * t);
      double alb[3];
      if (lp->ext.albedo < 0.f) { alb[0] = rgb[0]; alb[1] = rgb[1]; alb[2] = rgb[2]; }
      else { alb[0] = alb[1] = alb[2] = lp->ext.albedo; }
      double L = 1.0;
      if (numLights > 0) {
        /* expectation over the uniformly chosen light */
        L = 0.0;
        for (int li = 0; li < numLights; ++li) {
          d3 ldir; double dist, fall = 1.0;
          if (lp->ext.lightType[li] == EXA_LIGHT_DIRECTIONAL) {
            ldir = dk(lp->lights[li].pos.x, lp->lights[li].pos.y, lp->lights[li].pos.z);
            const double n = sqrt(ldir.x * ldir.x + ldir.y * ldir.y + ldir.z * ldir.z);
            ldir = dk(ldir.x / n, ldir.y / n, ldir.z / n);
            dist = 1e30;
          } else {
            ldir = dk(lp->lights[li].pos.x - pos.x, lp->lights[li].pos.y - pos.y, lp->lights[li].pos.z - pos.z);
            dist = sqrt(ldir.x * ldir.x + ldir.y * ldir.y + ldir.z * ldir.z);
            ldir = dk(ldir.x / dist, ldir.y / dist, ldir.z / dist);
            fall = 1.0 / (dist * dist);
          }
          double te = 1e30;
          const double po[3] = {pos.x, pos.y, pos.z}, ld3[3] = {ldir.x, ldir.y, ldir.z};
          for (int a = 0; a < 3; ++a) {
            const double ta = (bl[a] - po[a]) / ld3[a], tb2 = (bu[a] - po[a]) / ld3[a];
            const double tf = ta > tb2 ? ta : tb2;
            if (tf < te) te = tf;
          }
          if (dist < te) te = dist;
          L += d_transmittance(f, lp, pos, ldir, te, &rs) * fall * lp->lights[li].intensity;
        }
        L /= numLights;
      }
      acc[0] += alb[0] * L; acc[1] += alb[1] * L; acc[2] += alb[2] * L;
    }
    out[(p - pb) * 3 + 0] = acc[0] / lp->render.spp;
    out[(p - pb) * 3 + 1] = acc[1] / lp->render.spp;
    out[(p - pb) * 3 + 2] = acc[2] / lp->render.spp;
  }
}
