// exa_device.cuh -- device-side math, RNG and cell/element interpolation of
// the ExaStitch path.
//
// Every float expression follows the operation order of the reference line
// it cites (paths relative to the owlExaStitcher tree).  The library is built
// with --fmad=false, so no multiply-add is contracted and results match a
// binary32 evaluation of the same expressions on the host bit for bit.
// Helpers the reference takes from the (un-vendored) OWL library are defined
// with textbook semantics: dot = x*x'+y*y'+z*z', min/max as (a<b?a:b),
// normalize(v) = v * (1.f/sqrtf(dot(v,v))), rcp(x) = 1.f/x.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/exastitch.h"

#define EXA_HD __host__ __device__ __forceinline__
#define EXA_D __device__ __forceinline__

// The bounds-checked build (EXA_CHECKS=1, libexastitch_checks.so): the
// kernels test the indices they read through (gridlet and element ids from
// tables, lists, caches and BVH leaves, BVH nodes, macrocells, queue slots)
// before the access; an index out of range sets EXA_DEVERR_BOUNDS and the
// access is skipped.  Compiled out otherwise.
#ifndef EXA_CHECKS
#define EXA_CHECKS 0
#endif
EXA_HD bool exa_in_range(long long i, long long n, uint32_t &err)
{
  if (!EXA_CHECKS || (i >= 0 && i < n)) return true;
  err |= EXA_DEVERR_BOUNDS;
  return false;
}

namespace exa {

struct V3 { float x, y, z; };
struct V3i { int x, y, z; };

EXA_HD V3 mk3(float x, float y, float z) { return V3{x, y, z}; }
EXA_HD V3 mk3(exa_vec3f v) { return V3{v.x, v.y, v.z}; }
EXA_HD V3 add3(V3 a, V3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
EXA_HD V3 sub3(V3 a, V3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
EXA_HD V3 mul3(V3 a, V3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
EXA_HD V3 div3(V3 a, V3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
EXA_HD V3 muls(V3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
EXA_HD V3 smul(float s, V3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
EXA_HD float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
EXA_HD V3 cross3(V3 a, V3 b)
{
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
EXA_HD float fmin_t(float a, float b) { return a < b ? a : b; }
EXA_HD float fmax_t(float a, float b) { return a > b ? a : b; }
EXA_HD V3 min3(V3 a, V3 b) { return mk3(fmin_t(a.x, b.x), fmin_t(a.y, b.y), fmin_t(a.z, b.z)); }
EXA_HD V3 max3(V3 a, V3 b) { return mk3(fmax_t(a.x, b.x), fmax_t(a.y, b.y), fmax_t(a.z, b.z)); }
EXA_HD float rmin3(V3 a) { return fmin_t(a.x, fmin_t(a.y, a.z)); }
EXA_HD float rmax3(V3 a) { return fmax_t(a.x, fmax_t(a.y, a.z)); }
EXA_HD int imin_t(int a, int b) { return a < b ? a : b; }
EXA_HD int imax_t(int a, int b) { return a > b ? a : b; }
EXA_HD int iclamp(int v, int lo, int hi) { return imin_t(imax_t(v, lo), hi); }
EXA_D float len3(V3 a) { return __fsqrt_rn(dot3(a, a)); }
EXA_D V3 norm3(V3 a) { return muls(a, __fdiv_rn(1.f, __fsqrt_rn(dot3(a, a)))); }

// owl LinearSpace3f * vec3f: v.x*vx + v.y*vy + v.z*vz
EXA_HD V3 xfm_vector(const exa_affine3f &A, V3 v)
{
  return add3(add3(smul(v.x, mk3(A.l.vx)), smul(v.y, mk3(A.l.vy))), smul(v.z, mk3(A.l.vz)));
}
EXA_HD V3 xfm_point(const exa_affine3f &A, V3 p) { return add3(xfm_vector(A, p), mk3(A.p)); }

// ------------------------------------------------------------------ math
EXA_HD uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Natural log for positive normal floats: x = m*2^e, m in [sqrt(1/2),
// sqrt(2)), log(m) = 2 atanh(s), s = (m-1)/(m+1), Taylor series through
// s^9; log(2) split into a 16-bit head and a tail.
EXA_D float exa_log(float x)
{
  const uint32_t bits = __float_as_uint(x);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  float m = __uint_as_float((bits & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421354f) { m = m * 0.5f; e = e + 1; }
  const float s = __fdiv_rn(m - 1.f, m + 1.f);
  const float s2 = s * s;
  const float p = s2 * (0.333333343f + s2 * (0.200000003f + s2 * (0.142857149f + s2 * 0.111111112f)));
  const float lm = 2.f * s + (2.f * s) * p;
  const float fe = (float)e;
  return fe * 0.693145752f + (fe * 1.42860677e-06f + lm);
}

// sin and cos of 2*pi*u by quadrant reduction and Taylor series
EXA_D void exa_sincos_turns(float u, float &s, float &c)
{
  const float u4 = u * 4.f;
  const float q = floorf(u4 + 0.5f);
  const float r = u4 - q;
  const float t = r * 1.57079637f;
  const float t2 = t * t;
  const float sp = t + (t * t2) * (-0.166666672f + t2 * (0.00833333377f + t2 * (-0.000198412701f + t2 * 2.75573188e-06f)));
  const float cp = 1.f + t2 * (-0.5f + t2 * (0.0416666679f + t2 * (-0.00138888892f + t2 * 2.48015876e-05f)));
  const int qi = ((int)q) & 3;
  if (qi == 0) { s = sp; c = cp; }
  else if (qi == 1) { s = cp; c = -sp; }
  else if (qi == 2) { s = -sp; c = -cp; }
  else { s = -cp; c = sp; }
}

// Counter-based stream (stands in for owl::common::LCG<4>,
// deviceCode.cu:41,1278): key from (pixel, accumID, frameID, sample); the
// n-th draw is mix64(key + n*golden) >> 40 scaled by 2^-24.  One stream per
// camera sample makes every (pixel, sample) an independent unit of work.
// The state is the running sum key + n*golden (mod 2^64), so a draw is one
// 64-bit add and the mix.
struct Rng {
  uint64_t state;
  EXA_D void init(uint32_t pixelID, uint32_t accumID, uint32_t frameID, uint32_t sampleID)
  {
    state = mix64((((uint64_t)pixelID << 32) | (uint64_t)accumID) ^
                  mix64((((uint64_t)frameID << 32) | (uint64_t)sampleID) + 0x5851f42d4c957f2dull));
  }
  EXA_D float next()
  {
    state += 0x9e3779b97f4a7c15ull;
    const uint64_t z = mix64(state);
    return (float)(uint32_t)(z >> 40) * 5.96046448e-08f;
  }
};

// ------------------------------------------------------------------ Gridlet.h
EXA_D float lerpf_(float a, float b, float x) { return (1.f - x) * a + x * b; }  // common.h:64-68

// Gridlet.h:39-98 for a header already loaded: h0 = (lower, level),
// h1 = (dims, begin)
EXA_D bool intersect_gridlet_hdr(float &value, int &cellID, V3 pos, const int4 h0, const int4 h1,
                                 const float *__restrict__ scalars)
{
  const int level = h0.w;
  const float cw = (float)(1 << level);
  const V3 lo = muls(mk3((float)h0.x + 0.5f, (float)h0.y + 0.5f, (float)h0.z + 0.5f), cw);
  const V3 hi = muls(mk3(((float)h0.x + (float)h1.x) + 0.5f, ((float)h0.y + (float)h1.y) + 0.5f,
                         ((float)h0.z + (float)h1.z) + 0.5f), cw);
  if (!(lo.x <= pos.x && lo.y <= pos.y && lo.z <= pos.z && pos.x <= hi.x && pos.y <= hi.y && pos.z <= hi.z))
    return false;
  const int nx = h1.x + 1, ny = h1.y + 1, nz = h1.z + 1;
  // x / 2^level == x * 2^-level exactly in IEEE arithmetic (both are the
  // correctly rounded quotient), so the division of Gridlet.h:50 is a
  // multiplication here
  const float icw = __uint_as_float((uint32_t)(127 - level) << 23);
  const V3 p = mk3((pos.x - lo.x) * icw, (pos.y - lo.y) * icw, (pos.z - lo.z) * icw);
  const int ix = (int)p.x, iy = (int)p.y, iz = (int)p.z;
  const int ax = imin_t(ix + 1, nx - 1), ay = imin_t(iy + 1, ny - 1), az = imin_t(iz + 1, nz - 1);
  const float *S = scalars + (uint32_t)h1.w;
  const int r00 = (iz * ny + iy) * nx, r01 = (iz * ny + ay) * nx;
  const int r10 = (az * ny + iy) * nx, r11 = (az * ny + ay) * nx;
  const float f1 = __ldg(S + r00 + ix), f2 = __ldg(S + r00 + ax);
  const float f3 = __ldg(S + r01 + ix), f4 = __ldg(S + r01 + ax);
  const float f5 = __ldg(S + r10 + ix), f6 = __ldg(S + r10 + ax);
  const float f7 = __ldg(S + r11 + ix), f8 = __ldg(S + r11 + ax);
  if (isnan(f1) || isnan(f2) || isnan(f3) || isnan(f4) || isnan(f5) || isnan(f6) || isnan(f7) || isnan(f8))
    return false;
  const V3 frac = mk3(p.x - (float)ix, p.y - (float)iy, p.z - (float)iz);
  const float f12 = lerpf_(f1, f2, frac.x);
  const float f56 = lerpf_(f5, f6, frac.x);
  const float f34 = lerpf_(f3, f4, frac.x);
  const float f78 = lerpf_(f7, f8, frac.x);
  const float f1234 = lerpf_(f12, f34, frac.y);
  const float f5678 = lerpf_(f56, f78, frac.y);
  value = lerpf_(f1234, f5678, frac.z);
  cellID = iz * h1.y * h1.x + iy * h1.x + ix;
  return true;
}

// Gridlet.h:39-98.  Header loaded as two 16-byte vectors (one 32 B sector).
EXA_D bool intersect_gridlet(float &value, int &cellID, V3 pos, const exa_gridlet *gp, const float *__restrict__ scalars)
{
  const int4 h0 = __ldg(reinterpret_cast<const int4 *>(gp));
  const int4 h1 = __ldg(reinterpret_cast<const int4 *>(gp) + 1);
  return intersect_gridlet_hdr(value, cellID, pos, h0, h1, scalars);
}

// ------------------------------------------------------------------ Plane.h
struct Plane { V3 N; float d; };
EXA_D Plane make_plane(V3 a, V3 b, V3 c)  // Plane.h:32-38
{
  Plane p;
  p.N = cross3(sub3(b, a), sub3(c, a));
  p.d = dot3(a, p.N);
  return p;
}
EXA_D float plane_eval(const Plane &p, V3 v) { return dot3(v, p.N) - p.d; }

// Plane.h:57-99, including its fa > 1 test for fb/fc/fd (Plane.h:89,92,95)
EXA_D bool intersect_tet(float &value, V3 P, float4 a, float4 b, float4 c, float4 d)
{
  const V3 va = sub3(mk3(a.x, a.y, a.z), P), vb = sub3(mk3(b.x, b.y, b.z), P);
  const V3 vc = sub3(mk3(c.x, c.y, c.z), P), vd = sub3(mk3(d.x, d.y, d.z), P);
  const Plane pa = make_plane(vb, vd, vc);
  const Plane pb = make_plane(va, vc, vd);
  const Plane pc = make_plane(va, vd, vb);
  const Plane pd = make_plane(va, vb, vc);
  const V3 zero = mk3(0.f, 0.f, 0.f);
  const float fa = __fdiv_rn(plane_eval(pa, zero), plane_eval(pa, va));
  if (fa < 0.f || fa > 1.f) return false;
  const float fb = __fdiv_rn(plane_eval(pb, zero), plane_eval(pb, vb));
  if (fb < 0.f || fa > 1.f) return false;
  const float fc = __fdiv_rn(plane_eval(pc, zero), plane_eval(pc, vc));
  if (fc < 0.f || fa > 1.f) return false;
  const float fd = __fdiv_rn(plane_eval(pd, zero), plane_eval(pd, vd));
  if (fd < 0.f || fa > 1.f) return false;
  value = fa * a.w + fb * b.w + fc * c.w + fd * d.w;
  return true;
}

// ------------------------------------------------------------------ UElems.h
EXA_D float det3(V3 x, V3 y, V3 z) { return dot3(x, cross3(y, z)); }

// Shape functions and derivatives of UElems.h:46-86 (pyramid),
// :180-217 (wedge), :313-370 (hex); KIND 5, 6, 8 = vertex count.
template <int NV>
EXA_D void shape_fns(const float *pc, float *sf, float *d)
{
  if constexpr (NV == 5) {
    const float rm = 1.f - pc[0], sm = 1.f - pc[1], tm = 1.f - pc[2];
    sf[0] = rm * sm * tm; sf[1] = pc[0] * sm * tm; sf[2] = pc[0] * pc[1] * tm;
    sf[3] = rm * pc[1] * tm; sf[4] = pc[2];
    d[0] = -(pc[1] - 1.f) * (pc[2] - 1.f); d[1] = (pc[1] - 1.f) * (pc[2] - 1.f);
    d[2] = pc[1] - pc[1] * pc[2]; d[3] = pc[1] * (pc[2] - 1.f); d[4] = 0.f;
    d[5] = -(pc[0] - 1.f) * (pc[2] - 1.f); d[6] = pc[0] * (pc[2] - 1.f);
    d[7] = pc[0] - pc[0] * pc[2]; d[8] = (pc[0] - 1.f) * (pc[2] - 1.f); d[9] = 0.f;
    d[10] = -(pc[0] - 1.f) * (pc[1] - 1.f); d[11] = pc[0] * (pc[1] - 1.f);
    d[12] = -pc[0] * pc[1]; d[13] = (pc[0] - 1.f) * pc[1]; d[14] = 1.f;
  } else if constexpr (NV == 6) {
    sf[0] = (1.f - pc[0] - pc[1]) * (1.f - pc[2]); sf[1] = pc[0] * (1.f - pc[2]);
    sf[2] = pc[1] * (1.f - pc[2]); sf[3] = (1.f - pc[0] - pc[1]) * pc[2];
    sf[4] = pc[0] * pc[2]; sf[5] = pc[1] * pc[2];
    d[0] = -1.f + pc[2]; d[1] = 1.f - pc[2]; d[2] = 0.f; d[3] = -pc[2]; d[4] = pc[2]; d[5] = 0.f;
    d[6] = -1.f + pc[2]; d[7] = 0.f; d[8] = 1.f - pc[2]; d[9] = -pc[2]; d[10] = 0.f; d[11] = pc[2];
    d[12] = -1.f + pc[0] + pc[1]; d[13] = -pc[0]; d[14] = -pc[1];
    d[15] = 1.f - pc[0] - pc[1]; d[16] = pc[0]; d[17] = pc[1];
  } else {
    const float rm = 1.f - pc[0], sm = 1.f - pc[1], tm = 1.f - pc[2];
    sf[0] = rm * sm * tm; sf[1] = pc[0] * sm * tm; sf[2] = pc[0] * pc[1] * tm; sf[3] = rm * pc[1] * tm;
    sf[4] = rm * sm * pc[2]; sf[5] = pc[0] * sm * pc[2]; sf[6] = pc[0] * pc[1] * pc[2]; sf[7] = rm * pc[1] * pc[2];
    d[0] = -sm * tm; d[1] = sm * tm; d[2] = pc[1] * tm; d[3] = -pc[1] * tm;
    d[4] = -sm * pc[2]; d[5] = sm * pc[2]; d[6] = pc[1] * pc[2]; d[7] = -pc[1] * pc[2];
    d[8] = -rm * tm; d[9] = -pc[0] * tm; d[10] = pc[0] * tm; d[11] = rm * tm;
    d[12] = -rm * pc[2]; d[13] = -pc[0] * pc[2]; d[14] = pc[0] * pc[2]; d[15] = rm * pc[2];
    d[16] = -rm * sm; d[17] = -pc[0] * sm; d[18] = -pc[0] * pc[1]; d[19] = -rm * pc[1];
    d[20] = rm * sm; d[21] = pc[0] * sm; d[22] = pc[0] * pc[1]; d[23] = rm * pc[1];
  }
}

// Newton inversion shared by intersectPyrEXT / WedgeEXT / HexEXT
// (UElems.h:88-177, 219-310, 372-464).  The 1e-4 / 1e6 tolerances are
// double literals there, so those comparisons run in double here too.
template <int NV>
EXA_D bool newton_elem(float &value, V3 P, const float4 *V)
{
  float pc[3] = {0.5f, 0.5f, 0.5f};
  float d[3 * NV];
  float w[NV];
  bool converged = false;
  for (int it = 0; !converged && it < 10; it++) {
    shape_fns<NV>(pc, w, d);
    V3 fcol = mk3(0.f, 0.f, 0.f), rcol = fcol, scol = fcol, tcol = fcol;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const V3 pt = mk3(V[i].x, V[i].y, V[i].z);
      fcol = add3(fcol, muls(pt, w[i]));
      rcol = add3(rcol, muls(pt, d[i]));
      scol = add3(scol, muls(pt, d[i + NV]));
      tcol = add3(tcol, muls(pt, d[i + 2 * NV]));
    }
    fcol = sub3(fcol, P);
    const float dd = det3(rcol, scol, tcol);
    if (fabsf(dd) < 1e-6f) return false;
    const float d0 = __fdiv_rn(det3(fcol, scol, tcol), dd);
    const float d1 = __fdiv_rn(det3(rcol, fcol, tcol), dd);
    const float d2 = __fdiv_rn(det3(rcol, scol, fcol), dd);
    pc[0] = pc[0] - d0;
    pc[1] = pc[1] - d1;
    pc[2] = pc[2] - d2;
    if (((double)fabsf(d0) < 1e-4) & ((double)fabsf(d1) < 1e-4) & ((double)fabsf(d2) < 1e-4)) {
      converged = true;
    } else if (((double)fabsf(pc[0]) > 1e6) | ((double)fabsf(pc[1]) > 1e6) | ((double)fabsf(pc[2]) > 1e6)) {
      return false;
    }
  }
  if (!converged) return false;
  const float lower = (float)(0.0 - 1e-6);
  const float upper = (float)(1.0 + 1e-6);
  bool inside = pc[0] >= lower && pc[0] <= upper && pc[1] >= lower && pc[1] <= upper && pc[2] >= lower &&
                pc[2] <= upper;
  if (NV == 6) inside = inside && (pc[0] + pc[1] <= upper);
  if (!inside) return false;
  float val = 0.f;
#pragma unroll
  for (int i = 0; i < NV; i++) val += w[i] * V[i].w;
  value = val;
  return true;
}

// sampler/programs/ExaStitchSampler.cu:133-161: the vertex count of the
// -1-padded 8-wide index row selects the element type.
EXA_D bool intersect_elem(float &value, V3 P, const int32_t *__restrict__ idx8, const float4 *__restrict__ verts)
{
  const int4 i0 = __ldg(reinterpret_cast<const int4 *>(idx8));
  const int4 i1 = __ldg(reinterpret_cast<const int4 *>(idx8) + 1);
  // rows of fewer than 4 vertices name no element type and are never hit
  // (the model rejects rows with a vertex after the padding)
  if (i0.w < 0) return false;
  const int nv = 4 + (i1.x >= 0) + (i1.y >= 0) + (i1.z >= 0) + (i1.w >= 0);
  float4 v[8];
  v[0] = __ldg(verts + i0.x); v[1] = __ldg(verts + i0.y); v[2] = __ldg(verts + i0.z); v[3] = __ldg(verts + i0.w);
  if (nv == 4) return intersect_tet(value, P, v[0], v[1], v[2], v[3]);
  v[4] = __ldg(verts + i1.x);
  if (nv == 5) return newton_elem<5>(value, P, v);
  v[5] = __ldg(verts + i1.y);
  if (nv == 6) return newton_elem<6>(value, P, v);
  if (nv == 8) {
    v[6] = __ldg(verts + i1.z);
    v[7] = __ldg(verts + i1.w);
    return newton_elem<8>(value, P, v);
  }
  return false;
}

// Grid.cuh:51-59
EXA_HD V3i project_on_grid(V3 V, V3i dims, const exa_box3f &b)
{
  const V3 lo = mk3(b.lower), hi = mk3(b.upper);
  const V3 V01 = div3(sub3(V, lo), sub3(hi, lo));
  V3i r;
  r.x = iclamp((int)(V01.x * (float)dims.x), 0, dims.x - 1);
  r.y = iclamp((int)(V01.y * (float)dims.y), 0, dims.y - 1);
  r.z = iclamp((int)(V01.z * (float)dims.z), 0, dims.z - 1);
  return r;
}

// the table entries the linear transfer-function filter
// (EXA_TF_FILTER_LINEAR) can blend for normalised values in [l, u]:
// floor(l*N - 0.5) .. floor(u*N - 0.5) + 1, clipped to the table (the
// products and differences are the lookup's own operations, so a value in
// [l, u] never reads outside the span); false when the span misses the table
EXA_HD bool tf_linear_span(float l, float u, int n, int &lo, int &hi)
{
  const float N = (float)n;
  const float a = floorf(l * N - 0.5f), b = floorf(u * N - 0.5f) + 1.f;
  if (!(b >= 0.f) || !(a <= N - 1.f)) return false;
  lo = a < 0.f ? 0 : (int)a;
  hi = b > N - 1.f ? n - 1 : (int)b;
  return true;
}

// Grid.cu:687-719 (== sampler/ExaStitchSampler.cu:144-176, 208-226); under
// the linear filter the entry span of tf_linear_span
EXA_HD float range_max_opacity(exa_range1f vr, const float4 *cm, int n, exa_range1f xf, int filter)
{
  if (vr.upper < vr.lower) return 0.f;
  vr.lower -= xf.lower;
  vr.lower /= xf.upper - xf.lower;
  vr.upper -= xf.lower;
  vr.upper /= xf.upper - xf.lower;
  int lo, hi;
  if (filter == EXA_TF_FILTER_LINEAR) {
    if (!tf_linear_span(vr.lower, vr.upper, n, lo, hi)) return 0.f;
  } else {
    lo = iclamp((int)(vr.lower * (float)(n - 1)), 0, n - 1);
    hi = iclamp((int)(vr.upper * (float)(n - 1)) + 1, 0, n - 1);
  }
  float m = 0.f;
  for (int i = lo; i <= hi; ++i) m = fmaxf(m, cm[i].w);
  return m;
}

// Order-independent float min/max on the integer image of IEEE floats:
// non-negative floats order like signed ints, negative ones inversely as
// unsigned ints (the sign bit decides, so -0 takes the negative branch).
EXA_D void atomic_min_float(float *addr, float v)
{
  if (!signbit(v)) atomicMin(reinterpret_cast<int *>(addr), __float_as_int(v));
  else atomicMax(reinterpret_cast<unsigned *>(addr), __float_as_uint(v));
}
EXA_D void atomic_max_float(float *addr, float v)
{
  if (!signbit(v)) atomicMax(reinterpret_cast<int *>(addr), __float_as_int(v));
  else atomicMin(reinterpret_cast<unsigned *>(addr), __float_as_uint(v));
}

} // namespace exa
