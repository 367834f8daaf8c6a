// exa_render.cu -- the hot path: field sampling (sample(),
// sampler/ExaStitchSampler.h:128-140) and the per-pixel integrators of
// deviceCode.cu: generateRay (:88-101), sampleInteraction with Woodcock
// and ratio tracking (:699-854) over the DDA majorant grid (DDA.h:26-113),
// sampleLight (:856-926), henyeyGreensteinSample (:965-985),
// pathTracingIntegrate (:991-1120), directLightingIntegrate (:1126-1207)
// and renderFrame_Impl (:1268-1345).
//
// The launch parameters and the accel view are kernel parameters (constant
// bank).
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "exa_host.h"
#include "exa_mesh.cuh"
#include "exa_surrogate.cuh"

namespace exa {


// resident 128-thread blocks per SM the render kernel is compiled for
// (bounds its registers: 65536 / (128 * n))
#ifndef EXA_RENDER_MIN_BLOCKS
#define EXA_RENDER_MIN_BLOCKS 4
#endif

// work counters of a counting launch (lp.ext.stepCounters set); the index is
// the slot in stepCounters
enum : int {
  CNT_FIELD, CNT_GRIDLET, CNT_ELEM, CNT_DDA, CNT_PATHS, CNT_MISS, CNT_TABLES, CNT_GTESTS, CNT_ELEMQ, CNT_WALKS,
  CNT_SURR, CNT_VIOL, CNT_N
};
// one column per thread in shared memory, so that an ordinary launch holds no
// registers for them; every render kernel runs 128 threads per block
static __shared__ unsigned s_cnt[CNT_N][128];

struct RayS {
  V3 org, dir;
  float tmin, tmax;
};

enum { BOUNDARY = 0, SCATTERING = 1 };

// one channel of the linear filter: the blend of the two entries, limited
// to their range (so the filtered opacity never exceeds the larger entry)
EXA_D float tf_lerp(float p, float q, float a)
{
  const float r = (1.f - a) * p + a * q;
  return fminf(fmaxf(r, fminf(p, q)), fmaxf(p, q));
}

// EXA_TF_FILTER_LINEAR: the texture fetch of deviceCode.cu:331-332 with
// the texture of OWLRenderer.cpp:659-707 (normalised coordinates, linear
// filtering, zero border) in binary32 arithmetic
EXA_D float4 lookup_tf_linear(const float4 *__restrict__ T, int n, float f)
{
  const float xB = f * (float)n - 0.5f;
  if (!(xB >= -1.f && xB < (float)n)) return make_float4(0.f, 0.f, 0.f, 0.f);  // both entries are border
  const float fi = floorf(xB);
  const int i = (int)fi;
  const float a = xB - fi;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 p = i >= 0 ? __ldg(T + i) : z;
  const float4 q = i + 1 < n ? __ldg(T + i + 1) : z;
  return make_float4(tf_lerp(p.x, q.x, a), tf_lerp(p.y, q.y, a), tf_lerp(p.z, q.z, a), tf_lerp(p.w, q.w, a));
}

// deviceCode.cu:320-341: the buffer variant, or the texture variant under
// EXA_TF_FILTER_LINEAR
EXA_D float4 lookup_tf(const exa_launch_params &lp, float f)
{
  const exa_range1f d = lp.transferFunc.domain;
  if (d.lower >= d.upper) return make_float4(0.f, 0.f, 0.f, 0.f);
  f -= d.lower;
  f /= (d.upper - d.lower);
  if (lp.transferFunc.numValues == 0) return make_float4(0.f, 0.f, 0.f, 0.f);
  if (lp.ext.tfFilter == EXA_TF_FILTER_LINEAR)
    return lookup_tf_linear(reinterpret_cast<const float4 *>(lp.transferFunc.values), lp.transferFunc.numValues, f);
  // min(1, f) in std::min's operand order (fminf gives the same): a NaN
  // value, which an element with collapsed vertices yields, clamps to 1 (the
  // last entry), and no NaN reaches the conversion to int
  f = fmax_t(0.f, f < 1.f ? f : 1.f);
  const int i = imin_t(lp.transferFunc.numValues - 1, (int)(f * (float)lp.transferFunc.numValues));
  return __ldg(reinterpret_cast<const float4 *>(lp.transferFunc.values) + i);
}

// sampler/Sampler.h:105-122
EXA_D bool box_test(const RayS &r, const exa_box3f &b, float &t0, float &t1)
{
  const V3 lo = div3(sub3(mk3(b.lower), r.org), r.dir);
  const V3 hi = div3(sub3(mk3(b.upper), r.org), r.dir);
  const V3 nr = min3(lo, hi), fr = max3(lo, hi);
  t0 = fmax_t(r.tmin, rmax3(nr));
  t1 = fmin_t(r.tmax, rmin3(fr));
  return t0 < t1;
}

// generateRay (deviceCode.cu:88-101) for the jittered screen position
// (px + rx, py + ry), remapped into the sub-image window when one is active
// (renderFrame_Impl, deviceCode.cu:1286-1294)
EXA_D V3 camera_dir(const exa_launch_params &lp, int px, int py, float rx, float ry, int width, int height)
{
  float sx = (float)px + rx, sy = (float)py + ry;
  if (lp.subImage.active) {
    const float W = (float)width, H = (float)height;
    sx = __fdiv_rn(sx, W);
    sy = __fdiv_rn(sy, H);
    sx = (1.f - sx) * lp.subImage.value.lower.x + sx * lp.subImage.value.upper.x;
    sy = (1.f - sy) * lp.subImage.value.lower.y + sy * lp.subImage.value.upper.y;
    sx *= W;
    sy *= H;
  }
  V3 dir = add3(add3(mk3(lp.camera.dir_00), smul(sx, mk3(lp.camera.dir_du))), smul(sy, mk3(lp.camera.dir_dv)));
  dir = norm3(dir);
  if (fabsf(dir.x) < 1e-5f) dir.x = 1e-5f;
  if (fabsf(dir.y) < 1e-5f) dir.y = 1e-5f;
  if (fabsf(dir.z) < 1e-5f) dir.z = 1e-5f;
  return dir;
}

// the gridlet checker of the Gridlets and Teaser shade modes
// (deviceCode.cu:635-649, 655-670): 0 stitching element (red), 1 white,
// 2 blue cell
EXA_D int checker_index(const AccelView &A, const exa_sample &s)
{
  if (s.cellID == -1) return 0;
  const exa_gridlet g = A.gridlets[s.primID];
  const int ix = s.cellID % g.dims.x, iy = s.cellID / g.dims.x % g.dims.y, iz = s.cellID / (g.dims.x * g.dims.y);
  int col = (ix % 2 == iy % 2);
  col = (iz % 2 == 0) ? col : !col;
  return col == 0 ? 1 : 2;
}

// the Teaser shade mode's colour (deviceCode.cu:652-695): the TF colour
// rgb1 on one side of a screen-space diagonal band, the checker colour on
// the other, blended across the band
EXA_D V3 teaser_rgb(V3 rgb1, int checker, int px, int py, int width, int height)
{
  const V3 rgb2 = checker == 0 ? mk3(1.f, 0.f, 0.f) : (checker == 1 ? mk3(1.f, 1.f, 1.f) : mk3(0.f, 0.f, .7f));
  const float u = __fdiv_rn((float)px, (float)width), v = __fdiv_rn((float)py, (float)height);
  const float A = .6f - .4f, B = .4f - .6f;
  const float C1 = A * .4f + B * .6f, C2 = A * .6f + B * .4f, C = A * u + B * v;
  if (C <= C1) return rgb1;
  if (C >= C2) return rgb2;
  return mk3(__fdiv_rn(rgb1.x * (C2 - C) + rgb2.x * (C - C1), C2 - C1),
             __fdiv_rn(rgb1.y * (C2 - C) + rgb2.y * (C - C1), C2 - C1),
             __fdiv_rn(rgb1.z * (C2 - C) + rgb2.z * (C - C1), C2 - C1));
}

// deviceCode.cu:625-651 (Default, Gridlets)
EXA_D float4 classify(const AccelView &A, const exa_launch_params &lp, const exa_sample &s)
{
  float4 xf = lookup_tf(lp, s.value);
  if (lp.shadeMode == EXA_SHADE_MODE_GRIDLETS) {
    if (s.cellID == -1) {
      xf.x = 1.f; xf.y = 0.f; xf.z = 0.f;
    } else {
      const exa_gridlet g = A.gridlets[s.primID];
      const int ix = s.cellID % g.dims.x, iy = s.cellID / g.dims.x % g.dims.y, iz = s.cellID / (g.dims.x * g.dims.y);
      int col = (ix % 2 == iy % 2);
      col = (iz % 2 == 0) ? col : !col;
      if (col == 0) { xf.x = 1.f; xf.y = 1.f; xf.z = 1.f; }
      else { xf.x = 0.f; xf.y = 0.f; xf.z = 0.7f; }
    }
  }
  return xf;
}

// dda3 state (DDA.h:34-70)
struct Dda {
  V3 tnext, dist;
  V3i cell, step, stop;
  float t0, tmax;
};

EXA_D void dda_init(Dda &d, V3 org, V3 dir, float tmin, float tmax, const exa_grid_traversable &G)
{
  const V3i dims = {G.dims.x, G.dims.y, G.dims.z};
  const V3 rcp = mk3(__fdiv_rn(1.f, dir.x), __fdiv_rn(1.f, dir.y), __fdiv_rn(1.f, dir.z));
  const V3 lo = mul3(sub3(mk3(G.bounds.lower), org), rcp);
  const V3 hi = mul3(sub3(mk3(G.bounds.upper), org), rcp);
  const V3 tnear = min3(lo, hi), tfar = max3(lo, hi);
  d.cell = project_on_grid(org, dims, G.bounds);
  d.dist = div3(sub3(tfar, tnear), mk3((float)dims.x, (float)dims.y, (float)dims.z));
  d.step.x = dir.x > 0.f ? 1 : -1; d.step.y = dir.y > 0.f ? 1 : -1; d.step.z = dir.z > 0.f ? 1 : -1;
  d.stop.x = dir.x > 0.f ? dims.x : -1; d.stop.y = dir.y > 0.f ? dims.y : -1; d.stop.z = dir.z > 0.f ? dims.z : -1;
  d.tnext.x = dir.x > 0.f ? tnear.x + (float)(d.cell.x + 1) * d.dist.x : tnear.x + (float)(dims.x - d.cell.x) * d.dist.x;
  d.tnext.y = dir.y > 0.f ? tnear.y + (float)(d.cell.y + 1) * d.dist.y : tnear.y + (float)(dims.y - d.cell.y) * d.dist.y;
  d.tnext.z = dir.z > 0.f ? tnear.z + (float)(d.cell.z + 1) * d.dist.z : tnear.z + (float)(dims.z - d.cell.z) * d.dist.z;
  // A direction component of 0 (or one whose reciprocal overflows) makes
  // that axis's crossing NaN, and DDA.h's loop then never advances; such an
  // axis is never crossed, so its next crossing is at +inf.  Every other ray
  // is unaffected.
  if (isnan(d.tnext.x)) d.tnext.x = INFINITY;
  if (isnan(d.tnext.y)) d.tnext.y = INFINITY;
  if (isnan(d.tnext.z)) d.tnext.z = INFINITY;
  d.t0 = fmax_t(tmin, 0.f);
  d.tmax = tmax;
}

// DDA.h:352-375: advance every axis tied with the closest crossing
// dda_next with the step and stop of each axis taken from the ray
// direction (as dda_init sets them), so that a walk does not carry them
EXA_D bool dda_next_dir(Dda &d, V3 dir, const exa_vec3i dims)
{
  const float t1 = fmin_t(rmin3(d.tnext), d.tmax);
  const float tc = rmin3(d.tnext);
  if (d.tnext.x == tc) {
    d.tnext.x += d.dist.x;
    d.cell.x += dir.x > 0.f ? 1 : -1;
    if (d.cell.x == (dir.x > 0.f ? dims.x : -1)) return false;
  }
  if (d.tnext.y == tc) {
    d.tnext.y += d.dist.y;
    d.cell.y += dir.y > 0.f ? 1 : -1;
    if (d.cell.y == (dir.y > 0.f ? dims.y : -1)) return false;
  }
  if (d.tnext.z == tc) {
    d.tnext.z += d.dist.z;
    d.cell.z += dir.z > 0.f ? 1 : -1;
    if (d.cell.z == (dir.z > 0.f ? dims.z : -1)) return false;
  }
  d.t0 = t1;
  return true;
}

EXA_D bool dda_next(Dda &d)
{
  const float t1 = fmin_t(rmin3(d.tnext), d.tmax);
  const float tc = rmin3(d.tnext);
  if (d.tnext.x == tc) { d.tnext.x += d.dist.x; d.cell.x += d.step.x; if (d.cell.x == d.stop.x) return false; }
  if (d.tnext.y == tc) { d.tnext.y += d.dist.y; d.cell.y += d.step.y; if (d.cell.y == d.stop.y) return false; }
  if (d.tnext.z == tc) { d.tnext.z += d.dist.z; d.cell.z += d.step.z; if (d.cell.z == d.stop.z) return false; }
  d.t0 = t1;
  return true;
}

// clip planes as the integrators apply them after the box test
// (deviceCode.cu:53-60 intersect; :882-893, 1010-1021, 1097-1106, 1143-1154,
// 1229-1240): a front-facing plane moves t0 forward, a back-facing one t1
// back.  A ray parallel to a plane gets FLT_MAX with backFace false, which
// moves t0 to FLT_MAX, as in the reference.
EXA_D void clip_planes(const exa_launch_params &lp, const RayS &ray, float &t0, float &t1)
{
  for (int i = 0; i < EXA_CLIP_PLANES_MAX; ++i) {
    if (!lp.clipPlanes[i].enabled) continue;
    const V3 N = mk3(lp.clipPlanes[i].N);
    const float sd = dot3(N, ray.dir);
    bool backFace = false;
    float pt = 3.40282347e+38f;
    if (sd != 0.f) {
      backFace = sd > 0.f;
      pt = __fdiv_rn(lp.clipPlanes[i].d - dot3(N, ray.org), sd);
    }
    if (pt > t0 && !backFace) t0 = fmax_t(t0, pt);
    if (pt < t1 && backFace) t1 = fmin_t(pt, t1);
  }
}

struct PathCtx {
  const AccelView &A;
  const exa_launch_params &lp;
  uint32_t err;
  bool counting;
};

EXA_D void cnt_add(const PathCtx &c, int k, unsigned v = 1)
{
  if (c.counting) s_cnt[k][threadIdx.x] += v;
}

EXA_D PathCtx make_ctx(const AccelView &A, const exa_launch_params &lp)
{
  PathCtx c{A, lp, 0u, lp.ext.stepCounters != nullptr};
  if (c.counting)
    for (int k = 0; k < CNT_N; ++k) s_cnt[k][threadIdx.x] = 0u;
  return c;
}

// device-error bits and this thread's counters to global memory; any lane
// mask
EXA_D void flush_counters(const PathCtx &c, const exa_launch_params &lp)
{
  if (c.err && lp.ext.deviceErrors) atomicOr(lp.ext.deviceErrors, c.err);
  if (c.counting)
    for (int k = 0; k < CNT_N; ++k) {
      const unsigned v = s_cnt[k][threadIdx.x];
      if (v) atomicAdd(lp.ext.stepCounters + k, (unsigned long long)v);
    }
}

// make_orthonormal_basis (deviceCode.cu:144-149) + HG sampling (:965-985)
EXA_D V3 hg_sample(V3 wo, float g, Rng &rng)
{
  const bool gnz = fabsf(g) >= 1.19209290e-07f;
  const float u1 = rng.next();
  const float u2 = rng.next();
  const float a = gnz ? __fdiv_rn(1.f - g * g, 1.f - g + 2.f * g * u1) : 0.f;
  const float cost = gnz ? __fdiv_rn(1.f + g * g - a * a, 2.f * g) : 1.f - 2.f * u1;
  const float sint = __fsqrt_rn(fmaxf(0.f, 1.f - cost * cost));
  float sphi, cphi;
  exa_sincos_turns(u2, sphi, cphi);
  const V3 v = fabsf(wo.x) > fabsf(wo.y) ? norm3(mk3(-wo.z, 0.f, wo.x)) : norm3(mk3(0.f, wo.z, -wo.y));
  const V3 u = cross3(v, wo);
  const V3 mw = mk3(-wo.x, -wo.y, -wo.z);
  return add3(add3(muls(u, sint * cphi), muls(v, sint * sphi)), muls(mw, cost));
}

EXA_D int num_lights(const exa_launch_params &lp)
{
  int n = 0;
  for (int i = 0; i < EXA_LIGHTS_MAX; ++i) if (lp.lights[i].on) n++;
  return n;
}

EXA_D uint32_t make_8bit(float f) { return (uint32_t)imin_t(255, imax_t(0, (int)(f * 256.f))); }

// ------------------------------------------------------------------------
// sampleInteraction (deviceCode.cu:699-854) as a resumable walk: begin()
// is the ray set-up and dda3 prologue, step() is one iteration of the
// delta-tracking (Woodcock, :726-783) or ratio-tracking (:785-839) loop,
// with the DDA advance (DDA.h:339-376) folded in whenever the free flight
// leaves the current macrocell.  Executing step() until it returns false
// performs exactly the operations of the nested reference loops.
struct Walk {
  V3 org, dir;      // voxel space
  Dda dda;
  V3 pos;           // last sample position (voxel space)
  float4 xf;        // last classified sample
  float t, t1, maj, Tr;
  int primID;       // the cached gridlet (testSample), -1: none
  int steps, ncells;
  int type;
  bool needCell;
};

EXA_D void walk_begin(Walk &w, const exa_launch_params &lp, RayS ray)
{
  ray.org = xfm_point(lp.voxelSpaceTransform, ray.org);
  ray.dir = xfm_vector(lp.voxelSpaceTransform, ray.dir);
  const float dt_scale = len3(ray.dir);
  ray.dir = norm3(ray.dir);
  ray.tmin = ray.tmin * dt_scale;
  ray.tmax = ray.tmax * dt_scale;
  w.org = ray.org;
  w.dir = ray.dir;
  dda_init(w.dda, ray.org, ray.dir, ray.tmin, ray.tmax, lp.majorantGrid);
  w.t = w.dda.t0;  // the walk's position along the ray: here its entry into the grid
  w.pos = mk3(0.f, 0.f, 0.f);
  w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
  w.Tr = 1.f;
  w.type = BOUNDARY;
  w.ncells = 0;
  w.primID = -1;
  w.needCell = true;
}

// walk_advance: the DDA advance and the free flight of one step.
// Returns 0 when the walk ended, 1 when the step took no sample (the flight
// left the macrocell), 2 when a sample at w.pos is due.
enum : int { WALK_END = 0, WALK_ON = 1, WALK_SAMPLE = 2 };

EXA_D int walk_advance(Walk &w, PathCtx &c, Rng &rng)
{
  const exa_launch_params &lp = c.lp;
  const exa_grid_traversable &G = lp.majorantGrid;
  const float scale = lp.transferFunc.opacityScale;
  while (w.needCell) {
    if (++w.ncells > lp.ext.ddaCellCap) {  // the host fills the caps (fillLoopCaps)
      c.err |= EXA_DEVERR_DDA_CAP;
      return WALK_END;
    }
    w.t1 = fmin_t(rmin3(w.dda.tnext), w.dda.tmax);
    const int leafID = (w.dda.cell.z * G.dims.y + w.dda.cell.y) * G.dims.x + w.dda.cell.x;
    cnt_add(c, CNT_DDA);
    if (!exa_in_range(leafID, (long long)G.dims.x * G.dims.y * G.dims.z, c.err)) return WALK_END;
    w.maj = __ldg(lp.maxOpacities + leafID);
    // w.t is the macrocell's entry distance: the walk's start, or the exit of
    // the macrocell before, which is where dda_next_dir puts its t0
    w.primID = -1;  // the gridlet cache ends with the macrocell (deviceCode.cu:731-760)
    w.steps = 0;
    if (w.maj <= 0.f) {
      w.t = w.t1;
      if (!dda_next_dir(w.dda, w.dir, G.dims)) return WALK_END;
      continue;
    }
    w.needCell = false;
  }
  if (++w.steps > lp.ext.trackStepCap) {
    c.err |= EXA_DEVERR_TRACK_CAP;
    return WALK_END;
  }
  w.t -= __fdiv_rn(exa_log(1.f - rng.next()), w.maj * scale);
  if (w.t >= w.t1) {
    w.needCell = true;
    w.t = w.t1;  // the next macrocell's entry (a walk that ends here reports no distance)
    return dda_next_dir(w.dda, w.dir, G.dims) ? WALK_ON : WALK_END;
  }
  w.pos = add3(w.org, muls(w.dir, w.t));
  return WALK_SAMPLE;
}

// the exact sampler at w.pos: the cached gridlet first (testSample,
// deviceCode.cu:749), then the full point location
EXA_D exa_sample walk_sample_exact(const Walk &w, PathCtx &c)
{
  exa_sample s =
      test_sample(c.A, w.pos, w.primID < 0 || exa_in_range(w.primID, c.A.numGridlets, c.err) ? w.primID : -1);
  if (s.primID < 0) {
    QueryStats q{0u, 0u, 0u};
    s = sample_field(c.A, w.pos, c.lp.ext.cullTransparentPrims != 0, c.err, &q);
    if (c.counting) {
      cnt_add(c, CNT_MISS);
      cnt_add(c, CNT_TABLES, q.tables);
      cnt_add(c, CNT_GTESTS, q.gridletTests);
      cnt_add(c, CNT_ELEMQ, q.elemLists);
    }
  }
  if (c.counting) {
    cnt_add(c, CNT_FIELD);
    if (s.primID >= 0) cnt_add(c, s.cellID != -1 ? CNT_GRIDLET : CNT_ELEM);
  }
  return s;
}

// the collision test of one step given its sample; primID -1 is empty
// space, -2 a value of the learned field (never cached).  Returns false
// when the walk ended.  `teaser`: the frame renders the Teaser shade mode;
// `learned`: the sample may come from the learned field (both compile-time
// constants in every caller, so that the other walks carry none of their
// code).
EXA_D bool walk_collide(Walk &w, PathCtx &c, Rng &rng, const bool shadow, const exa_sample &s,
                        const bool teaser = false, const bool learned = false)
{
  const exa_launch_params &lp = c.lp;
  const float scale = lp.transferFunc.opacityScale;
  if (s.primID == -1) return true;
  if (s.cellID != -1) w.primID = s.primID;
  w.xf = classify(c.A, lp, s);
  const float sigmaT = w.xf.w;
  float sigmaS = sigmaT * scale;
  if (learned && s.primID == -2 && sigmaS > w.maj) {
    // a learned density above the macrocell's widened majorant is limited
    // to it: tracking stays unbiased for the limited field
    if (c.counting) cnt_add(c, CNT_VIOL);
    sigmaS = w.maj;
  }
  if (!shadow) {
    const float u = rng.next();
    if (sigmaS >= u * w.maj) {
      w.Tr = 0.f;
      w.type = SCATTERING;
      // the Teaser shade mode blends the albedo by screen position at the
      // event; the walk passes on the sample's checker colour in xf.w,
      // which the event does not read otherwise
      if (teaser) w.xf.w = (float)checker_index(c.A, s);
      return false;
    }
  } else {
    w.Tr *= 1.f - __fdiv_rn(sigmaS, w.maj);
    if (w.Tr <= 0.f) {
      w.type = SCATTERING;
      return false;
    }
  }
  return true;
}

EXA_D bool walk_step(Walk &w, PathCtx &c, Rng &rng, const bool shadow)
{
  const int st = walk_advance(w, c, rng);
  if (st != WALK_SAMPLE) return st == WALK_ON;
  const exa_sample s = walk_sample_exact(w, c);
  return walk_collide(w, c, rng, shadow, s);
}

// The wavefront walk kernels' unit of work per loop iteration: up to
// EXA_WF_ITER_STEPS steps, each with up to EXA_WF_ADVANCE_MAX macrocell
// advances before its sample.  A lane's own sequence of operations (and so
// its result) does not depend on these; they trade loop overhead against
// divergence between lanes.  Measured on the 1024^2 x 16 spp medium
// workload: 1 advance per iteration 182 M paths/s, 2: 218 M, 3: 231 M,
// 4: 232 M, 6: 226 M, 8: 219 M, 64: 188 M; two steps per iteration no
// better.  Again with the later walk kernel: 3: 287.2 M, 4: 287.3 M, 6:
// 275.4 M.
#ifndef EXA_WF_ADVANCE_MAX
#define EXA_WF_ADVANCE_MAX 4
#endif
#ifndef EXA_WF_ITER_STEPS
#define EXA_WF_ITER_STEPS 1
#endif
template <bool TEASER = false>
EXA_D bool walk_iteration(Walk &w, PathCtx &c, Rng &rng, const bool shadow)
{
  for (int k = 0; k < EXA_WF_ITER_STEPS; ++k) {
    int st, a = 0;
    do {
      st = walk_advance(w, c, rng);
    } while (st == WALK_ON && ++a < EXA_WF_ADVANCE_MAX);
    if (st == WALK_END) return false;
    if (st == WALK_ON) continue;
    const exa_sample s = walk_sample_exact(w, c);
    if (!walk_collide(w, c, rng, shadow, s, TEASER)) return false;
  }
  return true;
}

// ------------------------------------------------------------------------
// renderFrame_Impl (deviceCode.cu:1268-1345) with directLightingIntegrate
// (:1126-1207) or pathTracingIntegrate (:991-1120) and sampleLight
// (:856-926), as a per-lane state machine in a persistent kernel.  The unit
// of work is one camera sample (pixel, s) with its own RNG stream; each loop
// iteration advances every lane by one tracking step or integrator event,
// and a lane that finishes its sample takes the next one from a global
// counter (one atomic per warp).  Jobs run pixel-major (the spp samples of
// a pixel are adjacent) over 16x8 pixel tiles.  Each sample's colour goes to
// a scratch slot; k_resolve then sums a pixel's samples in sample order, as
// renderFrame_Impl's spp loop does, and applies the progressive average.
enum : int { PH_FETCH = 0, PH_TRACK = 1, PH_DONE = 2 };

struct Lane {
  int px, py, pixelID, s;
  int frame = 0;           // frame of a batch (0 for a single frame)
  RayS ray;
  V3 throughput, Ld, pos, albedo;
  unsigned bounce;
  float lightDen, lightI;  // point light: (Tr / lightDen) * lightI; directional: Tr * lightI
  bool lightDirectional = false;
  bool shadow;             // the running walk is a shadow walk
  // surface mesh: the first triangle on the running walk's ray (-1: none;
  // after a primary walk, >= 0 only if the walk ended on that surface)
  int meshPrim = -1;
  float meshT = 0.f;
  float shadowMesh = -1.f; // shadow walk that reached a surface: max(0, N.l), else -1
  int phase;
  Rng rng;
  Walk w;
};

// lambertianSample (deviceCode.cu:932-951): cosine-weighted direction about
// N; the two draws are taken in order (u1, then u2), 2 pi u2 via the
// project's turn-based sine/cosine
EXA_D V3 lambertian_sample(V3 N, Rng &rng)
{
  const V3 w = N;
  const V3 v = fabsf(w.x) > fabsf(w.y) ? norm3(mk3(-w.z, 0.f, w.x)) : norm3(mk3(0.f, w.z, -w.y));
  const V3 u = cross3(v, w);
  const float u1 = rng.next();
  const float u2 = rng.next();
  const float r = __fsqrt_rn(u1);
  float sn, cs;
  exa_sincos_turns(u2, sn, cs);
  const V3 sp = mk3(r * cs, r * sn, __fsqrt_rn(1.f - u1));
  return norm3(add3(add3(smul(sp.x, u), smul(sp.y, v)), smul(sp.z, w)));
}

template <int INTEGRATOR>
struct Machine {
  PathCtx &c;
  const exa_launch_params &lp;
  int width, height, numLights;
  unsigned maxB;
  float4 *colors;

  EXA_D float4 background(const Lane &L) const
  {
    const float tb = __fdiv_rn((float)L.py, (float)height);
    return make_float4((1.f - tb) * 1.f + tb * 0.5f, (1.f - tb) * 1.f + tb * 0.7f, (1.f - tb) * 1.f + tb * 1.f, 1.f);
  }

  EXA_D void finish_sample(Lane &L, float4 col)
  {
    colors[(size_t)L.pixelID * lp.render.spp + L.s] = col;
    cnt_add(c, CNT_PATHS);
    L.phase = PH_FETCH;
  }

  // generateRay (deviceCode.cu:88-101) and the integrator's box test
  EXA_D void begin_sample(Lane &L)
  {
    L.pixelID = L.px + width * L.py;
    L.rng.init((uint32_t)L.pixelID, (uint32_t)lp.accumID, lp.ext.frameID, (uint32_t)L.s);
    if (L.s == 0) {
      if (lp.ext.traceT) lp.ext.traceT[L.pixelID] = -1.f;
      if (lp.ext.traceTr) lp.ext.traceTr[L.pixelID] = -1.f;
    }
    const float rx = L.rng.next();
    const float ry = L.rng.next();
    const V3 dir = camera_dir(lp, L.px, L.py, rx, ry, width, height);
    L.ray.org = mk3(lp.camera.org);
    L.ray.dir = dir;
    L.ray.tmin = 0.f;
    L.ray.tmax = 1e10f;
    L.throughput = mk3(1.f, 1.f, 1.f);
    L.Ld = mk3(0.f, 0.f, 0.f);
    L.bounce = 0;
    float t0 = 1e30f, t1 = -1e30f;
    if (!box_test(L.ray, lp.worldSpaceBounds, t0, t1)) {
      if (INTEGRATOR == EXA_PATH_TRACING_INTEGRATOR) finish_path(L);
      else finish_sample(L, background(L));
      return;
    }
    clip_planes(lp, L.ray, t0, t1);
    L.ray.org = add3(L.ray.org, muls(L.ray.dir, t0));
    t1 -= t0;
    L.ray.tmax = t1;
    mesh_clip(L, L.ray);
    L.shadow = false;
    walk_begin(L.w, lp, L.ray);
    L.phase = PH_TRACK;
  }

  // the first surface along a walk's ray ends the walk there
  // (deviceCode.cu:1032-1039)
  EXA_D void mesh_clip(Lane &L, RayS &ray)
  {
    L.meshPrim = -1;
    if (!lp.meshBVH) return;
    const MeshHit h = trace_mesh(*reinterpret_cast<const MeshView *>(lp.meshBVH), ray.org, ray.dir, ray.tmax);
    if (h.primID >= 0) {
      L.meshPrim = h.primID;
      L.meshT = h.t;
      ray.tmax = fmin_t(ray.tmax, h.t);
    }
  }

  // the geometric normal of mesh triangle prim, as the closest hit computes
  // it (path records keep the triangle, not its normal)
  EXA_D V3 mesh_normal(int prim) const
  {
    const MeshView &M = *reinterpret_cast<const MeshView *>(lp.meshBVH);
    const V3 a = tri_vertex(M, prim, 0), b = tri_vertex(M, prim, 1), c = tri_vertex(M, prim, 2);
    return norm3(cross3(sub3(b, a), sub3(c, a)));
  }

  // sampleLight's mesh test (deviceCode.cu:897-904, 921-922)
  EXA_D void shadow_mesh(Lane &L, RayS &ray)
  {
    L.shadowMesh = -1.f;
    if (!lp.meshBVH) return;
    const MeshHit h = trace_mesh(*reinterpret_cast<const MeshView *>(lp.meshBVH), ray.org, ray.dir, ray.tmax);
    if (h.primID >= 0) {
      ray.tmax = fmin_t(ray.tmax, h.t);
      L.shadowMesh = fmaxf(0.f, dot3(h.Ng, ray.dir));
    }
  }

  // sampleLight prologue (deviceCode.cu:866-895): pick a light, start the
  // shadow walk from pos (world space)
  EXA_D void begin_light(Lane &L)
  {
    int which = (int)(L.rng.next() * (float)numLights);
    if (which == numLights) which = 0;
    RayS ray;
    float t00 = 1e30f, t11 = -1e30f;
    ray.org = L.pos;
    ray.tmin = 0.f;
    if (lp.ext.lightType[which] == EXA_LIGHT_DIRECTIONAL) {
      ray.dir = norm3(mk3(lp.lights[which].pos));
      ray.tmax = 1e30f;
      box_test(ray, lp.worldSpaceBounds, t00, t11);
      clip_planes(lp, ray, t00, t11);
      ray.tmax = t11;
      shadow_mesh(L, ray);
      L.lightDirectional = true;
    } else {
      V3 lightDir = sub3(mk3(lp.lights[which].pos), L.pos);
      const float ld = len3(xfm_vector(lp.lightSpaceTransform, lightDir));
      const float ldWorld = len3(lightDir);
      lightDir = norm3(lightDir);
      ray.dir = lightDir;
      ray.tmax = ldWorld;
      box_test(ray, lp.worldSpaceBounds, t00, t11);
      clip_planes(lp, ray, t00, t11);
      ray.tmax = t11;
      shadow_mesh(L, ray);
      L.lightDen = ld * ld;
      L.lightDirectional = false;
    }
    L.lightI = lp.lights[which].intensity;
    L.shadow = true;
    walk_begin(L.w, lp, ray);
    L.phase = PH_TRACK;
  }

  // end of pathTracingIntegrate (deviceCode.cu:1111-1119)
  EXA_D void finish_path(Lane &L)
  {
    if (numLights == 0) L.Ld = mk3(1.f, 1.f, 1.f);
    const V3 Lr = mul3(L.Ld, L.throughput);
    finish_sample(L, L.bounce ? make_float4(Lr.x, Lr.y, Lr.z, 1.f) : background(L));
  }

  // pathTracingIntegrate (:1092-1107): phase function, next segment
  EXA_D void scatter(Lane &L)
  {
    V3 sd;
    if (L.meshPrim >= 0) {
      // the event was a surface: Lambertian BRDF (deviceCode.cu:1084-1087)
      const V3 Ng = mesh_normal(L.meshPrim);
      sd = lambertian_sample(Ng, L.rng);
      L.throughput = muls(L.throughput, fmaxf(0.f, dot3(sd, Ng)));
      L.pos = add3(L.pos, smul(16.f, norm3(sd)));
    } else {
      const V3 wo = mk3(-L.ray.dir.x, -L.ray.dir.y, -L.ray.dir.z);
      sd = hg_sample(wo, lp.ext.hgG, L.rng);
    }
    L.ray.org = L.pos;
    L.ray.dir = sd;
    float t0 = 1e30f, t1 = -1e30f;
    box_test(L.ray, lp.worldSpaceBounds, t0, t1);
    clip_planes(lp, L.ray, t0, t1);
    L.ray.tmax = t1;
    mesh_clip(L, L.ray);
    L.shadow = false;
    walk_begin(L.w, lp, L.ray);
  }

  EXA_D void primary_done(Lane &L)
  {
    // first interaction of the pixel's first sample: its free-flight distance
    if (L.s == 0 && L.bounce == 0 && L.w.type == SCATTERING && lp.ext.traceT) lp.ext.traceT[L.pixelID] = L.w.t;
    L.pos = xfm_point(lp.ext.voxelSpaceTransformInv, L.w.pos);
    float4 xf = L.w.xf;
    if (lp.shadeMode == EXA_SHADE_MODE_TEASER && L.w.type == SCATTERING) {
      const V3 rgb = teaser_rgb(mk3(xf.x, xf.y, xf.z), (int)xf.w, L.px, L.py, width, height);
      xf.x = rgb.x; xf.y = rgb.y; xf.z = rgb.z;
    }
    const bool surface = L.w.type == BOUNDARY && L.meshPrim >= 0;
    if (!surface) L.meshPrim = -1;  // scatter() reads it as "the event was a surface"
    // a surface event (deviceCode.cu:1056-1059, 1182-1185): just past the hit, albedo kd = 0.8
    if (surface) L.pos = add3(add3(L.ray.org, muls(L.ray.dir, L.meshT)), muls(norm3(L.ray.dir), 1.f));
    if (INTEGRATOR == EXA_PATH_TRACING_INTEGRATOR) {
      if (L.w.type == BOUNDARY && !surface) { finish_path(L); return; }
      if (L.bounce++ >= maxB) {
        L.throughput = mk3(0.f, 0.f, 0.f);
        finish_path(L);
        return;
      }
      const V3 albedo = surface ? mk3(.8f, .8f, .8f)
                                : (lp.ext.albedo < 0.f ? mk3(xf.x, xf.y, xf.z)
                                                       : mk3(lp.ext.albedo, lp.ext.albedo, lp.ext.albedo));
      L.throughput = mul3(L.throughput, albedo);
      const float P = rmax3(L.throughput);
      if (P < 0.2f) {
        if (L.rng.next() > P) {
          L.throughput = mk3(0.f, 0.f, 0.f);
          finish_path(L);
          return;
        }
        L.throughput = div3(L.throughput, mk3(P, P, P));
      }
      L.throughput = add3(L.throughput, mk3(0.f, 0.f, 0.f));
      if (numLights > 0) begin_light(L);
      else scatter(L);
    } else {
      if (L.w.type == BOUNDARY && !surface) { finish_sample(L, background(L)); return; }
      L.albedo = surface ? mk3(.8f, .8f, .8f)
                         : (lp.ext.albedo < 0.f ? mk3(xf.x, xf.y, xf.z)
                                                : mk3(lp.ext.albedo, lp.ext.albedo, lp.ext.albedo));
      if (numLights > 0) {
        begin_light(L);
      } else {
        V3 tp = mul3(mk3(1.f, 1.f, 1.f), L.albedo);
        // surfaces without lights: a headlight (deviceCode.cu:1196-1198)
        if (surface)
          tp = muls(tp, fmaxf(0.f, dot3(mk3(-L.ray.dir.x, -L.ray.dir.y, -L.ray.dir.z), mesh_normal(L.meshPrim))));
        finish_sample(L, make_float4(tp.x, tp.y, tp.z, 1.f));
      }
    }
  }

  EXA_D void shadow_done(Lane &L)
  {
    // a shadow walk that reached a surface scales by max(0, N.l)
    // (deviceCode.cu:921-925)
    const bool lit = L.w.type == BOUNDARY && L.shadowMesh >= 0.f;
    float I;
    if (L.lightDirectional) I = lit ? L.shadowMesh * L.w.Tr * L.lightI : L.w.Tr * L.lightI;
    else I = lit ? __fdiv_rn(L.shadowMesh * L.w.Tr, L.lightDen) * L.lightI : __fdiv_rn(L.w.Tr, L.lightDen) * L.lightI;
    const bool first = L.s == 0 && (INTEGRATOR != EXA_PATH_TRACING_INTEGRATOR || L.bounce == 1);
    if (first && lp.ext.traceTr) lp.ext.traceTr[L.pixelID] = L.w.Tr;
    if (INTEGRATOR == EXA_PATH_TRACING_INTEGRATOR) {
      L.Ld = add3(L.Ld, mul3(L.throughput, mk3(I, I, I)));
      scatter(L);
    } else {
      const V3 tp = mul3(mk3(1.f, 1.f, 1.f), mul3(L.albedo, mk3(I, I, I)));
      finish_sample(L, make_float4(tp.x, tp.y, tp.z, 1.f));
    }
  }

  EXA_D void advance(Lane &L)
  {
    if (walk_step(L.w, c, L.rng, L.shadow)) return;
    if (L.shadow) shadow_done(L);
    else primary_done(L);
  }
};

template <int INTEGRATOR>
__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_render(const __grid_constant__ AccelView A,
                                                const __grid_constant__ exa_launch_params lp, int width, int height,
                                                unsigned *jobCounter, float4 *colors)
{
  PathCtx c = make_ctx(A, lp);
  Machine<INTEGRATOR> M{c, lp, width, height, num_lights(lp), (unsigned)lp.ext.maxBounces, colors};
  const int spp = lp.render.spp;
  const int tilesX = (width + 15) / 16;
  const unsigned numJobs = (unsigned)(tilesX * ((height + 7) / 8) * 128) * (unsigned)spp;
  const unsigned lane = threadIdx.x & 31;
  Lane L;
  L.phase = PH_FETCH;
  while (true) {
    // warp-aggregated job fetch for the lanes that need a sample
    unsigned need = __ballot_sync(0xffffffffu, L.phase == PH_FETCH);
    while (need) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if ((int)lane == leader) base = atomicAdd(jobCounter, (unsigned)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (L.phase == PH_FETCH) {
        const unsigned job = base + __popc(need & ((1u << lane) - 1u));
        if (job >= numJobs) {
          L.phase = PH_DONE;
        } else {
          const unsigned pj = job / (unsigned)spp;
          L.s = (int)(job - pj * (unsigned)spp);
          const int tile = (int)(pj >> 7), within = (int)(pj & 127);
          L.px = (tile % tilesX) * 16 + (within & 15);
          L.py = (tile / tilesX) * 8 + (within >> 4);
          if (L.px < width && L.py < height) M.begin_sample(L);
        }
      }
      // lanes whose job fell outside the frame, or whose sample finished
      // without tracking, fetch again
      need = __ballot_sync(0xffffffffu, L.phase == PH_FETCH);
    }
    if (__all_sync(0xffffffffu, L.phase == PH_DONE)) break;
    if (L.phase == PH_TRACK) M.advance(L);
  }
  flush_counters(c, lp);
}

// ------------------------------------------------------------------------
// Nested-loop form of the same integrators (one thread runs a whole camera
// sample, or a whole pixel, to completion): sampleInteraction as one walk
// run to its end, then the integrator logic in program order.
// EXA_TRACK_NOINLINE 1: one out-of-line copy of the walk, shared by primary
// and shadow rays (smaller code); 0: inlined at both call sites
#ifndef EXA_TRACK_NOINLINE
#define EXA_TRACK_NOINLINE 1
#endif
#if EXA_TRACK_NOINLINE
#define EXA_TRACK_ATTR static __device__ __noinline__
#else
#define EXA_TRACK_ATTR EXA_D
#endif

EXA_TRACK_ATTR int track_walk(PathCtx &c, RayS ray, const bool shadow, Rng &rngRef, V3 &posOut, float &TrOut,
                              float4 &xf, float &tOut)
{
  Rng rng = rngRef;
  Walk w;
  walk_begin(w, c.lp, ray);
  while (walk_step(w, c, rng, shadow)) {
  }
  rngRef = rng;
  posOut = xfm_point(c.lp.ext.voxelSpaceTransformInv, w.pos);
  TrOut = w.Tr;
  xf = w.xf;
  tOut = w.t;
  return w.type;
}

template <bool SHADOW>
EXA_D int track(PathCtx &c, RayS ray, V3 &posOut, float &TrOut, float4 &xf, Rng &rng, float &tOut)
{
  return track_walk(c, ray, SHADOW, rng, posOut, TrOut, xf, tOut);
}

EXA_D V3 light_nested(PathCtx &c, V3 pos, Rng &rng, int numLights, float *trOut)
{
  const exa_launch_params &lp = c.lp;
  int which = (int)(rng.next() * (float)numLights);
  if (which == numLights) which = 0;
  RayS ray;
  float Tr, t00 = 1e30f, t11 = -1e30f, tt;
  V3 np;
  float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);
  ray.org = pos;
  ray.tmin = 0.f;
  if (lp.ext.lightType[which] == EXA_LIGHT_DIRECTIONAL) {
    ray.dir = norm3(mk3(lp.lights[which].pos));
    ray.tmax = 1e30f;
    box_test(ray, lp.worldSpaceBounds, t00, t11);
    clip_planes(lp, ray, t00, t11);
    ray.tmax = t11;
    track<true>(c, ray, np, Tr, xf, rng, tt);
    if (trOut) *trOut = Tr;
    const float I = Tr * lp.lights[which].intensity;
    return mk3(I, I, I);
  }
  V3 lightDir = sub3(mk3(lp.lights[which].pos), pos);
  const float ld = len3(xfm_vector(lp.lightSpaceTransform, lightDir));
  const float ldWorld = len3(lightDir);
  lightDir = norm3(lightDir);
  ray.dir = lightDir;
  ray.tmax = ldWorld;
  box_test(ray, lp.worldSpaceBounds, t00, t11);
  clip_planes(lp, ray, t00, t11);
  ray.tmax = t11;
  track<true>(c, ray, np, Tr, xf, rng, tt);
  if (trOut) *trOut = Tr;
  const float I = __fdiv_rn(Tr, ld * ld) * lp.lights[which].intensity;
  return mk3(I, I, I);
}

template <int INTEGRATOR>
EXA_D float4 sample_nested(PathCtx &c, int px, int py, int pixelID, int s, int height, int numLights, float *tHit,
                           float *trv)
{
  const exa_launch_params &lp = c.lp;
  Rng rng;
  rng.init((uint32_t)pixelID, (uint32_t)lp.accumID, lp.ext.frameID, (uint32_t)s);
  const float tb = __fdiv_rn((float)py, (float)height);
  const float4 bg = make_float4((1.f - tb) * 1.f + tb * 0.5f, (1.f - tb) * 1.f + tb * 0.7f, (1.f - tb) * 1.f + tb * 1.f, 1.f);
  const float rx = rng.next();
  const float ry = rng.next();
  const float sx = (float)px + rx, sy = (float)py + ry;
  V3 dir = add3(add3(mk3(lp.camera.dir_00), smul(sx, mk3(lp.camera.dir_du))), smul(sy, mk3(lp.camera.dir_dv)));
  dir = norm3(dir);
  if (fabsf(dir.x) < 1e-5f) dir.x = 1e-5f;
  if (fabsf(dir.y) < 1e-5f) dir.y = 1e-5f;
  if (fabsf(dir.z) < 1e-5f) dir.z = 1e-5f;
  RayS ray;
  ray.org = mk3(lp.camera.org);
  ray.dir = dir;
  ray.tmin = 0.f;
  ray.tmax = 1e10f;
  float t0 = 1e30f, t1 = -1e30f, tt;
  if (INTEGRATOR == EXA_PATH_TRACING_INTEGRATOR) {
    V3 throughput = mk3(1.f, 1.f, 1.f), Ld = mk3(0.f, 0.f, 0.f);
    unsigned bounce = 0;
    const unsigned maxB = (unsigned)lp.ext.maxBounces;
    if (box_test(ray, lp.worldSpaceBounds, t0, t1)) {
      clip_planes(lp, ray, t0, t1);
      ray.org = add3(ray.org, muls(ray.dir, t0));
      t1 -= t0;
      while (true) {
        float Tr;
        V3 pos;
        float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);
        ray.tmax = t1;
        const int ct = track<false>(c, ray, pos, Tr, xf, rng, tt);
        if (bounce == 0 && ct == SCATTERING && tHit) *tHit = tt;
        if (ct == BOUNDARY) break;
        if (bounce++ >= maxB) {
          throughput = mk3(0.f, 0.f, 0.f);
          break;
        }
        const V3 albedo = lp.ext.albedo < 0.f ? mk3(xf.x, xf.y, xf.z) : mk3(lp.ext.albedo, lp.ext.albedo, lp.ext.albedo);
        throughput = mul3(throughput, albedo);
        const float P = rmax3(throughput);
        if (P < 0.2f) {
          if (rng.next() > P) {
            throughput = mk3(0.f, 0.f, 0.f);
            break;
          }
          throughput = div3(throughput, mk3(P, P, P));
        }
        throughput = add3(throughput, mk3(0.f, 0.f, 0.f));
        if (numLights > 0)
          Ld = add3(Ld, mul3(throughput, light_nested(c, pos, rng, numLights, bounce == 1 ? trv : nullptr)));
        const V3 wo = mk3(-ray.dir.x, -ray.dir.y, -ray.dir.z);
        const V3 sd = hg_sample(wo, lp.ext.hgG, rng);
        ray.org = pos;
        ray.dir = sd;
        box_test(ray, lp.worldSpaceBounds, t0, t1);
        clip_planes(lp, ray, t0, t1);
      }
    }
    if (numLights == 0) Ld = mk3(1.f, 1.f, 1.f);
    const V3 L = mul3(Ld, throughput);
    return bounce ? make_float4(L.x, L.y, L.z, 1.f) : bg;
  } else {
    V3 throughput = mk3(1.f, 1.f, 1.f);
    if (!box_test(ray, lp.worldSpaceBounds, t0, t1)) return bg;
    clip_planes(lp, ray, t0, t1);
    ray.org = add3(ray.org, muls(ray.dir, t0));
    t1 -= t0;
    ray.tmax = t1;
    float Tr;
    V3 pos;
    float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);
    const int ct = track<false>(c, ray, pos, Tr, xf, rng, tt);
    if (ct == SCATTERING && tHit) *tHit = tt;
    if (ct == BOUNDARY) return bg;
    const V3 albedo = lp.ext.albedo < 0.f ? mk3(xf.x, xf.y, xf.z) : mk3(lp.ext.albedo, lp.ext.albedo, lp.ext.albedo);
    if (numLights > 0) throughput = mul3(throughput, mul3(albedo, light_nested(c, pos, rng, numLights, trv)));
    else throughput = mul3(throughput, albedo);
    return make_float4(throughput.x, throughput.y, throughput.z, 1.f);
  }
}

// S1: one thread per pixel, the spp loop inside (renderFrame_Impl as is)
template <int INTEGRATOR>
__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_render_pixel(const __grid_constant__ AccelView A,
                                                                             const __grid_constant__ exa_launch_params lp,
                                                                             int width, int height)
{
  const int tilesX = (width + 15) / 16;
  const int px = (blockIdx.x % tilesX) * 16 + (threadIdx.x & 15);
  const int py = (blockIdx.x / tilesX) * 8 + (threadIdx.x >> 4);
  PathCtx c = make_ctx(A, lp);
  if (px < width && py < height) {
    const int pixelID = px + width * py;
    const int numLights = num_lights(lp);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float tHit = -1.f, trv = -1.f;
    for (int s = 0; s < lp.render.spp; ++s) {
      const float4 col = sample_nested<INTEGRATOR>(c, px, py, pixelID, s, height, numLights, s == 0 ? &tHit : nullptr,
                                                   s == 0 ? &trv : nullptr);
      acc.x += col.x; acc.y += col.y; acc.z += col.z; acc.w += col.w;
      cnt_add(c, CNT_PATHS);
    }
    if (lp.accumID > 0 && lp.accumBuffer) {
      const float4 o = reinterpret_cast<const float4 *>(lp.accumBuffer)[pixelID];
      acc.x += o.x; acc.y += o.y; acc.z += o.z; acc.w += o.w;
    }
    if (lp.accumBuffer) reinterpret_cast<float4 *>(lp.accumBuffer)[pixelID] = acc;
    const float inv = __fdiv_rn(1.f, (float)(lp.accumID + 1));
    acc.x *= inv; acc.y *= inv; acc.z *= inv; acc.w *= inv;
    const float is = __fdiv_rn(1.f, (float)lp.render.spp);
    const uint32_t rgba = make_8bit(acc.x * is) | (make_8bit(acc.y * is) << 8) | (make_8bit(acc.z * is) << 16) |
                          (make_8bit(acc.w * is) << 24);
    if (lp.fbPointer) lp.fbPointer[pixelID] = rgba;
    if (lp.ext.traceT) lp.ext.traceT[pixelID] = tHit;
    if (lp.ext.traceTr) lp.ext.traceTr[pixelID] = trv;
  }
  flush_counters(c, lp);
}

// rayMarchingIntegrate + integrateDVR (deviceCode.cu:348-398, 1213-1260)
// for one camera sample: front-to-back compositing of TF samples at
// spacing lp.render.dt from a jittered first sample (firstSampleT,
// deviceCode.cu:104-112), early exit at opacity 0.99, over the background.
// The shading normal is g / |g + 1e-4| with the gradient g left at 0 (its
// computation is commented out in the reference), so lights add cd * 0.
// Clip planes and surface meshes are not part of this path.
constexpr long long kMarchCap = 1ll << 24;  // samples per ray

// steps: the march's sample positions (the heat map's work measure)
EXA_D float4 raymarch_sample(PathCtx &c, int px, int py, int pixelID, int s, int width, int height, int numLights,
                             unsigned &steps)
{
  const exa_launch_params &lp = c.lp;
  Rng rng;
  rng.init((uint32_t)pixelID, (uint32_t)lp.accumID, lp.ext.frameID, (uint32_t)s);
  const float tb = __fdiv_rn((float)py, (float)height);
  const float4 bg = make_float4((1.f - tb) * 1.f + tb * 0.5f, (1.f - tb) * 1.f + tb * 0.7f, (1.f - tb) * 1.f + tb * 1.f, 1.f);
  const float rx = rng.next();
  const float ry = rng.next();
  const V3 dir = camera_dir(lp, px, py, rx, ry, width, height);
  steps = 0;
  RayS ray;
  ray.org = mk3(lp.camera.org);
  ray.dir = dir;
  ray.tmin = 0.f;
  ray.tmax = 1e10f;
  float4 color = bg;
  float t0 = 1e30f, t1 = -1e30f;
  if (box_test(ray, lp.worldSpaceBounds, t0, t1)) {
    clip_planes(lp, ray, t0, t1);
    if (lp.meshBVH) {
      // a surface ends the march and shades the background behind the
      // volume with a headlight (deviceCode.cu:1243-1251)
      const MeshHit h = trace_mesh(*reinterpret_cast<const MeshView *>(lp.meshBVH), ray.org, ray.dir, ray.tmax);
      if (h.primID >= 0) {
        t1 = fmin_t(t1, h.t);
        const float cs = fmaxf(0.f, dot3(mk3(-ray.dir.x, -ray.dir.y, -ray.dir.z), h.Ng));
        color = make_float4(cs, cs, cs, cs);
      }
    }
    const float ils = rng.next();
    const V3 org = xfm_point(lp.voxelSpaceTransform, ray.org);
    const V3 vd = norm3(xfm_vector(lp.voxelSpaceTransform, ray.dir));
    const float dt = lp.render.dt;
    const float numSegsf = floorf(__fdiv_rn(t0 - dt * ils, dt));
    float t = dt * (ils + numSegsf);
    if (t < t0) t += dt;
    const V3 g = mk3(0.f, 0.f, 0.f);
    const V3 N = muls(g, __fdiv_rn(1.f, len3(add3(g, mk3(1e-4f, 1e-4f, 1e-4f)))));
    const bool cull = lp.ext.cullTransparentPrims != 0;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (long long k = 0; t <= t1; t += dt, ++k) {
      if (k >= kMarchCap) {
        c.err |= EXA_DEVERR_TRACK_CAP;
        break;
      }
      ++steps;
      const V3 pos = add3(org, muls(vd, t));
      const exa_sample smp = sample_field(c.A, pos, cull, c.err);
      if (smp.primID < 0) continue;
      const float4 xf = lookup_tf(lp, smp.value);
      const V3 cd = mk3(xf.x, xf.y, xf.z);
      V3 shaded = smul(.1f, cd);
      if (numLights == 0) shaded = cd;
      for (int l = 0; l < numLights; ++l) {
        const V3 lv = sub3(mk3(lp.lights[l].pos), pos);
        const V3 L = norm3(lv);
        const float ld = len3(lv);
        shaded = add3(shaded, muls(cd, __fdiv_rn(.9f * dot3(N, L), ld * ld) * lp.lights[l].intensity));
      }
      const float a = (1.f - acc.w) * xf.w;
      acc.x += a * shaded.x;
      acc.y += a * shaded.y;
      acc.z += a * shaded.z;
      acc.w += a * 1.f;
      if (acc.w >= 0.99f) break;
    }
    // over(A, B) = A + (1 - A.w) B  (deviceCode.cu:151-154)
    const float r = 1.f - acc.w;
    color = make_float4(acc.x + r * color.x, acc.y + r * color.y, acc.z + r * color.z, acc.w + r * color.w);
  }
  return color;
}

// ray marching: one thread per camera sample (pixel-major), colours to
// scratch, resolved by k_resolve
__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_render_march(const __grid_constant__ AccelView A,
                                                                             const __grid_constant__ exa_launch_params lp,
                                                                             int width, int height, float4 *colors)
{
  const int spp = lp.render.spp;
  const int tilesX = (width + 15) / 16;
  const unsigned job = blockIdx.x * 128u + threadIdx.x;
  const unsigned pj = job / (unsigned)spp;
  const int s = (int)(job - pj * (unsigned)spp);
  const int tile = (int)(pj >> 7), within = (int)(pj & 127);
  const int px = (tile % tilesX) * 16 + (within & 15);
  const int py = (tile / tilesX) * 8 + (within >> 4);
  PathCtx c = make_ctx(A, lp);
  if (px < width && py < height) {
    const int pixelID = px + width * py;
    unsigned steps;
    colors[(size_t)pixelID * spp + s] = raymarch_sample(c, px, py, pixelID, s, width, height, num_lights(lp), steps);
    if (lp.render.heatMapEnabled && lp.ext.heatCounts) atomicAdd(lp.ext.heatCounts + pixelID, steps);
    cnt_add(c, CNT_PATHS);
    if (s == 0) {
      if (lp.ext.traceT) lp.ext.traceT[pixelID] = -1.f;
      if (lp.ext.traceTr) lp.ext.traceTr[pixelID] = -1.f;
    }
  }
  flush_counters(c, lp);
}

// S2: one thread per camera sample (pixel-major), colours to scratch
template <int INTEGRATOR>
__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_render_sample(const __grid_constant__ AccelView A,
                                                                              const __grid_constant__ exa_launch_params lp,
                                                                              int width, int height, float4 *colors)
{
  const int spp = lp.render.spp;
  const int tilesX = (width + 15) / 16;
  const unsigned job = blockIdx.x * 128u + threadIdx.x;
  const unsigned pj = job / (unsigned)spp;
  const int s = (int)(job - pj * (unsigned)spp);
  const int tile = (int)(pj >> 7), within = (int)(pj & 127);
  const int px = (tile % tilesX) * 16 + (within & 15);
  const int py = (tile / tilesX) * 8 + (within >> 4);
  PathCtx c = make_ctx(A, lp);
  if (px < width && py < height) {
    const int pixelID = px + width * py;
    float tHit = -1.f, trv = -1.f;
    const float4 col = sample_nested<INTEGRATOR>(c, px, py, pixelID, s, height, num_lights(lp), &tHit, &trv);
    colors[(size_t)pixelID * spp + s] = col;
    cnt_add(c, CNT_PATHS);
    if (s == 0) {
      if (lp.ext.traceT) lp.ext.traceT[pixelID] = tHit;
      if (lp.ext.traceTr) lp.ext.traceTr[pixelID] = trv;
    }
  }
  flush_counters(c, lp);
}

// renderFrame_Impl (deviceCode.cu:1283-1344) after the spp loop: sum the
// pixel's samples in order, progressive accumulation, RGBA8 output
// temperature_to_rgb / hue_to_rgb (deviceCode.cu:155-170)
EXA_D V3 heat_map(float t)
{
  const float K = 4.0f / 6.0f;
  const float hue = K - K * t;
  const float v = .5f + 0.5f * t;
  const float s = __saturatef(hue) * 6.0f;
  const float r = __saturatef(fabsf(s - 3.f) - 1.0f);
  const float g = __saturatef(2.0f - fabsf(s - 2.0f));
  const float b = __saturatef(2.0f - fabsf(s - 4.0f));
  return mk3(v * r, v * g, v * b);
}

__global__ void k_resolve(const __grid_constant__ exa_launch_params lp, int width, int height,
                          const float4 *__restrict__ colors, int pixelBegin = 0, int pixelEnd = -1)
{
  const int pixelID = pixelBegin + blockIdx.x * blockDim.x + threadIdx.x;
  if (pixelID >= (pixelEnd < 0 ? width * height : pixelEnd)) return;
  const int spp = lp.render.spp;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 *cp = colors + (size_t)pixelID * spp;
  for (int s = 0; s < spp; ++s) {
    const float4 col = __ldg(cp + s);
    acc.x += col.x; acc.y += col.y; acc.z += col.z; acc.w += col.w;
  }
  if (lp.render.heatMapEnabled && lp.ext.heatCounts) {
    // the heat map over the pixel's samples (deviceCode.cu:1323-1327): the
    // pixel's work (DDA cells of its walks; march positions of the ray
    // marcher) in place of the reference's clock cycles
    const float t = (float)lp.ext.heatCounts[pixelID] * __fdiv_rn(lp.render.heatMapScale, (float)spp);
    const V3 h = heat_map(t);
    acc.x = h.x + (1.f - .5f) * acc.x;
    acc.y = h.y + (1.f - .5f) * acc.y;
    acc.z = h.z + (1.f - .5f) * acc.z;
    acc.w = .5f + (1.f - .5f) * acc.w;
  }
  if (lp.accumID > 0 && lp.accumBuffer) {
    const float4 o = reinterpret_cast<const float4 *>(lp.accumBuffer)[pixelID];
    acc.x += o.x; acc.y += o.y; acc.z += o.z; acc.w += o.w;
  }
  if (lp.accumBuffer) reinterpret_cast<float4 *>(lp.accumBuffer)[pixelID] = acc;
  const float inv = __fdiv_rn(1.f, (float)(lp.accumID + 1));
  acc.x *= inv; acc.y *= inv; acc.z *= inv; acc.w *= inv;
  if (lp.subImage.selecting) {
    // the selection window's border, inverted (deviceCode.cu:1337-1342)
    const int px = pixelID % width, py = pixelID / width;
    const int lx = min(max((int)(lp.subImage.selection.lower.x * (float)width), 0), width - 1);
    const int ly = min(max((int)(lp.subImage.selection.lower.y * (float)height), 0), height - 1);
    const int hx = min(max((int)(lp.subImage.selection.upper.x * (float)width), 0), width - 1);
    const int hy = min(max((int)(lp.subImage.selection.upper.y * (float)height), 0), height - 1);
    if (((px == lx || px == hx) && py >= ly && py <= hy) || ((py == ly || py == hy) && px >= lx && px <= hx)) {
      acc.x = 1.f - acc.x; acc.y = 1.f - acc.y; acc.z = 1.f - acc.z; acc.w = 1.f - acc.w;
    }
  }
  const float is = __fdiv_rn(1.f, (float)spp);
  const uint32_t rgba = make_8bit(acc.x * is) | (make_8bit(acc.y * is) << 8) | (make_8bit(acc.z * is) << 16) |
                        (make_8bit(acc.w * is) << 24);
  if (lp.fbPointer) lp.fbPointer[pixelID] = rgba;
}

// ------------------------------------------------------------------------
// Wavefront form: path records in queue buffers (walk state as
// structure-of-arrays, so a warp's loads and stores coalesce).  A
// walk kernel advances each queued walk by at most K tracking steps and
// compacts the records into a continue queue and an event queue with
// warp-aggregated appends (ballot, popc, one atomic per warp, shuffle of the
// base); an event kernel applies the integrator step that follows a walk
// (sampleLight, Russian roulette, HG scatter, sample end) and queues the next
// walk; a camera kernel refills the free capacity with new camera samples.
// Each path runs the same operations in the same order as in the nested
// form, so the result is bit-identical; only the interleaving of paths
// differs.
// record = path part (AoS: record i at words [i * kPathStride, +kPathWords))
// + walk part (SoA: word k of record i at (kPathStride + k) * cap + i); the
// walk kernel reads and writes only walk parts, and an ended walk leaves a
// short event record that points at its path part.
constexpr int kPathWords = 28;
constexpr int kPathStride = 28;  // path words padded to whole 16-byte vectors
constexpr int kPathFrameWord = 24;  // light kind | frame << 1
static_assert(kPathWords <= kPathStride && kPathStride % 4 == 0, "path part: whole uint4 vectors");
constexpr int kWalkWords = 35;
constexpr int kLaneWords = kPathStride + kWalkWords;
static_assert(kLaneWords == kWfLaneWords, "record size");

// round control of a frame on the device (after the queue counters): the
// jobs issued so far and in all, the round's carried walks and new camera
// jobs, whether its walk kernel may park, whether another round is needed
struct WfFrameCtl {
  unsigned long long issued, total;
  unsigned nIn, nNew, rounds, peak, park, more, error, pad;
};
static_assert(4 * sizeof(unsigned) + sizeof(WfFrameCtl) <= kWfCounterWords * sizeof(unsigned), "counter words");

struct WfQueues {
  uint32_t *in, *out, *ev;  // record buffers (kLaneWords * cap words each)
  unsigned *cnt;            // [0] in, [1] out, [2] ev, [3] walk fetch cursor
  unsigned cap;
  int park;                 // walk kernel may park unfinished walks in out
  const WfFrameCtl *ctl;    // non-null: camera jobs and parking from here
};

// a warp whose input is used up parks its unfinished walks in the next
// round's input once fewer than this many of its lanes are still walking,
// instead of stepping the round's longest walks with the other lanes idle
// preferred shared-memory carveout of the walk kernels in percent (-1: the
// driver's choice).  Measured on the medium workload: 4 %: 160 M paths/s
// (fewer resident blocks), 8 %: 247 M, 12 %: 247 M, 16 %: 243 M, 25 % and
// the driver's choice: 243 M, 100 %: 203 M; with the later walk kernel
// 6 %: 175.6 M, 10 %: 287.3 M, 16 %: 284.5 M.
#ifndef EXA_WALK_CARVEOUT
#define EXA_WALK_CARVEOUT 10
#endif

#ifndef EXA_WF_PARK_LANES
#define EXA_WF_PARK_LANES 28
#endif

#define W(v) b[(size_t)(k++) * cap + i] = (v)
#define WF(v) W(__float_as_uint(v))
// record words are read once: streaming loads keep them from displacing the
// field and table lines in L1 (1.3 % faster frames than __ldg)
#define R() __ldcs(b + (size_t)(k++) * cap + i)
#define RF() __uint_as_float(R())

// path part: AoS, kPathStride words per record (16-byte aligned), so that
// the integrator step, which reads records in an order unrelated to their
// slots, touches 4 sectors per record instead of one per word
EXA_D void wf_store_path(const Lane &L, uint32_t *b, unsigned cap, unsigned i)
{
  (void)cap;
  uint4 *p = reinterpret_cast<uint4 *>(b + (size_t)i * kPathStride);
  const auto f = [](float v) { return __float_as_uint(v); };
  p[0] = make_uint4((uint32_t)L.pixelID, (uint32_t)L.s, f(L.ray.org.x), f(L.ray.org.y));
  p[1] = make_uint4(f(L.ray.org.z), f(L.ray.dir.x), f(L.ray.dir.y), f(L.ray.dir.z));
  p[2] = make_uint4(f(L.ray.tmax), f(L.throughput.x), f(L.throughput.y), f(L.throughput.z));
  p[3] = make_uint4(f(L.Ld.x), f(L.Ld.y), f(L.Ld.z), f(L.pos.x));
  p[4] = make_uint4(f(L.pos.y), f(L.pos.z), f(L.albedo.x), f(L.albedo.y));
  p[5] = make_uint4(f(L.albedo.z), L.bounce, f(L.lightDen), f(L.lightI));
  p[6] = make_uint4((L.lightDirectional ? 1u : 0u) | ((uint32_t)L.frame << 1), (uint32_t)L.meshPrim, f(L.meshT),
                    f(L.shadowMesh));
}

EXA_D void wf_load_path(Lane &L, const uint32_t *__restrict__ b, unsigned cap, unsigned i, int width)
{
  (void)cap;
  const uint4 *p = reinterpret_cast<const uint4 *>(b + (size_t)i * kPathStride);
  const uint4 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3), q4 = __ldg(p + 4),
              q5 = __ldg(p + 5), q6 = __ldg(p + 6);
  const auto f = [](uint32_t v) { return __uint_as_float(v); };
  L.pixelID = (int)q0.x; L.s = (int)q0.y;
  if (width > 0) {  // (a batch's frame width is known only after the frame index)
    L.py = (int)((unsigned)L.pixelID / (unsigned)width);
    L.px = L.pixelID - L.py * width;
  }
  L.ray.org = mk3(f(q0.z), f(q0.w), f(q1.x));
  L.ray.dir = mk3(f(q1.y), f(q1.z), f(q1.w));
  L.ray.tmax = f(q2.x); L.ray.tmin = 0.f;
  L.throughput = mk3(f(q2.y), f(q2.z), f(q2.w));
  L.Ld = mk3(f(q3.x), f(q3.y), f(q3.z));
  L.pos = mk3(f(q3.w), f(q4.x), f(q4.y));
  L.albedo = mk3(f(q4.z), f(q4.w), f(q5.x));
  L.bounce = q5.y; L.lightDen = f(q5.z); L.lightI = f(q5.w);
  L.lightDirectional = (q6.x & 1u) != 0u;
  L.frame = (int)(q6.x >> 1);
  L.meshPrim = (int)q6.y;
  L.meshT = f(q6.z);
  L.shadowMesh = f(q6.w);
}

// shadow flag, RNG and the walk
// A walk that has not taken a step yet (walk_begin's state) is stored
// "fresh": flags, RNG, ray and DDA state (the first 21 of the 35 words); the
// loader sets the rest to walk_begin's values.  (Storing only the ray and
// re-running dda_init in the walk kernel saves more traffic but costs the
// latency-bound walk kernel more than it saves.)
constexpr uint32_t kWalkFresh = 0x80000000u;

EXA_D void wf_store_walk(const Lane &L, uint32_t *b, unsigned cap, unsigned i, bool fresh = false)
{
  unsigned k = kPathStride;
  const Walk &w = L.w;
  W((uint32_t)L.shadow | ((uint32_t)w.needCell << 1) | ((uint32_t)w.type << 2) | (fresh ? kWalkFresh : 0u));
  W((uint32_t)L.rng.state); W((uint32_t)(L.rng.state >> 32)); ++k;  // word 3: unused
  WF(w.org.x); WF(w.org.y); WF(w.org.z); WF(w.dir.x); WF(w.dir.y); WF(w.dir.z);
  WF(w.dda.tnext.x); WF(w.dda.tnext.y); WF(w.dda.tnext.z); WF(w.dda.dist.x); WF(w.dda.dist.y); WF(w.dda.dist.z);
  W((uint32_t)w.dda.cell.x); W((uint32_t)w.dda.cell.y); W((uint32_t)w.dda.cell.z); WF(w.t); WF(w.dda.tmax);
  if (fresh) return;
  k += 7;  // words 21-27 unused: a parked walk's last sample and classification are not read again
  WF(w.t); WF(w.t1); WF(w.maj); WF(w.Tr);
  W((uint32_t)w.primID); W((uint32_t)w.steps); W((uint32_t)w.ncells);
}

EXA_D void wf_load_walk(Lane &L, const uint32_t *__restrict__ b, unsigned cap, unsigned i,
                        const exa_grid_traversable &G)
{
  unsigned k = kPathStride;
  Walk &w = L.w;
  const uint32_t flags = R();
  L.shadow = flags & 1u;
  w.needCell = (flags >> 1) & 1u;
  w.type = (int)((flags & ~kWalkFresh) >> 2);
  const uint32_t lo = R(), hi = R();
  L.rng.state = ((uint64_t)hi << 32) | lo;
  ++k;
  w.org.x = RF(); w.org.y = RF(); w.org.z = RF(); w.dir.x = RF(); w.dir.y = RF(); w.dir.z = RF();
  w.dda.tnext.x = RF(); w.dda.tnext.y = RF(); w.dda.tnext.z = RF();
  w.dda.dist.x = RF(); w.dda.dist.y = RF(); w.dda.dist.z = RF();
  w.dda.cell.x = (int)R(); w.dda.cell.y = (int)R(); w.dda.cell.z = (int)R();
  w.t = RF(); w.dda.tmax = RF();
  w.dda.t0 = w.t;
  // step / stop follow from the ray direction as in dda_init
  w.dda.step.x = w.dir.x > 0.f ? 1 : -1; w.dda.step.y = w.dir.y > 0.f ? 1 : -1; w.dda.step.z = w.dir.z > 0.f ? 1 : -1;
  w.dda.stop.x = w.dir.x > 0.f ? G.dims.x : -1; w.dda.stop.y = w.dir.y > 0.f ? G.dims.y : -1;
  w.dda.stop.z = w.dir.z > 0.f ? G.dims.z : -1;
  if (flags & kWalkFresh) {
    w.pos = mk3(0.f, 0.f, 0.f);
    w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
    w.t1 = w.maj = 0.f;
    w.Tr = 1.f;
    w.primID = -1;
    w.steps = 0;
    w.ncells = 0;
    return;
  }
  w.pos = mk3(0.f, 0.f, 0.f);
  w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
  k += 7;
  w.t = RF(); w.t1 = RF(); w.maj = RF(); w.Tr = RF();
  w.primID = (int)R(); w.steps = (int)R(); w.ncells = (int)R();
}

// event record of a walk that ended: the fields the integrator step reads,
// and the slot of the walk's path part, which stays in the round's input
// queue (that buffer is rewritten only in the next round)
constexpr int kEventWords = 14;
static_assert(kEventWords <= kWfLaneWords, "an event record fits a queue slot");

// event records are read once, by the next events kernel: streaming stores
// (for the walk and path records, which the next walk kernel reads, plain
// stores measured faster)
// (withXf false: the frame's events never read the classification -- a
// fixed albedo and no Teaser shading -- and those four words are skipped)
EXA_D void wf_store_event(const Lane &L, uint32_t *b, unsigned cap, unsigned i, unsigned src, bool withXf = true)
{
#undef W
#define W(v) __stcs(b + (size_t)(k++) * cap + i, (uint32_t)(v))
  unsigned k = 0;
  const Walk &w = L.w;
  W((uint32_t)L.shadow | ((uint32_t)w.type << 2) | ((uint32_t)w.ncells << 8));
  W(src);
  W((uint32_t)L.rng.state); W((uint32_t)(L.rng.state >> 32)); ++k;  // word 4: unused
  WF(w.t); WF(w.Tr);
  WF(w.pos.x); WF(w.pos.y); WF(w.pos.z);
  if (withXf) { WF(w.xf.x); WF(w.xf.y); WF(w.xf.z); WF(w.xf.w); }
#undef W
#define W(v) b[(size_t)(k++) * cap + i] = (v)
}

// whether a frame's events read the classification of the walk's last sample
EXA_D bool events_read_xf(const exa_launch_params &lp)
{
  return lp.ext.albedo < 0.f || lp.shadeMode == EXA_SHADE_MODE_TEASER;
}

// returns the slot of the path part
EXA_D unsigned wf_load_event(Lane &L, const uint32_t *__restrict__ b, unsigned cap, unsigned i, bool withXf = true)
{
  unsigned k = 0;
  Walk &w = L.w;
  const uint32_t flags = R();
  L.shadow = flags & 1u;
  w.type = (int)((flags >> 2) & 0x3fu);
  w.ncells = (int)(flags >> 8);
  const unsigned src = R();
  const uint32_t lo = R(), hi = R();
  L.rng.state = ((uint64_t)hi << 32) | lo;
  ++k;
  w.t = RF(); w.Tr = RF();
  w.pos.x = RF(); w.pos.y = RF(); w.pos.z = RF();
  if (withXf) {
    w.xf.x = RF(); w.xf.y = RF(); w.xf.z = RF(); w.xf.w = RF();
  } else {
    w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  return src;
}

#undef W
#undef WF
#undef R
#undef RF

// a lane that has just begun a walk
EXA_D void wf_store(const Lane &L, uint32_t *b, unsigned cap, unsigned i)
{
  wf_store_path(L, b, cap, i);
  wf_store_walk(L, b, cap, i, true);
}

EXA_D void wf_load(Lane &L, const uint32_t *__restrict__ b, unsigned cap, unsigned i, int width,
                   const exa_grid_traversable &G)
{
  wf_load_path(L, b, cap, i, width);
  wf_load_walk(L, b, cap, i, G);
}

EXA_D void wf_copy_path(const uint32_t *__restrict__ src, unsigned i, uint32_t *dst, unsigned j, unsigned cap)
{
  (void)cap;
  const uint4 *a = reinterpret_cast<const uint4 *>(src + (size_t)i * kPathStride);
  uint4 *d = reinterpret_cast<uint4 *>(dst + (size_t)j * kPathStride);
#pragma unroll
  for (int k = 0; k < kPathStride / 4; ++k) d[k] = __ldg(a + k);
}

// warp-aggregated append: returns this lane's slot (valid where pred)
EXA_D unsigned warp_append(unsigned *counter, bool pred)
{
  const unsigned mask = __activemask();
  const unsigned ballot = __ballot_sync(mask, pred);
  const unsigned lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  unsigned base = 0;
  if ((int)lane == leader && ballot) base = atomicAdd(counter, (unsigned)__popc(ballot));
  base = __shfl_sync(mask, base, leader);
  return base + __popc(ballot & ((1u << lane) - 1u));
}


// camera: samples [first, first + n) of the frame's job order; those that
// start a walk are appended to the input queue
template <int INTEGRATOR>
__global__ void __launch_bounds__(128) k_wf_camera(const __grid_constant__ AccelView A,
                                                   const __grid_constant__ exa_launch_params lp, int width, int height,
                                                   float4 *colors, WfQueues Q, unsigned first, unsigned n)
{
  if (Q.ctl) {
    first = (unsigned)Q.ctl->issued;
    n = Q.ctl->nNew;
  }
  PathCtx c = make_ctx(A, lp);
  Machine<INTEGRATOR> M{c, lp, width, height, num_lights(lp), (unsigned)lp.ext.maxBounces, colors};
  const int spp = lp.render.spp;
  const int tilesX = (width + 15) / 16;
  for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const unsigned i = base + threadIdx.x;
    Lane L;
    bool tracking = false;
    if (i < n) {
      const unsigned job = first + i;
      const unsigned pj = job / (unsigned)spp;
      L.s = (int)(job - pj * (unsigned)spp);
      const int tile = (int)(pj >> 7), within = (int)(pj & 127);
      L.px = (tile % tilesX) * 16 + (within & 15);
      L.py = (tile / tilesX) * 8 + (within >> 4);
      if (L.px < width && L.py < height) {
        M.begin_sample(L);
        tracking = L.phase == PH_TRACK;
      }
    }
    const unsigned slot = warp_append(&Q.cnt[0], tracking);
    if (tracking) wf_store(L, Q.in, Q.cap, slot);
  }
  flush_counters(c, lp);
}

// walks: persistent warps; every lane takes one tracking step per
// iteration, and a lane whose walk ended appends the record to the event
// queue and fetches the next walk (one atomic per warp).  Lanes stay busy
// until the input is used up; then, in a large round, a warp left with few
// walking lanes parks their walks in the next round's input and exits.
template <bool TEASER>
__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_wf_walk(const __grid_constant__ AccelView A,
                                                                        const __grid_constant__ exa_launch_params lp,
                                                                        WfQueues Q)
{
  PathCtx c = make_ctx(A, lp);
  const unsigned n = Q.cnt[0];
  const bool park = Q.ctl ? Q.ctl->park != 0u : Q.park != 0;
  const unsigned lane = threadIdx.x & 31;
  Lane L;
  bool active = false, exhausted = false;
  unsigned src = 0;
  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !active);
    if (need && !exhausted) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if ((int)lane == leader) base = atomicAdd(&Q.cnt[3], (unsigned)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (unsigned)__popc(need) >= n) exhausted = true;
      if (!active) {
        const unsigned idx = base + __popc(need & ((1u << lane) - 1u));
        if (idx < n) {
          wf_load_walk(L, Q.in, Q.cap, idx, lp.majorantGrid);
          active = true;
          src = idx;
          cnt_add(c, CNT_WALKS);
        }
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act) break;
    if (exhausted && park && __popc(act) < EXA_WF_PARK_LANES) {
      // the walk record holds the complete walk state (position in the DDA,
      // RNG counter, cached gridlet), so a parked walk resumes exactly
      const unsigned slot = warp_append(&Q.cnt[1], active);
      if (active) {
        wf_store_walk(L, Q.out, Q.cap, slot);
        wf_copy_path(Q.in, src, Q.out, slot, Q.cap);
      }
      break;
    }
    // a step's sample position and classification, and the kind of end, are
    // read only by the event of a walk that ends in the same iteration:
    // cleared here, they hold no registers across iterations
    L.w.pos = mk3(0.f, 0.f, 0.f);
    L.w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
    L.w.type = BOUNDARY;
    const bool ended = active && !walk_iteration<TEASER>(L.w, c, L.rng, L.shadow);
    const unsigned slot = warp_append(&Q.cnt[2], ended);
    if (ended) {
      wf_store_event(L, Q.ev, Q.cap, slot, src, events_read_xf(lp));
      active = false;
    }
  }
  flush_counters(c, lp);
}

// walks with the learned field: k_wf_walk with the sample of a step taken
// from the surrogate in macrocells marked for it (one warp-wide evaluation
// per iteration for all lanes that need one) and from the exact sampler
// elsewhere; lp.maxOpacities holds the widened majorants.  Dynamic shared
// memory: the network and the warps' scratch (kSurWalkSmem bytes).
constexpr size_t kSurWalkSmem = sizeof(SurWeightsSmem) + 4 * sizeof(SurWarpSmem);
// (learned walk on the medium field: 12 lanes 105.1 M paths/s, 20: 103.2 M,
// 26: 92.1 M, 32: 72.3 M; the trained fields of the runs differ slightly)
#ifndef EXA_SUR_BATCH
#define EXA_SUR_BATCH 20
#endif

__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_wf_walk_sur(const __grid_constant__ AccelView A,
                                                                            const __grid_constant__ exa_launch_params lp,
                                                                            WfQueues Q,
                                                                            const __grid_constant__ SurrogateView S)
{
  extern __shared__ __align__(16) unsigned char surSm[];
  SurWeightsSmem &W = *reinterpret_cast<SurWeightsSmem *>(surSm);
  SurWarpSmem &ws = reinterpret_cast<SurWarpSmem *>(surSm + sizeof(SurWeightsSmem))[threadIdx.x >> 5];
  sur_load_weights(W, S);
  __syncthreads();
  PathCtx c = make_ctx(A, lp);
  const exa_grid_traversable &G = lp.majorantGrid;
  const unsigned n = Q.cnt[0];
  const bool park = Q.ctl ? Q.ctl->park != 0u : Q.park != 0;
  const unsigned lane = threadIdx.x & 31;
  Lane L;
  bool active = false, exhausted = false, pending = false;
  unsigned src = 0;
  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !active);
    if (need && !exhausted) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if ((int)lane == leader) base = atomicAdd(&Q.cnt[3], (unsigned)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (unsigned)__popc(need) >= n) exhausted = true;
      if (!active) {
        const unsigned idx = base + __popc(need & ((1u << lane) - 1u));
        if (idx < n) {
          wf_load_walk(L, Q.in, Q.cap, idx, lp.majorantGrid);
          active = true;
          src = idx;
          cnt_add(c, CNT_WALKS);
        }
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act) break;
    // a lane waiting for a learned sample is never parked: its free flight
    // is done, its sample not yet taken
    if (exhausted && park && __popc(act) < EXA_WF_PARK_LANES && !__any_sync(0xffffffffu, pending)) {
      const unsigned slot = warp_append(&Q.cnt[1], active);
      if (active) {
        wf_store_walk(L, Q.out, Q.cap, slot);
        wf_copy_path(Q.in, src, Q.out, slot, Q.cap);
      }
      break;
    }
    bool ended = false;
    // the classification as in k_wf_walk; the position stays for a lane
    // that waits for its learned sample
    L.w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
    L.w.type = BOUNDARY;
    if (active && !pending) {
      int st, a = 0;
      do {
        st = walk_advance(L.w, c, L.rng);
      } while (st == WALK_ON && ++a < EXA_WF_ADVANCE_MAX);
      if (st == WALK_END) {
        ended = true;
      } else if (st == WALK_SAMPLE) {
        const int leafID = (L.w.dda.cell.z * G.dims.y + L.w.dda.cell.y) * G.dims.x + L.w.dda.cell.x;
        if (__ldg(S.mcMode + leafID) != 0) {
          pending = true;
        } else {
          const exa_sample s = walk_sample_exact(L.w, c);
          ended = !walk_collide(L.w, c, L.rng, L.shadow, s);
        }
      }
    }
    // the network runs for a batch of waiting lanes: at least
    // EXA_SUR_BATCH of them, or every lane still walking
    const unsigned pm = __ballot_sync(0xffffffffu, pending);
    const unsigned am = __ballot_sync(0xffffffffu, active && !ended);
    if (pm && (__popc(pm) >= EXA_SUR_BATCH || pm == am || exhausted)) {
      const float y = sur_eval_warp(S, W, ws, L.w.pos, pending);
      if (pending) {
        exa_sample s;
        s.primID = -2;
        s.cellID = -1;
        s.value = S.vmin + y * S.vrange;
        cnt_add(c, CNT_SURR);
        pending = false;
        ended = !walk_collide(L.w, c, L.rng, L.shadow, s, false, true);
      }
    }
    ended = active && ended;
    const unsigned slot = warp_append(&Q.cnt[2], ended);
    if (ended) {
      wf_store_event(L, Q.ev, Q.cap, slot, src, events_read_xf(lp));
      active = false;
    }
  }
  flush_counters(c, lp);
}

// walk ends: the integrator step after a primary or shadow walk
template <int INTEGRATOR>
__global__ void __launch_bounds__(128) k_wf_events(const __grid_constant__ AccelView A,
                                                   const __grid_constant__ exa_launch_params lp, int width, int height,
                                                   float4 *colors, WfQueues Q)
{
  PathCtx c = make_ctx(A, lp);
  Machine<INTEGRATOR> M{c, lp, width, height, num_lights(lp), (unsigned)lp.ext.maxBounces, colors};
  const unsigned n = Q.cnt[2];
  for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const unsigned i = base + threadIdx.x;
    Lane L;
    bool tracking = false;
    if (i < n) {
      wf_load_path(L, Q.in, Q.cap, wf_load_event(L, Q.ev, Q.cap, i, events_read_xf(lp)), width);
      if (lp.render.heatMapEnabled && lp.ext.heatCounts) atomicAdd(lp.ext.heatCounts + L.pixelID, (unsigned)L.w.ncells);
      L.phase = PH_TRACK;
      if (L.shadow) M.shadow_done(L);
      else M.primary_done(L);
      tracking = L.phase == PH_TRACK;
    }
    const unsigned slot = warp_append(&Q.cnt[1], tracking);
    if (tracking) wf_store(L, Q.out, Q.cap, slot);
  }
  flush_counters(c, lp);
}

// end of a round on the device: the output queue becomes the next input,
// the camera jobs and the parking of the next round are decided, and
// whether another round is needed; a round cap stops a frame that makes no
// progress (EXA_DEVERR_WATCHDOG).  Rounds after the last one find nothing
// to do.
__global__ void k_wf_round_end(unsigned *cnt, WfFrameCtl *ctl, unsigned cap, unsigned parkWalks,
                               uint32_t *deviceErrors)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const unsigned nOut = cnt[1], nEv = cnt[2];
  if (ctl->nIn + ctl->nNew > 0u) ctl->rounds += 1u;
  ctl->issued += ctl->nNew;
  if (nEv > ctl->peak) ctl->peak = nEv;
  cnt[0] = nOut;
  cnt[1] = cnt[2] = cnt[3] = 0u;
  const unsigned long long left = ctl->total - ctl->issued;
  const unsigned nNew = (unsigned)(left < (unsigned long long)(cap - nOut) ? left : (unsigned long long)(cap - nOut));
  ctl->nIn = nOut;
  ctl->nNew = nNew;
  // parking pays while a round has several walks per walk-kernel thread;
  // small rounds (the end of the frame) run their walks to completion
  ctl->park = (unsigned long long)nOut + nNew >= (unsigned long long)parkWalks ? 1u : 0u;
  unsigned more = (nOut > 0u || ctl->issued < ctl->total) ? 1u : 0u;
  if (more && ctl->rounds >= kBatchRoundCap) {
    more = 0u;
    ctl->error = 1u;
    if (deviceErrors) atomicOr(deviceErrors, EXA_DEVERR_WATCHDOG);
  }
  ctl->more = more;
}

// host loop of the wavefront renderer: rounds are launched in groups and
// driven by the device (k_wf_round_end); the host reads the round control
// once per group to see whether the frame is done
void renderWavefront(const AccelView &A, const exa_launch_params &lp, int width, int height, float4 *colors,
                     uint32_t *bufs, unsigned cap, unsigned *counters, cudaStream_t s, WfStats *stats,
                     const SurrogateView *sur)
{
  const bool pt = lp.integrator == EXA_PATH_TRACING_INTEGRATOR;
  int dev = 0, sms = 152;
  cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  // the jobs of the frame (16 x 8-pixel tiles, row-major, spp each), or of
  // its band of rows [rowBegin, rowEnd): the band's tile rows
  const int rowBegin = lp.ext.rowEnd > 0 ? lp.ext.rowBegin : 0, rowEnd = lp.ext.rowEnd > 0 ? lp.ext.rowEnd : height;
  const unsigned long long jobsPerTileRow = (unsigned long long)((width + 15) / 16) * 128ull * lp.render.spp;
  const unsigned long long total = jobsPerTileRow * (unsigned long long)((rowEnd + 7) / 8);
  // path parts are read as 16-byte vectors: every queue must start 16-byte
  // aligned (capacities are multiples of the 128-job tile)
  if (cap % 4 != 0) throw Error(EXA_ERR_INVALID, "queue capacity must be a multiple of 4");
  const size_t words = (size_t)kLaneWords * cap;
  uint32_t *buf[3] = {bufs, bufs + words, bufs + 2 * words};
  const unsigned grid = (unsigned)sms * 16;
  int perSM = 4;
  if (sur) {
    cudaCheck(cudaFuncSetAttribute(k_wf_walk_sur, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSurWalkSmem),
              "walk smem");
    cudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_wf_walk_sur, 128, kSurWalkSmem), "occupancy");
  } else {
#if EXA_WALK_CARVEOUT >= 0
    // the walk kernel needs little shared memory; the rest of the unified
    // L1 / shared array serves as L1 for its field and table loads
    for (auto *k : {k_wf_walk<false>, k_wf_walk<true>})
      cudaCheck(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, EXA_WALK_CARVEOUT),
                "walk carveout");
#endif
    cudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_wf_walk<false>, 128, 0), "occupancy");
  }
  const unsigned walkGrid = (unsigned)sms * (unsigned)(perSM > 0 ? perSM : 1);
  // the first round's control: no carried walks, the first camera jobs
  WfFrameCtl *ctl = reinterpret_cast<WfFrameCtl *>(counters + 4);
  WfFrameCtl c0{};
  c0.issued = jobsPerTileRow * (unsigned long long)(rowBegin / 8);
  c0.total = total;
  c0.nNew = (unsigned)std::min<unsigned long long>(cap, total - c0.issued);
  const unsigned parkWalks = 4u * walkGrid * 128u;
  c0.park = c0.nNew >= parkWalks ? 1u : 0u;
  c0.more = 1u;
  cudaCheck(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned), s), "reset queues");
  cudaCheck(cudaMemcpyAsync(ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice, s), "frame control");
  // per-kernel-class timing on this stream (camera, walk, events), four
  // events per round from a pool kept across calls
  thread_local std::map<int, std::vector<cudaEvent_t>> pools;
  std::vector<cudaEvent_t> &pool = pools[dev];
  const bool timing = stats != nullptr;
  int inIdx = 0, outIdx = 1, launched = 0;
  unsigned kernels = 0;
  WfFrameCtl h{};
  // no camera launch once every job is issued: after the first round of a
  // frame whose jobs all fit it, or once a group's check has seen it
  bool issuedAll = false;
  const bool oneIssue = c0.nNew == total - c0.issued;
  // rounds per host check: few at first (small frames end in a few rounds),
  // more once the frame proves long
  for (int group = 0; launched < (int)kBatchRoundCap; ++group) {
    const int rounds = group == 0 ? 4 : 8;
    for (int r = 0; r < rounds; ++r, ++launched) {
      if (timing)
        while (pool.size() < 4 * (size_t)(launched + 1)) {
          cudaEvent_t e;
          cudaCheck(cudaEventCreate(&e), "cudaEventCreate");
          pool.push_back(e);
        }
      cudaEvent_t *ev = timing ? &pool[4 * (size_t)launched] : nullptr;
      WfQueues Q{buf[inIdx], buf[outIdx], buf[2], counters, cap, 0, ctl};
      if (timing) cudaCheck(cudaEventRecord(ev[0], s), "event");
      if (launched == 0 || (!oneIssue && !issuedAll)) {
        // (the first round's job count is known here; later rounds read theirs)
        const unsigned g = launched == 0 ? std::max(1u, std::min<unsigned>(grid, (c0.nNew + 127) / 128)) : grid;
        if (pt) k_wf_camera<EXA_PATH_TRACING_INTEGRATOR><<<g, 128, 0, s>>>(A, lp, width, height, colors, Q, 0u, 0u);
        else k_wf_camera<EXA_DIRECT_LIGHT_INTEGRATOR><<<g, 128, 0, s>>>(A, lp, width, height, colors, Q, 0u, 0u);
        ++kernels;
      }
      if (timing) cudaCheck(cudaEventRecord(ev[1], s), "event");
      if (sur) k_wf_walk_sur<<<walkGrid, 128, kSurWalkSmem, s>>>(A, lp, Q, *sur);
      else if (lp.shadeMode == EXA_SHADE_MODE_TEASER) k_wf_walk<true><<<walkGrid, 128, 0, s>>>(A, lp, Q);
      else k_wf_walk<false><<<walkGrid, 128, 0, s>>>(A, lp, Q);
      if (timing) cudaCheck(cudaEventRecord(ev[2], s), "event");
      if (pt) k_wf_events<EXA_PATH_TRACING_INTEGRATOR><<<grid, 128, 0, s>>>(A, lp, width, height, colors, Q);
      else k_wf_events<EXA_DIRECT_LIGHT_INTEGRATOR><<<grid, 128, 0, s>>>(A, lp, width, height, colors, Q);
      if (timing) cudaCheck(cudaEventRecord(ev[3], s), "event");
      k_wf_round_end<<<1, 32, 0, s>>>(counters, ctl, cap, parkWalks, lp.ext.deviceErrors);
      kernels += 3;  // walk, events, round end
      cudaCheck(cudaGetLastError(), "wavefront round");
      std::swap(inIdx, outIdx);
    }
    cudaCheck(cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s), "read frame control");
    cudaCheck(cudaStreamSynchronize(s), "wavefront rounds");
    if (!h.more) break;
    issuedAll = h.issued >= h.total;
  }
  if (stats) {
    for (int r = 0; r < launched; ++r) {
      float ms[3] = {0.f, 0.f, 0.f};
      for (int k = 0; k < 3; ++k)
        cudaCheck(cudaEventElapsedTime(&ms[k], pool[4 * (size_t)r + k], pool[4 * (size_t)r + k + 1]), "event time");
      stats->cameraMs += ms[0];
      stats->walkMs += ms[1];
      stats->eventMs += ms[2];
    }
    stats->rounds = h.rounds;
    stats->walkLaunches = (unsigned)launched;
    stats->kernelLaunches = kernels + 1;  // and the resolve
    stats->peakQueue = std::max(stats->peakQueue, h.peak);
  }
  const int pb = rowBegin * width, pe = rowEnd * width;
  k_resolve<<<(unsigned)(((long long)(pe - pb) + 255) / 256), 256, 0, s>>>(lp, width, height, colors, pb, pe);
  cudaCheck(cudaGetLastError(), "k_resolve");
}

// ======================================================== batched frames
// Many frames -- each with its own camera, size, spp, transfer function and
// output buffers, given as a full launch-parameter block per frame -- share
// one set of queues.  The batch's jobs are the frames' jobs one after the
// other, a path record carries its frame, and every kernel reads the
// frame's parameters (and the point-location view of the frame's transfer
// function, whose primitive opacities decide culling) where the
// single-frame kernels read the launch's, so each frame's result is the one
// exa_render gives for it.  Rounds are driven from the device: after each
// round an update kernel moves the queue counters and decides whether
// another round runs, which lets the whole batch be one CUDA graph (a
// conditional while node around the round).

EXA_D int batch_frame_of(const WfFrame *F, int n, unsigned long long v, bool pixels)
{
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const unsigned long long b = pixels ? F[mid].pixelBase : F[mid].jobBase;
    if (b <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct WfQueuesB {
  uint32_t *buf[2];  // input / output queues, swapped every round (WfCtl.flip)
  uint32_t *ev;
  unsigned *cnt;     // [0] in, [1] out, [2] ev, [3] walk fetch cursor
  unsigned cap;
};

__global__ void k_wfb_init(WfCtl *ctl, unsigned *cnt)
{
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    ctl->issued = 0;
    ctl->nIn = 0;
    ctl->nNew = 0;
    ctl->rounds = 0;
    ctl->peak = 0;
    ctl->flip = 0;
    ctl->more = 1;
    ctl->error = 0;
    for (int k = 0; k < 4; ++k) cnt[k] = 0;
  }
}

template <int INTEGRATOR>
__global__ void __launch_bounds__(128) k_wfb_camera(const __grid_constant__ AccelView A,
                                                    const __grid_constant__ exa_launch_params lp0, WfBatchView B,
                                                    WfQueuesB Q, WfCtl *ctl, float4 *colors)
{
  PathCtx c = make_ctx(A, lp0);
  const unsigned long long first = ctl->issued;
  const unsigned nIn = ctl->nIn;
  const unsigned long long left = B.totalJobs - first;
  const unsigned n = (unsigned)(left < (unsigned long long)(Q.cap - nIn) ? left : (unsigned long long)(Q.cap - nIn));
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->nNew = n;
  uint32_t *in = Q.buf[ctl->flip];
  const int tw = B.tileW, th = 128 / B.tileW;
  for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const unsigned i = base + threadIdx.x;
    Lane L;
    bool tracking = false;
    if (i < n) {
      const unsigned long long job = first + i;
      const int f = batch_frame_of(B.frames, B.numFrames, job, false);
      const WfFrame F = B.frames[f];
      const exa_launch_params &flp = B.lps[f];
      PathCtx cf{A, flp, 0u, c.counting};
      Machine<INTEGRATOR> M{cf, flp, F.width, F.height, num_lights(flp), (unsigned)flp.ext.maxBounces,
                            colors + F.sampleBase};
      const unsigned long long local = job - F.jobBase;
      const unsigned spp = (unsigned)flp.render.spp;
      const unsigned long long pj = local / spp;
      L.s = (int)(local - pj * spp);
      L.frame = f;
      const int tilesX = (F.width + tw - 1) / tw;
      const int tile = (int)(pj >> 7), within = (int)(pj & 127);
      L.px = (tile % tilesX) * tw + within % tw;
      L.py = (tile / tilesX) * th + within / tw;
      if (L.px < F.width && L.py < F.height) {
        M.begin_sample(L);
        tracking = L.phase == PH_TRACK;
      }
      c.err |= cf.err;
    }
    const unsigned slot = warp_append(&Q.cnt[0], tracking);
    if (tracking) wf_store(L, in, Q.cap, slot);
  }
  flush_counters(c, lp0);
}

__global__ void __launch_bounds__(128, EXA_RENDER_MIN_BLOCKS) k_wfb_walk(const __grid_constant__ AccelView A,
                                                                         const __grid_constant__ exa_launch_params lp0,
                                                                         WfBatchView B, WfQueuesB Q, const WfCtl *ctl)
{
  PathCtx c = make_ctx(A, lp0);
  const unsigned n = Q.cnt[0];
  const int flip = ctl->flip;
  const uint32_t *in = Q.buf[flip];
  uint32_t *out = Q.buf[flip ^ 1];
  const bool park = n >= 4u * gridDim.x * blockDim.x;
  const unsigned lane = threadIdx.x & 31;
  Lane L;
  const exa_launch_params *flp = &lp0;
  const AccelView *fa = &A;  // the frame's transfer function decides which primitives are culled
  bool active = false, exhausted = false;
  unsigned src = 0;
  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, !active);
    if (need && !exhausted) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if ((int)lane == leader) base = atomicAdd(&Q.cnt[3], (unsigned)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (base + (unsigned)__popc(need) >= n) exhausted = true;
      if (!active) {
        const unsigned idx = base + __popc(need & ((1u << lane) - 1u));
        if (idx < n) {
          wf_load_walk(L, in, Q.cap, idx, lp0.majorantGrid);
          // the frame index sits in the path part of the record
          L.frame = (int)(__ldg(in + (size_t)idx * kPathStride + kPathFrameWord) >> 1);
          flp = B.lps + L.frame;
          fa = B.accels + B.frames[L.frame].tf;
          active = true;
          src = idx;
          cnt_add(c, CNT_WALKS);
        }
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act) break;
    if (exhausted && park && __popc(act) < EXA_WF_PARK_LANES) {
      const unsigned slot = warp_append(&Q.cnt[1], active);
      if (active) {
        wf_store_walk(L, out, Q.cap, slot);
        wf_copy_path(in, src, out, slot, Q.cap);
      }
      break;
    }
    bool ended = false;
    L.w.pos = mk3(0.f, 0.f, 0.f);  // as in k_wf_walk
    L.w.xf = make_float4(0.f, 0.f, 0.f, 0.f);
    L.w.type = BOUNDARY;
    if (active) {
      PathCtx cf{*fa, *flp, 0u, c.counting};
      ended = !walk_iteration(L.w, cf, L.rng, L.shadow);
      c.err |= cf.err;
    }
    const unsigned slot = warp_append(&Q.cnt[2], ended);
    if (ended) {
      wf_store_event(L, Q.ev, Q.cap, slot, src);
      active = false;
    }
  }
  flush_counters(c, lp0);
}

template <int INTEGRATOR>
__global__ void __launch_bounds__(128) k_wfb_events(const __grid_constant__ AccelView A,
                                                    const __grid_constant__ exa_launch_params lp0, WfBatchView B,
                                                    WfQueuesB Q, const WfCtl *ctl, float4 *colors)
{
  PathCtx c = make_ctx(A, lp0);
  const unsigned n = Q.cnt[2];
  uint32_t *out = Q.buf[ctl->flip ^ 1];
  for (unsigned base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const unsigned i = base + threadIdx.x;
    Lane L;
    bool tracking = false;
    if (i < n) {
      wf_load_path(L, Q.buf[ctl->flip], Q.cap, wf_load_event(L, Q.ev, Q.cap, i), 0);
      const WfFrame F = B.frames[L.frame];
      L.py = (int)((unsigned)L.pixelID / (unsigned)F.width);
      L.px = L.pixelID - L.py * F.width;
      const exa_launch_params &flp = B.lps[L.frame];
      PathCtx cf{A, flp, 0u, c.counting};
      Machine<INTEGRATOR> M{cf, flp, F.width, F.height, num_lights(flp), (unsigned)flp.ext.maxBounces,
                            colors + F.sampleBase};
      L.phase = PH_TRACK;
      if (L.shadow) M.shadow_done(L);
      else M.primary_done(L);
      tracking = L.phase == PH_TRACK;
      c.err |= cf.err;
    }
    const unsigned slot = warp_append(&Q.cnt[1], tracking);
    if (tracking) wf_store(L, out, Q.cap, slot);
  }
  flush_counters(c, lp0);
}

// end of a round: the output queue becomes the next input; another round
// runs while walks remain or camera jobs are left.  A round cap stops a
// batch that makes no progress (error bit EXA_DEVERR_WATCHDOG).
__global__ void k_wfb_update(WfBatchView B, WfQueuesB Q, WfCtl *ctl, uint32_t *deviceErrors,
                             cudaGraphConditionalHandle handle, int useHandle)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const unsigned nOut = Q.cnt[1], nEv = Q.cnt[2];
  ctl->issued += ctl->nNew;
  ctl->nIn = nOut;
  ctl->rounds += 1;
  if (nEv > ctl->peak) ctl->peak = nEv;
  ctl->flip ^= 1;
  Q.cnt[0] = nOut;
  Q.cnt[1] = 0;
  Q.cnt[2] = 0;
  Q.cnt[3] = 0;
  unsigned more = (nOut > 0 || ctl->issued < B.totalJobs) ? 1u : 0u;
  if (more && ctl->rounds >= kBatchRoundCap) {
    more = 0;
    ctl->error = 1;
    if (deviceErrors) atomicOr(deviceErrors, EXA_DEVERR_WATCHDOG);
  }
  ctl->more = more;
  if (useHandle) cudaGraphSetConditional(handle, more);
}

// resolve of every frame's pixels (k_resolve per frame)
__global__ void k_wfb_resolve(WfBatchView B, const float4 *__restrict__ colors)
{
  const unsigned long long p = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (p >= B.totalPixels) return;
  const int f = batch_frame_of(B.frames, B.numFrames, p, true);
  const WfFrame F = B.frames[f];
  const exa_launch_params &lp = B.lps[f];
  const int pixelID = (int)(p - F.pixelBase);
  const int spp = lp.render.spp;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 *cp = colors + F.sampleBase + (size_t)pixelID * spp;
  for (int s = 0; s < spp; ++s) {
    const float4 col = __ldg(cp + s);
    acc.x += col.x; acc.y += col.y; acc.z += col.z; acc.w += col.w;
  }
  if (lp.accumID > 0 && lp.accumBuffer) {
    const float4 o = reinterpret_cast<const float4 *>(lp.accumBuffer)[pixelID];
    acc.x += o.x; acc.y += o.y; acc.z += o.z; acc.w += o.w;
  }
  if (lp.accumBuffer) reinterpret_cast<float4 *>(lp.accumBuffer)[pixelID] = acc;
  const float inv = __fdiv_rn(1.f, (float)(lp.accumID + 1));
  acc.x *= inv; acc.y *= inv; acc.z *= inv; acc.w *= inv;
  const float is = __fdiv_rn(1.f, (float)spp);
  const uint32_t rgba = make_8bit(acc.x * is) | (make_8bit(acc.y * is) << 8) | (make_8bit(acc.z * is) << 16) |
                        (make_8bit(acc.w * is) << 24);
  if (lp.fbPointer) lp.fbPointer[pixelID] = rgba;
}

namespace {
// the kernels of one round (camera, walk, events, update) on stream s
void batchRound(const AccelView &A, const exa_launch_params &lp0, const WfBatchView &B, const WfQueuesB &Q,
                WfCtl *ctl, float4 *colors, uint32_t *deviceErrors, cudaGraphConditionalHandle handle,
                int useHandle, unsigned grid, unsigned walkGrid, cudaStream_t s)
{
  const bool pt = lp0.integrator == EXA_PATH_TRACING_INTEGRATOR;
  if (pt) k_wfb_camera<EXA_PATH_TRACING_INTEGRATOR><<<grid, 128, 0, s>>>(A, lp0, B, Q, ctl, colors);
  else k_wfb_camera<EXA_DIRECT_LIGHT_INTEGRATOR><<<grid, 128, 0, s>>>(A, lp0, B, Q, ctl, colors);
  k_wfb_walk<<<walkGrid, 128, 0, s>>>(A, lp0, B, Q, ctl);
  if (pt) k_wfb_events<EXA_PATH_TRACING_INTEGRATOR><<<grid, 128, 0, s>>>(A, lp0, B, Q, ctl, colors);
  else k_wfb_events<EXA_DIRECT_LIGHT_INTEGRATOR><<<grid, 128, 0, s>>>(A, lp0, B, Q, ctl, colors);
  k_wfb_update<<<1, 32, 0, s>>>(B, Q, ctl, deviceErrors, handle, useHandle);
}
}  // namespace

void BatchGraph::release()
{
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
}

BatchGraph::~BatchGraph()
{
  release();
  if (captureStream) cudaStreamDestroy(captureStream);
}

void renderWavefrontBatch(const AccelView &A, const exa_launch_params &lp0, const WfBatchView &B, uint32_t *bufs,
                          unsigned cap, unsigned *counters, WfCtl *ctl, float4 *colors, uint32_t *deviceErrors,
                          bool useGraph, BatchGraph *cache, cudaStream_t s, WfStats *stats)
{
  int dev = 0, sms = 152;
  cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  int perSM = 4;
#if EXA_WALK_CARVEOUT >= 0
  cudaCheck(cudaFuncSetAttribute(k_wfb_walk, cudaFuncAttributePreferredSharedMemoryCarveout, EXA_WALK_CARVEOUT),
            "walk carveout");
#endif
  cudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_wfb_walk, 128, 0), "occupancy");
  const unsigned walkGrid = (unsigned)sms * (unsigned)(perSM > 0 ? perSM : 1);
  const unsigned grid = (unsigned)sms * 16;
  // path parts are read as 16-byte vectors: every queue must start 16-byte
  // aligned (capacities are multiples of the 128-job tile)
  if (cap % 4 != 0) throw Error(EXA_ERR_INVALID, "queue capacity must be a multiple of 4");
  const size_t words = (size_t)kLaneWords * cap;
  WfQueuesB Q{{bufs, bufs + words}, bufs + 2 * words, counters, cap};
  const unsigned long long totalPixels = B.totalPixels;
  cudaEvent_t e0, e1;
  cudaCheck(cudaEventCreate(&e0), "cudaEventCreate");
  cudaCheck(cudaEventCreate(&e1), "cudaEventCreate");
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
  } evGuard{e0, e1};
  cudaCheck(cudaEventRecord(e0, s), "event");
  if (useGraph) {
    // the graph bakes in every pointer and the batch's shape; the frame
    // tables it reads are device memory, so new cameras need no rebuild
    BatchKey key;
    std::memset(&key, 0, sizeof(key));  // padding too: keys are compared bytewise
    key.accel = A.gridlets;
    key.accels = B.accels;
    key.lps = B.lps;
    key.frames = B.frames;
    key.numFrames = B.numFrames;
    key.tileW = B.tileW;
    key.totalJobs = B.totalJobs;
    key.totalPixels = B.totalPixels;
    key.bufs = bufs;
    key.cap = cap;
    key.counters = counters;
    key.ctl = ctl;
    key.colors = colors;
    key.errors = deviceErrors;
    key.integrator = lp0.integrator;
    key.grid = grid;
    key.walkGrid = walkGrid;
    if (!cache->exec || std::memcmp(&cache->key, &key, sizeof(key)) != 0) {
      cache->release();
      // captured on the cache's own stream (the legacy default stream, which
      // a caller may render on, cannot be captured); launched on s
      if (!cache->captureStream)
        cudaCheck(cudaStreamCreateWithFlags(&cache->captureStream, cudaStreamNonBlocking), "capture stream");
      cudaStream_t cs = cache->captureStream;
      // load every kernel of the graph before capturing (lazy module loading)
      cudaFuncAttributes fa;
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_init), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_camera<EXA_PATH_TRACING_INTEGRATOR>), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_camera<EXA_DIRECT_LIGHT_INTEGRATOR>), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_walk), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_events<EXA_PATH_TRACING_INTEGRATOR>), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_events<EXA_DIRECT_LIGHT_INTEGRATOR>), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_update), "load");
      cudaCheck(cudaFuncGetAttributes(&fa, k_wfb_resolve), "load");
      cudaCheck(cudaStreamSynchronize(s), "batch inputs");
      cudaGraph_t g;
      cudaCheck(cudaGraphCreate(&g, 0), "cudaGraphCreate");
      cache->graph = g;
      cudaGraphConditionalHandle handle;
      cudaCheck(cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault), "conditional handle");
      cudaCheck(cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                "capture");
      k_wfb_init<<<1, 1, 0, cs>>>(ctl, counters);
      cudaStreamCaptureStatus st;
      const cudaGraphNode_t *deps = nullptr;
      size_t ndeps = 0;
      cudaCheck(cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, nullptr, &ndeps), "capture info");
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t loop;
      cudaCheck(cudaGraphAddNode(&loop, g, deps, nullptr, ndeps, &cp), "conditional node");
      cudaCheck(cudaStreamUpdateCaptureDependencies(cs, &loop, nullptr, 1, cudaStreamSetCaptureDependencies),
                "capture dependencies");
      k_wfb_resolve<<<(unsigned)((totalPixels + 255) / 256), 256, 0, cs>>>(B, colors);
      cudaGraph_t captured = nullptr;
      cudaCheck(cudaStreamEndCapture(cs, &captured), "end capture");
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      cudaCheck(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                "capture body");
      batchRound(A, lp0, B, Q, ctl, colors, deviceErrors, handle, 1, grid, walkGrid, cs);
      cudaGraph_t bodyOut = nullptr;
      cudaCheck(cudaStreamEndCapture(cs, &bodyOut), "end capture body");
      cudaCheck(cudaGraphInstantiate(&cache->exec, g, 0), "cudaGraphInstantiate");
      cache->key = key;
    }
    cudaCheck(cudaGraphLaunch(cache->exec, s), "cudaGraphLaunch");
  } else {
    k_wfb_init<<<1, 1, 0, s>>>(ctl, counters);
    for (unsigned round = 0; round < kBatchRoundCap; ++round) {
      batchRound(A, lp0, B, Q, ctl, colors, deviceErrors, 0, 0, grid, walkGrid, s);
      cudaCheck(cudaGetLastError(), "batch round");
      unsigned more = 0;
      cudaCheck(cudaMemcpyAsync(&more, &ctl->more, sizeof(more), cudaMemcpyDeviceToHost, s), "read ctl");
      cudaCheck(cudaStreamSynchronize(s), "batch round");
      if (!more) break;
    }
    k_wfb_resolve<<<(unsigned)((totalPixels + 255) / 256), 256, 0, s>>>(B, colors);
  }
  cudaCheck(cudaGetLastError(), "batch");
  cudaCheck(cudaEventRecord(e1, s), "event");
  if (stats) {
    WfCtl h;
    cudaCheck(cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s), "read ctl");
    cudaCheck(cudaStreamSynchronize(s), "batch");
    float ms = 0.f;
    cudaCheck(cudaEventElapsedTime(&ms, e0, e1), "event time");
    stats->rounds = h.rounds;
    stats->peakQueue = h.peak;
    stats->walkLaunches = h.rounds;
    stats->cameraMs = 0.f;
    stats->walkMs = ms;  // whole batch (kernel classes are not timed apart inside a graph)
    stats->eventMs = 0.f;
  }
}

// EXA_RENDER_STRATEGY (the single-launch renderer): 1 thread per pixel,
// 2 thread per sample + resolve, 3 persistent state machine + resolve.
// EXA_WAVEFRONT 1: exa_render uses the wavefront renderer instead.
#ifndef EXA_RENDER_STRATEGY
#define EXA_RENDER_STRATEGY 2
#endif
#ifndef EXA_WAVEFRONT
#define EXA_WAVEFRONT 1
#endif

bool useWavefront() { return EXA_WAVEFRONT != 0; }

void launchRender(const AccelView &A, const exa_launch_params &lp, int width, int height, unsigned *jobCounter,
                  float4 *colors, cudaStream_t s)
{
  const bool pt = lp.integrator == EXA_PATH_TRACING_INTEGRATOR;
  const int tiles = ((width + 15) / 16) * ((height + 7) / 8);
  const long long jobs = (long long)tiles * 128 * lp.render.spp;
  if (lp.integrator == EXA_RAY_MARCHING_INTEGRATOR) {
    k_render_march<<<(unsigned)((jobs + 127) / 128), 128, 0, s>>>(A, lp, width, height, colors);
    cudaCheck(cudaGetLastError(), "k_render_march");
    k_resolve<<<(unsigned)(((long long)width * height + 255) / 256), 256, 0, s>>>(lp, width, height, colors);
    cudaCheck(cudaGetLastError(), "k_resolve");
    return;
  }
  if (EXA_RENDER_STRATEGY == 1) {
    if (pt) k_render_pixel<EXA_PATH_TRACING_INTEGRATOR><<<tiles, 128, 0, s>>>(A, lp, width, height);
    else k_render_pixel<EXA_DIRECT_LIGHT_INTEGRATOR><<<tiles, 128, 0, s>>>(A, lp, width, height);
    cudaCheck(cudaGetLastError(), "k_render_pixel");
    return;
  }
  if (EXA_RENDER_STRATEGY == 2) {
    const unsigned blocks = (unsigned)((jobs + 127) / 128);
    if (pt) k_render_sample<EXA_PATH_TRACING_INTEGRATOR><<<blocks, 128, 0, s>>>(A, lp, width, height, colors);
    else k_render_sample<EXA_DIRECT_LIGHT_INTEGRATOR><<<blocks, 128, 0, s>>>(A, lp, width, height, colors);
    cudaCheck(cudaGetLastError(), "k_render_sample");
  } else {
    int dev = 0, sms = 152, perSM = 4;
    cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
    cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    cudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                  &perSM, pt ? k_render<EXA_PATH_TRACING_INTEGRATOR> : k_render<EXA_DIRECT_LIGHT_INTEGRATOR>, 128, 0),
              "occupancy");
    long long blocks = (long long)sms * (perSM > 0 ? perSM : 1);
    if (blocks * 128 > jobs) blocks = (jobs + 127) / 128;
    cudaCheck(cudaMemsetAsync(jobCounter, 0, sizeof(unsigned), s), "reset job counter");
    if (pt)
      k_render<EXA_PATH_TRACING_INTEGRATOR><<<(unsigned)blocks, 128, 0, s>>>(A, lp, width, height, jobCounter, colors);
    else
      k_render<EXA_DIRECT_LIGHT_INTEGRATOR><<<(unsigned)blocks, 128, 0, s>>>(A, lp, width, height, jobCounter, colors);
    cudaCheck(cudaGetLastError(), "k_render");
  }
  k_resolve<<<(unsigned)(((long long)width * height + 255) / 256), 256, 0, s>>>(lp, width, height, colors);
  cudaCheck(cudaGetLastError(), "k_resolve");
}

// ------------------------------------------------------------ point query
__global__ void __launch_bounds__(256) k_sample_points(const __grid_constant__ AccelView A,
                                                       const exa_vec3f *__restrict__ pos, size_t n,
                                                       exa_sample *out, int cull, uint32_t *errors)
{
  uint32_t err = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const exa_vec3f p = pos[i];
    out[i] = sample_field(A, mk3(p.x, p.y, p.z), cull != 0, err);
  }
  if (err && errors) atomicOr(errors, err);
}

void launchSamplePoints(const AccelView &A, const exa_vec3f *pos, size_t n, exa_sample *out, int cull,
                        uint32_t *errors, cudaStream_t s)
{
  if (!n) return;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  size_t blocks = (n + 255) / 256;
  const size_t cap = (size_t)sms * 16;
  if (blocks > cap) blocks = cap;
  k_sample_points<<<(unsigned)blocks, 256, 0, s>>>(A, pos, n, out, cull, errors);
  cudaCheck(cudaGetLastError(), "k_sample_points");
}

} // namespace exa
