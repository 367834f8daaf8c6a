// exa_render.cu -- the hot path: field sampling (sample(),
// sampler/ExaStitchSampler.h:128-140) and the per-pixel integrators of
// deviceCode.cu: generateRay (:88-101), sampleInteraction with Woodcock
// and ratio tracking (:699-854) over the DDA majorant grid (DDA.h:26-113),
// sampleLight (:856-926), henyeyGreensteinSample (:965-985),
// pathTracingIntegrate (:991-1120), directLightingIntegrate (:1126-1207)
// and renderFrame_Impl (:1268-1345).
//
// One thread per pixel; pixels are assigned in 8x16 tiles so that a warp's
// rays start coherent.  The launch parameters and the accel view are kernel
// parameters (constant bank).
#include "exa_host.h"

namespace exa {

constexpr int kTrackCap = 1 << 22;  // delta / ratio tracking steps per macrocell

struct Counters {
  unsigned long long fieldSamples, gridletSamples, elemSamples, ddaCells;
};

struct RayS {
  V3 org, dir;
  float tmin, tmax;
};

enum { BOUNDARY = 0, SCATTERING = 1 };

// deviceCode.cu:320-341, buffer variant
EXA_D float4 lookup_tf(const exa_launch_params &lp, float f)
{
  const exa_range1f d = lp.transferFunc.domain;
  if (d.lower >= d.upper) return make_float4(0.f, 0.f, 0.f, 0.f);
  f -= d.lower;
  f /= (d.upper - d.lower);
  if (lp.transferFunc.numValues == 0) return make_float4(0.f, 0.f, 0.f, 0.f);
  f = fmax_t(0.f, fmin_t(1.f, f));
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
  d.t0 = fmax_t(tmin, 0.f);
  d.tmax = tmax;
}

// DDA.h:352-375: advance every axis tied with the closest crossing
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

struct PathCtx {
  const AccelView &A;
  const exa_launch_params &lp;
  uint32_t err;
  Counters cnt;
  bool counting;
};

// sampleInteraction (deviceCode.cu:699-854); SHADOW selects ratio tracking
template <bool SHADOW>
EXA_D int sample_interaction(PathCtx &c, RayS ray, V3 &posOut, float &TrOut, float4 &xf, Rng &rng, float *tHit)
{
  const exa_launch_params &lp = c.lp;
  ray.org = xfm_point(lp.voxelSpaceTransform, ray.org);
  ray.dir = xfm_vector(lp.voxelSpaceTransform, ray.dir);
  const float dt_scale = len3(ray.dir);
  ray.dir = norm3(ray.dir);
  ray.tmin = ray.tmin * dt_scale;
  ray.tmax = ray.tmax * dt_scale;
  int type = BOUNDARY;
  float Tr = 1.f;
  V3 pos = mk3(0.f, 0.f, 0.f);
  const float scale = lp.transferFunc.opacityScale;
  const bool cull = lp.ext.cullTransparentPrims != 0;
  const exa_grid_traversable &G = lp.majorantGrid;
  Dda dda;
  dda_init(dda, ray.org, ray.dir, ray.tmin, ray.tmax, G);
  const int cellCap = G.dims.x + G.dims.y + G.dims.z + 3;
  int ncells = 0;
  bool done = false;
  while (!done) {
    if (++ncells > cellCap) { c.err |= EXA_DEVERR_DDA_CAP; break; }
    const float t1 = fmin_t(rmin3(dda.tnext), dda.tmax);
    const int leafID = (dda.cell.z * G.dims.y + dda.cell.y) * G.dims.x + dda.cell.x;
    if (c.counting) c.cnt.ddaCells++;
    const float majorant = __ldg(lp.maxOpacities + leafID);
    float t = dda.t0;
    int primID = -1;
    int steps = 0;
    while (true) {
      if (majorant <= 0.f) break;
      if (++steps > kTrackCap) { c.err |= EXA_DEVERR_TRACK_CAP; done = true; break; }
      t -= __fdiv_rn(exa_log(1.f - rng.next()), majorant * scale);
      if (t >= t1) break;
      pos = add3(ray.org, muls(ray.dir, t));
      exa_sample s = test_sample(c.A, pos, primID);
      if (s.primID < 0) s = sample_field(c.A, pos, cull, c.err);
      if (c.counting) {
        c.cnt.fieldSamples++;
        if (s.primID >= 0) { if (s.cellID != -1) c.cnt.gridletSamples++; else c.cnt.elemSamples++; }
      }
      if (s.primID < 0) continue;
      if (s.cellID != -1) primID = s.primID;
      xf = classify(c.A, lp, s);
      const float sigmaT = xf.w;
      if (!SHADOW) {
        const float u = rng.next();
        if (sigmaT * scale >= u * majorant) {
          Tr = 0.f;
          type = SCATTERING;
          done = true;
          if (tHit) *tHit = t;
          break;
        }
      } else {
        Tr *= 1.f - __fdiv_rn(sigmaT * scale, majorant);
        if (Tr <= 0.f) { type = SCATTERING; done = true; break; }
      }
    }
    if (done) break;
    if (!dda_next(dda)) break;
  }
  posOut = xfm_point(lp.ext.voxelSpaceTransformInv, pos);
  TrOut = Tr;
  return type;
}

// sampleLight (deviceCode.cu:856-926); directional lights (extension) use
// lights[i].pos as the direction towards the light, no falloff
EXA_D V3 sample_light(PathCtx &c, V3 pos, Rng &rng, int numLights, float *trOut)
{
  const exa_launch_params &lp = c.lp;
  int which = (int)(rng.next() * (float)numLights);
  if (which == numLights) which = 0;
  RayS ray;
  float Tr, t00 = 1e30f, t11 = -1e30f;
  V3 np;
  float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);
  ray.org = pos;
  ray.tmin = 0.f;
  if (lp.ext.lightType[which] == EXA_LIGHT_DIRECTIONAL) {
    ray.dir = norm3(mk3(lp.lights[which].pos));
    ray.tmax = 1e30f;
    box_test(ray, lp.worldSpaceBounds, t00, t11);
    ray.tmax = t11;
    sample_interaction<true>(c, ray, np, Tr, xf, rng, nullptr);
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
  ray.tmax = t11;
  sample_interaction<true>(c, ray, np, Tr, xf, rng, nullptr);
  if (trOut) *trOut = Tr;
  const float I = __fdiv_rn(Tr, ld * ld) * lp.lights[which].intensity;
  return mk3(I, I, I);
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

// pathTracingIntegrate (deviceCode.cu:991-1120)
EXA_D float4 path_trace(PathCtx &c, RayS ray, Rng &rng, float4 bg, int numLights, float *tHit, float *trOut)
{
  const exa_launch_params &lp = c.lp;
  V3 throughput = mk3(1.f, 1.f, 1.f), Ld = mk3(0.f, 0.f, 0.f);
  unsigned bounce = 0;
  float t0 = 1e30f, t1 = -1e30f;
  const unsigned maxB = (unsigned)lp.ext.maxBounces;
  if (box_test(ray, lp.worldSpaceBounds, t0, t1)) {
    ray.org = add3(ray.org, muls(ray.dir, t0));
    t1 -= t0;
    while (true) {
      float Tr;
      V3 pos;
      float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);
      ray.tmax = t1;
      const int ct = sample_interaction<false>(c, ray, pos, Tr, xf, rng, bounce == 0 ? tHit : nullptr);
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
      if (numLights > 0) Ld = add3(Ld, mul3(throughput, sample_light(c, pos, rng, numLights, bounce == 1 ? trOut : nullptr)));
      const V3 wo = mk3(-ray.dir.x, -ray.dir.y, -ray.dir.z);
      const V3 sd = hg_sample(wo, lp.ext.hgG, rng);
      ray.org = pos;
      ray.dir = sd;
      box_test(ray, lp.worldSpaceBounds, t0, t1);
    }
  }
  if (numLights == 0) Ld = mk3(1.f, 1.f, 1.f);
  const V3 L = mul3(Ld, throughput);
  return bounce ? make_float4(L.x, L.y, L.z, 1.f) : bg;
}

// directLightingIntegrate (deviceCode.cu:1126-1207)
EXA_D float4 direct_light(PathCtx &c, RayS ray, Rng &rng, float4 bg, int numLights, float *tHit, float *trOut)
{
  const exa_launch_params &lp = c.lp;
  V3 throughput = mk3(1.f, 1.f, 1.f);
  float t0 = 1e30f, t1 = -1e30f;
  if (!box_test(ray, lp.worldSpaceBounds, t0, t1)) return bg;
  ray.org = add3(ray.org, muls(ray.dir, t0));
  t1 -= t0;
  ray.tmax = t1;
  float Tr;
  V3 pos;
  float4 xf = make_float4(0.f, 0.f, 0.f, 0.f);
  const int ct = sample_interaction<false>(c, ray, pos, Tr, xf, rng, tHit);
  if (ct == BOUNDARY) return bg;
  const V3 albedo = lp.ext.albedo < 0.f ? mk3(xf.x, xf.y, xf.z) : mk3(lp.ext.albedo, lp.ext.albedo, lp.ext.albedo);
  if (numLights > 0) throughput = mul3(throughput, mul3(albedo, sample_light(c, pos, rng, numLights, trOut)));
  else throughput = mul3(throughput, albedo);
  return make_float4(throughput.x, throughput.y, throughput.z, 1.f);
}

EXA_D uint32_t make_8bit(float f) { return (uint32_t)imin_t(255, imax_t(0, (int)(f * 256.f))); }

template <int INTEGRATOR>
__global__ void __launch_bounds__(128) k_render(const AccelView A, const exa_launch_params lp, int width, int height)
{
  // 8x16 tiles: block = 128 threads
  const int tilesX = (width + 15) / 16;
  const int tile = blockIdx.x;
  const int px = (tile % tilesX) * 16 + (threadIdx.x & 15);
  const int py = (tile / tilesX) * 8 + (threadIdx.x >> 4);
  const bool active = px < width && py < height;
  PathCtx c{A, lp, 0u, {0, 0, 0, 0}, lp.ext.stepCounters != nullptr};
  if (active) {
    const int pixelID = px + width * py;
    const float tb = __fdiv_rn((float)py, (float)height);
    const float4 bg = make_float4((1.f - tb) * 1.f + tb * 0.5f, (1.f - tb) * 1.f + tb * 0.7f, (1.f - tb) * 1.f + tb * 1.f, 1.f);
    const int numLights = num_lights(lp);
    Rng rng;
    rng.init((uint32_t)pixelID, (uint32_t)lp.accumID, lp.ext.frameID);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float tHit = -1.f, trv = -1.f;
    for (int s = 0; s < lp.render.spp; ++s) {
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
      float4 col;
      if (INTEGRATOR == EXA_PATH_TRACING_INTEGRATOR)
        col = path_trace(c, ray, rng, bg, numLights, s == 0 ? &tHit : nullptr, s == 0 ? &trv : nullptr);
      else
        col = direct_light(c, ray, rng, bg, numLights, s == 0 ? &tHit : nullptr, s == 0 ? &trv : nullptr);
      acc.x += col.x; acc.y += col.y; acc.z += col.z; acc.w += col.w;
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
  if (c.err && lp.ext.deviceErrors) atomicOr(lp.ext.deviceErrors, c.err);
  if (c.counting) {
    unsigned long long v[5] = {c.cnt.fieldSamples, c.cnt.gridletSamples, c.cnt.elemSamples, c.cnt.ddaCells,
                               active ? 1ull : 0ull};
    for (int k = 0; k < 5; ++k) {
      unsigned long long x = v[k];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) == 0 && x) atomicAdd(lp.ext.stepCounters + k, x);
    }
  }
}

void launchRender(const AccelView &A, const exa_launch_params &lp, int width, int height, cudaStream_t s)
{
  const int tiles = ((width + 15) / 16) * ((height + 7) / 8);
  if (lp.integrator == EXA_PATH_TRACING_INTEGRATOR)
    k_render<EXA_PATH_TRACING_INTEGRATOR><<<tiles, 128, 0, s>>>(A, lp, width, height);
  else
    k_render<EXA_DIRECT_LIGHT_INTEGRATOR><<<tiles, 128, 0, s>>>(A, lp, width, height);
  cudaCheck(cudaGetLastError(), "k_render");
}

// ------------------------------------------------------------ point query
__global__ void __launch_bounds__(256) k_sample_points(const AccelView A, const exa_vec3f *__restrict__ pos, size_t n,
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
