// exa_mesh.cuh -- surface meshes beside the volume: the reference traces
// triangle meshes with OptiX (MeshGeomCH, deviceCode.cu:295-318) to clip a
// volume segment at the first surface and shade that surface.  Here a
// triangle mesh is a LBVH over its triangles (the element BVH's build, with
// 3-vertex rows) and the closest hit is found by a stack walk.
//
// Closest hit: the smallest t in [0, tmax] over the triangles, the lowest
// triangle index among equal t (OptiX leaves the choice among equal hits
// unspecified).  Triangle test: Moeller and Trumbore 1997 ("Fast, minimum
// storage ray-triangle intersection"), no back-face culling.  Geometric
// normal: normalize(cross(b - a, c - a)) (MeshGeomCH).  Node boxes are
// widened by a relative 1e-5 in the slab test, and a box is pruned only
// when it starts 0.1 % beyond the closest hit so far, so that rounding in
// the slab test does not drop a triangle the triangle test accepts: the
// result is the brute-force closest hit over all triangles.
#pragma once

#include "exa_accel.cuh"

namespace exa {

struct MeshView {
  const float4 *vertices;  // x, y, z, unused
  const int32_t *indices;  // 8 per triangle: a, b, c, then -1 (the BVH's element rows)
  const BvhNode *nodes;
  int numTris;
};

struct MeshHit {
  int primID;  // -1: no hit
  float t;
  V3 Ng;
};

constexpr int kMeshStack = 96;

#ifdef __CUDACC__

EXA_D bool tri_intersect(V3 org, V3 dir, V3 a, V3 b, V3 c, float tmax, float &t)
{
  const V3 e1 = sub3(b, a), e2 = sub3(c, a);
  const V3 p = cross3(dir, e2);
  const float det = dot3(e1, p);
  if (!(det != 0.f)) return false;
  const float inv = 1.f / det;
  const V3 s = sub3(org, a);
  const float u = dot3(s, p) * inv;
  if (!(u >= 0.f && u <= 1.f)) return false;
  const V3 q = cross3(s, e1);
  const float v = dot3(dir, q) * inv;
  if (!(v >= 0.f && u + v <= 1.f)) return false;
  t = dot3(e2, q) * inv;
  return t >= 0.f && t <= tmax;
}


EXA_D V3 tri_vertex(const MeshView &M, int tri, int k)
{
  const float4 v = __ldg(M.vertices + __ldg(M.indices + (size_t)tri * 8 + k));
  return mk3(v.x, v.y, v.z);
}

// conservative slab test of a widened box: entry distance, or false
EXA_D bool mesh_box(const float *lo, const float *hi, V3 org, V3 dir, float tmax, float &tn)
{
  const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
  float t0 = 0.f, t1 = tmax;
  for (int a = 0; a < 3; ++a) {
    if (!(lo[a] <= hi[a])) return false;  // empty child slot
    const float eps = 1e-5f * fmaxf(1.f, fmaxf(fabsf(lo[a]), fabsf(hi[a])));
    const float l = lo[a] - eps, h = hi[a] + eps;
    if (d[a] == 0.f) {
      if (o[a] < l || o[a] > h) return false;
      continue;
    }
    const float inv = 1.f / d[a];
    const float ta = (l - o[a]) * inv, tb = (h - o[a]) * inv;
    t0 = fmaxf(t0, fminf(ta, tb));
    t1 = fminf(t1, fmaxf(ta, tb));
  }
  tn = t0;
  return t0 <= t1;
}

EXA_D MeshHit trace_mesh(const MeshView &M, V3 org, V3 dir, float tmax)
{
  MeshHit h;
  h.primID = -1;
  h.t = tmax;
  h.Ng = mk3(0.f, 0.f, 0.f);
  if (M.numTris <= 0) return h;
  float best = tmax;
  int bestID = -1;
  auto test = [&](int tri) {
    float t;
    if (tri_intersect(org, dir, tri_vertex(M, tri, 0), tri_vertex(M, tri, 1), tri_vertex(M, tri, 2), best, t) &&
        (t < best || (t == best && (bestID < 0 || tri < bestID)))) {
      best = t;
      bestID = tri;
    }
  };
  int stack[kMeshStack];
  int sp = 0, node = 0;
  for (int visits = 0; visits <= 2 * M.numTris + 2; ++visits) {
    const float4 *np = reinterpret_cast<const float4 *>(M.nodes + node);
    const float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3);
    const float lo0[3] = {q0.x, q0.y, q0.z}, hi0[3] = {q0.w, q1.x, q1.y};
    const float lo1[3] = {q1.z, q1.w, q2.x}, hi1[3] = {q2.y, q2.z, q2.w};
    const int c[2] = {__float_as_int(q3.x), __float_as_int(q3.y)};
    float tn0, tn1;
    const float reach = best + 1e-3f * fmaxf(1.f, best);
    const bool in[2] = {mesh_box(lo0, hi0, org, dir, reach, tn0), mesh_box(lo1, hi1, org, dir, reach, tn1)};
    int next = -1;
    for (int k = 0; k < 2; ++k) {
      if (!in[k]) continue;
      if (c[k] < 0) {
        test(~c[k]);
      } else if (next < 0) {
        next = c[k];
      } else if (sp < kMeshStack) {
        stack[sp++] = c[k];
      }
    }
    if (next < 0) {
      if (sp == 0) break;
      next = stack[--sp];
    }
    node = next;
  }
  if (bestID >= 0) {
    h.primID = bestID;
    h.t = best;
    const V3 a = tri_vertex(M, bestID, 0), b = tri_vertex(M, bestID, 1), c = tri_vertex(M, bestID, 2);
    h.Ng = norm3(cross3(sub3(b, a), sub3(c, a)));
  }
  return h;
}

#endif  // __CUDACC__

} // namespace exa
