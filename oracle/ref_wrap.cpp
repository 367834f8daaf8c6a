// Test infrastructure: extern "C" wrappers around the reference's own
// sampling headers (Gridlet.h, Plane.h, UElems.h, Grid.cuh, DDA.h), compiled
// unmodified from the reference tree against the project-written OWL shim in
// ref_shim/.  The resulting oracle/_ref/libexaref.so pins the oracle's
// restatement; it is never part of the product.
#include <common.h>
#include <Gridlet.h>
#include <Plane.h>
#include <UElems.h>
#include <Grid.cuh>
#include <DDA.h>

using namespace exa;

static inline float4 f4(const float *p) { return make_float4(p[0], p[1], p[2], p[3]); }

extern "C" {

int ref_intersect_gridlet(float *value, int *cellID, const float *pos,
                          const Gridlet *g, const float *scalars)
{
  return intersectGridlet(*value, *cellID, vec3f(pos[0], pos[1], pos[2]), *g, scalars) ? 1 : 0;
}

int ref_intersect_tet(float *value, const float *P, const float *v)
{
  return intersectTet(*value, vec3f(P[0], P[1], P[2]), f4(v), f4(v + 4), f4(v + 8), f4(v + 12)) ? 1 : 0;
}

int ref_intersect_pyr(float *value, const float *P, const float *v)
{
  return intersectPyrEXT(*value, vec3f(P[0], P[1], P[2]), f4(v), f4(v + 4), f4(v + 8),
                         f4(v + 12), f4(v + 16)) ? 1 : 0;
}

int ref_intersect_wedge(float *value, const float *P, const float *v)
{
  return intersectWedgeEXT(*value, vec3f(P[0], P[1], P[2]), f4(v), f4(v + 4), f4(v + 8),
                           f4(v + 12), f4(v + 16), f4(v + 20)) ? 1 : 0;
}

int ref_intersect_hex(float *value, const float *P, const float *v)
{
  return intersectHexEXT(*value, vec3f(P[0], P[1], P[2]), f4(v), f4(v + 4), f4(v + 8),
                         f4(v + 12), f4(v + 16), f4(v + 20), f4(v + 24), f4(v + 28)) ? 1 : 0;
}

void ref_project_on_grid(const float *V, const int *dims, const float *box, int *out)
{
  const vec3i r = projectOnGrid(vec3f(V[0], V[1], V[2]), vec3i(dims[0], dims[1], dims[2]),
                                box3f(vec3f(box[0], box[1], box[2]), vec3f(box[3], box[4], box[5])));
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ref_gridlet_bounds(const Gridlet *g, float *box)
{
  const box3f b = g->getBounds();
  box[0] = b.lower.x; box[1] = b.lower.y; box[2] = b.lower.z;
  box[3] = b.upper.x; box[4] = b.upper.y; box[5] = b.upper.z;
}

// dda3 with a recording functor: writes up to maxCells (cellID, t0, t1)
// triples and stops early when maxCells is reached.  Returns the count.
int ref_dda3(const float *org, const float *dir, float tmin, float tmax,
             const int *dims, const float *box, int maxCells,
             long long *cellIDs, float *t0s, float *t1s)
{
  owl::RayT<0, 1> ray;
  ray.origin = vec3f(org[0], org[1], org[2]);
  ray.direction = vec3f(dir[0], dir[1], dir[2]);
  ray.tmin = tmin;
  ray.tmax = tmax;
  int n = 0;
  dda3(ray, vec3i(dims[0], dims[1], dims[2]),
       box3f(vec3f(box[0], box[1], box[2]), vec3f(box[3], box[4], box[5])),
       [&](size_t id, float t0, float t1) {
         cellIDs[n] = (long long)id; t0s[n] = t0; t1s[n] = t1;
         return ++n < maxCells;
       });
  return n;
}

} // extern "C"
