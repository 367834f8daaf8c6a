/*
 * oracle.h -- CPU restatement of the owlExaStitcher ExaStitch rendering path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * (tests/, the smoke check and the timed CPU baseline in bench.py use it); it
 * is never linked into, loaded by or called from the product library.
 *
 * Arithmetic discipline: every function is plain IEEE-754 binary32 with no
 * contraction (built with -ffp-contract=off), in the operation order of the
 * reference source it cites.  The CUDA kernels follow the same order and are
 * built with --fmad=false, so results are bit-comparable.  log, sin and cos on
 * the path are the project's own series implementations (oc_log,
 * oc_sincos_turns) because the reference calls the CUDA math library there.
 */
#ifndef EXA_ORACLE_H
#define EXA_ORACLE_H

#include <stdint.h>
#include <stddef.h>
#include "../include/exastitch.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- project-defined math and RNG (shared definitions with the GPU) ---- */
uint64_t oc_mix64(uint64_t z);
float    oc_log(float x);
void     oc_sincos_turns(float u, float *s, float *c);

typedef struct { uint64_t key; uint64_t counter; } oc_rng;
void  oc_rng_init(oc_rng *r, uint32_t pixelID, uint32_t accumID, uint32_t frameID, uint32_t sampleID);
float oc_rng_next(oc_rng *r);

/* ---- cell / element interpolation (Gridlet.h, Plane.h, UElems.h) ---- */
int oc_intersect_gridlet(float *value, int *cellID, exa_vec3f pos,
                         const exa_gridlet *g, const float *scalars);
int oc_intersect_tet(float *value, exa_vec3f P, exa_vec4f a, exa_vec4f b,
                     exa_vec4f c, exa_vec4f d);
int oc_intersect_pyr(float *value, exa_vec3f P, const exa_vec4f *v5);
int oc_intersect_wedge(float *value, exa_vec3f P, const exa_vec4f *v6);
int oc_intersect_hex(float *value, exa_vec3f P, const exa_vec4f *v8);
/* element test dispatching on the vertex count of an 8-wide index row */
int oc_intersect_elem(float *value, exa_vec3f P, const int32_t *idx8,
                      const exa_vec4f *vertices);
exa_vec3i oc_project_on_grid(exa_vec3f V, exa_vec3i dims, exa_box3f bounds);
/* dda3 (DDA.h:26-113) recording (cellID, t0, t1) for each visited cell */
int oc_dda3(exa_vec3f org, exa_vec3f dir, float tmin, float tmax, exa_vec3i dims,
            exa_box3f box, int maxCells, long long *ids, float *t0s, float *t1s);

/* ---- field container with a uniform-grid point-location accel ---- */
typedef struct oc_field oc_field;
oc_field *oc_field_create(const exa_vec4f *vertices, uint64_t numVertices,
                          const int32_t *indices, uint64_t numElems,
                          const exa_gridlet *gridlets, uint64_t numGridlets,
                          const float *scalars, uint64_t numScalars);
void oc_field_destroy(oc_field *f);
/* per-primitive max opacities used for culling (NULL: no culling data) */
void oc_field_set_prim_opacities(oc_field *f, const float *gridletMaxOps,
                                 const float *elemMaxOps);
/* the field becomes the tent-basis reconstruction over AMR cells (16-byte
 * records pos[3], level; one scalar each; arrays not copied).  0 on
 * success; non-zero for fewer scalars than cells, a bad level, a position
 * that is not a multiple of the cell width, or a duplicate cell. */
int oc_field_set_amr(oc_field *f, const int32_t *cells, uint64_t numCells,
                     const float *scalars, uint64_t numScalars);
/* the field becomes the ExaBrick basis over bricks (arrays not copied); the
 * active brick regions are built here.  0 on success; non-zero for a bad
 * level, an empty brick or scalars past the end. */
int oc_field_set_bricks(oc_field *f, const exa_brick *bricks, uint64_t numBricks,
                        const float *scalars, uint64_t numScalars);
void oc_field_abrs(const oc_field *f, const exa_abr **abrs, uint64_t *numAbrs,
                   const int32_t **leafList, uint64_t *leafListSize);
/* surface mesh the integrators trace where lp->meshBVH != 0 (arrays are
 * not copied: numTris int3 rows into the float3 vertices) */
void oc_field_set_mesh(oc_field *f, const exa_vec3f *vertices,
                       const exa_vec3i *indices, uint64_t numTris);
/* cellBounds / valueRange as ExaStitchModel::load computes them */
void oc_field_bounds(const oc_field *f, exa_box3f *cellBounds,
                     exa_range1f *valueRange);
/* canonical point query: lowest-index containing gridlet, else
 * lowest-index containing element, else {-1,-1,0} */
exa_sample oc_sample(const oc_field *f, exa_vec3f pos, int cull);
void oc_sample_points(const oc_field *f, const exa_vec3f *pos, uint64_t n,
                      exa_sample *out, int cull, int nthreads);
/* every containing primitive: kinds[i] 0 = gridlet, 1 = element */
int oc_sample_all(const oc_field *f, exa_vec3f pos, int cull, int maxOut,
                  int *kinds, int *ids, float *values);

/* ---- majorants (Grid.cu, sampler/ExaStitchSampler.cu) ---- */
void oc_build_majorants(const oc_field *f, exa_vec3i dims, exa_box3f bounds,
                        exa_range1f *valueRanges);
void oc_compute_max_opacities(const exa_range1f *ranges, uint64_t n,
                              const exa_vec4f *colorMap, int numColors,
                              exa_range1f xfRange, int filter, float *out);
void oc_gridlet_value_ranges(const oc_field *f, exa_range1f *out);
void oc_elem_max_opacities(const oc_field *f, const exa_vec4f *colorMap,
                           int numColors, exa_range1f xfRange, int filter, float *out);

/* ---- rendering (deviceCode.cu) ----
 * lp holds HOST pointers: transferFunc.values, maxOpacities, accumBuffer,
 * fbPointer.  Renders pixels [pixelBegin, pixelEnd) of a width x height
 * frame.  Returns the OR of EXA_DEVERR_* bits raised. */
void oc_lookup_tf(const exa_launch_params *lp, float f, exa_vec4f *out);
uint32_t oc_render(const oc_field *f, const exa_launch_params *lp,
                   int width, int height, int64_t pixelBegin, int64_t pixelEnd,
                   int nthreads);
/* Same frame computed in binary64 arithmetic with independent random
 * numbers: the converged reference image for RMSE checks.  The
 * direct-lighting integrator tracks under the global majorant (delta
 * tracking to the first collision, ratio-tracking shadow rays); the path
 * tracer (integrator 0: albedo, HG g and bounce limit of lp.ext; no
 * meshes or clip planes) tracks through the majorant grid with a binary64
 * DDA.  Writes linear RGB (3 doubles/pixel, averaged over spp) into
 * outRGB for pixels [pixelBegin, pixelEnd). */
void oc_render_f64(const oc_field *f, const exa_launch_params *lp, int width,
                   int height, int64_t pixelBegin, int64_t pixelEnd,
                   double *outRGB, int nthreads);

/* ---- learned field (surrogate.c): hash-grid encoding + MLP ---- */
typedef struct os_geom {
  int32_t log2T;
  uint32_t denseMask;
  int32_t res[16];
  float lo[3], inv[3];
  float vmin, vrange;
} os_geom;
float os_bf16(float f);
void os_set_exact(int on);
float os_half(float f);
void os_geom_init(os_geom *g, int log2T, int baseRes, float growth, const float lo[3], const float hi[3], float vmin,
                  float vmax);
void os_encode(const os_geom *g, const float *table, const float pos[3], int half, float feat[32]);
void os_forward(const os_geom *g, const float *w, const float *table, const float *pos, int64_t n, double *y);
double os_gradients(const os_geom *g, const float *w, const float *table, const float *pairs, int n, double *gW,
                    double *gTable);

#ifdef __cplusplus
}
#endif
#endif
