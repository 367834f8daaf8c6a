/*
 * exastitch.h -- C ABI of the GB300-native ExaStitch volume-rendering path.
 *
 * The path: per-macrocell majorant build, ExaStitch field sampling (gridlet
 * trilinear lookup plus point location in the stitched unstructured boundary
 * elements) and Woodcock / ratio tracking through a DDA-traversed majorant
 * grid.  Every entry point is a plain C function taking plain pointers and
 * sizes; no C++ or CUDA type crosses this boundary.  All functions return an
 * int status (EXA_OK == 0); on failure exa_last_error() holds a message for
 * the calling thread.  No exception crosses the boundary.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the owlExaStitcher source tree).
 *
 * Threading: one exa_context per host thread.  All device work of a context
 * is issued on the context's CUDA stream (its own, or one the caller hands
 * in).  Build steps are synchronous at return; exa_render and
 * exa_sample_points are asynchronous on that stream (call exa_sync).
 */
#ifndef EXASTITCH_H
#define EXASTITCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* status codes                                                        */
/* ------------------------------------------------------------------ */
#define EXA_OK               0
#define EXA_ERR_INVALID      1  /* bad argument, unsupported option     */
#define EXA_ERR_CUDA         2  /* CUDA runtime error                    */
#define EXA_ERR_STATE        3  /* call out of order (e.g. no model)     */
#define EXA_ERR_OOM          4  /* device allocation failed              */
#define EXA_ERR_DEVICE_LIMIT 5  /* a device-side iteration cap was hit   */

/* device error-flag bits (exa_get_device_errors) */
#define EXA_DEVERR_DDA_CAP      1u  /* DDA walked more cells than the grid has */
#define EXA_DEVERR_TRACK_CAP    2u  /* delta/ratio tracking step cap            */
#define EXA_DEVERR_BVH_STACK    4u  /* reserved (element point location keeps no stack) */
#define EXA_DEVERR_BOUNCE_CAP   8u  /* reserved (paths end at ext.maxBounces)    */
#define EXA_DEVERR_WATCHDOG    16u  /* persistent-kernel work loop cap          */
#define EXA_DEVERR_COPY_WAIT   32u  /* bulk copy to shared memory: wait limit   */
#define EXA_DEVERR_BOUNDS      64u  /* bounds-checked build (EXA_CHECKS=1): an  */
                                    /* index out of range, its access skipped  */

/* exa_debug_set_flags: simulations of error paths for tests */
#define EXA_DEBUG_COPY_WAIT_TIMEOUT 1u  /* the majorant build's first bulk-copy */
                                        /* wait in block 0 counts as timed out  */
                                        /* after the copy completed             */

/* ------------------------------------------------------------------ */
/* plain data types (layouts equal to the owl::common types they       */
/* stand in for: vec3f, vec4f, vec3i, box3f, interval<float>, affine3f) */
/* ------------------------------------------------------------------ */
typedef struct { float x, y; } exa_vec2f;
typedef struct { float x, y, z; } exa_vec3f;
typedef struct { float x, y, z, w; } exa_vec4f;
typedef struct { int32_t x, y, z; } exa_vec3i;
typedef struct { exa_vec2f lower, upper; } exa_box2f;
typedef struct { exa_vec3f lower, upper; } exa_box3f;
typedef struct { float lower, upper; } exa_range1f;
typedef struct { exa_vec3f vx, vy, vz; } exa_linear3f;
typedef struct { exa_linear3f l; exa_vec3f p; } exa_affine3f;

/* Gridlet.h:22-37 -- a brick of level-`level` dual cells, scalars
 * (dims+1)^3 fp32 starting at gridletScalars[begin], NaN = absent. */
typedef struct {
  exa_vec3i lower;
  int32_t   level;
  exa_vec3i dims;
  uint32_t  begin;
} exa_gridlet;

/* sampler/Sampler.h:72-76 -- primID < 0: empty space; cellID == -1: the
 * sample came from a stitching element, else from gridlet primID. */
typedef struct {
  int32_t primID;
  int32_t cellID;
  float   value;
} exa_sample;

/* Grid.cuh:21-24 */
typedef struct {
  exa_vec3i dims;
  exa_box3f bounds;
} exa_grid_traversable;

/* KDTree.cuh:141-144 (slot kept for layout; unused by this sampler) */
typedef struct {
  void     *nodes;
  void     *primRefs;
  exa_box3f modelBounds;
} exa_kdtree_traversable;

/* sampler/ExaStitchSampler.h:42-49.  sampleBVH holds this library's
 * point-location handle (an opaque device address) in the slot that held
 * the OptixTraversableHandle. */
typedef struct {
  uint64_t     sampleBVH;
  exa_gridlet *gridletBuffer;
  float       *gridletScalarBuffer;
} exa_stitch_lp;

/* sampler/AMRCellSampler.h:30-35: the AMR-cell sampler's handle. */
typedef struct {
  uint64_t     sampleBVH;
} exa_amrcell_lp;

/* model/ABRs.h:28-63: a brick of size.x*size.y*size.z level-`level` cells
 * from `lower` (finest units); its scalars start at scalars[begin], x
 * fastest. */
typedef struct {
  exa_vec3i lower;
  exa_vec3i size;
  int32_t   level;
  uint32_t  begin;
} exa_brick;

/* model/ABRs.h:65-77: an active brick region, a box in which a fixed set of
 * bricks' basis functions overlap (leafList[leafListBegin ..
 * leafListBegin + leafListSize), ascending brick ids). */
typedef struct {
  exa_box3f   domain;
  exa_range1f valueRange;
  int32_t     leafListBegin;
  int32_t     leafListSize;
  float       finestLevelCellWidth;
} exa_abr;

/* sampler/ExaBrickSampler.h:37-46: the ExaBrick sampler's handle and
 * buffers. */
typedef struct {
  uint64_t   sampleBVH;
  exa_brick *brickBuffer;
  exa_abr   *abrBuffer;
  float     *scalarBuffer;
  int32_t   *abrLeafListBuffer;
} exa_exabrick_lp;

#define EXA_CLIP_PLANES_MAX 1   /* common.h:36 */
#define EXA_LIGHTS_MAX      4   /* common.h:37 */

#define EXA_PATH_TRACING_INTEGRATOR 0   /* common.h:46-48 */
#define EXA_DIRECT_LIGHT_INTEGRATOR 1
#define EXA_RAY_MARCHING_INTEGRATOR 2

#define EXA_SHADE_MODE_DEFAULT  0       /* common.h:50-52 */
#define EXA_SHADE_MODE_GRIDLETS 1
#define EXA_SHADE_MODE_TEASER   2

#define EXA_LIGHT_POINT       0
#define EXA_LIGHT_DIRECTIONAL 1

/* Transfer-function lookup (deviceCode.cu:320-341).  NEAREST is the
 * reference's buffer variant: the entry int(f * N) of the clamped,
 * normalised value f.  LINEAR restates its default texture variant
 * (EXASTITCH_CUDA_TEXTURE_TF, CMakeLists.txt:179-187; the texture set up in
 * OWLRenderer.cpp:659-707: normalised coordinates, linear filtering, border
 * address mode with a zero border colour) in binary32 arithmetic:
 * xB = f * N - 0.5, i = floor(xB), a = xB - i,
 * result = (1 - a) * T[i] + a * T[i + 1] per channel, limited to the
 * channel's range of the two entries, with T[k] = 0 outside [0, N).  The
 * hardware filter's 8-bit fraction of `a` is not reproduced. */
#define EXA_TF_FILTER_NEAREST 0
#define EXA_TF_FILTER_LINEAR  1

/* Fields appended after the reference's LaunchParams fields.  They have no
 * reference counterpart; their defaults (exa_launch_params_init) reproduce
 * the reference's hard-coded behaviour. */
typedef struct {
  int32_t   maxBounces;      /* deviceCode.cu:1050 hard-codes 1024          */
  float     albedo;          /* < 0: albedo = TF rgb (deviceCode.cu:1061)    */
  float     hgG;             /* HG anisotropy; reference uses 0 (:1089)      */
  int32_t   lightType[EXA_LIGHTS_MAX]; /* EXA_LIGHT_POINT / _DIRECTIONAL;   */
                             /* a directional light's lights[i].pos is the  */
                             /* direction towards the light                 */
  exa_affine3f voxelSpaceTransformInv; /* rcp(voxelSpaceTransform)         */
  int32_t   cullTransparentPrims;      /* 1: primitives with max opacity 0  */
                             /* are invisible to point location (the        */
                             /* reference's empty-AABB culling)             */
  uint32_t  frameID;         /* RNG stream selector for batched frames       */
  uint32_t *deviceErrors;    /* optional: EXA_DEVERR_* bits are OR-ed here   */
  unsigned long long *stepCounters; /* optional counting launch (16 u64): */
                             /* [0] field samples, [1] gridlet samples,      */
                             /* [2] element samples, [3] DDA cells,          */
                             /* [4] paths; wavefront renderer also: [5]      */
                             /* gridlet-cache misses, [6] table queries,     */
                             /* [7] gridlet tests, [8] element cell-list walks, */
                             /* [9] walks, [10] learned-field samples,       */
                             /* [11] learned samples limited to the         */
                             /* macrocell's widened majorant                 */
  float    *traceT;          /* optional, per pixel: distance (voxel space) */
                             /* of the first sample's first interaction, -1 */
                             /* if the ray left the volume                  */
  float    *traceTr;         /* optional, per pixel: transmittance of the   */
                             /* first sample's first shadow ray, -1 if none */
  uint32_t *heatCounts;      /* set by the library: per-pixel work of the   */
                             /* heat map (render.heatMapEnabled)            */
  int32_t   tfFilter;        /* EXA_TF_FILTER_NEAREST / _LINEAR; set by    */
                             /* exa_sampler_set_lps from the filter the max */
                             /* opacities were computed for                 */
  int32_t   trackStepCap;    /* > 0: tracking steps per macrocell after     */
                             /* which a walk ends with EXA_DEVERR_TRACK_CAP; */
                             /* 0: the built-in cap (2^22)                  */
  int32_t   ddaCellCap;      /* > 0: macrocells a walk may visit before it  */
                             /* ends with EXA_DEVERR_DDA_CAP; 0: the grid's */
                             /* dims.x + dims.y + dims.z + 3                */
  int32_t   rowBegin;        /* rowEnd > 0: exa_render / _surrogate render  */
  int32_t   rowEnd;          /* only the frame's rows [rowBegin, rowEnd)    */
                             /* (rowBegin a multiple of 8; rowEnd a multiple */
                             /* of 8 or the height), each pixel exactly as   */
                             /* in the whole frame (same rays and random     */
                             /* numbers); the other rows' outputs are not    */
                             /* written.  A frame split across GPUs.         */
  int32_t   pad0;
  int32_t   pad1;
} exa_lp_ext;

/* LaunchParams.h:56-119, field order and types kept; the sampler union
 * holds the ExaStitch, AMR-cell and ExaBrick members (all start with
 * sampleBVH);
 * transferFunc is the buffer variant (values/numValues,
 * LaunchParams.h:84-87). */
typedef struct {
  union { exa_stitch_lp ess; exa_amrcell_lp acs; exa_exabrick_lp ebs; } sampler;
  uint32_t  *fbPointer;
  float     *fbDepth;
  exa_vec4f *accumBuffer;
  int32_t    accumID;
  int32_t    integrator;
  int32_t    shadeMode;
  float     *maxOpacities;
  uint64_t   meshBVH;
  uint64_t   majorantBVH;
  exa_kdtree_traversable majorantKDTree;
  exa_grid_traversable   majorantGrid;
  exa_box3f    worldSpaceBounds;
  exa_affine3f voxelSpaceTransform;
  exa_affine3f lightSpaceTransform;
  struct {
    exa_vec4f  *values;
    int32_t     numValues;
    exa_range1f domain;
    float       opacityScale;
  } transferFunc;
  struct {
    exa_vec3f org;
    exa_vec3f dir_00;
    exa_vec3f dir_du;
    exa_vec3f dir_dv;
  } camera;
  struct {
    exa_box2f value;
    exa_box2f selection;
    int32_t   active;
    int32_t   selecting;
  } subImage;
  struct {
    float   dt;
    int32_t heatMapEnabled;
    float   heatMapScale;
    int32_t spp;
  } render;
  struct {
    int32_t   enabled;
    exa_vec3f N;
    float     d;
  } clipPlanes[EXA_CLIP_PLANES_MAX];
  struct {
    exa_vec3f pos;
    float     intensity;
    int32_t   on;
  } lights[EXA_LIGHTS_MAX];
  exa_lp_ext ext;
} exa_launch_params;

/* model/ExaStitchModel.cpp:259-279 (memStats) plus device footprint */
typedef struct {
  uint64_t elemVertexBytes;
  uint64_t elemIndexBytes;
  uint64_t gridletBytes;
  uint64_t emptyScalarsBytes;
  uint64_t nonEmptyScalarsBytes;
  uint64_t deviceFieldBytes;     /* field arrays resident in HBM           */
  uint64_t deviceAccelBytes;     /* gridlet tables + element cell lists      */
  uint64_t deviceMajorantBytes;  /* value ranges + max opacities            */
  uint64_t amrCellBytes;         /* AMR-cell model: cells (AMRCellModel::memStats) */
  uint64_t amrScalarBytes;       /* AMR-cell model: scalars                 */
  uint64_t bricksBytes;          /* ExaBrick model (ExaBrickModel::memStats) */
  uint64_t brickScalarsBytes;
  uint64_t abrsBytes;
  uint64_t abrLeafListBytes;
} exa_mem_stats;

typedef struct exa_context exa_context;

/* ------------------------------------------------------------------ */
/* context                                                             */
/* ------------------------------------------------------------------ */

/* Replaces owlContextCreate(nullptr,1) (OWLRenderer.cpp:331).  stream: the
 * cudaStream_t to issue all work on (0 is the CUDA default stream), or
 * EXA_STREAM_PRIVATE to have the context create and own a stream. */
#define EXA_STREAM_PRIVATE (~(uint64_t)0)
int exa_context_create(exa_context **out, int device, uint64_t stream);
int exa_context_destroy(exa_context *ctx);
/* Message of the last failed call on this thread ("" if none). */
const char *exa_last_error(void);
/* Waits for the context's stream; returns EXA_ERR_DEVICE_LIMIT if a
 * kernel raised a device error flag since the last call. */
int exa_sync(exa_context *ctx);
/* Reads and clears the context's device error bits (EXA_DEVERR_*). */
int exa_get_device_errors(exa_context *ctx, uint32_t *bits);
/* Test hook without a reference counterpart: EXA_DEBUG_* flags for the
 * context's next sampler builds (0 clears them).  A simulated failure
 * follows the real failure's path (the build returns EXA_ERR_CUDA) without
 * leaving any device work unfinished. */
int exa_debug_set_flags(exa_context *ctx, uint32_t flags);
/* Library version string. */
const char *exa_version(void);
/* sizeof of the ABI structs, for FFI bindings to check their layouts:
 * 0 exa_launch_params, 1 exa_gridlet, 2 exa_sample, 3 exa_mem_stats,
 * 4 exa_lp_ext, 5 exa_surrogate_params, 6 exa_surrogate_stats,
 * 7 exa_surrogate_geometry, 8 exa_batch_frame, 9 exa_batch_tuning,
 * 10 exa_xf, 11 exa_amr_cell, 12 exa_render_stats, 13 exa_build_stats,
 * 14 exa_brick, 15 exa_abr; 0 for other keys. */
uint64_t exa_abi_sizeof(int32_t which);

/* ------------------------------------------------------------------ */
/* model  (model/Model.h:29-65, model/ExaStitchModel.h:26-55)          */
/* ------------------------------------------------------------------ */

/* Replaces ExaStitchModel::load (model/ExaStitchModel.cpp:24-257) for
 * in-memory arrays: vertices (x,y,z,value), indices 8 per element padded
 * with -1 (4 = tet, 5 = pyramid, 6 = wedge, 8 = hex; rows of other counts
 * are never hit), gridlets and their scalars.  Host pointers; arrays are
 * copied.  Computes cellBounds and valueRange as the loader does.  Either
 * part may be empty.  EXA_ERR_INVALID for an index past the vertices, a row
 * with a vertex after its -1 padding, a gridlet header with negative dims or
 * a level outside 0..30, or scalars past the scalar array. */
int exa_model_create(exa_context *ctx,
                     const exa_vec4f *vertices, uint64_t numVertices,
                     const int32_t *indices, uint64_t numElems,
                     const exa_gridlet *gridlets, uint64_t numGridlets,
                     const float *gridletScalars, uint64_t numGridletScalars);

/* On-disk inputs.  Host-only parsers (no context, no device): call once
 * with null output arrays to get the counts, then again with arrays of
 * those sizes.  Files are little-endian as the reference writes them. */

/* '.grids' + '.scalars' as ExaStitchModel::load reads them
 * (model/ExaStitchModel.cpp:44-55, 191-247): per gridlet int32 lower[3],
 * level, dims[3] and (dims+1)^3 int32 scalar IDs into the '.scalars' file
 * (raw float32); IDs outside that file become NaN (absent).  Gridlet
 * 'begin' offsets are assigned in file order. */
int exa_read_grids(const char *gridsFile, const char *scalarsFile, exa_gridlet *gridlets, uint64_t *numGridlets,
                   float *gridletScalars, uint64_t *numGridletScalars);
/* ExaStitchModel::load for a gridlet-only model (no '.umesh' part: that
 * format belongs to the un-vendored umesh library): exa_read_grids then
 * exa_model_create. */
int exa_model_load(exa_context *ctx, const char *gridsFile, const char *scalarsFile);

/* '.xf' transfer function (headless.cpp:258-283): uint64 magic
 * 0x1235abc000, float opacityScale, absDomain (2 floats), relDomain (2
 * floats, percent), int32 count, float4 colours. */
typedef struct exa_xf {
  float opacityScale;
  exa_range1f absDomain, relDomain;
  int32_t numColors;
} exa_xf;
int exa_read_xf(const char *xfFile, exa_xf *xf, exa_vec4f *colors, int32_t maxColors);
/* The value range the transfer function spans (Headless::xfRange,
 * headless.cpp:285-298): absDomain ordered, relDomain / 100 ordered,
 * range = lerp(abs, rel.lower) .. lerp(abs, rel.upper). */
exa_range1f exa_xf_range(const exa_xf *xf);
/* LaunchParams.transferFunc.opacityScale for a viewer opacity setting s:
 * 1.1^(s - 100) (OWLRenderer.cpp:743). */
float exa_opacity_scale(float s);

/* AMR '.cells' (tools/amrMakeDualMesh/makeDual.cpp:932-940): 16-byte
 * records int32 pos[3], level; the matching scalars are a raw float32 file
 * in the same order. */
typedef struct exa_amr_cell {
  exa_vec3i pos;
  int32_t level;
} exa_amr_cell;
int exa_read_cells(const char *cellsFile, exa_amr_cell *cells, uint64_t *numCells);
/* AMRCellModel (model/AMRCellModel.h, AMRCellModel.cpp:24-67): the
 * context's model becomes the AMR leaf cells with one scalar each (numScalars
 * >= numCells; a cell's pos must be a multiple of its width 2^level, and no
 * cell may repeat).  cellBounds is the union of the cells [pos, pos + 2^level],
 * valueRange spans the non-NaN scalars of the cells.  exa_sampler_build then
 * builds the AMRCellSampler (tent-basis reconstruction, the reference's
 * comparison sampler; sampler/AMRCellSampler.*). */
int exa_amrcell_model_create(exa_context *ctx, const exa_amr_cell *cells, uint64_t numCells, const float *scalars,
                             uint64_t numScalars);
/* AMRCellModel::load (AMRCellModel.cpp:24-67): '.cells' records and a raw
 * float32 scalars file. */
int exa_amrcell_model_load(exa_context *ctx, const char *cellsFile, const char *scalarsFile);
/* ExaBrickModel::load(bricks, scalars, numBricks) (model/ExaBrickModel.cpp:
 * 120-143) and init() (:145-168): the context's model becomes the bricks;
 * the scalars array holds the bricks' cells (bricks[i].begin +
 * size.x*size.y*size.z <= numScalars).  The active brick regions are built
 * on the host (ABRs::buildFrom, model/ABRs.cpp).  exa_sampler_build then
 * builds the ExaBrickSampler in the reference's "majorant grid + DDA"
 * traversal mode (EXA_STITCH_EXA_BRICK_TRAVERSAL_MODE 1) with ABR sampling
 * (sampler mode 0). */
int exa_exabrick_model_create(exa_context *ctx, const exa_brick *bricks, uint64_t numBricks, const float *scalars,
                              uint64_t numScalars);
/* ExaBrickModel::load(brickFile, scalarFile) (ExaBrickModel.cpp:28-117):
 * '.bricks' records int32 size[3], lower[3], level, then size.x*size.y*size.z
 * int32 cell ids into the float32 scalars file. */
int exa_exabrick_model_load(exa_context *ctx, const char *bricksFile, const char *scalarsFile);
/* the model's active brick regions and their leaf list (null arrays: counts
 * only) */
int exa_exabrick_get_abrs(exa_context *ctx, exa_abr *abrs, uint64_t *numAbrs, int32_t *leafList,
                          uint64_t *leafListSize);

/* Surface meshes (TriangleMesh.cpp:27-76; OWLRenderer.cpp:446-545).  A mesh
 * file is a sequence of meshes, each int32 numVerts, numVerts float3,
 * int32 numTris, numTris int3; an index outside its mesh is "broken
 * triangle model".  exa_read_mesh concatenates the meshes into one
 * triangle soup (indices offset by the vertices before them); call it with
 * null arrays for the counts, then with arrays that large. */
int exa_read_mesh(const char *meshFile, exa_vec3f *vertices, uint64_t *numVertices,
                  exa_vec3i *indices, uint64_t *numTriangles);
/* The context's surface mesh (one triangle soup; the reference's instance
 * group of meshes without transforms): uploads it and builds its BVH
 * (replacing the OptiX triangle GAS and TLAS).  numTriangles == 0 removes
 * the mesh.  While a mesh is set, exa_sampler_set_lps sets lp->meshBVH to
 * it and extends worldSpaceBounds by the triangles' bounds
 * (OWLRenderer.cpp:453-465, 520).  Meshes are drawn by the path tracer,
 * the direct-light integrator (wavefront path) and the ray marcher; the
 * batched and the no-allocation entry points reject them. */
int exa_mesh_set(exa_context *ctx, const exa_vec3f *vertices, uint64_t numVertices,
                 const exa_vec3i *indices, uint64_t numTriangles);
/* bounds of the mesh's triangles; EXA_ERR_STATE when none is set */
int exa_mesh_get_bounds(exa_context *ctx, exa_box3f *bounds);

/* Model::cellBounds / Model::valueRange (model/Model.h:54-55). */
int exa_model_get_bounds(exa_context *ctx, exa_box3f *cellBounds,
                         exa_range1f *valueRange);
/* Model::setNumGridCells (model/Model.cpp:25-33): fails if the grid was
 * already set. */
int exa_model_set_num_grid_cells(exa_context *ctx, exa_vec3i numMCs);
/* Model::setVoxelSpaceTransform (model/Model.cpp:35-48). */
int exa_model_set_voxel_space_transform(exa_context *ctx, exa_box3f remapFrom,
                                        exa_box3f remapTo);
/* Model::getBounds (model/Model.cpp:50-70): world-space bounds. */
int exa_model_get_world_bounds(exa_context *ctx, exa_box3f *bounds);
/* ExaStitchModel::memStats (model/ExaStitchModel.cpp:259-279). */
int exa_model_mem_stats(exa_context *ctx, exa_mem_stats *out);

/* ------------------------------------------------------------------ */
/* sampler  (sampler/Sampler.h:28-69, sampler/ExaStitchSampler.h)      */
/* ------------------------------------------------------------------ */

/* ExaStitchSampler::build (sampler/ExaStitchSampler.cpp:23-340): uploads
 * the field, builds the per-primitive value ranges, the point-location
 * accel (gridlet tables + element cell lists, replacing the OptiX TLAS) and the
 * majorant grid (Grid::build, Grid.cu:457-594).  EXA_ERR_STATE where the
 * reference returns false. */
int exa_sampler_build(exa_context *ctx);
/* ExaStitchSampler::computeMaxOpacities (sampler/ExaStitchSampler.cu:
 * 279-376) and Grid::computeMaxOpacities (Grid.cu:721-737).  colorMap is a
 * host array of numColors RGBA entries. */
int exa_sampler_compute_max_opacities(exa_context *ctx,
                                      const exa_vec4f *colorMap,
                                      int32_t numColors, exa_range1f xfRange);
/* The transfer-function lookup of the context's renders
 * (EXA_TF_FILTER_NEAREST, the default, or EXA_TF_FILTER_LINEAR); replaces
 * the reference's compile-time choice EXASTITCH_CUDA_TEXTURE_TF
 * (CMakeLists.txt:179-187).  Takes effect at the next
 * exa_sampler_compute_max_opacities: under LINEAR the max opacities of a
 * value range take every entry the filter can blend for it, floor(l*N-0.5)
 * to floor(u*N-0.5)+1 (the reference maps a range to int(l*(N-1)) ..
 * int(u*(N-1))+1 for both lookups, which under its texture filter can miss
 * an entry the filter reads), so that they stay a bound on the filtered
 * opacity.  exa_sampler_set_lps writes the filter to lp.ext.tfFilter; a
 * render whose lp.ext.tfFilter differs is rejected. */
int exa_set_transfer_function_filter(exa_context *ctx, int32_t filter);
/* How exa_render runs a path-traced or direct-light frame (no reference
 * counterpart; every choice renders the same frame bit for bit):
 * EXA_RENDER_PATH_AUTO (the default) renders a frame of at most one wave of
 * samples (about 78K on a GB300) with one launch of a thread per sample and
 * larger frames with the wavefront renderer; _WAVEFRONT and _SINGLE_LAUNCH
 * force one.  Frames with a surface mesh, the Teaser shade mode, the heat
 * map or a band of rows, and learned-field frames, always use the
 * wavefront renderer. */
#define EXA_RENDER_PATH_AUTO           0
#define EXA_RENDER_PATH_WAVEFRONT      1
#define EXA_RENDER_PATH_SINGLE_LAUNCH  2
int exa_set_render_path(exa_context *ctx, int32_t path);
/* ExaStitchSampler::setLPs (sampler/ExaStitchSampler.cpp:356-365) plus the
 * majorant-grid and max-opacity LP variables OWLRenderer::initGPU and
 * setColorMap set (OWLRenderer.cpp:435-436, 652-657). */
int exa_sampler_set_lps(exa_context *ctx, exa_launch_params *lp);
/* Sampler::className (sampler/ExaStitchSampler.h:59). */
const char *exa_sampler_class_name(void);
/* className() of the context's built sampler ("ExaStitchSampler",
 * "AMRCellSampler" or "ExaBrickSampler"), "" before exa_sampler_build. */
const char *exa_sampler_get_class_name(exa_context *ctx);
/* Grid::valueRanges / Grid::maxOpacities (Grid.h:70-73), copied to host
 * arrays of numMCs entries (either pointer may be NULL). */
int exa_get_majorants(exa_context *ctx, exa_range1f *valueRanges,
                      float *maxOpacities);
/* Per-primitive value ranges and max opacities (gridletValueRanges,
 * gridletMaxOpacities, umeshMaxOpacities: sampler/ExaStitchSampler.h:
 * 97-103), host arrays; any pointer may be NULL. */
int exa_get_prim_majorants(exa_context *ctx, exa_range1f *gridletRanges,
                           float *gridletMaxOpacities,
                           float *elemMaxOpacities);

/* ------------------------------------------------------------------ */
/* field sampling: sample() (sampler/ExaStitchSampler.h:128-140)       */
/* ------------------------------------------------------------------ */

/* Point query at n positions (voxel space).  Device pointers; async on the
 * context stream.  cullTransparent: 1 = primitives whose max opacity is 0
 * are invisible, as in the reference after computeMaxOpacities. */
int exa_sample_points(exa_context *ctx, const exa_vec3f *posDevice,
                      uint64_t n, exa_sample *outDevice,
                      int32_t cullTransparent);
/* Same, host buffers: copies in, samples, copies out; synchronous. */
int exa_sample_points_host(exa_context *ctx, const exa_vec3f *posHost,
                           uint64_t n, exa_sample *outHost,
                           int32_t cullTransparent);

/* ------------------------------------------------------------------ */
/* rendering: renderFrame_ExaStitchSampler (deviceCode.cu:1390-1400)   */
/* ------------------------------------------------------------------ */

/* Fills lp with the reference defaults (OWLRenderer::initGPU,
 * OWLRenderer.cpp:548-578; render(), :610-622) and the extension
 * defaults that reproduce the reference behaviour. */
int exa_launch_params_init(exa_launch_params *lp);
/* One frame: width*height pixels, lp->render.spp samples each, into
 * lp->fbPointer (RGBA8) and lp->accumBuffer (device pointers owned by the
 * caller).  Replaces owlLaunch2D(rayGen,w,h,lp) (OWLRenderer.cpp:621).
 * The wavefront renderer reads back whether another round is needed once
 * per group of rounds (4, then 8), so the call returns after the frame's
 * kernels have been issued and most of them have run; call exa_sync before
 * reading the outputs.  EXA_ERR_INVALID, before any launch, for launch
 * parameters that exa_sampler_set_lps did not set for this context's
 * sampler (the sampler handle, the majorant grid's dims, the transfer-
 * function filter) and for unsupported options. */
int exa_render(exa_context *ctx, const exa_launch_params *lp,
               int32_t width, int32_t height);

/* How the last exa_render call ran (no reference counterpart). */
typedef struct {
  uint32_t wavefront;      /* 1: the wavefront renderer ran               */
  uint32_t rounds;         /* camera / walk / event rounds with work      */
  uint32_t peakQueue;      /* most path records queued after a round      */
  uint32_t queueCapacity;  /* record capacity of each queue               */
  uint32_t walkLaunches;   /* rounds launched (the last group's tail finds no work) */
  float    cameraMs;       /* summed GPU time of the camera kernels       */
  float    walkMs;         /* summed GPU time of the walk kernels         */
  float    eventMs;        /* summed GPU time of the event kernels        */
  uint32_t kernelLaunches; /* this library's kernel launches of the frame */
} exa_render_stats;
int exa_get_render_stats(exa_context *ctx, exa_render_stats *out);

/* How the last exa_sampler_build ran (no reference counterpart): GPU times
 * from CUDA events on the context's stream around the majorant kernels
 * (ExaStitch sampler; 0 for the other samplers) and the call's host time. */
typedef struct {
  float    totalMs;           /* exa_sampler_build, host wall time          */
  float    elemMajorantMs;    /* element value ranges into the grid         */
  float    gridletMajorantMs; /* gridlet value ranges into the grid         */
  uint32_t majorantBlocks;    /* gridlet pipelines (warps) of the majorant  */
                              /* build's separable kernel                   */
} exa_build_stats;
int exa_get_build_stats(exa_context *ctx, exa_build_stats *out);

/* ------------------------------------------------------------------ */
/* allocation-free rendering                                           */
/* ------------------------------------------------------------------ */

/* Largest width * height * spp one exa_render_noalloc call accepts. */
#define EXA_NOALLOC_MAX_SAMPLES (1u << 20)

/* The same frame as exa_render, for callers that must not allocate device
 * memory in their frame loop: exa_render allocates its per-sample colour
 * buffer with cudaMalloc the first time it sees a frame size, and cudaMalloc
 * synchronizes the device (stalling a pipelined render loop) and fails in
 * hosts that have handed all device memory to their own pool.  This entry
 * point calls no cudaMalloc, cudaFree or other allocating routine; its
 * scratch is a fixed 16 MiB array in the library's device image
 * (EXA_NOALLOC_MAX_SAMPLES float4 sample colours), which every GPU that
 * loads the library holds until the process exits.  Frames with
 * width * height * lp->render.spp above EXA_NOALLOC_MAX_SAMPLES are
 * rejected with EXA_ERR_INVALID.
 * The first call on a device looks up that array's device address (and,
 * with lazy module loading, loads the module): make the first call before
 * any stream capture.  All calls share the one array; calls whose kernels
 * overlap on the GPU (e.g. from two contexts on different streams) race on
 * it.  Every sample slot a frame reads is written by the same frame, so
 * nothing has to be cleared between calls.
 * This entry point has no counterpart in the reference. */
int exa_render_noalloc(exa_context *ctx, const exa_launch_params *lp,
                       int32_t width, int32_t height);

/* ------------------------------------------------------------------ */
/* batched frames (no counterpart in the reference)                    */
/* ------------------------------------------------------------------ */

/* One frame of a batch: camera (LaunchParams.camera), size, samples per
 * pixel, transfer function (index into exa_batch_set_transfer_functions),
 * progressive-accumulation index and RNG frame index, and device output
 * buffers (either may be null; accumBuffer is needed when accumID > 0). */
typedef struct exa_batch_frame {
  exa_vec3f org, dir_00, dir_du, dir_dv;
  int32_t width, height, spp, tf;
  uint32_t accumID, frameID;
  uint32_t *fbPointer;
  exa_vec4f *accumBuffer;
} exa_batch_frame;

/* Result of exa_batch_autotune: the chosen majorant-grid resolution and job
 * tile width, and every trial's time for the sampled workload. */
typedef struct exa_batch_tuning {
  exa_vec3i dims;
  int32_t tileWidth;
  float msBest;
  int32_t numTrials;
  exa_vec3i trialDims[16];
  int32_t trialTileWidth[16];
  float trialMs[16];
} exa_batch_tuning;

/* Transfer functions of the batch: host colour maps (RGBA), their sizes,
 * value ranges and opacity scales (null: 1).  Computes each one's max
 * opacities on the batch's majorant grid and its primitive culling data. */
int exa_batch_set_transfer_functions(exa_context *ctx, int32_t numTFs, const exa_vec4f *const *colorMaps,
                                     const int32_t *numColors, const exa_range1f *xfRanges,
                                     const float *opacityScales);
/* Majorant grid of the batch over the model's cell bounds (default: the
 * model's grid).  Rebuilds the value ranges and every transfer function's
 * max opacities. */
int exa_batch_set_majorant_grid(exa_context *ctx, exa_vec3i dims);
/* Width of the 128-job pixel tiles of the batch's job order: 8, 16 or 32. */
int exa_batch_set_tile_width(exa_context *ctx, int32_t tileWidth);
/* Renders numFrames frames in one wavefront (one set of queues; each
 * frame's result equals exa_render of that frame with the same parameters
 * and majorant grid).  lpTemplate supplies everything a frame does not
 * (integrator, lights, bounces, albedo, phase function, shade mode,
 * transforms, counters); exa_sampler_set_lps must have filled it.
 * useGraph != 0: the rounds run from the device inside one CUDA graph (built
 * on the first call for a batch shape, then replayed); else a host loop
 * synchronizes once per round.  Asynchronous (exa_sync). */
int exa_render_batch(exa_context *ctx, const exa_launch_params *lpTemplate, const exa_batch_frame *frames,
                     int32_t numFrames, int32_t useGraph);
/* Times the batch's workload (every sampleEvery-th frame at 1 spp) on
 * majorant grids of 32^3, 64^3, 128^3 and 256^3 and tile widths 8, 16 and
 * 32, keeps the fastest setting for the batch, and reports all trials. */
int exa_batch_autotune(exa_context *ctx, const exa_launch_params *lpTemplate, const exa_batch_frame *frames,
                       int32_t numFrames, int32_t sampleEvery, exa_batch_tuning *out);

/* ------------------------------------------------------------------ */
/* learned field (no counterpart in the reference)                     */
/* ------------------------------------------------------------------ */

/* A multiresolution hash-grid encoding (16 levels x 2 FP16 features) and
 * an MLP (32 -> 64 -> 64 -> 1, ReLU, BF16 weights, FP32 accumulation on the
 * tensor cores) trained on (position, value) pairs that the exact sampler
 * draws.  Majorants of macrocells where it is used are widened by the
 * macrocell's measured maximum error; the other macrocells keep the exact
 * sampler. */
typedef struct exa_surrogate_params {
  int32_t log2TableSize;      /* hash-table entries per level: 2^this (19)  */
  int32_t baseResolution;     /* coarsest level's grid resolution (16)      */
  float growth;               /* resolution factor between levels (1.5)     */
  float importanceFraction;   /* share of pairs drawn inside refined        */
                              /* gridlets, the rest uniform (0.5)           */
  uint64_t numSamples;        /* training pairs (2^24)                      */
  int32_t batch;              /* pairs per training step (2^18)             */
  float learningRate;         /* Adam step size at the start of each        */
                              /* exa_surrogate_train call (1e-2)            */
  uint64_t seed;
  float learningRateFinal;    /* step size at its end, reached by           */
                              /* exponential decay (1e-3)                   */
  int32_t pad0;
} exa_surrogate_params;

typedef struct exa_surrogate_stats {
  float loss;                 /* mean squared error of the last training    */
                              /* batch, value range normalised to 1         */
  int32_t steps;              /* training steps taken                       */
  float tolerance;            /* of the last exa_surrogate_evaluate         */
  int32_t pad0;
  double rmse;                /* over the probe points, / value range       */
  double maxError;            /* largest |error| / value range              */
  uint64_t probePoints;
  uint64_t numMacrocells;
  uint64_t numSurrogateMacrocells;  /* macrocells using the learned field   */
  uint64_t tableBytes;        /* FP16 inference table                       */
  uint64_t weightBytes;       /* BF16 weights                               */
  uint64_t inferenceBytes;    /* table + weights + macrocell modes and      */
                              /* widened majorants                          */
  uint64_t fieldBytes;        /* exact field: gridlets, scalars, vertices,  */
                              /* indices and point-location structures      */
  uint64_t fallbackFieldBytes; /* the part of fieldBytes the exact-sampler  */
                              /* macrocells still need (primitives whose    */
                              /* bounds touch one) plus the point-location  */
                              /* structures                                 */
} exa_surrogate_stats;

/* Geometry of the encoding: per-level grid resolutions, levels indexed
 * densely (bit l), normalisation x = (pos - lo) * inv and value = vmin +
 * y * vrange. */
typedef struct exa_surrogate_geometry {
  int32_t log2TableSize;
  uint32_t denseMask;
  int32_t res[16];
  float lo[3], inv[3];
  float vmin, vrange;
} exa_surrogate_geometry;

void exa_surrogate_params_default(exa_surrogate_params *p);
/* Initialises the encoding and network and draws the training pairs with
 * the exact sampler (needs exa_sampler_build). */
int exa_surrogate_create(exa_context *ctx, const exa_surrogate_params *p);
/* steps training steps; loss (may be null) as in exa_surrogate_stats. */
int exa_surrogate_train(exa_context *ctx, int32_t steps, float *loss);
/* Probes every macrocell of the majorant grid (about pointsTarget points
 * in all, at least 8 per macrocell), sets each macrocell's mode (learned
 * field where it holds no empty space and its largest error is at most
 * tolerance x value range) and the widened majorants for the current
 * transfer function (recomputed by exa_sampler_compute_max_opacities). */
int exa_surrogate_evaluate(exa_context *ctx, float tolerance, uint64_t pointsTarget);
int exa_surrogate_get_stats(exa_context *ctx, exa_surrogate_stats *out);
int exa_surrogate_get_geometry(exa_context *ctx, exa_surrogate_geometry *out);
/* Learned-field values at n device positions (device output). */
int exa_surrogate_sample_points(exa_context *ctx, const exa_vec3f *posDevice, uint64_t n, float *outDevice);
/* FP32 master parameters, host arrays: weights 6208 floats (W1 64x32,
 * W2 64x64, w3 64, row-major out x in); table 2 x 16 x 2^log2TableSize
 * floats (level-major, feature pairs).  Either pointer may be null. */
int exa_surrogate_get_params(exa_context *ctx, float *weights, float *table);
int exa_surrogate_set_params(exa_context *ctx, const float *weights, const float *table);
/* Gradients of the training loss over n pairs (host float x 4: x, y, z,
 * value; NaN value = no sample) at the current parameters, without a
 * step: host outputs as in exa_surrogate_get_params (either may be null). */
int exa_surrogate_gradients(exa_context *ctx, const float *pairs, int32_t n, float *gWeights, float *gTable,
                            float *loss);
/* Per-macrocell results of exa_surrogate_evaluate, host arrays of
 * numMacrocells (any may be null): mode 1 = learned field, largest
 * measured |error| in value units, widened majorant. */
int exa_surrogate_get_macrocells(exa_context *ctx, uint8_t *mode, double *maxError, float *majorants);
/* exa_render with the learned field in the macrocells that use it. */
int exa_render_surrogate(exa_context *ctx, const exa_launch_params *lp, int32_t width, int32_t height);

#ifdef __cplusplus
}
#endif

#endif /* EXASTITCH_H */
