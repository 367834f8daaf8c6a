/*
 * exastitch_gen.h -- C ABI of the synthetic AMR / dual-mesh generator.
 *
 * Replaces the reference's offline toolchain for in-memory use:
 *   AMR cells          -> tools/amrMakeDualMesh/makeDual.cpp (input .cells)
 *   dual cells         -> makeDual.cpp:596-872 (doCell)
 *   gridlets (.grids)  -> makeGrids.cpp:191-209, 114-168 (8^3 bricks)
 *   ExaStitch arrays   -> model/ExaStitchModel.cpp:24-257 (vertex values,
 *                         8-wide index rows, NaN for absent gridlet scalars)
 * Host code (C++/OpenMP) and a GPU version of the same stages (CUDA); the
 * output feeds exa_model_create.
 *
 * Level convention (the reference's): level L cells are 2^L finest units
 * wide, level 0 is the finest; the root level is numLevels-1.
 */
#ifndef EXASTITCH_GEN_H
#define EXASTITCH_GEN_H

#include <stdint.h>
#include "exastitch.h"

#ifdef __cplusplus
extern "C" {
#endif

#define EXA_FIELD_GAUSSIANS 0  /* sum of anisotropic Gaussians + value noise */
#define EXA_FIELD_CLOUD     1  /* sparse exp(3*fBm) cloud                     */

typedef struct {
  int32_t  numLevels;        /* levels in the hierarchy (root = numLevels-1) */
  int32_t  rootDims[3];      /* root-level cells per axis                    */
  int32_t  fieldKind;        /* EXA_FIELD_*                                  */
  int32_t  numGaussians;     /* gaussians field: count                       */
  uint64_t seed;             /* field seed                                   */
  float    refineThreshold;  /* gaussians: refine where |f| > t * max|f|     */
                             /* cloud: root refine threshold on f            */
  float    noiseAmplitude;   /* gaussians: value-noise amplitude             */
  int32_t  noiseOctaves;     /* gaussians: 4; cloud: fBm octaves (6)         */
  float    cloudEmptyFraction; /* cloud: fraction of root cells mapped to 0  */
  int32_t  balance;          /* 1: enforce 2:1 level balance                 */
  int32_t  numThreads;       /* 0: all                                       */
} exa_gen_params;

typedef struct exa_gen_result exa_gen_result;

typedef struct {
  uint64_t numAmrCells;      /* leaf cells                                   */
  uint64_t numCellsPerLevel[16];
  uint64_t numPerfectCubes;  /* dual cells that went into gridlets           */
  uint64_t numTets, numPyramids, numWedges, numHexes;
  uint64_t numVertices;      /* element vertices after compaction            */
  uint64_t numGridlets, numGridletScalars, numEmptyGridletScalars;
  uint64_t numSkippedDegenerate;
  double   seconds;
  float    fieldMin, fieldMax;
  double   stageSeconds[6];  /* field set-up, Gaussian tables, tree + 2:1
                                balance, cell values, elements, gridlets  */
} exa_gen_stats;

/* Fills p with the defaults of the small config (3 levels, 32^3 root,
 * 32 Gaussians, seed 1234, threshold 0.5, noise 0.1 over 4 octaves). */
void exa_gen_params_default(exa_gen_params *p);
/* Generates AMR cells, their dual mesh and the ExaStitch arrays. */
int  exa_gen_run(const exa_gen_params *p, exa_gen_result **out);
/* The same generator with every stage after the field set-up as CUDA
 * kernels on GPU `device`; the result is identical bit for bit to
 * exa_gen_run's and is returned in host memory like it (stageSeconds time
 * the GPU stages, including the copies back). */
int  exa_gen_run_gpu(const exa_gen_params *p, int32_t device, exa_gen_result **out);
void exa_gen_free(exa_gen_result *r);
void exa_gen_get_stats(const exa_gen_result *r, exa_gen_stats *s);
/* Borrowed pointers into the result (valid until exa_gen_free). */
const exa_vec4f   *exa_gen_vertices(const exa_gen_result *r, uint64_t *n);
const int32_t     *exa_gen_indices(const exa_gen_result *r, uint64_t *numElems);
const exa_gridlet *exa_gen_gridlets(const exa_gen_result *r, uint64_t *n);
const float       *exa_gen_gridlet_scalars(const exa_gen_result *r, uint64_t *n);
/* AMR leaf cells: pos (finest units, multiple of 2^level) and level, 16 B
 * each (the .cells record of makeDual.cpp:932-940), and their values. */
const int32_t     *exa_gen_amr_cells(const exa_gen_result *r, uint64_t *n);
const float       *exa_gen_amr_scalars(const exa_gen_result *r, uint64_t *n);
/* Analytic field at voxel-space points (finest units), for surrogate
 * training and error checks. */
void exa_gen_eval_field(const exa_gen_result *r, const exa_vec3f *pos,
                        uint64_t n, float *out);
const char *exa_gen_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
