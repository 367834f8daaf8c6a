// exa_host.h -- C++ host side of the ExaStitch path: the reference's plugin
// classes (model/Model.h:29-65, model/ExaStitchModel.h:26-55,
// sampler/Sampler.h:28-69, sampler/ExaStitchSampler.h:37-106, Grid.h:33-86)
// with the OWL handles replaced by owned device buffers.  The C ABI in
// exastitch.h is a thin layer over these classes.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/exastitch.h"
#include "exa_accel.cuh"
#include "exa_surrogate.cuh"

namespace exa {

// status-carrying exception used inside the library; converted to an int
// status at the C boundary
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void cudaCheck(cudaError_t e, const char *what);

// owned device allocation
template <typename T>
struct DBuf {
  T *ptr = nullptr;
  size_t count = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : ptr(o.ptr), count(o.count) { o.ptr = nullptr; o.count = 0; }
  DBuf &operator=(DBuf &&o) noexcept
  {
    if (this != &o) { release(); ptr = o.ptr; count = o.count; o.ptr = nullptr; o.count = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void release()
  {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
  void alloc(size_t n)
  {
    release();
    if (n == 0) return;
    cudaError_t e = cudaMalloc(&ptr, n * sizeof(T));
    if (e != cudaSuccess) {
      ptr = nullptr;
      (void)cudaGetLastError();
      throw Error(e == cudaErrorMemoryAllocation ? EXA_ERR_OOM : EXA_ERR_CUDA,
                  std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) + " bytes: " + cudaGetErrorString(e));
    }
    count = n;
  }
  void upload(const T *host, size_t n, cudaStream_t s)
  {
    if (n != count || !ptr) alloc(n);
    if (n) cudaCheck(cudaMemcpyAsync(ptr, host, n * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  }
  size_t bytes() const { return count * sizeof(T); }
};

struct Grid {  // Grid.h:33-86
  exa_vec3i dims{0, 0, 0};
  exa_box3f worldBounds{};
  DBuf<exa_range1f> valueRanges;
  DBuf<float> maxOpacities;
  exa_grid_traversable deviceTraversable{};
};

struct Model {  // model/Model.h:29-65
  Model();  // identity voxel- and light-space transforms (Model.h:57-61)
  virtual ~Model() = default;
  void setNumGridCells(exa_vec3i numMCs);                     // Model.cpp:25-33
  void setVoxelSpaceTransform(exa_box3f from, exa_box3f to);  // Model.cpp:35-48
  exa_box3f getBounds() const;                                // Model.cpp:50-70
  std::shared_ptr<Grid> grid;
  exa_box3f cellBounds{};
  exa_range1f valueRange{1e30f, -1e30f};
  exa_affine3f voxelSpaceTransform{};
  exa_affine3f voxelSpaceTransformInv{};
  exa_affine3f lightSpaceTransform{};
};

struct ExaStitchModel : Model {  // model/ExaStitchModel.h:26-55
  std::vector<int32_t> indices;
  std::vector<exa_vec4f> vertices;
  std::vector<exa_gridlet> gridlets;
  std::vector<float> gridletScalars;
  size_t numScalarsTotal = 0;
  size_t numEmptyScalars = 0;
  // arrays in, then the loader's bounds / value-range / statistics pass
  // (model/ExaStitchModel.cpp:78-114, 188-254)
  void assign(const exa_vec4f *v, size_t nv, const int32_t *idx, size_t ne, const exa_gridlet *g, size_t ng,
              const float *s, size_t ns);
  void memStats(size_t &elemVertexBytes, size_t &elemIndexBytes, size_t &gridletBytes, size_t &emptyScalarsBytes,
                size_t &nonEmptyScalarsBytes) const;
};

// AMRCellModel (model/AMRCellModel.h:26-44): leaf cells of an AMR
// hierarchy (position in finest units, level) with one scalar each
struct AMRCellModel : Model {
  std::vector<exa_amr_cell> cells;
  std::vector<float> scalars;
  // arrays in, then AMRCellModel::load's bounds / value-range pass
  // (model/AMRCellModel.cpp:56-64)
  void assign(const exa_amr_cell *c, size_t nc, const float *s, size_t ns);
  void memStats(size_t &cellsBytes, size_t &scalarsBytes) const;  // AMRCellModel.cpp:69-73
};

// ExaBrickModel (model/ExaBrickModel.h:27-52): bricks of same-level cells
// and their scalars; init() builds the active brick regions (ABRs::buildFrom,
// model/ABRs.cpp:264-333), cellBounds and valueRange
struct ExaBrickModel : Model {
  std::vector<exa_brick> bricks;
  std::vector<float> scalars;
  std::vector<exa_abr> abrs;
  std::vector<int32_t> leafList;
  void assign(const exa_brick *b, size_t nb, const float *s, size_t ns);
  void init();
  void memStats(size_t &bricksBytes, size_t &scalarsBytes, size_t &abrsBytes, size_t &leafListBytes) const;
};

struct Sampler {  // sampler/Sampler.h:28-69
  virtual ~Sampler() = default;
  virtual bool build(std::shared_ptr<Model> model, cudaStream_t s) = 0;
  virtual void computeMaxOpacities(const exa_vec4f *colorMap, int numColors, exa_range1f xfRange,
                                   cudaStream_t s) = 0;
  virtual void setLPs(exa_launch_params &lp) = 0;
  virtual std::string className() = 0;
  // device footprint: field arrays, point-location structures
  virtual size_t fieldBytes() const = 0;
  virtual size_t accelBytes() const = 0;
  struct {
    std::shared_ptr<Grid> grid;
  } majorantAccel;
  float *maxOpacities = nullptr;
  // the point-location view the kernels read; its device copy is the
  // handle stored in LP.sampler.*.sampleBVH
  AccelView accel{};
  DBuf<AccelView> deviceAccel;
  bool hasTF = false;
  DBuf<float4> colorMap;
  // EXA_TF_FILTER_* the max opacities are computed for (set before
  // computeMaxOpacities)
  int tfFilter = EXA_TF_FILTER_NEAREST;
  // EXA_DEBUG_* simulations of the build's error paths (set before build)
  uint32_t debugFlags = 0;
};

class ExaStitchSampler : public Sampler {  // sampler/ExaStitchSampler.h:37-106
 public:
  bool build(std::shared_ptr<Model> model, cudaStream_t s) override;
  void computeMaxOpacities(const exa_vec4f *colorMap, int numColors, exa_range1f xfRange, cudaStream_t s) override;
  void setLPs(exa_launch_params &lp) override;
  std::string className() override { return "ExaStitchSampler"; }

  std::shared_ptr<ExaStitchModel> model;
  // device field
  DBuf<exa_gridlet> gridletBuffer;
  DBuf<float> gridletScalarBuffer;
  DBuf<float4> vertexBuffer;
  DBuf<int32_t> indexBuffer;
  // per-primitive ranges and opacities
  DBuf<exa_range1f> gridletValueRanges;
  DBuf<float> gridletMaxOpacities;
  DBuf<exa_range1f> elemValueRanges;
  DBuf<float> umeshMaxOpacities;
  // the majorant build's list of gridlets for its general kernel
  DBuf<uint32_t> majorantScratch;
  // EXA_DEVERR_* bits of the build kernels
  DBuf<uint32_t> buildErrors;
  // GPU times of the last build's majorant kernels
  exa_build_stats buildStats{};
  // point-location accel
  std::vector<DBuf<int32_t>> tableEntries, tableItems;
  // element cells: bits, marked cells before each word, per marked cell its
  // entry, the lists, and per element its AABB
  DBuf<uint32_t> occBits, occRank;
  DBuf<int32_t> occEntries, occItems;
  DBuf<float4> elemBoxes;

  size_t fieldBytes() const override;
  size_t accelBytes() const override;

 private:
  void buildGridletTables(cudaStream_t s);
  void buildElementCells(cudaStream_t s);
};

// AMRCellSampler (sampler/AMRCellSampler.h:26-56, AMRCellSampler.cpp): the
// tent-basis field over AMR cells.  Point location by dense per-level
// lattices (replacing the OptiX user-geometry BVH); the majorant grid over
// the cells' supports (Grid.cu:248-285, 314-364).
class AMRCellSampler : public Sampler {
 public:
  bool build(std::shared_ptr<Model> model, cudaStream_t s) override;
  void computeMaxOpacities(const exa_vec4f *colorMap, int numColors, exa_range1f xfRange, cudaStream_t s) override;
  void setLPs(exa_launch_params &lp) override;
  std::string className() override { return "AMRCellSampler"; }
  size_t fieldBytes() const override;
  size_t accelBytes() const override;

  std::shared_ptr<AMRCellModel> model;
  DBuf<exa_amr_cell> cellBuffer;
  DBuf<float> scalarBuffer;
  std::vector<DBuf<uint32_t>> levelBits, levelRank;
  std::vector<DBuf<int32_t>> levelCell;
  AmrCellView view{};
  DBuf<AmrCellView> deviceView;
};

// ExaBrickSampler (sampler/ExaBrickSampler.h:30-96, ExaBrickSampler.cpp) in
// the majorant grid + DDA traversal mode: region point location by an LBVH
// over the region domains (replacing the OptiX ABR BVH); the majorant grid
// from every brick cell's basis support (Grid.cu:362-430)
class ExaBrickSampler : public Sampler {
 public:
  bool build(std::shared_ptr<Model> model, cudaStream_t s) override;
  void computeMaxOpacities(const exa_vec4f *colorMap, int numColors, exa_range1f xfRange, cudaStream_t s) override;
  void setLPs(exa_launch_params &lp) override;
  std::string className() override { return "ExaBrickSampler"; }
  size_t fieldBytes() const override;
  size_t accelBytes() const override;

  std::shared_ptr<ExaBrickModel> model;
  DBuf<exa_brick> brickBuffer;
  DBuf<float> scalarBuffer;
  DBuf<exa_abr> abrBuffer;
  DBuf<int32_t> abrLeafListBuffer;
  DBuf<float4> abrCorners;     // two corners per region: the BVH's vertex rows
  DBuf<int32_t> abrRows;
  DBuf<BvhNode> abrNodes;
  DBuf<int32_t> abrParents, abrLeafElem;
  BrickView view{};
  DBuf<BrickView> deviceView;
};

// default delta / ratio tracking steps per macrocell (EXA_DEVERR_TRACK_CAP)
constexpr int kTrackCapDefault = 1 << 22;

// the walks' loop caps the kernels read: lp.ext's values, or the defaults
// where they are 0 (tracking steps per macrocell; macrocells per walk:
// dims.x + dims.y + dims.z + 3, more than a DDA walk visits)
inline void fillLoopCaps(exa_launch_params &lp)
{
  if (lp.ext.trackStepCap <= 0) lp.ext.trackStepCap = kTrackCapDefault;
  if (lp.ext.ddaCellCap <= 0)
    lp.ext.ddaCellCap = lp.majorantGrid.dims.x + lp.majorantGrid.dims.y + lp.majorantGrid.dims.z + 3;
}

// ---------------------------------------------------------------- kernels
// launchers implemented in exa_build.cu / exa_render.cu
void launchInitRanges(exa_range1f *r, size_t n, cudaStream_t s);
// scratch: ng + 1 words (the gridlets the separable kernel leaves to the
// general one); returns the number of warps of the separable kernel
unsigned launchGridletMajorants(const exa_gridlet *g, const float *scalars, size_t ng, size_t nScalars,
                                exa_vec3i dims, exa_box3f wb, exa_range1f *mcRanges, exa_range1f *gridletRanges,
                                uint32_t *errors, uint32_t debugFlags, uint32_t *scratch, cudaStream_t s);
void launchElemMajorants(const float4 *verts, const int32_t *idx, size_t ne, exa_vec3i dims, exa_box3f wb,
                         exa_range1f *mcRanges, exa_range1f *elemRanges, cudaStream_t s);
// Grid.cu:248-285: every cell's value into the macrocells its support
// projects onto
void launchAmrCellMajorants(const exa_amr_cell *cells, const float *scalars, size_t n, exa_vec3i dims, exa_box3f wb,
                            exa_range1f *mcRanges, cudaStream_t s);
// the AMR sampler's level lattices: existence bits (with a duplicate
// check), ranks, and the rank -> cell map
void launchAmrLevelBits(const exa_amr_cell *cells, size_t n, int level, const int lo[3], const int nl[3],
                        uint32_t *bits, unsigned *dupFlag, cudaStream_t s);
void launchAmrLevelRank(const uint32_t *bits, size_t words, uint32_t *rank, cudaStream_t s);
void launchAmrLevelCells(const exa_amr_cell *cells, size_t n, int level, const int lo[3], const int nl[3],
                         const uint32_t *bits, const uint32_t *rank, int32_t *cellOf, cudaStream_t s);
// Grid.cu:399-430: every brick cell's value into the macrocells its basis
// support projects onto
void launchBrickMajorants(const exa_brick *bricks, size_t nb, const float *scalars, exa_vec3i dims, exa_box3f wb,
                          exa_range1f *mcRanges, cudaStream_t s);
void launchMaxOpacity(const exa_range1f *ranges, size_t n, const float4 *cmap, int ncolors, exa_range1f xf, int filter,
                      float *out, cudaStream_t s);
void launchBuildBVH(const float4 *verts, const int32_t *idx, size_t ne, exa_box3f sceneBounds, BvhNode *nodes,
                    int32_t *parents, int32_t *leafElem, cudaStream_t s);
// element cells over the grid O (origin, invCell, n set): fills O's
// arrays (allocated into the buffers)
void launchElemCells(const float4 *verts, const int32_t *idx, size_t ne, ElemOccupancy &O, DBuf<uint32_t> &bits,
                     DBuf<uint32_t> &rank, DBuf<int32_t> &entries, DBuf<int32_t> &items, DBuf<float4> &boxes,
                     cudaStream_t s);
// wavefront renderer: bufs holds 3 * kWfLaneWords * cap words, counters
// kWfCounterWords words
struct WfStats {
  unsigned rounds = 0, peakQueue = 0, walkLaunches = 0, kernelLaunches = 0;
  float cameraMs = 0.f, walkMs = 0.f, eventMs = 0.f;
};
void renderWavefront(const AccelView &A, const exa_launch_params &lp, int width, int height, float4 *colors,
                     uint32_t *bufs, unsigned cap, unsigned *counters, cudaStream_t s, WfStats *stats,
                     const SurrogateView *sur = nullptr);

// ------------------------------------------------------------ learned field
constexpr int kSurParams = kSurHidden * kSurIn + kSurHidden * kSurHidden + kSurHidden;  // 6208

struct SurrogateConfig {
  int levels = kSurLevels;
  int log2T = 19;
  int baseRes = 16;
  float growth = 1.5f;
  size_t numSamples = (size_t)1 << 24;
  float importance = 0.5f;  // fraction of samples inside refined gridlets
  int batch = 1 << 18;
  float lrTable = 1e-2f, lrMlp = 1e-2f;
  float lrFinal = 1e-3f;  // each trainSteps call decays lr exponentially to this
  uint64_t seed = 1234;
};

struct SurrogateStats {
  double rmse = 0.0, maxError = 0.0;  // over the probe points, in units of the value range
  size_t probePoints = 0, numMacrocells = 0, numSurrogateMCs = 0;
};

// hash-grid encoding + MLP trained on the exact sampler's values
struct Surrogate {
  SurrogateConfig cfg;
  SurrogateView view{};  // geometry of the encoding (pointers set by deviceView)
  DBuf<float2> table, gtable, mTable, vTable;  // FP32 master table, gradient, Adam moments
  DBuf<__half2> table16;                       // inference copy
  DBuf<float> w32, gw, mw, vw;                 // MLP: w1 | w2 | w3
  DBuf<__nv_bfloat16> wbf;
  DBuf<float4> samples;                        // (x, y, z, value or NaN)
  DBuf<__nv_bfloat16> feats;
  DBuf<float> dfeat, lossBuf;
  DBuf<uint32_t> trainErrors;  // EXA_DEVERR_* of the tensor-core training kernel
  DBuf<uint8_t> mcMode;
  DBuf<unsigned long long> mcErr;
  DBuf<unsigned> mcEmpty;
  DBuf<exa_range1f> widenedRanges;
  DBuf<float> majorants;
  uint64_t cursor = 0;
  int step = 0;
  float lastLoss = 0.f;
  bool evaluated = false;
  exa_vec3i evalDims{0, 0, 0};
  SurrogateStats stats;

  void configure(const SurrogateConfig &c, const ExaStitchModel &model);
  void allocate(cudaStream_t s);
  void setWeights(const float *w, cudaStream_t s);
  void setTable(const float *t, cudaStream_t s);
  void generateSamples(const ExaStitchSampler &sampler, cudaStream_t s);
  float trainSteps(int steps, cudaStream_t s);
  void gradients(const float4 *hostSamples, int n, float *gW, float *gTable, float *loss, cudaStream_t s);
  void evaluate(const ExaStitchSampler &sampler, const Grid &grid, double tol, size_t pointsTarget, cudaStream_t s);
  void computeMajorants(const float4 *cmap, int ncolors, exa_range1f xf, int filter, cudaStream_t s);
  SurrogateView deviceView() const;
  size_t inferenceBytes() const;
};
void launchSurrogatePoints(const SurrogateView &S, const exa_vec3f *pos, size_t n, float *out, cudaStream_t s);
bool useWavefront();
constexpr int kWfLaneWords = 63;
constexpr int kWfCounterWords = 16;  // wavefront queue counters + the frame's round control

// ---------------------------------------------------------- batched frames
struct WfFrame {                    // per frame of a batch (device table)
  int width, height;
  int tf, pad;                      // transfer function (index into WfBatchView.accels)
  unsigned long long jobBase;       // first job of the frame in the batch
  unsigned long long sampleBase;    // first colour slot of the frame
  unsigned long long pixelBase;     // first pixel of the frame (resolve)
};
struct WfBatchView {
  const AccelView *accels;          // per transfer function: primitive culling opacities (device)
  const exa_launch_params *lps;     // per frame (device)
  const WfFrame *frames;            // per frame (device)
  int numFrames;
  int tileW;                        // job tile width (tile height 128 / tileW)
  unsigned long long totalJobs, totalPixels;
};
struct WfCtl {                      // device-side round control
  unsigned long long issued;
  unsigned nIn, nNew, rounds, peak;
  int flip;
  unsigned more, error;
};
constexpr unsigned kBatchRoundCap = 1u << 20;
struct BatchKey {
  const void *accel, *accels, *lps, *frames;
  int numFrames, tileW;
  unsigned long long totalJobs, totalPixels;
  const void *bufs;
  unsigned cap;
  const void *counters, *ctl, *colors, *errors;
  int integrator;
  unsigned grid, walkGrid;
};
struct BatchGraph {                 // instantiated graph of one batch shape
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  BatchKey key{};
  cudaStream_t captureStream = nullptr;
  void release();
  ~BatchGraph();
};
void renderWavefrontBatch(const AccelView &A, const exa_launch_params &lp0, const WfBatchView &B, uint32_t *bufs,
                          unsigned cap, unsigned *counters, WfCtl *ctl, float4 *colors, uint32_t *deviceErrors,
                          bool useGraph, BatchGraph *cache, cudaStream_t s, WfStats *stats);
void launchSamplePoints(const AccelView &A, const exa_vec3f *pos, size_t n, exa_sample *out, int cull,
                        uint32_t *errors, cudaStream_t s);
void launchRender(const AccelView &A, const exa_launch_params &lp, int width, int height, unsigned *jobCounter,
                  float4 *colors, cudaStream_t s);

} // namespace exa
