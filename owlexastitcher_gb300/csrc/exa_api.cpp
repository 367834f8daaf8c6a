// exa_api.cpp -- host classes (Model, ExaStitchModel, ExaStitchSampler,
// Grid) and the C ABI of exastitch.h.  No exception crosses the C boundary.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "exa_host.h"
#include "exa_mesh.cuh"

namespace exa {

// ================================================================ Model
void Model::setNumGridCells(exa_vec3i numMCs)
{
  if (grid) throw Error(EXA_ERR_STATE, "must set num grid cells before calling initGPU!");
  if (numMCs.x <= 0 || numMCs.y <= 0 || numMCs.z <= 0) throw Error(EXA_ERR_INVALID, "grid dims must be positive");
  grid = std::make_shared<Grid>();
  grid->dims = numMCs;
}

static exa_affine3f affine_identity()
{
  exa_affine3f a;
  std::memset(&a, 0, sizeof(a));
  a.l.vx.x = a.l.vy.y = a.l.vz.z = 1.f;
  return a;
}

// affine3f::translate(lower) * affine3f::scale(span), and its inverse
static exa_affine3f affine_box(exa_box3f b, bool inverse)
{
  exa_affine3f a = affine_identity();
  const float sx = b.upper.x - b.lower.x, sy = b.upper.y - b.lower.y, sz = b.upper.z - b.lower.z;
  if (!inverse) {
    a.l.vx.x = sx; a.l.vy.y = sy; a.l.vz.z = sz;
    a.p = b.lower;
  } else {
    a.l.vx.x = 1.f / sx; a.l.vy.y = 1.f / sy; a.l.vz.z = 1.f / sz;
    a.p.x = -b.lower.x / sx; a.p.y = -b.lower.y / sy; a.p.z = -b.lower.z / sz;
  }
  return a;
}

// composition of two diagonal-linear affines: (A*B)(p) = A(B(p))
static exa_affine3f affine_mul_diag(const exa_affine3f &A, const exa_affine3f &B)
{
  exa_affine3f r = affine_identity();
  r.l.vx.x = A.l.vx.x * B.l.vx.x;
  r.l.vy.y = A.l.vy.y * B.l.vy.y;
  r.l.vz.z = A.l.vz.z * B.l.vz.z;
  r.p.x = A.l.vx.x * B.p.x + A.p.x;
  r.p.y = A.l.vy.y * B.p.y + A.p.y;
  r.p.z = A.l.vz.z * B.p.z + A.p.z;
  return r;
}

// Model.cpp:35-48: voxel = voxelCoordSys * rcp(worldCoordSys)
Model::Model()
{
  voxelSpaceTransform = affine_identity();
  voxelSpaceTransformInv = affine_identity();
  lightSpaceTransform = affine_identity();
}

void Model::setVoxelSpaceTransform(exa_box3f from, exa_box3f to)
{
  voxelSpaceTransform = affine_mul_diag(affine_box(from, false), affine_box(to, true));
  voxelSpaceTransformInv = affine_mul_diag(affine_box(to, false), affine_box(from, true));
}

static exa_vec3f xfm_point_h(const exa_affine3f &A, exa_vec3f p)
{
  exa_vec3f r;
  r.x = (p.x * A.l.vx.x + p.y * A.l.vy.x + p.z * A.l.vz.x) + A.p.x;
  r.y = (p.x * A.l.vx.y + p.y * A.l.vy.y + p.z * A.l.vz.y) + A.p.y;
  r.z = (p.x * A.l.vx.z + p.y * A.l.vy.z + p.z * A.l.vz.z) + A.p.z;
  return r;
}

exa_box3f Model::getBounds() const
{
  exa_box3f b;
  b.lower = xfm_point_h(voxelSpaceTransformInv, cellBounds.lower);
  b.upper = xfm_point_h(voxelSpaceTransformInv, cellBounds.upper);
  return b;
}

void ExaStitchModel::assign(const exa_vec4f *v, size_t nv, const int32_t *idx, size_t ne, const exa_gridlet *g,
                            size_t ng, const float *s, size_t ns)
{
  vertices.assign(v, v + nv);
  indices.assign(idx, idx + ne * 8);
  gridlets.assign(g, g + ng);
  gridletScalars.assign(s, s + ns);
  voxelSpaceTransform = affine_identity();
  voxelSpaceTransformInv = affine_identity();
  lightSpaceTransform = affine_identity();
  // model/ExaStitchModel.cpp:78-114 (elements) and 188-247 (gridlets)
  cellBounds.lower = {INFINITY, INFINITY, INFINITY};
  cellBounds.upper = {-INFINITY, -INFINITY, -INFINITY};
  valueRange = {1e30f, -1e30f};
  auto extend = [&](float x, float y, float z) {
    cellBounds.lower.x = std::min(cellBounds.lower.x, x); cellBounds.upper.x = std::max(cellBounds.upper.x, x);
    cellBounds.lower.y = std::min(cellBounds.lower.y, y); cellBounds.upper.y = std::max(cellBounds.upper.y, y);
    cellBounds.lower.z = std::min(cellBounds.lower.z, z); cellBounds.upper.z = std::max(cellBounds.upper.z, z);
  };
  for (size_t e = 0; e < ne; ++e)
    for (int j = 0, padded = 0; j < 8; ++j) {
      const int id = indices[e * 8 + j];
      if (id < 0) { padded = 1; continue; }
      // rows are -1 padded: a vertex after the padding would leave the
      // reference's vertex slots unset (programs/ExaStitchSampler.cu:135-143)
      if (padded) throw Error(EXA_ERR_INVALID, "element index row with a vertex after its -1 padding");
      if ((size_t)id >= nv) throw Error(EXA_ERR_INVALID, "element index out of range");
      const exa_vec4f &p = vertices[id];
      extend(p.x, p.y, p.z);
      valueRange.lower = std::min(valueRange.lower, p.w);
      valueRange.upper = std::max(valueRange.upper, p.w);
    }
  numScalarsTotal = 0;
  numEmptyScalars = 0;
  for (size_t k = 0; k < ng; ++k) {
    const exa_gridlet &gl = gridlets[k];
    if (gl.dims.x < 0 || gl.dims.y < 0 || gl.dims.z < 0 || gl.level < 0 || gl.level > 30)
      throw Error(EXA_ERR_INVALID, "invalid gridlet header");
    const size_t n = (size_t)(gl.dims.x + 1) * (gl.dims.y + 1) * (gl.dims.z + 1);
    if ((size_t)gl.begin + n > ns) throw Error(EXA_ERR_INVALID, "gridlet scalars out of range");
    for (size_t i = 0; i < n; ++i) {
      const float v = gridletScalars[gl.begin + i];
      if (std::isnan(v)) numEmptyScalars++;
      valueRange.lower = std::min(valueRange.lower, v);
      valueRange.upper = std::max(valueRange.upper, v);
    }
    numScalarsTotal += n;
    const float cw = (float)(1 << gl.level);
    extend(((float)gl.lower.x + 0.5f) * cw, ((float)gl.lower.y + 0.5f) * cw, ((float)gl.lower.z + 0.5f) * cw);
    extend((((float)gl.lower.x + (float)gl.dims.x) + 0.5f) * cw, (((float)gl.lower.y + (float)gl.dims.y) + 0.5f) * cw,
           (((float)gl.lower.z + (float)gl.dims.z) + 0.5f) * cw);
  }
}

// model/ExaStitchModel.cpp:259-279
void ExaStitchModel::memStats(size_t &elemVertexBytes, size_t &elemIndexBytes, size_t &gridletBytes,
                              size_t &emptyScalarsBytes, size_t &nonEmptyScalarsBytes) const
{
  elemVertexBytes = vertices.size() * sizeof(exa_vec4f);
  elemIndexBytes = indices.size() * sizeof(int32_t);
  gridletBytes = gridlets.size() * sizeof(exa_gridlet);
  emptyScalarsBytes = numEmptyScalars * sizeof(float);
  nonEmptyScalarsBytes = (numScalarsTotal - numEmptyScalars) * sizeof(float);
}

// ================================================================ sampler
size_t ExaStitchSampler::fieldBytes() const
{
  return gridletBuffer.bytes() + gridletScalarBuffer.bytes() + vertexBuffer.bytes() + indexBuffer.bytes();
}

size_t ExaStitchSampler::accelBytes() const
{
  size_t b = occBits.bytes() + occRank.bytes() + occEntries.bytes() + occItems.bytes() + elemBoxes.bytes();
  for (auto &t : tableEntries) b += t.bytes();
  for (auto &t : tableItems) b += t.bytes();
  return b;
}

// Per-level block tables over the dual-cell lattice.  Block width 8
// (makeGrids bricks); widened when a level's table would be very large.
// Block tables over dual-cell lattices.  A gridlet of level L covers, along
// each axis, the closed interval [lower + 0.5, lower + dims + 0.5] * 2^L of
// voxel space, which is [(2 lower + 1) r - 1, (2 (lower + dims) + 1) r - 1] / 2
// in units of the dual lattice of a table of level Lt <= L (r = 2^(L - Lt)).
// A gridlet is listed in every block whose open interior meets that
// interval; a query exactly on a block's low face also looks at the block
// below, so every gridlet whose closed box holds the point is seen.
//
// One table over the finest lattice holds every gridlet when its block grid
// fits with blocks of 8 or 16 cells (one lookup per query, lists sorted so
// the first hit is the lowest index); otherwise there is one table per
// level.
// widest blocks (2^n finest dual cells) of the one table over all levels;
// wider fields get one table per level.  Measured on the cloud (one table
// at 16-cell blocks against five per-level tables): 69.1 against 65.6 M
// paths/s (one table lookup per full query instead of 4.9, 1.41 gridlet
// tests instead of 1.08).
// element cells: at most 2^n cells (the cell width doubles from 2 finest
// units until the grid fits).  2^29 against 2^27 on the cloud: 75.2 against
// 71.2 M paths/s (narrower cells, shorter lists); the medium field is the
// same (295.0 against 295.2 M)
#ifndef EXA_ELEM_CELLS_LOG2
#define EXA_ELEM_CELLS_LOG2 29
#endif

// records a wavefront queue holds at most (walks in flight per round)
#ifndef EXA_WF_MAX_QUEUE
#define EXA_WF_MAX_QUEUE (1u << 22)
#endif

#ifndef EXA_TABLE_UNIFIED_MAX_SHIFT
#define EXA_TABLE_UNIFIED_MAX_SHIFT 4
#endif

void ExaStitchSampler::buildGridletTables(cudaStream_t s)
{
  const auto &G = model->gridlets;
  struct Tab { GridletTable t; std::vector<int32_t> entries, items; int minIdx, maxIdx; };
  // doubled extents of gridlet gi in the lattice of level lt, relative to
  // nothing (origin subtracted later)
  auto extent2 = [&](int gi, int lt, int64_t lo2[3], int64_t hi2[3]) {
    const exa_gridlet &g = G[gi];
    const int64_t r = (int64_t)1 << (g.level - lt);
    const int64_t gl[3] = {g.lower.x, g.lower.y, g.lower.z};
    const int64_t gd[3] = {std::max(g.dims.x, 1), std::max(g.dims.y, 1), std::max(g.dims.z, 1)};
    for (int a = 0; a < 3; ++a) {
      lo2[a] = (2 * gl[a] + 1) * r - 1;
      hi2[a] = (2 * (gl[a] + gd[a]) + 1) * r - 1;
    }
  };
  auto floorDiv = [](int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
  // blocks [b0, b1] of a table (lattice origin org, block width 2^shift)
  // whose open interiors meet the gridlet's interval
  auto blockRange = [&](int gi, int lt, const int org[3], int shift, int b0[3], int b1[3]) {
    int64_t lo2[3], hi2[3];
    extent2(gi, lt, lo2, hi2);
    const int64_t w2 = (int64_t)2 << shift;
    for (int a = 0; a < 3; ++a) {
      b0[a] = (int)floorDiv(lo2[a] - 2 * (int64_t)org[a], w2);
      b1[a] = (int)(floorDiv(hi2[a] - 2 * (int64_t)org[a] + w2 - 1, w2) - 1);
    }
  };
  auto makeTable = [&](const std::vector<int> &ids, int lt, int shift, Tab &T) {
    std::memset(&T.t, 0, sizeof(T.t));
    T.t.level = lt;
    T.t.shift = shift;
    T.minIdx = INT32_MAX;
    T.maxIdx = -1;
    int64_t lo[3] = {INT64_MAX, INT64_MAX, INT64_MAX}, hi[3] = {INT64_MIN, INT64_MIN, INT64_MIN};
    for (int gi : ids) {
      int64_t lo2[3], hi2[3];
      extent2(gi, lt, lo2, hi2);
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], floorDiv(lo2[a], 2));
        hi[a] = std::max(hi[a], floorDiv(hi2[a] + 1, 2));
      }
      T.minIdx = std::min(T.minIdx, gi);
      T.maxIdx = std::max(T.maxIdx, gi);
    }
    for (int a = 0; a < 3; ++a) {
      // blocks start on multiples of their width in the level's lattice, as
      // makeGrids' bricks do, so that a brick fills one block
      lo[a] = floorDiv(lo[a], (int64_t)1 << shift) * ((int64_t)1 << shift);
      if (lo[a] < INT32_MIN / 2 || hi[a] > INT32_MAX / 2) throw Error(EXA_ERR_INVALID, "gridlet lattice out of range");
      T.t.origin[a] = (int)lo[a];
      T.t.n[a] = (int)(((hi[a] - lo[a]) + (1ll << shift) - 1) >> shift) + 1;
    }
    const size_t nb = (size_t)T.t.n[0] * T.t.n[1] * T.t.n[2];
    // two passes over the listings (count, fill) into flat arrays; ids come
    // in ascending order, so every list is filled in ascending order
    auto forBlocks = [&](int gi, auto &&f) {
      int b0[3], b1[3];
      blockRange(gi, lt, T.t.origin, shift, b0, b1);
      for (int z = std::max(b0[2], 0); z <= std::min(b1[2], T.t.n[2] - 1); ++z)
        for (int y = std::max(b0[1], 0); y <= std::min(b1[1], T.t.n[1] - 1); ++y)
          for (int x = std::max(b0[0], 0); x <= std::min(b1[0], T.t.n[0] - 1); ++x)
            f(((size_t)z * T.t.n[1] + y) * T.t.n[0] + x);
    };
    std::vector<uint32_t> cnt(nb, 0u), cur(nb, 0u);
    for (int gi : ids) forBlocks(gi, [&](size_t b) { cnt[b]++; });
    T.entries.assign(nb, -1);
    size_t total = 0;
    for (size_t b = 0; b < nb; ++b)
      if (cnt[b] >= 2u) {
        T.entries[b] = -(int32_t)total - 2;
        cur[b] = (uint32_t)total + 1u;
        total += (size_t)cnt[b] + 1;
        if (total >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "gridlet table lists too long");
      }
    T.items.assign(total, 0);
    for (size_t b = 0; b < nb; ++b)
      if (cnt[b] >= 2u) T.items[cur[b] - 1u] = (int32_t)cnt[b];
    for (int gi : ids)
      forBlocks(gi, [&](size_t b) {
        if (cnt[b] == 1u) T.entries[b] = gi;
        else T.items[cur[b]++] = gi;
      });
    if (!std::is_sorted(ids.begin(), ids.end()))
      for (size_t b = 0; b < nb; ++b)
        if (T.entries[b] <= -2) {
          int32_t *L = T.items.data() + (-T.entries[b] - 2);
          std::sort(L + 1, L + 1 + L[0]);
        }
  };
  // smallest shift >= 3 whose block grid has at most 2^27 blocks
  auto pickShift = [&](const std::vector<int> &ids, int lt, int64_t &listed) {
    int64_t lo[3] = {INT64_MAX, INT64_MAX, INT64_MAX}, hi[3] = {INT64_MIN, INT64_MIN, INT64_MIN};
    for (int gi : ids) {
      int64_t lo2[3], hi2[3];
      extent2(gi, lt, lo2, hi2);
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], floorDiv(lo2[a], 2));
        hi[a] = std::max(hi[a], floorDiv(hi2[a] + 1, 2));
      }
    }
    int shift = 3;
    // (origins aligned to the block width, as makeTable places them)
    auto alignedLo = [&](int sh, int a) { return floorDiv(lo[a], (int64_t)1 << sh) * ((int64_t)1 << sh); };
    auto blocks = [&](int sh, int a) { return ((hi[a] - alignedLo(sh, a)) + (1ll << sh) - 1) / (1ll << sh) + 1; };
    while (blocks(shift, 0) * blocks(shift, 1) * blocks(shift, 2) > (1ll << 27) && shift < 20) shift++;
    const int org[3] = {(int)std::max<int64_t>(alignedLo(shift, 0), INT32_MIN / 2),
                        (int)std::max<int64_t>(alignedLo(shift, 1), INT32_MIN / 2),
                        (int)std::max<int64_t>(alignedLo(shift, 2), INT32_MIN / 2)};
    listed = 0;
    for (int gi : ids) {
      int b0[3], b1[3];
      blockRange(gi, lt, org, shift, b0, b1);
      listed += (int64_t)(b1[0] - b0[0] + 1) * (b1[1] - b0[1] + 1) * (b1[2] - b0[2] + 1);
    }
    return shift;
  };

  std::map<int, std::vector<int>> byLevel;
  for (size_t i = 0; i < G.size(); ++i) {
    if (G[i].level < 0 || G[i].level > 30) throw Error(EXA_ERR_INVALID, "gridlet level out of range");
    byLevel[G[i].level].push_back((int)i);
  }
  std::vector<Tab> tabs;
  bool unified = false;
  if (byLevel.size() > 1) {
    std::vector<int> all(G.size());
    for (size_t i = 0; i < G.size(); ++i) all[i] = (int)i;
    const int lmin = byLevel.begin()->first;
    int64_t listed = 0;
    const int shift = pickShift(all, lmin, listed);
    // one table when its blocks stay at most 2^EXA_TABLE_UNIFIED_MAX_SHIFT
    // finest dual cells wide and the lists stay modest next to the gridlets
    // themselves
    if (shift <= EXA_TABLE_UNIFIED_MAX_SHIFT && listed <= std::max<int64_t>(64 * (int64_t)G.size(), 1 << 20) &&
        listed < (1ll << 28)) {
      Tab T;
      makeTable(all, lmin, shift, T);
      tabs.push_back(std::move(T));
      unified = true;
    }
  }
  if (!unified) {
    if ((int)byLevel.size() > kMaxLevels) throw Error(EXA_ERR_INVALID, "more than 16 gridlet levels");
    for (auto &kv : byLevel) {
      int64_t listed = 0;
      const int shift = pickShift(kv.second, kv.first, listed);
      Tab T;
      makeTable(kv.second, kv.first, shift, T);
      tabs.push_back(std::move(T));
    }
  }
  std::sort(tabs.begin(), tabs.end(), [](const Tab &a, const Tab &b) { return a.minIdx < b.minIdx; });
  bool sorted = true;
  for (size_t i = 1; i < tabs.size(); ++i)
    if (tabs[i].minIdx <= tabs[i - 1].maxIdx) sorted = false;
  tableEntries.clear();
  tableItems.clear();
  tableEntries.resize(tabs.size());
  tableItems.resize(tabs.size());
  accel.numTables = (int)tabs.size();
  accel.tablesSorted = sorted ? 1 : 0;
  for (size_t i = 0; i < tabs.size(); ++i) {
    tableEntries[i].upload(tabs[i].entries.data(), tabs[i].entries.size(), s);
    if (tabs[i].items.empty()) tabs[i].items.push_back(0);
    tableItems[i].upload(tabs[i].items.data(), tabs[i].items.size(), s);
    accel.tables[i] = tabs[i].t;
    accel.tables[i].entries = tableEntries[i].ptr;
    accel.tables[i].items = tableItems[i].ptr;
    accel.tables[i].numItems = (int)tabs[i].items.size();
  }
}

void ExaStitchSampler::buildElementCells(cudaStream_t s)
{
  const size_t ne = model->indices.size() / 8;
  accel.numElems = (int)ne;
  exa_box3f sb;
  sb.lower = {INFINITY, INFINITY, INFINITY};
  sb.upper = {-INFINITY, -INFINITY, -INFINITY};
  for (const exa_vec4f &v : model->vertices) {
    sb.lower.x = std::min(sb.lower.x, v.x); sb.upper.x = std::max(sb.upper.x, v.x);
    sb.lower.y = std::min(sb.lower.y, v.y); sb.upper.y = std::max(sb.upper.y, v.y);
    sb.lower.z = std::min(sb.lower.z, v.z); sb.upper.z = std::max(sb.upper.z, v.z);
  }
  if (!ne) sb.lower = sb.upper = exa_vec3f{0.f, 0.f, 0.f};
  // cell grid: about 2 finest-cell widths per cell, at most 2^EXA_ELEM_CELLS_LOG2 cells
  ElemOccupancy &O = accel.occ;
  const float ext[3] = {sb.upper.x - sb.lower.x, sb.upper.y - sb.lower.y, sb.upper.z - sb.lower.z};
  const float org[3] = {sb.lower.x, sb.lower.y, sb.lower.z};
  float cs = 2.f;
  auto cells = [&](float c) {
    double t = 1;
    for (int a = 0; a < 3; ++a) t *= std::max(1.0, std::ceil((double)ext[a] / c) + 1);
    return t;
  };
  while (cells(cs) > (double)(1ull << EXA_ELEM_CELLS_LOG2)) cs *= 2.f;
  for (int a = 0; a < 3; ++a) {
    O.origin[a] = org[a];
    O.invCell[a] = 1.f / cs;  // exact: cs is a power of two
    O.n[a] = (int)std::max(1.0, std::ceil((double)ext[a] / cs) + 1);
  }
  launchElemCells(vertexBuffer.ptr, indexBuffer.ptr, ne, O, occBits, occRank, occEntries, occItems, elemBoxes, s);
}

// CUDA events recorded on a stream; times between them once it has synchronised
struct StreamTimer {
  std::vector<cudaEvent_t> ev;
  cudaStream_t s;
  StreamTimer(int n, cudaStream_t st) : ev((size_t)n, nullptr), s(st)
  {
    for (auto &e : ev) cudaCheck(cudaEventCreate(&e), "cudaEventCreate");
  }
  ~StreamTimer()
  {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
  void mark(int i) { cudaCheck(cudaEventRecord(ev[(size_t)i], s), "cudaEventRecord"); }
  float ms(int a, int b) const
  {
    float t = 0.f;
    cudaCheck(cudaEventElapsedTime(&t, ev[(size_t)a], ev[(size_t)b]), "cudaEventElapsedTime");
    return t;
  }
};

// the build kernels' error bits, read after the build's stream synchronised
static void checkBuildErrors(const uint32_t *dev)
{
  uint32_t e = 0;
  if (dev) cudaCheck(cudaMemcpy(&e, dev, sizeof(e), cudaMemcpyDeviceToHost), "read build errors");
  if (e & EXA_DEVERR_COPY_WAIT)
    throw Error(EXA_ERR_CUDA, "majorant build: a bulk copy into shared memory did not complete");
}

// sampler/ExaStitchSampler.cpp:23-340
bool ExaStitchSampler::build(std::shared_ptr<Model> mod, cudaStream_t s)
{
  if (!mod) return false;
  model = std::dynamic_pointer_cast<ExaStitchModel>(mod);
  if (!model) return false;
  if (model->gridlets.empty() && model->indices.empty()) return false;
  if (!model->grid || model->grid->dims.x == 0) return false;
  std::memset(&accel, 0, sizeof(accel));
  // gridlet geometry
  gridletBuffer.upload(model->gridlets.data(), model->gridlets.size(), s);
  gridletScalarBuffer.upload(model->gridletScalars.data(), model->gridletScalars.size(), s);
  gridletValueRanges.alloc(model->gridlets.size());
  gridletMaxOpacities.alloc(model->gridlets.size());
  // stitching geometry
  static_assert(sizeof(float4) == sizeof(exa_vec4f), "vec4f layout");
  vertexBuffer.upload(reinterpret_cast<const float4 *>(model->vertices.data()), model->vertices.size(), s);
  indexBuffer.upload(model->indices.data(), model->indices.size(), s);
  elemValueRanges.alloc(model->indices.size() / 8);
  umeshMaxOpacities.alloc(model->indices.size() / 8);
  accel.gridlets = gridletBuffer.ptr;
  accel.scalars = gridletScalarBuffer.ptr;
  accel.vertices = vertexBuffer.ptr;
  accel.indices = indexBuffer.ptr;
  accel.numGridlets = (int)model->gridlets.size();
  buildGridletTables(s);
  buildElementCells(s);
  // the majorant grid (Grid::build, Grid.cu:457-594) over cellBounds
  Grid &g = *model->grid;
  g.worldBounds = model->cellBounds;
  const size_t numMCs = (size_t)g.dims.x * g.dims.y * g.dims.z;
  g.valueRanges.alloc(numMCs);
  g.maxOpacities.alloc(numMCs);
  cudaCheck(cudaMemsetAsync(g.maxOpacities.ptr, 0, g.maxOpacities.bytes(), s), "memset maxOpacities");
  launchInitRanges(g.valueRanges.ptr, numMCs, s);
  launchInitRanges(gridletValueRanges.ptr, gridletValueRanges.count, s);
  if (!buildErrors.ptr) buildErrors.alloc(1);
  cudaCheck(cudaMemsetAsync(buildErrors.ptr, 0, sizeof(uint32_t), s), "memset build errors");
  StreamTimer timer(3, s);
  timer.mark(0);
  launchElemMajorants(vertexBuffer.ptr, indexBuffer.ptr, model->indices.size() / 8, g.dims, g.worldBounds,
                      g.valueRanges.ptr, elemValueRanges.ptr, s);
  timer.mark(1);
  buildStats = {};
  majorantScratch.alloc(model->gridlets.size() + 1);
  buildStats.majorantBlocks =
      launchGridletMajorants(gridletBuffer.ptr, gridletScalarBuffer.ptr, model->gridlets.size(),
                             model->gridletScalars.size(), g.dims, g.worldBounds, g.valueRanges.ptr,
                             gridletValueRanges.ptr, buildErrors.ptr, debugFlags, majorantScratch.ptr, s);
  timer.mark(2);
  g.deviceTraversable.dims = g.dims;
  g.deviceTraversable.bounds = g.worldBounds;
  deviceAccel.alloc(1);
  cudaCheck(cudaMemcpyAsync(deviceAccel.ptr, &accel, sizeof(accel), cudaMemcpyHostToDevice, s), "accel handle");
  cudaCheck(cudaStreamSynchronize(s), "sampler build");
  checkBuildErrors(buildErrors.ptr);
  buildStats.elemMajorantMs = timer.ms(0, 1);
  buildStats.gridletMajorantMs = timer.ms(1, 2);
  majorantAccel.grid = model->grid;
  maxOpacities = g.maxOpacities.ptr;
  hasTF = false;
  return true;
}

// sampler/ExaStitchSampler.cu:279-376 + Grid::computeMaxOpacities
void ExaStitchSampler::computeMaxOpacities(const exa_vec4f *cmap, int numColors, exa_range1f xf, cudaStream_t s)
{
  if (!model || !model->grid || model->grid->dims.x == 0) return;
  if (numColors <= 0) throw Error(EXA_ERR_INVALID, "empty color map");
  colorMap.upload(reinterpret_cast<const float4 *>(cmap), (size_t)numColors, s);
  Grid &g = *model->grid;
  launchMaxOpacity(g.valueRanges.ptr, g.valueRanges.count, colorMap.ptr, numColors, xf, tfFilter, g.maxOpacities.ptr, s);
  launchMaxOpacity(gridletValueRanges.ptr, gridletValueRanges.count, colorMap.ptr, numColors, xf, tfFilter,
                   gridletMaxOpacities.ptr, s);
  launchMaxOpacity(elemValueRanges.ptr, elemValueRanges.count, colorMap.ptr, numColors, xf, tfFilter, umeshMaxOpacities.ptr,
                   s);
  accel.gridletMaxOps = gridletMaxOpacities.ptr;
  accel.elemMaxOps = umeshMaxOpacities.ptr;
  cudaCheck(cudaMemcpyAsync(deviceAccel.ptr, &accel, sizeof(accel), cudaMemcpyHostToDevice, s), "accel handle");
  cudaCheck(cudaStreamSynchronize(s), "computeMaxOpacities");
  hasTF = true;
}

// sampler/ExaStitchSampler.cpp:356-365
void ExaStitchSampler::setLPs(exa_launch_params &lp)
{
  lp.sampler.ess.sampleBVH = (uint64_t)(uintptr_t)deviceAccel.ptr;
  lp.sampler.ess.gridletBuffer = gridletBuffer.ptr;
  lp.sampler.ess.gridletScalarBuffer = gridletScalarBuffer.ptr;
}

// ================================================================ AMR cells
// model/AMRCellModel.cpp:56-64 (bounds and value range of the loaded cells)
void AMRCellModel::assign(const exa_amr_cell *c, size_t nc, const float *s, size_t ns)
{
  if (ns < nc) throw Error(EXA_ERR_INVALID, "fewer scalars than AMR cells");
  cells.assign(c, c + nc);
  scalars.assign(s, s + ns);
  exa_box3f b;
  b.lower = {INFINITY, INFINITY, INFINITY};
  b.upper = {-INFINITY, -INFINITY, -INFINITY};
  exa_range1f r{1e30f, -1e30f};
  for (size_t i = 0; i < nc; ++i) {
    const exa_amr_cell &a = cells[i];
    if (a.level < 0 || a.level > 30) throw Error(EXA_ERR_INVALID, "AMR cell level out of range");
    const int64_t w = 1ll << a.level;
    const int64_t p[3] = {a.pos.x, a.pos.y, a.pos.z};
    for (int k = 0; k < 3; ++k) {
      if (p[k] % w != 0) throw Error(EXA_ERR_INVALID, "AMR cell position is not a multiple of its width");
      if (p[k] + w > 0x7fffffffll) throw Error(EXA_ERR_INVALID, "AMR cell position out of range");
    }
    const float lo[3] = {(float)a.pos.x, (float)a.pos.y, (float)a.pos.z};
    const float hi[3] = {(float)(a.pos.x + (int32_t)w), (float)(a.pos.y + (int32_t)w), (float)(a.pos.z + (int32_t)w)};
    b.lower = {std::min(b.lower.x, lo[0]), std::min(b.lower.y, lo[1]), std::min(b.lower.z, lo[2])};
    b.upper = {std::max(b.upper.x, hi[0]), std::max(b.upper.y, hi[1]), std::max(b.upper.z, hi[2])};
    const float v = scalars[i];
    if (!std::isnan(v)) {
      r.lower = std::min(r.lower, v);
      r.upper = std::max(r.upper, v);
    }
  }
  cellBounds = b;
  valueRange = r;
}

void AMRCellModel::memStats(size_t &cellsBytes, size_t &scalarsBytes) const
{
  cellsBytes = cells.size() * sizeof(exa_amr_cell);
  scalarsBytes = cells.empty() ? 0 : scalars.size() * sizeof(float);
}

size_t AMRCellSampler::fieldBytes() const { return cellBuffer.bytes() + scalarBuffer.bytes(); }

size_t AMRCellSampler::accelBytes() const
{
  size_t b = deviceView.bytes();
  for (auto &x : levelBits) b += x.bytes();
  for (auto &x : levelRank) b += x.bytes();
  for (auto &x : levelCell) b += x.bytes();
  return b;
}

// sampler/AMRCellSampler.cpp:23-108: the cells on the device, their point
// location (dense per-level lattices instead of the OptiX user-geometry
// BVH) and the majorant grid over cellBounds (Grid::build, Grid.cu:314-364)
bool AMRCellSampler::build(std::shared_ptr<Model> mod, cudaStream_t s)
{
  if (!mod) return false;
  model = std::dynamic_pointer_cast<AMRCellModel>(mod);
  if (!model || model->cells.empty()) return false;
  if (!model->grid || model->grid->dims.x == 0) return false;
  const size_t n = model->cells.size();
  cellBuffer.upload(model->cells.data(), n, s);
  scalarBuffer.upload(model->scalars.data(), model->scalars.size(), s);
  // per-level lattice boxes (host pass over the cells)
  int lo[kMaxLevels][3], hi[kMaxLevels][3];
  bool has[kMaxLevels] = {};
  int maxLevel = 0;
  for (const exa_amr_cell &c : model->cells) {
    if (c.level >= kMaxLevels) throw Error(EXA_ERR_INVALID, "AMR cell level above 15");
    const int L = c.level;
    const int q[3] = {c.pos.x >> L, c.pos.y >> L, c.pos.z >> L};
    for (int a = 0; a < 3; ++a) {
      lo[L][a] = has[L] ? std::min(lo[L][a], q[a]) : q[a];
      hi[L][a] = has[L] ? std::max(hi[L][a], q[a]) : q[a];
    }
    has[L] = true;
    maxLevel = std::max(maxLevel, L);
  }
  std::memset(&view, 0, sizeof(view));
  view.numLevels = maxLevel + 1;
  view.scalars = scalarBuffer.ptr;
  levelBits.clear();
  levelRank.clear();
  levelCell.clear();
  levelBits.resize(view.numLevels);
  levelRank.resize(view.numLevels);
  levelCell.resize(view.numLevels);
  DBuf<unsigned> dup;
  dup.alloc(1);
  cudaCheck(cudaMemsetAsync(dup.ptr, 0, sizeof(unsigned), s), "memset");
  uint64_t totalBits = 0;
  for (int L = 0; L < view.numLevels; ++L) {
    if (!has[L]) continue;
    int nl[3];
    uint64_t bits = 1;
    for (int a = 0; a < 3; ++a) {
      nl[a] = hi[L][a] - lo[L][a] + 1;
      bits *= (uint64_t)nl[a];
    }
    totalBits += bits;
    if (totalBits > (1ull << 37))
      throw Error(EXA_ERR_INVALID, "AMR cells too sparse for the dense per-level lattices");
    const size_t words = (size_t)((bits + 31) / 32);
    levelBits[L].alloc(words);
    levelRank[L].alloc(words);
    cudaCheck(cudaMemsetAsync(levelBits[L].ptr, 0, levelBits[L].bytes(), s), "memset bits");
    launchAmrLevelBits(cellBuffer.ptr, n, L, lo[L], nl, levelBits[L].ptr, dup.ptr, s);
    launchAmrLevelRank(levelBits[L].ptr, words, levelRank[L].ptr, s);
    size_t count = 0;
    for (const exa_amr_cell &c : model->cells) count += c.level == L;
    levelCell[L].alloc(count);
    launchAmrLevelCells(cellBuffer.ptr, n, L, lo[L], nl, levelBits[L].ptr, levelRank[L].ptr, levelCell[L].ptr, s);
    AmrLevel &V = view.lv[L];
    for (int a = 0; a < 3; ++a) {
      V.lo[a] = lo[L][a];
      V.n[a] = nl[a];
    }
    V.bits = levelBits[L].ptr;
    V.rank = levelRank[L].ptr;
    V.cell = levelCell[L].ptr;
  }
  unsigned dupHost = 0;
  cudaCheck(cudaMemcpyAsync(&dupHost, dup.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "dup flag");
  cudaCheck(cudaStreamSynchronize(s), "amr lattices");
  if (dupHost) throw Error(EXA_ERR_INVALID, "duplicate AMR cell");
  deviceView.upload(&view, 1, s);
  std::memset(&accel, 0, sizeof(accel));
  accel.amr = deviceView.ptr;
  // the majorant grid over cellBounds (Grid.cu:314-364)
  Grid &g = *model->grid;
  g.worldBounds = model->cellBounds;
  const size_t numMCs = (size_t)g.dims.x * g.dims.y * g.dims.z;
  g.valueRanges.alloc(numMCs);
  g.maxOpacities.alloc(numMCs);
  cudaCheck(cudaMemsetAsync(g.maxOpacities.ptr, 0, g.maxOpacities.bytes(), s), "memset maxOpacities");
  launchInitRanges(g.valueRanges.ptr, numMCs, s);
  launchAmrCellMajorants(cellBuffer.ptr, scalarBuffer.ptr, n, g.dims, g.worldBounds, g.valueRanges.ptr, s);
  g.deviceTraversable.dims = g.dims;
  g.deviceTraversable.bounds = g.worldBounds;
  deviceAccel.alloc(1);
  cudaCheck(cudaMemcpyAsync(deviceAccel.ptr, &accel, sizeof(accel), cudaMemcpyHostToDevice, s), "accel handle");
  cudaCheck(cudaStreamSynchronize(s), "sampler build");
  majorantAccel.grid = model->grid;
  maxOpacities = g.maxOpacities.ptr;
  hasTF = false;
  return true;
}

// AMRCellSampler.cpp:112-118 (Grid::computeMaxOpacities)
void AMRCellSampler::computeMaxOpacities(const exa_vec4f *cmap, int numColors, exa_range1f xf, cudaStream_t s)
{
  if (!model || !model->grid || model->grid->dims.x == 0) return;
  if (numColors <= 0) throw Error(EXA_ERR_INVALID, "empty color map");
  colorMap.upload(reinterpret_cast<const float4 *>(cmap), (size_t)numColors, s);
  Grid &g = *model->grid;
  launchMaxOpacity(g.valueRanges.ptr, g.valueRanges.count, colorMap.ptr, numColors, xf, tfFilter, g.maxOpacities.ptr, s);
  cudaCheck(cudaStreamSynchronize(s), "computeMaxOpacities");
  hasTF = true;
}

// AMRCellSampler.cpp:133-140
void AMRCellSampler::setLPs(exa_launch_params &lp)
{
  std::memset(&lp.sampler, 0, sizeof(lp.sampler));
  lp.sampler.acs.sampleBVH = (uint64_t)(uintptr_t)deviceAccel.ptr;
}

} // namespace exa

// ================================================================ C ABI
using namespace exa;

struct exa_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool ownStream = false;
  std::shared_ptr<Model> model;
  std::shared_ptr<Sampler> sampler;
  exa_range1f xfRange{0.f, 1.f};
  int numColors = 0;
  int tfFilter = EXA_TF_FILTER_NEAREST;  // for the next computeMaxOpacities
  int renderPath = EXA_RENDER_PATH_AUTO; // exa_set_render_path
  uint32_t debugFlags = 0;               // EXA_DEBUG_*, for the next sampler build
  DBuf<uint32_t> errors;
  DBuf<unsigned> jobCounter; // work counter of the persistent render kernel
  DBuf<float4> sampleColors; // one colour per camera sample of the frame
  DBuf<uint32_t> wfRecords;  // wavefront path records: 3 queues x 60 words x capacity
  DBuf<unsigned> wfCounters; // wavefront queue sizes
  unsigned wfCap = 0;
  exa_render_stats lastStats{};
  exa_build_stats lastBuild{};
  DBuf<exa_vec3f> hostPos;   // staging for exa_sample_points_host
  DBuf<exa_sample> hostOut;
  DBuf<uint32_t> heat;       // heat map: per-pixel work of the frame
  std::unique_ptr<Surrogate> surrogate;
  float surrogateTol = 0.f;
  std::unique_ptr<struct BatchState> batch;
  std::unique_ptr<struct MeshState> mesh;
};

// the context's surface mesh: float4 vertices, 8-int triangle rows (a, b, c,
// then -1: the LBVH builder's row format), its BVH and the device
// copy of the view the kernels trace
struct MeshState {
  DBuf<float4> vertices;
  DBuf<int32_t> indices;
  DBuf<BvhNode> nodes;
  DBuf<int32_t> parents, leafElem;
  DBuf<MeshView> view;
  exa_box3f bounds{};
};

// state of exa_render_batch: transfer functions, the batch's majorant grid,
// per-transfer-function culling data, frame tables, scratch and the cached
// CUDA graph
struct BatchState {
  std::vector<DBuf<float4>> tfColors;
  std::vector<int> tfCount;
  std::vector<exa_range1f> tfRange;
  std::vector<float> tfScale;
  exa_vec3i dims{0, 0, 0};
  DBuf<exa_range1f> ranges;
  std::vector<DBuf<float>> maxOps;  // per transfer function, on dims
  // per transfer function: primitive max opacities and the point-location
  // view that culls by them
  std::vector<DBuf<float>> gOps, eOps;
  DBuf<AccelView> accels;
  int tileW = 16;
  DBuf<exa_launch_params> lps;
  DBuf<WfFrame> frames;
  DBuf<WfCtl> ctl;
  DBuf<float4> colors;
  DBuf<uint32_t> records;
  DBuf<unsigned> counters;
  unsigned cap = 0;
  BatchGraph graph;
  WfStats last;
};

namespace {
thread_local std::string g_lastError;

template <typename F>
int guarded(F &&f)
{
  try {
    f();
    g_lastError.clear();
    return EXA_OK;
  } catch (const Error &e) {
    g_lastError = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_lastError = "host allocation failed";
    return EXA_ERR_OOM;
  } catch (const std::exception &e) {
    g_lastError = e.what();
    return EXA_ERR_INVALID;
  }
}

void need(bool c, int code, const char *msg)
{
  if (!c) throw Error(code, msg);
}

void setDevice(exa_context *ctx) { cudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice"); }

// the launch parameters' filter and loop caps: the filter must be the one
// the max opacities were computed for (else they may not bound the
// filtered opacity); the caps are non-negative
void needLpCaps(const exa_launch_params &lp, int samplerFilter)
{
  need(lp.ext.tfFilter == samplerFilter, EXA_ERR_INVALID,
       "lp.ext.tfFilter differs from the filter of the max opacities (call exa_sampler_set_lps)");
  need(lp.ext.trackStepCap >= 0 && lp.ext.ddaCellCap >= 0, EXA_ERR_INVALID, "negative loop cap");
}

// the DDA indexes lp.maxOpacities by the cells of lp.majorantGrid: its dims
// must be those of the grid the sampler built (exa_sampler_set_lps copies
// them), else the walks would read past the max opacities
void needGridDims(const exa_context *ctx, const exa_launch_params &lp)
{
  const exa_vec3i g = ctx->model && ctx->model->grid ? ctx->model->grid->dims : exa_vec3i{0, 0, 0};
  need(lp.majorantGrid.dims.x == g.x && lp.majorantGrid.dims.y == g.y && lp.majorantGrid.dims.z == g.z,
       EXA_ERR_INVALID, "lp.majorantGrid.dims are not the built majorant grid's (call exa_sampler_set_lps)");
}

// the context's model / sampler where a call needs the ExaStitch kind
ExaStitchModel &esModel(exa_context *ctx)
{
  auto *m = dynamic_cast<ExaStitchModel *>(ctx->model.get());
  need(m != nullptr, EXA_ERR_STATE, "this call needs an ExaStitch model");
  return *m;
}

ExaStitchSampler &esSampler(exa_context *ctx)
{
  auto *s = dynamic_cast<ExaStitchSampler *>(ctx->sampler.get());
  need(s != nullptr, EXA_ERR_STATE, "this call needs an ExaStitch sampler");
  return *s;
}
} // namespace

namespace {
void renderFrame(exa_context *ctx, const exa_launch_params *lp, int32_t width, int32_t height, bool learned)
{
  {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(lp != nullptr, EXA_ERR_INVALID, "null lp");
    need(width > 0 && height > 0, EXA_ERR_INVALID, "bad frame size");
    need(lp->render.spp >= 1, EXA_ERR_INVALID, "spp must be >= 1");
    need((long long)((width + 15) / 16) * ((height + 7) / 8) * 128 * lp->render.spp < 0xffffffffll, EXA_ERR_INVALID,
         "frame too large: width*height*spp must stay below 2^32 samples per launch");
    need(lp->integrator == EXA_PATH_TRACING_INTEGRATOR || lp->integrator == EXA_DIRECT_LIGHT_INTEGRATOR ||
             (lp->integrator == EXA_RAY_MARCHING_INTEGRATOR && !learned),
         EXA_ERR_INVALID, "integrator not supported");
    need(lp->integrator != EXA_RAY_MARCHING_INTEGRATOR || (lp->render.dt > 0.f && std::isfinite(lp->render.dt)),
         EXA_ERR_INVALID, "ray marching needs render.dt > 0");
    need(lp->shadeMode == EXA_SHADE_MODE_DEFAULT || lp->shadeMode == EXA_SHADE_MODE_GRIDLETS ||
             lp->shadeMode == EXA_SHADE_MODE_TEASER,
         EXA_ERR_INVALID, "shade mode not supported");
    // the non-wavefront build renders path tracing and direct lighting
    // without these (the ray marcher and the wavefront renderer have them)
    const bool wavefrontOrMarch = useWavefront() || learned || lp->integrator == EXA_RAY_MARCHING_INTEGRATOR;
    need(wavefrontOrMarch || (!lp->subImage.active && !lp->render.heatMapEnabled &&
                              lp->shadeMode != EXA_SHADE_MODE_TEASER),
         EXA_ERR_INVALID, "sub-image, heat map and the teaser shade mode need the wavefront renderer");
    need(lp->meshBVH == 0 || (ctx->mesh && lp->meshBVH == (uint64_t)(uintptr_t)ctx->mesh->view.ptr), EXA_ERR_INVALID,
         "lp.meshBVH is not this context's mesh (call exa_mesh_set and exa_sampler_set_lps)");
    need(lp->meshBVH == 0 || useWavefront() || learned || lp->integrator == EXA_RAY_MARCHING_INTEGRATOR,
         EXA_ERR_INVALID, "surface meshes need the wavefront renderer");
    need(lp->sampler.ess.sampleBVH == (uint64_t)(uintptr_t)ctx->sampler->deviceAccel.ptr, EXA_ERR_INVALID,
         "lp.sampler.ess.sampleBVH is not this context's sampler (call exa_sampler_set_lps)");
    need(lp->maxOpacities != nullptr && lp->transferFunc.values != nullptr, EXA_ERR_STATE,
         "no transfer function (call exa_sampler_compute_max_opacities and exa_sampler_set_lps)");
    need(lp->ext.maxBounces >= 0, EXA_ERR_INVALID, "maxBounces must be >= 0");
    needLpCaps(*lp, ctx->sampler->tfFilter);
    needGridDims(ctx, *lp);
    if (lp->ext.rowEnd > 0) {
      need(lp->ext.rowBegin >= 0 && lp->ext.rowBegin % 8 == 0 && lp->ext.rowBegin < lp->ext.rowEnd &&
               lp->ext.rowEnd <= height && (lp->ext.rowEnd % 8 == 0 || lp->ext.rowEnd == height),
           EXA_ERR_INVALID, "row band: need 0 <= rowBegin < rowEnd <= height, rowBegin a multiple of 8, rowEnd a "
                            "multiple of 8 or the height");
      need((useWavefront() || learned) && lp->integrator != EXA_RAY_MARCHING_INTEGRATOR, EXA_ERR_INVALID,
           "row bands need the wavefront renderer (path tracing or direct lighting)");
    }
    // the AMR-cell and ExaBrick samplers render shade mode default
    // (renderFrame_AMRCellSampler / _ExaBrickSampler, deviceCode.cu:1360-1387)
    need((ctx->sampler->accel.amr == nullptr && ctx->sampler->accel.bricks == nullptr) ||
             (lp->shadeMode == EXA_SHADE_MODE_DEFAULT && !learned),
         EXA_ERR_INVALID, "the AMR-cell and ExaBrick samplers render shade mode default with the exact field only");
    setDevice(ctx);
    const size_t ns = (size_t)width * height * (size_t)lp->render.spp;
    if (ctx->sampleColors.count < ns) ctx->sampleColors.alloc(ns);
    exa_launch_params lpUse = *lp;
    fillLoopCaps(lpUse);
    lpUse.ext.heatCounts = nullptr;
    if (lp->render.heatMapEnabled) {
      // per-pixel work of this frame for the heat map
      if (ctx->heat.count < (size_t)width * height) ctx->heat.alloc((size_t)width * height);
      cudaCheck(cudaMemsetAsync(ctx->heat.ptr, 0, (size_t)width * height * sizeof(uint32_t), ctx->stream), "heat");
      lpUse.ext.heatCounts = ctx->heat.ptr;
    }
    SurrogateView sv{};
    if (learned) {
      Surrogate *S = ctx->surrogate.get();
      need(S && S->evaluated, EXA_ERR_STATE, "no evaluated surrogate (call exa_surrogate_evaluate)");
      const exa_vec3i d = ctx->model->grid->dims;
      need(d.x == S->evalDims.x && d.y == S->evalDims.y && d.z == S->evalDims.z, EXA_ERR_STATE,
           "majorant grid changed since exa_surrogate_evaluate");
      need(lp->shadeMode == EXA_SHADE_MODE_DEFAULT, EXA_ERR_INVALID, "the learned field renders shade mode default only");
      lpUse.maxOpacities = S->majorants.ptr;
      sv = S->deviceView();
    }
    // the single-launch renderer (a thread per sample) takes frames of at
    // most one wave of samples: it saves the wavefront's rounds, whose
    // launches dominate such frames (a 256^2 x 1 spp direct-light frame:
    // 0.26 against 0.46 ms); frames with the features only the wavefront
    // renderer draws stay there
    const bool singleAble = !learned && !lpUse.meshBVH && lpUse.shadeMode == EXA_SHADE_MODE_DEFAULT &&
                            !lpUse.render.heatMapEnabled && lpUse.ext.rowEnd <= 0;
    bool wavefront = useWavefront() || learned;
    if (singleAble && ctx->renderPath == EXA_RENDER_PATH_SINGLE_LAUNCH) wavefront = false;
    if (singleAble && ctx->renderPath == EXA_RENDER_PATH_AUTO && wavefront) {
      int dev = 0, sms = 152;
      cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
      cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
      const size_t jobs = (size_t)((width + 15) / 16) * ((height + 7) / 8) * 128 * (size_t)lp->render.spp;
      if (jobs <= (size_t)sms * 4 * 128) wavefront = false;
    }
    if (ctx->renderPath == EXA_RENDER_PATH_WAVEFRONT) wavefront = true;
    if (wavefront && lpUse.integrator != EXA_RAY_MARCHING_INTEGRATOR) {
      // queue capacity: the frame's samples, at most 4M records in flight
      const unsigned cap = (unsigned)std::min<size_t>((size_t)((width + 15) / 16) * ((height + 7) / 8) * 128 *
                                                          (size_t)lp->render.spp, (size_t)EXA_WF_MAX_QUEUE);
      if (ctx->wfCap < cap) {
        ctx->wfRecords.alloc((size_t)3 * kWfLaneWords * cap);
        ctx->wfCounters.alloc(kWfCounterWords);
        ctx->wfCap = cap;
      }
      WfStats st;
      renderWavefront(ctx->sampler->accel, lpUse, width, height, ctx->sampleColors.ptr, ctx->wfRecords.ptr, ctx->wfCap,
                      ctx->wfCounters.ptr, ctx->stream, &st, learned ? &sv : nullptr);
      ctx->lastStats.wavefront = 1;
      ctx->lastStats.rounds = st.rounds;
      ctx->lastStats.peakQueue = st.peakQueue;
      ctx->lastStats.queueCapacity = ctx->wfCap;
      ctx->lastStats.walkLaunches = st.walkLaunches;
      ctx->lastStats.cameraMs = st.cameraMs;
      ctx->lastStats.walkMs = st.walkMs;
      ctx->lastStats.eventMs = st.eventMs;
      ctx->lastStats.kernelLaunches = st.kernelLaunches;
    } else {
      ctx->lastStats = exa_render_stats{};
      ctx->lastStats.kernelLaunches = 2;  // the single launch and the resolve
      launchRender(ctx->sampler->accel, lpUse, width, height, ctx->jobCounter.ptr, ctx->sampleColors.ptr,
                   ctx->stream);
    }
  }
}

}  // namespace

extern "C" {

const char *exa_version(void) { return "exastitch-gb300 0.1 (sm_103a)"; }

uint64_t exa_abi_sizeof(int32_t which)
{
  switch (which) {
    case 0: return sizeof(exa_launch_params);
    case 1: return sizeof(exa_gridlet);
    case 2: return sizeof(exa_sample);
    case 3: return sizeof(exa_mem_stats);
    case 4: return sizeof(exa_lp_ext);
    case 5: return sizeof(exa_surrogate_params);
    case 6: return sizeof(exa_surrogate_stats);
    case 7: return sizeof(exa_surrogate_geometry);
    case 8: return sizeof(exa_batch_frame);
    case 9: return sizeof(exa_batch_tuning);
    case 10: return sizeof(exa_xf);
    case 11: return sizeof(exa_amr_cell);
    case 12: return sizeof(exa_render_stats);
    case 13: return sizeof(exa_build_stats);
    case 14: return sizeof(exa_brick);
    case 15: return sizeof(exa_abr);
    default: return 0;
  }
}

const char *exa_last_error(void) { return g_lastError.c_str(); }

const char *exa_sampler_class_name(void) { return "ExaStitchSampler"; }

const char *exa_sampler_get_class_name(exa_context *ctx)
{
  if (!ctx || !ctx->sampler) return "";
  if (dynamic_cast<AMRCellSampler *>(ctx->sampler.get())) return "AMRCellSampler";
  if (dynamic_cast<ExaBrickSampler *>(ctx->sampler.get())) return "ExaBrickSampler";
  return "ExaStitchSampler";
}

int exa_context_create(exa_context **out, int device, uint64_t stream)
{
  return guarded([&] {
    need(out != nullptr, EXA_ERR_INVALID, "out is null");
    int n = 0;
    cudaCheck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    need(device >= 0 && device < n, EXA_ERR_INVALID, "device index out of range");
    std::unique_ptr<exa_context> c(new exa_context());
    c->device = device;
    cudaCheck(cudaSetDevice(device), "cudaSetDevice");
    if (stream != EXA_STREAM_PRIVATE) {
      c->stream = reinterpret_cast<cudaStream_t>(stream);
    } else {
      cudaCheck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
      c->ownStream = true;
    }
    c->errors.alloc(1);
    c->jobCounter.alloc(1);
    cudaCheck(cudaMemsetAsync(c->errors.ptr, 0, sizeof(uint32_t), c->stream), "memset errors");
    cudaCheck(cudaStreamSynchronize(c->stream), "sync");
    *out = c.release();
  });
}

int exa_context_destroy(exa_context *ctx)
{
  return guarded([&] {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    const bool own = ctx->ownStream;
    cudaStream_t s = ctx->stream;
    delete ctx;
    if (own) cudaStreamDestroy(s);
  });
}

int exa_get_device_errors(exa_context *ctx, uint32_t *bits)
{
  return guarded([&] {
    need(ctx && bits, EXA_ERR_INVALID, "null argument");
    setDevice(ctx);
    uint32_t v = 0;
    cudaCheck(cudaMemcpyAsync(&v, ctx->errors.ptr, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream), "read errors");
    cudaCheck(cudaMemsetAsync(ctx->errors.ptr, 0, sizeof(v), ctx->stream), "clear errors");
    cudaCheck(cudaStreamSynchronize(ctx->stream), "sync");
    *bits = v;
  });
}

int exa_sync(exa_context *ctx)
{
  uint32_t bits = 0;
  const int rc = guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    setDevice(ctx);
    cudaCheck(cudaStreamSynchronize(ctx->stream), "exa_sync");
  });
  if (rc != EXA_OK) return rc;
  const int rc2 = exa_get_device_errors(ctx, &bits);
  if (rc2 != EXA_OK) return rc2;
  if (bits) {
    g_lastError = "device iteration cap hit (EXA_DEVERR bits " + std::to_string(bits) + ")";
    return EXA_ERR_DEVICE_LIMIT;
  }
  return EXA_OK;
}

int exa_model_create(exa_context *ctx, const exa_vec4f *vertices, uint64_t numVertices, const int32_t *indices,
                     uint64_t numElems, const exa_gridlet *gridlets, uint64_t numGridlets,
                     const float *gridletScalars, uint64_t numGridletScalars)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    need(numVertices == 0 || vertices, EXA_ERR_INVALID, "vertices is null");
    need(numElems == 0 || indices, EXA_ERR_INVALID, "indices is null");
    need(numGridlets == 0 || gridlets, EXA_ERR_INVALID, "gridlets is null");
    need(numGridletScalars == 0 || gridletScalars, EXA_ERR_INVALID, "gridletScalars is null");
    need(numElems < 0x7fffffffull && numGridlets < 0x7fffffffull && numVertices < 0x7fffffffull &&
             numGridletScalars <= 0xffffffffull,
         EXA_ERR_INVALID, "array too large for 32-bit indices");
    auto m = std::make_shared<ExaStitchModel>();
    m->assign(vertices, numVertices, indices, numElems, gridlets, numGridlets, gridletScalars, numGridletScalars);
    ctx->model = m;
    ctx->sampler.reset();
  });
}

int exa_amrcell_model_create(exa_context *ctx, const exa_amr_cell *cells, uint64_t numCells, const float *scalars,
                             uint64_t numScalars)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    need(numCells == 0 || cells, EXA_ERR_INVALID, "cells is null");
    need(numScalars == 0 || scalars, EXA_ERR_INVALID, "scalars is null");
    need(numCells < 0x7fffffffull, EXA_ERR_INVALID, "array too large for 32-bit indices");
    auto m = std::make_shared<AMRCellModel>();
    m->assign(cells, numCells, scalars, numScalars);
    ctx->model = m;
    ctx->sampler.reset();
  });
}

namespace {
std::vector<char> readFile(const char *path, bool required)
{
  std::vector<char> data;
  if (!path || !*path) {
    if (required) throw Error(EXA_ERR_INVALID, "no file name");
    return data;
  }
  FILE *f = std::fopen(path, "rb");
  if (!f) {
    if (required) throw Error(EXA_ERR_INVALID, std::string("cannot open ") + path);
    return data;  // the loader treats a missing scalars file as empty
  }
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (n > 0) {
    data.resize((size_t)n);
    if (std::fread(data.data(), 1, (size_t)n, f) != (size_t)n) {
      std::fclose(f);
      throw Error(EXA_ERR_INVALID, std::string("short read of ") + path);
    }
  }
  std::fclose(f);
  return data;
}

// ExaStitchModel::load's gridlet loop: records until the data runs out
void parseGrids(const std::vector<char> &g, const std::vector<char> &sc, std::vector<exa_gridlet> &gl,
                std::vector<float> &vals)
{
  const size_t nsc = sc.size() / sizeof(float);
  const float *scalars = reinterpret_cast<const float *>(sc.data());
  size_t off = 0;
  while (off + 28 <= g.size()) {
    exa_gridlet q;
    int32_t hdr[7];
    std::memcpy(hdr, g.data() + off, 28);
    off += 28;
    q.lower = exa_vec3i{hdr[0], hdr[1], hdr[2]};
    q.level = hdr[3];
    q.dims = exa_vec3i{hdr[4], hdr[5], hdr[6]};
    if (q.dims.x < 0 || q.dims.y < 0 || q.dims.z < 0 || q.level < 0 || q.level > 30)
      throw Error(EXA_ERR_INVALID, "corrupt .grids record");
    const size_t ns = (size_t)(q.dims.x + 1) * (size_t)(q.dims.y + 1) * (size_t)(q.dims.z + 1);
    if (off + ns * 4 > g.size()) throw Error(EXA_ERR_INVALID, "truncated .grids record");
    q.begin = (uint32_t)vals.size();
    for (size_t i = 0; i < ns; ++i) {
      int32_t id;
      std::memcpy(&id, g.data() + off + 4 * i, 4);
      vals.push_back((unsigned)id < nsc ? scalars[(unsigned)id] : NAN);
    }
    off += ns * 4;
    gl.push_back(q);
  }
}
}  // namespace

int exa_read_grids(const char *gridsFile, const char *scalarsFile, exa_gridlet *gridlets, uint64_t *numGridlets,
                   float *gridletScalars, uint64_t *numGridletScalars)
{
  return guarded([&] {
    need(numGridlets && numGridletScalars, EXA_ERR_INVALID, "null count");
    std::vector<exa_gridlet> gl;
    std::vector<float> vals;
    parseGrids(readFile(gridsFile, true), readFile(scalarsFile, false), gl, vals);
    if (gridlets || gridletScalars) {
      need(gridlets && gridletScalars && *numGridlets >= gl.size() && *numGridletScalars >= vals.size(),
           EXA_ERR_INVALID, "output arrays too small");
      std::memcpy(gridlets, gl.data(), gl.size() * sizeof(exa_gridlet));
      std::memcpy(gridletScalars, vals.data(), vals.size() * sizeof(float));
    }
    *numGridlets = gl.size();
    *numGridletScalars = vals.size();
  });
}

int exa_model_load(exa_context *ctx, const char *gridsFile, const char *scalarsFile)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    std::vector<exa_gridlet> gl;
    std::vector<float> vals;
    parseGrids(readFile(gridsFile, true), readFile(scalarsFile, false), gl, vals);
    need(gl.size() < 0x7fffffffull && vals.size() <= 0xffffffffull, EXA_ERR_INVALID, "model too large");
    auto m = std::make_shared<ExaStitchModel>();
    m->assign(nullptr, 0, nullptr, 0, gl.data(), gl.size(), vals.data(), vals.size());
    ctx->model = m;
    ctx->sampler.reset();
  });
}

// AMRCellModel::load (AMRCellModel.cpp:24-67): a missing scalars file
// leaves the model without scalars (the build then fails)
int exa_amrcell_model_load(exa_context *ctx, const char *cellsFile, const char *scalarsFile)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    const std::vector<char> c = readFile(cellsFile, true);
    const std::vector<char> v = readFile(scalarsFile, false);
    std::vector<exa_amr_cell> cells(c.size() / sizeof(exa_amr_cell));
    std::vector<float> vals(v.size() / sizeof(float));
    if (!cells.empty()) std::memcpy(cells.data(), c.data(), cells.size() * sizeof(exa_amr_cell));
    if (!vals.empty()) std::memcpy(vals.data(), v.data(), vals.size() * sizeof(float));
    need(cells.size() < 0x7fffffffull, EXA_ERR_INVALID, "model too large");
    auto m = std::make_shared<AMRCellModel>();
    m->assign(cells.data(), cells.size(), vals.data(), vals.size());
    ctx->model = m;
    ctx->sampler.reset();
  });
}

int exa_exabrick_model_create(exa_context *ctx, const exa_brick *bricks, uint64_t numBricks, const float *scalars,
                              uint64_t numScalars)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    need(numBricks == 0 || bricks, EXA_ERR_INVALID, "bricks is null");
    need(numScalars == 0 || scalars, EXA_ERR_INVALID, "scalars is null");
    need(numBricks < 0x3fffffffull && numScalars <= 0xffffffffull, EXA_ERR_INVALID, "model too large");
    auto m = std::make_shared<ExaBrickModel>();
    m->assign(bricks, numBricks, scalars, numScalars);
    ctx->model = m;
    ctx->sampler.reset();
  });
}

// ExaBrickModel::load (model/ExaBrickModel.cpp:28-117): brick records until
// the data runs out; every cell id must index the scalars file
int exa_exabrick_model_load(exa_context *ctx, const char *bricksFile, const char *scalarsFile)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    const std::vector<char> d = readFile(bricksFile, true);
    const std::vector<char> sv = readFile(scalarsFile, false);
    const size_t numValues = sv.size() / sizeof(float);
    std::vector<float> ordered(numValues);
    if (numValues) std::memcpy(ordered.data(), sv.data(), numValues * sizeof(float));
    std::vector<exa_brick> bricks;
    std::vector<float> scalars;
    size_t at = 0;
    while (d.size() - at >= 7 * sizeof(int32_t)) {
      int32_t h[7];
      std::memcpy(h, d.data() + at, sizeof(h));
      exa_brick b;
      b.size = {h[0], h[1], h[2]};
      b.lower = {h[3], h[4], h[5]};
      b.level = h[6];
      need(b.size.x > 0 && b.size.y > 0 && b.size.z > 0, EXA_ERR_INVALID, "bad brick size");
      const uint64_t n = (uint64_t)b.size.x * b.size.y * b.size.z;
      if (d.size() - at - sizeof(h) < n * sizeof(int32_t)) break;  // the loader stops at a short record
      at += sizeof(h);
      b.begin = (uint32_t)scalars.size();
      for (uint64_t k = 0; k < n; ++k) {
        int32_t id;
        std::memcpy(&id, d.data() + at + k * sizeof(int32_t), sizeof(id));
        need(id >= 0, EXA_ERR_INVALID, "negative cell ID");
        need((size_t)id < numValues, EXA_ERR_INVALID, "invalid cell ID");
        scalars.push_back(ordered[id]);
      }
      at += n * sizeof(int32_t);
      need(scalars.size() <= 0xffffffffull, EXA_ERR_INVALID, "model too large");
      bricks.push_back(b);
    }
    auto m = std::make_shared<ExaBrickModel>();
    m->assign(bricks.data(), bricks.size(), scalars.data(), scalars.size());
    ctx->model = m;
    ctx->sampler.reset();
  });
}

int exa_exabrick_get_abrs(exa_context *ctx, exa_abr *abrs, uint64_t *numAbrs, int32_t *leafList,
                          uint64_t *leafListSize)
{
  return guarded([&] {
    need(ctx && numAbrs && leafListSize, EXA_ERR_INVALID, "null argument");
    auto *m = dynamic_cast<ExaBrickModel *>(ctx->model.get());
    need(m != nullptr, EXA_ERR_STATE, "no ExaBrick model");
    if (abrs) {
      need(*numAbrs >= m->abrs.size(), EXA_ERR_INVALID, "region array too small");
      std::memcpy(abrs, m->abrs.data(), m->abrs.size() * sizeof(exa_abr));
    }
    if (leafList) {
      need(*leafListSize >= m->leafList.size(), EXA_ERR_INVALID, "leaf list array too small");
      std::memcpy(leafList, m->leafList.data(), m->leafList.size() * sizeof(int32_t));
    }
    *numAbrs = m->abrs.size();
    *leafListSize = m->leafList.size();
  });
}

int exa_read_xf(const char *xfFile, exa_xf *xf, exa_vec4f *colors, int32_t maxColors)
{
  return guarded([&] {
    need(xf != nullptr, EXA_ERR_INVALID, "null xf");
    const std::vector<char> d = readFile(xfFile, true);
    const uint64_t kMagic = 0x1235abc000ull;
    need(d.size() >= 8 + 5 * 4 + 4, EXA_ERR_INVALID, "not a valid '.xf' transfer function file");
    uint64_t magic;
    std::memcpy(&magic, d.data(), 8);
    need(magic == kMagic, EXA_ERR_INVALID, "not a valid '.xf' transfer function file");
    float f[5];
    std::memcpy(f, d.data() + 8, 20);
    int32_t n;
    std::memcpy(&n, d.data() + 28, 4);
    need(n >= 0 && d.size() >= 32 + (size_t)n * 16, EXA_ERR_INVALID, "truncated '.xf' file");
    xf->opacityScale = f[0];
    xf->absDomain = exa_range1f{f[1], f[2]};
    xf->relDomain = exa_range1f{f[3], f[4]};
    xf->numColors = n;
    if (colors) {
      need(maxColors >= n, EXA_ERR_INVALID, "colour array too small");
      std::memcpy(colors, d.data() + 32, (size_t)n * 16);
    }
  });
}

exa_range1f exa_xf_range(const exa_xf *xf)
{
  if (!xf) return exa_range1f{0.f, 1.f};
  const float a0 = std::min(xf->absDomain.lower, xf->absDomain.upper);
  const float a1 = std::max(xf->absDomain.lower, xf->absDomain.upper);
  const float r0 = .01f * xf->relDomain.lower, r1 = .01f * xf->relDomain.upper;
  const float q0 = std::min(r0, r1), q1 = std::max(r0, r1);
  return exa_range1f{(1.f - q0) * a0 + q0 * a1, (1.f - q1) * a0 + q1 * a1};
}

float exa_opacity_scale(float s) { return std::pow(1.1f, s - 100.f); }

int exa_read_cells(const char *cellsFile, exa_amr_cell *cells, uint64_t *numCells)
{
  return guarded([&] {
    need(numCells != nullptr, EXA_ERR_INVALID, "null count");
    const std::vector<char> d = readFile(cellsFile, true);
    const size_t n = d.size() / sizeof(exa_amr_cell);
    if (cells) {
      need(*numCells >= n, EXA_ERR_INVALID, "output array too small");
      std::memcpy(cells, d.data(), n * sizeof(exa_amr_cell));
    }
    *numCells = n;
  });
}

// TriangleMesh::load / loadOne (TriangleMesh.cpp:27-76), the meshes
// concatenated; a file that ends inside a mesh record is an error (the
// reference keeps the zero-filled remainder)
int exa_read_mesh(const char *meshFile, exa_vec3f *vertices, uint64_t *numVertices, exa_vec3i *indices,
                  uint64_t *numTriangles)
{
  return guarded([&] {
    need(numVertices && numTriangles, EXA_ERR_INVALID, "null count");
    const std::vector<char> d = readFile(meshFile, true);
    size_t at = 0, nv = 0, nt = 0;
    auto take = [&](void *dst, size_t bytes) {
      need(d.size() - at >= bytes, EXA_ERR_INVALID, "truncated mesh file");
      if (dst) std::memcpy(dst, d.data() + at, bytes);
      at += bytes;
    };
    const bool fill = vertices && indices;
    const uint64_t capV = fill ? *numVertices : 0, capT = fill ? *numTriangles : 0;
    while (d.size() - at >= sizeof(int32_t)) {
      int32_t mv = 0, mt = 0;
      take(&mv, sizeof(mv));
      need(mv >= 0, EXA_ERR_INVALID, "broken triangle model");
      need(fill ? nv + (size_t)mv <= capV : true, EXA_ERR_INVALID, "vertex array too small");
      take(fill ? vertices + nv : nullptr, (size_t)mv * sizeof(exa_vec3f));
      take(&mt, sizeof(mt));
      need(mt >= 0, EXA_ERR_INVALID, "broken triangle model");
      need(fill ? nt + (size_t)mt <= capT : true, EXA_ERR_INVALID, "triangle array too small");
      std::vector<exa_vec3i> tri((size_t)mt);
      take(tri.data(), (size_t)mt * sizeof(exa_vec3i));
      for (exa_vec3i &t : tri) {
        need(t.x >= 0 && t.x < mv && t.y >= 0 && t.y < mv && t.z >= 0 && t.z < mv, EXA_ERR_INVALID,
             "broken triangle model");
        if (fill) indices[nt++] = exa_vec3i{t.x + (int32_t)nv, t.y + (int32_t)nv, t.z + (int32_t)nv};
      }
      if (!fill) nt += (size_t)mt;
      nv += (size_t)mv;
      need(nv < 0x7fffffffull && nt < 0x7fffffffull, EXA_ERR_INVALID, "mesh too large");
    }
    *numVertices = nv;
    *numTriangles = nt;
  });
}

int exa_mesh_set(exa_context *ctx, const exa_vec3f *vertices, uint64_t numVertices, const exa_vec3i *indices,
                 uint64_t numTriangles)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_INVALID, "null context");
    setDevice(ctx);
    if (numTriangles == 0) {
      cudaCheck(cudaStreamSynchronize(ctx->stream), "mesh release");
      ctx->mesh.reset();
      return;
    }
    need(vertices && indices, EXA_ERR_INVALID, "null mesh arrays");
    need(numVertices < 0x7fffffffull && numTriangles < 0x7fffffffull, EXA_ERR_INVALID, "mesh too large");
    std::vector<float4> v((size_t)numVertices);
    for (size_t i = 0; i < v.size(); ++i) v[i] = make_float4(vertices[i].x, vertices[i].y, vertices[i].z, 0.f);
    std::vector<int32_t> rows((size_t)numTriangles * 8, -1);
    exa_box3f b;
    b.lower = {INFINITY, INFINITY, INFINITY};
    b.upper = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t t = 0; t < (size_t)numTriangles; ++t) {
      const int32_t id[3] = {indices[t].x, indices[t].y, indices[t].z};
      for (int k = 0; k < 3; ++k) {
        need(id[k] >= 0 && (uint64_t)id[k] < numVertices, EXA_ERR_INVALID, "broken triangle model");
        rows[t * 8 + k] = id[k];
        const exa_vec3f &p = vertices[id[k]];
        b.lower = {std::min(b.lower.x, p.x), std::min(b.lower.y, p.y), std::min(b.lower.z, p.z)};
        b.upper = {std::max(b.upper.x, p.x), std::max(b.upper.y, p.y), std::max(b.upper.z, p.z)};
      }
    }
    cudaCheck(cudaStreamSynchronize(ctx->stream), "mesh replace");
    auto M = std::make_unique<MeshState>();
    const size_t nt = (size_t)numTriangles;
    M->vertices.upload(v.data(), v.size(), ctx->stream);
    M->indices.upload(rows.data(), rows.size(), ctx->stream);
    M->nodes.alloc(nt > 1 ? nt - 1 : 1);
    M->parents.alloc((nt > 1 ? nt - 1 : 0) + nt);
    M->leafElem.alloc(nt);
    launchBuildBVH(M->vertices.ptr, M->indices.ptr, nt, b, M->nodes.ptr, M->parents.ptr, M->leafElem.ptr,
                   ctx->stream);
    MeshView mv{M->vertices.ptr, M->indices.ptr, M->nodes.ptr, (int)nt};
    M->view.upload(&mv, 1, ctx->stream);
    cudaCheck(cudaStreamSynchronize(ctx->stream), "mesh upload");
    M->bounds = b;
    ctx->mesh = std::move(M);
  });
}

int exa_mesh_get_bounds(exa_context *ctx, exa_box3f *bounds)
{
  return guarded([&] {
    need(ctx && bounds, EXA_ERR_INVALID, "null argument");
    need(ctx->mesh != nullptr, EXA_ERR_STATE, "no mesh");
    *bounds = ctx->mesh->bounds;
  });
}

int exa_model_get_bounds(exa_context *ctx, exa_box3f *cellBounds, exa_range1f *valueRange)
{
  return guarded([&] {
    need(ctx && ctx->model, EXA_ERR_STATE, "no model");
    if (cellBounds) *cellBounds = ctx->model->cellBounds;
    if (valueRange) *valueRange = ctx->model->valueRange;
  });
}

int exa_model_set_num_grid_cells(exa_context *ctx, exa_vec3i numMCs)
{
  return guarded([&] {
    need(ctx && ctx->model, EXA_ERR_STATE, "no model");
    ctx->model->setNumGridCells(numMCs);
  });
}

int exa_model_set_voxel_space_transform(exa_context *ctx, exa_box3f from, exa_box3f to)
{
  return guarded([&] {
    need(ctx && ctx->model, EXA_ERR_STATE, "no model");
    ctx->model->setVoxelSpaceTransform(from, to);
  });
}

int exa_model_get_world_bounds(exa_context *ctx, exa_box3f *bounds)
{
  return guarded([&] {
    need(ctx && ctx->model && bounds, EXA_ERR_STATE, "no model");
    *bounds = ctx->model->getBounds();
  });
}

int exa_model_mem_stats(exa_context *ctx, exa_mem_stats *out)
{
  return guarded([&] {
    need(ctx && ctx->model && out, EXA_ERR_STATE, "no model");
    std::memset(out, 0, sizeof(*out));
    if (auto *em = dynamic_cast<ExaStitchModel *>(ctx->model.get())) {
      size_t a, b, c, d, e;
      em->memStats(a, b, c, d, e);
      out->elemVertexBytes = a;
      out->elemIndexBytes = b;
      out->gridletBytes = c;
      out->emptyScalarsBytes = d;
      out->nonEmptyScalarsBytes = e;
    } else if (auto *am = dynamic_cast<AMRCellModel *>(ctx->model.get())) {
      size_t a, b;
      am->memStats(a, b);
      out->amrCellBytes = a;
      out->amrScalarBytes = b;
    } else if (auto *bm = dynamic_cast<ExaBrickModel *>(ctx->model.get())) {
      size_t a, b, c, d;
      bm->memStats(a, b, c, d);
      out->bricksBytes = a;
      out->brickScalarsBytes = b;
      out->abrsBytes = c;
      out->abrLeafListBytes = d;
    }
    if (auto &S = ctx->sampler) {
      out->deviceFieldBytes = S->fieldBytes();
      out->deviceAccelBytes = S->accelBytes();
      const auto &g = *ctx->model->grid;
      out->deviceMajorantBytes = g.valueRanges.bytes() + g.maxOpacities.bytes();
      if (auto *es = dynamic_cast<ExaStitchSampler *>(S.get()))
        out->deviceMajorantBytes += es->gridletValueRanges.bytes() + es->gridletMaxOpacities.bytes() +
                                    es->elemValueRanges.bytes() + es->umeshMaxOpacities.bytes();
    }
  });
}

int exa_sampler_build(exa_context *ctx)
{
  return guarded([&] {
    need(ctx && ctx->model, EXA_ERR_STATE, "no model");
    need(ctx->model->grid != nullptr, EXA_ERR_STATE, "numGridCells not set");
    setDevice(ctx);
    // the sampler that goes with the model (OWLRenderer.cpp:150-200)
    std::shared_ptr<Sampler> s;
    if (dynamic_cast<AMRCellModel *>(ctx->model.get()))
      s = std::make_shared<AMRCellSampler>();
    else if (dynamic_cast<ExaBrickModel *>(ctx->model.get()))
      s = std::make_shared<ExaBrickSampler>();
    else
      s = std::make_shared<ExaStitchSampler>();
    const auto t0 = std::chrono::steady_clock::now();
    s->debugFlags = ctx->debugFlags;
    if (!s->build(ctx->model, ctx->stream)) throw Error(EXA_ERR_STATE, s->className() + "::build failed");
    ctx->sampler = s;
    ctx->lastBuild = {};
    if (auto *es = dynamic_cast<ExaStitchSampler *>(s.get())) ctx->lastBuild = es->buildStats;
    ctx->lastBuild.totalMs =
        std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  });
}

int exa_get_build_stats(exa_context *ctx, exa_build_stats *out)
{
  return guarded([&] {
    need(ctx && out, EXA_ERR_INVALID, "null argument");
    *out = ctx->lastBuild;
  });
}

int exa_sampler_compute_max_opacities(exa_context *ctx, const exa_vec4f *colorMap, int32_t numColors,
                                      exa_range1f xfRange)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(colorMap && numColors > 0, EXA_ERR_INVALID, "empty color map");
    setDevice(ctx);
    ctx->sampler->tfFilter = ctx->tfFilter;
    ctx->sampler->computeMaxOpacities(colorMap, numColors, xfRange, ctx->stream);
    ctx->xfRange = xfRange;
    ctx->numColors = numColors;
    if (ctx->surrogate && ctx->surrogate->evaluated)
      ctx->surrogate->computeMajorants(ctx->sampler->colorMap.ptr, numColors, xfRange, ctx->sampler->tfFilter,
                                       ctx->stream);
  });
}

int exa_debug_set_flags(exa_context *ctx, uint32_t flags)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_STATE, "null context");
    need((flags & ~(uint32_t)EXA_DEBUG_COPY_WAIT_TIMEOUT) == 0, EXA_ERR_INVALID, "unknown debug flag");
    ctx->debugFlags = flags;
  });
}

int exa_set_render_path(exa_context *ctx, int32_t path)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_STATE, "null context");
    need(path == EXA_RENDER_PATH_AUTO || path == EXA_RENDER_PATH_WAVEFRONT || path == EXA_RENDER_PATH_SINGLE_LAUNCH,
         EXA_ERR_INVALID, "unknown render path");
    ctx->renderPath = path;
  });
}

int exa_set_transfer_function_filter(exa_context *ctx, int32_t filter)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_STATE, "null context");
    need(filter == EXA_TF_FILTER_NEAREST || filter == EXA_TF_FILTER_LINEAR, EXA_ERR_INVALID,
         "unknown transfer-function filter");
    ctx->tfFilter = filter;
  });
}

int exa_sampler_set_lps(exa_context *ctx, exa_launch_params *lp)
{
  return guarded([&] {
    need(ctx && ctx->sampler && lp, EXA_ERR_STATE, "sampler not built");
    ctx->sampler->setLPs(*lp);
    const auto &m = *ctx->model;
    lp->majorantGrid = m.grid->deviceTraversable;         // OWLRenderer.cpp:435-436
    lp->maxOpacities = ctx->sampler->maxOpacities;         // :655-657
    lp->worldSpaceBounds = m.getBounds();                  // :548-555
    lp->meshBVH = 0;
    if (ctx->mesh) {                                       // :453-465, 520, 544
      lp->meshBVH = (uint64_t)(uintptr_t)ctx->mesh->view.ptr;
      exa_box3f &b = lp->worldSpaceBounds;
      const exa_box3f &mb = ctx->mesh->bounds;
      b.lower = {std::min(b.lower.x, mb.lower.x), std::min(b.lower.y, mb.lower.y), std::min(b.lower.z, mb.lower.z)};
      b.upper = {std::max(b.upper.x, mb.upper.x), std::max(b.upper.y, mb.upper.y), std::max(b.upper.z, mb.upper.z)};
    }
    lp->voxelSpaceTransform = m.voxelSpaceTransform;       // :577
    lp->lightSpaceTransform = m.lightSpaceTransform;       // :578
    lp->ext.voxelSpaceTransformInv = m.voxelSpaceTransformInv;
    if (ctx->sampler->hasTF) {                             // :710-711, 724
      lp->transferFunc.values = reinterpret_cast<exa_vec4f *>(ctx->sampler->colorMap.ptr);
      lp->transferFunc.numValues = ctx->numColors;
      lp->transferFunc.domain = ctx->xfRange;
    }
    lp->ext.tfFilter = ctx->sampler->tfFilter;
    lp->ext.deviceErrors = ctx->errors.ptr;
  });
}

int exa_get_majorants(exa_context *ctx, exa_range1f *valueRanges, float *maxOpacities)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    setDevice(ctx);
    const Grid &g = *ctx->model->grid;
    if (valueRanges)
      cudaCheck(cudaMemcpyAsync(valueRanges, g.valueRanges.ptr, g.valueRanges.bytes(), cudaMemcpyDeviceToHost,
                                ctx->stream), "copy ranges");
    if (maxOpacities)
      cudaCheck(cudaMemcpyAsync(maxOpacities, g.maxOpacities.ptr, g.maxOpacities.bytes(), cudaMemcpyDeviceToHost,
                                ctx->stream), "copy maxOpacities");
    cudaCheck(cudaStreamSynchronize(ctx->stream), "sync");
  });
}

int exa_get_prim_majorants(exa_context *ctx, exa_range1f *gridletRanges, float *gridletMaxOpacities,
                           float *elemMaxOpacities)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    setDevice(ctx);
    auto &S = esSampler(ctx);
    if (gridletRanges && S.gridletValueRanges.count)
      cudaCheck(cudaMemcpyAsync(gridletRanges, S.gridletValueRanges.ptr, S.gridletValueRanges.bytes(),
                                cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (gridletMaxOpacities && S.gridletMaxOpacities.count)
      cudaCheck(cudaMemcpyAsync(gridletMaxOpacities, S.gridletMaxOpacities.ptr, S.gridletMaxOpacities.bytes(),
                                cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (elemMaxOpacities && S.umeshMaxOpacities.count)
      cudaCheck(cudaMemcpyAsync(elemMaxOpacities, S.umeshMaxOpacities.ptr, S.umeshMaxOpacities.bytes(),
                                cudaMemcpyDeviceToHost, ctx->stream), "copy");
    cudaCheck(cudaStreamSynchronize(ctx->stream), "sync");
  });
}

int exa_sample_points(exa_context *ctx, const exa_vec3f *posDevice, uint64_t n, exa_sample *outDevice,
                      int32_t cullTransparent)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(n == 0 || (posDevice && outDevice), EXA_ERR_INVALID, "null buffer");
    need(!cullTransparent || ctx->sampler->hasTF, EXA_ERR_STATE, "culling needs computeMaxOpacities first");
    setDevice(ctx);
    launchSamplePoints(ctx->sampler->accel, posDevice, n, outDevice, cullTransparent, ctx->errors.ptr, ctx->stream);
  });
}

int exa_sample_points_host(exa_context *ctx, const exa_vec3f *posHost, uint64_t n, exa_sample *outHost,
                           int32_t cullTransparent)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(n == 0 || (posHost && outHost), EXA_ERR_INVALID, "null buffer");
    need(!cullTransparent || ctx->sampler->hasTF, EXA_ERR_STATE, "culling needs computeMaxOpacities first");
    setDevice(ctx);
    if (ctx->hostPos.count < n) { ctx->hostPos.alloc(n); ctx->hostOut.alloc(n); }
    cudaCheck(cudaMemcpyAsync(ctx->hostPos.ptr, posHost, n * sizeof(exa_vec3f), cudaMemcpyHostToDevice, ctx->stream),
              "copy in");
    launchSamplePoints(ctx->sampler->accel, ctx->hostPos.ptr, n, ctx->hostOut.ptr, cullTransparent, ctx->errors.ptr,
                       ctx->stream);
    cudaCheck(cudaMemcpyAsync(outHost, ctx->hostOut.ptr, n * sizeof(exa_sample), cudaMemcpyDeviceToHost, ctx->stream),
              "copy out");
    cudaCheck(cudaStreamSynchronize(ctx->stream), "sync");
  });
}

int exa_get_render_stats(exa_context *ctx, exa_render_stats *out)
{
  return guarded([&] {
    need(ctx && out, EXA_ERR_INVALID, "null argument");
    *out = ctx->lastStats;
  });
}

int exa_launch_params_init(exa_launch_params *lp)
{
  return guarded([&] {
    need(lp != nullptr, EXA_ERR_INVALID, "null lp");
    std::memset(lp, 0, sizeof(*lp));
    lp->integrator = EXA_PATH_TRACING_INTEGRATOR;     // OWLRenderer.cpp:569
    lp->shadeMode = EXA_SHADE_MODE_DEFAULT;           // :571
    lp->subImage.value.upper.y = 1.f;                 // :562-565
    lp->subImage.selection.upper.x = 1.f;
    lp->subImage.selection.upper.y = 1.f;
    lp->render.dt = 1.f;                              // :616
    lp->render.spp = 1;                               // :617
    lp->render.heatMapScale = 1.f;
    lp->transferFunc.opacityScale = 1.f;              // 1.1^(100-100)
    lp->transferFunc.domain.lower = 0.f;
    lp->transferFunc.domain.upper = 1.f;
    exa_affine3f I;
    std::memset(&I, 0, sizeof(I));
    I.l.vx.x = I.l.vy.y = I.l.vz.z = 1.f;
    lp->voxelSpaceTransform = I;
    lp->lightSpaceTransform = I;
    lp->ext.voxelSpaceTransformInv = I;
    lp->ext.maxBounces = 1024;                        // deviceCode.cu:1050
    lp->ext.albedo = -1.f;                            // :1061 (TF rgb)
    lp->ext.hgG = 0.f;                                // :1089
    lp->ext.cullTransparentPrims = 1;
  });
}

int exa_render(exa_context *ctx, const exa_launch_params *lp, int32_t width, int32_t height)
{
  return guarded([&] { renderFrame(ctx, lp, width, height, false); });
}

// ------------------------------------------------------------ learned field
void exa_surrogate_params_default(exa_surrogate_params *p)
{
  if (!p) return;
  const SurrogateConfig c;
  std::memset(p, 0, sizeof(*p));
  p->log2TableSize = c.log2T;
  p->baseResolution = c.baseRes;
  p->growth = c.growth;
  p->importanceFraction = c.importance;
  p->numSamples = c.numSamples;
  p->batch = c.batch;
  p->learningRate = c.lrTable;
  p->learningRateFinal = c.lrFinal;
  p->seed = c.seed;
}

int exa_surrogate_create(exa_context *ctx, const exa_surrogate_params *p)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(p != nullptr, EXA_ERR_INVALID, "null params");
    need(p->numSamples >= 32 && p->numSamples <= ((uint64_t)1 << 28), EXA_ERR_INVALID, "numSamples out of range");
    need(p->baseResolution >= 1 && p->growth >= 1.f && p->growth <= 4.f, EXA_ERR_INVALID, "bad grid resolutions");
    need(p->importanceFraction >= 0.f && p->importanceFraction <= 1.f, EXA_ERR_INVALID, "bad importance fraction");
    need(p->learningRate > 0.f && p->learningRateFinal > 0.f, EXA_ERR_INVALID, "bad learning rate");
    setDevice(ctx);
    SurrogateConfig c;
    c.log2T = p->log2TableSize;
    c.baseRes = p->baseResolution;
    c.growth = p->growth;
    c.importance = p->importanceFraction;
    c.numSamples = (size_t)p->numSamples;
    c.batch = p->batch;
    c.lrTable = c.lrMlp = p->learningRate;
    c.lrFinal = p->learningRateFinal;
    c.seed = p->seed;
    auto S = std::make_unique<Surrogate>();
    S->configure(c, esModel(ctx));
    S->allocate(ctx->stream);
    S->generateSamples(esSampler(ctx), ctx->stream);
    ctx->surrogate = std::move(S);
  });
}

int exa_surrogate_train(exa_context *ctx, int32_t steps, float *loss)
{
  return guarded([&] {
    need(ctx && ctx->surrogate, EXA_ERR_STATE, "no surrogate");
    need(steps >= 0, EXA_ERR_INVALID, "negative steps");
    setDevice(ctx);
    const float l = steps > 0 ? ctx->surrogate->trainSteps(steps, ctx->stream) : ctx->surrogate->lastLoss;
    ctx->surrogate->evaluated = false;  // the network changed: errors must be measured again
    if (loss) *loss = l;
  });
}

int exa_surrogate_evaluate(exa_context *ctx, float tolerance, uint64_t pointsTarget)
{
  return guarded([&] {
    need(ctx && ctx->surrogate && ctx->sampler, EXA_ERR_STATE, "no surrogate");
    need(tolerance >= 0.f, EXA_ERR_INVALID, "negative tolerance");
    need(ctx->sampler->hasTF && ctx->numColors > 0, EXA_ERR_STATE, "no transfer function (compute max opacities first)");
    setDevice(ctx);
    Surrogate &S = *ctx->surrogate;
    const Grid &g = *ctx->model->grid;
    S.evaluate(esSampler(ctx), g, (double)tolerance, (size_t)std::max<uint64_t>(pointsTarget, 1), ctx->stream);
    S.computeMajorants(ctx->sampler->colorMap.ptr, ctx->numColors, ctx->xfRange, ctx->sampler->tfFilter, ctx->stream);
    cudaCheck(cudaStreamSynchronize(ctx->stream), "surrogate majorants");
    ctx->surrogateTol = tolerance;
  });
}

namespace {
// exact-field bytes the exact-sampler macrocells still need: primitives
// whose bounds touch a macrocell in exact mode, plus the point-location
// structures
size_t fallbackBytes(exa_context *ctx)
{
  const ExaStitchModel &m = esModel(ctx);
  const Grid &g = *m.grid;
  const size_t nmc = (size_t)g.dims.x * g.dims.y * g.dims.z;
  std::vector<uint8_t> mode(nmc);
  cudaCheck(cudaMemcpy(mode.data(), ctx->surrogate->mcMode.ptr, nmc, cudaMemcpyDeviceToHost), "d2h");
  const exa_box3f wb = g.worldBounds;
  auto proj = [&](float v, float lo, float hi, int d) {
    int i = (int)((v - lo) / (hi - lo) * (float)d);
    return i < 0 ? 0 : (i > d - 1 ? d - 1 : i);
  };
  auto touchesExact = [&](exa_vec3f lo, exa_vec3f hi) {
    const int x0 = proj(lo.x, wb.lower.x, wb.upper.x, g.dims.x), x1 = proj(hi.x, wb.lower.x, wb.upper.x, g.dims.x);
    const int y0 = proj(lo.y, wb.lower.y, wb.upper.y, g.dims.y), y1 = proj(hi.y, wb.lower.y, wb.upper.y, g.dims.y);
    const int z0 = proj(lo.z, wb.lower.z, wb.upper.z, g.dims.z), z1 = proj(hi.z, wb.lower.z, wb.upper.z, g.dims.z);
    for (int z = z0; z <= z1; ++z)
      for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x)
          if (!mode[((size_t)z * g.dims.y + y) * g.dims.x + x]) return true;
    return false;
  };
  size_t bytes = ctx->sampler->accelBytes();
  for (const exa_gridlet &gl : m.gridlets) {
    const float cw = (float)(1 << gl.level);
    const exa_vec3f lo{((float)gl.lower.x + 0.5f) * cw, ((float)gl.lower.y + 0.5f) * cw, ((float)gl.lower.z + 0.5f) * cw};
    const exa_vec3f hi{((float)(gl.lower.x + gl.dims.x) + 0.5f) * cw, ((float)(gl.lower.y + gl.dims.y) + 0.5f) * cw,
                       ((float)(gl.lower.z + gl.dims.z) + 0.5f) * cw};
    if (touchesExact(lo, hi))
      bytes += sizeof(exa_gridlet) + sizeof(float) * (size_t)(gl.dims.x + 1) * (gl.dims.y + 1) * (gl.dims.z + 1);
  }
  const size_t ne = m.indices.size() / 8;
  std::vector<uint8_t> vertUsed(m.vertices.size(), 0);
  for (size_t e = 0; e < ne; ++e) {
    exa_vec3f lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
    for (int j = 0; j < 8; ++j) {
      const int id = m.indices[e * 8 + j];
      if (id < 0) break;
      const exa_vec4f &v = m.vertices[id];
      lo = {std::min(lo.x, v.x), std::min(lo.y, v.y), std::min(lo.z, v.z)};
      hi = {std::max(hi.x, v.x), std::max(hi.y, v.y), std::max(hi.z, v.z)};
    }
    if (!touchesExact(lo, hi)) continue;
    bytes += 8 * sizeof(int32_t);
    for (int j = 0; j < 8; ++j) {
      const int id = m.indices[e * 8 + j];
      if (id < 0) break;
      if (!vertUsed[id]) { vertUsed[id] = 1; bytes += sizeof(exa_vec4f); }
    }
  }
  return bytes;
}
}  // namespace

int exa_surrogate_get_stats(exa_context *ctx, exa_surrogate_stats *out)
{
  return guarded([&] {
    need(ctx && ctx->surrogate && out, EXA_ERR_STATE, "no surrogate");
    setDevice(ctx);
    const Surrogate &S = *ctx->surrogate;
    std::memset(out, 0, sizeof(*out));
    out->loss = S.lastLoss;
    out->steps = S.step;
    out->tolerance = ctx->surrogateTol;
    out->rmse = S.stats.rmse;
    out->maxError = S.stats.maxError;
    out->probePoints = S.stats.probePoints;
    out->numMacrocells = S.stats.numMacrocells;
    out->numSurrogateMacrocells = S.stats.numSurrogateMCs;
    out->tableBytes = S.table16.bytes();
    out->weightBytes = S.wbf.bytes();
    out->inferenceBytes = S.inferenceBytes();
    const ExaStitchSampler &sm = esSampler(ctx);
    out->fieldBytes = sm.gridletBuffer.bytes() + sm.gridletScalarBuffer.bytes() + sm.vertexBuffer.bytes() +
                      sm.indexBuffer.bytes() + sm.accelBytes();
    out->fallbackFieldBytes = S.evaluated ? fallbackBytes(ctx) : out->fieldBytes;
  });
}

int exa_surrogate_get_geometry(exa_context *ctx, exa_surrogate_geometry *out)
{
  return guarded([&] {
    need(ctx && ctx->surrogate && out, EXA_ERR_STATE, "no surrogate");
    const SurrogateView &v = ctx->surrogate->view;
    std::memset(out, 0, sizeof(*out));
    out->log2TableSize = v.log2T;
    out->denseMask = v.denseMask;
    for (int l = 0; l < 16; ++l) out->res[l] = v.res[l];
    for (int a = 0; a < 3; ++a) { out->lo[a] = v.lo[a]; out->inv[a] = v.inv[a]; }
    out->vmin = v.vmin;
    out->vrange = v.vrange;
  });
}

int exa_surrogate_sample_points(exa_context *ctx, const exa_vec3f *posDevice, uint64_t n, float *outDevice)
{
  return guarded([&] {
    need(ctx && ctx->surrogate, EXA_ERR_STATE, "no surrogate");
    need(n == 0 || (posDevice && outDevice), EXA_ERR_INVALID, "null buffer");
    setDevice(ctx);
    launchSurrogatePoints(ctx->surrogate->deviceView(), posDevice, n, outDevice, ctx->stream);
  });
}

int exa_surrogate_get_params(exa_context *ctx, float *weights, float *table)
{
  return guarded([&] {
    need(ctx && ctx->surrogate, EXA_ERR_STATE, "no surrogate");
    setDevice(ctx);
    const Surrogate &S = *ctx->surrogate;
    if (weights) cudaCheck(cudaMemcpy(weights, S.w32.ptr, S.w32.bytes(), cudaMemcpyDeviceToHost), "d2h");
    if (table) cudaCheck(cudaMemcpy(table, S.table.ptr, S.table.bytes(), cudaMemcpyDeviceToHost), "d2h");
  });
}

int exa_surrogate_set_params(exa_context *ctx, const float *weights, const float *table)
{
  return guarded([&] {
    need(ctx && ctx->surrogate, EXA_ERR_STATE, "no surrogate");
    setDevice(ctx);
    Surrogate &S = *ctx->surrogate;
    if (weights) S.setWeights(weights, ctx->stream);
    if (table) S.setTable(table, ctx->stream);
    cudaCheck(cudaStreamSynchronize(ctx->stream), "surrogate params");
    S.evaluated = false;
  });
}

int exa_surrogate_gradients(exa_context *ctx, const float *pairs, int32_t n, float *gWeights, float *gTable,
                            float *loss)
{
  return guarded([&] {
    need(ctx && ctx->surrogate, EXA_ERR_STATE, "no surrogate");
    need(pairs != nullptr && n > 0, EXA_ERR_INVALID, "no pairs");
    setDevice(ctx);
    ctx->surrogate->gradients(reinterpret_cast<const float4 *>(pairs), n, gWeights, gTable, loss, ctx->stream);
  });
}

int exa_surrogate_get_macrocells(exa_context *ctx, uint8_t *mode, double *maxError, float *majorants)
{
  return guarded([&] {
    need(ctx && ctx->surrogate && ctx->surrogate->evaluated, EXA_ERR_STATE, "no evaluated surrogate");
    setDevice(ctx);
    const Surrogate &S = *ctx->surrogate;
    if (mode) cudaCheck(cudaMemcpy(mode, S.mcMode.ptr, S.mcMode.bytes(), cudaMemcpyDeviceToHost), "d2h");
    if (maxError) cudaCheck(cudaMemcpy(maxError, S.mcErr.ptr, S.mcErr.bytes(), cudaMemcpyDeviceToHost), "d2h");
    if (majorants) cudaCheck(cudaMemcpy(majorants, S.majorants.ptr, S.majorants.bytes(), cudaMemcpyDeviceToHost), "d2h");
  });
}

int exa_render_surrogate(exa_context *ctx, const exa_launch_params *lp, int32_t width, int32_t height)
{
  return guarded([&] { renderFrame(ctx, lp, width, height, true); });
}

// ------------------------------------------------------------ batched frames
namespace {
BatchState &batchOf(exa_context *ctx)
{
  if (!ctx->batch) ctx->batch = std::make_unique<BatchState>();
  return *ctx->batch;
}

// value ranges of the batch's majorant grid (Grid::build's kernels) and
// every transfer function's max opacities on it
void rebuildBatchMajorants(exa_context *ctx, BatchState &B)
{
  const ExaStitchSampler &S = esSampler(ctx);
  const ExaStitchModel &m = esModel(ctx);
  const size_t n = (size_t)B.dims.x * B.dims.y * B.dims.z;
  B.ranges.alloc(n);
  launchInitRanges(B.ranges.ptr, n, ctx->stream);
  DBuf<exa_range1f> gr, er;
  gr.alloc(std::max<size_t>(m.gridlets.size(), 1));
  er.alloc(std::max<size_t>(m.indices.size() / 8, 1));
  launchInitRanges(gr.ptr, gr.count, ctx->stream);
  launchInitRanges(er.ptr, er.count, ctx->stream);
  launchElemMajorants(S.vertexBuffer.ptr, S.indexBuffer.ptr, m.indices.size() / 8, B.dims, m.cellBounds, B.ranges.ptr,
                      er.ptr, ctx->stream);
  cudaCheck(cudaMemsetAsync(S.buildErrors.ptr, 0, sizeof(uint32_t), ctx->stream), "memset build errors");
  DBuf<uint32_t> scratch;
  scratch.alloc(m.gridlets.size() + 1);
  launchGridletMajorants(S.gridletBuffer.ptr, S.gridletScalarBuffer.ptr, m.gridlets.size(), m.gridletScalars.size(),
                         B.dims, m.cellBounds, B.ranges.ptr, gr.ptr, S.buildErrors.ptr, 0u, scratch.ptr, ctx->stream);
  B.maxOps.resize(B.tfColors.size());
  for (size_t t = 0; t < B.tfColors.size(); ++t) {
    B.maxOps[t].alloc(n);
    launchMaxOpacity(B.ranges.ptr, n, B.tfColors[t].ptr, B.tfCount[t], B.tfRange[t], ctx->sampler->tfFilter,
                     B.maxOps[t].ptr, ctx->stream);
  }
  cudaCheck(cudaStreamSynchronize(ctx->stream), "batch majorants");
  checkBuildErrors(S.buildErrors.ptr);
}

// the culling data of every transfer function (ExaStitchSampler::
// computeMaxOpacities for each one, into the batch's own buffers)
void rebuildBatchCulling(exa_context *ctx, BatchState &B)
{
  ExaStitchSampler &S = esSampler(ctx);
  const size_t ng = S.gridletValueRanges.count;
  const size_t nt = B.tfColors.size();
  B.gOps.clear();
  B.eOps.clear();
  B.gOps.resize(nt);
  B.eOps.resize(nt);
  std::vector<AccelView> views(nt, S.accel);
  for (size_t t = 0; t < nt; ++t) {
    B.gOps[t].alloc(std::max<size_t>(ng, 1));
    B.eOps[t].alloc(std::max<size_t>(S.elemValueRanges.count, 1));
    launchMaxOpacity(S.gridletValueRanges.ptr, ng, B.tfColors[t].ptr, B.tfCount[t], B.tfRange[t], S.tfFilter, B.gOps[t].ptr,
                     ctx->stream);
    launchMaxOpacity(S.elemValueRanges.ptr, S.elemValueRanges.count, B.tfColors[t].ptr, B.tfCount[t], B.tfRange[t], S.tfFilter,
                     B.eOps[t].ptr, ctx->stream);
    views[t].gridletMaxOps = B.gOps[t].ptr;
    views[t].elemMaxOps = B.eOps[t].ptr;
  }
  B.accels.upload(views.data(), nt, ctx->stream);
  cudaCheck(cudaStreamSynchronize(ctx->stream), "batch culling");
}

void renderBatch(exa_context *ctx, const exa_launch_params *tpl, const exa_batch_frame *fr, int numFrames,
                 bool useGraph)
{
  need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
  need(tpl != nullptr && fr != nullptr && numFrames > 0, EXA_ERR_INVALID, "no frames");
  BatchState &B = batchOf(ctx);
  need(!B.tfColors.empty(), EXA_ERR_STATE, "no transfer functions (exa_batch_set_transfer_functions)");
  need(tpl->integrator == EXA_PATH_TRACING_INTEGRATOR || tpl->integrator == EXA_DIRECT_LIGHT_INTEGRATOR,
       EXA_ERR_INVALID, "integrator not supported (batches render path tracing and direct lighting)");
  need(tpl->shadeMode == EXA_SHADE_MODE_DEFAULT || tpl->shadeMode == EXA_SHADE_MODE_GRIDLETS, EXA_ERR_INVALID,
       "shade mode not supported");
  need(!tpl->subImage.active && !tpl->render.heatMapEnabled && tpl->meshBVH == 0, EXA_ERR_INVALID,
       "sub-image, heat map and surface meshes are not supported");
  need(tpl->sampler.ess.sampleBVH == (uint64_t)(uintptr_t)ctx->sampler->deviceAccel.ptr, EXA_ERR_INVALID,
       "lpTemplate.sampler.ess.sampleBVH is not this context's sampler (call exa_sampler_set_lps)");
  need(tpl->ext.maxBounces >= 0, EXA_ERR_INVALID, "maxBounces must be >= 0");
  needLpCaps(*tpl, ctx->sampler->tfFilter);
  need(tpl->ext.rowEnd <= 0, EXA_ERR_INVALID, "row bands are not supported in batches");
  need(B.tileW == 8 || B.tileW == 16 || B.tileW == 32, EXA_ERR_INVALID, "bad tile width");
  setDevice(ctx);
  const int th = 128 / B.tileW;
  std::vector<exa_launch_params> lps((size_t)numFrames);
  std::vector<WfFrame> frames((size_t)numFrames);
  unsigned long long jobs = 0, samples = 0, pixels = 0;
  for (int i = 0; i < numFrames; ++i) {
    const exa_batch_frame &f = fr[i];
    need(f.width > 0 && f.height > 0 && f.spp >= 1, EXA_ERR_INVALID, "bad frame size or spp");
    need(f.tf >= 0 && f.tf < (int)B.tfColors.size(), EXA_ERR_INVALID, "frame transfer function out of range");
    need(f.accumID == 0 || f.accumBuffer != nullptr, EXA_ERR_INVALID, "accumID > 0 needs an accumBuffer");
    exa_launch_params lp = *tpl;
    lp.camera.org = f.org;
    lp.camera.dir_00 = f.dir_00;
    lp.camera.dir_du = f.dir_du;
    lp.camera.dir_dv = f.dir_dv;
    lp.render.spp = f.spp;
    lp.accumID = (int32_t)f.accumID;
    lp.ext.frameID = f.frameID;
    lp.fbPointer = f.fbPointer;
    lp.accumBuffer = f.accumBuffer;
    lp.transferFunc.values = reinterpret_cast<exa_vec4f *>(B.tfColors[f.tf].ptr);
    lp.transferFunc.numValues = B.tfCount[f.tf];
    lp.transferFunc.domain = B.tfRange[f.tf];
    lp.transferFunc.opacityScale = B.tfScale[f.tf];
    lp.maxOpacities = B.maxOps[f.tf].ptr;
    lp.majorantGrid.dims = B.dims;
    lp.majorantGrid.bounds = ctx->model->cellBounds;
    fillLoopCaps(lp);
    lp.ext.traceT = nullptr;
    lp.ext.traceTr = nullptr;
    lp.ext.deviceErrors = ctx->errors.ptr;
    lps[i] = lp;
    WfFrame &F = frames[i];
    F.width = f.width;
    F.height = f.height;
    F.tf = f.tf;
    F.pad = 0;
    F.jobBase = jobs;
    F.sampleBase = samples;
    F.pixelBase = pixels;
    jobs += (unsigned long long)((f.width + B.tileW - 1) / B.tileW) * ((f.height + th - 1) / th) * 128ull *
            (unsigned long long)f.spp;
    samples += (unsigned long long)f.width * f.height * f.spp;
    pixels += (unsigned long long)f.width * f.height;
  }
  // lps / frames keep their device addresses while the batch size stays
  if (B.lps.count != (size_t)numFrames) {
    B.lps.alloc(numFrames);
    B.frames.alloc(numFrames);
  }
  cudaCheck(cudaMemcpyAsync(B.lps.ptr, lps.data(), lps.size() * sizeof(exa_launch_params), cudaMemcpyHostToDevice,
                            ctx->stream), "frame table");
  cudaCheck(cudaMemcpyAsync(B.frames.ptr, frames.data(), frames.size() * sizeof(WfFrame), cudaMemcpyHostToDevice,
                            ctx->stream), "frame table");
  if (!B.ctl.ptr) B.ctl.alloc(1);
  if (B.colors.count < samples) B.colors.alloc(samples);
  const unsigned cap = (unsigned)std::min<unsigned long long>(jobs, 1ull << 22);
  if (B.cap < cap) {
    B.records.alloc((size_t)3 * kWfLaneWords * cap);
    B.counters.alloc(4);
    B.cap = cap;
  }
  WfBatchView V;
  V.accels = B.accels.ptr;
  V.lps = B.lps.ptr;
  V.frames = B.frames.ptr;
  V.numFrames = numFrames;
  V.tileW = B.tileW;
  V.totalJobs = jobs;
  V.totalPixels = pixels;
  renderWavefrontBatch(ctx->sampler->accel, lps[0], V, B.records.ptr, B.cap, B.counters.ptr, B.ctl.ptr, B.colors.ptr,
                       ctx->errors.ptr, useGraph, &B.graph, ctx->stream, &B.last);
  ctx->lastStats = exa_render_stats{};
  ctx->lastStats.wavefront = 2;
  ctx->lastStats.rounds = B.last.rounds;
  ctx->lastStats.peakQueue = B.last.peakQueue;
  ctx->lastStats.queueCapacity = B.cap;
  ctx->lastStats.walkLaunches = B.last.walkLaunches;
  ctx->lastStats.walkMs = B.last.walkMs;
}
}  // namespace

int exa_batch_set_transfer_functions(exa_context *ctx, int32_t numTFs, const exa_vec4f *const *colorMaps,
                                     const int32_t *numColors, const exa_range1f *xfRanges,
                                     const float *opacityScales)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(numTFs > 0 && colorMaps && numColors && xfRanges, EXA_ERR_INVALID, "no transfer functions");
    setDevice(ctx);
    BatchState &B = batchOf(ctx);
    B.tfColors.clear();
    B.tfColors.resize(numTFs);
    B.tfCount.assign(numTFs, 0);
    B.tfRange.assign(xfRanges, xfRanges + numTFs);
    B.tfScale.assign(numTFs, 1.f);
    for (int t = 0; t < numTFs; ++t) {
      need(colorMaps[t] && numColors[t] > 0, EXA_ERR_INVALID, "empty colour map");
      B.tfColors[t].upload(reinterpret_cast<const float4 *>(colorMaps[t]), (size_t)numColors[t], ctx->stream);
      B.tfCount[t] = numColors[t];
      if (opacityScales) B.tfScale[t] = opacityScales[t];
    }
    if (B.dims.x == 0) B.dims = ctx->model->grid->dims;
    rebuildBatchMajorants(ctx, B);
    rebuildBatchCulling(ctx, B);
  });
}

int exa_batch_set_majorant_grid(exa_context *ctx, exa_vec3i dims)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(dims.x > 0 && dims.y > 0 && dims.z > 0 && (int64_t)dims.x * dims.y * dims.z <= (1ll << 30), EXA_ERR_INVALID,
         "bad majorant grid");
    setDevice(ctx);
    BatchState &B = batchOf(ctx);
    B.dims = dims;
    rebuildBatchMajorants(ctx, B);
  });
}

int exa_batch_set_tile_width(exa_context *ctx, int32_t tileWidth)
{
  return guarded([&] {
    need(ctx != nullptr, EXA_ERR_STATE, "no context");
    need(tileWidth == 8 || tileWidth == 16 || tileWidth == 32, EXA_ERR_INVALID, "tile width must be 8, 16 or 32");
    batchOf(ctx).tileW = tileWidth;
  });
}

int exa_render_batch(exa_context *ctx, const exa_launch_params *lpTemplate, const exa_batch_frame *frames,
                     int32_t numFrames, int32_t useGraph)
{
  return guarded([&] { renderBatch(ctx, lpTemplate, frames, numFrames, useGraph != 0); });
}

int exa_batch_autotune(exa_context *ctx, const exa_launch_params *lpTemplate, const exa_batch_frame *frames,
                       int32_t numFrames, int32_t sampleEvery, exa_batch_tuning *out)
{
  return guarded([&] {
    need(ctx && ctx->sampler && frames && numFrames > 0 && out, EXA_ERR_INVALID, "bad arguments");
    need(sampleEvery >= 1, EXA_ERR_INVALID, "sampleEvery must be >= 1");
    setDevice(ctx);
    BatchState &B = batchOf(ctx);
    need(!B.tfColors.empty(), EXA_ERR_STATE, "no transfer functions (exa_batch_set_transfer_functions)");
    // the sampled workload: every sampleEvery-th frame at 1 spp, no outputs
    std::vector<exa_batch_frame> sub;
    for (int i = 0; i < numFrames; i += sampleEvery) {
      exa_batch_frame f = frames[i];
      f.spp = 1;
      f.accumID = 0;
      f.fbPointer = nullptr;
      f.accumBuffer = nullptr;
      sub.push_back(f);
    }
    std::memset(out, 0, sizeof(*out));
    const int res[4] = {32, 64, 128, 256};
    const int tiles[3] = {8, 16, 32};
    cudaEvent_t e0, e1;
    cudaCheck(cudaEventCreate(&e0), "cudaEventCreate");
    cudaCheck(cudaEventCreate(&e1), "cudaEventCreate");
    struct EvGuard {
      cudaEvent_t a, b;
      ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } evGuard{e0, e1};
    float best = 1e30f;
    exa_vec3i bestDims{0, 0, 0};
    int bestTile = 16;
    for (int r : res) {
      B.dims = exa_vec3i{r, r, r};
      rebuildBatchMajorants(ctx, B);
      for (int tw : tiles) {
        B.tileW = tw;
        renderBatch(ctx, lpTemplate, sub.data(), (int)sub.size(), true);  // builds the graph
        cudaCheck(cudaEventRecord(e0, ctx->stream), "event");
        renderBatch(ctx, lpTemplate, sub.data(), (int)sub.size(), true);
        cudaCheck(cudaEventRecord(e1, ctx->stream), "event");
        cudaCheck(cudaStreamSynchronize(ctx->stream), "autotune");
        float ms = 0.f;
        cudaCheck(cudaEventElapsedTime(&ms, e0, e1), "event time");
        const int k = out->numTrials++;
        out->trialDims[k] = B.dims;
        out->trialTileWidth[k] = tw;
        out->trialMs[k] = ms;
        if (ms < best) { best = ms; bestDims = B.dims; bestTile = tw; }
      }
    }
    B.dims = bestDims;
    B.tileW = bestTile;
    rebuildBatchMajorants(ctx, B);
    out->dims = bestDims;
    out->tileWidth = bestTile;
    out->msBest = best;
  });
}

} // extern "C"

// ================================================================ no-alloc
// Scratch of exa_render_noalloc: one colour per camera sample, in the
// library's device image instead of a cudaMalloc'd buffer.  The host-side
// name is a stand-in for the symbol; kernels get the device address that
// cudaGetSymbolAddress returns (looked up once per device).
static __device__ __align__(256) float4 g_noallocSampleColors[EXA_NOALLOC_MAX_SAMPLES];

namespace {
std::mutex g_noallocMutex;
float4 *g_noallocAddr[256] = {};
}

extern "C" int exa_render_noalloc(exa_context *ctx, const exa_launch_params *lp, int32_t width, int32_t height)
{
  return guarded([&] {
    need(ctx && ctx->sampler, EXA_ERR_STATE, "sampler not built");
    need(lp != nullptr, EXA_ERR_INVALID, "null lp");
    need(width > 0 && height > 0, EXA_ERR_INVALID, "bad frame size");
    need(lp->render.spp >= 1, EXA_ERR_INVALID, "spp must be >= 1");
    const unsigned long long samples = (unsigned long long)width * (unsigned long long)height * (unsigned)lp->render.spp;
    if (samples > EXA_NOALLOC_MAX_SAMPLES)
      throw Error(EXA_ERR_INVALID, "exa_render_noalloc: width*height*spp = " + std::to_string(samples) +
                                       " exceeds its static scratch of " + std::to_string(EXA_NOALLOC_MAX_SAMPLES) +
                                       " samples; use exa_render for larger frames");
    need(lp->integrator == EXA_PATH_TRACING_INTEGRATOR || lp->integrator == EXA_DIRECT_LIGHT_INTEGRATOR,
         EXA_ERR_INVALID, "integrator not supported (exa_render_noalloc renders path tracing and direct lighting)");
    need(lp->shadeMode == EXA_SHADE_MODE_DEFAULT || lp->shadeMode == EXA_SHADE_MODE_GRIDLETS, EXA_ERR_INVALID,
         "shade mode not supported");
    need(!lp->clipPlanes[0].enabled, EXA_ERR_INVALID, "clip planes are not supported");
    need(!lp->subImage.active && !lp->render.heatMapEnabled, EXA_ERR_INVALID, "sub-image / heat map not supported");
    need(lp->meshBVH == 0, EXA_ERR_INVALID, "surface meshes are not supported");
    need(lp->sampler.ess.sampleBVH == (uint64_t)(uintptr_t)ctx->sampler->deviceAccel.ptr, EXA_ERR_INVALID,
         "lp.sampler.ess.sampleBVH is not this context's sampler (call exa_sampler_set_lps)");
    need(lp->maxOpacities != nullptr && lp->transferFunc.values != nullptr, EXA_ERR_STATE,
         "no transfer function (call exa_sampler_compute_max_opacities and exa_sampler_set_lps)");
    need(lp->ext.maxBounces >= 0, EXA_ERR_INVALID, "maxBounces must be >= 0");
    needLpCaps(*lp, ctx->sampler->tfFilter);
    needGridDims(ctx, *lp);
    need(lp->ext.rowEnd <= 0, EXA_ERR_INVALID, "row bands are not supported (exa_render renders them)");
    // as in exa_render: the AMR-cell and ExaBrick samplers have no gridlet
    // cells to colour
    need((ctx->sampler->accel.amr == nullptr && ctx->sampler->accel.bricks == nullptr) ||
             lp->shadeMode == EXA_SHADE_MODE_DEFAULT,
         EXA_ERR_INVALID, "the AMR-cell and ExaBrick samplers render shade mode default only");
    need(ctx->device >= 0 && ctx->device < 256, EXA_ERR_INVALID, "device index out of range");
    setDevice(ctx);
    float4 *scratch = nullptr;
    {
      std::lock_guard<std::mutex> lock(g_noallocMutex);
      if (!g_noallocAddr[ctx->device]) {
        void *p = nullptr;
        cudaCheck(cudaGetSymbolAddress(&p, g_noallocSampleColors), "cudaGetSymbolAddress(noalloc scratch)");
        g_noallocAddr[ctx->device] = static_cast<float4 *>(p);
      }
      scratch = g_noallocAddr[ctx->device];
    }
    exa_launch_params lpUse = *lp;
    fillLoopCaps(lpUse);
    launchRender(ctx->sampler->accel, lpUse, width, height, ctx->jobCounter.ptr, scratch, ctx->stream);
  });
}
