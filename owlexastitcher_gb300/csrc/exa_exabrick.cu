// exa_exabrick.cu -- the ExaBrick comparison sampler: the model's active
// brick regions (model/ABRs.cpp), the sampler's device buffers, region LBVH
// and majorant grid (sampler/ExaBrickSampler.cpp, Grid.cu:362-430).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <utility>
#include <vector>

#include "exa_host.h"

namespace exa {

namespace {

struct Box {
  float lo[3], hi[3];
};

// ExaBrick::getDomain (model/ABRs.h:42-47): the brick grown by half a cell
Box brick_domain(const exa_brick &b)
{
  const float cw = (float)(1 << b.level);
  const int lower[3] = {b.lower.x, b.lower.y, b.lower.z}, size[3] = {b.size.x, b.size.y, b.size.z};
  Box d;
  for (int a = 0; a < 3; ++a) {
    d.lo[a] = (float)lower[a] - 0.5f * cw;
    d.hi[a] = (float)lower[a] + ((float)size[a] + 0.5f) * cw;
  }
  return d;
}

using Prim = std::pair<Box, int>;

// ABRs::buildRec / addLeaf (model/ABRs.cpp:33-209), restated: split at the
// primitive face closest to the domain centre, trying the widest axis first
// (ties: the lowest axis), partition the clipped primitives, recurse into
// the upper half first; a domain without a split is a region listing its
// bricks in ascending id order.
struct AbrBuilder {
  std::vector<exa_abr> &abrs;
  std::vector<int32_t> &leafList;

  void addLeaf(const std::vector<Prim> &prims, const Box &d)
  {
    for (int a = 0; a < 3; ++a)
      if (d.lo[a] >= d.hi[a]) return;
    std::set<int> ids;
    for (const Prim &p : prims) ids.insert(p.second);
    if (ids.empty()) return;
    exa_abr r;
    std::memset(&r, 0, sizeof(r));
    r.domain.lower = {d.lo[0], d.lo[1], d.lo[2]};
    r.domain.upper = {d.hi[0], d.hi[1], d.hi[2]};
    r.leafListBegin = (int32_t)leafList.size();
    r.leafListSize = (int32_t)ids.size();
    for (int id : ids) leafList.push_back(id);
    abrs.push_back(r);
  }

  void buildRec(std::vector<Prim> &prims, const Box &d)
  {
    if (prims.empty()) return;
    for (int a = 0; a < 3; ++a)
      if (d.hi[a] == d.lo[a]) return;
    float tgt[3], bestPos[3], bestDist[3], span[3];
    for (int a = 0; a < 3; ++a) {
      tgt[a] = (d.lo[a] + d.hi[a]) * 0.5f;
      bestPos[a] = d.lo[a];
      span[a] = d.hi[a] - d.lo[a];
      bestDist[a] = span[a];
    }
    for (const Prim &p : prims)
      for (int dim = 0; dim < 3; ++dim)
        for (int side = 0; side < 2; ++side) {
          const float pos = side ? p.first.lo[dim] : p.first.hi[dim];
          if (pos <= d.lo[dim] || pos >= d.hi[dim]) continue;
          const float dist = std::fabs(tgt[dim] - pos);
          if (dist < bestDist[dim]) {
            bestPos[dim] = pos;
            bestDist[dim] = dist;
          }
        }
    const int widest = (span[0] >= span[1] && span[0] >= span[2]) ? 0 : (span[1] >= span[2] ? 1 : 2);
    int splitDim = -1;
    float splitPos = 0.f;
    for (int i = 0; i < 3; ++i) {
      const int dim = (widest + i) % 3;
      if (bestPos[dim] <= d.lo[dim] || bestPos[dim] >= d.hi[dim]) continue;
      splitDim = dim;
      splitPos = bestPos[dim];
      break;
    }
    if (splitDim < 0) {
      addLeaf(prims, d);
      return;
    }
    Box dl = d, dr = d;
    dl.hi[splitDim] = splitPos;
    dr.lo[splitDim] = splitPos;
    std::vector<Prim> pl, pr;
    for (const Prim &p : prims) {
      Box cl, cr;
      bool okl = true, okr = true;
      for (int a = 0; a < 3; ++a) {
        cl.lo[a] = std::max(p.first.lo[a], dl.lo[a]);
        cl.hi[a] = std::min(p.first.hi[a], dl.hi[a]);
        cr.lo[a] = std::max(p.first.lo[a], dr.lo[a]);
        cr.hi[a] = std::min(p.first.hi[a], dr.hi[a]);
        okl = okl && cl.lo[a] < cl.hi[a];
        okr = okr && cr.lo[a] < cr.hi[a];
      }
      if (okl) pl.push_back({cl, p.second});
      if (okr) pr.push_back({cr, p.second});
    }
    prims.clear();
    prims.shrink_to_fit();
    buildRec(pr, dr);
    buildRec(pl, dl);
  }
};

// ABRs::computeValueRange (model/ABRs.cpp:212-262): the scalars of the
// cells whose basis support ([centre - w, centre + w]) meets the region
void abr_value_range(exa_abr &r, const exa_brick *bricks, const float *scalars, const int32_t *leafList)
{
  r.valueRange = exa_range1f{1e30f, -1e30f};
  const float dlo[3] = {r.domain.lower.x, r.domain.lower.y, r.domain.lower.z};
  const float dhi[3] = {r.domain.upper.x, r.domain.upper.y, r.domain.upper.z};
  for (int i = 0; i < r.leafListSize; ++i) {
    const exa_brick &b = bricks[leafList[r.leafListBegin + i]];
    const float cw = (float)(1 << b.level);
    const int lower[3] = {b.lower.x, b.lower.y, b.lower.z}, size[3] = {b.size.x, b.size.y, b.size.z};
    std::vector<char> valid[3];
    for (int a = 0; a < 3; ++a) {
      valid[a].resize(size[a]);
      for (int k = 0; k < size[a]; ++k) {
        const float pos = (float)lower[a] + ((float)k + .5f) * cw;
        const float lo = pos - cw, hi = pos + cw;
        valid[a][k] = (lo <= dhi[a]) && (hi >= dlo[a]);
      }
    }
    for (int iz = 0; iz < size[2]; ++iz) {
      if (!valid[2][iz]) continue;
      for (int iy = 0; iy < size[1]; ++iy) {
        if (!valid[1][iy]) continue;
        for (int ix = 0; ix < size[0]; ++ix) {
          if (!valid[0][ix]) continue;
          const float v = scalars[(size_t)b.begin + ix + (size_t)size[0] * iy + (size_t)size[0] * size[1] * iz];
          if (v < r.valueRange.lower) r.valueRange.lower = v;
          if (r.valueRange.upper < v) r.valueRange.upper = v;
        }
      }
    }
  }
}

} // namespace

// ExaBrickModel::load(bricks, scalars, n) (model/ExaBrickModel.cpp:120-143)
void ExaBrickModel::assign(const exa_brick *b, size_t nb, const float *s, size_t ns)
{
  for (size_t i = 0; i < nb; ++i) {
    if (b[i].level < 0 || b[i].level > 30) throw Error(EXA_ERR_INVALID, "brick level out of range");
    if (b[i].size.x < 1 || b[i].size.y < 1 || b[i].size.z < 1) throw Error(EXA_ERR_INVALID, "empty brick");
    const uint64_t n = (uint64_t)b[i].size.x * b[i].size.y * b[i].size.z;
    if ((uint64_t)b[i].begin + n > ns) throw Error(EXA_ERR_INVALID, "brick scalars past the end of the scalars");
  }
  bricks.assign(b, b + nb);
  scalars.assign(s, s + ns);
  init();
}

// ExaBrickModel::init (model/ExaBrickModel.cpp:145-168) with
// ABRs::buildFrom (model/ABRs.cpp:264-333)
void ExaBrickModel::init()
{
  abrs.clear();
  leafList.clear();
  std::vector<Prim> prims;
  prims.reserve(bricks.size());
  Box bounds;
  for (int a = 0; a < 3; ++a) {
    bounds.lo[a] = INFINITY;
    bounds.hi[a] = -INFINITY;
  }
  for (size_t i = 0; i < bricks.size(); ++i) {
    const Box d = brick_domain(bricks[i]);
    for (int a = 0; a < 3; ++a) {
      bounds.lo[a] = std::min(bounds.lo[a], d.lo[a]);
      bounds.hi[a] = std::max(bounds.hi[a], d.hi[a]);
    }
    prims.push_back({d, (int)i});
  }
  AbrBuilder B{abrs, leafList};
  B.buildRec(prims, bounds);
  for (exa_abr &r : abrs) {
    int finest = 1 << 30;
    for (int i = 0; i < r.leafListSize; ++i) finest = std::min(finest, (int)bricks[leafList[r.leafListBegin + i]].level);
    r.finestLevelCellWidth = (float)(1 << finest);
    abr_value_range(r, bricks.data(), scalars.data(), leafList.data());
  }
  exa_box3f cb;
  cb.lower = {INFINITY, INFINITY, INFINITY};
  cb.upper = {-INFINITY, -INFINITY, -INFINITY};
  for (const exa_brick &b : bricks) {
    // ExaBrick::getBounds (model/ABRs.h:35-40)
    const int w = 1 << b.level;
    const float lo[3] = {(float)b.lower.x, (float)b.lower.y, (float)b.lower.z};
    const float hi[3] = {(float)(b.lower.x + b.size.x * w), (float)(b.lower.y + b.size.y * w),
                         (float)(b.lower.z + b.size.z * w)};
    cb.lower = {std::min(cb.lower.x, lo[0]), std::min(cb.lower.y, lo[1]), std::min(cb.lower.z, lo[2])};
    cb.upper = {std::max(cb.upper.x, hi[0]), std::max(cb.upper.y, hi[1]), std::max(cb.upper.z, hi[2])};
  }
  cellBounds = cb;
  exa_range1f vr{1e30f, -1e30f};
  for (const exa_abr &r : abrs) {
    vr.lower = std::min(vr.lower, r.valueRange.lower);
    vr.upper = std::max(vr.upper, r.valueRange.upper);
  }
  valueRange = vr;
}

// ExaBrickModel::memStats (model/ExaBrickModel.cpp:214-225)
void ExaBrickModel::memStats(size_t &bricksBytes, size_t &scalarsBytes, size_t &abrsBytes,
                             size_t &leafListBytes) const
{
  bricksBytes = bricks.size() * sizeof(exa_brick);
  scalarsBytes = scalars.size() * sizeof(float);
  abrsBytes = abrs.size() * sizeof(exa_abr);
  leafListBytes = leafList.size() * sizeof(int32_t);
}

size_t ExaBrickSampler::fieldBytes() const { return brickBuffer.bytes() + scalarBuffer.bytes(); }

size_t ExaBrickSampler::accelBytes() const
{
  return abrBuffer.bytes() + abrLeafListBuffer.bytes() + abrCorners.bytes() + abrRows.bytes() + abrNodes.bytes() +
         abrParents.bytes() + abrLeafElem.bytes() + deviceView.bytes();
}

namespace {
inline unsigned gridFor(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }
} // namespace

// Grid.cu:399-430 (the active branch of the ExaBrick Grid::build): per brick
// cell, its box grown by half a cell projected onto the grid; NaN values
// add nothing (std::min / std::max keep the running value).  One block per
// brick.
__global__ void k_brick_majorants(const exa_brick *__restrict__ bricks, const float *__restrict__ scalars,
                                  exa_vec3i dims, exa_box3f wb, exa_range1f *mcRanges)
{
  const exa_brick b = bricks[blockIdx.x];
  const int n = b.size.x * b.size.y * b.size.z;
  const int w = 1 << b.level;
  const float half = (float)w * .5f;
  const V3i D = {dims.x, dims.y, dims.z};
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const int x = c % b.size.x, y = c / b.size.x % b.size.y, z = c / (b.size.x * b.size.y);
    const float value = scalars[(size_t)b.begin + x + (size_t)b.size.x * (y + (size_t)b.size.y * z)];
    if (isnan(value)) continue;
    const int lx = b.lower.x + x * w, ly = b.lower.y + y * w, lz = b.lower.z + z * w;
    const V3 lo = mk3((float)lx - half, (float)ly - half, (float)lz - half);
    const V3 hi = mk3((float)(lx + w) + half, (float)(ly + w) + half, (float)(lz + w) + half);
    const V3i a = project_on_grid(lo, D, wb), e = project_on_grid(hi, D, wb);
    for (int mz = a.z; mz <= e.z; ++mz)
      for (int my = a.y; my <= e.y; ++my)
        for (int mx = a.x; mx <= e.x; ++mx) {
          exa_range1f *m = mcRanges + ((size_t)mz * dims.y + my) * dims.x + mx;
          atomic_min_float(&m->lower, value);
          atomic_max_float(&m->upper, value);
        }
  }
}

void launchBrickMajorants(const exa_brick *bricks, size_t nb, const float *scalars, exa_vec3i dims, exa_box3f wb,
                          exa_range1f *mcRanges, cudaStream_t s)
{
  if (!nb) return;
  if (nb >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "too many bricks");
  k_brick_majorants<<<(unsigned)nb, 128, 0, s>>>(bricks, scalars, dims, wb, mcRanges);
  cudaCheck(cudaGetLastError(), "k_brick_majorants");
}

// ExaBrickSampler::build (sampler/ExaBrickSampler.cpp:26-128), grid + DDA
// traversal with ABR sampling
bool ExaBrickSampler::build(std::shared_ptr<Model> mod, cudaStream_t s)
{
  if (!mod) return false;
  model = std::dynamic_pointer_cast<ExaBrickModel>(mod);
  if (!model || model->bricks.empty() || model->abrs.empty()) return false;
  if (!model->grid || model->grid->dims.x == 0) return false;
  const ExaBrickModel &m = *model;
  brickBuffer.upload(m.bricks.data(), m.bricks.size(), s);
  scalarBuffer.upload(m.scalars.data(), m.scalars.size(), s);
  abrBuffer.upload(m.abrs.data(), m.abrs.size(), s);
  abrLeafListBuffer.upload(m.leafList.data(), m.leafList.size(), s);
  // the region LBVH: each region a row of its two domain corners
  const size_t na = m.abrs.size();
  if (na >= 0x3fffffffull) throw Error(EXA_ERR_INVALID, "too many brick regions");
  std::vector<float4> corners(2 * na);
  std::vector<int32_t> rows(8 * na, -1);
  exa_box3f sb;
  sb.lower = {INFINITY, INFINITY, INFINITY};
  sb.upper = {-INFINITY, -INFINITY, -INFINITY};
  for (size_t i = 0; i < na; ++i) {
    const exa_box3f &d = m.abrs[i].domain;
    corners[2 * i] = make_float4(d.lower.x, d.lower.y, d.lower.z, 0.f);
    corners[2 * i + 1] = make_float4(d.upper.x, d.upper.y, d.upper.z, 0.f);
    rows[8 * i] = (int32_t)(2 * i);
    rows[8 * i + 1] = (int32_t)(2 * i + 1);
    sb.lower = {std::min(sb.lower.x, d.lower.x), std::min(sb.lower.y, d.lower.y), std::min(sb.lower.z, d.lower.z)};
    sb.upper = {std::max(sb.upper.x, d.upper.x), std::max(sb.upper.y, d.upper.y), std::max(sb.upper.z, d.upper.z)};
  }
  abrCorners.upload(corners.data(), corners.size(), s);
  abrRows.upload(rows.data(), rows.size(), s);
  abrNodes.alloc(na > 1 ? na - 1 : 1);
  abrParents.alloc((na > 1 ? na - 1 : 0) + na);
  abrLeafElem.alloc(na);
  launchBuildBVH(abrCorners.ptr, abrRows.ptr, na, sb, abrNodes.ptr, abrParents.ptr, abrLeafElem.ptr, s);
  std::memset(&view, 0, sizeof(view));
  view.bricks = brickBuffer.ptr;
  view.scalars = scalarBuffer.ptr;
  view.abrs = abrBuffer.ptr;
  view.leafList = abrLeafListBuffer.ptr;
  view.nodes = abrNodes.ptr;
  view.numAbrs = (int)na;
  deviceView.upload(&view, 1, s);
  std::memset(&accel, 0, sizeof(accel));
  accel.bricks = deviceView.ptr;
  // the majorant grid over cellBounds (Grid.cu:362-430)
  Grid &g = *model->grid;
  g.worldBounds = model->cellBounds;
  const size_t numMCs = (size_t)g.dims.x * g.dims.y * g.dims.z;
  g.valueRanges.alloc(numMCs);
  g.maxOpacities.alloc(numMCs);
  cudaCheck(cudaMemsetAsync(g.maxOpacities.ptr, 0, g.maxOpacities.bytes(), s), "memset maxOpacities");
  launchInitRanges(g.valueRanges.ptr, numMCs, s);
  launchBrickMajorants(brickBuffer.ptr, m.bricks.size(), scalarBuffer.ptr, g.dims, g.worldBounds, g.valueRanges.ptr,
                       s);
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

// Grid::computeMaxOpacities for the grid traversal mode
// (ExaBrickSampler.cpp:185-200)
void ExaBrickSampler::computeMaxOpacities(const exa_vec4f *cmap, int numColors, exa_range1f xf, cudaStream_t s)
{
  if (!model || !model->grid || model->grid->dims.x == 0) return;
  if (numColors <= 0) throw Error(EXA_ERR_INVALID, "empty color map");
  colorMap.upload(reinterpret_cast<const float4 *>(cmap), (size_t)numColors, s);
  Grid &g = *model->grid;
  launchMaxOpacity(g.valueRanges.ptr, g.valueRanges.count, colorMap.ptr, numColors, xf, tfFilter, g.maxOpacities.ptr, s);
  cudaCheck(cudaStreamSynchronize(s), "computeMaxOpacities");
  hasTF = true;
}

// ExaBrickSampler::setLPs (ExaBrickSampler.cpp:167-178)
void ExaBrickSampler::setLPs(exa_launch_params &lp)
{
  std::memset(&lp.sampler, 0, sizeof(lp.sampler));
  lp.sampler.ebs.sampleBVH = (uint64_t)(uintptr_t)deviceAccel.ptr;
  lp.sampler.ebs.brickBuffer = brickBuffer.ptr;
  lp.sampler.ebs.abrBuffer = abrBuffer.ptr;
  lp.sampler.ebs.scalarBuffer = scalarBuffer.ptr;
  lp.sampler.ebs.abrLeafListBuffer = abrLeafListBuffer.ptr;
}

} // namespace exa
