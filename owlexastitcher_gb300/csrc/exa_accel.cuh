// exa_accel.cuh -- point location for the ExaStitch field, replacing the
// OptiX TLAS over the gridlet and stitching-element BLASes
// (sampler/ExaStitchSampler.cpp:71-323) and the zero-length-ray query of
// sample() (sampler/ExaStitchSampler.h:128-140).
//
// Gridlets: block tables over a dual-cell lattice, one entry per
// 2^shift-wide block (8 for makeGrids bricks, makeGrids.cpp:46): one table
// over the finest level's lattice listing the gridlets of every level, or,
// when that grid would be too large, one table per level.  An entry holds
// the single gridlet whose extent meets the block's open interior, or an
// ascending list.  A query on an exact block face also looks at the
// neighbouring block, so the reference's inclusive box test is honoured.
// Stitching elements: a uniform grid of cells over the elements' bounds
// (about two finest-cell widths wide); a bit per cell marks the cells that
// some element's closed AABB touches, and each marked cell lists those
// elements in ascending order, so the first element that holds the point
// is the lowest-index one.
//
// Canonical answer when several primitives contain the point (shared
// faces): the lowest-index gridlet, else the lowest-index element.
// Primitives whose max opacity is 0 are invisible when culling (the
// reference gives them empty AABBs: programs/ExaStitchSampler.cu:35-41,81-83).
#pragma once

#include "exa_device.cuh"

namespace exa {

constexpr int kMaxLevels = 16;
constexpr int kBvhStack = 64;

struct GridletTable {
  int level;
  int shift;       // block width 2^shift dual cells
  int origin[3];   // lattice coordinate of block (0,0,0)
  int n[3];        // blocks per axis
  const int32_t *entries;  // -1 empty; >= 0 gridlet; <= -2 list at items[-e-2]
  const int32_t *items;    // list: count, ids ascending
  int numItems;            // length of items (for the bounds-checked build)
};

struct BvhNode {   // 64 B: two child boxes, two child refs (ExaBrick regions, surface meshes)
  float lo0[3], hi0[3];
  float lo1[3], hi1[3];
  int32_t child[2];     // >= 0 internal node, < 0 leaf ~child
  float op[2];          // 1 (the trees are not culled; keeps the 64-byte node)
};

// Element cells: one bit per cell of a uniform grid over the elements'
// bounds, set where any element's closed AABB touches the cell.
// cell(p) = floor((p - origin) / width) is monotonic in p, so a point
// inside an element's AABB always maps to a marked cell that lists the
// element; a clear bit proves no element contains the point.  Marked cells
// are numbered in cell order (rank: the marked cells before each 32-cell
// word); entry of a marked cell: >= 0 its only element, <= -2 a list at
// items[-e-2] (count, then the ids ascending).
struct ElemOccupancy {
  float origin[3];
  float invCell[3];        // 1 / cell width (the width a power of two)
  int n[3];
  const uint32_t *bits;
  const uint32_t *rank;
  const int32_t *entries;
  const int32_t *items;
  const float4 *boxes;     // per element its closed AABB: (lo, hi.x), (hi.y, hi.z, 0, 0)
  int numMarked, numItems;
};

// AMR cells (the comparison sampler of sampler/AMRCellSampler.h): per level
// a dense box of the level's cell lattice with one existence bit per cell,
// the exclusive prefix popcount per 32-bit word, and the model index of
// each present cell in lattice order (x fastest)
struct AmrLevel {
  int lo[3];               // first lattice index per axis (cell pos / 2^level)
  int n[3];                // lattice cells per axis; 0: no cells on this level
  const uint32_t *bits;
  const uint32_t *rank;
  const int32_t *cell;     // rank -> model cell index
};

struct AmrCellView {
  int numLevels;           // highest level present + 1
  const float *scalars;    // per model cell
  AmrLevel lv[kMaxLevels];
};

// ExaBricks (the comparison sampler of sampler/ExaBrickSampler.h): bricks,
// their scalars, the active brick regions with their leaf lists, and an
// LBVH over the regions' domains (rows of two corner vertices)
struct BrickView {
  const exa_brick *bricks;
  const float *scalars;
  const exa_abr *abrs;
  const int32_t *leafList;
  const BvhNode *nodes;
  int numAbrs;
};

struct AccelView {
  const exa_gridlet *gridlets;
  const float *scalars;
  const float *gridletMaxOps;   // may be null (no TF yet)
  const float4 *vertices;
  const int32_t *indices;
  const float *elemMaxOps;      // may be null
  int numGridlets;
  int numElems;
  int numTables;
  int tablesSorted;             // 1: tables in ascending gridlet-index order
  ElemOccupancy occ;
  GridletTable tables[kMaxLevels];
  const AmrCellView *amr;       // non-null: the AMR-cell sampler (no gridlets, no elements)
  const BrickView *bricks;      // non-null: the ExaBrick sampler (no gridlets, no elements)
};

// cell of p along one axis: floor((p - origin) / width), the width a power of
// two, so the multiplication by its reciprocal is the exact quotient
EXA_HD int occ_coord(float p, float origin, float invWidth, int n)
{
  const float f = floorf((p - origin) * invWidth);
  return f < 0.f ? -1 : (f >= (float)n ? n : (int)f);
}


EXA_D int floor_div_pow2(int v, int shift) { return v >> shift; }  // arithmetic shift floors

// optional per-thread work counters of the point query (counting launches)
struct QueryStats {
  unsigned tables, gridletTests, elemLists;
};

// the block of table T holding pos, and whether pos lies on the block's low
// face along each axis (then the block below is looked at too); false when
// pos is NaN or far outside the lattice
EXA_D bool table_block(const GridletTable &T, V3 pos, int b0[3], int nb[3])
{
  const float inv = __uint_as_float((uint32_t)(127 - T.level) << 23);  // 2^-level
  const float u[3] = {pos.x * inv - 0.5f, pos.y * inv - 0.5f, pos.z * inv - 0.5f};
  for (int a = 0; a < 3; ++a) {
    const float fu = floorf(u[a]);
    if (!(fu >= -2147483520.f && fu <= 2147483520.f)) return false;
    const int iu = (int)fu - T.origin[a];
    const int b = floor_div_pow2(iu, T.shift);
    // exactly on a block face: the gridlet ending there is listed in the
    // block below
    const bool face = (fu == u[a]) && ((iu & ((1 << T.shift) - 1)) == 0);
    nb[a] = face ? 2 : 1;
    b0[a] = face ? b - 1 : b;
  }
  return true;
}

EXA_D int table_entry(const GridletTable &T, int bx, int by, int bz)
{
  if (bx < 0 || by < 0 || bz < 0 || bx >= T.n[0] || by >= T.n[1] || bz >= T.n[2]) return -1;
  return __ldg(T.entries + ((size_t)bz * T.n[1] + by) * T.n[0] + bx);
}

// test every candidate gridlet of one table; keeps the lowest index hit
EXA_D void query_table(const AccelView &A, const GridletTable &T, V3 pos, bool cull, int &best,
                       float &bestVal, int &bestCell, QueryStats *qs, uint32_t &err)
{
  if (qs) qs->tables++;
  int b0[3], nb[3];
  if (!table_block(T, pos, b0, nb)) return;
  for (int dz = 0; dz < nb[2]; ++dz)
    for (int dy = 0; dy < nb[1]; ++dy)
      for (int dx = 0; dx < nb[0]; ++dx) {
        const int e = table_entry(T, b0[0] + dx, b0[1] + dy, b0[2] + dz);
        if (e == -1) continue;
        int cnt = 1;
        const int32_t *list = nullptr;
        if (e <= -2) {
          if (!exa_in_range(-e - 2, T.numItems, err)) continue;
          list = T.items + (-e - 2);
          cnt = __ldg(list);
          if (!exa_in_range(-e - 2 + cnt, T.numItems, err)) continue;
        }
        for (int k = 0; k < cnt; ++k) {
          const int g = list ? __ldg(list + 1 + k) : e;
          if (g >= best) break;  // lists are ascending
          if (!exa_in_range(g, A.numGridlets, err)) continue;
          if (cull && A.gridletMaxOps && __ldg(A.gridletMaxOps + g) == 0.f) continue;
          float v;
          int c;
          if (qs) qs->gridletTests++;
          if (intersect_gridlet(v, c, pos, A.gridlets + g, A.scalars)) {
            best = g;
            bestVal = v;
            bestCell = c;
          }
        }
      }
}

EXA_D bool box_contains(const float *lo, const float *hi, V3 p)
{
  return lo[0] <= p.x && lo[1] <= p.y && lo[2] <= p.z && p.x <= hi[0] && p.y <= hi[1] && p.z <= hi[2];
}

// the entry of pos's element cell: -1 when no element's closed AABB can hold
// pos (the cell's bit is clear), else the cell's entry (>= 0 its only
// element, <= -2 its list)
EXA_D int elem_cell_entry(const AccelView &A, V3 pos, uint32_t &err)
{
  const ElemOccupancy &O = A.occ;
  const int x = occ_coord(pos.x, O.origin[0], O.invCell[0], O.n[0]);
  const int y = occ_coord(pos.y, O.origin[1], O.invCell[1], O.n[1]);
  const int z = occ_coord(pos.z, O.origin[2], O.invCell[2], O.n[2]);
  if (x < 0 || y < 0 || z < 0 || x >= O.n[0] || y >= O.n[1] || z >= O.n[2]) return -1;
  const size_t c = ((size_t)z * O.n[1] + y) * O.n[0] + x;
  // the word's bits and its rank do not depend on each other: both loads
  // are in flight together
  const uint32_t word = __ldg(O.bits + (c >> 5));
  const uint32_t before = __ldg(O.rank + (c >> 5));
  const uint32_t bit = 1u << (c & 31);
  if (!(word & bit)) return -1;
  const int m = (int)(before + __popc(word & (bit - 1u)));
  if (!exa_in_range(m, O.numMarked, err)) return -1;
  return __ldg(O.entries + m);  // (a marked cell always lists an element)
}

// the lowest-index element of a cell entry that holds pos (its closed AABB,
// then the element's own test), -1 if none.  Out of line: element samples
// are rare next to gridlet samples, and keeping the list walk and the three
// Newton solvers out of the tracking loop keeps that loop's code small.
static __device__ __noinline__ int query_element_entry(const AccelView &A, V3 pos, int e, bool cull, float &val,
                                                       uint32_t &err)
{
  const ElemOccupancy &O = A.occ;
  if (e == -1) return -1;
  int cnt = 1;
  const int32_t *list = nullptr;
  if (e <= -2) {
    if (!exa_in_range(-e - 2, O.numItems, err)) return -1;
    list = O.items + (-e - 2);
    cnt = __ldg(list);
    if (!exa_in_range(-e - 2 + cnt, O.numItems, err)) return -1;
  }
  const bool useOps = cull && A.elemMaxOps;
  for (int k = 0; k < cnt; ++k) {
    const int id = list ? __ldg(list + 1 + k) : e;
    if (!exa_in_range(id, A.numElems, err)) continue;
    if (useOps && __ldg(A.elemMaxOps + id) == 0.f) continue;
    const float4 b0 = __ldg(O.boxes + 2 * (size_t)id), b1 = __ldg(O.boxes + 2 * (size_t)id + 1);
    const float lo[3] = {b0.x, b0.y, b0.z}, hi[3] = {b0.w, b1.x, b1.y};
    if (!box_contains(lo, hi, pos)) continue;
    float v;
    if (intersect_elem(v, pos, A.indices + (size_t)id * 8, A.vertices)) {
      val = v;
      return id;  // lists are ascending: the first hit is the lowest index
    }
  }
  return -1;
}

EXA_D int query_elements(const AccelView &A, V3 pos, bool cull, float &val, uint32_t &err, QueryStats *qs)
{
  const int e = elem_cell_entry(A, pos, err);
  if (e == -1) return -1;
  if (qs) qs->elemLists++;
  return query_element_entry(A, pos, e, cull, val, err);
}

// sample() (sampler/ExaStitchSampler.h:128-140); sets EXA_DEVERR bits in err
// AMRCellSampler's sample() (sampler/AMRCellSampler.h:66-84) with the
// intersection program AMRCellGeomIsect (programs/AMRCellSampler.cu:43-69):
// every cell whose support -- its box grown by half a cell on each side --
// contains pos (inclusive) adds its scalar with the tent weight
// prod(1 - |p - c| / (size / 2)); the sample is the weighted mean, absent
// (primID -1) when the weights sum to 0.  The reference sums in OptiX's
// traversal order; here the order is fixed: levels ascending, then cells in
// z, y, x order.  The candidates per level are the 3 lattice cells per axis
// around floor(p / w), which contain every cell whose support can hold p.
static __device__ __noinline__ exa_sample amr_sample(const AmrCellView &V, V3 pos)
{
  float sumW = 0.f, sumWV = 0.f;
  const float P[3] = {pos.x, pos.y, pos.z};
  for (int L = 0; L < V.numLevels; ++L) {
    const AmrLevel &l = V.lv[L];
    if (l.n[0] <= 0) continue;
    const int w = 1 << L;
    const float half = (float)w * .5f;
    int cand[3][3], nc[3];
    bool any = true;
    for (int a = 0; a < 3 && any; ++a) {
      nc[a] = 0;
      const float q = floorf(P[a] / (float)w);
      // outside the level's lattice (with a margin of 2 cells): nothing here
      if (!(q >= (float)l.lo[a] - 2.f && q <= (float)(l.lo[a] + l.n[a]) + 1.f)) { any = false; break; }
      const int b = (int)q;
      for (int i = b - 1; i <= b + 1; ++i) {
        if (i < l.lo[a] || i >= l.lo[a] + l.n[a]) continue;
        const float lower = (float)(i * w) - half, upper = (float)(i * w + w) + half;
        if (lower <= P[a] && P[a] <= upper) cand[a][nc[a]++] = i;
      }
      any = nc[a] > 0;
    }
    if (!any) continue;
    for (int kz = 0; kz < nc[2]; ++kz)
      for (int ky = 0; ky < nc[1]; ++ky)
        for (int kx = 0; kx < nc[0]; ++kx) {
          const int i = cand[0][kx], j = cand[1][ky], k = cand[2][kz];
          const size_t c = ((size_t)(k - l.lo[2]) * l.n[1] + (j - l.lo[1])) * l.n[0] + (i - l.lo[0]);
          const uint32_t word = __ldg(l.bits + (c >> 5));
          if (!((word >> (c & 31)) & 1u)) continue;
          const int cellIdx = __ldg(l.cell + __ldg(l.rank + (c >> 5)) + __popc(word & ((1u << (c & 31)) - 1u)));
          const int id[3] = {i, j, k};
          float wgt = 1.f;
          for (int a = 0; a < 3; ++a) {
            const float lower = (float)(id[a] * w) - half, upper = (float)(id[a] * w + w) + half;
            const float center = (lower + upper) / 2.f, size = upper - lower;
            wgt = wgt * (1.f - fabsf(P[a] - center) / (size * .5f));
          }
          const float scalar = __ldg(V.scalars + cellIdx);
          sumW += wgt;
          sumWV += scalar * wgt;
        }
  }
  exa_sample s;
  s.primID = -1;
  s.cellID = -1;
  s.value = 0.f;
  if (sumW > 0.f) {
    s.primID = 0;
    s.value = sumWV / sumW;
  }
  return s;
}

// addBasisFunctions (sampler/ExaBrickSampler.h:113-200): the brick's
// trilinear basis functions around pos, in the reference's corner order
EXA_D void add_basis(const BrickView &V, int brickID, V3 pos, float &sumWV, float &sumW)
{
  const exa_brick b = V.bricks[brickID];
  const float cw = (float)(1 << b.level);
  const float lx = (pos.x - (float)b.lower.x) / cw - .5f;
  const float ly = (pos.y - (float)b.lower.y) / cw - .5f;
  const float lz = (pos.z - (float)b.lower.z) / cw - .5f;
  const int ilx = max(-1, (int)floorf(lx)), ily = max(-1, (int)floorf(ly)), ilz = max(-1, (int)floorf(lz));
  const int ihx = ilx + 1, ihy = ily + 1, ihz = ilz + 1;
  const float fx = lx - (float)ilx, fy = ly - (float)ily, fz = lz - (float)ilz;
  const float nx = 1.f - fx, ny = 1.f - fy, nz = 1.f - fz;
  const float *S = V.scalars + b.begin;
  auto add = [&](int x, int y, int z, float w) {
    const float scalar = __ldg(S + x + y * b.size.x + z * b.size.x * b.size.y);
    sumW += w;
    sumWV += w * scalar;
  };
  if (ilz >= 0 && ilz < b.size.z) {
    if (ily >= 0 && ily < b.size.y) {
      if (ilx >= 0 && ilx < b.size.x) add(ilx, ily, ilz, nz * ny * nx);
      if (ihx < b.size.x) add(ihx, ily, ilz, nz * ny * fx);
    }
    if (ihy < b.size.y) {
      if (ilx >= 0 && ilx < b.size.x) add(ilx, ihy, ilz, nz * fy * nx);
      if (ihx < b.size.x) add(ihx, ihy, ilz, nz * fy * fx);
    }
  }
  if (ihz < b.size.z) {
    if (ily >= 0 && ily < b.size.y) {
      if (ilx >= 0 && ilx < b.size.x) add(ilx, ily, ihz, fz * ny * nx);
      if (ihx < b.size.x) add(ihx, ily, ihz, fz * ny * fx);
    }
    if (ihy < b.size.y) {
      if (ilx >= 0 && ilx < b.size.x) add(ilx, ihy, ihz, fz * fy * nx);
      if (ihx < b.size.x) add(ihx, ihy, ihz, fz * fy * fx);
    }
  }
}

// ExaBrickSampler's sample() in the grid + DDA traversal mode (sampler/
// ExaBrickSampler.h:202-239, programs/ExaBrickSampler.cu:67-89): the region
// whose closed domain holds pos adds the basis functions of its bricks;
// value sumWV / sumW, 0 where no region holds pos or the weights sum to 0
// (primID is 0 in every case, as there).  Where several regions share a
// face the lowest-index one is taken (OptiX reports them in an unspecified
// order).  The region is found by a complete walk of the region LBVH.
static __device__ __noinline__ exa_sample brick_sample(const BrickView &V, V3 pos, uint32_t &err)
{
  exa_sample s;
  s.primID = 0;
  s.cellID = -1;
  s.value = 0.f;
  if (V.numAbrs <= 0) return s;
  int best = 0x7fffffff;
  int stack[kBvhStack];
  int sp = 0, node = 0;
  bool done = false;
  for (int visits = 0; visits <= V.numAbrs + 1 && !done; ++visits) {
    const float4 *np = reinterpret_cast<const float4 *>(V.nodes + node);
    const float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3);
    const float lo0[3] = {q0.x, q0.y, q0.z}, hi0[3] = {q0.w, q1.x, q1.y};
    const float lo1[3] = {q1.z, q1.w, q2.x}, hi1[3] = {q2.y, q2.z, q2.w};
    const int c[2] = {__float_as_int(q3.x), __float_as_int(q3.y)};
    const bool in[2] = {box_contains(lo0, hi0, pos), box_contains(lo1, hi1, pos)};
    int next = -1;
    for (int k = 0; k < 2; ++k) {
      if (!in[k]) continue;
      if (c[k] < 0) {
        best = min(best, ~c[k]);
      } else if (next < 0) {
        next = c[k];
      } else if (sp < kBvhStack) {
        stack[sp++] = c[k];
      } else {
        err |= EXA_DEVERR_BVH_STACK;
      }
    }
    if (next < 0) {
      if (sp == 0) done = true;
      else next = stack[--sp];
    }
    node = next;
  }
  if (best == 0x7fffffff) return s;
  const exa_abr R = V.abrs[best];
  float sumWV = 0.f, sumW = 0.f;
  for (int i = 0; i < R.leafListSize; ++i) add_basis(V, __ldg(V.leafList + R.leafListBegin + i), pos, sumWV, sumW);
  if (sumW > 0.f) s.value = sumWV / sumW;
  return s;
}

// the stitching elements' part of sample(): where no gridlet holds pos
EXA_D exa_sample sample_elements(const AccelView &A, V3 pos, bool cull, uint32_t &err, QueryStats *qs)
{
  exa_sample s;
  s.primID = -1;
  s.cellID = -1;
  s.value = 0.f;
  float ev = 0.f;
  const int be = A.numElems > 0 ? query_elements(A, pos, cull, ev, err, qs) : -1;
  if (be >= 0) {
    s.primID = be;
    s.cellID = -1;
    s.value = ev;
  }
  return s;
}

// the gridlet part of sample(): the lowest-index gridlet that holds pos
// (primID -1: none)
EXA_D exa_sample sample_gridlets(const AccelView &A, V3 pos, bool cull, uint32_t &err, QueryStats *qs = nullptr)
{
  int best = 0x7fffffff, cell = -1;
  float val = 0.f;
  for (int t = 0; t < A.numTables; ++t) {
    query_table(A, A.tables[t], pos, cull, best, val, cell, qs, err);
    if (A.tablesSorted && best != 0x7fffffff) break;
  }
  exa_sample s;
  s.primID = best != 0x7fffffff ? best : -1;
  s.cellID = best != 0x7fffffff ? cell : -1;
  s.value = best != 0x7fffffff ? val : 0.f;
  return s;
}

EXA_D exa_sample sample_field(const AccelView &A, V3 pos, bool cull, uint32_t &err, QueryStats *qs = nullptr)
{
  if (A.amr) return amr_sample(*A.amr, pos);
  if (A.bricks) return brick_sample(*A.bricks, pos, err);
  const exa_sample s = sample_gridlets(A, pos, cull, err, qs);
  if (s.primID >= 0) return s;
  return sample_elements(A, pos, cull, err, qs);
}

// testSample (sampler/ExaStitchSampler.h:108-126): the cached gridlet only
EXA_D exa_sample test_sample(const AccelView &A, V3 pos, int primID)
{
  exa_sample s;
  s.primID = -1;
  s.cellID = -1;
  s.value = 0.f;
  if (primID < 0) return s;
  if (intersect_gridlet(s.value, s.cellID, pos, A.gridlets + primID, A.scalars)) s.primID = primID;
  return s;
}

} // namespace exa
