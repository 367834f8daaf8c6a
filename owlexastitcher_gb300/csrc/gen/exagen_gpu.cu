// exagen_gpu.cu -- the generator of exagen.cpp on the GPU.
//
// Same definition, same output bit for bit (the field code is shared:
// exagen_field.h); the stages after the field set-up run as CUDA kernels
// over bit sets held in HBM:
//   * tree: per level a "refined" and a "leaf" bit set (32-bit words), each
//     word written whole by one warp from a ballot (no atomics), except the
//     2:1 balance pass, which ORs neighbour bits in;
//   * leaf ids: level offset + rank in the level's linear order, from a
//     per-word exclusive prefix popcount (block scan + scan of block sums);
//   * elements (makeDual.cpp:596-872): one count pass over the leaves, a
//     compaction of the leaves that emit anything, per-type scans, and a
//     write pass that reproduces the CPU order (type, leaf id, corner);
//   * gridlets (makeGrids.cpp:57-209): per 8^3 macrocell cube masks from the
//     leaf bits, scans for brick ids and scalar offsets, then the corner
//     values.
// The result is copied into the same host-side result object exa_gen_run
// fills, so every accessor of exastitch_gen.h works on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cub/cub.cuh>

#include "exagen_internal.h"

namespace {

using exagen::FieldView;
using exagen::kMaxLevels;

void ck(cudaError_t e, const char *what)
{
  if (e != cudaSuccess) throw std::runtime_error(std::string("exa_gen_run_gpu: ") + what + ": " + cudaGetErrorString(e));
}

template <typename T>
struct Dev {
  T *p = nullptr;
  size_t n = 0;
  Dev() = default;
  explicit Dev(size_t count) { alloc(count); }
  Dev(const Dev &) = delete;
  Dev &operator=(const Dev &) = delete;
  Dev(Dev &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  Dev &operator=(Dev &&o) noexcept
  {
    if (this != &o) {
      if (p) cudaFree(p);
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~Dev() { if (p) cudaFree(p); }
  void alloc(size_t count)
  {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (count) ck(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
  }
  void zero(cudaStream_t s) { if (n) ck(cudaMemsetAsync(p, 0, n * sizeof(T), s), "memset"); }
  void upload(const T *h, size_t count, cudaStream_t s)
  {
    alloc(count);
    if (count) ck(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  }
  void download(T *h, size_t count, cudaStream_t s) const
  {
    if (count) ck(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s), "download");
  }
};

// ------------------------------------------------------------------ tree

struct LevelD {
  int64_t n[3];
  uint64_t cells;
  uint64_t words;     // 32-bit words of the bit sets
  uint32_t *refined;  // null on level 0
  uint32_t *leaf;
  uint32_t *rank;     // exclusive prefix popcount of leaf, per word
  uint64_t leafOffset;
};

struct TreeD {
  int Lroot;
  LevelD lv[kMaxLevels];
};

__device__ __forceinline__ bool bit(const uint32_t *w, uint64_t i) { return (w[i >> 5] >> (i & 31)) & 1u; }

__device__ __forceinline__ uint64_t lin(const LevelD &l, int64_t i, int64_t j, int64_t k)
{
  return ((uint64_t)k * l.n[1] + j) * l.n[0] + i;
}

__device__ __forceinline__ bool inside(const LevelD &l, int64_t i, int64_t j, int64_t k)
{
  return i >= 0 && j >= 0 && k >= 0 && i < l.n[0] && j < l.n[1] && k < l.n[2];
}

__device__ __forceinline__ void coords(const LevelD &l, uint64_t c, int64_t &i, int64_t &j, int64_t &k)
{
  i = (int64_t)(c % l.n[0]);
  j = (int64_t)((c / l.n[0]) % l.n[1]);
  k = (int64_t)(c / ((uint64_t)l.n[0] * l.n[1]));
}

__device__ __forceinline__ uint64_t leaf_id(const LevelD &l, uint64_t c)
{
  const uint32_t w = l.leaf[c >> 5] & ((1u << (c & 31)) - 1u);
  return l.leafOffset + l.rank[c >> 5] + (uint64_t)__popc(w);
}

// grid-stride over the cells of a level in whole warps: every warp handles
// 32 consecutive cells (one bit-set word) per iteration
#define FOR_WORD_CELLS(count, c, w, lane)                                                             \
  const unsigned lane = threadIdx.x & 31;                                                             \
  const uint64_t nwords_ = ((count) + 31) / 32;                                                       \
  const uint64_t warp0_ = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;                     \
  const uint64_t nwarps_ = (gridDim.x * (uint64_t)blockDim.x) / 32;                                   \
  for (uint64_t w = warp0_, c = w * 32 + lane; w < nwords_; w += nwarps_, c = w * 32 + lane)

// Calls f(c, i, j, k) for every set bit c of a level's bit set.  A warp
// loads 32 words at once (one per lane, coalesced) and then works through
// the non-zero ones together, one lane per bit, so the mostly empty words of
// the fine levels cost one load each.
template <typename Fn>
__device__ __forceinline__ void for_set_bits(const uint32_t *bits, const LevelD &l, Fn &&f)
{
  const unsigned lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) / 32;
  for (uint64_t w0 = warp * 32; w0 < l.words; w0 += nwarps * 32) {
    const uint64_t mw = w0 + lane;
    const uint32_t mine = mw < l.words ? bits[mw] : 0u;
    uint32_t nz = __ballot_sync(0xffffffffu, mine != 0u);
    while (nz) {
      const int src = __ffs(nz) - 1;
      nz &= nz - 1;
      const uint32_t word = __shfl_sync(0xffffffffu, mine, src);
      if ((word >> lane) & 1u) {
        const uint64_t c = (w0 + src) * 32 + lane;
        int64_t i, j, k;
        coords(l, c, i, j, k);
        f(c, i, j, k);
      }
    }
  }
}

// the cloud's raw root values exp(3 fBm), for its mapping range
__global__ void k_cloud_raw(FieldView F, TreeD T, double *raw)
{
  const LevelD &l = T.lv[T.Lroot];
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < l.cells;
       c += gridDim.x * (uint64_t)blockDim.x) {
    int64_t i, j, k;
    coords(l, c, i, j, k);
    raw[c] = exagen::cloud_raw(F, exagen::cell_center(T.Lroot, i) / F.extent[0],
                               exagen::cell_center(T.Lroot, j) / F.extent[1],
                               exagen::cell_center(T.Lroot, k) / F.extent[2]);
  }
}

// root values, their max |f|
__global__ void k_root_eval(FieldView F, TreeD T, float *rootVal, unsigned long long *maxAbsBits)
{
  const LevelD &l = T.lv[T.Lroot];
  double m = 0;
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < l.cells;
       c += gridDim.x * (uint64_t)blockDim.x) {
    int64_t i, j, k;
    coords(l, c, i, j, k);
    const double v = exagen::eval_cell(F, T.Lroot, i, j, k);
    rootVal[c] = (float)v;
    m = fmax(m, fabs(v));
  }
  // non-negative doubles order like their bit patterns
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxAbsBits, (unsigned long long)__double_as_longlong(m));
}

// the root's refined bits, from its binary32 values as the CPU keeps them
__global__ void k_root_refine(TreeD T, const float *rootVal, int kind, double thr, double maxAbs)
{
  const LevelD &l = T.lv[T.Lroot];
  FOR_WORD_CELLS(l.cells, c, w, lane)
  {
    const bool r = c < l.cells && exagen::refine_crit(kind, (double)rootVal[c], T.Lroot, T.Lroot, thr, maxAbs);
    const uint32_t b = __ballot_sync(0xffffffffu, r);
    if (lane == 0) l.refined[w] = b;
  }
}

// level L < root: children of refined parents, refined where the field says
// (the child level's bits start zeroed)
__global__ void k_refine_level(FieldView F, TreeD T, int L, int kind, double thr, double maxAbs)
{
  const LevelD &l = T.lv[L];
  const LevelD &p = T.lv[L + 1];
  for_set_bits(p.refined, p, [&](uint64_t, int64_t pi, int64_t pj, int64_t pk) {
    for (int d = 0; d < 8; ++d) {
      const int64_t i = 2 * pi + (d & 1), j = 2 * pj + ((d >> 1) & 1), k = 2 * pk + (d >> 2);
      if (exagen::refine_crit(kind, exagen::eval_cell(F, L, i, j, k), L, T.Lroot, thr, maxAbs)) {
        const uint64_t c = lin(l, i, j, k);
        atomicOr(l.refined + (c >> 5), 1u << (c & 31));
      }
    }
  });
}

// 2:1 balance: the parents of all same-level neighbours of a refined cell
// are refined (one level at a time, ascending)
__global__ void k_balance(TreeD T, int L)
{
  const LevelD &l = T.lv[L];
  const LevelD &p = T.lv[L + 1];
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < l.words; w += gridDim.x * (uint64_t)blockDim.x) {
    uint32_t word = l.refined[w];
    while (word) {
      const int b = __ffs(word) - 1;
      word &= word - 1;
      int64_t i, j, k;
      coords(l, w * 32 + b, i, j, k);
      for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            const int64_t ni = i + dx, nj = j + dy, nk = k + dz;
            if (!inside(l, ni, nj, nk)) continue;
            const uint64_t pc = lin(p, ni >> 1, nj >> 1, nk >> 1);
            atomicOr(p.refined + (pc >> 5), 1u << (pc & 31));
          }
    }
  }
}

// leaves: on the root every unrefined cell, below it every child of a
// refined parent that is not refined itself (all of them on level 0)
__global__ void k_leaf_bits(TreeD T, int L)
{
  const LevelD &l = T.lv[L];
  FOR_WORD_CELLS(l.cells, c, w, lane)
  {
    bool f = false;
    if (c < l.cells) {
      const bool ref = L > 0 && bit(l.refined, c);
      if (L == T.Lroot) {
        f = !ref;
      } else {
        const LevelD &p = T.lv[L + 1];
        int64_t i, j, k;
        coords(l, c, i, j, k);
        f = bit(p.refined, lin(p, i >> 1, j >> 1, k >> 1)) && !ref;
      }
    }
    const uint32_t b = __ballot_sync(0xffffffffu, f);
    if (lane == 0) l.leaf[w] = b;
  }
}

// the same, a word at a time, for levels whose rows are whole words
// (n.x % 32 == 0): the 32 cells of a word have 16 parents that are 16
// aligned bits of one parent word, each parent bit standing for two cells
__global__ void k_leaf_words(TreeD T, int L)
{
  const LevelD &l = T.lv[L];
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < l.words;
       w += gridDim.x * (uint64_t)blockDim.x) {
    const uint32_t ref = L > 0 ? l.refined[w] : 0u;
    uint32_t out;
    if (L == T.Lroot) {
      out = ~ref;
    } else {
      const LevelD &p = T.lv[L + 1];
      int64_t i, j, k;
      coords(l, w * 32, i, j, k);
      const uint64_t pc = lin(p, i >> 1, j >> 1, k >> 1);
      uint32_t x = (p.refined[pc >> 5] >> (pc & 31)) & 0xffffu;
      // spread the 16 bits to the even positions, then double them
      x = (x | (x << 8)) & 0x00ff00ffu;
      x = (x | (x << 4)) & 0x0f0f0f0fu;
      x = (x | (x << 2)) & 0x33333333u;
      x = (x | (x << 1)) & 0x55555555u;
      out = (x | (x << 1)) & ~ref;
    }
    l.leaf[w] = out;
  }
}

// per-word popcounts scanned within blocks of kScanBlock words
constexpr int kScanBlock = 1024;

__global__ void k_rank_blocks(const uint32_t *bits, uint64_t words, uint32_t *rank, uint32_t *blockSum)
{
  typedef cub::BlockScan<uint32_t, kScanBlock> Scan;
  __shared__ typename Scan::TempStorage tmp;
  const uint64_t w = blockIdx.x * (uint64_t)kScanBlock + threadIdx.x;
  const uint32_t v = w < words ? (uint32_t)__popc(bits[w]) : 0u;
  uint32_t ex, total;
  Scan(tmp).ExclusiveSum(v, ex, total);
  if (w < words) rank[w] = ex;
  if (threadIdx.x == 0) blockSum[blockIdx.x] = total;
}

__global__ void k_rank_add(uint32_t *rank, uint64_t words, const uint32_t *blockBase)
{
  const uint64_t w = blockIdx.x * (uint64_t)kScanBlock + threadIdx.x;
  if (w < words) rank[w] += blockBase[blockIdx.x];
}

// cell values and AMR records of a level's leaves
__global__ void k_values(FieldView F, TreeD T, int L, float *value, int32_t *cells)
{
  const LevelD &l = T.lv[L];
  for_set_bits(l.leaf, l, [&](uint64_t c, int64_t i, int64_t j, int64_t k) {
    const uint64_t id = leaf_id(l, c);
    value[id] = (float)exagen::eval_cell(F, L, i, j, k);
    int4 rec;
    rec.x = (int32_t)(i << L);
    rec.y = (int32_t)(j << L);
    rec.z = (int32_t)(k << L);
    rec.w = L;
    reinterpret_cast<int4 *>(cells)[id] = rec;
  });
}

// ------------------------------------------------------------------ dual cells

struct LeafRefD {
  int level;
  uint64_t lin;
  uint64_t id;
};

// leaf containing the point q (half finest units), or level -1
__device__ LeafRefD find_half(const TreeD &T, int64_t qx, int64_t qy, int64_t qz)
{
  LeafRefD r{-1, 0, 0};
  if (qx < 0 || qy < 0 || qz < 0) return r;
  for (int L = T.Lroot; L >= 0; --L) {
    const LevelD &l = T.lv[L];
    const int sh = L + 1;
    const int64_t i = qx >> sh, j = qy >> sh, k = qz >> sh;
    if (!inside(l, i, j, k)) return r;
    const uint64_t c = lin(l, i, j, k);
    if (bit(l.leaf, c)) {
      r.level = L;
      r.lin = c;
      r.id = leaf_id(l, c);
      return r;
    }
    if (L == 0 || !bit(l.refined, c)) return r;
  }
  return r;
}

// LogicalCell order of makeDual.cpp:115-122: (pos.y, pos.x, pos.z)
__device__ __forceinline__ bool cell_less(int64_t ai, int64_t aj, int64_t ak, int64_t bi, int64_t bj, int64_t bk)
{
  if (aj != bj) return aj < bj;
  if (ai != bi) return ai < bi;
  return ak < bk;
}

// element emission: counts per type, or rows written at per-type cursors
struct Emit {
  bool write;
  uint32_t n[4];        // per type, this leaf so far
  uint64_t base[4];     // write: first row of this leaf per type (global)
  int32_t *rows;        // write: 8 leaf ids per row
  uint8_t *used;        // write: vertex-used flags per leaf id
  uint32_t skipped;
  __device__ void put(int type, const uint64_t *v)
  {
    const int nv = type == 0 ? 4 : type == 1 ? 5 : type == 2 ? 6 : 8;
    if (write) {
      int32_t *row = rows + (base[type] + n[type]) * 8;
      for (int i = 0; i < 8; ++i) row[i] = i < nv ? (int32_t)v[i] : -1;
      for (int i = 0; i < nv; ++i) used[v[i]] = 1;
    }
    n[type]++;
  }
  __device__ void tet(uint64_t a, uint64_t b, uint64_t c, uint64_t d)
  {
    const uint64_t v[4] = {a, b, c, d};
    put(0, v);
  }
  __device__ void wedge(const uint64_t *v, int f0, int f1, int f2, int b0, int b1, int b2)
  {
    const uint64_t w[6] = {v[f0], v[f1], v[f2], v[b0], v[b1], v[b2]};
    put(2, w);
  }
};

// makeDual.cpp:496-547
__device__ void try_pyramid(Emit &E, const uint64_t *base, uint64_t top, int numUnique)
{
  if (numUnique == 5) {
    const uint64_t v[5] = {base[0], base[1], base[2], base[3], top};
    E.put(1, v);
    return;
  }
  if (numUnique == 4) {
    if (base[0] == base[1]) { E.tet(base[1], base[2], base[3], top); return; }
    if (base[1] == base[2]) { E.tet(base[2], base[3], base[0], top); return; }
    if (base[2] == base[3]) { E.tet(base[3], base[0], base[1], top); return; }
    if (base[3] == base[0]) { E.tet(base[0], base[1], base[2], top); return; }
  }
  E.skipped++;  // the reference throws ("this case should not happen") or skips
}

// makeDual.cpp:734-870, non-uniform dual cells only
__device__ void classify(Emit &E, const uint64_t *v, int numUnique)
{
  auto allSame = [&](int a, int b, int c, int d) { return v[a] == v[b] && v[a] == v[c] && v[a] == v[d]; };
  auto same = [&](int a, int b) { return v[a] == v[b]; };
  if (numUnique == 8) { E.put(3, v); return; }
  if (numUnique < 4) { E.skipped++; return; }
  if (allSame(0, 1, 2, 3)) { const uint64_t b[4] = {v[4], v[7], v[6], v[5]}; try_pyramid(E, b, v[0], numUnique); return; }
  if (allSame(4, 5, 6, 7)) { const uint64_t b[4] = {v[0], v[1], v[2], v[3]}; try_pyramid(E, b, v[4], numUnique); return; }
  if (allSame(0, 1, 4, 5)) { const uint64_t b[4] = {v[2], v[6], v[7], v[3]}; try_pyramid(E, b, v[0], numUnique); return; }
  if (allSame(2, 3, 6, 7)) { const uint64_t b[4] = {v[0], v[4], v[5], v[1]}; try_pyramid(E, b, v[2], numUnique); return; }
  if (allSame(0, 3, 4, 7)) { const uint64_t b[4] = {v[1], v[5], v[6], v[2]}; try_pyramid(E, b, v[0], numUnique); return; }
  if (allSame(1, 2, 5, 6)) { const uint64_t b[4] = {v[0], v[3], v[7], v[4]}; try_pyramid(E, b, v[1], numUnique); return; }
  if (same(0, 1) && same(4, 5)) { E.wedge(v, 3, 2, 0, 7, 6, 4); return; }
  if (same(0, 4) && same(1, 5)) { E.wedge(v, 2, 6, 5, 3, 7, 4); return; }
  if (same(3, 7) && same(2, 6)) { E.wedge(v, 5, 1, 2, 4, 0, 3); return; }
  if (same(2, 3) && same(6, 7)) { E.wedge(v, 1, 0, 3, 5, 4, 7); return; }
  if (same(4, 7) && same(5, 6)) { E.wedge(v, 3, 0, 4, 2, 1, 6); return; }
  if (same(4, 5) && same(6, 7)) { E.wedge(v, 0, 1, 4, 3, 2, 7); return; }
  if (same(0, 1) && same(3, 2)) { E.wedge(v, 5, 4, 0, 6, 7, 3); return; }
  if (same(0, 3) && same(1, 2)) { E.wedge(v, 4, 7, 3, 5, 6, 2); return; }
  if (same(0, 3) && same(4, 7)) { E.wedge(v, 5, 6, 7, 1, 2, 3); return; }
  if (same(0, 4) && same(3, 7)) { E.wedge(v, 1, 5, 4, 2, 6, 7); return; }
  if (same(1, 2) && same(5, 6)) { E.wedge(v, 7, 4, 5, 3, 0, 1); return; }
  if (same(1, 5) && same(2, 6)) { E.wedge(v, 4, 0, 1, 7, 3, 2); return; }
  E.put(3, v);
}

__device__ __forceinline__ void swap64(uint64_t &a, uint64_t &b)
{
  const uint64_t t = a;
  a = b;
  b = t;
}

// doCell (makeDual.cpp:596-872) for the level-L leaf (ci, cj, ck)
__device__ void do_cell(const TreeD &T, int L, int64_t ci, int64_t cj, int64_t ck, Emit &E)
{
  const LevelD &l = T.lv[L];
  bool uniform = true;
  for (int d = 0; d < 27 && uniform; ++d) {
    const int64_t i = ci + d % 3 - 1, j = cj + (d / 3) % 3 - 1, k = ck + d / 9 - 1;
    if (!inside(l, i, j, k)) continue;
    if (!bit(l.leaf, lin(l, i, j, k))) uniform = false;
  }
  if (uniform) return;
  LeafRefD nb[27];
  const int64_t w = 1ll << L;
  for (int d = 0; d < 27; ++d) {
    const int64_t i = ci + d % 3 - 1, j = cj + (d / 3) % 3 - 1, k = ck + d / 9 - 1;
    if (inside(l, i, j, k) && bit(l.leaf, lin(l, i, j, k))) {
      const uint64_t c = lin(l, i, j, k);
      nb[d] = LeafRefD{L, c, leaf_id(l, c)};
    } else {
      nb[d] = find_half(T, 2 * i * w + w, 2 * j * w + w, 2 * k * w + w);
    }
  }
  const uint64_t selfId = nb[13].id;
  for (int dz = -1; dz <= 1; dz += 2)
    for (int dy = -1; dy <= 1; dy += 2)
      for (int dx = -1; dx <= 1; dx += 2) {
        uint64_t vtx[2][2][2];
        int minLevel = 1000, maxLevel = -1, numFound = 0;
        bool isMin = true;
        for (int iz = 0; iz < 2; iz++)
          for (int iy = 0; iy < 2; iy++)
            for (int ix = 0; ix < 2; ix++) {
              const LeafRefD &r = nb[(dz * iz + 1) * 9 + (dy * iy + 1) * 3 + (dx * ix + 1)];
              vtx[iz][iy][ix] = r.id;
              if (r.level < 0) continue;
              minLevel = min(minLevel, r.level);
              maxLevel = max(maxLevel, r.level);
              ++numFound;
            }
        if (numFound < 8) continue;
        if (minLevel < L) continue;
        if (minLevel == maxLevel) continue;  // perfect cube: a gridlet cell
        // generated by the lowest same-level corner (makeDual.cpp:641-655)
        for (int iz = 0; iz < 2 && isMin; iz++)
          for (int iy = 0; iy < 2 && isMin; iy++)
            for (int ix = 0; ix < 2 && isMin; ix++) {
              const LeafRefD &r = nb[(dz * iz + 1) * 9 + (dy * iy + 1) * 3 + (dx * ix + 1)];
              if (r.level != L || r.id == selfId) continue;
              int64_t i, j, k;
              coords(l, r.lin, i, j, k);
              if (cell_less(i, j, k, ci, cj, ck)) isMin = false;
            }
        if (!isMin) continue;
        if (dx < 0) { swap64(vtx[0][0][0], vtx[0][0][1]); swap64(vtx[0][1][0], vtx[0][1][1]);
                      swap64(vtx[1][0][0], vtx[1][0][1]); swap64(vtx[1][1][0], vtx[1][1][1]); }
        if (dy < 0) { swap64(vtx[0][0][0], vtx[0][1][0]); swap64(vtx[0][0][1], vtx[0][1][1]);
                      swap64(vtx[1][0][0], vtx[1][1][0]); swap64(vtx[1][0][1], vtx[1][1][1]); }
        if (dz < 0) { swap64(vtx[0][0][0], vtx[1][0][0]); swap64(vtx[0][0][1], vtx[1][0][1]);
                      swap64(vtx[0][1][0], vtx[1][1][0]); swap64(vtx[0][1][1], vtx[1][1][1]); }
        const uint64_t v[8] = {vtx[0][0][0], vtx[0][0][1], vtx[0][1][1], vtx[0][1][0],
                               vtx[1][0][0], vtx[1][0][1], vtx[1][1][1], vtx[1][1][0]};
        int numUnique = 0;
        for (int a = 0; a < 8; ++a) {
          bool seen = false;
          for (int b = 0; b < a; ++b) seen |= v[b] == v[a];
          numUnique += !seen;
        }
        classify(E, v, numUnique);
      }
}

// count pass: packed per-type counts (8 bits each, at most 8) per leaf id
__global__ void k_elem_count(TreeD T, int L, uint32_t *packed, unsigned long long *skipped)
{
  const LevelD &l = T.lv[L];
  for_set_bits(l.leaf, l, [&](uint64_t c, int64_t i, int64_t j, int64_t k) {
    Emit E{};
    E.write = false;
    do_cell(T, L, i, j, k, E);
    packed[leaf_id(l, c)] = E.n[0] | (E.n[1] << 8) | (E.n[2] << 16) | (E.n[3] << 24);
    if (E.skipped) atomicAdd(skipped, (unsigned long long)E.skipped);
  });
}

__global__ void k_flag_nonzero(const uint32_t *packed, uint64_t n, uint32_t *flag)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x)
    flag[i] = packed[i] != 0u;
}

__global__ void k_compact(const uint32_t *packed, uint64_t n, const uint32_t *pos, uint32_t *ids, uint32_t *cnt)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x)
    if (packed[i]) {
      ids[pos[i]] = (uint32_t)i;
      cnt[pos[i]] = packed[i];
    }
}

__global__ void k_type_counts(const uint32_t *cnt, uint32_t m, int t, uint32_t *out)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += gridDim.x * (uint64_t)blockDim.x)
    out[i] = (cnt[i] >> (8 * t)) & 0xffu;
}

// write pass over the leaves that emit elements
__global__ void k_elem_write(TreeD T, const uint32_t *ids, uint32_t m, const int32_t *cells, const uint32_t *off0,
                             const uint32_t *off1, const uint32_t *off2, const uint32_t *off3, uint64_t tb1,
                             uint64_t tb2, uint64_t tb3, int32_t *rows, uint8_t *used)
{
  for (uint64_t a = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; a < m; a += gridDim.x * (uint64_t)blockDim.x) {
    const uint32_t id = ids[a];
    const int4 rec = reinterpret_cast<const int4 *>(cells)[id];
    const int L = rec.w;
    Emit E{};
    E.write = true;
    E.rows = rows;
    E.used = used;
    E.base[0] = off0[a];
    E.base[1] = tb1 + off1[a];
    E.base[2] = tb2 + off2[a];
    E.base[3] = tb3 + off3[a];
    do_cell(T, L, rec.x >> L, rec.y >> L, rec.z >> L, E);
  }
}

__global__ void k_u8_to_u32(const uint8_t *in, uint64_t n, uint32_t *out)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x)
    out[i] = in[i];
}

// element vertices: used leaves in ascending leaf id, at their cell centres
__global__ void k_vertices(const uint8_t *used, const uint32_t *vpos, uint64_t n, const int32_t *cells,
                           const float *value, float4 *verts)
{
  for (uint64_t id = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; id < n; id += gridDim.x * (uint64_t)blockDim.x) {
    if (!used[id]) continue;
    const int4 rec = reinterpret_cast<const int4 *>(cells)[id];
    const float h = 0.5f * (float)(1 << rec.w);
    verts[vpos[id]] = make_float4((float)rec.x + h, (float)rec.y + h, (float)rec.z + h, value[id]);
  }
}

__global__ void k_remap(int32_t *rows, uint64_t n, const uint32_t *vpos)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x)
    if (rows[i] >= 0) rows[i] = (int32_t)vpos[rows[i]];
}

// ------------------------------------------------------------------ gridlets

constexpr int kMCW = 8;  // makeGrids.cpp:46

// leaf bits of cells x0 .. x0+8 of row (j, k)
__device__ __forceinline__ uint32_t row_bits(const LevelD &l, int64_t x0, int64_t j, int64_t k)
{
  if (j >= l.n[1] || k >= l.n[2] || x0 >= l.n[0]) return 0;
  const uint64_t b = lin(l, x0, j, k);
  uint64_t w0 = l.leaf[b >> 5] >> (b & 31);
  if ((b & 31) > 23 && (b >> 5) + 1 < l.words) w0 |= (uint64_t)l.leaf[(b >> 5) + 1] << (32 - (b & 31));
  uint32_t m = (uint32_t)(w0 & 0x1ffu);
  const int64_t valid = l.n[0] - x0;
  if (valid < 9) m &= (1u << valid) - 1u;
  return m;
}

// bit t of mask[kk * 8 + jj]: a perfect cube with min corner (x0+t, y0+jj, z0+kk)
__device__ void cube_masks(const LevelD &l, const int64_t *m, uint64_t mc, uint8_t *mask)
{
  const int64_t mx = (int64_t)(mc % m[0]), my = (int64_t)((mc / m[0]) % m[1]), mz = (int64_t)(mc / (m[0] * m[1]));
  const int64_t x0 = mx * kMCW, y0 = my * kMCW, z0 = mz * kMCW;
  uint32_t rows[9][9];
  for (int kk = 0; kk < 9; ++kk)
    for (int jj = 0; jj < 9; ++jj) rows[kk][jj] = row_bits(l, x0, y0 + jj, z0 + kk);
  for (int kk = 0; kk < 8; ++kk)
    for (int jj = 0; jj < 8; ++jj) {
      const uint32_t a = rows[kk][jj] & rows[kk][jj + 1] & rows[kk + 1][jj] & rows[kk + 1][jj + 1];
      mask[kk * 8 + jj] = (uint8_t)(a & (a >> 1) & 0xffu);
    }
}

struct McGrid {
  int64_t m[3];
  uint64_t count;
};

// cubes per macrocell, the brick's cell box, its scalar count
__global__ void k_mc_boxes(TreeD T, int L, McGrid G, uint32_t *cnt, int4 *boxLo, int4 *boxHi, uint32_t *isBrick,
                           unsigned long long *ns)
{
  const LevelD &l = T.lv[L];
  for (uint64_t mc = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; mc < G.count;
       mc += gridDim.x * (uint64_t)blockDim.x) {
    uint8_t mask[64];
    cube_masks(l, G.m, mc, mask);
    const int64_t mx = (int64_t)(mc % G.m[0]), my = (int64_t)((mc / G.m[0]) % G.m[1]),
                  mz = (int64_t)(mc / (G.m[0] * G.m[1]));
    int32_t lo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, hi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    uint32_t c = 0;
    for (int kk = 0; kk < 8; ++kk)
      for (int jj = 0; jj < 8; ++jj) {
        const uint32_t bm = mask[kk * 8 + jj];
        if (!bm) continue;
        c += (uint32_t)__popc(bm);
        const int32_t i0 = (int32_t)(mx * kMCW) + __ffs(bm) - 1;
        const int32_t i1 = (int32_t)(mx * kMCW) + 31 - __clz(bm);
        const int32_t j = (int32_t)(my * kMCW + jj), k = (int32_t)(mz * kMCW + kk);
        lo[0] = min(lo[0], i0); hi[0] = max(hi[0], i1 + 1);
        lo[1] = min(lo[1], j); hi[1] = max(hi[1], j + 1);
        lo[2] = min(lo[2], k); hi[2] = max(hi[2], k + 1);
      }
    cnt[mc] = c;
    isBrick[mc] = c ? 1u : 0u;
    boxLo[mc] = make_int4(lo[0], lo[1], lo[2], 0);
    boxHi[mc] = make_int4(hi[0], hi[1], hi[2], 0);
    ns[mc] = c ? (unsigned long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) : 0ull;
  }
}

__global__ void k_mc_gridlets(int L, uint64_t count, const uint32_t *cnt, const int4 *boxLo, const int4 *boxHi,
                              const uint32_t *brickOf, const unsigned long long *scalarOff, uint64_t brickBase,
                              uint64_t scalarBase, exa_gridlet *gridlets)
{
  for (uint64_t mc = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; mc < count;
       mc += gridDim.x * (uint64_t)blockDim.x) {
    if (!cnt[mc]) continue;
    exa_gridlet g;
    const int4 lo = boxLo[mc], hi = boxHi[mc];
    g.lower = exa_vec3i{lo.x, lo.y, lo.z};
    g.level = L;
    g.dims = exa_vec3i{hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    g.begin = (uint32_t)(scalarBase + scalarOff[mc]);
    gridlets[brickBase + brickOf[mc]] = g;
  }
}

__global__ void k_fill_nan(float *p, uint64_t n)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x)
    p[i] = __int_as_float(0x7fc00000);
}

// corner values (Brick::write, makeGrids.cpp:114-168)
__global__ void k_mc_scalars(TreeD T, int L, McGrid G, const uint32_t *cnt, const uint32_t *brickOf,
                             uint64_t brickBase, const exa_gridlet *gridlets, const float *value, float *scalars)
{
  const LevelD &l = T.lv[L];
  for (uint64_t mc = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; mc < G.count;
       mc += gridDim.x * (uint64_t)blockDim.x) {
    if (!cnt[mc]) continue;
    uint8_t mask[64];
    cube_masks(l, G.m, mc, mask);
    const int64_t mx = (int64_t)(mc % G.m[0]), my = (int64_t)((mc / G.m[0]) % G.m[1]),
                  mz = (int64_t)(mc / (G.m[0] * G.m[1]));
    const exa_gridlet g = gridlets[brickBase + brickOf[mc]];
    const int64_t nx = g.dims.x + 1, ny = g.dims.y + 1;
    for (int kk = 0; kk < 8; ++kk)
      for (int jj = 0; jj < 8; ++jj) {
        uint32_t bm = mask[kk * 8 + jj];
        while (bm) {
          const int t = __ffs(bm) - 1;
          bm &= bm - 1;
          const int64_t i = mx * kMCW + t, j = my * kMCW + jj, k = mz * kMCW + kk;
          for (int d = 0; d < 8; ++d) {
            const int64_t ix = d & 1, iy = (d >> 1) & 1, iz = d >> 2;
            const uint64_t id = leaf_id(l, lin(l, i + ix, j + iy, k + iz));
            const int64_t lx = i + ix - g.lower.x, ly = j + iy - g.lower.y, lz = k + iz - g.lower.z;
            scalars[g.begin + (uint64_t)((lz * ny + ly) * nx + lx)] = value[id];
          }
        }
      }
  }
}

__global__ void k_count_nan(const float *p, uint64_t n, unsigned long long *out)
{
  unsigned long long c = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x)
    c += p[i] != p[i];
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void k_minmax(const float *v, uint64_t n, float *mm)
{
  float lo = INFINITY, hi = -INFINITY;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (uint64_t)blockDim.x) {
    lo = fminf(lo, v[i]);
    hi = fmaxf(hi, v[i]);
  }
  for (int o = 16; o; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    // ordered-integer min / max of floats
    auto key = [](float f) {
      const int b = __float_as_int(f);
      return b >= 0 ? b : b ^ 0x7fffffff;
    };
    atomicMin(reinterpret_cast<int *>(mm), key(lo));
    atomicMax(reinterpret_cast<int *>(mm) + 1, key(hi));
  }
}

// ------------------------------------------------------------------ driver

struct GpuBuilder {
  const exa_gen_params &P;
  exa_gen_result &R;
  cudaStream_t s = nullptr;
  int grid = 0;  // resident blocks for grid-stride kernels
  static constexpr int kThreads = 256;
  TreeD T{};
  std::vector<Dev<uint32_t>> refined, leaf, rank;
  std::vector<Dev<double>> gtabD[3];
  std::vector<Dev<float>> latD;
  FieldView fv{};
  Dev<float> value;
  Dev<int32_t> cells;

  GpuBuilder(const exa_gen_params &p, exa_gen_result &r, int device) : P(p), R(r)
  {
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    int sms = 0;
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attribute");
    grid = sms * 8;
    T.Lroot = p.numLevels - 1;
    refined.resize(p.numLevels);
    leaf.resize(p.numLevels);
    rank.resize(p.numLevels);
    for (int L = 0; L <= T.Lroot; ++L) {
      LevelD &l = T.lv[L];
      for (int a = 0; a < 3; ++a) l.n[a] = (int64_t)p.rootDims[a] << (T.Lroot - L);
      l.cells = (uint64_t)l.n[0] * l.n[1] * l.n[2];
      l.words = (l.cells + 31) / 32;
    }
  }
  ~GpuBuilder()
  {
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }
  void sync(const char *what) { ck(cudaStreamSynchronize(s), what); }
  void launched(const char *what) { ck(cudaGetLastError(), what); }
  int blocksFor(uint64_t n) const
  {
    const uint64_t b = (n + kThreads - 1) / kThreads;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(b, (uint64_t)grid));
  }

  // the field on the device: lattices, Gaussian tables (built on the host
  // by the same code as the CPU generator), cloud mapping range
  void setupField()
  {
    exagen::Field &F = R.field;
    F.setup(P);
    fv = F.view();
    latD.resize(F.latTab.size());
    for (size_t o = 0; o < F.latTab.size(); ++o) {
      latD[o].upload(F.latTab[o].data(), F.latTab[o].size(), s);
      fv.lat[o] = latD[o].p;
    }
    if (F.kind == EXA_FIELD_CLOUD) {
      const LevelD &l = T.lv[T.Lroot];
      const uint64_t n = l.cells;
      if (n >= 0x7fffffffull) throw std::runtime_error("root grid too large");
      Dev<double> raw(n), sorted(n);
      k_cloud_raw<<<blocksFor(n), kThreads, 0, s>>>(fv, T, raw.p);
      launched("k_cloud_raw");
      size_t tb = 0;
      ck(cub::DeviceRadixSort::SortKeys(nullptr, tb, raw.p, sorted.p, (int)n, 0, 64, s), "sort size");
      Dev<unsigned char> tmp(tb ? tb : 1);
      ck(cub::DeviceRadixSort::SortKeys(tmp.p, tb, raw.p, sorted.p, (int)n, 0, 64, s), "sort");
      const size_t q = std::min<size_t>(n - 1, (size_t)(P.cloudEmptyFraction * (double)n));
      double lo = 0, hi = 0;
      ck(cudaMemcpyAsync(&lo, sorted.p + q, sizeof(double), cudaMemcpyDeviceToHost, s), "cloud lo");
      ck(cudaMemcpyAsync(&hi, sorted.p + n - 1, sizeof(double), cudaMemcpyDeviceToHost, s), "cloud hi");
      sync("cloud range");
      F.cloudLo = lo;
      F.cloudHi = hi > lo ? hi : lo + 1.0;
      fv.cloudLo = F.cloudLo;
      fv.cloudHi = F.cloudHi;
    }
    sync("field set-up");
  }

  void buildGaussTables()
  {
    exagen::Field &F = R.field;
    for (int a = 0; a < 3; ++a) F.gtab[a].assign(T.Lroot + 1, {});
    if (F.kind != EXA_FIELD_GAUSSIANS) return;
    const int nt = exagen::numThreadsOf(&P);
    for (int a = 0; a < 3; ++a) gtabD[a].resize(T.Lroot + 1);
    for (int L = 0; L <= T.Lroot; ++L)
      for (int a = 0; a < 3; ++a) {
        const int64_t n = T.lv[L].n[a];
        auto &Tb = F.gtab[a][L];
        Tb.resize((size_t)n * F.K);
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t i = 0; i < n; ++i) F.gaussRow(a, L, i, &Tb[(size_t)i * F.K]);
        gtabD[a][L].upload(Tb.data(), Tb.size(), s);
        fv.gtab[a][L] = gtabD[a][L].p;
      }
    sync("gaussian tables");
  }

  void buildRank(int L)
  {
    LevelD &l = T.lv[L];
    const uint64_t nb = (l.words + kScanBlock - 1) / kScanBlock;
    if (nb >= 0x7fffffffull) throw std::runtime_error("level too large");
    Dev<uint32_t> bsum(nb), bbase(nb);
    k_rank_blocks<<<(unsigned)nb, kScanBlock, 0, s>>>(l.leaf, l.words, l.rank, bsum.p);
    launched("k_rank_blocks");
    size_t tb = 0;
    ck(cub::DeviceScan::ExclusiveSum(nullptr, tb, bsum.p, bbase.p, (int)nb, s), "scan size");
    Dev<unsigned char> tmp(tb ? tb : 1);
    ck(cub::DeviceScan::ExclusiveSum(tmp.p, tb, bsum.p, bbase.p, (int)nb, s), "scan");
    k_rank_add<<<(unsigned)nb, kScanBlock, 0, s>>>(l.rank, l.words, bbase.p);
    launched("k_rank_add");
    uint32_t lastBase = 0, lastSum = 0;
    ck(cudaMemcpyAsync(&lastBase, bbase.p + nb - 1, 4, cudaMemcpyDeviceToHost, s), "rank total");
    ck(cudaMemcpyAsync(&lastSum, bsum.p + nb - 1, 4, cudaMemcpyDeviceToHost, s), "rank total");
    sync("rank");
    R.stats.numCellsPerLevel[L] = (uint64_t)lastBase + lastSum;
  }

  void buildTree()
  {
    const int Lroot = T.Lroot;
    const double thr = (double)P.refineThreshold;
    for (int L = 0; L <= Lroot; ++L) {
      LevelD &l = T.lv[L];
      leaf[L].alloc(l.words);
      rank[L].alloc(l.words);
      l.leaf = leaf[L].p;
      l.rank = rank[L].p;
      if (L >= 1) {
        refined[L].alloc(l.words);
        refined[L].zero(s);
        l.refined = refined[L].p;
      }
    }
    double maxAbs = 0;
    {
      const LevelD &root = T.lv[Lroot];
      Dev<float> rootVal(root.cells);
      Dev<unsigned long long> mx(1);
      mx.zero(s);
      k_root_eval<<<blocksFor(root.cells), kThreads, 0, s>>>(fv, T, rootVal.p, mx.p);
      launched("k_root_eval");
      unsigned long long bits = 0;
      ck(cudaMemcpyAsync(&bits, mx.p, 8, cudaMemcpyDeviceToHost, s), "max");
      sync("root eval");
      std::memcpy(&maxAbs, &bits, 8);
      if (Lroot > 0) {
        k_root_refine<<<blocksFor(root.cells), kThreads, 0, s>>>(T, rootVal.p, P.fieldKind, thr, maxAbs);
        launched("k_root_refine");
      }
      sync("root refine");
    }
    for (int L = Lroot - 1; L >= 1; --L) {
      k_refine_level<<<blocksFor(T.lv[L + 1].words), kThreads, 0, s>>>(fv, T, L, P.fieldKind, thr, maxAbs);
      launched("k_refine_level");
    }
    if (P.balance)
      for (int L = 1; L < Lroot; ++L) {
        k_balance<<<blocksFor(T.lv[L].words), kThreads, 0, s>>>(T, L);
        launched("k_balance");
      }
    uint64_t off = 0;
    for (int L = 0; L <= Lroot; ++L) {
      if (T.lv[L].n[0] % 32 == 0) {
        k_leaf_words<<<blocksFor(T.lv[L].words), kThreads, 0, s>>>(T, L);
        launched("k_leaf_words");
      } else {
        k_leaf_bits<<<blocksFor(T.lv[L].cells), kThreads, 0, s>>>(T, L);
        launched("k_leaf_bits");
      }
      buildRank(L);
      T.lv[L].leafOffset = off;
      off += R.stats.numCellsPerLevel[L];
    }
    R.stats.numAmrCells = off;
  }

  void computeValues()
  {
    const uint64_t n = R.stats.numAmrCells;
    value.alloc(n);
    cells.alloc(n * 4);
    for (int L = 0; L <= T.Lroot; ++L) {
      k_values<<<blocksFor(T.lv[L].words), kThreads, 0, s>>>(fv, T, L, value.p, cells.p);
      launched("k_values");
    }
    Dev<float> mm(2);
    const int init[2] = {0x7fffffff, (int)0x80000000};
    ck(cudaMemcpyAsync(mm.p, init, 8, cudaMemcpyHostToDevice, s), "minmax init");
    if (n) {
      k_minmax<<<blocksFor(n), kThreads, 0, s>>>(value.p, n, mm.p);
      launched("k_minmax");
    }
    int k[2];
    ck(cudaMemcpyAsync(k, mm.p, 8, cudaMemcpyDeviceToHost, s), "minmax");
    sync("values");
    auto unkey = [](int b) {
      const int f = b >= 0 ? b : b ^ 0x7fffffff;
      float v;
      std::memcpy(&v, &f, 4);
      return v;
    };
    R.stats.fieldMin = n ? unkey(k[0]) : INFINITY;
    R.stats.fieldMax = n ? unkey(k[1]) : -INFINITY;
    R.amrScalars.resize(n);
    R.amrCells.resize(n * 4);
    value.download(R.amrScalars.data(), n, s);
    cells.download(R.amrCells.data(), n * 4, s);
  }

  template <typename T_>
  void exclusiveScan(const T_ *in, T_ *out, uint64_t n, const char *what)
  {
    if (n >= 0x7fffffffull) throw std::runtime_error(std::string(what) + ": too many items");
    size_t tb = 0;
    ck(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, (int)n, s), what);
    Dev<unsigned char> tmp(tb ? tb : 1);
    ck(cub::DeviceScan::ExclusiveSum(tmp.p, tb, in, out, (int)n, s), what);
  }

  void buildElements()
  {
    const uint64_t n = R.stats.numAmrCells;
    Dev<uint32_t> packed(n);
    Dev<unsigned long long> skipped(1);
    skipped.zero(s);
    for (int L = 0; L <= T.Lroot; ++L) {
      k_elem_count<<<blocksFor(T.lv[L].words), kThreads, 0, s>>>(T, L, packed.p, skipped.p);
      launched("k_elem_count");
    }
    // the leaves that emit elements, in leaf-id order
    Dev<uint32_t> flag(n), pos(n);
    k_flag_nonzero<<<blocksFor(n), kThreads, 0, s>>>(packed.p, n, flag.p);
    launched("k_flag_nonzero");
    exclusiveScan(flag.p, pos.p, n, "active scan");
    uint32_t lastPos = 0, lastFlag = 0;
    if (n) {
      ck(cudaMemcpyAsync(&lastPos, pos.p + n - 1, 4, cudaMemcpyDeviceToHost, s), "active count");
      ck(cudaMemcpyAsync(&lastFlag, flag.p + n - 1, 4, cudaMemcpyDeviceToHost, s), "active count");
    }
    unsigned long long sk = 0;
    ck(cudaMemcpyAsync(&sk, skipped.p, 8, cudaMemcpyDeviceToHost, s), "skipped");
    sync("element count");
    R.stats.numSkippedDegenerate = sk;
    const uint32_t m = lastPos + lastFlag;
    Dev<uint32_t> ids(m), cnt(m), tc(m);
    Dev<uint32_t> off[4];
    uint64_t total[4] = {0, 0, 0, 0};
    if (m) {
      k_compact<<<blocksFor(n), kThreads, 0, s>>>(packed.p, n, pos.p, ids.p, cnt.p);
      launched("k_compact");
      for (int t = 0; t < 4; ++t) {
        off[t].alloc(m);
        k_type_counts<<<blocksFor(m), kThreads, 0, s>>>(cnt.p, m, t, tc.p);
        launched("k_type_counts");
        exclusiveScan(tc.p, off[t].p, m, "type scan");
        uint32_t lo = 0, lc = 0;
        ck(cudaMemcpyAsync(&lo, off[t].p + m - 1, 4, cudaMemcpyDeviceToHost, s), "type total");
        ck(cudaMemcpyAsync(&lc, tc.p + m - 1, 4, cudaMemcpyDeviceToHost, s), "type total");
        sync("type scan");
        total[t] = (uint64_t)lo + lc;
      }
    }
    packed = Dev<uint32_t>();
    flag = Dev<uint32_t>();
    R.stats.numTets = total[0];
    R.stats.numPyramids = total[1];
    R.stats.numWedges = total[2];
    R.stats.numHexes = total[3];
    const uint64_t ne = total[0] + total[1] + total[2] + total[3];
    Dev<int32_t> rows(ne * 8);
    Dev<uint8_t> used(n);
    used.zero(s);
    if (m) {
      k_elem_write<<<blocksFor(m), kThreads, 0, s>>>(T, ids.p, m, cells.p, off[0].p, off[1].p, off[2].p, off[3].p,
                                                      total[0], total[0] + total[1], total[0] + total[1] + total[2],
                                                      rows.p, used.p);
      launched("k_elem_write");
    }
    // vertex compaction: used leaves in ascending leaf id
    Dev<uint32_t> used32(n), vpos(n);
    k_u8_to_u32<<<blocksFor(n), kThreads, 0, s>>>(used.p, n, used32.p);
    launched("k_u8_to_u32");
    exclusiveScan(used32.p, vpos.p, n, "vertex scan");
    uint32_t lv = 0, lu = 0;
    if (n) {
      ck(cudaMemcpyAsync(&lv, vpos.p + n - 1, 4, cudaMemcpyDeviceToHost, s), "vertex count");
      ck(cudaMemcpyAsync(&lu, used32.p + n - 1, 4, cudaMemcpyDeviceToHost, s), "vertex count");
    }
    sync("vertex scan");
    const uint64_t nv = (uint64_t)lv + lu;
    Dev<float4> verts(nv);
    k_vertices<<<blocksFor(n), kThreads, 0, s>>>(used.p, vpos.p, n, cells.p, value.p, verts.p);
    launched("k_vertices");
    k_remap<<<blocksFor(ne * 8), kThreads, 0, s>>>(rows.p, ne * 8, vpos.p);
    launched("k_remap");
    R.vertices.resize(nv);
    R.indices.resize(ne * 8);
    verts.download(reinterpret_cast<float4 *>(R.vertices.data()), nv, s);
    rows.download(R.indices.data(), ne * 8, s);
    sync("elements");
    R.stats.numVertices = nv;
  }

  void buildGridlets()
  {
    // pass 1 per level: brick boxes and sizes
    struct LevelBricks {
      McGrid G;
      Dev<uint32_t> cnt, brickOf;
      Dev<unsigned long long> scalarOff;
      Dev<int4> lo, hi;
      uint64_t bricks = 0, scalars = 0, brickBase = 0, scalarBase = 0;
    };
    std::vector<LevelBricks> B(T.Lroot + 1);
    uint64_t brickTotal = 0, scalarTotal = 0, cubes = 0;
    for (int L = 0; L <= T.Lroot; ++L) {
      const LevelD &l = T.lv[L];
      LevelBricks &b = B[L];
      for (int a = 0; a < 3; ++a) b.G.m[a] = (l.n[a] + kMCW - 1) / kMCW;
      b.G.count = (uint64_t)b.G.m[0] * b.G.m[1] * b.G.m[2];
      const uint64_t nmc = b.G.count;
      b.cnt.alloc(nmc);
      b.brickOf.alloc(nmc);
      b.scalarOff.alloc(nmc);
      b.lo.alloc(nmc);
      b.hi.alloc(nmc);
      Dev<uint32_t> isBrick(nmc);
      Dev<unsigned long long> ns(nmc);
      k_mc_boxes<<<blocksFor(nmc), kThreads, 0, s>>>(T, L, b.G, b.cnt.p, b.lo.p, b.hi.p, isBrick.p, ns.p);
      launched("k_mc_boxes");
      exclusiveScan(isBrick.p, b.brickOf.p, nmc, "brick scan");
      exclusiveScan(ns.p, b.scalarOff.p, nmc, "scalar scan");
      // cube count of the level
      Dev<unsigned long long> cubeSum(1);
      cubeSum.zero(s);
      uint32_t lb = 0, li = 0;
      unsigned long long lso = 0, lns = 0;
      ck(cudaMemcpyAsync(&lb, b.brickOf.p + nmc - 1, 4, cudaMemcpyDeviceToHost, s), "brick count");
      ck(cudaMemcpyAsync(&li, isBrick.p + nmc - 1, 4, cudaMemcpyDeviceToHost, s), "brick count");
      ck(cudaMemcpyAsync(&lso, b.scalarOff.p + nmc - 1, 8, cudaMemcpyDeviceToHost, s), "scalar count");
      ck(cudaMemcpyAsync(&lns, ns.p + nmc - 1, 8, cudaMemcpyDeviceToHost, s), "scalar count");
      {
        size_t tb = 0;
        if (nmc >= 0x7fffffffull) throw std::runtime_error("too many macrocells");
        ck(cub::DeviceReduce::Sum(nullptr, tb, b.cnt.p, cubeSum.p, (int)nmc, s), "cube sum");
        Dev<unsigned char> tmp(tb ? tb : 1);
        ck(cub::DeviceReduce::Sum(tmp.p, tb, b.cnt.p, cubeSum.p, (int)nmc, s), "cube sum");
        unsigned long long cs = 0;
        ck(cudaMemcpyAsync(&cs, cubeSum.p, 8, cudaMemcpyDeviceToHost, s), "cube sum");
        sync("bricks");
        cubes += cs;
      }
      b.bricks = (uint64_t)lb + li;
      b.scalars = lso + lns;
      b.brickBase = brickTotal;
      b.scalarBase = scalarTotal;
      brickTotal += b.bricks;
      scalarTotal += b.scalars;
      if (scalarTotal > 0xffffffffull) throw std::runtime_error("gridlet scalar offset overflow");
    }
    R.stats.numPerfectCubes = cubes;
    Dev<exa_gridlet> gridlets(brickTotal);
    Dev<float> scalars(scalarTotal);
    if (scalarTotal) {
      k_fill_nan<<<blocksFor(scalarTotal), kThreads, 0, s>>>(scalars.p, scalarTotal);
      launched("k_fill_nan");
    }
    for (int L = 0; L <= T.Lroot; ++L) {
      LevelBricks &b = B[L];
      k_mc_gridlets<<<blocksFor(b.G.count), kThreads, 0, s>>>(L, b.G.count, b.cnt.p, b.lo.p, b.hi.p, b.brickOf.p,
                                                               b.scalarOff.p, b.brickBase, b.scalarBase, gridlets.p);
      launched("k_mc_gridlets");
      k_mc_scalars<<<blocksFor(b.G.count), kThreads, 0, s>>>(T, L, b.G, b.cnt.p, b.brickOf.p, b.brickBase,
                                                              gridlets.p, value.p, scalars.p);
      launched("k_mc_scalars");
    }
    Dev<unsigned long long> nanCount(1);
    nanCount.zero(s);
    if (scalarTotal) {
      k_count_nan<<<blocksFor(scalarTotal), kThreads, 0, s>>>(scalars.p, scalarTotal, nanCount.p);
      launched("k_count_nan");
    }
    unsigned long long empty = 0;
    ck(cudaMemcpyAsync(&empty, nanCount.p, 8, cudaMemcpyDeviceToHost, s), "nan count");
    R.gridlets.resize(brickTotal);
    R.gridletScalars.resize(scalarTotal);
    gridlets.download(R.gridlets.data(), brickTotal, s);
    scalars.download(R.gridletScalars.data(), scalarTotal, s);
    sync("gridlets");
    R.stats.numGridlets = brickTotal;
    R.stats.numGridletScalars = scalarTotal;
    R.stats.numEmptyGridletScalars = empty;
  }
};

} // namespace

extern "C" int exa_gen_run_gpu(const exa_gen_params *p, int device, exa_gen_result **out)
{
  exa_gen_result *r = nullptr;
  try {
    if (!out) throw std::runtime_error("null argument");
    exagen::checkParams(p);
    const auto t0 = std::chrono::steady_clock::now();
    r = new exa_gen_result();
    r->params = *p;
    std::memset(&r->stats, 0, sizeof(r->stats));
    {
      GpuBuilder B(*p, *r, device);
      auto stage = [&](int k, auto &&fn) {
        const auto a = std::chrono::steady_clock::now();
        fn();
        r->stats.stageSeconds[k] = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
      };
      stage(0, [&] { B.setupField(); });
      stage(1, [&] { B.buildGaussTables(); });
      stage(2, [&] { B.buildTree(); });
      if (r->stats.numAmrCells >= 0x7fffffffull) throw std::runtime_error("too many AMR cells for 32-bit ids");
      stage(3, [&] { B.computeValues(); });
      stage(4, [&] { B.buildElements(); });
      stage(5, [&] { B.buildGridlets(); });
    }
    r->stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = r;
    return 0;
  } catch (const std::exception &e) {
    delete r;
    exagen::setLastError(e.what());
    return 1;
  }
}
