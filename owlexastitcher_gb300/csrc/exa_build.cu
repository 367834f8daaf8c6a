// exa_build.cu -- build-time kernels: the per-macrocell majorant grid
// (Grid.cu:61-246), per-primitive value ranges and max opacities
// (sampler/ExaStitchSampler.cu:27-227, Grid.cu:687-719) and the GPU linear
// BVH over stitching elements that replaces the OptiX BLAS build.
#include <cub/block/block_scan.cuh>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "exa_host.h"

namespace exa {

void cudaCheck(cudaError_t e, const char *what)
{
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? EXA_ERR_OOM : EXA_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
  }
}

static inline unsigned gridFor(size_t n, unsigned block)
{
  return (unsigned)((n + block - 1) / block);
}

// ------------------------------------------------------------ Grid.cu:61-70
__global__ void k_init_ranges(exa_range1f *r, size_t n)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  r[i].lower = +1e30f;
  r[i].upper = -1e30f;
}

void launchInitRanges(exa_range1f *r, size_t n, cudaStream_t s)
{
  if (!n) return;
  k_init_ranges<<<gridFor(n, 256), 256, 0, s>>>(r, n);
  cudaCheck(cudaGetLastError(), "k_init_ranges");
}

__device__ __forceinline__ void update_mc(exa_range1f *mc, const exa_vec3i dims, int x, int y, int z, float lo,
                                          float hi)
{
  exa_range1f *m = mc + ((size_t)z * dims.y + y) * dims.x + x;
  atomic_min_float(&m->lower, lo);
  atomic_max_float(&m->upper, hi);
}

// Grid.cu:134-246 fused with computeGridletValueRangesGPU
// (sampler/ExaStitchSampler.cu:52-142): one block per gridlet, one thread
// per cell.  A cell only tests the macrocells within one of its own
// projection (the reference tests every macrocell of the gridlet's range;
// the exact overlap test below decides in both cases, so the set of
// updated macrocells is the same).
__global__ void __launch_bounds__(128) k_gridlet_majorants(const exa_gridlet *__restrict__ gridlets,
                                                           const float *__restrict__ scalars, exa_vec3i dims,
                                                           exa_box3f wb, exa_range1f *mcRanges,
                                                           exa_range1f *gridletRanges)
{
  const exa_gridlet g = gridlets[blockIdx.x];
  const float cw = (float)(1 << g.level);
  exa_box3f gb;
  gb.lower.x = ((float)g.lower.x + 0.5f) * cw;
  gb.lower.y = ((float)g.lower.y + 0.5f) * cw;
  gb.lower.z = ((float)g.lower.z + 0.5f) * cw;
  gb.upper.x = (((float)g.lower.x + (float)g.dims.x) + 0.5f) * cw;
  gb.upper.y = (((float)g.lower.y + (float)g.dims.y) + 0.5f) * cw;
  gb.upper.z = (((float)g.lower.z + (float)g.dims.z) + 0.5f) * cw;
  const V3i D = {dims.x, dims.y, dims.z};
  const V3i loMC = project_on_grid(mk3(gb.lower), D, wb);
  const V3i hiMC = project_on_grid(mk3(gb.upper), D, wb);
  const V3 mcSize = div3(sub3(mk3(wb.upper), mk3(wb.lower)), mk3((float)dims.x, (float)dims.y, (float)dims.z));
  const int nx = g.dims.x + 1, ny = g.dims.y + 1;
  const int ncells = g.dims.x * g.dims.y * g.dims.z;
  const float *S = scalars + g.begin;
  float glo = 1e30f, ghi = -1e30f;
  for (int c = threadIdx.x; c < ncells; c += blockDim.x) {
    const int x = c % g.dims.x, y = (c / g.dims.x) % g.dims.y, z = c / (g.dims.x * g.dims.y);
    const float f[8] = {__ldg(S + (z * ny + y) * nx + x), __ldg(S + (z * ny + y) * nx + x + 1),
                        __ldg(S + (z * ny + y + 1) * nx + x), __ldg(S + (z * ny + y + 1) * nx + x + 1),
                        __ldg(S + ((z + 1) * ny + y) * nx + x), __ldg(S + ((z + 1) * ny + y) * nx + x + 1),
                        __ldg(S + ((z + 1) * ny + y + 1) * nx + x), __ldg(S + ((z + 1) * ny + y + 1) * nx + x + 1)};
    float lo = 1e30f, hi = -1e30f;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (!isnan(f[k])) { lo = fminf(lo, f[k]); hi = fmaxf(hi, f[k]); }
    glo = fminf(glo, lo);
    ghi = fmaxf(ghi, hi);
    if (hi < lo) continue;  // no non-NaN corner: the reference's update is a no-op
    // Grid.cu:181-182
    const V3 clo = add3(muls(mk3((float)(g.lower.x + x), (float)(g.lower.y + y), (float)(g.lower.z + z)), cw),
                        mk3(0.5f * cw, 0.5f * cw, 0.5f * cw));
    const V3 chi = add3(muls(mk3((float)(g.lower.x + x + 1), (float)(g.lower.y + y + 1), (float)(g.lower.z + z + 1)), cw),
                        mk3(0.5f * cw, 0.5f * cw, 0.5f * cw));
    const V3i pl = project_on_grid(clo, D, wb), ph = project_on_grid(chi, D, wb);
    const int x0 = imax_t(loMC.x, pl.x - 1), x1 = imin_t(hiMC.x, ph.x + 1);
    const int y0 = imax_t(loMC.y, pl.y - 1), y1 = imin_t(hiMC.y, ph.y + 1);
    const int z0 = imax_t(loMC.z, pl.z - 1), z1 = imin_t(hiMC.z, ph.z + 1);
    for (int mz = z0; mz <= z1; ++mz)
      for (int my = y0; my <= y1; ++my)
        for (int mx = x0; mx <= x1; ++mx) {
          const V3 mlo = add3(mk3(wb.lower), mul3(mk3((float)mx, (float)my, (float)mz), mcSize));
          const V3 mhi = add3(mk3(wb.lower), mul3(mk3((float)(mx + 1), (float)(my + 1), (float)(mz + 1)), mcSize));
          if (mlo.x <= chi.x && mlo.y <= chi.y && mlo.z <= chi.z && clo.x <= mhi.x && clo.y <= mhi.y &&
              clo.z <= mhi.z)
            update_mc(mcRanges, dims, mx, my, mz, lo, hi);
        }
  }
  // block reduction of the gridlet's range
  __shared__ float sLo[4], sHi[4];
  for (int o = 16; o > 0; o >>= 1) {
    glo = fminf(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmaxf(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sLo[warp] = glo; sHi[warp] = ghi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { glo = fminf(glo, sLo[w]); ghi = fmaxf(ghi, sHi[w]); }
    gridletRanges[blockIdx.x].lower = glo;
    gridletRanges[blockIdx.x].upper = ghi;
  }
}

void launchGridletMajorants(const exa_gridlet *g, const float *scalars, size_t ng, exa_vec3i dims, exa_box3f wb,
                            exa_range1f *mcRanges, exa_range1f *gridletRanges, cudaStream_t s)
{
  if (!ng) return;
  for (size_t off = 0; off < ng; off += 0x7fffffff) {
    const size_t cnt = ng - off < 0x7fffffff ? ng - off : 0x7fffffff;
    k_gridlet_majorants<<<(unsigned)cnt, 128, 0, s>>>(g + off, scalars, dims, wb, mcRanges, gridletRanges + off);
  }
  cudaCheck(cudaGetLastError(), "k_gridlet_majorants");
}

// Grid.cu:73-117 (buildGrid<8>) plus the element's own range with the
// min/max of computeUmeshMaxOpacitiesGPU (sampler/ExaStitchSampler.cu:
// 201-206)
__global__ void k_elem_majorants(const float4 *__restrict__ verts, const int32_t *__restrict__ indices, size_t ne,
                                 exa_vec3i dims, exa_box3f wb, exa_range1f *mcRanges, exa_range1f *elemRanges)
{
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int4 i0 = __ldg(reinterpret_cast<const int4 *>(indices + e * 8));
  const int4 i1 = __ldg(reinterpret_cast<const int4 *>(indices + e * 8) + 1);
  const int I[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
  V3 blo = mk3(INFINITY, INFINITY, INFINITY), bhi = mk3(-INFINITY, -INFINITY, -INFINITY);
  float lo = 1e30f, hi = -1e30f;
  float elo = 1e30f, ehi = -1e30f;
  bool any = false;
  for (int i = 0; i < 8; ++i) {
    if (I[i] < 0) break;
    const float4 V = __ldg(verts + I[i]);
    elo = fmin_t(elo, V.w);
    ehi = fmax_t(ehi, V.w);
    if (!isnan(V.w)) {
      blo = min3(blo, mk3(V.x, V.y, V.z));
      bhi = max3(bhi, mk3(V.x, V.y, V.z));
      lo = fminf(lo, V.w);
      hi = fmaxf(hi, V.w);
      any = true;
    }
  }
  elemRanges[e].lower = elo;
  elemRanges[e].upper = ehi;
  if (!any) return;
  const V3i D = {dims.x, dims.y, dims.z};
  const V3i a = project_on_grid(blo, D, wb), b = project_on_grid(bhi, D, wb);
  for (int z = a.z; z <= b.z; ++z)
    for (int y = a.y; y <= b.y; ++y)
      for (int x = a.x; x <= b.x; ++x) update_mc(mcRanges, dims, x, y, z, lo, hi);
}

void launchElemMajorants(const float4 *verts, const int32_t *idx, size_t ne, exa_vec3i dims, exa_box3f wb,
                         exa_range1f *mcRanges, exa_range1f *elemRanges, cudaStream_t s)
{
  if (!ne) return;
  k_elem_majorants<<<gridFor(ne, 256), 256, 0, s>>>(verts, idx, ne, dims, wb, mcRanges, elemRanges);
  cudaCheck(cudaGetLastError(), "k_elem_majorants");
}

// Grid.cu:248-285 (the AMR-cell overload of buildGrid): a cell's support
// [pos - w/2, pos + w + w/2] projected onto the grid; NaN values add nothing
__global__ void k_amrcell_majorants(const exa_amr_cell *__restrict__ cells, const float *__restrict__ scalars,
                                    size_t n, exa_vec3i dims, exa_box3f wb, exa_range1f *mcRanges)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const exa_amr_cell c = cells[i];
  const float value = scalars[i];
  if (isnan(value)) return;
  const int w = 1 << c.level;
  const float half = (float)w * .5f;
  const V3 lo = mk3((float)c.pos.x - half, (float)c.pos.y - half, (float)c.pos.z - half);
  const V3 hi = mk3((float)(c.pos.x + w) + half, (float)(c.pos.y + w) + half, (float)(c.pos.z + w) + half);
  const V3i D = {dims.x, dims.y, dims.z};
  const V3i a = project_on_grid(lo, D, wb), b = project_on_grid(hi, D, wb);
  for (int z = a.z; z <= b.z; ++z)
    for (int y = a.y; y <= b.y; ++y)
      for (int x = a.x; x <= b.x; ++x) update_mc(mcRanges, dims, x, y, z, value, value);
}

void launchAmrCellMajorants(const exa_amr_cell *cells, const float *scalars, size_t n, exa_vec3i dims, exa_box3f wb,
                            exa_range1f *mcRanges, cudaStream_t s)
{
  if (!n) return;
  k_amrcell_majorants<<<gridFor(n, 256), 256, 0, s>>>(cells, scalars, n, dims, wb, mcRanges);
  cudaCheck(cudaGetLastError(), "k_amrcell_majorants");
}

__device__ __forceinline__ bool amr_lattice(const exa_amr_cell &c, int level, const int *lo, const int *nl,
                                            size_t &lin)
{
  if (c.level != level) return false;
  const int x = (c.pos.x >> level) - lo[0], y = (c.pos.y >> level) - lo[1], z = (c.pos.z >> level) - lo[2];
  lin = ((size_t)z * nl[1] + y) * nl[0] + x;
  return true;
}

struct AmrLattice {
  int lo[3], n[3];
};

__global__ void k_amr_level_bits(const exa_amr_cell *cells, size_t n, int level, AmrLattice G, uint32_t *bits,
                                 unsigned *dupFlag)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  size_t c;
  if (!amr_lattice(cells[i], level, G.lo, G.n, c)) return;
  const uint32_t m = 1u << (c & 31);
  if (atomicOr(bits + (c >> 5), m) & m) atomicOr(dupFlag, 1u);
}

void launchAmrLevelBits(const exa_amr_cell *cells, size_t n, int level, const int lo[3], const int nl[3],
                        uint32_t *bits, unsigned *dupFlag, cudaStream_t s)
{
  if (!n) return;
  const AmrLattice G{{lo[0], lo[1], lo[2]}, {nl[0], nl[1], nl[2]}};
  k_amr_level_bits<<<gridFor(n, 256), 256, 0, s>>>(cells, n, level, G, bits, dupFlag);
  cudaCheck(cudaGetLastError(), "k_amr_level_bits");
}

constexpr int kRankBlock = 1024;

__global__ void k_rank_blocks(const uint32_t *bits, size_t words, uint32_t *rank, uint32_t *blockSum)
{
  typedef cub::BlockScan<uint32_t, kRankBlock> Scan;
  __shared__ typename Scan::TempStorage tmp;
  const size_t w = blockIdx.x * (size_t)kRankBlock + threadIdx.x;
  const uint32_t v = w < words ? (uint32_t)__popc(bits[w]) : 0u;
  uint32_t ex, total;
  Scan(tmp).ExclusiveSum(v, ex, total);
  if (w < words) rank[w] = ex;
  if (threadIdx.x == 0) blockSum[blockIdx.x] = total;
}

__global__ void k_rank_add(uint32_t *rank, size_t words, const uint32_t *blockBase)
{
  const size_t w = blockIdx.x * (size_t)kRankBlock + threadIdx.x;
  if (w < words) rank[w] += blockBase[blockIdx.x];
}

// exclusive prefix popcount per word: block scans, a scan of the block sums
void launchAmrLevelRank(const uint32_t *bits, size_t words, uint32_t *rank, cudaStream_t s)
{
  if (!words) return;
  const size_t nb = (words + kRankBlock - 1) / kRankBlock;
  if (nb >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "AMR level lattice too large");
  DBuf<uint32_t> bsum, bbase;
  bsum.alloc(nb);
  bbase.alloc(nb);
  k_rank_blocks<<<(unsigned)nb, kRankBlock, 0, s>>>(bits, words, rank, bsum.ptr);
  cudaCheck(cudaGetLastError(), "k_rank_blocks");
  size_t tb = 0;
  cudaCheck(cub::DeviceScan::ExclusiveSum(nullptr, tb, bsum.ptr, bbase.ptr, (int)nb, s), "scan size");
  DBuf<unsigned char> tmp;
  tmp.alloc(tb ? tb : 1);
  cudaCheck(cub::DeviceScan::ExclusiveSum(tmp.ptr, tb, bsum.ptr, bbase.ptr, (int)nb, s), "scan");
  k_rank_add<<<(unsigned)nb, kRankBlock, 0, s>>>(rank, words, bbase.ptr);
  cudaCheck(cudaGetLastError(), "k_rank_add");
  cudaCheck(cudaStreamSynchronize(s), "amr rank");
}

__global__ void k_amr_level_cells(const exa_amr_cell *cells, size_t n, int level, AmrLattice G, const uint32_t *bits,
                                  const uint32_t *rank, int32_t *cellOf)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  size_t c;
  if (!amr_lattice(cells[i], level, G.lo, G.n, c)) return;
  cellOf[rank[c >> 5] + __popc(bits[c >> 5] & ((1u << (c & 31)) - 1u))] = (int32_t)i;
}

void launchAmrLevelCells(const exa_amr_cell *cells, size_t n, int level, const int lo[3], const int nl[3],
                         const uint32_t *bits, const uint32_t *rank, int32_t *cellOf, cudaStream_t s)
{
  if (!n) return;
  const AmrLattice G{{lo[0], lo[1], lo[2]}, {nl[0], nl[1], nl[2]}};
  k_amr_level_cells<<<gridFor(n, 256), 256, 0, s>>>(cells, n, level, G, bits, rank, cellOf);
  cudaCheck(cudaGetLastError(), "k_amr_level_cells");
}

// Grid.cu:687-719; the color map is staged in shared memory
__global__ void k_max_opacity(const exa_range1f *__restrict__ ranges, size_t n, const float4 *__restrict__ cmap,
                              int ncolors, exa_range1f xf, float *out)
{
  extern __shared__ float4 sCmap[];
  for (int i = threadIdx.x; i < ncolors; i += blockDim.x) sCmap[i] = cmap[i];
  __syncthreads();
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = range_max_opacity(ranges[i], sCmap, ncolors, xf);
}

__global__ void k_max_opacity_global(const exa_range1f *__restrict__ ranges, size_t n,
                                     const float4 *__restrict__ cmap, int ncolors, exa_range1f xf, float *out)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = range_max_opacity(ranges[i], cmap, ncolors, xf);
}

void launchMaxOpacity(const exa_range1f *ranges, size_t n, const float4 *cmap, int ncolors, exa_range1f xf,
                      float *out, cudaStream_t s)
{
  if (!n) return;
  const size_t smem = (size_t)ncolors * sizeof(float4);
  if (smem <= 48 * 1024)
    k_max_opacity<<<gridFor(n, 256), 256, smem, s>>>(ranges, n, cmap, ncolors, xf, out);
  else
    k_max_opacity_global<<<gridFor(n, 256), 256, 0, s>>>(ranges, n, cmap, ncolors, xf, out);
  cudaCheck(cudaGetLastError(), "k_max_opacity");
}

// ------------------------------------------------------------ element LBVH
__device__ __forceinline__ uint32_t expand_bits10(uint32_t v)
{
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__device__ __forceinline__ void elem_box(const float4 *verts, const int32_t *indices, size_t e, V3 &lo, V3 &hi)
{
  lo = mk3(INFINITY, INFINITY, INFINITY);
  hi = mk3(-INFINITY, -INFINITY, -INFINITY);
  for (int i = 0; i < 8; ++i) {
    const int id = __ldg(indices + e * 8 + i);
    if (id < 0) break;
    const float4 v = __ldg(verts + id);
    lo = min3(lo, mk3(v.x, v.y, v.z));
    hi = max3(hi, mk3(v.x, v.y, v.z));
  }
}

// 30-bit Morton code of the box centre, tie-broken by element id
__global__ void k_bvh_keys(const float4 *verts, const int32_t *indices, size_t ne, exa_box3f sb, uint64_t *keys)
{
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  V3 lo, hi;
  elem_box(verts, indices, e, lo, hi);
  const V3 c = muls(add3(lo, hi), 0.5f);
  const V3 ext = sub3(mk3(sb.upper), mk3(sb.lower));
  uint32_t q[3];
  const float cc[3] = {c.x, c.y, c.z}, sl[3] = {sb.lower.x, sb.lower.y, sb.lower.z}, ex[3] = {ext.x, ext.y, ext.z};
  for (int a = 0; a < 3; ++a) {
    float t = ex[a] > 0.f ? (cc[a] - sl[a]) / ex[a] : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    q[a] = (uint32_t)fminf(t * 1024.f, 1023.f);
  }
  const uint32_t m = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
  keys[e] = ((uint64_t)m << 32) | (uint64_t)e;
}

__device__ __forceinline__ int lcp(const uint64_t *keys, int n, int i, int j)
{
  if (j < 0 || j >= n) return -1;
  return __clzll(keys[i] ^ keys[j]);
}

// Karras 2012, Algorithm 4: internal node i covers a key range whose split
// is the highest differing bit; children are leaves when the range ends.
__global__ void k_bvh_karras(const uint64_t *keys, int n, BvhNode *nodes, int32_t *parents, int32_t *leafElem)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) leafElem[i] = (int32_t)(keys[i] & 0xffffffffu);
  if (i >= n - 1) return;
  const int d = lcp(keys, n, i, i + 1) > lcp(keys, n, i, i - 1) ? 1 : -1;
  const int dmin = lcp(keys, n, i, i - d);
  int lmax = 2;
  while (lcp(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (lcp(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = lcp(keys, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (lcp(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + (d < 0 ? d : 0);
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  // children: internal index >= 0, leaf position p encoded as -(p+1) here
  const int left = (lo == gamma) ? -(gamma + 1) : gamma;
  const int right = (hi == gamma + 1) ? -(gamma + 2) : gamma + 1;
  const int ch[2] = {left, right};
  for (int k = 0; k < 2; ++k) {
    const int c = ch[k];
    if (c >= 0) {
      nodes[i].child[k] = c;
      parents[c] = i * 2 + k;
    } else {
      const int p = -c - 1;
      nodes[i].child[k] = ~(int32_t)(keys[p] & 0xffffffffu);
      parents[(n - 1) + p] = i * 2 + k;
    }
  }
}

// single-element tree: root slot 0 = the element, slot 1 = empty box
__global__ void k_bvh_single(const uint64_t *keys, BvhNode *nodes, int32_t *parents, int32_t *leafElem)
{
  const int e = (int)(keys[0] & 0xffffffffu);
  leafElem[0] = e;
  nodes[0].child[0] = ~e;
  nodes[0].child[1] = ~e;
  for (int a = 0; a < 3; ++a) { nodes[0].lo1[a] = INFINITY; nodes[0].hi1[a] = -INFINITY; }
  nodes[0].op[1] = 0.f;
  parents[0] = 0;  // leaf position 0 -> node 0 slot 0 (parents[(n-1)+0])
}

// bottom-up refit: each leaf writes its box and opacity into its parent's
// slot; the second thread to reach a node merges and moves up
__global__ void k_bvh_refit(const float4 *verts, const int32_t *indices, int n, BvhNode *nodes,
                            const int32_t *parents, const int32_t *leafElem, const float *elemOps, bool boxes,
                            unsigned *counters)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int e = leafElem[p];
  V3 lo = mk3(0.f, 0.f, 0.f), hi = lo;
  if (boxes) elem_box(verts, indices, (size_t)e, lo, hi);
  float op = elemOps ? elemOps[e] : 1.f;
  int par = parents[(n - 1) + p];
  // a Karras tree over unique 64-bit keys is at most 64 levels deep
  for (int depth = 0; depth < 128; ++depth) {
    const int node = par >> 1, slot = par & 1;
    volatile BvhNode *vn = nodes + node;
    if (boxes) {
      if (slot == 0) {
        vn->lo0[0] = lo.x; vn->lo0[1] = lo.y; vn->lo0[2] = lo.z;
        vn->hi0[0] = hi.x; vn->hi0[1] = hi.y; vn->hi0[2] = hi.z;
      } else {
        vn->lo1[0] = lo.x; vn->lo1[1] = lo.y; vn->lo1[2] = lo.z;
        vn->hi1[0] = hi.x; vn->hi1[1] = hi.y; vn->hi1[2] = hi.z;
      }
    }
    vn->op[slot] = op;
    __threadfence();
    if (atomicAdd(counters + node, 1u) == 0u) return;
    __threadfence();
    if (boxes) {
      lo = min3(mk3(vn->lo0[0], vn->lo0[1], vn->lo0[2]), mk3(vn->lo1[0], vn->lo1[1], vn->lo1[2]));
      hi = max3(mk3(vn->hi0[0], vn->hi0[1], vn->hi0[2]), mk3(vn->hi1[0], vn->hi1[1], vn->hi1[2]));
    }
    op = fmaxf(vn->op[0], vn->op[1]);
    if (node == 0) return;
    par = parents[node];
  }
}

// element occupancy bitmap: mark every cell an element's closed AABB
// touches (same monotonic cell mapping as the query)
__global__ void k_elem_occupancy(const float4 *verts, const int32_t *indices, size_t ne, ElemOccupancy O,
                                 uint32_t *bits)
{
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  V3 lo, hi;
  elem_box(verts, indices, e, lo, hi);
  const int x0 = imax_t(0, occ_coord(lo.x, O.origin[0], O.cellSize[0], O.n[0]));
  const int y0 = imax_t(0, occ_coord(lo.y, O.origin[1], O.cellSize[1], O.n[1]));
  const int z0 = imax_t(0, occ_coord(lo.z, O.origin[2], O.cellSize[2], O.n[2]));
  const int x1 = imin_t(O.n[0] - 1, occ_coord(hi.x, O.origin[0], O.cellSize[0], O.n[0]));
  const int y1 = imin_t(O.n[1] - 1, occ_coord(hi.y, O.origin[1], O.cellSize[1], O.n[1]));
  const int z1 = imin_t(O.n[2] - 1, occ_coord(hi.z, O.origin[2], O.cellSize[2], O.n[2]));
  for (int z = z0; z <= z1; ++z)
    for (int y = y0; y <= y1; ++y)
      for (int x = x0; x <= x1; ++x) {
        const size_t c = ((size_t)z * O.n[1] + y) * O.n[0] + x;
        atomicOr(bits + (c >> 5), 1u << (c & 31));
      }
}

void launchElemOccupancy(const float4 *verts, const int32_t *idx, size_t ne, const ElemOccupancy &O, uint32_t *bits,
                         size_t words, cudaStream_t s)
{
  cudaCheck(cudaMemsetAsync(bits, 0, words * sizeof(uint32_t), s), "memset occupancy");
  if (!ne) return;
  k_elem_occupancy<<<gridFor(ne, 256), 256, 0, s>>>(verts, idx, ne, O, bits);
  cudaCheck(cudaGetLastError(), "k_elem_occupancy");
}

void launchBuildBVH(const float4 *verts, const int32_t *idx, size_t ne, exa_box3f sb, BvhNode *nodes,
                    int32_t *parents, int32_t *leafElem, cudaStream_t s)
{
  if (!ne) return;
  if (ne >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "too many elements for the BVH");
  const int n = (int)ne;
  DBuf<uint64_t> keys, sorted;
  keys.alloc(ne);
  sorted.alloc(ne);
  k_bvh_keys<<<gridFor(ne, 256), 256, 0, s>>>(verts, idx, ne, sb, keys.ptr);
  cudaCheck(cudaGetLastError(), "k_bvh_keys");
  size_t tempBytes = 0;
  cudaCheck(cub::DeviceRadixSort::SortKeys(nullptr, tempBytes, keys.ptr, sorted.ptr, n, 0, 64, s), "sort size");
  DBuf<unsigned char> temp;
  temp.alloc(tempBytes ? tempBytes : 1);
  cudaCheck(cub::DeviceRadixSort::SortKeys(temp.ptr, tempBytes, keys.ptr, sorted.ptr, n, 0, 64, s), "sort");
  cudaCheck(cudaMemsetAsync(nodes, 0, sizeof(BvhNode) * (size_t)(n > 1 ? n - 1 : 1), s), "memset nodes");
  if (n == 1)
    k_bvh_single<<<1, 1, 0, s>>>(sorted.ptr, nodes, parents, leafElem);
  else
    k_bvh_karras<<<gridFor(ne, 256), 256, 0, s>>>(sorted.ptr, n, nodes, parents, leafElem);
  cudaCheck(cudaGetLastError(), "k_bvh_karras");
  launchRefitBVH(verts, idx, ne, nodes, parents, leafElem, nullptr, true, s);
  cudaCheck(cudaStreamSynchronize(s), "bvh build");
}

void launchRefitBVH(const float4 *verts, const int32_t *idx, size_t ne, BvhNode *nodes, const int32_t *parents,
                    const int32_t *leafElem, const float *elemOps, bool boxes, cudaStream_t s)
{
  if (!ne) return;
  const int n = (int)ne;
  DBuf<unsigned> counters;
  counters.alloc(n > 1 ? n - 1 : 1);
  cudaCheck(cudaMemsetAsync(counters.ptr, 0, counters.bytes(), s), "memset counters");
  k_bvh_refit<<<gridFor(ne, 256), 256, 0, s>>>(verts, idx, n, nodes, parents, leafElem, elemOps, boxes, counters.ptr);
  cudaCheck(cudaGetLastError(), "k_bvh_refit");
  cudaCheck(cudaStreamSynchronize(s), "bvh refit");
}

} // namespace exa
