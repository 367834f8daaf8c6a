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

// ------------------------------------------------------------------------
// Bulk copies into shared memory: cp.async.bulk (the TMA unit's untiled
// copy; both addresses and the size multiples of 16 bytes), completed on an
// mbarrier that the issuing thread arms with the expected byte count.
EXA_D uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

EXA_D void mbar_init(uint64_t *bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}

EXA_D void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// orders this thread's earlier generic-proxy accesses to shared memory (made
// visible to it by a block barrier) before its next bulk copy
EXA_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

EXA_D void bulk_load_smem(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

EXA_D bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// waits for the phase of the given parity to complete; false when it did
// not within the poll limit
constexpr int kMbarPollLimit = 1 << 24;
EXA_D bool mbar_wait(uint64_t *bar, uint32_t parity)
{
  for (int i = 0; i < kMbarPollLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ------------------------------------------------------------------------
// Grid.cu:134-246 fused with computeGridletValueRangesGPU
// (sampler/ExaStitchSampler.cu:52-142).
//
// Persistent blocks take gridlets in turn.  A gridlet's corner scalars (one
// contiguous brick of (dims+1)^3 floats, <= 729 for makeGrids' 8^3 cells)
// are staged in shared memory by one bulk copy, double-buffered so that the
// next gridlet's copy runs while this one is processed.  The copy starts at
// the 16-byte boundary at or below the brick and ends at the 16-byte
// boundary at or above it, clipped to the last boundary inside the scalar
// buffer; the at most 3 scalars past that clip are loaded by threads.
//
// A thread takes one x-row of cells and reuses each x-face of corners for
// the next cell.  The macrocell overlap test of Grid.cu:172-183 is an AND of
// per-axis interval tests, so a cell's macrocells are the product of three
// index ranges: the row's y and z ranges are computed once, the x range per
// cell, each from the candidates within one macrocell of the cell's own
// projection (the reference tests every macrocell of the gridlet's range;
// the exact test decides in both cases, so the same macrocells are
// updated).  Runs of cells with the same x range are merged first; the
// updates then go to a shared-memory copy of the gridlet's macrocell window
// and from there, one atomic min and max per touched macrocell, to the
// grid.  Windows larger than kMajWindow update the grid directly.  Min and
// max are exact, so none of this changes the result; merges and the window
// use the same total order (-0 below +0) as the atomics.
constexpr int kMajThreads = 64;
constexpr int kBrickCap = 736;    // floats per staging buffer: 729 scalars + alignment (multiple of 4)
constexpr int kMajWindow = 512;   // macrocells of a gridlet reduced in shared memory

constexpr int kAxisTab = 64;      // cells per axis whose macrocell ranges are tabled per gridlet

// the staging of one gridlet's scalars: copy [f0, f0 + bulk/4) in bulk and
// `tail` floats after it by threads; the brick starts `lead` floats in
struct BrickPlan {
  size_t f0;
  uint32_t bulk;
  int lead, tail;
  bool staged;
};

EXA_D BrickPlan brick_plan(const exa_gridlet &g, size_t nScalars, bool stage)
{
  BrickPlan p;
  const size_t n = (size_t)(g.dims.x + 1) * (g.dims.y + 1) * (g.dims.z + 1);
  const size_t s0 = (uint32_t)g.begin, s1 = s0 + n;
  p.f0 = s0 & ~(size_t)3;
  p.lead = (int)(s0 - p.f0);
  // s1 - f0 + 3 bounds the rounded-up copy
  p.staged = stage && s1 - p.f0 + 3 <= (size_t)kBrickCap;
  size_t f1 = (s1 + 3) & ~(size_t)3;
  const size_t fend = nScalars & ~(size_t)3;
  if (f1 > fend) f1 = fend > p.f0 ? fend : p.f0;
  p.bulk = p.staged ? (uint32_t)((f1 - p.f0) * 4) : 0u;
  p.tail = p.staged && s1 > f1 ? (int)(s1 - f1) : 0;
  return p;
}

// what the block needs to know of a gridlet before its cells: prepared by
// thread 0 when it issues the gridlet's copy, one gridlet ahead
struct GridletPlan {
  exa_gridlet g;
  BrickPlan P;
  V3i loMC, hiMC;   // the gridlet's macrocell range (projectOnGrid of its box)
};

struct alignas(16) MajSmem {
  float brick[2][kBrickCap];
  uint32_t winLo[kMajWindow], winHi[kMajWindow];  // ord_key of the window's ranges
  int2 axisRange[3][kAxisTab];    // per axis and cell index: its macrocell range [x, y]
  GridletPlan plan[2];            // of the gridlet in each staging buffer
  uint64_t bar[2];
  float redLo[kMajThreads / 32], redHi[kMajThreads / 32];
};

// projectOnGrid (Grid.cuh:55-63) along one axis
EXA_D int proj_axis(float v, float lo, float hi, int n)
{
  return iclamp((int)(((v - lo) / (hi - lo)) * (float)n), 0, n - 1);
}

// the macrocells [m0, m1] along one axis whose slab overlaps the closed
// interval [clo, chi]: the candidates within one of the interval's own
// projection and the gridlet's range, tested as Grid.cu:172-183 does
// (empty: m0 > m1)
EXA_D void mc_axis_range(float clo, float chi, float wlo, float whi, float size, int n, int loMC, int hiMC, int &m0,
                         int &m1)
{
  const int c0 = imax_t(loMC, proj_axis(clo, wlo, whi, n) - 1);
  const int c1 = imin_t(hiMC, proj_axis(chi, wlo, whi, n) + 1);
  m0 = 0;
  m1 = -1;
  for (int m = c0; m <= c1; ++m) {
    const float mlo = wlo + (float)m * size, mhi = wlo + (float)(m + 1) * size;
    if (mlo <= chi && clo <= mhi) {
      if (m1 < m0) m0 = m;
      m1 = m;
    }
  }
}

// keys in the order of atomic_min_float / atomic_max_float (-0 below +0),
// compared as unsigned integers; ord_value inverts ord_key
EXA_D uint32_t ord_key(float v)
{
  const uint32_t b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
EXA_D float ord_value(uint32_t k) { return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k); }

// thread 0: the plan of gridlet g and the bulk copy of its brick into
// buffer buf
EXA_D void prepare_gridlet(MajSmem &sm, int buf, const exa_gridlet &hdr, const float *scalars, size_t nScalars,
                           bool stage, const V3i D, const exa_box3f &wb)
{
  GridletPlan &pl = sm.plan[buf];
  pl.g = hdr;
  pl.P = brick_plan(pl.g, nScalars, stage);
  if (pl.P.bulk) bulk_load_smem(sm.brick[buf], scalars + pl.P.f0, pl.P.bulk, &sm.bar[buf]);
  const exa_gridlet &g = pl.g;
  const float cw = (float)(1 << g.level);
  const V3 lo = mk3(((float)g.lower.x + 0.5f) * cw, ((float)g.lower.y + 0.5f) * cw, ((float)g.lower.z + 0.5f) * cw);
  const V3 hi = mk3((((float)g.lower.x + (float)g.dims.x) + 0.5f) * cw,
                    (((float)g.lower.y + (float)g.dims.y) + 0.5f) * cw,
                    (((float)g.lower.z + (float)g.dims.z) + 0.5f) * cw);
  pl.loMC = project_on_grid(lo, D, wb);
  pl.hiMC = project_on_grid(hi, D, wb);
}

//
// list != null: the gridlets list[0 .. *listCount) instead of 0 .. ng (the
// gridlets the separable kernel below leaves to this one).
__global__ void __launch_bounds__(kMajThreads, 16) k_gridlet_majorants(const exa_gridlet *__restrict__ gridlets, size_t ng,
                                                                   const float *__restrict__ scalars, size_t nScalars,
                                                                   bool stage, exa_vec3i dims, exa_box3f wb,
                                                                   exa_range1f *mcRanges, exa_range1f *gridletRanges,
                                                                   uint32_t *errors, uint32_t debugFlags,
                                                                   const uint32_t *__restrict__ list,
                                                                   const unsigned *__restrict__ listCount)
{
  __shared__ MajSmem sm;
  const int tid = threadIdx.x;
  const V3i D = {dims.x, dims.y, dims.z};
  if (list) ng = *listCount;
  auto idOf = [&](size_t i) -> size_t { return list ? (size_t)list[i] : i; };
  // thread 0 holds the header of the gridlet after the next one, loaded an
  // iteration before it is planned
  exa_gridlet ahead{};
  if (tid == 0) {
    mbar_init(&sm.bar[0]);
    mbar_init(&sm.bar[1]);
    mbar_init_fence();
    if (blockIdx.x < ng) prepare_gridlet(sm, 0, gridlets[idOf(blockIdx.x)], scalars, nScalars, stage, D, wb);
    if (blockIdx.x + gridDim.x < ng) ahead = gridlets[idOf(blockIdx.x + gridDim.x)];
  }
  __syncthreads();
  const V3 mcSize = div3(sub3(mk3(wb.upper), mk3(wb.lower)), mk3((float)dims.x, (float)dims.y, (float)dims.z));
  uint32_t parity = 0;  // bit b: parity of the next phase of buffer b
  int it = 0;
  for (size_t gi = blockIdx.x; gi < ng; gi += gridDim.x, ++it) {
    const int buf = it & 1;
    const exa_gridlet g = sm.plan[buf].g;
    const BrickPlan P = sm.plan[buf].P;
    const V3i loMC = sm.plan[buf].loMC, hiMC = sm.plan[buf].hiMC;
    const size_t gn = gi + gridDim.x;
    if (tid == 0 && gn < ng) {
      fence_proxy_async_smem();
      prepare_gridlet(sm, buf ^ 1, ahead, scalars, nScalars, stage, D, wb);
      if (gn + gridDim.x < ng) ahead = gridlets[idOf(gn + gridDim.x)];
    }
    const float *S = scalars + (uint32_t)g.begin;
    if (P.staged) {
      bool ok = true;
      const uint32_t ph = (parity >> buf) & 1u;
      if (P.bulk) {
        ok = mbar_wait(&sm.bar[buf], ph);
        // the simulated time-out of the error-path test: block 0 treats its
        // first wait as failed after it completed, so no copy is in flight
        if ((debugFlags & EXA_DEBUG_COPY_WAIT_TIMEOUT) && blockIdx.x == 0 && it == 0) ok = false;
        parity ^= 1u << buf;
      }
      if (__syncthreads_or(!ok)) {
        // give up: flag it and wait (bounded again) for this buffer's copy
        // and the other buffer's before the block's shared memory is
        // released.  A copy that never completes is still in flight when
        // the block exits; the host reports the build as failed.
        if (tid == 0) {
          if (errors) atomicOr(errors, EXA_DEVERR_COPY_WAIT);
          if (P.bulk) (void)mbar_wait(&sm.bar[buf], ph);
          if (gn < ng && sm.plan[buf ^ 1].P.bulk)
            (void)mbar_wait(&sm.bar[buf ^ 1], (parity >> (buf ^ 1)) & 1u);
        }
        return;
      }
      float *B = sm.brick[buf];
      for (int k = tid; k < P.tail; k += blockDim.x) B[P.bulk / 4 + k] = __ldg(scalars + P.f0 + P.bulk / 4 + k);
      S = B + P.lead;
    }
    const float cw = (float)(1 << g.level);
    const int wx = hiMC.x - loMC.x + 1, wy = hiMC.y - loMC.y + 1, wz = hiMC.z - loMC.z + 1;
    const int wn = wx * wy * wz;
    const bool useWin = wn <= kMajWindow;
    if (useWin)
      for (int k = tid; k < wn; k += blockDim.x) {
        sm.winLo[k] = 0xffffffffu;  // untouched: lower key above upper key
        sm.winHi[k] = 0u;
      }
    const float hc = 0.5f * cw;
    // a cell's macrocell range along an axis depends only on its index
    // along that axis: table them once per gridlet
    const bool tabled = g.dims.x <= kAxisTab && g.dims.y <= kAxisTab && g.dims.z <= kAxisTab;
    auto axis_range = [&](int a, int i, int &m0, int &m1) {
      const int lower = a == 0 ? g.lower.x : a == 1 ? g.lower.y : g.lower.z;
      const float wlo = a == 0 ? wb.lower.x : a == 1 ? wb.lower.y : wb.lower.z;
      const float whi = a == 0 ? wb.upper.x : a == 1 ? wb.upper.y : wb.upper.z;
      const float size = a == 0 ? mcSize.x : a == 1 ? mcSize.y : mcSize.z;
      const int n = a == 0 ? dims.x : a == 1 ? dims.y : dims.z;
      const int lo = a == 0 ? loMC.x : a == 1 ? loMC.y : loMC.z;
      const int hi = a == 0 ? hiMC.x : a == 1 ? hiMC.y : hiMC.z;
      mc_axis_range((float)(lower + i) * cw + hc, (float)(lower + i + 1) * cw + hc, wlo, whi, size, n, lo, hi, m0,
                    m1);
    };
    if (tabled)
      for (int k = tid; k < g.dims.x + g.dims.y + g.dims.z; k += blockDim.x) {
        const int a = k < g.dims.x ? 0 : k < g.dims.x + g.dims.y ? 1 : 2;
        const int i = a == 0 ? k : a == 1 ? k - g.dims.x : k - g.dims.x - g.dims.y;
        int m0, m1;
        axis_range(a, i, m0, m1);
        sm.axisRange[a][i] = make_int2(m0, m1);
      }
    __syncthreads();
    const int nx = g.dims.x + 1, ny = g.dims.y + 1;
    float glo = 1e30f, ghi = -1e30f;
    for (int r = tid; r < g.dims.y * g.dims.z; r += blockDim.x) {
      const int y = r % g.dims.y, z = r / g.dims.y;
      int my0, my1, mz0, mz1;
      if (tabled) {
        const int2 ry = sm.axisRange[1][y], rz = sm.axisRange[2][z];
        my0 = ry.x; my1 = ry.y; mz0 = rz.x; mz1 = rz.y;
      } else {
        axis_range(1, y, my0, my1);
        axis_range(2, z, mz0, mz1);
      }
      const bool rowHits = my0 <= my1 && mz0 <= mz1;
      const float *R0 = S + (z * ny + y) * nx, *R1 = R0 + nx, *R2 = R0 + nx * ny, *R3 = R2 + nx;
      float a0 = R0[0], a1 = R1[0], a2 = R2[0], a3 = R3[0];
      int rx0 = 0, rx1 = -1;
      uint32_t rlo = 0xffffffffu, rhi = 0u;  // the run's range as ord_key
      auto flush = [&]() {
        if (rx1 < rx0) return;
        for (int mz = mz0; mz <= mz1; ++mz)
          for (int my = my0; my <= my1; ++my)
            for (int mx = rx0; mx <= rx1; ++mx) {
              if (useWin) {
                const int k = ((mz - loMC.z) * wy + (my - loMC.y)) * wx + (mx - loMC.x);
                atomicMin(&sm.winLo[k], rlo);
                atomicMax(&sm.winHi[k], rhi);
              } else {
                update_mc(mcRanges, dims, mx, my, mz, ord_value(rlo), ord_value(rhi));
              }
            }
      };
      for (int x = 0; x < g.dims.x; ++x) {
        const float b0 = R0[x + 1], b1 = R1[x + 1], b2 = R2[x + 1], b3 = R3[x + 1];
        const float f[8] = {a0, b0, a1, b1, a2, b2, a3, b3};
        a0 = b0; a1 = b1; a2 = b2; a3 = b3;
        // fminf / fmaxf return the other operand where one is NaN, so NaN
        // corners drop out as the reference's isnan tests drop them
        float lo = 1e30f, hi = -1e30f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          lo = fminf(lo, f[k]);
          hi = fmaxf(hi, f[k]);
        }
        glo = fminf(glo, lo);
        ghi = fmaxf(ghi, hi);
        if (hi < lo || !rowHits) continue;  // no non-NaN corner: the reference's update is a no-op
        int mx0, mx1;
        if (tabled) {
          const int2 rx = sm.axisRange[0][x];
          mx0 = rx.x; mx1 = rx.y;
        } else {
          axis_range(0, x, mx0, mx1);
        }
        if (mx1 < mx0) continue;
        if (mx0 == rx0 && mx1 == rx1) {
          rlo = min(rlo, ord_key(lo));
          rhi = max(rhi, ord_key(hi));
        } else {
          flush();
          rx0 = mx0;
          rx1 = mx1;
          rlo = ord_key(lo);
          rhi = ord_key(hi);
        }
      }
      flush();
    }
    // the gridlet's own range
    for (int o = 16; o > 0; o >>= 1) {
      glo = fminf(glo, __shfl_xor_sync(0xffffffffu, glo, o));
      ghi = fmaxf(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    }
    if ((tid & 31) == 0) {
      sm.redLo[tid >> 5] = glo;
      sm.redHi[tid >> 5] = ghi;
    }
    __syncthreads();
    if (useWin)
      for (int k = tid; k < wn; k += blockDim.x) {
        const uint32_t lo = sm.winLo[k], hi = sm.winHi[k];
        if (lo > hi) continue;  // untouched
        const int mx = loMC.x + k % wx, my = loMC.y + (k / wx) % wy, mz = loMC.z + k / (wx * wy);
        update_mc(mcRanges, dims, mx, my, mz, ord_value(lo), ord_value(hi));
      }
    if (tid == 0) {
      for (int w = 1; w < kMajThreads / 32; ++w) {
        glo = fminf(glo, sm.redLo[w]);
        ghi = fmaxf(ghi, sm.redHi[w]);
      }
      gridletRanges[idOf(gi)].lower = glo;
      gridletRanges[idOf(gi)].upper = ghi;
    }
    // buffer, window and reduction slots are free for the next gridlet
    __syncthreads();
  }
}

// ------------------------------------------------------------------------
// The same build, separable: one warp per gridlet, no per-cell loop.
//
// The macrocells a cell updates are a product of per-axis index ranges (the
// AND of per-axis interval tests of Grid.cu:172-183, as above), and a cell
// with a non-NaN corner updates each of them with the min / max over its
// non-NaN corners (and the +-1e30 of the empty range).  So a corner with a
// non-NaN value reaches exactly the macrocells in the product over the axes
// of U_a(j) = the union of the ranges of the (one or two) cells that have
// corner index j along axis a: every combination of those cells is a cell
// holding the corner.  A macrocell's update is then the min / max over the
// corners whose three unions contain it, which is reduced one axis at a
// time: along x for every corner row and macrocell column (the corners of a
// column are an interval [ca, cb] of the row), then along y for every
// macrocell column and row and corner plane, then along z; one atomic min /
// max per touched macrocell.  Min and max are exact, so the result is the
// per-cell loop's.  The gridlet's own range (every scalar) is the min / max
// of the x step's results when every corner along x lies in some column.
//
// A gridlet takes this path when its brick is staged (<= kBrickCap floats,
// so <= 8 cells per axis), its macrocell window is at most kSepWin wide on
// every axis and every macrocell's corner set is an interval; the others are
// appended to a list for k_gridlet_majorants.  Where the y step's results do
// not fit beside the x step's (the widest windows), the y and z steps run as
// one, over each window macrocell's rectangle of corner rows.
constexpr int kSepWarps = 4;      // warps (independent gridlet pipelines) per block
constexpr int kSepWin = 9;        // macrocells per axis of a gridlet's window
constexpr int kSepPool = 729;     // (min, max) entries of the x and y steps

struct alignas(16) SepWarpSmem {
  float brick[kBrickCap];
  float2 pool[kSepPool];          // x step: (column, corner row); then y step: (column, row, corner plane)
  int2 cellRange[3][8];           // per axis and cell index: its macrocell range
  int2 cornerIv[3][kSepWin];      // per axis and window macrocell: corners [ca, cb]
  GridletPlan plan;               // of the gridlet whose brick is staged
  uint64_t bar;
};

// k / d for 0 <= k < 2048 and k * d < 2^21 (every index decoded below:
// k < 729, d <= 81) as a multiply and a shift: with inv = 2^21 / d + 1 the
// product k * inv / 2^21 exceeds k / d by less than k / 2^21 < 1 / d, which
// cannot reach the next integer, and k * inv stays below 2^32
struct SepDiv {
  uint32_t inv;
  EXA_D explicit SepDiv(int d) : inv((1u << 21) / (uint32_t)d + 1u) {}
  EXA_D int operator()(int k) const { return (int)(((uint32_t)k * inv) >> 21); }
};

// One staging buffer per warp: the next gridlet's brick is copied in as soon
// as the current one's corners are reduced along x, so the copy runs during
// the current gridlet's macrocell updates (and, at 9.3 KB of shared memory
// per warp, 24 warps per SM hide what it does not cover).
__global__ void __launch_bounds__(kSepWarps * 32) k_gridlet_majorants_sep(
    const exa_gridlet *__restrict__ gridlets, size_t ng, const float *__restrict__ scalars, size_t nScalars,
    bool stage, exa_vec3i dims, exa_box3f wb, exa_range1f *mcRanges, exa_range1f *gridletRanges, uint32_t *errors,
    uint32_t debugFlags, uint32_t *fallback, unsigned *fallbackCount)
{
  extern __shared__ __align__(16) unsigned char sepSm[];
  SepWarpSmem &sm = reinterpret_cast<SepWarpSmem *>(sepSm)[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31;
  const size_t w0 = (size_t)blockIdx.x * kSepWarps + (threadIdx.x >> 5);
  const size_t stride = (size_t)gridDim.x * kSepWarps;
  // the warp stages a gridlet (every lane calls this, with the same header;
  // the buffer's readers are done: a __syncwarp precedes every call): lane 0
  // plans the brick and issues its bulk copy, lanes 1..6 project the
  // gridlet's box on the grid, one bound of one axis each (projectOnGrid)
  auto prepare = [&](const exa_gridlet &hdr) {
    GridletPlan &pl = sm.plan;
    if (lane == 0) {
      pl.g = hdr;
      pl.P = brick_plan(hdr, nScalars, stage);
      if (pl.P.bulk) {
        fence_proxy_async_smem();
        bulk_load_smem(sm.brick, scalars + pl.P.f0, pl.P.bulk, &sm.bar);
      }
    } else if (lane <= 6) {
      const int a = (int)(lane - 1) % 3;
      const bool upper = lane > 3;
      const int lower = a == 0 ? hdr.lower.x : a == 1 ? hdr.lower.y : hdr.lower.z;
      const int cells = a == 0 ? hdr.dims.x : a == 1 ? hdr.dims.y : hdr.dims.z;
      const float cw = (float)(1 << hdr.level);
      const float v = upper ? (((float)lower + (float)cells) + 0.5f) * cw : ((float)lower + 0.5f) * cw;
      const float wlo = a == 0 ? wb.lower.x : a == 1 ? wb.lower.y : wb.lower.z;
      const float whi = a == 0 ? wb.upper.x : a == 1 ? wb.upper.y : wb.upper.z;
      const int n = a == 0 ? dims.x : a == 1 ? dims.y : dims.z;
      // project_on_grid, one component
      const int m = iclamp((int)(((v - wlo) / (whi - wlo)) * (float)n), 0, n - 1);
      V3i &dst = upper ? pl.hiMC : pl.loMC;
      if (a == 0) dst.x = m;
      else if (a == 1) dst.y = m;
      else dst.z = m;
    }
  };
  if (lane == 0) {
    mbar_init(&sm.bar);
    mbar_init_fence();
  }
  __syncwarp();
  if (w0 < ng) prepare(gridlets[w0]);
  __syncwarp();
  const V3 mcSize = div3(sub3(mk3(wb.upper), mk3(wb.lower)), mk3((float)dims.x, (float)dims.y, (float)dims.z));
  uint32_t parity = 0;
  for (size_t gi = w0; gi < ng; gi += stride) {
    const exa_gridlet g = sm.plan.g;
    const BrickPlan P = sm.plan.P;
    const V3i loMC = sm.plan.loMC, hiMC = sm.plan.hiMC;
    const size_t gn = gi + stride;
    // the next gridlet's header is loaded now and planned after this one's
    // x step, when the load has long arrived
    exa_gridlet next{};
    if (gn < ng) next = gridlets[gn];
    bool ok = true;
    if (P.bulk) {
      ok = mbar_wait(&sm.bar, parity);
      // the simulated time-out of the error-path test (see k_gridlet_majorants)
      if ((debugFlags & EXA_DEBUG_COPY_WAIT_TIMEOUT) && gi == 0) ok = false;
    }
    if (__any_sync(0xffffffffu, !ok)) {
      // give up: flag it and wait (bounded) once more for the copy
      if (lane == 0) {
        if (errors) atomicOr(errors, EXA_DEVERR_COPY_WAIT);
        (void)mbar_wait(&sm.bar, parity);
      }
      return;
    }
    if (P.bulk) parity ^= 1u;
    const int wx = hiMC.x - loMC.x + 1, wy = hiMC.y - loMC.y + 1, wz = hiMC.z - loMC.z + 1;
    bool sep = P.staged && g.dims.x <= 8 && g.dims.y <= 8 && g.dims.z <= 8 && wx <= kSepWin && wy <= kSepWin &&
               wz <= kSepWin;
    const int nx = g.dims.x + 1, ny = g.dims.y + 1, nz = g.dims.z + 1;
    const int rows = ny * nz;
    // the x step's results and, when they fit beside them, the y step's
    // (else the y and z steps run as one, over the rectangle of rows)
    sep = sep && wx * rows <= kSepPool;
    const bool yStep = wx * rows + wx * wy * nz <= kSepPool;
    float *B = sm.brick;
    bool fold = false;
    if (sep) {
      for (int k = lane; k < P.tail; k += 32) B[P.bulk / 4 + k] = __ldg(scalars + P.f0 + P.bulk / 4 + k);
      // each cell's macrocell range along each axis
      const float cw = (float)(1 << g.level), hc = 0.5f * cw;
      bool xEmpty = false;
      if (lane < g.dims.x + g.dims.y + g.dims.z) {
        const int a = (int)lane < g.dims.x ? 0 : (int)lane < g.dims.x + g.dims.y ? 1 : 2;
        const int i = a == 0 ? lane : a == 1 ? lane - g.dims.x : lane - g.dims.x - g.dims.y;
        const int lower = a == 0 ? g.lower.x : a == 1 ? g.lower.y : g.lower.z;
        const float wlo = a == 0 ? wb.lower.x : a == 1 ? wb.lower.y : wb.lower.z;
        const float whi = a == 0 ? wb.upper.x : a == 1 ? wb.upper.y : wb.upper.z;
        const float size = a == 0 ? mcSize.x : a == 1 ? mcSize.y : mcSize.z;
        const int n = a == 0 ? dims.x : a == 1 ? dims.y : dims.z;
        const int lo = a == 0 ? loMC.x : a == 1 ? loMC.y : loMC.z;
        const int hi = a == 0 ? hiMC.x : a == 1 ? hiMC.y : hiMC.z;
        int m0, m1;
        mc_axis_range((float)(lower + i) * cw + hc, (float)(lower + i + 1) * cw + hc, wlo, whi, size, n, lo, hi, m0,
                      m1);
        sm.cellRange[a][i] = make_int2(m0, m1);
        xEmpty = a == 0 && m1 < m0;
      }
      // every corner along x is in some column's interval when every cell
      // along x reaches a macrocell
      fold = !__any_sync(0xffffffffu, xEmpty) && g.dims.x > 0 && g.dims.y > 0 && g.dims.z > 0;
      __syncwarp();
      // per axis and window macrocell: the corners whose cells reach it, an
      // interval [ca, cb] (empty: ca > cb); a gap sends the gridlet to the
      // general kernel.  Nine lanes per window macrocell, one corner index
      // each; the ballot gives the macrocell's corner set.
      bool gap = false;
      const int nMC = wx + wy + wz;
      const int q = (int)lane / 9, j = (int)lane - 9 * q;
      for (int t0 = 0; t0 < nMC; t0 += 3) {
        const int t = t0 + q;
        const bool mine = q < 3 && t < nMC;
        int a = 0, off = 0, d = 0;
        bool in = false;
        if (mine) {
          a = t < wx ? 0 : t < wx + wy ? 1 : 2;
          off = a == 0 ? t : a == 1 ? t - wx : t - wx - wy;
          const int m = off + (a == 0 ? loMC.x : a == 1 ? loMC.y : loMC.z);
          d = a == 0 ? g.dims.x : a == 1 ? g.dims.y : g.dims.z;
          if (j <= d) {
            if (j > 0) { const int2 r = sm.cellRange[a][j - 1]; in = in || (r.x <= m && m <= r.y); }
            if (j < d) { const int2 r = sm.cellRange[a][j]; in = in || (r.x <= m && m <= r.y); }
          }
        }
        const unsigned bits = (__ballot_sync(0xffffffffu, in) >> (9 * (q < 3 ? q : 0))) & 0x1ffu;
        if (mine && j == 0) {
          if (bits) {
            const int ca = __ffs(bits) - 1, cb = 31 - __clz(bits);
            gap = gap || bits != (((2u << cb) - 1u) & ~((1u << ca) - 1u));
            sm.cornerIv[a][off] = make_int2(ca, cb);
          } else {
            sm.cornerIv[a][off] = make_int2(1 << 20, -1);
          }
        }
      }
      sep = !__any_sync(0xffffffffu, gap);
      __syncwarp();
    }
    if (!sep) {
      if (lane == 0) fallback[atomicAdd(fallbackCount, 1u)] = (uint32_t)gi;
      __syncwarp();
      if (gn < ng) prepare(next);
      __syncwarp();
      continue;
    }
    // the gridlet's own range: over every scalar (cell-less gridlets: empty)
    float glo = 1e30f, ghi = -1e30f;
    if (!fold && g.dims.x > 0 && g.dims.y > 0 && g.dims.z > 0)
      for (int k = lane; k < nx * rows; k += 32) {
        const float v = B[P.lead + k];
        glo = fminf(glo, v);
        ghi = fmaxf(ghi, v);
      }
    // along x: every (macrocell column, corner row), a lane per row
    float2 *X = sm.pool;
    for (int r = lane; r < rows; r += 32) {
      const float *R = B + P.lead + r * nx;
      for (int m = 0; m < wx; ++m) {
        const int2 iv = sm.cornerIv[0][m];
        float lo = 1e30f, hi = -1e30f;
        for (int c = iv.x; c <= iv.y; ++c) {
          const float v = R[c];
          lo = fminf(lo, v);
          hi = fmaxf(hi, v);
        }
        X[m * rows + r] = make_float2(lo, hi);
        if (fold) {
          glo = fminf(glo, lo);
          ghi = fmaxf(ghi, hi);
        }
      }
    }
    // the brick is read: the next gridlet's copy runs from here on
    __syncwarp();
    if (gn < ng) prepare(next);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      glo = fminf(glo, __shfl_xor_sync(0xffffffffu, glo, o));
      ghi = fmaxf(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    }
    if (lane == 0) {
      gridletRanges[gi].lower = glo;
      gridletRanges[gi].upper = ghi;
    }
    const SepDiv byX(wx), byXY(wx * wy);
    if (yStep) {
      // along y: every (macrocell column, macrocell row, corner plane), a
      // lane per (column, plane)
      float2 *Y = sm.pool + wx * rows;
      const SepDiv byZ(nz);
      for (int k = lane; k < wx * nz; k += 32) {
        const int mx = byZ(k), cz = k - mx * nz;
        const float2 *S = X + mx * rows + cz * ny;
        for (int my = 0; my < wy; ++my) {
          const int2 iy = sm.cornerIv[1][my];
          float lo = 1e30f, hi = -1e30f;
          for (int cy = iy.x; cy <= iy.y; ++cy) {
            const float2 v = S[cy];
            lo = fminf(lo, v.x);
            hi = fmaxf(hi, v.y);
          }
          Y[(mx * wy + my) * nz + cz] = make_float2(lo, hi);
        }
      }
      __syncwarp();
      // along z: every window macrocell
      for (int k = lane; k < wx * wy * wz; k += 32) {
        const int mz = byXY(k), kxy = k - mz * wx * wy;
        const int my = byX(kxy), mx = kxy - my * wx;
        const int2 iz = sm.cornerIv[2][mz];
        const float2 *S = Y + (mx * wy + my) * nz;
        float lo = 1e30f, hi = -1e30f;
        for (int cz = iz.x; cz <= iz.y; ++cz) {
          const float2 v = S[cz];
          lo = fminf(lo, v.x);
          hi = fmaxf(hi, v.y);
        }
        if (lo <= hi) update_mc(mcRanges, dims, loMC.x + mx, loMC.y + my, loMC.z + mz, lo, hi);
      }
    } else {
      // wide windows: per window macrocell over its y x z rectangle of rows
      for (int k = lane; k < wx * wy * wz; k += 32) {
        const int mz = byXY(k), kxy = k - mz * wx * wy;
        const int my = byX(kxy), mx = kxy - my * wx;
        const int2 iy = sm.cornerIv[1][my], iz = sm.cornerIv[2][mz];
        const float2 *S = X + mx * rows;
        float lo = 1e30f, hi = -1e30f;
        for (int cz = iz.x; cz <= iz.y; ++cz)
          for (int cy = iy.x; cy <= iy.y; ++cy) {
            const float2 v = S[cz * ny + cy];
            lo = fminf(lo, v.x);
            hi = fmaxf(hi, v.y);
          }
        if (lo <= hi) update_mc(mcRanges, dims, loMC.x + mx, loMC.y + my, loMC.z + mz, lo, hi);
      }
    }
    // the tables and the plan are free for the next gridlet
    __syncwarp();
  }
}

unsigned launchGridletMajorants(const exa_gridlet *g, const float *scalars, size_t ng, size_t nScalars,
                                exa_vec3i dims, exa_box3f wb, exa_range1f *mcRanges, exa_range1f *gridletRanges,
                                uint32_t *errors, uint32_t debugFlags, uint32_t *scratch, cudaStream_t s)
{
  if (!ng) return 0;
  int dev = 0, sms = 0;
  cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  const bool stage = (reinterpret_cast<uintptr_t>(scalars) & 15u) == 0;
  // scratch: [0] the count of gridlets left to the general kernel, then
  // their indices
  unsigned *count = scratch;
  uint32_t *list = scratch + 1;
  cudaCheck(cudaMemsetAsync(count, 0, sizeof(unsigned), s), "memset fallback count");
  const size_t sepSmem = kSepWarps * sizeof(SepWarpSmem);
  cudaCheck(cudaFuncSetAttribute(k_gridlet_majorants_sep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sepSmem),
            "separable majorant kernel shared memory");
  int sepPerSM = 0;
  cudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sepPerSM, k_gridlet_majorants_sep, kSepWarps * 32,
                                                          sepSmem),
            "occupancy");
  const size_t sepBlocks = std::min<size_t>((ng + kSepWarps - 1) / kSepWarps,
                                            (size_t)std::max(sms, 1) * (size_t)std::max(sepPerSM, 1));
  k_gridlet_majorants_sep<<<(unsigned)sepBlocks, kSepWarps * 32, sepSmem, s>>>(
      g, ng, scalars, nScalars, stage, dims, wb, mcRanges, gridletRanges, errors, debugFlags, list, count);
  cudaCheck(cudaGetLastError(), "k_gridlet_majorants_sep");
  // the general kernel over the list (its blocks read the count)
  int perSM = 0;
  cudaCheck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_gridlet_majorants, kMajThreads, 0),
            "occupancy");
  const size_t blocks = std::min<size_t>(ng, (size_t)std::max(sms, 1) * (size_t)std::max(perSM, 1));
  k_gridlet_majorants<<<(unsigned)blocks, kMajThreads, 0, s>>>(g, ng, scalars, nScalars, stage, dims, wb, mcRanges,
                                                               gridletRanges, errors, 0u, list, count);
  cudaCheck(cudaGetLastError(), "k_gridlet_majorants");
  return (unsigned)std::min<size_t>(sepBlocks * kSepWarps, ng);
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
                              int ncolors, exa_range1f xf, int filter, float *out)
{
  extern __shared__ float4 sCmap[];
  for (int i = threadIdx.x; i < ncolors; i += blockDim.x) sCmap[i] = cmap[i];
  __syncthreads();
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = range_max_opacity(ranges[i], sCmap, ncolors, xf, filter);
}

__global__ void k_max_opacity_global(const exa_range1f *__restrict__ ranges, size_t n,
                                     const float4 *__restrict__ cmap, int ncolors, exa_range1f xf, int filter,
                                     float *out)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = range_max_opacity(ranges[i], cmap, ncolors, xf, filter);
}

void launchMaxOpacity(const exa_range1f *ranges, size_t n, const float4 *cmap, int ncolors, exa_range1f xf,
                      int filter, float *out, cudaStream_t s)
{
  if (!n) return;
  const size_t smem = (size_t)ncolors * sizeof(float4);
  if (smem <= 48 * 1024)
    k_max_opacity<<<gridFor(n, 256), 256, smem, s>>>(ranges, n, cmap, ncolors, xf, filter, out);
  else
    k_max_opacity_global<<<gridFor(n, 256), 256, 0, s>>>(ranges, n, cmap, ncolors, xf, filter, out);
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

// bottom-up refit: each leaf writes its box into its parent's slot; the
// second thread to reach a node merges and moves up (child opacities are
// left at 1: no query of these trees culls)
__global__ void k_bvh_refit(const float4 *verts, const int32_t *indices, int n, BvhNode *nodes,
                            const int32_t *parents, const int32_t *leafElem, unsigned *counters)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int e = leafElem[p];
  V3 lo, hi;
  elem_box(verts, indices, (size_t)e, lo, hi);
  int par = parents[(n - 1) + p];
  // a Karras tree over unique 64-bit keys is at most 64 levels deep
  for (int depth = 0; depth < 128; ++depth) {
    const int node = par >> 1, slot = par & 1;
    volatile BvhNode *vn = nodes + node;
    if (slot == 0) {
      vn->lo0[0] = lo.x; vn->lo0[1] = lo.y; vn->lo0[2] = lo.z;
      vn->hi0[0] = hi.x; vn->hi0[1] = hi.y; vn->hi0[2] = hi.z;
    } else {
      vn->lo1[0] = lo.x; vn->lo1[1] = lo.y; vn->lo1[2] = lo.z;
      vn->hi1[0] = hi.x; vn->hi1[1] = hi.y; vn->hi1[2] = hi.z;
    }
    vn->op[slot] = 1.f;
    __threadfence();
    if (atomicAdd(counters + node, 1u) == 0u) return;
    __threadfence();
    lo = min3(mk3(vn->lo0[0], vn->lo0[1], vn->lo0[2]), mk3(vn->lo1[0], vn->lo1[1], vn->lo1[2]));
    hi = max3(mk3(vn->hi0[0], vn->hi0[1], vn->hi0[2]), mk3(vn->hi1[0], vn->hi1[1], vn->hi1[2]));
    if (node == 0) return;
    par = parents[node];
  }
}

// ------------------------------------------------------------ element cells
// the cells an element's closed AABB touches, by the query's monotonic cell
// mapping (occ_coord), clamped to the grid
EXA_D void elem_cell_range(const ElemOccupancy &O, V3 lo, V3 hi, int &x0, int &y0, int &z0, int &x1, int &y1, int &z1)
{
  x0 = imax_t(0, occ_coord(lo.x, O.origin[0], O.invCell[0], O.n[0]));
  y0 = imax_t(0, occ_coord(lo.y, O.origin[1], O.invCell[1], O.n[1]));
  z0 = imax_t(0, occ_coord(lo.z, O.origin[2], O.invCell[2], O.n[2]));
  x1 = imin_t(O.n[0] - 1, occ_coord(hi.x, O.origin[0], O.invCell[0], O.n[0]));
  y1 = imin_t(O.n[1] - 1, occ_coord(hi.y, O.origin[1], O.invCell[1], O.n[1]));
  z1 = imin_t(O.n[2] - 1, occ_coord(hi.z, O.origin[2], O.invCell[2], O.n[2]));
}

// pass 1: each element's AABB, and the bit of every cell it touches
__global__ void k_elem_cells_mark(const float4 *verts, const int32_t *indices, size_t ne, ElemOccupancy O,
                                  uint32_t *bits, float4 *boxes)
{
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  V3 lo, hi;
  elem_box(verts, indices, e, lo, hi);
  boxes[2 * e] = make_float4(lo.x, lo.y, lo.z, hi.x);
  boxes[2 * e + 1] = make_float4(hi.y, hi.z, 0.f, 0.f);
  int x0, y0, z0, x1, y1, z1;
  elem_cell_range(O, lo, hi, x0, y0, z0, x1, y1, z1);
  for (int z = z0; z <= z1; ++z)
    for (int y = y0; y <= y1; ++y)
      for (int x = x0; x <= x1; ++x) {
        const size_t c = ((size_t)z * O.n[1] + y) * O.n[0] + x;
        atomicOr(bits + (c >> 5), 1u << (c & 31));
      }
}

__global__ void k_popc_words(const uint32_t *bits, size_t words, uint32_t *out)
{
  const size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (w < words) out[w] = (uint32_t)__popc(bits[w]);
}

EXA_D uint32_t marked_index(const ElemOccupancy &O, const uint32_t *bits, const uint32_t *rank, size_t c)
{
  const uint32_t bit = 1u << (c & 31);
  return rank[c >> 5] + (uint32_t)__popc(bits[c >> 5] & (bit - 1u));
}

// pass 2 (fill == false): elements per marked cell; pass 3 (fill): the
// lists, a cell with one element holds it in its entry
__global__ void k_elem_cells_lists(size_t ne, ElemOccupancy O, const uint32_t *bits, const uint32_t *rank,
                                   const float4 *boxes, uint32_t *count, const uint32_t *off, uint32_t *cursor,
                                   int32_t *entries, int32_t *items, bool fill)
{
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const float4 b0 = boxes[2 * e], b1 = boxes[2 * e + 1];
  int x0, y0, z0, x1, y1, z1;
  elem_cell_range(O, mk3(b0.x, b0.y, b0.z), mk3(b0.w, b1.x, b1.y), x0, y0, z0, x1, y1, z1);
  for (int z = z0; z <= z1; ++z)
    for (int y = y0; y <= y1; ++y)
      for (int x = x0; x <= x1; ++x) {
        const uint32_t m = marked_index(O, bits, rank, ((size_t)z * O.n[1] + y) * O.n[0] + x);
        if (!fill) {
          atomicAdd(count + m, 1u);
        } else if (count[m] == 1u) {
          entries[m] = (int32_t)e;
        } else {
          items[off[m] + 1u + atomicAdd(cursor + m, 1u)] = (int32_t)e;
        }
      }
}

// list lengths: count + 1 words for a cell with two or more elements
__global__ void k_elem_cells_seg(const uint32_t *count, size_t nm, uint32_t *seg)
{
  const size_t m = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (m < nm) seg[m] = count[m] >= 2u ? count[m] + 1u : 0u;
}

__global__ void k_elem_cells_heads(const uint32_t *count, const uint32_t *off, size_t nm, int32_t *entries,
                                   int32_t *items)
{
  const size_t m = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (m >= nm) return;
  if (count[m] >= 2u) {
    entries[m] = -(int32_t)off[m] - 2;
    items[off[m]] = (int32_t)count[m];
  } else {
    entries[m] = -1;
  }
}

// each list in ascending order (insertion sort: lists are short)
__global__ void k_elem_cells_sort(const uint32_t *count, const uint32_t *off, size_t nm, int32_t *items)
{
  const size_t m = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (m >= nm || count[m] < 2u) return;
  int32_t *L = items + off[m] + 1;
  const int n = (int)count[m];
  for (int i = 1; i < n; ++i) {
    const int32_t v = L[i];
    int j = i - 1;
    while (j >= 0 && L[j] > v) {
      L[j + 1] = L[j];
      --j;
    }
    L[j + 1] = v;
  }
}

// exclusive prefix sum of n words into out; returns the total
static uint64_t exclusiveSum(const uint32_t *in, uint32_t *out, size_t n, cudaStream_t s)
{
  if (n >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "element cell grid too large");
  size_t tb = 0;
  cudaCheck(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, (int)n, s), "scan size");
  DBuf<unsigned char> temp;
  temp.alloc(tb ? tb : 1);
  cudaCheck(cub::DeviceScan::ExclusiveSum(temp.ptr, tb, in, out, (int)n, s), "scan");
  uint32_t last[2] = {0u, 0u};
  cudaCheck(cudaMemcpyAsync(&last[0], out + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "scan last");
  cudaCheck(cudaMemcpyAsync(&last[1], in + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "scan last");
  cudaCheck(cudaStreamSynchronize(s), "scan");
  return (uint64_t)last[0] + last[1];
}

void launchElemCells(const float4 *verts, const int32_t *idx, size_t ne, ElemOccupancy &O, DBuf<uint32_t> &bits,
                     DBuf<uint32_t> &rank, DBuf<int32_t> &entries, DBuf<int32_t> &items, DBuf<float4> &boxes,
                     cudaStream_t s)
{
  const size_t nc = (size_t)O.n[0] * O.n[1] * O.n[2];
  const size_t words = (nc + 31) / 32;
  bits.alloc(words);
  rank.alloc(words);
  boxes.alloc(2 * std::max<size_t>(ne, 1));
  cudaCheck(cudaMemsetAsync(bits.ptr, 0, words * sizeof(uint32_t), s), "memset cell bits");
  O.bits = bits.ptr;
  O.rank = rank.ptr;
  O.boxes = boxes.ptr;
  O.entries = nullptr;
  O.items = nullptr;
  O.numMarked = O.numItems = 0;
  if (!ne) return;
  k_elem_cells_mark<<<gridFor(ne, 256), 256, 0, s>>>(verts, idx, ne, O, bits.ptr, boxes.ptr);
  cudaCheck(cudaGetLastError(), "k_elem_cells_mark");
  DBuf<uint32_t> pc;
  pc.alloc(words);
  k_popc_words<<<gridFor(words, 256), 256, 0, s>>>(bits.ptr, words, pc.ptr);
  cudaCheck(cudaGetLastError(), "k_popc_words");
  const uint64_t nm = exclusiveSum(pc.ptr, rank.ptr, words, s);
  if (nm == 0 || nm >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "element cells: bad marked-cell count");
  DBuf<uint32_t> count, off, cursor;
  count.alloc(nm);
  off.alloc(nm);
  cursor.alloc(nm);
  cudaCheck(cudaMemsetAsync(count.ptr, 0, nm * sizeof(uint32_t), s), "memset counts");
  cudaCheck(cudaMemsetAsync(cursor.ptr, 0, nm * sizeof(uint32_t), s), "memset cursors");
  entries.alloc(nm);
  k_elem_cells_lists<<<gridFor(ne, 256), 256, 0, s>>>(ne, O, bits.ptr, rank.ptr, boxes.ptr, count.ptr, nullptr,
                                                      nullptr, nullptr, nullptr, false);
  cudaCheck(cudaGetLastError(), "k_elem_cells_lists count");
  k_elem_cells_seg<<<gridFor(nm, 256), 256, 0, s>>>(count.ptr, nm, cursor.ptr);  // cursor as scratch
  const uint64_t ni = exclusiveSum(cursor.ptr, off.ptr, nm, s);
  if (ni >= 0x7fffffffull) throw Error(EXA_ERR_INVALID, "element cells: lists too long");
  cudaCheck(cudaMemsetAsync(cursor.ptr, 0, nm * sizeof(uint32_t), s), "memset cursors");
  items.alloc(std::max<uint64_t>(ni, 1));
  k_elem_cells_heads<<<gridFor(nm, 256), 256, 0, s>>>(count.ptr, off.ptr, nm, entries.ptr, items.ptr);
  cudaCheck(cudaGetLastError(), "k_elem_cells_heads");
  k_elem_cells_lists<<<gridFor(ne, 256), 256, 0, s>>>(ne, O, bits.ptr, rank.ptr, boxes.ptr, count.ptr, off.ptr,
                                                      cursor.ptr, entries.ptr, items.ptr, true);
  cudaCheck(cudaGetLastError(), "k_elem_cells_lists fill");
  k_elem_cells_sort<<<gridFor(nm, 256), 256, 0, s>>>(count.ptr, off.ptr, nm, items.ptr);
  cudaCheck(cudaGetLastError(), "k_elem_cells_sort");
  cudaCheck(cudaStreamSynchronize(s), "element cells");
  O.entries = entries.ptr;
  O.items = items.ptr;
  O.numMarked = (int)nm;
  O.numItems = (int)std::max<uint64_t>(ni, 1);
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
  DBuf<unsigned> counters;
  counters.alloc(n > 1 ? n - 1 : 1);
  cudaCheck(cudaMemsetAsync(counters.ptr, 0, counters.bytes(), s), "memset counters");
  k_bvh_refit<<<gridFor(ne, 256), 256, 0, s>>>(verts, idx, n, nodes, parents, leafElem, counters.ptr);
  cudaCheck(cudaGetLastError(), "k_bvh_refit");
  cudaCheck(cudaStreamSynchronize(s), "bvh build");
}

} // namespace exa
