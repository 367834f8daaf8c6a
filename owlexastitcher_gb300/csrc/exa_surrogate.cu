// exa_surrogate.cu -- training, error bounds and majorants of the learned
// field (hash-grid encoding + MLP, exa_surrogate.cuh).  No counterpart in
// the reference: this is the learned stand-in beside the exact ExaStitch
// sampler.
//
// Training data: (position, value) pairs drawn by the exact sampler
// (sample() of sampler/ExaStitchSampler.h:128-140, here sample_field), half
// uniform over the cell bounds and half uniform inside gridlets of the
// refined levels.  One training step on a batch of B pairs is three kernels:
//   k_sur_encode_fwd  encoding of the batch from the FP32 master table
//                     (one thread per pair) -> BF16 inputs [B][32]
//   k_sur_mlp_train_tc forward and backward of the MLP on the 5th-generation
//                     tensor cores (tcgen05.mma, accumulators in tensor
//                     memory), 128 pairs per tile; weight gradients
//                     accumulated in tensor memory per block; input
//                     gradients [B][32] FP32
//   k_sur_encode_bwd  scatter of the input gradients into the table
//                     gradient (float2 atomics)
// then Adam over the table and the weights, which also refreshes the FP16
// table and BF16 weights used for inference.
//
// Error bounds: every macrocell is probed on a jittered s^3 lattice; the
// largest |surrogate - exact| (FP64) of a macrocell widens its value range
// before the max-opacity lookup, and a macrocell whose error exceeds the
// tolerance, or that holds empty space, keeps the exact sampler.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "exa_host.h"
#include "exa_surrogate.cuh"
#include "exa_tcgen05.cuh"

namespace exa {

namespace {

inline unsigned gridFor(size_t n, unsigned bs)
{
  const size_t g = (n + bs - 1) / bs;
  return (unsigned)std::min<size_t>(g, 1u << 30);
}

EXA_HD float u01(uint64_t key, uint64_t n)
{
  return (float)(uint32_t)(mix64(key + n * 0x9e3779b97f4a7c15ull) >> 40) * 5.96046448e-08f;
}

}  // namespace

// ----------------------------------------------------------- training data
// samples[i] = (x, y, z, value); value is NaN where no primitive holds the
// point.  The first nUniform are uniform over the bounds, the rest uniform
// inside a gridlet picked uniformly from refined[].
__global__ void k_sur_samples(const __grid_constant__ AccelView A, exa_box3f bounds, size_t n, size_t nUniform,
                              const int32_t *__restrict__ refined, int numRefined, uint64_t seed, float4 *out)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t key = mix64(seed ^ mix64(i + 0x632be59bd9b4e019ull));
  V3 pos;
  if (i < nUniform || numRefined == 0) {
    pos = mk3(bounds.lower.x + u01(key, 1) * (bounds.upper.x - bounds.lower.x),
              bounds.lower.y + u01(key, 2) * (bounds.upper.y - bounds.lower.y),
              bounds.lower.z + u01(key, 3) * (bounds.upper.z - bounds.lower.z));
  } else {
    const int pick = min((int)(u01(key, 4) * (float)numRefined), numRefined - 1);
    const exa_gridlet g = A.gridlets[refined[pick]];
    const float cw = (float)(1 << g.level);
    const V3 lo = muls(mk3((float)g.lower.x + 0.5f, (float)g.lower.y + 0.5f, (float)g.lower.z + 0.5f), cw);
    pos = mk3(lo.x + u01(key, 1) * (float)g.dims.x * cw, lo.y + u01(key, 2) * (float)g.dims.y * cw,
              lo.z + u01(key, 3) * (float)g.dims.z * cw);
  }
  uint32_t err = 0;
  const exa_sample s = sample_field(A, pos, false, err);
  out[i] = make_float4(pos.x, pos.y, pos.z, s.primID >= 0 ? s.value : __int_as_float(0x7fc00000));
}

// ------------------------------------------------------- encoding, forward
__global__ void k_sur_encode_fwd(const __grid_constant__ SurrogateView S, const float2 *__restrict__ table,
                                 const float4 *__restrict__ samples, size_t first, size_t numSamples, int B,
                                 __nv_bfloat16 *feats)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const float4 sp = samples[(first + (size_t)i) % numSamples];
  const V3 x = sur_normalize(S, mk3(sp.x, sp.y, sp.z));
  const size_t T = (size_t)1 << S.log2T;
  uint32_t packed[kSurIn / 2];
  for (int l = 0; l < kSurLevels; ++l) {
    uint32_t idx[8];
    float w[8];
    sur_corners(S, l, x, idx, w);
    float f0 = 0.f, f1 = 0.f;
    const float2 *tab = table + (size_t)l * T;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float2 e = __ldg(tab + idx[k]);
      f0 += w[k] * e.x;
      f1 += w[k] * e.y;
    }
    const __nv_bfloat162 v = __floats2bfloat162_rn(f0, f1);
    packed[l] = *reinterpret_cast<const uint32_t *>(&v);
  }
  uint4 *dst = reinterpret_cast<uint4 *>(feats + (size_t)i * kSurIn);
  for (int q = 0; q < 4; ++q) dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
}

// ------------------------------------------------------ encoding, backward
__global__ void k_sur_encode_bwd(const __grid_constant__ SurrogateView S, const float4 *__restrict__ samples,
                                 size_t first, size_t numSamples, int B, const float *__restrict__ dfeat, float2 *gtable)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const float4 sp = samples[(first + (size_t)i) % numSamples];
  const V3 x = sur_normalize(S, mk3(sp.x, sp.y, sp.z));
  const size_t T = (size_t)1 << S.log2T;
  const float *d = dfeat + (size_t)i * kSurIn;
  for (int l = 0; l < kSurLevels; ++l) {
    const float g0 = d[2 * l], g1 = d[2 * l + 1];
    if (g0 == 0.f && g1 == 0.f) continue;
    uint32_t idx[8];
    float w[8];
    sur_corners(S, l, x, idx, w);
    float2 *tab = gtable + (size_t)l * T;
#pragma unroll
    for (int k = 0; k < 8; ++k) atomicAdd(tab + idx[k], make_float2(w[k] * g0, w[k] * g1));
  }
}

// ------------------------------------------------ MLP training, tcgen05
// The same forward and backward on the 5th-generation tensor cores: one
// block of 128 threads per SM takes 128-pair tiles in turn; every product is
// a tcgen05.mma of M = 128 rows with BF16 operands in shared memory
// (K-major tiles, exa_tcgen05.cuh) and an FP32 accumulator in tensor memory,
// issued by one thread and completed on an mbarrier; thread r owns pair r
// of the tile (tensor-memory lane r) for the element-wise steps:
//   layer 1  D1 = x W1^T            (K 32)  -> h1 = bf16(relu(D1))
//   layer 2  D2 = h1 W2^T           (K 64)  -> h2, y, g, gw3, d2
//   d1       D1 = d2 W2             (K 64)  -> d1 = bf16(D1) where h1 > 0
//   din      D2 = d1 W1             (K 64)  -> din (FP32) to global
//   weights  GW += [d2^T; d1^T] [h1 | x]   (K = the tile's 128 pairs): rows
//            0..63 x columns 0..63 are gw2, rows 64..127 x columns 64..95
//            gw1 (the two other blocks are not read); GW accumulates over
//            the block's tiles and is added to gw once.
// Operands and tensor-memory columns are reused step by step; every step
// starts after the previous one's commit.  Waits are bounded: a wait that
// gives up sets EXA_DEVERR_WATCHDOG in *errors and the block stops.  The
// tensor-memory loads (tcgen05.ld) are warp-collective: every thread of a
// warp executes each of them, also for pairs past the batch.
struct alignas(1024) TcTrainSmem {
  __nv_bfloat16 w1[kSurHidden * kSurIn];        // B of layer 1: (j, k), K 32
  __nv_bfloat16 w2[kSurHidden * kSurHidden];    // B of layer 2: (j, i), K 64
  __nv_bfloat16 w2t[kSurHidden * kSurHidden];   // B of d1: (i, j), K 64
  __nv_bfloat16 w1t[kSurIn * kSurHidden];       // B of din: (k, j), K 64
  __nv_bfloat16 x[128 * kSurIn];                // A of layer 1: (r, k)
  __nv_bfloat16 h1[128 * kSurHidden];           // A of layer 2: (r, i); then A of din: d1 (r, j)
  __nv_bfloat16 d2[128 * kSurHidden];           // A of d1: (r, j)
  __nv_bfloat16 aw[128 * 128];                  // A of the weight product: d2^T, d1^T; K = pair
  __nv_bfloat16 bw[96 * 128];                   // B of the weight product: h1^T, x^T; K = pair
  float w3[kSurHidden];
  float gw3[kSurHidden];
  float loss;
  uint32_t tmem;
  uint32_t stop;
  uint64_t bar;
};
constexpr uint32_t kTcCols = 256;    // tensor-memory columns per block
constexpr uint32_t kColD1 = 0, kColD2 = 64, kColGW = 128;

__global__ void __launch_bounds__(128, 1) k_sur_mlp_train_tc(
    const __nv_bfloat16 *__restrict__ w1g, const __nv_bfloat16 *__restrict__ w2g, const __nv_bfloat16 *__restrict__ w3g,
    const __nv_bfloat16 *__restrict__ feats, const float4 *__restrict__ samples, size_t first, size_t numSamples, int B,
    float vmin, float invRange, float invB, float *gw, float *lossOut, float *dfeat, uint32_t *errors)
{
  extern __shared__ __align__(1024) unsigned char tcSmRaw[];
  TcTrainSmem &S = *reinterpret_cast<TcTrainSmem *>(tcSmRaw);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < kSurHidden * kSurIn; i += blockDim.x) {
    const int j = i / kSurIn, k = i % kSurIn;
    S.w1[tc::kmajor(j, k, kSurIn)] = w1g[i];
    S.w1t[tc::kmajor(k, j, kSurHidden)] = w1g[i];
  }
  for (int i = tid; i < kSurHidden * kSurHidden; i += blockDim.x) {
    const int j = i / kSurHidden, k = i % kSurHidden;
    S.w2[tc::kmajor(j, k, kSurHidden)] = w2g[i];
    S.w2t[tc::kmajor(k, j, kSurHidden)] = w2g[i];
  }
  if (tid < kSurHidden) {
    S.w3[tid] = __bfloat162float(w3g[tid]);
    S.gw3[tid] = 0.f;
  }
  if (tid == 0) {
    S.loss = 0.f;
    S.stop = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::smem_addr(&S.bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&S.tmem, kTcCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = S.tmem;
  const uint32_t lanes = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's lane quarter
  uint32_t phase = 0;
  // operands written by the threads -> visible to the tensor core, then one
  // thread issues
  auto sync_operands = [&]() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  };
  // every thread waits for the committed products, at most about a second
  auto wait_products = [&]() -> bool {
    bool done = tc::mbar_try_wait(&S.bar, phase);
    const uint64_t t0 = tc::globaltimer_ns();
    for (int i = 0; i < (1 << 22) && !done && tc::globaltimer_ns() - t0 < 1000000000ull; ++i)
      done = tc::mbar_try_wait(&S.bar, phase);
    phase ^= 1u;
    if (!done) atomicOr(&S.stop, 1u);
    __syncthreads();
    tc::fence_after_sync();
    return S.stop == 0;
  };
  float gw3acc[kSurHidden];
#pragma unroll
  for (int j = 0; j < kSurHidden; ++j) gw3acc[j] = 0.f;
  float lossAcc = 0.f;
  const int tiles = (B + 127) / 128;
  bool any = false;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int r = tile * 128 + tid;
    const bool inB = r < B;
    // inputs (x and x^T) and the target
    uint4 q[4] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    float target = 0.f;
    bool valid = false;
    if (inB) {
      const uint4 *src = reinterpret_cast<const uint4 *>(feats + (size_t)r * kSurIn);
#pragma unroll
      for (int c = 0; c < 4; ++c) q[c] = src[c];
      const float v = samples[(first + (size_t)r) % numSamples].w;
      valid = v == v;
      target = valid ? (v - vmin) * invRange : 0.f;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) *reinterpret_cast<uint4 *>(S.x + tc::kmajor(tid, 8 * c, kSurIn)) = q[c];
    {
      const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(q);
#pragma unroll
      for (int k = 0; k < kSurIn; ++k) S.bw[tc::kmajor(64 + k, tid, 128)] = e[k];
    }
    sync_operands();
    // layer 1
    if (tid == 0) {
      for (int kk = 0; kk < kSurIn / 16; ++kk)
        tc::mma_bf16(tmem + kColD1, tc::desc_kslice(S.x, kSurIn, kk), tc::desc_kslice(S.w1, kSurIn, kk),
                     tc::idesc_bf16_f32(128, kSurHidden), kk > 0);
      tc::commit(&S.bar);
    }
    if (!wait_products()) break;
    for (int c = 0; c < kSurHidden / 16; ++c) {
      float v[16];
      tc::ld16(lanes + kColD1 + 16 * c, v);
      __align__(16) __nv_bfloat16 h[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) h[j] = __float2bfloat16_rn(fmaxf(v[j], 0.f));
      *reinterpret_cast<uint4 *>(S.h1 + tc::kmajor(tid, 16 * c, kSurHidden)) = *reinterpret_cast<const uint4 *>(h);
      *reinterpret_cast<uint4 *>(S.h1 + tc::kmajor(tid, 16 * c + 8, kSurHidden)) =
          *reinterpret_cast<const uint4 *>(h + 8);
#pragma unroll
      for (int j = 0; j < 16; ++j) S.bw[tc::kmajor(16 * c + j, tid, 128)] = h[j];
    }
    sync_operands();
    // layer 2
    if (tid == 0) {
      for (int kk = 0; kk < kSurHidden / 16; ++kk)
        tc::mma_bf16(tmem + kColD2, tc::desc_kslice(S.h1, kSurHidden, kk), tc::desc_kslice(S.w2, kSurHidden, kk),
                     tc::idesc_bf16_f32(128, kSurHidden), kk > 0);
      tc::commit(&S.bar);
    }
    if (!wait_products()) break;
    // output, loss and its gradient (pair tid)
    float y = 0.f;
    for (int c = 0; c < kSurHidden / 16; ++c) {
      float v[16];
      tc::ld16(lanes + kColD2 + 16 * c, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) y += bf16_round(fmaxf(v[j], 0.f)) * S.w3[16 * c + j];
    }
    const float diff = y - target;
    const float gr = (inB && valid) ? 2.f * diff * invB : 0.f;
    if (inB && valid) lossAcc += diff * diff;
    // gw3 and d2 = bf16(g w3) where h2 > 0
#pragma unroll
    for (int c = 0; c < kSurHidden / 16; ++c) {
      float v[16];
      tc::ld16(lanes + kColD2 + 16 * c, v);
      __align__(16) __nv_bfloat16 d[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float h2 = bf16_round(fmaxf(v[j], 0.f));
        gw3acc[16 * c + j] += gr * h2;
        d[j] = __float2bfloat16_rn(h2 > 0.f ? gr * S.w3[16 * c + j] : 0.f);
      }
      *reinterpret_cast<uint4 *>(S.d2 + tc::kmajor(tid, 16 * c, kSurHidden)) = *reinterpret_cast<const uint4 *>(d);
      *reinterpret_cast<uint4 *>(S.d2 + tc::kmajor(tid, 16 * c + 8, kSurHidden)) =
          *reinterpret_cast<const uint4 *>(d + 8);
#pragma unroll
      for (int j = 0; j < 16; ++j) S.aw[tc::kmajor(16 * c + j, tid, 128)] = d[j];
    }
    sync_operands();
    // d1 = d2 W2
    if (tid == 0) {
      for (int kk = 0; kk < kSurHidden / 16; ++kk)
        tc::mma_bf16(tmem + kColD1, tc::desc_kslice(S.d2, kSurHidden, kk), tc::desc_kslice(S.w2t, kSurHidden, kk),
                     tc::idesc_bf16_f32(128, kSurHidden), kk > 0);
      tc::commit(&S.bar);
    }
    if (!wait_products()) break;
    for (int c = 0; c < kSurHidden / 16; ++c) {
      float v[16];
      tc::ld16(lanes + kColD1 + 16 * c, v);
      __align__(16) __nv_bfloat16 h[16], d[16];
      *reinterpret_cast<uint4 *>(h) = *reinterpret_cast<const uint4 *>(S.h1 + tc::kmajor(tid, 16 * c, kSurHidden));
      *reinterpret_cast<uint4 *>(h + 8) =
          *reinterpret_cast<const uint4 *>(S.h1 + tc::kmajor(tid, 16 * c + 8, kSurHidden));
#pragma unroll
      for (int j = 0; j < 16; ++j) d[j] = __float2bfloat16_rn(__bfloat162float(h[j]) > 0.f ? v[j] : 0.f);
      *reinterpret_cast<uint4 *>(S.h1 + tc::kmajor(tid, 16 * c, kSurHidden)) = *reinterpret_cast<const uint4 *>(d);
      *reinterpret_cast<uint4 *>(S.h1 + tc::kmajor(tid, 16 * c + 8, kSurHidden)) =
          *reinterpret_cast<const uint4 *>(d + 8);
#pragma unroll
      for (int j = 0; j < 16; ++j) S.aw[tc::kmajor(64 + 16 * c + j, tid, 128)] = d[j];
    }
    sync_operands();
    // din = d1 W1 and the weight product
    if (tid == 0) {
      for (int kk = 0; kk < kSurHidden / 16; ++kk)
        tc::mma_bf16(tmem + kColD2, tc::desc_kslice(S.h1, kSurHidden, kk), tc::desc_kslice(S.w1t, kSurHidden, kk),
                     tc::idesc_bf16_f32(128, kSurIn), kk > 0);
      for (int kk = 0; kk < 128 / 16; ++kk)
        tc::mma_bf16(tmem + kColGW, tc::desc_kslice(S.aw, 128, kk), tc::desc_kslice(S.bw, 128, kk),
                     tc::idesc_bf16_f32(128, 96), any || kk > 0);
      tc::commit(&S.bar);
    }
    any = true;
    if (!wait_products()) break;
    // every thread of a warp takes part in the (warp-collective) loads;
    // pairs past B store nothing
    for (int c = 0; c < kSurIn / 16; ++c) {
      float v[16];
      tc::ld16(lanes + kColD2 + 16 * c, v);
      if (inB) {
        float4 *dst = reinterpret_cast<float4 *>(dfeat + (size_t)r * kSurIn);
#pragma unroll
        for (int k = 0; k < 4; ++k) dst[4 * c + k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (S.stop && errors && tid == 0) atomicOr(errors, EXA_DEVERR_WATCHDOG);
  // weight gradients: gw2 (rows 0..63, columns 0..63), gw1 (rows 64..127,
  // columns 64..95) of the accumulator
  if (any && !S.stop) {
    if (tid < kSurHidden) {
      for (int c = 0; c < kSurHidden / 16; ++c) {
        float v[16];
        tc::ld16(lanes + kColGW + 16 * c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (v[j] != 0.f) atomicAdd(gw + kSurHidden * kSurIn + tid * kSurHidden + 16 * c + j, v[j]);
      }
    } else {
      for (int c = 0; c < kSurIn / 16; ++c) {
        float v[16];
        tc::ld16(lanes + kColGW + 64 + 16 * c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (v[j] != 0.f) atomicAdd(gw + (tid - kSurHidden) * kSurIn + 16 * c + j, v[j]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kSurHidden; ++j) atomicAdd(&S.gw3[j], gw3acc[j]);
  for (int o = 16; o > 0; o >>= 1) lossAcc += __shfl_xor_sync(0xffffffffu, lossAcc, o);
  if ((tid & 31) == 0) atomicAdd(&S.loss, lossAcc);
  tc::fence_before_sync();
  __syncthreads();
  if (tid < kSurHidden && S.gw3[tid] != 0.f)
    atomicAdd(gw + kSurHidden * kSurIn + kSurHidden * kSurHidden + tid, S.gw3[tid]);
  if (tid == 0) atomicAdd(lossOut, S.loss);
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcCols);
  }
}

// --------------------------------------------------------------------- Adam
// p -= lr * mhat / (sqrt(vhat) + eps); the gradient is cleared.  n2 pairs.
__global__ void k_sur_adam_table(float2 *p, float2 *gr, float2 *m, float2 *v, size_t n, float lr, float b1, float b2,
                                 float c1, float c2, float eps, __half2 *half)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 g = gr[i];
  float2 mm = m[i], vv = v[i], pp = p[i];
  mm.x = b1 * mm.x + (1.f - b1) * g.x;
  mm.y = b1 * mm.y + (1.f - b1) * g.y;
  vv.x = b2 * vv.x + (1.f - b2) * g.x * g.x;
  vv.y = b2 * vv.y + (1.f - b2) * g.y * g.y;
  pp.x -= lr * (mm.x * c1) / (sqrtf(vv.x * c2) + eps);
  pp.y -= lr * (mm.y * c1) / (sqrtf(vv.y * c2) + eps);
  m[i] = mm;
  v[i] = vv;
  p[i] = pp;
  gr[i] = make_float2(0.f, 0.f);
  half[i] = __floats2half2_rn(pp.x, pp.y);
}

__global__ void k_sur_adam_mlp(float *p, float *gr, float *m, float *v, int n, float lr, float b1, float b2, float c1,
                               float c2, float eps, __nv_bfloat16 *bf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = gr[i];
  const float mm = b1 * m[i] + (1.f - b1) * g;
  const float vv = b2 * v[i] + (1.f - b2) * g * g;
  const float pp = p[i] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
  m[i] = mm;
  v[i] = vv;
  p[i] = pp;
  gr[i] = 0.f;
  bf[i] = __float2bfloat16_rn(pp);
}

__global__ void k_sur_init_table(float2 *p, size_t n, uint64_t seed, float scale, __half2 *half)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t key = mix64(seed ^ (i * 0x9e3779b97f4a7c15ull));
  const float a = (u01(key, 1) * 2.f - 1.f) * scale, b = (u01(key, 2) * 2.f - 1.f) * scale;
  p[i] = make_float2(a, b);
  half[i] = __floats2half2_rn(a, b);
}

__global__ void k_f32_to_bf16(const float *p, int n, __nv_bfloat16 *bf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) bf[i] = __float2bfloat16_rn(p[i]);
}

// -------------------------------------------------------------- inference
// values of n points (one warp per 32 points); value = vmin + y * vrange
__global__ void __launch_bounds__(128) k_sur_points(const __grid_constant__ SurrogateView S, const exa_vec3f *pos,
                                                     size_t n, float *out)
{
  __shared__ SurWeightsSmem W;
  __shared__ SurWarpSmem ws[4];
  sur_load_weights(W, S);
  __syncthreads();
  const size_t warps = (size_t)gridDim.x * 4;
  for (size_t base = (blockIdx.x * (size_t)4 + (threadIdx.x >> 5)) * 32; base < n; base += warps * 32) {
    const size_t i = base + (threadIdx.x & 31);
    const bool want = i < n;
    V3 p = mk3(0.f, 0.f, 0.f);
    if (want) p = mk3(pos[i].x, pos[i].y, pos[i].z);
    const float y = sur_eval_warp(S, W, ws[threadIdx.x >> 5], p, want);
    if (want) out[i] = S.vmin + y * S.vrange;
  }
}

// ---------------------------------------------------------- error bounds
// point p of n: macrocell p / s^3, jittered lattice point p % s^3 in it
__global__ void __launch_bounds__(128) k_sur_mc_error(const __grid_constant__ AccelView A,
                                                       const __grid_constant__ SurrogateView S, exa_vec3i dims,
                                                       exa_box3f wb, int s, size_t n, uint64_t seed,
                                                       unsigned long long *mcErr, unsigned *mcEmpty, double *sums)
{
  __shared__ SurWeightsSmem W;
  __shared__ SurWarpSmem ws[4];
  sur_load_weights(W, S);
  __syncthreads();
  const size_t warps = (size_t)gridDim.x * 4;
  const size_t s3 = (size_t)s * s * s;
  double sq = 0.0, cnt = 0.0;
  for (size_t base = (blockIdx.x * (size_t)4 + (threadIdx.x >> 5)) * 32; base < n; base += warps * 32) {
    const size_t i = base + (threadIdx.x & 31);
    const bool inRange = i < n;
    size_t mc = 0;
    V3 p = mk3(0.f, 0.f, 0.f);
    exa_sample ex{-1, -1, 0.f};
    if (inRange) {
      mc = i / s3;
      const size_t sub = i - mc * s3;
      const int mx = (int)(mc % dims.x), my = (int)((mc / dims.x) % dims.y), mz = (int)(mc / ((size_t)dims.x * dims.y));
      const int sx = (int)(sub % s), sy = (int)((sub / s) % s), sz = (int)(sub / ((size_t)s * s));
      const uint64_t key = mix64(seed ^ mix64(i + 0x2545f4914f6cdd1dull));
      const float fx = ((float)mx + ((float)sx + u01(key, 1)) / (float)s) / (float)dims.x;
      const float fy = ((float)my + ((float)sy + u01(key, 2)) / (float)s) / (float)dims.y;
      const float fz = ((float)mz + ((float)sz + u01(key, 3)) / (float)s) / (float)dims.z;
      p = mk3(wb.lower.x + fx * (wb.upper.x - wb.lower.x), wb.lower.y + fy * (wb.upper.y - wb.lower.y),
              wb.lower.z + fz * (wb.upper.z - wb.lower.z));
      uint32_t err = 0;
      ex = sample_field(A, p, false, err);
    }
    const float y = sur_eval_warp(S, W, ws[threadIdx.x >> 5], p, inRange);
    if (inRange) {
      if (ex.primID < 0) {
        atomicOr(mcEmpty + mc, 1u);
      } else {
        const double e = fabs((double)(S.vmin + y * S.vrange) - (double)ex.value);
        atomicMax(mcErr + mc, (unsigned long long)__double_as_longlong(e));
        sq += e * e;
        cnt += 1.0;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums, sq);
    atomicAdd(sums + 1, cnt);
  }
}

// mode and widened value range of every macrocell
__global__ void k_sur_widen(const exa_range1f *ranges, const unsigned long long *mcErr, const unsigned *mcEmpty,
                            size_t n, double tolAbs, uint8_t *mode, exa_range1f *widened, unsigned *numSurrogate)
{
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const exa_range1f r = ranges[i];
  const double e = __longlong_as_double((long long)mcErr[i]);
  const bool ok = mcEmpty[i] == 0u && r.lower <= r.upper && e <= tolAbs;
  mode[i] = ok ? 1 : 0;
  if (ok) {
    // widened outward: the FP32 bounds are rounded away from the range
    const float ef = __double2float_ru(e);
    widened[i] = exa_range1f{__fsub_rd(r.lower, ef), __fadd_ru(r.upper, ef)};
    atomicAdd(numSurrogate, 1u);
  } else {
    widened[i] = r;
  }
}

// ------------------------------------------------------------------- host
void Surrogate::configure(const SurrogateConfig &c, const ExaStitchModel &model)
{
  cfg = c;
  if (cfg.levels != kSurLevels) throw Error(EXA_ERR_INVALID, "the surrogate has 16 levels");
  if (cfg.log2T < 10 || cfg.log2T > 24) throw Error(EXA_ERR_INVALID, "log2 table size must be in [10, 24]");
  if (cfg.batch < 32 || cfg.batch > (1 << 22)) throw Error(EXA_ERR_INVALID, "batch must be in [32, 2^22]");
  std::memset(&view, 0, sizeof(view));
  view.levels = kSurLevels;
  view.log2T = cfg.log2T;
  view.denseMask = 0;
  const uint64_t T = 1ull << cfg.log2T;
  for (int l = 0; l < kSurLevels; ++l) {
    const int r = (int)std::floor((double)cfg.baseRes * std::pow((double)cfg.growth, (double)l));
    view.res[l] = std::max(r, 1);
    const uint64_t side = (uint64_t)view.res[l] + 1;
    if (side * side * side <= T) view.denseMask |= 1u << l;
  }
  const exa_box3f b = model.cellBounds;
  view.lo[0] = b.lower.x;
  view.lo[1] = b.lower.y;
  view.lo[2] = b.lower.z;
  view.inv[0] = 1.f / std::max(b.upper.x - b.lower.x, 1e-30f);
  view.inv[1] = 1.f / std::max(b.upper.y - b.lower.y, 1e-30f);
  view.inv[2] = 1.f / std::max(b.upper.z - b.lower.z, 1e-30f);
  float vmin = model.valueRange.lower, vmax = model.valueRange.upper;
  if (!(vmin <= vmax)) { vmin = 0.f; vmax = 1.f; }
  view.vmin = vmin;
  view.vrange = vmax > vmin ? vmax - vmin : 1.f;
}

void Surrogate::allocate(cudaStream_t s)
{
  const size_t n = (size_t)kSurLevels << cfg.log2T;
  table.alloc(n);
  gtable.alloc(n);
  mTable.alloc(n);
  vTable.alloc(n);
  table16.alloc(n);
  cudaCheck(cudaMemsetAsync(gtable.ptr, 0, gtable.bytes(), s), "memset");
  cudaCheck(cudaMemsetAsync(mTable.ptr, 0, mTable.bytes(), s), "memset");
  cudaCheck(cudaMemsetAsync(vTable.ptr, 0, vTable.bytes(), s), "memset");
  k_sur_init_table<<<gridFor(n, 256), 256, 0, s>>>(table.ptr, n, cfg.seed ^ 0x7a1b, 1e-4f, table16.ptr);
  cudaCheck(cudaGetLastError(), "k_sur_init_table");
  // MLP: uniform He-style initialisation from a host RNG stream
  std::vector<float> w(kSurParams);
  uint64_t key = mix64(cfg.seed ^ 0x5eedull);
  auto uni = [&](uint64_t k) { return (float)(uint32_t)(mix64(key + k * 0x9e3779b97f4a7c15ull) >> 40) * 5.96046448e-08f; };
  const float a1 = std::sqrt(6.f / (float)(kSurIn + kSurHidden));
  const float a2 = std::sqrt(6.f / (float)(kSurHidden + kSurHidden));
  const float a3 = std::sqrt(6.f / (float)(kSurHidden + 1));
  for (int i = 0; i < kSurParams; ++i) {
    const float a = i < kSurHidden * kSurIn ? a1 : (i < kSurHidden * kSurIn + kSurHidden * kSurHidden ? a2 : a3);
    w[i] = (uni((uint64_t)i + 1) * 2.f - 1.f) * a;
  }
  setWeights(w.data(), s);
  std::vector<float> z(kSurParams, 0.f);
  gw.upload(z.data(), z.size(), s);
  mw.upload(z.data(), z.size(), s);
  vw.upload(z.data(), z.size(), s);
  step = 0;
}

void Surrogate::setWeights(const float *w, cudaStream_t s)
{
  w32.upload(w, kSurParams, s);
  if (wbf.count != (size_t)kSurParams) wbf.alloc(kSurParams);
  k_f32_to_bf16<<<gridFor(kSurParams, 256), 256, 0, s>>>(w32.ptr, kSurParams, wbf.ptr);
  cudaCheck(cudaGetLastError(), "k_f32_to_bf16");
}

void Surrogate::setTable(const float *t, cudaStream_t s)
{
  const size_t n = (size_t)kSurLevels << cfg.log2T;
  table.upload(reinterpret_cast<const float2 *>(t), n, s);
  std::vector<__half2> h(n);
  for (size_t i = 0; i < n; ++i) h[i] = __floats2half2_rn(t[2 * i], t[2 * i + 1]);
  table16.upload(h.data(), n, s);
}

SurrogateView Surrogate::deviceView() const
{
  SurrogateView v = view;
  v.table = table16.ptr;
  v.w1 = wbf.ptr;
  v.w2 = wbf.ptr + kSurHidden * kSurIn;
  v.w3 = wbf.ptr + kSurHidden * kSurIn + kSurHidden * kSurHidden;
  v.mcMode = mcMode.ptr;
  return v;
}

void Surrogate::generateSamples(const ExaStitchSampler &sampler, cudaStream_t s)
{
  const auto &G = sampler.model->gridlets;
  int maxLevel = 0;
  for (const auto &g : G) maxLevel = std::max(maxLevel, g.level);
  std::vector<int32_t> refined;
  for (size_t i = 0; i < G.size(); ++i)
    if (G[i].level < maxLevel) refined.push_back((int32_t)i);
  DBuf<int32_t> dRefined;
  if (!refined.empty()) dRefined.upload(refined.data(), refined.size(), s);
  samples.alloc(cfg.numSamples);
  const size_t nUniform = refined.empty() ? cfg.numSamples : (size_t)((double)cfg.numSamples * (1.0 - cfg.importance));
  k_sur_samples<<<gridFor(cfg.numSamples, 256), 256, 0, s>>>(sampler.accel, sampler.model->cellBounds,
                                                              cfg.numSamples, nUniform, dRefined.ptr,
                                                              (int)refined.size(), cfg.seed, samples.ptr);
  cudaCheck(cudaGetLastError(), "k_sur_samples");
  cudaCheck(cudaStreamSynchronize(s), "surrogate samples");
}

// the MLP training step of B pairs on the tensor cores: one block of
// k_sur_mlp_train_tc per SM (its 124 KB of operands), 128 pairs per tile
static void launchMlpTrain(const SurrogateView &v, const __nv_bfloat16 *feats, const float4 *samples, size_t first,
                           size_t numSamples, int B, float vmin, float invRange, float invB, float *gw, float *loss,
                           float *dfeat, uint32_t *errors, cudaStream_t s)
{
  int dev = 0, sms = 152;
  cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  cudaCheck(cudaFuncSetAttribute(k_sur_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(TcTrainSmem)),
            "train smem");
  const unsigned blocks = (unsigned)std::min<int>((B + 127) / 128, sms);
  k_sur_mlp_train_tc<<<blocks, 128, sizeof(TcTrainSmem), s>>>(v.w1, v.w2, v.w3, feats, samples, first, numSamples, B,
                                                              vmin, invRange, invB, gw, loss, dfeat, errors);
  cudaCheck(cudaGetLastError(), "MLP training step");
}

float Surrogate::trainSteps(int steps, cudaStream_t s)
{
  if (!samples.ptr) throw Error(EXA_ERR_INVALID, "no training samples");
  const int B = cfg.batch;
  if (feats.count < (size_t)B * kSurIn) feats.alloc((size_t)B * kSurIn);
  if (dfeat.count < (size_t)B * kSurIn) dfeat.alloc((size_t)B * kSurIn);
  if (!lossBuf.ptr) lossBuf.alloc(2);
  const size_t nTab = (size_t)kSurLevels << cfg.log2T;
  const SurrogateView v = deviceView();
  if (!trainErrors.ptr) trainErrors.alloc(1);
  cudaCheck(cudaMemsetAsync(trainErrors.ptr, 0, sizeof(uint32_t), s), "memset train errors");
  cudaCheck(cudaMemsetAsync(lossBuf.ptr, 0, 2 * sizeof(float), s), "memset loss");
  for (int it = 0; it < steps; ++it) {
    const size_t first = (size_t)(cursor % cfg.numSamples);
    cursor += (uint64_t)B;
    k_sur_encode_fwd<<<gridFor(B, 128), 128, 0, s>>>(v, table.ptr, samples.ptr, first, cfg.numSamples, B, feats.ptr);
    float *lossSlot = lossBuf.ptr + (it == steps - 1 ? 1 : 0);
    if (it == steps - 1) cudaCheck(cudaMemsetAsync(lossSlot, 0, sizeof(float), s), "memset loss");
    launchMlpTrain(v, feats.ptr, samples.ptr, first, cfg.numSamples, B, view.vmin, 1.f / view.vrange, 1.f / (float)B,
                   gw.ptr, lossSlot, dfeat.ptr, trainErrors.ptr, s);
    k_sur_encode_bwd<<<gridFor(B, 128), 128, 0, s>>>(v, samples.ptr, first, cfg.numSamples, B, dfeat.ptr, gtable.ptr);
    step++;
    const float b1 = 0.9f, b2 = 0.99f;
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)step)));
    // exponential decay from the configured rate to lrFinal over this call
    const double frac = steps > 1 ? (double)it / (double)(steps - 1) : 0.0;
    const float lrT = (float)((double)cfg.lrTable * std::pow((double)cfg.lrFinal / (double)cfg.lrTable, frac));
    const float lrM = (float)((double)cfg.lrMlp * std::pow((double)cfg.lrFinal / (double)cfg.lrMlp, frac));
    k_sur_adam_table<<<gridFor(nTab, 256), 256, 0, s>>>(table.ptr, gtable.ptr, mTable.ptr, vTable.ptr, nTab, lrT, b1,
                                                        b2, c1, c2, 1e-15f, table16.ptr);
    k_sur_adam_mlp<<<gridFor(kSurParams, 256), 256, 0, s>>>(w32.ptr, gw.ptr, mw.ptr, vw.ptr, kSurParams, lrM, b1, b2,
                                                           c1, c2, 1e-15f, wbf.ptr);
    cudaCheck(cudaGetLastError(), "surrogate training step");
    if ((it & 63) == 63) {  // a failed step ends the training early
      uint32_t terr = 0;
      cudaCheck(cudaMemcpyAsync(&terr, trainErrors.ptr, sizeof(terr), cudaMemcpyDeviceToHost, s), "train errors");
      cudaCheck(cudaStreamSynchronize(s), "surrogate training");
      if (terr) throw Error(EXA_ERR_CUDA, "surrogate training: a tensor-core product did not complete");
    }
  }
  float h[2] = {0.f, 0.f};
  uint32_t terr = 0;
  cudaCheck(cudaMemcpyAsync(h, lossBuf.ptr, sizeof(h), cudaMemcpyDeviceToHost, s), "loss");
  cudaCheck(cudaMemcpyAsync(&terr, trainErrors.ptr, sizeof(terr), cudaMemcpyDeviceToHost, s), "train errors");
  cudaCheck(cudaStreamSynchronize(s), "surrogate training");
  if (terr) throw Error(EXA_ERR_CUDA, "surrogate training: a tensor-core product did not complete");
  // mean squared error (normalised units) of the last step's batch
  lastLoss = h[1] / (float)B;
  return lastLoss;
}

void Surrogate::gradients(const float4 *hostSamples, int n, float *gW, float *gTable, float *loss, cudaStream_t s)
{
  // one step's gradients for the given pairs without updating anything
  if (n < 1 || n > cfg.batch) throw Error(EXA_ERR_INVALID, "gradient batch size out of range");
  DBuf<float4> sm;
  sm.upload(hostSamples, (size_t)n, s);
  DBuf<__nv_bfloat16> f;
  f.alloc((size_t)n * kSurIn);
  DBuf<float> df;
  df.alloc((size_t)n * kSurIn);
  DBuf<float> gwl, lossl;
  std::vector<float> z(kSurParams, 0.f);
  gwl.upload(z.data(), z.size(), s);
  float zero = 0.f;
  lossl.upload(&zero, 1, s);
  const size_t nTab = (size_t)kSurLevels << cfg.log2T;
  DBuf<float2> gt;
  gt.alloc(nTab);
  cudaCheck(cudaMemsetAsync(gt.ptr, 0, gt.bytes(), s), "memset");
  const SurrogateView v = deviceView();
  k_sur_encode_fwd<<<gridFor(n, 128), 128, 0, s>>>(v, table.ptr, sm.ptr, 0, (size_t)n, n, f.ptr);
  DBuf<uint32_t> terrBuf;
  terrBuf.alloc(1);
  cudaCheck(cudaMemsetAsync(terrBuf.ptr, 0, sizeof(uint32_t), s), "memset train errors");
  launchMlpTrain(v, f.ptr, sm.ptr, 0, (size_t)n, n, view.vmin, 1.f / view.vrange, 1.f / (float)n, gwl.ptr, lossl.ptr,
                 df.ptr, terrBuf.ptr, s);
  k_sur_encode_bwd<<<gridFor(n, 128), 128, 0, s>>>(v, sm.ptr, 0, (size_t)n, n, df.ptr, gt.ptr);
  cudaCheck(cudaGetLastError(), "surrogate gradients");
  if (gW) cudaCheck(cudaMemcpyAsync(gW, gwl.ptr, kSurParams * sizeof(float), cudaMemcpyDeviceToHost, s), "d2h");
  if (gTable) cudaCheck(cudaMemcpyAsync(gTable, gt.ptr, gt.bytes(), cudaMemcpyDeviceToHost, s), "d2h");
  float l = 0.f;
  uint32_t terr = 0;
  cudaCheck(cudaMemcpyAsync(&l, lossl.ptr, sizeof(float), cudaMemcpyDeviceToHost, s), "d2h");
  cudaCheck(cudaMemcpyAsync(&terr, terrBuf.ptr, sizeof(terr), cudaMemcpyDeviceToHost, s), "d2h");
  cudaCheck(cudaStreamSynchronize(s), "surrogate gradients");
  if (terr) throw Error(EXA_ERR_CUDA, "surrogate gradients: a tensor-core product did not complete");
  if (loss) *loss = l / (float)n;
}

void Surrogate::evaluate(const ExaStitchSampler &sampler, const Grid &grid, double tol, size_t pointsTarget,
                         cudaStream_t s)
{
  const size_t nmc = (size_t)grid.dims.x * grid.dims.y * grid.dims.z;
  if (!nmc) throw Error(EXA_ERR_INVALID, "no majorant grid");
  mcMode.alloc(nmc);
  mcErr.alloc(nmc);
  mcEmpty.alloc(nmc);
  widenedRanges.alloc(nmc);
  majorants.alloc(nmc);
  DBuf<double> sums;
  sums.alloc(2);
  DBuf<unsigned> nsur;
  nsur.alloc(1);
  cudaCheck(cudaMemsetAsync(mcErr.ptr, 0, mcErr.bytes(), s), "memset");
  cudaCheck(cudaMemsetAsync(mcEmpty.ptr, 0, mcEmpty.bytes(), s), "memset");
  cudaCheck(cudaMemsetAsync(sums.ptr, 0, sums.bytes(), s), "memset");
  cudaCheck(cudaMemsetAsync(nsur.ptr, 0, nsur.bytes(), s), "memset");
  int sp = (int)std::floor(std::cbrt((double)pointsTarget / (double)nmc));
  sp = std::max(2, std::min(sp, 16));
  const size_t n = nmc * (size_t)sp * sp * sp;
  int dev = 0, sms = 152;
  cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  const unsigned blocks = (unsigned)std::min<size_t>((n + 127) / 128, (size_t)sms * 8);
  const SurrogateView v = deviceView();
  k_sur_mc_error<<<blocks, 128, 0, s>>>(sampler.accel, v, grid.dims, grid.worldBounds, sp, n, cfg.seed ^ 0xe44,
                                        mcErr.ptr, mcEmpty.ptr, sums.ptr);
  cudaCheck(cudaGetLastError(), "k_sur_mc_error");
  k_sur_widen<<<gridFor(nmc, 256), 256, 0, s>>>(grid.valueRanges.ptr, mcErr.ptr, mcEmpty.ptr, nmc,
                                                tol * (double)view.vrange, mcMode.ptr, widenedRanges.ptr, nsur.ptr);
  cudaCheck(cudaGetLastError(), "k_sur_widen");
  double hs[2];
  unsigned hn = 0;
  cudaCheck(cudaMemcpyAsync(hs, sums.ptr, sizeof(hs), cudaMemcpyDeviceToHost, s), "d2h");
  cudaCheck(cudaMemcpyAsync(&hn, nsur.ptr, sizeof(hn), cudaMemcpyDeviceToHost, s), "d2h");
  std::vector<unsigned long long> errs(nmc);
  cudaCheck(cudaMemcpyAsync(errs.data(), mcErr.ptr, mcErr.bytes(), cudaMemcpyDeviceToHost, s), "d2h");
  cudaCheck(cudaStreamSynchronize(s), "surrogate evaluate");
  double emax = 0.0;
  for (unsigned long long e : errs) {
    double d;
    std::memcpy(&d, &e, sizeof(d));
    emax = std::max(emax, d);
  }
  stats.probePoints = n;
  stats.rmse = hs[1] > 0.0 ? std::sqrt(hs[0] / hs[1]) / (double)view.vrange : 0.0;
  stats.maxError = emax / (double)view.vrange;
  stats.numMacrocells = nmc;
  stats.numSurrogateMCs = hn;
  evalDims = grid.dims;
  evaluated = true;
}

void Surrogate::computeMajorants(const float4 *cmap, int ncolors, exa_range1f xf, int filter, cudaStream_t s)
{
  if (!evaluated) return;
  launchMaxOpacity(widenedRanges.ptr, widenedRanges.count, cmap, ncolors, xf, filter, majorants.ptr, s);
}

size_t Surrogate::inferenceBytes() const
{
  return table16.bytes() + wbf.bytes() + mcMode.bytes() + majorants.bytes();
}

void launchSurrogatePoints(const SurrogateView &S, const exa_vec3f *pos, size_t n, float *out, cudaStream_t s)
{
  if (!n) return;
  int dev = 0, sms = 152;
  cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  const unsigned blocks = (unsigned)std::min<size_t>((n + 127) / 128, (size_t)sms * 8);
  k_sur_points<<<blocks, 128, 0, s>>>(S, pos, n, out);
  cudaCheck(cudaGetLastError(), "k_sur_points");
}

} // namespace exa
