// exa_surrogate.cuh -- the learned stand-in for the ExaStitch field: a
// multiresolution hash-grid encoding (Mueller et al. 2022, "Instant neural
// graphics primitives with a multiresolution hash encoding") feeding a small
// MLP (32 -> 64 -> 64 -> 1, ReLU, no biases) whose products run on the
// tensor cores as BF16 x BF16 -> FP32 warp MMAs.
//
// Precision contract (the CPU oracle restates it):
//   x   = clamp((pos - lo) * inv, 0, 1) per axis
//   per level l: p = x * res_l, cell c = clamp(floor(p), 0, res_l - 1),
//     f = clamp(p - c, 0, 1); corners k = 0..7 (bit 0 x, bit 1 y, bit 2 z),
//     weight ((wx * wy) * wz) with w = f or 1 - f; index dense when
//     (res_l + 1)^3 <= T, else (x * 1 ^ y * 2654435761 ^ z * 805459861) mod T
//   feat[2l + j] = sum over corners in order k of weight * table[l][idx].j
//   a0 = bf16(feat); h1 = bf16(relu(W1 a0)); h2 = bf16(relu(W2 h1)) with FP32
//   accumulation; y = sum_j h2[j] * w3[j]; value = vmin + y * vrange.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "exa_device.cuh"

namespace exa {

constexpr int kSurLevels = 16;
constexpr int kSurIn = 2 * kSurLevels;  // MLP inputs
constexpr int kSurHidden = 64;
// shared-memory row strides (bf16 elements), padded by 8 so that the
// fragment loads of one MMA hit distinct banks
constexpr int kSurLdIn = kSurIn + 8;       // 40
constexpr int kSurLdHid = kSurHidden + 8;  // 72

struct SurrogateView {
  const __half2 *table;       // [levels][T] feature pairs (inference copy)
  const __nv_bfloat16 *w1;    // [64][32] (out, in)
  const __nv_bfloat16 *w2;    // [64][64]
  const __nv_bfloat16 *w3;    // [64]
  const uint8_t *mcMode;      // per macrocell: 1 surrogate, 0 exact sampler
  int levels, log2T;
  uint32_t denseMask;         // bit l: level l is indexed densely
  int res[kSurLevels];
  float lo[3], inv[3];
  float vmin, vrange;
};

EXA_HD float sur_clamp01(float v) { return v < 0.f ? 0.f : (v > 1.f ? 1.f : (v == v ? v : 0.f)); }

EXA_HD uint32_t sur_index(int res, int log2T, bool dense, uint32_t x, uint32_t y, uint32_t z)
{
  if (dense) {
    const uint32_t side = (uint32_t)res + 1u;
    return x + side * (y + side * z);
  }
  return (x * 1u ^ y * 2654435761u ^ z * 805459861u) & ((1u << log2T) - 1u);
}

// cell and in-cell fraction of level l along one axis
EXA_HD void sur_axis(float x, int res, int &c, float &f)
{
  const float p = x * (float)res;
  int ci = (int)floorf(p);
  ci = ci < 0 ? 0 : (ci > res - 1 ? res - 1 : ci);
  c = ci;
  f = sur_clamp01(p - (float)ci);
}

EXA_HD V3 sur_normalize(const SurrogateView &S, V3 pos)
{
  return mk3(sur_clamp01((pos.x - S.lo[0]) * S.inv[0]), sur_clamp01((pos.y - S.lo[1]) * S.inv[1]),
             sur_clamp01((pos.z - S.lo[2]) * S.inv[2]));
}

// the eight corners of level l: index and weight, in corner order
EXA_HD void sur_corners(const SurrogateView &S, int l, V3 x, uint32_t idx[8], float w[8])
{
  int cx, cy, cz;
  float fx, fy, fz;
  const int r = S.res[l];
  sur_axis(x.x, r, cx, fx);
  sur_axis(x.y, r, cy, fy);
  sur_axis(x.z, r, cz, fz);
  const bool dense = (S.denseMask >> l) & 1u;
  for (int k = 0; k < 8; ++k) {
    const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
    const float wx = dx ? fx : 1.f - fx;
    const float wy = dy ? fy : 1.f - fy;
    const float wz = dz ? fz : 1.f - fz;
    w[k] = (wx * wy) * wz;
    idx[k] = sur_index(r, S.log2T, dense, (uint32_t)(cx + dx), (uint32_t)(cy + dy), (uint32_t)(cz + dz));
  }
}

#ifdef __CUDACC__

// 16x8x16 BF16 MMA with FP32 accumulate (PTX ISA, mma.sync.aligned.m16n8k16)
EXA_D void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

EXA_D uint32_t lds32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// A fragment (16x16, row-major tile at A with row stride lda, rows m0..,
// columns k0..): lane = 4 * group + t holds rows group, group + 8 and
// columns 2t, 2t + 1, 2t + 8, 2t + 9
EXA_D void frag_a(uint32_t (&a)[4], const __nv_bfloat16 *A, int lda, int m0, int k0, int lane)
{
  const int g = lane >> 2, t = lane & 3;
  const __nv_bfloat16 *p = A + (m0 + g) * lda + k0 + 2 * t;
  a[0] = lds32(p);
  a[1] = lds32(p + 8 * lda);
  a[2] = lds32(p + 8);
  a[3] = lds32(p + 8 * lda + 8);
}

// B fragment (16x8, k by n) read from Bt, the n-major transpose (Bt[n][k],
// row stride ldb): lane holds k = 2t, 2t + 1 and 2t + 8, 2t + 9 of column
// n = group
EXA_D void frag_b(uint32_t (&b)[2], const __nv_bfloat16 *Bt, int ldb, int n0, int k0, int lane)
{
  const int g = lane >> 2, t = lane & 3;
  const __nv_bfloat16 *p = Bt + (n0 + g) * ldb + k0 + 2 * t;
  b[0] = lds32(p);
  b[1] = lds32(p + 8);
}

EXA_D float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// shared-memory copy of the network (one per block)
struct alignas(16) SurWeightsSmem {
  __nv_bfloat16 w1[kSurHidden * kSurLdIn];   // [64][40]
  __nv_bfloat16 w2[kSurHidden * kSurLdHid];  // [64][72]
  float w3[kSurHidden];
};

// per-warp scratch of the inference
struct alignas(16) SurWarpSmem {
  __nv_bfloat16 a[32 * kSurLdIn];    // encoded inputs, one row per lane
  __nv_bfloat16 h1[32 * kSurLdHid];  // first hidden layer
};

EXA_D void sur_load_weights(SurWeightsSmem &W, const SurrogateView &S)
{
  for (int i = threadIdx.x; i < kSurHidden * kSurIn; i += blockDim.x)
    W.w1[(i / kSurIn) * kSurLdIn + (i % kSurIn)] = S.w1[i];
  for (int i = threadIdx.x; i < kSurHidden * kSurHidden; i += blockDim.x)
    W.w2[(i / kSurHidden) * kSurLdHid + (i % kSurHidden)] = S.w2[i];
  for (int i = threadIdx.x; i < kSurHidden; i += blockDim.x) W.w3[i] = __bfloat162float(S.w3[i]);
}

// encoding of one position from the FP16 inference table, as BF16 pairs
// into row[0..15] (zeros when !want)
EXA_D void sur_encode_row(const SurrogateView &S, V3 pos, bool want, uint32_t *row)
{
  const V3 x = sur_normalize(S, pos);
  const size_t T = (size_t)1 << S.log2T;
#pragma unroll 2
  for (int l = 0; l < kSurLevels; ++l) {
    float f0 = 0.f, f1 = 0.f;
    if (want) {
      uint32_t idx[8];
      float w[8];
      sur_corners(S, l, x, idx, w);
      const __half2 *tab = S.table + (size_t)l * T;
      __half2 e[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) e[k] = __ldg(tab + idx[k]);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float2 v = __half22float2(e[k]);
        f0 += w[k] * v.x;
        f1 += w[k] * v.y;
      }
    }
    const __nv_bfloat162 v = __floats2bfloat162_rn(f0, f1);
    row[l] = *reinterpret_cast<const uint32_t *>(&v);
  }
}

// Warp-collective surrogate evaluation: every lane calls it (all 32 lanes
// converged); lanes with want set get the normalised field value y of their
// position.  Rows of lanes without want are zero.
EXA_D float sur_eval_warp(const SurrogateView &S, const SurWeightsSmem &W, SurWarpSmem &ws, V3 pos, bool want)
{
  const int lane = threadIdx.x & 31;
  sur_encode_row(S, pos, want, reinterpret_cast<uint32_t *>(ws.a + lane * kSurLdIn));
  __syncwarp();
  const int g = lane >> 2, t = lane & 3;
  // layer 1: h1 = bf16(relu(a W1^T)), 32 x 64
  for (int mt = 0; mt < 2; ++mt)
    for (int nt = 0; nt < kSurHidden / 8; ++nt) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kt = 0; kt < kSurIn / 16; ++kt) {
        uint32_t a[4], b[2];
        frag_a(a, ws.a, kSurLdIn, mt * 16, kt * 16, lane);
        frag_b(b, W.w1, kSurLdIn, nt * 8, kt * 16, lane);
        mma16816(d, a, b);
      }
      const int r = mt * 16 + g, c = nt * 8 + 2 * t;
      *reinterpret_cast<__nv_bfloat162 *>(ws.h1 + r * kSurLdHid + c) =
          __floats2bfloat162_rn(fmaxf(d[0], 0.f), fmaxf(d[1], 0.f));
      *reinterpret_cast<__nv_bfloat162 *>(ws.h1 + (r + 8) * kSurLdHid + c) =
          __floats2bfloat162_rn(fmaxf(d[2], 0.f), fmaxf(d[3], 0.f));
    }
  __syncwarp();
  // layer 2 and the output layer: y = sum_j bf16(relu(h1 W2^T))_j w3_j
  float y = 0.f;
  for (int mt = 0; mt < 2; ++mt) {
    float plo = 0.f, phi = 0.f;  // rows mt*16 + g and + 8, columns of this lane
    for (int nt = 0; nt < kSurHidden / 8; ++nt) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kt = 0; kt < kSurHidden / 16; ++kt) {
        uint32_t a[4], b[2];
        frag_a(a, ws.h1, kSurLdHid, mt * 16, kt * 16, lane);
        frag_b(b, W.w2, kSurLdHid, nt * 8, kt * 16, lane);
        mma16816(d, a, b);
      }
      const int c = nt * 8 + 2 * t;
      plo += bf16_round(fmaxf(d[0], 0.f)) * W.w3[c] + bf16_round(fmaxf(d[1], 0.f)) * W.w3[c + 1];
      phi += bf16_round(fmaxf(d[2], 0.f)) * W.w3[c] + bf16_round(fmaxf(d[3], 0.f)) * W.w3[c + 1];
    }
    plo += __shfl_xor_sync(0xffffffffu, plo, 1);
    plo += __shfl_xor_sync(0xffffffffu, plo, 2);
    phi += __shfl_xor_sync(0xffffffffu, phi, 1);
    phi += __shfl_xor_sync(0xffffffffu, phi, 2);
    // row r of this m tile sits in lanes 4 * (r & 7) (low half) / + 8
    const float vlo = __shfl_sync(0xffffffffu, plo, (lane & 7) * 4);
    const float vhi = __shfl_sync(0xffffffffu, phi, (lane & 7) * 4);
    if ((lane >> 4) == mt) y = ((lane >> 3) & 1) ? vhi : vlo;
  }
  __syncwarp();
  return y;
}

#endif  // __CUDACC__

} // namespace exa
