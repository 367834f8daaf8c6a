// exa_tcgen05.cuh -- the 5th-generation tensor core (tcgen05) in inline PTX:
// tensor-memory allocation, BF16 x BF16 -> FP32 matrix products with both
// operands in shared memory and the accumulator in tensor memory, commits
// to an mbarrier and tensor-memory loads (PTX ISA, "Tensor Core 5th
// Generation Family Instructions").
//
// Operand layout: K-major without swizzle.  A tile of R rows by K bf16
// elements (K a multiple of 16) is stored as 8 x 8-element core matrices of
// 128 contiguous bytes (row r of a core matrix at byte 16 r); the core
// matrices of one 8-row group are adjacent along K (leading byte offset
// 128), the 8-row groups (K / 8) * 128 bytes apart (stride byte offset).
// One MMA consumes 16 K elements, the next starts 256 bytes further.
#pragma once

#include <cstdint>

#include "exa_device.cuh"

namespace exa {
namespace tc {

// element offset of (row, k) in a K-major tile with K columns
EXA_HD int kmajor(int row, int k, int K) { return ((row >> 3) * (K >> 3) + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7); }

EXA_D uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all in 16-byte units), the fixed version bits 46-48 = 0b001, base
// offset 0, relative leading offset, no swizzle
EXA_D uint64_t desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | ((uint64_t)1 << 46);
}

// descriptor of the 16-wide K slice kk of a K-major tile with K columns
EXA_D uint64_t desc_kslice(const void *tile, int K, int kk)
{
  return desc(smem_addr(tile) + (uint32_t)kk * 256u, 128u, (uint32_t)(K / 8) * 128u);
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major;
// M 128 needs N a multiple of 16 in [16, 256]
EXA_HD constexpr uint32_t idesc_bf16_f32(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// tensor memory: one warp allocates `cols` columns (a power of two >= 32)
// and writes the address to *slot
EXA_D void tmem_alloc(uint32_t *slot, uint32_t cols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

EXA_D void tmem_dealloc(uint32_t taddr, uint32_t cols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// D (tensor memory) = A * B^T (+ D when accumulate), one thread issues
EXA_D void mma_bf16(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
      "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// the mbarrier's phase completes when this thread's earlier MMAs have
EXA_D void commit(uint64_t *bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// mbarrier phase test (the barrier's phase of the given parity completed)
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

// the global nanosecond timer (bounds waits in time)
EXA_D uint64_t globaltimer_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

EXA_D void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
EXA_D void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive 32-bit columns of this thread's lane (the warp reads its
// 32-lane quarter of tensor memory: lanes 32 (warp % 4) ...)
EXA_D void ld16(uint32_t taddr, float (&v)[16])
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace exa
