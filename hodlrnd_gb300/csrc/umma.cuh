// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a: tensor
// memory allocation, shared-memory matrix descriptors, the BF16 MMA with FP32
// accumulation in tensor memory, its completion on an mbarrier, and loads of
// the accumulator back to registers.  Inline PTX (PTX ISA 8.7+, tcgen05).
//
// Operand layout used throughout (no swizzle, K-major): a tile of R rows and
// K columns of BF16 is stored as "core matrices" of 8 rows x 16 bytes (8
// elements along K), each 128 contiguous bytes with row r of the core matrix
// at byte 16 r.  Core matrix (rg, kg) -- rows 8 rg .. 8 rg + 7, columns
// 8 kg .. 8 kg + 7 -- starts at byte (rg * KG + kg) * 128, KG = K / 8, so the
// descriptor's leading-dimension byte offset (between core matrices along K)
// is 128 and its stride-dimension byte offset (between 8-row groups) is
// KG * 128.  One MMA of kind::f16 consumes K = 16: the k-th step starts at
// byte 256 k of the tile.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "bulk.cuh"

namespace hodlr {

// byte offset of element (r, k) of a K-major no-swizzle BF16 tile with KG
// core matrices along K
__host__ __device__ __forceinline__ uint32_t umma_kmajor_offset(uint32_t r, uint32_t k, uint32_t KG) {
  return ((r >> 3) * KG + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all >> 4), descriptor version 1 (bits 46-47), base offset 0,
// relative leading-dimension mode, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t umma_desc(const void* smem, uint32_t lbo, uint32_t sbo) {
  uint64_t d = uint64_t((smem_addr(smem) >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// Tensor memory: ncols (a power of two, 32 .. 512) columns of all 128 lanes,
// allocated by one whole warp; the address is written to *slot (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D (tensor memory) = A B^T (+ D when accumulate != 0); A: M x 16, B: N x 16
// (BF16, shared memory, by descriptor).  Issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// The mbarrier receives one arrival once every MMA this thread issued before
// has completed (and its shared-memory operands may be overwritten).
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// 16 consecutive FP32 columns of the 32 tensor-memory lanes of this warp
// (warp w % 4 of the CTA reads lanes 32 (w % 4) .. + 31; lane l gets row
// 32 (w % 4) + l).  taddr: lane base in bits 16-31, column in bits 0-15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

// BF16 bits of an FP32 value, rounded to nearest even
__device__ __forceinline__ uint16_t bf16_bits(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ __forceinline__ float bf16_value(uint16_t b) { return __uint_as_float(uint32_t(b) << 16); }
// An FP32 value as two BF16 words packed in 32 bits: the value rounded to
// BF16 in the low half-word, the rounded remainder in the high half-word.
__device__ __forceinline__ uint32_t split_pack(float v) {
  const uint16_t h = bf16_bits(v);
  return uint32_t(h) | (uint32_t(bf16_bits(v - bf16_value(h))) << 16);
}

}  // namespace hodlr
