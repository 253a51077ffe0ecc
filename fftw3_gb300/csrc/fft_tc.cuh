/*
 * tcgen05 (5th-generation tensor core) building blocks, inline PTX.
 *
 * Used by the split-FP16 tensor-core form of the radix-16 stages: each
 * radix-16 butterfly is one row of a GEMM
 *     D[m][0..31] = A[m][0..95] . B[0..31][0..95]^T
 * with A = the butterfly's 16 complex inputs split into FP16 hi and lo parts
 * ([x_hi.re | x_hi.im | x_lo.re | x_lo.im | x_hi.re | x_hi.im]) and B the
 * real form of the 16-point DFT matrix, split the same way
 * ([F_hi | F_hi | F_lo] against those blocks), so that
 *     D = F_hi x_hi + F_hi x_lo + F_lo x_hi   (FP32 accumulation)
 * recovers the DFT to ~2^-22 relative per stage; D's columns are the 16
 * real then the 16 imaginary outputs.
 *
 * Operands live in shared memory in the canonical K-major layout without
 * swizzle: 8 rows x 16 bytes per core matrix, core matrices adjacent along
 * M (or N) SBO bytes apart and adjacent along K LBO bytes apart.  The
 * accumulator lives in tensor memory (TMEM): row m -> lane m, column n ->
 * column n.
 */
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace gb {
namespace tc {

/* shared-memory matrix descriptor (64 bit) */
__host__ __device__ constexpr uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
     return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
            ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46) /* version */ |
            ((uint64_t)0 << 61) /* no swizzle */;
}

/* instruction descriptor, kind::f16: D f32, A and B f16, both K-major */
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
     return (1u << 4) /* D = F32 */ | (0u << 7) /* A = F16 */ | (0u << 10) /* B = F16 */ |
            ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* byte offset of element (row, k) of a K-major f16 operand in the
 * canonical no-swizzle layout with core matrices contiguous along rows
 * (SBO = 128) and K-chunks of 8 elements lbo bytes apart */
__host__ __device__ constexpr uint32_t kmajor_off(int row, int k, uint32_t lbo)
{
     return (uint32_t)(k >> 3) * lbo + (uint32_t)(row >> 3) * 128u + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* TMEM allocation: executed by one whole warp; writes the TMEM base address
 * to *dst (shared memory) */
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
     asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
                  : "memory");
     asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
     asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

/* D (+)= A . B^T, one instruction of K = 16 (issued by a single thread) */
__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
     asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                  ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
                  : "memory");
}

/* arrive on an mbarrier when all earlier MMAs of this thread completed */
__device__ __forceinline__ void mma_commit(unsigned long long *bar)
{
     asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                  : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* 32 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes
 * 32*(w%4) .. +31; taddr carries lane << 16 | column) */
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
     uint32_t r[32];
     asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                  "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                  "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                  : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                    "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                    "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                    "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                  : "r"(taddr)
                  : "memory");
     asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
     for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

} /* namespace tc */
} /* namespace gb */
