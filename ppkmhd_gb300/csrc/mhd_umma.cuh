// Fifth-generation tensor-core primitives (tcgen05, sm_100a / sm_103a) used
// by the flux surrogate: TMEM allocation, shared-memory matrix descriptors,
// the BF16 x BF16 -> FP32 MMA with its accumulator in TMEM, completion
// through an mbarrier, and TMEM -> register loads.  All inline PTX; one CTA
// (cta_group::1), M = 128 rows: row r of the tile lives in TMEM lane r, and
// the warp w of a 128-thread block reads lanes 32w..32w+31.
//
// Operands are stored in shared memory in the K-major canonical layout
// without swizzle: an R x K bf16 matrix is a grid of "core matrices" of
// 8 rows x 16 bytes (8 elements of K), each core matrix 128 contiguous bytes:
//   byte offset(r, k) = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (core matrices adjacent in K) and SBO = K * 16 (adjacent
// 8-row groups).  One MMA consumes K = 16, i.e. two core matrices along K:
// the descriptor of K-step s starts 2 * LBO * s bytes further.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace mhd
{
namespace umma
{

constexpr uint32_t kLBO = 128;

__host__ __device__ constexpr uint32_t
canon_offset(int r, int k, int K)
{
  return (uint32_t)((r / 8) * (K * 16) + (k / 8) * (int)kLBO + (r % 8) * 16 + (k % 8) * 2);
}

// Instruction descriptor of tcgen05.mma .kind::f16: D F32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0),
// N / 8 in bits 17-22, M / 16 in bits 24-28.
__host__ __device__ constexpr uint32_t
idesc_bf16_f32(int m, int n)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t
smem_addr(const void * p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (no swizzle): start address, LBO and SBO
// in 16-byte units (bits 0-13, 16-29, 32-45), the fixed value 0b001 at bits
// 46-48, base offset 0, relative LBO mode, swizzle mode 0.
__device__ __forceinline__ uint64_t
desc_kmajor(uint32_t saddr, uint32_t sbo)
{
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kLBO >> 4) << 16) |
         ((uint64_t)(sbo >> 4) << 32) | ((uint64_t)1 << 46);
}

// TMEM allocation of ncols columns (a power of two >= 32) by one whole warp;
// the base address is written to the shared word at slot.
__device__ __forceinline__ void
tmem_alloc(uint32_t slot, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void
tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// D[tmem] (+)= A[adesc] * B[bdesc]^T, issued by one thread.
__device__ __forceinline__ void
mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
               "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
               : "memory");
}

// Arrive on the mbarrier when every MMA issued so far by this thread is done.
__device__ __forceinline__ void
commit(uint32_t mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                 mbar)
               : "memory");
}

__device__ __forceinline__ void
mbar_init(uint32_t mbar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for the phase with the given parity to complete, at most `limit`
// polls; false when the limit was reached.
__device__ __forceinline__ bool
mbar_wait(uint32_t mbar, uint32_t parity, int limit)
{
  uint32_t done = 0;
  for (int it = 0; it < limit && !done; ++it)
    asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}\n"
                 : "=r"(done)
                 : "r"(mbar), "r"(parity)
                 : "memory");
  return done != 0;
}

// Ordering of tcgen05 operations across thread barriers, and of generic
// shared-memory stores before tensor-core reads.
__device__ __forceinline__ void
fence_before_sync()
{
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void
fence_after_sync()
{
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void
fence_proxy_async()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk prefetch of [p, p + bytes) from global memory into L2 by the TMA
// engine (one instruction, no completion to wait for).  p 16-byte aligned,
// bytes a multiple of 16, the range inside one allocation.
__device__ __forceinline__ void
bulk_prefetch_l2(const void * p, uint32_t bytes)
{
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane (shape 32x32b);
// the warp's lane quarter is in bits 16-31 of taddr.
__device__ __forceinline__ void
ld32(uint32_t taddr, uint32_t (&v)[32])
{
  // the load and its wait in one statement: the registers are only read
  // after tcgen05.wait::ld
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
               "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
               "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
               "tcgen05.wait::ld.sync.aligned;"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                 "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                 "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
                 "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
                 "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                 "=r"(v[30]), "=r"(v[31])
               : "r"(taddr)
               : "memory");
}

#endif // __CUDACC__

} // namespace umma
} // namespace mhd
