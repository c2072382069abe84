// tcgen05.cuh — the 5th-generation tensor-core primitives used by the product
// kernels (sm_100 family): TMEM allocation, shared-memory matrix descriptors,
// kind::f16 MMAs with FP32 accumulation in TMEM, commit to an mbarrier, and
// TMEM loads.  Operands are K-major without swizzle: the shared-memory image
// of a tile is a grid of core matrices of 8 rows x 16 bytes, 128 bytes each,
// with a fixed byte stride between core matrices along K (lbo) and between
// 8-row groups (sbo).
#pragma once
#include <cstdint>

namespace dqmc {
namespace tc {

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// matrix descriptor: start address, lbo and sbo in 16-byte units, descriptor version 1
__device__ __forceinline__ uint64_t desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: BF16 A and B (both K-major), FP32 D, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(unsigned long long* mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(mbar)));
}
// an mbarrier whose phase completes after `count` plain arrivals
__device__ __forceinline__ void mbar_init_n(unsigned long long* mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(mbar)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;"); }
// one arrival (release: this thread's earlier writes are visible to a thread that waits on the phase)
__device__ __forceinline__ void mbar_arrive(unsigned long long* mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(mbar)) : "memory");
}

// waits for completion of the mbarrier phase with this parity; false after `limit` tries
__device__ __forceinline__ bool mbar_wait(unsigned long long* mbar, unsigned parity, int limit = 1 << 24) {
  unsigned done = 0;
  for (int it = 0; it < limit && !done; ++it)
    asm volatile(
        "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(done)
        : "r"(su32(mbar)), "r"(parity)
        : "memory");
  return done != 0;
}

// arm the mbarrier for `bytes` of bulk copies (this thread's arrival counts as the one expected)
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* mbar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(mbar)), "r"(bytes) : "memory");
}
// bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) global -> shared,
// completing on the mbarrier's transaction count
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   su32(dst)),
               "l"(src), "r"(bytes), "r"(su32(mbar))
               : "memory");
}

// one warp: allocate ncols TMEM columns (power of two >= 32), address into *dst
__device__ __forceinline__ void alloc(unsigned* dst, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(dst)), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] B[smem]^T, one thread
__device__ __forceinline__ void mma(unsigned dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accum) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.u32 q, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum ? 1u : 0u));
}
// the mbarrier completes once all earlier MMAs of this thread have finished
__device__ __forceinline__ void commit(unsigned long long* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(mbar)));
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32 (w % 4) + 0..31)
__device__ __forceinline__ void ld16(uint32_t (&v)[16], unsigned taddr) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
// 8 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void ld8(uint32_t (&v)[8], unsigned taddr) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}
template <int W>
__device__ __forceinline__ void ldw(uint32_t (&v)[W], unsigned taddr) {
  if constexpr (W == 16) ld16(v, taddr);
  else ld8(v, taddr);
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace tc
}  // namespace dqmc
