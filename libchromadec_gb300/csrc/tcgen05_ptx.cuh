// tcgen05_ptx.cuh -- inline-PTX wrappers for the 5th-generation tensor cores
// (sm_103a) shared by the tensor-core kernels: shared-memory matrix and
// instruction descriptors, tcgen05.mma issue and commit, mbarrier waits with
// an iteration limit, tensor-memory allocation and loads, and the
// no-swizzle K-major operand layout.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tpal {
namespace tc {

// Iterations of an mbarrier wait before it gives up (the caller then flags
// an error and leaves; no wait is expected to run out).
constexpr unsigned kWaitLimit = 1u << 22;

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading byte offset 128
// (K-adjacent core matrices), stride byte offset sbo (8-row groups), version
// 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
           (1ull << 46);
}

// instruction descriptor: FP32 accumulator, A/B format (TF32 = 2 for
// kind::tf32, BF16 = 1 for kind::f16), both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc(int fmt, int M, int N)
{
    return (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
    if (KIND == 0) {
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
                     "l"(a), "l"(b), "r"(id), "r"(acc));
    } else {
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
                     "l"(a), "l"(b), "r"(id), "r"(acc));
    }
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// A barrier whose phase completes after `count` arrivals (and the expected
// transaction bytes).
__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count = 1)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void bar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Wait for the barrier's phase `parity` to complete; false if the limit ran out.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_addr(bar);
    // kept rolled: the wait is inlined at every call site, and unrolled
    // copies made up a third of the mask network kernel's code
#pragma unroll 1
    for (unsigned it = 0; it < kWaitLimit; it++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
                     "selp.b32 %0, 1, 0, P1;\n\t}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

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

// 16 consecutive 32-bit columns of this thread's lane (the warp reads lanes
// 32 w .. 32 w + 31), then wait for the load
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

// ---------------------------------------------------------------------------
// Operand layout and splitting
// ---------------------------------------------------------------------------
// Byte offset of element k of row r in a K-major no-swizzle operand whose rows
// hold row_bytes of K.
__host__ __device__ __forceinline__ uint32_t elem_off(int r, int k, int eb, int row_bytes)
{
    const int kb = k * eb;
    return (uint32_t)((r >> 3) * (8 * row_bytes) + (kb >> 4) * 128 + (r & 7) * 16 + (kb & 15));
}


// Expect `bytes` of asynchronous copies on the barrier and arrive once.
__device__ __forceinline__ void bar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Bulk copy global -> shared by the TMA engine (both addresses 16-byte
// aligned, bytes a multiple of 16), completing `bytes` on the barrier.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// 16 consecutive 32-bit columns of this thread's lane into r, without
// waiting: the registers are valid after tmem_wait_ld.
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
}

// 8 consecutive 32-bit columns of this thread's lane into r, without waiting.
__device__ __forceinline__ void tmem_ld8_async(uint32_t taddr, uint32_t *r)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

// Wait for this thread's tensor-memory loads. The "+r" operands tie the
// registers being loaded to the wait, so no use of them moves above it; no
// memory clobber (it orders no shared or global access), so ordinary loads
// and stores may be scheduled across it.
template <int N>
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[N])
{
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < N; j++) asm volatile("" : "+r"(r[j]));
}

// Zero 16 consecutive 32-bit columns of this thread's lane (no wait: the
// caller issues tmem_wait_st before the columns are used).
__device__ __forceinline__ void tmem_zero16(uint32_t taddr)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
                 "{%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr),
                 "r"(0u)
                 : "memory");
}

// Zero 8 consecutive 32-bit columns of this thread's lane (no wait; tensor
// memory only, so no memory clobber: the tcgen05 instructions keep their
// order among themselves).
__device__ __forceinline__ void tmem_zero8(uint32_t taddr)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr),
                 "r"(0u));
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// 8 consecutive 32-bit columns of this thread's lane, then wait for the load
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = __uint_as_float(r[j]);
}

}  // namespace tc
}  // namespace tpal
