// Inline-PTX helpers for the fifth-generation tensor cores of sm_100-family
// GPUs: tiled TMA loads through a tensor map, tcgen05 MMAs whose fp32
// accumulators live in tensor memory (TMEM), TMEM loads, and bulk
// reductions from shared to global memory.  Only this CTA's own shared
// memory is addressed (no cluster multicast).
//
// Shared-memory operand layout: K-major tiles written by TMA with the 64-byte
// swizzle, i.e. rows of 32 fp16 (64 bytes), 8-row groups of 512 bytes, each
// tile starting on a 1024-byte boundary.
#pragma once
#include <cstdint>
#include <cuda.h>

#include "frmc_ptx.cuh"

namespace frmc {

// ------------------------------------------------------------------ TMA
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// dst[0, bytes / 4) += src[0, bytes / 4) in fp32, performed in L2 (both
// addresses 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_reduce_add_f32(float *dst, const void *src, uint32_t bytes)
{
    asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;" ::"l"(dst),
                 "r"(smem_addr(src)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit_group() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// wait until at most N of this thread's bulk groups still read shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// wait until at most N of this thread's bulk groups are incomplete
template <int N>
__device__ __forceinline__ void bulk_wait()
{
    asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}

// order this thread's completed async-proxy global writes before its later
// generic-proxy accesses (and the releases that follow them)
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// -------------------------------------------------------- tensor memory
// Allocate ncols (a power of two >= 32) TMEM columns for this CTA; the base
// address is written to *dst.  One whole warp executes it.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with the 64-byte swizzle: start address, stride between 8-row groups (512
// bytes), descriptor version 1, swizzle mode 4 (64 bytes).  The leading
// offset is unused by swizzled K-major layouts.
__device__ __forceinline__ uint64_t sdesc_k_sw64(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(512u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)4 << 61;
    return d;
}

// Instruction descriptor of kind::f16: fp16 A and B, both K-major, fp32
// accumulators, M = 128 rows, N columns (a multiple of 16, at most 256).
__host__ __device__ constexpr uint32_t idesc_f16_m128(uint32_t n)
{
    return (1u << 4) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

// D[tmem] = A B^T (+ D when accumulate), issued by one thread.
__device__ __forceinline__ void tc_mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                           uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier receives one arrival once every tcgen05 operation this thread
// issued before has completed.
__device__ __forceinline__ void tc_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 8 consecutive 32-bit columns of the warp's 32 TMEM lanes (lane = thread).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ------------------------------------------------------ bounded waits
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the mbarrier phase of the given parity, at most `limit_ns`; on
// time-out raise DS_BARRIER_TIMEOUT in *status and return false.
__device__ __forceinline__ bool mbar_wait_ns(uint64_t *bar, uint32_t parity, unsigned long long limit_ns,
                                             uint32_t *status)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity))
            return true;
        if (global_ns() - t0 > limit_ns)
            break;
    }
    if (status)
        atomicOr(status, DS_BARRIER_TIMEOUT);
    return false;
}

}  // namespace frmc
