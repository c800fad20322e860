// tma.cuh — inline-PTX helpers for Blackwell bulk asynchronous copies
// (cp.async.bulk, and tiled tensor copies cp.async.bulk.tensor) completed
// through shared-memory mbarriers, per-thread
// cp.async copies and L2 prefetches, with bounded waits.
//
// Every wait gives up after a budget of SM clock cycles (kWaitCycles, about
// 2 s at 2 GHz, unless the caller passes a shorter one); the caller then
// records NS3D_ERR_TIMEOUT in the step status word and returns instead of
// spinning forever. Waits that drain copies still in flight before a CTA
// exits always use the full kWaitCycles.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ns3d {

constexpr long long kWaitCycles = 4000000000LL;
constexpr int kStatusTimeout = 6;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make mbarrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic-proxy shared accesses before later
// async-proxy writes into the same buffer
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// 1D bulk copy global -> shared; dst/src 16-byte aligned, bytes % 16 == 0
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// per-thread asynchronous copy of BYTES (4, 8 or 16) global -> shared; the
// destination is zero-filled past src_bytes (0: nothing is read from src)
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// this thread's copies have landed (visible to this thread)
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// tiled tensor copy global -> shared of one box of a 4D tensor map at
// coordinates (c0 innermost .. c3); c0 x element size must be a multiple of 16
// bytes. The map lives in kernel parameter space (__grid_constant__).
__device__ __forceinline__ void tensor4_g2s(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// tiled tensor copy shared -> global of one box of a 4D tensor map at
// coordinates (c0 innermost .. c3), into the thread's bulk async-group; c0 x
// element size a multiple of 16 bytes and no coordinate negative (elements
// beyond the tensor's extent are not written). The shared source is read
// asynchronously: the writes into it must be ordered before the copy with
// fence_proxy_async_smem and a barrier.
__device__ __forceinline__ void tensor4_s2g(const CUtensorMap* map, const void* src, int c0, int c1, int c2, int c3) {
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(src))
                 : "memory");
}
// close the thread's current bulk async-group
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the thread's bulk async-groups have finished reading their shared sources
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the thread's bulk async-groups have completed (writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// bulk prefetch of global bytes into L2; src 16-byte aligned, bytes % 16 == 0
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// non-blocking test of phase `parity`
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// budgets below this are checked with non-blocking tests only: try_wait may
// suspend the thread for a hardware-defined time, longer than such a budget
constexpr long long kShortBudget = 100000;

// bounded wait on phase `parity`; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long budget = kWaitCycles) {
    if (budget < kShortBudget) {
        const long long t0 = clock64();
        do {
            if (mbar_test_wait(bar, parity)) return true;
        } while (clock64() - t0 <= budget);
        return false;
    }
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > budget) return false;
    }
    return true;
}

}  // namespace ns3d
