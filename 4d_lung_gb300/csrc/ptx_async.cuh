// ptx_async.cuh -- inline-PTX wrappers for the asynchronous copy engine
// (cp.async.bulk / cp.async.bulk.tensor between global and shared memory,
// mbarrier completion for loads, bulk async-groups for stores) used by the
// pipelined FFT passes on sm_103a.
#pragma once
#include <stdint.h>
#include "cgs_common.cuh"

namespace cgs {

CGS_D uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

CGS_D void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

CGS_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// arrive once and add `bytes` to the transaction count of the current phase
CGS_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

CGS_D bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

CGS_D uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase with the given parity; gives up after `limit_ns`
// nanoseconds and returns false (the caller reports the timeout).
CGS_D bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

// Contiguous bulk copy global -> shared (both 16-byte aligned, bytes a
// multiple of 16), completion counted on `bar`.
CGS_D void bulk_load(void* dst_smem, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// 4-D tensor-map tile load (TMA) into shared memory, completion on `bar`.
// Coordinates are element indices, innermost first.
CGS_D void tma_load_4d(void* dst_smem, const void* tmap, int c0, int c1, int c2, int c3, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(
            smem_addr(dst_smem)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}

// 3-D tensor-map tile load (TMA) into shared memory, completion on `bar`.
CGS_D void tma_load_3d(void* dst_smem, const void* tmap, int c0, int c1, int c2, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_addr(dst_smem)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}

// 4-D tensor-map tile store (TMA) from shared memory, tracked by the
// thread's bulk async-group (commit with bulk_commit, wait with
// bulk_wait_read / bulk_wait_all).  The shared-memory writes it reads must be
// made visible to the async proxy first (fence_proxy_async_smem).
CGS_D void tma_store_4d(const void* tmap, int c0, int c1, int c2, int c3, const void* src_smem)
{
    asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];" ::"l"(
                     tmap),
                 "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(src_smem))
                 : "memory");
}

CGS_D void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory sources of all committed bulk stores have been read
CGS_D void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// all committed bulk stores have completed
CGS_D void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
CGS_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace cgs
