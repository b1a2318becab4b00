// mbarrier and 1-D bulk-copy (TMA) helpers shared by the kernels that stream
// j tiles into shared memory: the single-system mixed tiled kernels and the
// ensemble's block-tiled items.
#pragma once
#include <stdint.h>

namespace h4 {
namespace tma {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes the barrier initialisation visible to the async proxy (the bulk copies).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// One arrival on `bar` (no transaction bytes): a consumer releasing a stage.
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later bulk copies into it (a buffer is refilled after it was read).
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 1-D bulk copy global -> shared, completion counted on `bar` (16-byte
// aligned addresses, size a multiple of 16).
__device__ __forceinline__ void load_1d(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Bounded wait for the phase of `bar` with the given parity; false when it
// gave up after `limit` polls.
__device__ __forceinline__ bool wait_bounded(uint64_t *bar, unsigned parity, unsigned limit) {
    unsigned spins = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (++spins > limit) return false;
    }
    return true;
}

// Double-buffered tile ring: tile number gt (counted per block) lives in
// buffer gt & 1 and completes phase gt >> 1 of that buffer's barrier.
// Timeout path: before the block leaves, wait (bounded again) for the copies
// it may still have in flight into its shared memory -- the tile that timed
// out and the one after it, if issued -- so that no bulk copy lands in the
// shared memory of a block that has exited.
__device__ __forceinline__ void drain_tiles(uint64_t *full, unsigned gt, int tiles_left, unsigned limit) {
    for (int k = 0; k < 2 && k < tiles_left; k++) {
        const unsigned g = gt + (unsigned)k;
        wait_bounded(&full[g & 1u], (g >> 1) & 1u, limit);
    }
}

}  // namespace tma
}  // namespace h4
