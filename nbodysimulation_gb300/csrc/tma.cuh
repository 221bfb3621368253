// tma.cuh -- mbarrier and bulk asynchronous copy (TMA, cp.async.bulk)
// helpers for the all-pairs kernels: 1-D bulk copies global -> shared with
// transaction-count completion, no cluster, no multicast.
#pragma once
#include "nbgb_internal.cuh"

namespace nbgb {

// ---- PTX helpers: mbarrier + bulk async copy (sm_90+) ----
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on a tile; on timeout records the status and keeps waiting
// (bounded again) so no copy into this block's shared memory is left in
// flight when the block exits.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, Ctrl *ctrl) {
    long long it = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (++it > kSpinCap) {
            set_status(ctrl, kStSpinTimeout, -1);
            long long it2 = 0;
            while (!mbar_try_wait(bar, parity) && ++it2 < kSpinCap) {
            }
            return false;
        }
    }
    return true;
}

}  // namespace nbgb
