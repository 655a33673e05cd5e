// mbarrier and bulk-copy (TMA) primitives shared by the kernels, as inline PTX.
// Every wait is bounded: a kernel that gives up records it in a device error
// word and lets its copies land before leaving.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace tcsem {

__host__ __device__ constexpr size_t rnd16(size_t b) { return (b + 15) & ~(size_t)15; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: gives up after `polls` polls, ~1e6 by default (each poll may suspend for a while)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, int polls = 1 << 20) {
    for (int it = 0; it < polls; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// the barrier's memory may be reused for other data after this (all its copies have landed)
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// A load of data an earlier kernel wrote (FRESH = false: through the read-only cache) or that
// another CTA of the same launch may have written (FRESH = true: cached in L2 only).
template <bool FRESH, typename T> __device__ __forceinline__ T ld_in(const T *p) {
    if constexpr (FRESH) return __ldcg(p);
    else return __ldg(p);
}
// gpu-scope acquire load / release store of a flag or counter in global memory
__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// gpu-scope fence: with a relaxed atomic after it a release, with a relaxed atomic before it an acquire
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
// orders this thread's generic-proxy accesses of global memory with its bulk copies (async proxy)
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Programmatic dependent launch: let the next kernel on the stream start (its blocks become
// resident and run up to their wait), and wait for the previous kernel's completion and memory.
// Without the launch attribute on the dependent kernel both are no-ops.
__device__ __forceinline__ void pdl_allow_next() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait_prev() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// 3-D tiled tensor copy global -> shared, completing on bar
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// contiguous bulk copy global -> shared completing on bar; both addresses
// 16-byte aligned and bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

}  // namespace tcsem
