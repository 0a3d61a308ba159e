// orbgpu_async.cuh -- mbarrier and bulk / tensor copy (TMA) wrappers shared by
// the kernels that stage global memory into shared memory asynchronously.
//
// Every wait is bounded: mbar_wait gives up after about one second (or
// ORBGPU_SPIN_LIMIT polls) and returns false, so a kernel can record an
// error flag and leave instead of hanging.
#pragma once

#include <cstdint>

namespace orbgpu {

#define ORBGPU_SPIN_LIMIT (1u << 26)
#define ORBGPU_WAIT_NS 1000000000ull  // one second

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
// Makes mbarrier initialisations visible to the asynchronous proxy.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait on phase 'parity': false after about one second (or
// ORBGPU_SPIN_LIMIT polls), whichever comes first.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    uint64_t t0 = 0;
    for (uint32_t i = 0; i < ORBGPU_SPIN_LIMIT; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 31) == 31) {
            const uint64_t t = global_ns();
            if (t0 == 0) t0 = t;
            else if (t - t0 > ORBGPU_WAIT_NS) return false;
        }
    }
    return false;
}
// Contiguous copy global -> shared (16-byte aligned addresses, size a
// multiple of 16), completing on 'bar'.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// Acquire a tensor map that the host copied into global memory before the
// launch (system scope: the writer is the host), before the first copy
// through it.
__device__ __forceinline__ void tensormap_acquire(const void* tmap) {
    asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(tmap) : "memory");
}
// Tiled 2-D copy of the tensor map's box at element (x, y) into shared
// memory (128-byte aligned), completing on 'bar'.  x times the element size
// must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace orbgpu
