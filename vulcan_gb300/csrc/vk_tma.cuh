// Bulk (1D TMA) copies global -> shared with mbarrier completion.
//
// Rules followed by the callers: source and destination 16-byte aligned, size a
// multiple of 16 bytes (block strides are padded to 4 floats); every wait is
// bounded -- on timeout the caller records an error status, waits (bounded
// again) for its own copy in flight and leaves the kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vk {

constexpr int kMbarSpin = 1 << 22;      // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: announce `bytes` of transaction and start the copy.
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of the barrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (int i = 0; i < kMbarSpin; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Padded stride (floats) of an n x n FP32 block so every block starts on 16 bytes.
__host__ __device__ __forceinline__ int block_stride32(int n) { return (n * n + 3) & ~3; }

}  // namespace vk
