// f8_tma.cuh — bulk asynchronous copies (the Tensor Memory Accelerator's
// cp.async.bulk) from global into shared memory, completed on shared-memory
// mbarriers, for the streaming kernels of the FP32-mixed step.
//
// The halo fields are (NX+2)(NY+2)(NZ+2) floats, x fastest; a row is
// 4(NX+2) bytes, which is not a multiple of 16 for the grids of the solver
// (NX a power of two), so a tiled tensor map (whose strides must be multiples
// of 16 bytes) cannot describe the layout.  Two consecutive rows starting at
// an even row of an even-NY grid are a contiguous, 16-byte aligned block of
// 8(NX+2) bytes, a multiple of 16: the kernels stage such row pairs with the
// non-tensor bulk copy.
//
// Every wait is bounded (about a second of SM clocks): a wait that runs out
// returns false, and the kernel records the failure for the host and stops
// issuing copies instead of spinning on.
#pragma once
#include <cstdint>

namespace f8 {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// make the initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic-proxy accesses of shared memory (after a
// block barrier: every thread's reads of a buffer) before later async-proxy
// writes into it
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// one arrival that also announces `bytes` of copies completing on the barrier
__device__ __forceinline__ void mbar_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
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

// wait for the phase with the given parity to complete; false after
// `budget` SM clock cycles
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long budget = 2000000000LL) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity))
        if (clock64() - t0 > budget) return false;
    return true;
}

// bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on `bar`
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace f8
