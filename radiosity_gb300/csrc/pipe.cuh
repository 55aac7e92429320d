// Device helpers of the asynchronous pipelines (the tcgen05 GEMM, the streaming residual):
// shared-memory addresses, the global timer and mbarrier operations with bounded waits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rad {

constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s bound on every wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

// Waits for the phase of the given parity; false (and the error word, when given, set) after
// limit_ns of global time.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, uint32_t* err,
                                          unsigned long long limit_ns = kWaitNs) {
    const uint32_t a = smem_u32(b);
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; it++) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 0) {
            const unsigned long long t = global_ns();
            if (it == 0) t0 = t;
            else if (t - t0 > limit_ns) {
                if (err) atomicOr(err, 1u);
                return false;
            }
        }
    }
}

}  // namespace rad
