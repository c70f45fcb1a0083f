// Bulk asynchronous copies (cp.async.bulk) and shared-memory mbarriers for
// sm_103a, as inline PTX. Every wait is bounded in time like the flag waits
// of device.cuh: on expiry it records GBCHOL_ETIMEOUT in the status word and
// returns false.
#pragma once
#include <cstdint>

#include "device.cuh"

namespace gbchol {
namespace bulk {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async proxy (bulk copies).
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the phase of `bar` with the given parity to complete. Gives up
// when the status word is set by another waiter (abort_on_status) or after
// limit_ns, recording a timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status, bool abort_on_status = true,
                                          unsigned long long limit_ns = dev::kWaitLimitNs) {
    if (mbar_test(bar, parity)) return true;
    unsigned long long t0 = 0;
    for (unsigned it = 1;; ++it) {
        if (mbar_test(bar, parity)) return true;
        if ((it & 15) == 0) {
            if (abort_on_status && dev::ld_volatile(status) != 0) return false;
            const unsigned long long now = dev::globaltimer();
            if (t0 == 0) t0 = now;
            else if (now - t0 > limit_ns) {
                atomicCAS(status, 0, dev::kStatusTimeout);
                return false;
            }
        }
    }
}

// Orders this thread's earlier generic-proxy accesses (e.g. the acquire of a
// flag) before its later async-proxy accesses of global memory.
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Global -> shared bulk copy completing on `bar` (bytes and both addresses
// multiples of 16).
__device__ __forceinline__ void copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Barrier among the `count` threads that name barrier `id` (id 0 is
// __syncthreads).
__device__ __forceinline__ void named_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

}  // namespace bulk
}  // namespace gbchol
