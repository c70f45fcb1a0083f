// Device-side helpers shared by the gbchol kernels: memory-ordering
// primitives for the sync-free (flag-based) sweeps and bounded waits.
//
// Every wait on another warp's flag is bounded in time (globaltimer): on
// expiry the waiter records GBCHOL_ETIMEOUT in the solver's status word and
// gives up, and every other waiter gives up as soon as it sees a non-zero
// status. A malformed factor therefore ends a kernel with an error status
// instead of hanging the GPU (the reference spins without bound,
// kernels/kernels.cu:20-21,47-48,108-109,176-177).
#pragma once
#include <cstdint>

namespace gbchol {
namespace dev {

constexpr int kStatusTimeout = 5;                       // == GBCHOL_ETIMEOUT
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile(const int* p) {
    return *reinterpret_cast<const volatile int*>(p);
}
__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits until *flag >= target. Returns false (after recording a timeout in
// *status if this wait expired) when the wait is abandoned.
__device__ __forceinline__ bool wait_geq(const int* flag, int target, int* status,
                                         unsigned long long limit_ns = kWaitLimitNs) {
    if (ld_acquire(flag) >= target) return true;
    unsigned long long t0 = 0;
    for (unsigned it = 1;; ++it) {
        if (it > 256) __nanosleep(64);
        if (ld_acquire(flag) >= target) return true;
        if ((it & 63) == 0) {
            if (ld_volatile(status) != 0) return false;
            unsigned long long now = globaltimer();
            if (t0 == 0) t0 = now;
            else if (now - t0 > limit_ns) {
                atomicCAS(status, 0, kStatusTimeout);
                return false;
            }
        }
    }
}

// Acquire fence: after relaxed/volatile loads that observed released flags,
// orders the following loads after those observations (acquire pattern).
__device__ __forceinline__ void fence_acquire() {
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

// L2-coherent loads of values produced by other SMs during the same launch.
template <typename T>
__device__ __forceinline__ T ld_cg(const T* p) { return __ldcg(p); }

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace dev
}  // namespace gbchol
