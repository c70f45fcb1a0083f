// Launch-shape helpers: persistent grids sized to the number of co-resident
// blocks (152 SMs on GB300). Results are cached per (kernel, device, block
// shape), so after the first launch a solve issues only kernel launches
// (nothing else runs while a CUDA graph is being captured).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <tuple>

namespace gbchol {

// Largest grid of `threads`-thread blocks using `smem` bytes of dynamic
// shared memory that can be co-resident on the current device. When smem
// exceeds the default 48 KB the kernel's attribute is raised first.
inline cudaError_t coop_grid(const void* fn, int threads, size_t smem, int* grid) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, int, size_t>, int> cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_tuple(fn, dev, threads, smem);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            *grid = it->second;
            return cudaSuccess;
        }
    }
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    *grid = sms * per_sm;
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = *grid;
    return cudaSuccess;
}

}  // namespace gbchol
