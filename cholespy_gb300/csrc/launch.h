// Launch-shape helpers: persistent, cooperatively launched grids sized to
// the number of co-resident blocks (152 SMs on GB300).
#pragma once
#include <cuda_runtime.h>

namespace gbchol {

// Largest grid of `threads`-thread blocks using `smem` bytes of dynamic
// shared memory that can be co-resident on the current device (for
// cudaLaunchCooperativeKernel).
inline cudaError_t coop_grid(const void* fn, int threads, size_t smem, int* grid) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    *grid = sms * per_sm;
    return cudaSuccess;
}

}  // namespace gbchol
