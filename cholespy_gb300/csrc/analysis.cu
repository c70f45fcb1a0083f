// Level analysis of L and L^T on the GPU (sm_103a).
//
// Computes, for every row of a triangular factor in CSR form, its level in
// the dependency DAG: 0 for a row with no off-diagonal entry, otherwise one
// more than the largest level among the rows it depends on. This is the
// quantity computed by the reference's analysis_lower / analysis_upper
// (kernels/kernels.cu:8-60); the values are fully determined by L, so the
// result is bit-identical to the reference's on the same factor.
//
// GB300 design: the reference runs n blocks of ONE thread each, handing rows
// out through a global atomic ticket and spinning without bound. Here one
// warp handles a row: its 32 lanes read the row's column indices coalesced,
// each lane waits (bounded) on its dependency's flag, and a warp max-reduce
// gives the level. Rows are assigned statically in dependency order
// (warp w takes rows w, w + W, w + 2W, ...) and the kernel is launched
// cooperatively, so every warp is resident: the smallest unfinished row can
// always make progress, which rules out deadlock without a ticket atomic.
#include "device.cuh"
#include "kernels.h"
#include "launch.h"

namespace gbchol {

namespace {

template <bool LOWER>
__global__ void __launch_bounds__(256) level_kernel(int n, const int* __restrict__ rowptr,
                                                    const int* __restrict__ cols, int* levels,
                                                    int* flags, int epoch, int* max_lvl,
                                                    int* status) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    int local_max = 0;
    for (int t = warp; t < n; t += nwarps) {
        const int row = LOWER ? t : n - 1 - t;
        const int s = rowptr[row], e = rowptr[row + 1];
        // off-diagonal entries: diagonal is last in L's rows, first in L^T's
        const int lo = LOWER ? s : s + 1;
        const int hi = LOWER ? e - 1 : e;
        int lvl = 0;
        // flags of 4 entries per lane are loaded together (independent
        // relaxed loads); only entries not yet published take the bounded
        // wait; one acquire fence then orders the level reads.
        for (int base = lo; base < hi; base += 128) {
            int c[4], f[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = base + lane + 32 * u;
                c[u] = k < hi ? cols[k] : -1;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) f[u] = c[u] >= 0 ? dev::ld_volatile(flags + c[u]) : epoch;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (f[u] < epoch) dev::wait_geq(flags + c[u], epoch, status);
            dev::fence_acquire();
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (c[u] >= 0) lvl = max(lvl, __ldcg(levels + c[u]) + 1);
        }
        lvl = dev::warp_max(lvl);
        local_max = max(local_max, lvl);
        if (lane == 0) {
            levels[row] = lvl;
            dev::st_release(flags + row, epoch);
        }
    }
    if (lane == 0 && local_max > 0) atomicMax(max_lvl, local_max);
}

}  // namespace

cudaError_t launch_level_analysis(bool lower, int n, const int* rowptr, const int* cols,
                                  int* levels, int* flags, int epoch, int* max_lvl, int* status,
                                  cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const void* fn = lower ? (const void*)level_kernel<true> : (const void*)level_kernel<false>;
    int grid = 0;
    cudaError_t e = coop_grid(fn, 256, 0, &grid);
    if (e != cudaSuccess) return e;
    const int need = (n + 7) / 8;  // 8 warps per block
    if (grid > need) grid = need;
    void* args[] = {&n, &rowptr, &cols, &levels, &flags, &epoch, &max_lvl, &status};
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, stream);
}

}  // namespace gbchol
