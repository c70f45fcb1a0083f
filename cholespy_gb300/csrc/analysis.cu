// Level analysis of L and L^T on the GPU (sm_103a).
//
// Computes, for every row of a triangular factor in CSR form, its level in
// the dependency DAG: 0 for a row with no off-diagonal entry, otherwise one
// more than the largest level among the rows it depends on. This is the
// quantity computed by the reference's analysis_lower / analysis_upper
// (kernels/kernels.cu:8-60); the values are fully determined by L, so the
// result is bit-identical to the reference's on the same factor.
//
// Fast path: for a factor whose pattern is closed under fill (every factor
// produced by a symbolic Cholesky factorisation, CHOLMOD's included), the
// level of row i of L is the height of i in the elimination tree and the
// level of row i of L^T its depth: the dependencies of a row form a subtree
// (L) or an ancestor path (L^T) of the etree along which levels strictly
// increase. The host derives these candidates in O(n) from parent(j) = first
// off-diagonal row of column j, and level_verify_kernel checks them against
// every nonzero of L in one parallel pass over L's columns (no transpose).
// Only a factor that fails the check runs the general sync-free kernel below.
//
// Why an entry-wise check suffices. Lower: the candidate is h(i) = 1 + max
// h(c) over the etree children c of i (0 for none), and every child is an
// entry L(i, c) (parent(c) is column c's first off-diagonal row). If every
// off-diagonal entry L(i, j) satisfies h(i) >= h(j) + 1, then for a row with
// children the maximum of h(j) + 1 over its entries is attained by a child and
// equals h(i); a row without children has h(i) = 0, so the inequality admits
// no entry in it. So h satisfies the level recurrence at every row, whose
// solution is unique: h is the level. Upper: d(j) = 1 + d(parent(j)) (0 at a
// root), the parent is an entry of column j, and every entry L(i, j) must
// satisfy d(j) >= d(i) + 1; the same argument applies.
//
// GB300 design of the general kernel: the reference runs n blocks of ONE thread each, handing rows
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
        bool gave_up = false;
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
                if (f[u] < epoch && !dev::wait_geq(flags + c[u], epoch, status)) gave_up = true;
            dev::fence_acquire();
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (c[u] >= 0) lvl = max(lvl, __ldcg(levels + c[u]) + 1);
        }
        // An abandoned wait (status already records the timeout) means a
        // dependency's level was never published: mark the row invalid
        // (-1), publish nothing built from unpublished data, and stop; the
        // other warps give up at their next wait.
        if (__any_sync(0xffffffffu, gave_up)) {
            if (lane == 0) levels[row] = -1;
            break;
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

// Checks candidate levels against every off-diagonal entry of L (CSC,
// diagonal first in each column), a warp per column, no waits: lower
// requires cand[i] >= cand[j] + 1, upper cand[j] >= cand[i] + 1, for every
// entry L(i, j). With candidates built from the elimination tree (see the top
// of this file) passing means they are exactly the levels.
template <bool LOWER>
__global__ void __launch_bounds__(256) level_verify_kernel(int n, const int* __restrict__ colptr,
                                                           const int* __restrict__ rowidx,
                                                           const int* __restrict__ cand,
                                                           int* mismatch) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int j = warp; j < n; j += nwarps) {
        const int s = colptr[j] + 1, e = colptr[j + 1];
        const int cj = cand[j];
        bool bad = false;
        for (int k = s + lane; k < e; k += 32) {
            const int ci = cand[rowidx[k]];
            bad |= LOWER ? (ci < cj + 1) : (cj < ci + 1);
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(mismatch, 1);
    }
}

// One warp waits (bounded) on a flag that nothing sets: exercises the
// timeout path of every sync-free kernel without hanging anything.
__global__ void selftest_wait_kernel(const int* flag, int* status, unsigned long long limit_ns) {
    if (threadIdx.x == 0) dev::wait_geq(flag, 1, status, limit_ns);
}

}  // namespace

cudaError_t launch_selftest_wait(const int* flag, int* status, unsigned long long limit_ns,
                                 cudaStream_t stream) {
    selftest_wait_kernel<<<1, 32, 0, stream>>>(flag, status, limit_ns);
    return cudaGetLastError();
}

cudaError_t launch_level_verify(bool lower, int n, const int* colptr, const int* rowidx,
                                const int* cand, int* mismatch, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = (n + 7) / 8;
    if (grid > sms * 16) grid = sms * 16;
    if (lower) level_verify_kernel<true><<<grid, 256, 0, stream>>>(n, colptr, rowidx, cand, mismatch);
    else level_verify_kernel<false><<<grid, 256, 0, stream>>>(n, colptr, rowidx, cand, mismatch);
    return cudaGetLastError();
}

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
