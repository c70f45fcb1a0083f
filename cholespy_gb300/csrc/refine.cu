// FP64 residual for iterative refinement (sm_103a).
//
// r = b - A x with A the symmetric FP64 matrix in its original ordering
// (CSR, both triangles), plus per-RHS ||r_k||^2 (and ||b_k||^2 on the first
// call) reduced deterministically: each block writes its partial sums, the
// last block to finish (atomic counter) adds them in block order, takes
// the convergence decision and stores it in the device-side RefineState.
// Later sweeps read RefineState::converged and exit at once, so a whole
// refinement loop is queued without any host synchronisation.
// No counterpart in the reference (the reference has no refinement).
#include <cuda_runtime.h>

#include <atomic>

#include "device.cuh"
#include "refine.h"

namespace gbchol {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

// One warp per row; lane l owns RHS columns l, l+32, l+64, l+96.
template <int Q>
__global__ void __launch_bounds__(kThreads) residual_kernel(ResidualArgs a) {
    RefineState* st = a.state;
    if (ld_flag(&st->converged)) return;
    __shared__ double red[kWarps][2 * 128];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nrhs = a.nrhs;
    double rn[Q], bn[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) rn[q] = bn[q] = 0.0;
    const int gw = blockIdx.x * kWarps + w;
    const int nw = gridDim.x * kWarps;
    for (int row = gw; row < a.n; row += nw) {
        const int s = a.rowptr[row], e = a.rowptr[row + 1];
        double acc[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) acc[q] = 0.0;
        for (int k = s; k < e; ++k) {
            const int c = a.cols[k];
            const double v = a.vals[k];
            const double* xc = a.x + (size_t)c * nrhs;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int j = lane + 32 * q;
                if (j < nrhs) acc[q] = fma(v, xc[j], acc[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int j = lane + 32 * q;
            if (j < nrhs) {
                const size_t o = (size_t)row * nrhs + j;
                const double bv = a.b[o];
                const double r = bv - acc[q];
                a.r[o] = r;
                rn[q] = fma(r, r, rn[q]);
                if (a.first) bn[q] = fma(bv, bv, bn[q]);  // ||b|| once per refined solve
            }
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = lane + 32 * q;
        if (j < 128) {
            red[w][j] = rn[q];
            red[w][128 + j] = bn[q];
        }
    }
    __syncthreads();
    // block partials, summed over warps in fixed order
    for (int j = threadIdx.x; j < nrhs; j += kThreads) {
        double sr = 0.0, sb = 0.0;
        for (int ww = 0; ww < kWarps; ++ww) {
            sr += red[ww][j];
            sb += red[ww][128 + j];
        }
        a.partials[(size_t)blockIdx.x * 2 * nrhs + j] = sr;
        a.partials[(size_t)blockIdx.x * 2 * nrhs + nrhs + j] = sb;
    }
    __threadfence();
    __syncthreads();
    __shared__ unsigned int ticket;
    if (threadIdx.x == 0) ticket = atomicAdd(&st->done_blocks, 1u);
    __syncthreads();
    if (ticket != gridDim.x - 1) return;
    // last block: reduce partials in block order and decide
    __threadfence();
    __shared__ double ratio[128];
    for (int j = threadIdx.x; j < nrhs; j += kThreads) {
        double sr = 0.0, sb = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) {
            sr += __ldcg(a.partials + (size_t)b * 2 * nrhs + j);
            sb += __ldcg(a.partials + (size_t)b * 2 * nrhs + nrhs + j);
        }
        if (a.first) st->bnorm2[j] = sb;
        const double bb = a.first ? sb : st->bnorm2[j];
        ratio[j] = bb > 0.0 ? sqrt(sr / bb) : sqrt(sr);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // The maximum carries NaN (fmax would drop it), and a RHS converges
        // only when its ratio compares <= tol, which NaN never does: a NaN
        // or Inf anywhere in b, x or the factor leaves the solve unconverged
        // and reports a non-finite max_rel.
        double m = 0.0;
        bool all_ok = true;
        for (int j = 0; j < nrhs; ++j) {
            const double v = ratio[j];
            if (!(v <= a.tol)) all_ok = false;
            if (!(v <= m) && !isnan(m)) m = v;
        }
        st->max_rel = m;
        st->checks += 1;
        if (all_ok) {
            st->converged = 1;
            st->iterations = a.iter;
        }
        st->done_blocks = 0;
    }
}

}  // namespace

cudaError_t launch_residual(const ResidualArgs& a, int grid, cudaStream_t stream) {
    ResidualArgs c = a;
    if (a.nrhs <= 32) residual_kernel<1><<<grid, kThreads, 0, stream>>>(c);
    else if (a.nrhs <= 64) residual_kernel<2><<<grid, kThreads, 0, stream>>>(c);
    else residual_kernel<4><<<grid, kThreads, 0, stream>>>(c);
    return cudaGetLastError();
}

int residual_grid(int n) {
    // Per-device SM counts, filled once per device; relaxed atomics make
    // concurrent callers on any thread or device safe (a race only repeats
    // the same attribute query).
    constexpr int kMaxDevices = 64;
    static std::atomic<int> sm_count[kMaxDevices];
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < kMaxDevices) sms = sm_count[dev].load(std::memory_order_relaxed);
    if (sms <= 0) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
        if (dev >= 0 && dev < kMaxDevices) sm_count[dev].store(sms, std::memory_order_relaxed);
    }
    int need = (n + kWarps - 1) / kWarps;
    int g = sms * 8;
    return need < g ? (need > 0 ? need : 1) : g;
}

}  // namespace gbchol
