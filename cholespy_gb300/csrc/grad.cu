// Gradient of x = A^{-1} b with respect to the stored entries of A (sm_103a).
// No counterpart in the reference.
//
// With gb = A^{-1} grad_x (the backward solve, same factor, A symmetric) the
// gradient of a scalar loss with respect to the symmetric matrix is
// dL/dA = -gb x^T. For a stored entry e at (r, c), summed over the RHS k:
//   symmetric mode (A treated as the symmetric matrix sym(A)):
//       r != c:  -1/2 * sum_k (gb[r,k] x[c,k] + gb[c,k] x[r,k])
//       r == c:  -sum_k gb[r,k] x[r,k]
//   lower mode (exact gradient of the reference's forward, which reads only
//   the lower triangle, CHOLMOD stype = -1):
//       r >  c:  -sum_k (gb[r,k] x[c,k] + gb[c,k] x[r,k])
//       r == c:  -sum_k gb[r,k] x[r,k]
//       r <  c:  0
// Duplicate entries each receive the gradient of their summed value.
// Up to 8 RHS: one thread per entry (its four row segments are one sector
// each). More: one warp per entry, lanes over the RHS (both rows of gb and x
// are contiguous, row-major (n, nrhs), so the loads are coalesced). Sums are
// accumulated in the solve's precision (FP32 for an FP32 solver).
#include <cuda_runtime.h>

#include "device.cuh"
#include "grad.h"

namespace gbchol {

namespace {

template <typename T, typename TG>
__device__ __forceinline__ TG grad_of(const GradArgs& a, int r, int c, T s) {
    T g = -s;
    if (a.symmetric && r != c) g *= T(0.5);
    if (!a.symmetric && r < c) g = T(0);
    return (TG)g;
}

template <typename T, typename TG>
__global__ void __launch_bounds__(256) grad_values_thread_kernel(GradArgs a) {
    const T* gb = static_cast<const T*>(a.grad_b);
    const T* x = static_cast<const T*>(a.x);
    TG* out = static_cast<TG*>(a.grad_vals);
    const int nrhs = a.nrhs;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < a.nnz; e += stride) {
        const int r = a.rows[e], c = a.cols[e];
        T s = T(0);
        if (a.symmetric || r >= c) {
            const T* gr = gb + (size_t)r * nrhs;
            const T* gc = gb + (size_t)c * nrhs;
            const T* xr = x + (size_t)r * nrhs;
            const T* xc = x + (size_t)c * nrhs;
            for (int k = 0; k < nrhs; ++k) {
                s = fma(gr[k], xc[k], s);
                if (r != c) s = fma(gc[k], xr[k], s);
            }
        }
        out[e] = grad_of<T, TG>(a, r, c, s);
    }
}

template <typename T, typename TG>
__global__ void __launch_bounds__(256) grad_values_kernel(GradArgs a) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const T* gb = static_cast<const T*>(a.grad_b);
    const T* x = static_cast<const T*>(a.x);
    TG* out = static_cast<TG*>(a.grad_vals);
    const int nrhs = a.nrhs;
    for (long long e = warp; e < a.nnz; e += nwarps) {
        const int r = a.rows[e], c = a.cols[e];
        T s = T(0);
        if (a.symmetric || r >= c) {
            const T* gr = gb + (size_t)r * nrhs;
            const T* gc = gb + (size_t)c * nrhs;
            const T* xr = x + (size_t)r * nrhs;
            const T* xc = x + (size_t)c * nrhs;
            for (int k = lane; k < nrhs; k += 32) {
                s = fma(gr[k], xc[k], s);
                if (r != c) s = fma(gc[k], xr[k], s);
            }
            s = dev::warp_sum(s);
        }
        if (lane == 0) out[e] = grad_of<T, TG>(a, r, c, s);
    }
}

}  // namespace

cudaError_t launch_grad_values(const GradArgs& a, bool f32, bool out_f32, cudaStream_t stream) {
    if (a.nnz == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    GradArgs c = a;
    if (a.nrhs <= 8) {  // thread per entry
        long long need = (a.nnz + 255) / 256;
        int grid = (int)(need < (long long)sms * 32 ? need : (long long)sms * 32);
        if (f32 && out_f32) grad_values_thread_kernel<float, float><<<grid, 256, 0, stream>>>(c);
        else if (f32) grad_values_thread_kernel<float, double><<<grid, 256, 0, stream>>>(c);
        else if (out_f32) grad_values_thread_kernel<double, float><<<grid, 256, 0, stream>>>(c);
        else grad_values_thread_kernel<double, double><<<grid, 256, 0, stream>>>(c);
        return cudaGetLastError();
    }
    long long need = (a.nnz + 7) / 8;
    int grid = (int)(need < (long long)sms * 16 ? need : (long long)sms * 16);
    if (f32 && out_f32) grad_values_kernel<float, float><<<grid, 256, 0, stream>>>(c);
    else if (f32) grad_values_kernel<float, double><<<grid, 256, 0, stream>>>(c);
    else if (out_f32) grad_values_kernel<double, float><<<grid, 256, 0, stream>>>(c);
    else grad_values_kernel<double, double><<<grid, 256, 0, stream>>>(c);
    return cudaGetLastError();
}

}  // namespace gbchol
