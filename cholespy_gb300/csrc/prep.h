// Construction input prep on the GPU (prep.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace gbchol {

// A CSC matrix in device memory (cudaMalloc'd; release() frees it).
struct DeviceCsc {
    int32_t n = 0;
    int32_t nnz = 0;
    int32_t* colptr = nullptr;
    int32_t* rowidx = nullptr;
    double* vals = nullptr;
    void release();
};

// Device arrays (fmt 0 CSC, 1 CSR, 2 COO, as gbchol_create) -> sorted,
// duplicate-summed CSC, equal to build_csc's result. Pointer arrays of CSR /
// CSC input must have been checked by the caller (ptr[0] = 0, non-
// decreasing, ptr[n] = nnz). *bad_index = 1 (and nothing built) when an
// index is out of range. Synchronises `s`.
cudaError_t device_csc(int32_t n, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x, int32_t fmt,
                       DeviceCsc& out, int* bad_index, cudaStream_t s);

// dst[k] = (float)src[k] (round to nearest even, as the host cast), device arrays.
cudaError_t cast_to_f32(const double* src, float* dst, int64_t n, cudaStream_t s);

}  // namespace gbchol
