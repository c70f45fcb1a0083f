// Launch interface of the sparse-gradient kernel (grad.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace gbchol {

struct GradArgs {
    long long nnz = 0;
    int nrhs = 0;
    int symmetric = 1;
    const int32_t* rows = nullptr;  // entry rows (original index space)
    const int32_t* cols = nullptr;  // entry columns
    const void* grad_b = nullptr;   // T (n, nrhs)
    const void* x = nullptr;        // T (n, nrhs)
    void* grad_vals = nullptr;      // TG (nnz)
};

cudaError_t launch_grad_values(const GradArgs& a, bool f32, bool out_f32, cudaStream_t stream);

}  // namespace gbchol
