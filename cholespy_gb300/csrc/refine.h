// Device-side state and launch interface of the refinement residual kernel.
#pragma once
#include <cuda_runtime.h>

namespace gbchol {

// Lives in device memory for the duration of one refined solve.
struct RefineState {
    int converged;           // set by the residual kernel; sweeps then exit at once
    int iterations;          // corrections applied when convergence was detected
    int checks;              // residual evaluations performed
    unsigned int done_blocks;
    double max_rel;          // max_k ||r_k|| / ||b_k|| at the last check
    double bnorm2[128];
};

struct ResidualArgs {
    int n = 0, nrhs = 0;
    const int* rowptr = nullptr;
    const int* cols = nullptr;
    const double* vals = nullptr;
    const double* b = nullptr;
    const double* x = nullptr;
    double* r = nullptr;
    double* partials = nullptr;  // grid * 2 * nrhs
    RefineState* state = nullptr;
    double tol = 0.0;
    int iter = 0;                // corrections applied to x so far
    int first = 0;               // 1 on the first check: also computes ||b||
};

__device__ __forceinline__ int ld_flag(const int* p) {
    return *reinterpret_cast<const volatile int*>(p);
}

int residual_grid(int n);
cudaError_t launch_residual(const ResidualArgs& a, int grid, cudaStream_t stream);

}  // namespace gbchol
