// Launch interface of the supernodal sweeps (solve_sn.cu).
#pragma once
#include <cuda_runtime.h>

#include "host/plan.h"
#include "kernels.h"

namespace gbchol {

struct SnSweepArgs {
    int n_units = 0;
    int nslices = 1;          // RHS slices of 32 (1 when nrhs <= 8)
    int nrhs = 0;
    const SnUnit* units = nullptr;
    const SnContrib* contribs = nullptr;
    const int32_t* sn_rows = nullptr;
    const void* panels = nullptr;   // T
    const int32_t* perm = nullptr;
    void* tmp = nullptr;            // T, n x nrhs, permuted space
    void* out = nullptr;            // upper: solution through perm (TOut)
    int* uflags = nullptr;          // n_units * nslices completion flags
    int epoch = 0;
    int* status = nullptr;
    const int* skip = nullptr;
};

int sn_slices(int nrhs);
cudaError_t launch_sn_sweep(const SnSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream);

}  // namespace gbchol
