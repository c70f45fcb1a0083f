// Launch interface of the supernodal sweeps (solve_sn.cu).
#pragma once
#include <cuda_runtime.h>

#include "host/plan.h"
#include "kernels.h"

namespace gbchol {

struct SnSweepArgs {
    int n_units = 0;
    int nslices = 1;          // RHS slices (see sn_slices)
    int nrhs = 0;
    const SnUnit* units = nullptr;
    const SnContrib* contribs = nullptr;
    const int32_t* sn_rows = nullptr;
    const void* panels = nullptr;   // T
    const int32_t* perm = nullptr;
    void* tmp = nullptr;            // T, n x nrhs, permuted space
    void* out = nullptr;            // upper: solution through perm (TOut)
    const int32_t* order = nullptr; // units in dependency-level order for this sweep
    const void* dinv = nullptr;     // T, per unit 32x32 inverse diagonal block (column-major)
    int* counters = nullptr;        // [ticket, exited CTAs], zero between launches
    int* uflags = nullptr;          // n_units * nslices completion flags
    int epoch = 0;
    int* status = nullptr;
    const int* skip = nullptr;
};

// RHS slices of one sweep: 1 for <= 8 RHS, else 32-wide (FP32) or 16-wide (FP64).
int sn_slices(int nrhs, bool f64);
cudaError_t launch_sn_sweep(const SnSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream);

}  // namespace gbchol
