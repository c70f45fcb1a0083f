// Launch interface of the supernodal sweeps (solve_sn.cu).
#pragma once
#include <cuda_runtime.h>

#include "host/plan.h"
#include "kernels.h"

namespace gbchol {

// One system of a supernodal sweep (several for a batch).
struct SnSys {
    const SnUnit* units = nullptr;
    const SnContrib* contribs = nullptr;
    const int32_t* sn_rows = nullptr;
    const void* panels = nullptr;   // T
    const void* dinv = nullptr;     // T, per unit 32x32 inverse diagonal block (column-major)
    const int32_t* perm = nullptr;
    void* tmp = nullptr;            // T, n x nrhs, permuted space
    void* out = nullptr;            // upper: solution through perm (TOut)
    int* uflags = nullptr;          // n_units * nslices completion flags
    const int32_t* unit_of_row = nullptr;  // unit holding each top row (upper sweep waits)
    int nrhs = 0;
    int nslices = 1;                // RHS slices (see sn_slices)
};

struct SnSweepArgs {
    SnSys sys0;                     // the system when item_sys is null
    const SnSys* sys = nullptr;     // device table of systems (batched sweep)
    const int32_t* order = nullptr; // single system: units in dependency-level order
    const int32_t* item_sys = nullptr;   // batched: system of each item
    const int32_t* item_code = nullptr;  // batched: (unit << 3) | RHS slice of each item
    int nitems = 0;
    int wide = 0;                   // 1: use the wide-RHS variant for every system (batched)
    int* epoch = nullptr;           // device sweep counter: read at start, +1 by the last CTA out
    int* status = nullptr;
    const int* skip = nullptr;
    int* counters = nullptr;        // [ticket, exited CTAs], zero between launches
};

// RHS slices of one sweep: 1 for <= 8 RHS, else 32-wide (FP32) or 16-wide (FP64).
int sn_slices(int nrhs, bool f64);
cudaError_t launch_sn_sweep(const SnSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream);

}  // namespace gbchol
