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
    const SnPartial* parts = nullptr;      // lower-sweep partial sums
    void* pbuf = nullptr;           // T, partial-sum slots: (part, slice) -> 32 x slice width
    int n_units = 0;                // partial p's flags follow the units': (n_units + p, slice)
    int nrhs = 0;
    int nslices = 1;                // RHS slices (see sn_slices)
};

struct SnSweepArgs {
    SnSys sys0;                     // the system when item_sys is null
    const SnSys* sys = nullptr;     // device table of systems (batched sweep)
    const int32_t* order = nullptr; // single system: units in dependency-level order
    const int32_t* item_sys = nullptr;   // batched: system of each item
    const int32_t* item_code = nullptr;  // batched: sn_item_code(item, slice) of each item
    int nitems = 0;
    int wide = 0;                   // 1: use the wide-RHS variant for every system (batched)
    int* epoch = nullptr;           // device sweep counter: read at start, +1 by the last CTA out
    int* status = nullptr;
    const int* skip = nullptr;
    int* counters = nullptr;        // [ticket, exited CTAs], zero between launches
};

// RHS slices of one sweep: 1 for <= 8 RHS, else 32-wide (FP32) or 16-wide (FP64).
int sn_slices(int nrhs, bool f64);
// Width of one RHS slice: 8 for a single narrow slice, else 32 (FP32) or 16 (FP64).
int sn_slice_width(int nrhs, bool f64, bool wide);
// Bytes of the partial-sum slots of `nparts` partial sums.
size_t sn_pbuf_bytes(int nparts, int nrhs, bool f64, bool wide);

// Batched item code: item is a unit (>= 0) or ~partial.
inline int32_t sn_item_code(int32_t item, int32_t slice) {
    return item >= 0 ? (item << 3) | slice : -((((~item) + 1) << 3) | slice);
}
cudaError_t launch_sn_sweep(const SnSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream);

}  // namespace gbchol
