// Launch interface of the bulk-copy supernodal sweeps (solve_snb.cu): the
// FP32 top-region sweeps for many right-hand sides.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "host/plan.h"
#include "kernels.h"

namespace gbchol {

struct SnbArgs {
    const SnUnit* units = nullptr;
    const SnContrib* contribs = nullptr;
    const int32_t* order = nullptr;     // tickets: unit u, or (lower sweep) partial sum p as ~p
    const float* lo_tiles = nullptr;    // per contribution block: 32 x 32, [source column][unit row]
                                        // (a group's tiles are consecutive: its rows are contiguous)
    const float* up_tiles = nullptr;    // per upper block: 32 x 32, [block row][unit column]
    const int32_t* up_begin = nullptr;  // per unit: first upper block (n_units + 1 entries)
    const int32_t* up_rows = nullptr;   // per upper block: 32 work-array rows (-1 past the block)
    const int32_t* up_dep = nullptr;    // per upper block: the unit whose flag it waits for
    const SnbGroup* groups = nullptr;   // lower: merged contribution blocks, per unit in list order
    const int32_t* unit_info = nullptr; // lower: per unit, first own group, end of groups, first / end partial
    const SnPartial* parts = nullptr;   // lower: partial sums over group ranges
    float* pbuf = nullptr;              // lower: partial-sum slots, 32 x nrhs each
    int n_units = 0;                    // partial p's flag follows the units': n_units + p
    const float* dinv = nullptr;        // per unit: D^-1, M_lo, M_up (32 x 32, column-major each)
    const float* fold2 = nullptr;       // per unit: M2_lo, M2_up (32 x 32, column-major each)
    int fold = 1;                       // 2: the chunk two before / after is folded too (the plans' fold)
    const int32_t* perm = nullptr;
    float* tmp = nullptr;               // n x nrhs work array (permuted space), 16-byte aligned
    void* out = nullptr;                // upper sweep: the solution, through perm (TOut)
    int* uflags = nullptr;              // completion flags: units, then partial sums
    int nrhs = 0;                       // RHS columns of one work item (a slice)
    int ld = 0;                         // row stride of the work array (0: nrhs)
    int nslices = 1;                    // column slices: items = (unit or partial sum, slice)
    int flag_stride = 0;                // flags per slice (n_units + partial sums)
    int nitems = 0;                     // tickets: (lower: n_units + partial sums; upper: n_units) x nslices
    int* epoch = nullptr;               // device sweep counter: read at start, +1 by the last CTA out
    int* status = nullptr;
    const int* skip = nullptr;
    int* counters = nullptr;            // [ticket, exited CTAs], zero between launches
    int tensor_cores = 0;               // 1: block products on the tensor cores (3 x TF32 split)
};

// The bulk sweeps take RHS counts that are multiples of 4 (rows of the work
// array are copied in 16-byte units) up to 128; one work item holds every
// RHS column of its unit, or one of `nslices` equal column slices (each a
// multiple of 4 wide): the slices are independent solves on the same tiles,
// each with its own flags, so a dependency chain steps through half (a
// quarter) of the columns per unit.
inline bool snb_supported(int nrhs) { return nrhs >= 4 && nrhs <= 128 && nrhs % 4 == 0; }
// Shared-memory width of a work item: 32, 64 or 128 columns.
inline int snb_width(int nrhs) { return nrhs <= 32 ? 32 : (nrhs <= 64 ? 64 : 128); }
// Source columns per lower-sweep group: 64 with the CUDA-core consumers, 32
// with the tensor-core ones.
inline int snb_group_cols(bool tensor_cores) { return tensor_cores ? 32 : 64; }

// The upper sweep writes the output only when a.out is set; otherwise this
// kernel writes the top rows' solution afterwards (out[perm[row]] = or +=
// tmp[row]), off the sweep's dependency chain.
cudaError_t launch_snb_sweep(const SnbArgs& a, bool lower, SweepIO io, cudaStream_t stream);
cudaError_t launch_snb_scatter(const SnbArgs& a, int nunits, SweepIO io, cudaStream_t stream);

// Expands the FP32 panels into the sweeps' 32 x 32 tiles (zero outside a
// block's rows and columns). Lower tiles: one per contribution block.
// Upper tiles: one per (panel offset, leading dimension, rows | columns << 16).
cudaError_t launch_snb_expand_lower(const SnContrib* contribs, int64_t n, const float* panels, float* tiles,
                                    cudaStream_t stream);
cudaError_t launch_snb_expand_upper(const int64_t* src, const int32_t* ld, const int32_t* nrw, int64_t n,
                                    const float* panels, float* tiles, cudaStream_t stream);

}  // namespace gbchol
