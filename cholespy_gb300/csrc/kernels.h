// Internal launch interface of the gbchol CUDA kernels (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace gbchol {

// ---- level analysis (analysis.cu) ----------------------------------------
// One warp per row; rows in dependency order (increasing for L, decreasing
// for L^T). levels[i] = 0 for rows without off-diagonal entries, else
// 1 + max level of the rows it depends on. Same definition as the
// reference's analysis_lower / analysis_upper (kernels/kernels.cu:8-60).
cudaError_t launch_level_analysis(bool lower, int n, const int* rowptr, const int* cols,
                                  int* levels, int* flags, int epoch, int* max_lvl, int* status,
                                  cudaStream_t stream);

// Parallel check of elimination-tree candidate levels against every
// off-diagonal entry of L, given in CSC (diagonal first in each column);
// sets *mismatch to 1 if any entry disagrees.
cudaError_t launch_level_verify(bool lower, int n, const int* colptr, const int* rowidx,
                                const int* cand, int* mismatch, cudaStream_t stream);

// Self-test of the bounded wait: one wait on a flag that nothing sets.
cudaError_t launch_selftest_wait(const int* flag, int* status, unsigned long long limit_ns,
                                 cudaStream_t stream);

// ---- row-wise sync-free sweeps (solve_rows.cu) ----------------------------
// Lower sweep (L y = b[perm]):    tmp[row] = (in[perm[row]] - sum L[row,c] tmp[c]) / L[row,row]
// Upper sweep (L^T x = y):        tmp[row] = (tmp[row] - sum U[row,c] tmp[c]) / U[row,row]
//                                 out[perm[row]] = tmp[row]   (or += in refinement mode)
// Same arithmetic as solve_lower / solve_upper (kernels/kernels.cu:64-202).
// A "partial" task (~row) has no diagonal: tmp[row] = (lower: in[perm[row]],
// upper: tmp[row]) - sum, and publishes nothing.

// One system of a row sweep (several for a batch).
struct RowSys {
    const int* rowptr = nullptr;
    const int* cols = nullptr;
    const void* vals = nullptr;   // T
    const int* perm = nullptr;
    const void* in = nullptr;     // lower: right-hand side (TIn), read through perm
    void* tmp = nullptr;          // T, n x nrhs, permuted space
    void* out = nullptr;          // upper: solution (TOut), written through perm
    int* flags = nullptr;         // row completion flags (epoch-valued)
    int nrhs = 0;
    int pad = 0;
    // upper sweep, optional: entries of each row whose values are final
    // before the launch (the top rows' terms of a leaf row), summed first
    // with no flag checks
    const int* nw_rowptr = nullptr;
    const int* nw_cols = nullptr;
    const void* nw_vals = nullptr;  // T
};

struct RowSweepArgs {
    RowSys sys0;                  // the system when task_sys is null
    const RowSys* sys = nullptr;  // device table of systems (batched sweep)
    const int* tasks = nullptr;   // task codes in dependency order: row, or ~row (partial)
    const int* task_sys = nullptr;// system of each task (batched sweep), else null
    int ntasks = 0;
    int* epoch = nullptr;         // device sweep counter: read at start, +1 by the last warp out
    int* status = nullptr;
    const int* skip = nullptr;    // if non-null and *skip != 0 the sweep does nothing
    int* counters = nullptr;      // [ticket, exited warps], zero between launches
    int chunk = 1;                // consecutive tasks taken per ticket
    int max_nrhs = 0;             // largest nrhs over the systems (kernel variant choice)
    int rhs_split = 0;            // 1: lanes over the RHS columns even for <= 8 RHS (autotuned)
    int batched_variant = 0;      // 1: per-system dispatch, two lane modes (<= 8 RHS, more);
                                  // 2: per-system dispatch to the mode fitted to its RHS count
                                  // (1 RHS: lanes over the nonzeros; 2..16: 16-lane groups over
                                  // the RHS; 17..32 / 64 / 128: 32 lanes x 1 / 2 / 4 columns)
};

enum class SweepIO {
    F32,          // T = float, in/out float
    F64,          // T = double, in/out double
    F32_MIXED,    // T = float, in double, out double (x = y): first refinement solve
    F32_REFINE,   // T = float, in double (residual), out double with x += d
};

cudaError_t launch_row_sweep(const RowSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream);

}  // namespace gbchol
