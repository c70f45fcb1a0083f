// Internal definitions shared by the C-ABI translation units (api.cu,
// batch.cu): device buffers, error helpers and the solver handle.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <string>
#include <vector>

#include "gbchol.h"
#include "host/host.h"
#include "host/plan.h"
#include "kernels.h"
#include "refine.h"
#include "solve_sn.h"
#include "solve_snb.h"

namespace gbchol {

// Records the message of a failed call (thread-local) and returns `code`.
int fail(int code, const std::string& msg);

// Rows per ticket of the row kernels (GBCHOL_ROW_CHUNK overrides; tuning).
int row_chunk();

}  // namespace gbchol

struct gbchol_solver;

namespace gbchol {
// One full solve (leaf lower, supernodal lower, supernodal upper, top-row
// terms, leaf upper) with `work` as the permuted-space work array.
// Bytes of the work array of one solve: the permuted-space copy of the RHS
// (n x nrhs, 256-byte aligned) followed by the partial-sum slots.
size_t work_bytes(const gbchol_solver* h, int nrhs, bool f32);
int run_sweeps_with(gbchol_solver* h, bool f32, SweepIO io, int nrhs, const void* in, void* out,
                    const int* skip, void* work, cudaStream_t s);
}  // namespace gbchol

namespace gbchol {

struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) {
            changed = cudaSetDevice(dev) == cudaSuccess;
        }
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

#define CUDA_TRY(expr)                                                                     \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess)                                                             \
            return fail(_e == cudaErrorMemoryAllocation ? GBCHOL_ENOMEM : GBCHOL_ECUDA,    \
                        std::string("CUDA error: ") + cudaGetErrorString(_e) + " (" #expr   \
                                                                               ")");        \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t count = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        count = 0;
    }
    cudaError_t alloc(size_t n) {
        release();
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e == cudaSuccess) count = n;
        else p = nullptr;
        return e;
    }
    cudaError_t upload(const T* h, size_t n) {
        cudaError_t e = alloc(n);
        if (e != cudaSuccess || n == 0) return e;
        return cudaMemcpy(p, h, n * sizeof(T), cudaMemcpyHostToDevice);
    }
};

// One triangle (L or L^T) in CSR form with its level analysis.
struct Triangle {
    DevBuf<int32_t> rowptr, cols, order;
    DevBuf<float> v32;
    DevBuf<double> v64;
    std::vector<int32_t> row_levels, order_h;
    int32_t max_lvl = 0;
    bool general_kernel = false;  // analysis needed the sync-free kernel
};

}  // namespace gbchol

using namespace gbchol;

struct gbchol_host_factor {
    Factor F;
    CpuSolvePlan cpu;         // host solve structure, built at the first host solve
    std::once_flag cpu_once;  // (solves only read the factor and the plan: they may run concurrently)
};

struct gbchol_solver {
    int device = 0;
    int32_t n = 0;
    int32_t store = 0;
    Factor F;                 // host copy of the factor
    int64_t nnz_a = 0;
    double t_factor = 0.0, t_analysis = 0.0;
    DevBuf<int32_t> perm;
    Triangle lower, upper;    // level analysis of L (CSR, diagonal last) and L^T
    // solve plan (see host/plan.cpp), its options and a counter of rebuilds
    // (batches record it and refuse a solver whose plan changed)
    SolvePlan plan;
    PlanOptions plan_opt;
    // upper leaf sweep: each leaf row sums its top-row terms itself (no
    // separate wait-free pass launch)
    bool up_merge = true;
    int32_t plan_gen = 0;
    DevBuf<int32_t> lo_rowptr, lo_cols, lo_tasks, up_rowptr, up_cols, up_tasks, sn_rows;
    DevBuf<int32_t> upt_rowptr, upt_cols, upt_tasks;
    DevBuf<float> lo_v32, up_v32, pan32, upt_v32;
    DevBuf<double> lo_v64, up_v64, pan64, upt_v64;
    DevBuf<SnUnit> units;
    DevBuf<SnContrib> contribs;
    DevBuf<SnPartial> parts;             // lower-sweep partial sums
    DevBuf<int32_t> uflags;   // units * RHS slices
    DevBuf<int32_t> order_lo, order_up;  // units in dependency-level order
    DevBuf<int32_t> unit_of_row;         // unit holding each top row
    DevBuf<float> dinv32;
    DevBuf<double> dinv64;    // inverse diagonal blocks of the units
    // bulk supernodal sweeps (FP32, 12..128 RHS): expanded 32 x 32 L tiles,
    // the upper sweep's block lists, the lower sweep's partial sums and both
    // ticket orders (solve_snb.cu)
    DevBuf<float> snb_lo_tiles, snb_up_tiles;
    DevBuf<int32_t> snb_up_begin, snb_up_dep, snb_up_rows;
    DevBuf<int32_t> snb_unit_info, snb_order_lo, snb_order_up;
    DevBuf<SnPartial> snb_parts;
    DevBuf<SnbGroup> snb_groups;
    DevBuf<float> snb_fold2;       // per unit: M2_lo, M2_up (the second folded block of the bulk sweeps)
    int32_t snb_fold = 1;
    int32_t snb_nparts = 0;
    bool snb_ready = false;
    // RHS counts from here on use the bulk sweeps (when supported). Measured,
    // 64^3 FP32, ms per solve, bulk / 32-column: 4 RHS 3.12 / 2.82, 8 3.55 /
    // 3.36, 16 3.20 / 4.28, 32 3.44 / 5.32
    int32_t snb_min_rhs = 12;
    bool snb_tc = false;       // bulk sweeps: block products on the tensor cores
    int32_t snb_slices = 1;    // bulk sweeps: column slices per unit when not tuned (1, 2 or 4)
    bool snb_tc_groups = false;  // build the lower groups for the tensor cores (<= 32 columns)
    int32_t snb_group_cols = 0;  // source columns per lower group the tiles were built for
    // per RHS count, the sweep variant chosen by gbchol_autotune_sweeps:
    // supernodal kernel (0 sliced, 1 bulk, 2 bulk on the tensor cores), row
    // sweeps with lanes over the RHS, rows per ticket; valid = 0: defaults
    struct SweepTune {
        int8_t valid = 0, sn = 0, rhs_split = 0, chunk = 1;
    };
    SweepTune tuned[GBCHOL_MAX_RHS + 1];
    DevBuf<int32_t> counters; // [ticket, exits] per sweep kernel (5 kernels)
    DevBuf<int32_t> dev_epoch;  // sweep counter of the solve kernels (device-resident)
    std::vector<int32_t> flags_init;  // 0 for leaf rows, INT_MAX for top rows
    DevBuf<int32_t> a_rowptr, a_cols;
    DevBuf<double> a_vals;    // symmetric A, original ordering
    DevBuf<int32_t> flags, status;
    DevBuf<int32_t> max_lvl;
    int epoch = 0;
    DevBuf<unsigned char> tmp;      // permuted-space work array
    DevBuf<double> r64;             // refinement residual
    DevBuf<double> partials;        // refinement block partial sums
    DevBuf<RefineState> rstate;
    cudaStream_t last_stream = nullptr;

    int next_epoch(cudaStream_t s) {
        if (epoch >= INT_MAX - 8) {
            if (!flags_init.empty())
                cudaMemcpyAsync(flags.p, flags_init.data(), sizeof(int32_t) * flags_init.size(),
                                cudaMemcpyHostToDevice, s);
            else
                cudaMemsetAsync(flags.p, 0, sizeof(int32_t) * (size_t)std::max(n, 1), s);
            if (uflags.p) cudaMemsetAsync(uflags.p, 0, sizeof(int32_t) * uflags.count, s);
            cudaStreamSynchronize(s);
            epoch = 0;
        }
        return ++epoch;
    }
};

