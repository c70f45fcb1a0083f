// Row-wise, sync-free sparse triangular sweeps (sm_103a).
//
// Same mathematics as the reference's solve_lower / solve_upper
// (kernels/kernels.cu:64-202): rows are visited in level order, each row
// waits for the rows it depends on and then publishes its own value through
// a flag. GB300 design differences:
//   * one WARP per row instead of one 128-thread block per row, and no
//     __syncthreads per nonzero: for up to 8 RHS the lanes split the row's
//     nonzeros (coalesced index/value loads, warp-shuffle reduction); for more
//     RHS the lanes split the RHS columns, so x loads are coalesced, and the
//     row's (col, val) pairs are loaded 32 at a time and broadcast by shuffle;
//   * flags of a batch of entries are read together, one acquire load per
//     lane (no dependent acquire per nonzero, no separate fence);
//   * persistent grid; warps take tasks (in level order) by an atomic ticket,
//     so a warp only waits on tasks with smaller tickets, all taken by running
//     warps (no deadlock); the last warp out resets the ticket;
//   * one launch can sweep many systems (a batch): each task names its
//     system, whose arrays come from a descriptor table;
//   * the upper leaf sweep's rows first sum the terms that were final before
//     the launch (the top rows' x, from a second CSR) with no flag checks, so
//     those gathers overlap the waits of the leaf chain;
//   * flags carry an epoch kept in device memory (read at kernel start,
//     advanced by the last warp out), so no per-solve memset of the flags
//     and the sweeps can be captured in a CUDA graph and replayed;
//   * bounded waits (device.cuh).
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.h"
#include "launch.h"

namespace gbchol {

namespace {

template <typename T, typename TIn, typename TOut, bool ACCUM>
struct IO {
    using t = T;
    using tin = TIn;
    using tout = TOut;
    static constexpr bool accum = ACCUM;
};

// Writes the solved value of (row, j) in permuted space and, for the upper
// sweep, to the user array through perm.
template <class io, bool LOWER>
__device__ __forceinline__ void emit(const RowSys& d, int row, int prow, int j, typename io::t v,
                                     bool partial) {
    using T = typename io::t;
    static_cast<T*>(d.tmp)[(size_t)row * d.nrhs + j] = v;
    if (!LOWER && !partial) {
        using TO = typename io::tout;
        TO* out = static_cast<TO*>(d.out);
        const size_t o = (size_t)prow * d.nrhs + j;
        if (io::accum) out[o] += (TO)v;
        else out[o] = (TO)v;
    }
}

template <class io, bool LOWER>
__device__ __forceinline__ typename io::t load_rhs(const RowSys& d, int row, int prow, int j) {
    using T = typename io::t;
    if (LOWER) return (T) static_cast<const typename io::tin*>(d.in)[(size_t)prow * d.nrhs + j];
    return static_cast<const T*>(d.tmp)[(size_t)row * d.nrhs + j];
}

// Lanes split the nonzeros of the row (entries [s, e) of its CSR row); R >=
// nrhs accumulators per lane. The row's own loads (perm, diagonal, right-hand
// side) go out before the waits on its dependencies.
template <class io, bool LOWER, int R>
__device__ __forceinline__ void row_nnz(const RowSys& d, int task, int s, int e, int epoch, int* status,
                                        int lane) {
    using T = typename io::t;
    const T* __restrict__ vals = static_cast<const T*>(d.vals);
    const T* tmp = static_cast<const T*>(d.tmp);
    const int nrhs = d.nrhs;
    const bool partial = task < 0;
    const int row = partial ? ~task : task;
    const int lo = (LOWER || partial) ? s : s + 1;
    const int hi = (LOWER && !partial) ? e - 1 : e;
    const T diag = partial ? T(1) : vals[LOWER ? e - 1 : s];
    const int prow = d.perm[row];
    const T rhs = lane < nrhs ? load_rhs<io, LOWER>(d, row, prow, lane) : T(0);
    T acc[R];
#pragma unroll
    for (int j = 0; j < R; ++j) acc[j] = T(0);
    if (!LOWER && !partial && d.nw_rowptr) {  // terms final before the launch: no flag checks
        const T* nv = static_cast<const T*>(d.nw_vals);
        const int ne = d.nw_rowptr[row + 1];
        for (int k = d.nw_rowptr[row] + lane; k < ne; k += 32) {
            const T v = nv[k];
            const T* xc = tmp + (size_t)d.nw_cols[k] * nrhs;
#pragma unroll
            for (int j = 0; j < R; ++j)
                if (j < nrhs) acc[j] = fma(v, __ldcg(xc + j), acc[j]);
        }
    }
    for (int base = lo; base < hi; base += 64) {
        // two entries per lane: flags checked together, then one fence
        int c[2];
        T v[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int k = base + lane + 32 * u;
            c[u] = k < hi ? d.cols[k] : -1;
            v[u] = k < hi ? vals[k] : T(0);
        }
        // acquire loads of the flags (no separate fence); a flag not yet set
        // is waited for with acquire loads too
        int f[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) f[u] = c[u] >= 0 ? dev::ld_acquire(d.flags + c[u]) : epoch;
#pragma unroll
        for (int u = 0; u < 2; ++u)
            if (f[u] < epoch) dev::wait_geq(d.flags + c[u], epoch, status);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            if (c[u] < 0) continue;
            const T* xc = tmp + (size_t)c[u] * nrhs;
#pragma unroll
            for (int j = 0; j < R; ++j)
                if (j < nrhs) acc[j] = fma(v[u], __ldcg(xc + j), acc[j]);
        }
    }
    T mine = T(0);
#pragma unroll
    for (int j = 0; j < R; ++j) {
        T sj = dev::warp_sum(acc[j]);
        if (j == lane) mine = sj;
    }
    if (lane < nrhs) {
        T v = rhs - mine;
        if (!partial) v = v / diag;
        emit<io, LOWER>(d, row, prow, lane, v, partial);
    }
    // partial rows publish nothing; the warp barrier orders the lanes'
    // writes before lane 0's release
    __syncwarp();
    if (lane == 0 && !partial) {
        dev::st_release(d.flags + row, epoch);
    }
}

// Lanes split the RHS columns: G lanes per group (32/G groups take
// alternating nonzeros), Q RHS columns per lane (nrhs <= G*Q).
template <class io, bool LOWER, int G, int Q>
__device__ __forceinline__ void row_rhs(const RowSys& d, int task, int s, int e, int epoch, int* status,
                                        int lane) {
    using T = typename io::t;
    constexpr int NG = 32 / G;
    const int grp = lane / G, sub = lane % G;
    const T* __restrict__ vals = static_cast<const T*>(d.vals);
    const T* tmp = static_cast<const T*>(d.tmp);
    const int nrhs = d.nrhs;
    const bool partial = task < 0;
    const int row = partial ? ~task : task;
    const int lo = (LOWER || partial) ? s : s + 1;
    const int hi = (LOWER && !partial) ? e - 1 : e;
    const T diag = partial ? T(1) : vals[LOWER ? e - 1 : s];
    const int prow = d.perm[row];
    T rhs[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = sub + q * G;
        rhs[q] = (grp == 0 && j < nrhs) ? load_rhs<io, LOWER>(d, row, prow, j) : T(0);
    }
    T acc[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = T(0);
    // the warp consumes `cnt` entries held one per lane (column, value)
    auto consume = [&](int mycol, T myv, int cnt) {
        const int steps = (cnt + NG - 1) / NG;
#pragma unroll 8
        for (int st = 0; st < steps; ++st) {
            const int eidx = st * NG + grp;
            const bool valid = eidx < cnt;
            const int col = __shfl_sync(0xffffffffu, mycol, valid ? eidx : 0);
            const T v = __shfl_sync(0xffffffffu, myv, valid ? eidx : 0);
            if (!valid) continue;
            const T* xc = tmp + (size_t)col * nrhs;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int j = sub + q * G;
                if (j < nrhs) acc[q] = fma(v, __ldcg(xc + j), acc[q]);
            }
        }
    };
    if (!LOWER && !partial && d.nw_rowptr) {  // terms final before the launch: no flag checks
        const T* nv = static_cast<const T*>(d.nw_vals);
        const int ns = d.nw_rowptr[row], ne = d.nw_rowptr[row + 1];
        for (int base = ns; base < ne; base += 32) {
            const int k = base + lane;
            consume(k < ne ? d.nw_cols[k] : 0, k < ne ? nv[k] : T(0), min(32, ne - base));
        }
    }
    for (int base = lo; base < hi; base += 32) {
        const int k = base + lane;
        const int mycol = k < hi ? d.cols[k] : 0;
        const T myv = k < hi ? vals[k] : T(0);
        // every lane waits for its own entry, then the warp consumes the 32
        // entries without further waits (independent loads in flight)
        if (k < hi && dev::ld_acquire(d.flags + mycol) < epoch)
            dev::wait_geq(d.flags + mycol, epoch, status);
        __syncwarp();  // orders every lane's observation before the warp's x loads
        consume(mycol, myv, min(32, hi - base));
    }
    if (NG > 1) {
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
            for (int o = G; o < 32; o <<= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
    }
    if (grp == 0) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int j = sub + q * G;
            if (j < nrhs) {
                T v = rhs[q] - acc[q];
                if (!partial) v = v / diag;
                emit<io, LOWER>(d, row, prow, j, v, partial);
            }
        }
    }
    __syncwarp();
    if (lane == 0 && !partial) {
        dev::st_release(d.flags + row, epoch);
    }
}

// MODE 1/2/4/8: nonzero-split with that many accumulators; 16: RHS-split
// 16 lanes; 32/64/128: RHS-split 32 lanes x 1/2/4 columns; 0: per-system
// choice (batched sweeps with mixed RHS counts).
template <class io, bool LOWER, int MODE>
__global__ void __launch_bounds__(256) row_sweep_kernel(RowSweepArgs a) {
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    if (a.skip && dev::ld_volatile(a.skip)) return;
    // every warp reads the sweep's epoch before the last warp out bumps it
    const int epoch = dev::ld_volatile(a.epoch);
    auto run = [&](const RowSys& d, int task, int s, int e) {
        if (MODE == 1) row_nnz<io, LOWER, 1>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 2) row_nnz<io, LOWER, 2>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 4) row_nnz<io, LOWER, 4>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 8) row_nnz<io, LOWER, 8>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 16) row_rhs<io, LOWER, 16, 1>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 32) row_rhs<io, LOWER, 32, 1>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 64) row_rhs<io, LOWER, 32, 2>(d, task, s, e, epoch, a.status, lane);
        else if (MODE == 128) row_rhs<io, LOWER, 32, 4>(d, task, s, e, epoch, a.status, lane);
        else if (a.batched_variant >= 2) {  // the variant fitted to the system's RHS count
            if (d.nrhs <= 1) row_nnz<io, LOWER, 1>(d, task, s, e, epoch, a.status, lane);
            else if (d.nrhs <= 16) row_rhs<io, LOWER, 16, 1>(d, task, s, e, epoch, a.status, lane);
            else if (d.nrhs <= 32) row_rhs<io, LOWER, 32, 1>(d, task, s, e, epoch, a.status, lane);
            else if (d.nrhs <= 64) row_rhs<io, LOWER, 32, 2>(d, task, s, e, epoch, a.status, lane);
            else row_rhs<io, LOWER, 32, 4>(d, task, s, e, epoch, a.status, lane);
        } else {
            if (d.nrhs <= 8) row_nnz<io, LOWER, 8>(d, task, s, e, epoch, a.status, lane);
            else row_rhs<io, LOWER, 32, 4>(d, task, s, e, epoch, a.status, lane);
        }
    };
    auto row_range = [&](const RowSys& d, int task, int& s, int& e) {
        const int row = task < 0 ? ~task : task;
        s = d.rowptr[row];
        e = d.rowptr[row + 1];
    };
    if (a.chunk == 1 && !a.task_sys) {
        // One task per ticket, the next ticket, task and row range fetched
        // while the current row is solved (a warp holds at most two tickets
        // and solves them in ticket order, so waits still point only to
        // smaller tickets).
        int t = 0;
        if (lane == 0) t = atomicAdd(a.counters, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        int task = 0, s = 0, e = 0;
        if (t < a.ntasks) {
            task = a.tasks[t];
            row_range(a.sys0, task, s, e);
        }
        while (t < a.ntasks) {
            int tn = 0;
            if (lane == 0) tn = atomicAdd(a.counters, 1);
            tn = __shfl_sync(0xffffffffu, tn, 0);
            int taskn = 0, sn = 0, en = 0;
            if (tn < a.ntasks) {
                taskn = a.tasks[tn];
                row_range(a.sys0, taskn, sn, en);
            }
            run(a.sys0, task, s, e);
            t = tn;
            task = taskn;
            s = sn;
            e = en;
        }
    } else {
        for (;;) {
            int t0 = 0;
            if (lane == 0) t0 = atomicAdd(a.counters, 1) * a.chunk;
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            if (t0 >= a.ntasks) break;
            const int tend = min(a.ntasks, t0 + a.chunk);
            for (int t = t0; t < tend; ++t) {
                const int task = a.tasks[t];
                const RowSys d = a.task_sys ? a.sys[a.task_sys[t]] : a.sys0;
                int s, e;
                row_range(d, task, s, e);
                run(d, task, s, e);
            }
        }
    }
    // the last warp out resets the ticket and advances the epoch for the
    // next launch (the launch boundary orders these writes)
    if (lane == 0) {
        __threadfence();
        if (atomicAdd(a.counters + 1, 1) == nwarps - 1) {
            a.counters[0] = 0;
            a.counters[1] = 0;
            *a.epoch = epoch + 1;
        }
    }
}

template <class io, bool LOWER>
cudaError_t launch_io(const RowSweepArgs& a, cudaStream_t stream) {
    const void* fn;
    const int r = a.max_nrhs;
    if (a.batched_variant) fn = (const void*)row_sweep_kernel<io, LOWER, 0>;
    else if (a.rhs_split && r <= 16) fn = (const void*)row_sweep_kernel<io, LOWER, 16>;
    else if (r <= 1) fn = (const void*)row_sweep_kernel<io, LOWER, 1>;
    else if (r <= 2) fn = (const void*)row_sweep_kernel<io, LOWER, 2>;
    else if (r <= 4) fn = (const void*)row_sweep_kernel<io, LOWER, 4>;
    else if (r <= 8) fn = (const void*)row_sweep_kernel<io, LOWER, 8>;
    else if (r <= 16) fn = (const void*)row_sweep_kernel<io, LOWER, 16>;
    else if (r <= 32) fn = (const void*)row_sweep_kernel<io, LOWER, 32>;
    else if (r <= 64) fn = (const void*)row_sweep_kernel<io, LOWER, 64>;
    else fn = (const void*)row_sweep_kernel<io, LOWER, 128>;
    int grid = 0;
    cudaError_t e = coop_grid(fn, 256, 0, &grid);  // resident blocks: a persistent grid
    if (e != cudaSuccess) return e;
    const int need = (a.ntasks + 8 * a.chunk - 1) / (8 * a.chunk);
    if (grid > need) grid = need;
    RowSweepArgs copy = a;
    void* args[] = {&copy};
    return cudaLaunchKernel(fn, dim3(grid), dim3(256), args, 0, stream);
}

}  // namespace

cudaError_t launch_row_sweep(const RowSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream) {
    if (a.ntasks == 0) return cudaSuccess;
    switch (io) {
        case SweepIO::F32:
            return lower ? launch_io<IO<float, float, float, false>, true>(a, stream)
                         : launch_io<IO<float, float, float, false>, false>(a, stream);
        case SweepIO::F64:
            return lower ? launch_io<IO<double, double, double, false>, true>(a, stream)
                         : launch_io<IO<double, double, double, false>, false>(a, stream);
        case SweepIO::F32_MIXED:
            return lower ? launch_io<IO<float, double, double, false>, true>(a, stream)
                         : launch_io<IO<float, double, double, false>, false>(a, stream);
        case SweepIO::F32_REFINE:
            return lower ? launch_io<IO<float, double, double, true>, true>(a, stream)
                         : launch_io<IO<float, double, double, true>, false>(a, stream);
    }
    return cudaErrorInvalidValue;
}

}  // namespace gbchol
