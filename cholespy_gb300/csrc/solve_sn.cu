// Supernodal triangular sweeps over the top region of the factor (sm_103a).
//
// The reference solves every row in its own block and waits on one flag per
// nonzero (kernels/kernels.cu:64-202), so a dense supernode of width w costs
// w global round trips in sequence. Here the top region's columns live in
// dense column-major panels and are cut into units of <= 32 columns. One CTA
// handles one (unit, 32-RHS slice) item:
//   lower sweep: t = (b - leaf terms, prepared by the row kernel); for every
//     dense block L[unit rows, source chunk] (in source order): wait for the
//     source unit's flag, stage the block and x_source in shared memory,
//     t[rows] -= L_block x_source; then solve the 32x32 diagonal block with
//     warp shuffles (one lane per row) and publish the unit's flag.
//   upper sweep: wait for the single unit that completes every row below the
//     unit; t = y - L[below, unit]^T x_below in 32-row blocks; solve the
//     transposed diagonal block; write x (and x through perm).
// Items are assigned round-robin in topological order on a cooperatively
// launched persistent grid, so all CTAs are resident and the smallest
// unfinished item can always run: no deadlock, no ticket atomic. Waits are
// bounded (device.cuh). Work per item is deterministic (fixed block order).
#include <cuda_runtime.h>

#include "device.cuh"
#include "host/plan.h"
#include "launch.h"
#include "solve_sn.h"

namespace gbchol {

namespace {

constexpr int kT = 256;  // threads per CTA
constexpr int kW = kChunk;

template <typename T, typename TOut, bool ACCUM>
struct SnIO {
    using t = T;
    using tout = TOut;
    static constexpr bool accum = ACCUM;
};

template <typename T>
struct SnSmem {
    T t[kW][kW + 1];   // accumulator: rows x RHS
    T L[kW][kW + 1];   // staged block of L
    T x[kW][kW + 1];   // staged x rows x RHS
    int rp[kW];        // destination positions of the block's rows
};

// Waits (thread 0) for a unit flag, then makes the whole CTA proceed.
__device__ __forceinline__ void cta_wait(const int* flag, int epoch, int* status) {
    if (threadIdx.x == 0) dev::wait_geq(flag, epoch, status);
    __syncthreads();
}

template <class io, bool LOWER, bool RED>
__global__ void __launch_bounds__(kT) sn_sweep_kernel(SnSweepArgs a) {
    using T = typename io::t;
    __shared__ SnSmem<T> sm;
    if (a.skip && dev::ld_volatile(a.skip)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const T* __restrict__ panels = static_cast<const T*>(a.panels);
    T* tmp = static_cast<T*>(a.tmp);
    const int nrhs = a.nrhs;
    const int nitems = a.n_units * a.nslices;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int uidx = LOWER ? item / a.nslices : a.n_units - 1 - item / a.nslices;
        const int slice = item % a.nslices;
        const int k0 = slice * kW;
        const int kw = min(kW, nrhs - k0);
        const SnUnit U = a.units[uidx];
        const int w = U.w;

        if (!LOWER && U.upper_dep >= 0)
            cta_wait(a.uflags + (size_t)U.upper_dep * a.nslices + slice, a.epoch, a.status);

        // t <- current values of the unit's rows (lower: b minus leaf terms; upper: y)
        for (int idx = tid; idx < kW * kW; idx += kT) {
            const int i = idx >> 5, k = idx & 31;
            sm.t[i][k] = (i < w && k < kw) ? tmp[(size_t)(U.c0 + i) * nrhs + k0 + k] : T(0);
        }

        if (LOWER) {
            int waited = -1;
            for (int e = U.contrib_begin; e < U.contrib_end; ++e) {
                const SnContrib C = a.contribs[e];
                if (C.src_unit != waited) {
                    cta_wait(a.uflags + (size_t)C.src_unit * a.nslices + slice, a.epoch, a.status);
                    waited = C.src_unit;
                }
                for (int idx = tid; idx < kW * kW; idx += kT) {
                    const int i = idx & 31, j = idx >> 5;  // column-major: coalesced over rows
                    if (i < C.nr && j < C.w) sm.L[i][j] = panels[C.panel_off + i + (size_t)j * C.ld];
                    const int jj = idx >> 5, k = idx & 31;  // x rows: coalesced over RHS
                    if (jj < C.w && k < kw)
                        sm.x[jj][k] = __ldcg(tmp + (size_t)(C.xcol + jj) * nrhs + k0 + k);
                }
                if (tid < C.nr) sm.rp[tid] = a.sn_rows[C.rows_off + tid] - U.c0;
                __syncthreads();
                if (RED) {
                    // 8 threads per row split the reduction over the block's columns
                    const int i = tid >> 3, sub = tid & 7;
                    for (int k = 0; k < kw; ++k) {
                        T acc = T(0);
                        if (i < C.nr)
                            for (int j = sub; j < C.w; j += 8) acc = fma(sm.L[i][j], sm.x[j][k], acc);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 4);
                        if (sub == 0 && i < C.nr) sm.t[sm.rp[i]][k] -= acc;
                    }
                } else {
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr) {
                        const int i = warp + 8 * rr;
                        if (i < C.nr && lane < kw) {
                            T acc = T(0);
                            for (int j = 0; j < C.w; ++j) acc = fma(sm.L[i][j], sm.x[j][lane], acc);
                            sm.t[sm.rp[i]][lane] -= acc;
                        }
                    }
                }
                __syncthreads();
            }
        } else {
            const int pbeg = U.pos0 + w;
            for (int p = pbeg; p < U.ld; p += kW) {
                const int nr = min(kW, U.ld - p);
                for (int idx = tid; idx < kW * kW; idx += kT) {
                    const int i = idx & 31, j = idx >> 5;
                    if (i < nr && j < w) sm.L[i][j] = panels[U.panel_col_off + p + i + (size_t)j * U.ld];
                    const int ii = idx >> 5, k = idx & 31;
                    if (ii < nr && k < kw) {
                        const int row = a.sn_rows[U.rows_off + p + ii];
                        sm.x[ii][k] = __ldcg(tmp + (size_t)row * nrhs + k0 + k);
                    }
                }
                __syncthreads();
                if (RED) {
                    const int j = tid >> 3, sub = tid & 7;
                    for (int k = 0; k < kw; ++k) {
                        T acc = T(0);
                        if (j < w)
                            for (int i = sub; i < nr; i += 8) acc = fma(sm.L[i][j], sm.x[i][k], acc);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
                        acc += __shfl_xor_sync(0xffffffffu, acc, 4);
                        if (sub == 0 && j < w) sm.t[j][k] -= acc;
                    }
                } else {
#pragma unroll
                    for (int rr = 0; rr < 4; ++rr) {
                        const int j = warp + 8 * rr;
                        if (j < w && lane < kw) {
                            T acc = T(0);
                            for (int i = 0; i < nr; ++i) acc = fma(sm.L[i][j], sm.x[i][lane], acc);
                            sm.t[j][lane] -= acc;
                        }
                    }
                }
                __syncthreads();
            }
        }

        // diagonal block
        for (int idx = tid; idx < kW * kW; idx += kT) {
            const int i = idx & 31, j = idx >> 5;
            if (i < w && j < w) sm.L[i][j] = panels[U.panel_col_off + U.pos0 + i + (size_t)j * U.ld];
        }
        __syncthreads();
        for (int k = warp; k < kw; k += 8) {
            T v = sm.t[lane][k];
            if (LOWER) {
                for (int j = 0; j < w; ++j) {
                    const T xj = __shfl_sync(0xffffffffu, v, j) / sm.L[j][j];
                    if (lane == j) v = xj;
                    else if (lane > j) v = fma(-sm.L[lane][j], xj, v);
                }
            } else {
                for (int j = w - 1; j >= 0; --j) {
                    const T xj = __shfl_sync(0xffffffffu, v, j) / sm.L[j][j];
                    if (lane == j) v = xj;
                    else if (lane < j) v = fma(-sm.L[j][lane], xj, v);
                }
            }
            if (lane < w) {
                const size_t o = (size_t)(U.c0 + lane) * nrhs + k0 + k;
                tmp[o] = v;
                if (!LOWER) {
                    using TO = typename io::tout;
                    TO* out = static_cast<TO*>(a.out);
                    const size_t oo = (size_t)a.perm[U.c0 + lane] * nrhs + k0 + k;
                    if (io::accum) out[oo] += (TO)v;
                    else out[oo] = (TO)v;
                }
            }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) dev::st_release(a.uflags + (size_t)uidx * a.nslices + slice, a.epoch);
    }
}

template <class io, bool LOWER>
cudaError_t launch_sn_io(const SnSweepArgs& a, cudaStream_t stream) {
    const bool red = a.nrhs <= 8;
    const void* fn = red ? (const void*)sn_sweep_kernel<io, LOWER, true>
                         : (const void*)sn_sweep_kernel<io, LOWER, false>;
    int grid = 0;
    cudaError_t e = coop_grid(fn, kT, 0, &grid);
    if (e != cudaSuccess) return e;
    const int items = a.n_units * a.nslices;
    if (grid > items) grid = items;
    SnSweepArgs copy = a;
    void* args[] = {&copy};
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kT), args, 0, stream);
}

}  // namespace

int sn_slices(int nrhs) { return nrhs <= 8 ? 1 : (nrhs + kW - 1) / kW; }

cudaError_t launch_sn_sweep(const SnSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream) {
    if (a.n_units == 0) return cudaSuccess;
    switch (io) {
        case SweepIO::F32:
            return lower ? launch_sn_io<SnIO<float, float, false>, true>(a, stream)
                         : launch_sn_io<SnIO<float, float, false>, false>(a, stream);
        case SweepIO::F64:
            return lower ? launch_sn_io<SnIO<double, double, false>, true>(a, stream)
                         : launch_sn_io<SnIO<double, double, false>, false>(a, stream);
        case SweepIO::F32_MIXED:
            return lower ? launch_sn_io<SnIO<float, double, false>, true>(a, stream)
                         : launch_sn_io<SnIO<float, double, false>, false>(a, stream);
        case SweepIO::F32_REFINE:
            return lower ? launch_sn_io<SnIO<float, double, true>, true>(a, stream)
                         : launch_sn_io<SnIO<float, double, true>, false>(a, stream);
    }
    return cudaErrorInvalidValue;
}

}  // namespace gbchol
