// Supernodal triangular sweeps over the top region of the factor (sm_103a).
//
// The reference solves every row in its own block and waits on one flag per
// nonzero (kernels/kernels.cu:64-202), so a dense supernode of width w costs
// w global round trips in sequence. Here the top region's columns live in
// dense column-major panels cut into units of <= 32 columns, and one CTA
// handles one (unit, RHS slice) item. The unit's 32 rows map to the 32 lanes.
//
// Lower sweep (L y = b): every dense block L[unit rows, source chunk] that
//   hits the unit (listed in source order) is taken by one of the 8 warps
//   (block b -> warp b % 8). The warp waits for the source unit's flag,
//   stages x_source (<= 32 x 32) in its own shared-memory slice, and each
//   lane accumulates its row of L_block x_source in registers. The rows of a
//   block are a sorted subset of the unit's rows, given as a 32-bit mask, so
//   lane p reads block row popc(mask below p) directly (no scatter). Long
//   block lists are cut into partial-sum items (other CTAs, started as soon
//   as their sources are done); the unit adds their sums. The warps' sums
//   are reduced in a fixed order, subtracted from t (b minus leaf terms),
//   and the 32x32 diagonal block is solved (one lane per row).
// Upper sweep (L^T x = y): the rows below the unit's diagonal block are cut
//   into 32-row blocks: the supernode's off-diagonal rows first, highest
//   block first, then the later chunks of the same supernode from the last
//   one down. Each block waits for one unit only: the off-diagonal rows of a
//   supernode lie on one etree path, and the unit holding a block's lowest
//   row finishes after every higher row of the path; so only the newest
//   32-row block sits on the dependency chain. Lane j holds
//   column j of the unit and accumulates L[block, j]^T x_block; then the same
//   fixed-order reduction and a transposed solve.
// The diagonal solve of a unit is one product with the precomputed inverse
// of its 32x32 diagonal block (no 32-step substitution on the dependency
// chain), and the block on the chain itself (from the neighbouring chunk of
// the same supernode) is folded into it: x = D^{-1} t' - M x_chain with M
// precomputed (host, FP64), so that after the chain wait a unit does one
// 32x32 product per RHS column, a warp per column, with no reduction across
// warps. Items are handed out by an atomic ticket in dependency-level order
// to a persistent grid: a CTA only waits on items with smaller tickets, all
// of which were taken by running CTAs, so there is no deadlock; the last CTA
// to leave resets the counters for the next launch. Waits are bounded
// (device.cuh). Results are deterministic: fixed block-to-warp assignment and
// fixed reduction order.
#include <cuda_runtime.h>

#include "device.cuh"
#include "host/plan.h"
#include "launch.h"
#include "solve_sn.h"

namespace gbchol {

namespace {

constexpr int kT = 256;    // threads per CTA
constexpr int kWarps = kT / 32;
constexpr int kW = kChunk; // 32 rows / columns per unit

template <typename T, typename TOut, bool ACCUM>
struct SnIO {
    using t = T;
    using tout = TOut;
    static constexpr bool accum = ACCUM;
};

// Row stride of the x staging area: a multiple of 16 bytes so that a row
// can be read with 16-byte vector loads (all lanes read the same row:
// broadcast), plus 16 bytes of skew against bank conflicts in the reduction.
template <typename T, int KW>
struct XsStride {
    static constexpr int value = KW + 16 / (int)sizeof(T);
};

template <typename T, int KW>
struct SnSmem {
    static constexpr int XS = XsStride<T, KW>::value;
    __align__(16) T xs[kWarps][kW][XS];  // per-warp staging of x blocks; reused for the reduction
    T t[kW][KW + 1];           // reduced right-hand side of the unit
    T d[kW][kW + 1];           // inverse diagonal block
    T m[kW][kW + 1];           // chain block folded into the diagonal solve (M_lo / M_up)
};

// acc[k] += a * row[k] for k < KW, reading `row` (16-byte aligned shared
// memory, same address in every lane) with 16-byte vector loads.
template <int KW>
__device__ __forceinline__ void axpy_row(float (&acc)[KW], float a, const float* row) {
#pragma unroll
    for (int k = 0; k < KW; k += 4) {
        const float4 v = *reinterpret_cast<const float4*>(row + k);
        acc[k] = fmaf(a, v.x, acc[k]);
        acc[k + 1] = fmaf(a, v.y, acc[k + 1]);
        acc[k + 2] = fmaf(a, v.z, acc[k + 2]);
        acc[k + 3] = fmaf(a, v.w, acc[k + 3]);
    }
}
template <int KW>
__device__ __forceinline__ void axpy_row(double (&acc)[KW], double a, const double* row) {
#pragma unroll
    for (int k = 0; k < KW; k += 2) {
        const double2 v = *reinterpret_cast<const double2*>(row + k);
        acc[k] = fma(a, v.x, acc[k]);
        acc[k + 1] = fma(a, v.y, acc[k + 1]);
    }
}

// Lane 0 waits for a flag; the warp proceeds together. Loads of data
// published under the flag use ld.cg (L2), which holds the producer's
// writes once the flag is observed.
__device__ __forceinline__ void warp_wait(const int* flag, int epoch, int* status, int lane) {
    if (lane == 0) dev::wait_geq(flag, epoch, status);
    __syncwarp();
}

// One warp's share of a lower-sweep block: inner columns [j0, j0 + J) of
// L[unit rows, source chunk] times the matching rows of x_source, added into
// acc (lane = unit row); J = 32: the whole block. Lane p holds block row
// popc(rowmask below p) when bit p of rowmask is set. `ready`: the source's
// flag was already seen set (no wait).
template <typename T, int KW, int J>
__device__ __forceinline__ void lower_block(const SnSys& d, long long panel_off, int ld, int xcol, int w,
                                            int src_unit, unsigned rowmask, bool ready, int j0, int slice,
                                            int k0, int kw, int epoch, int* status, int lane,
                                            T (*xs)[XsStride<T, KW>::value], T (&acc)[KW]) {
    const T* __restrict__ panels = static_cast<const T*>(d.panels);
    const T* tmp = static_cast<const T*>(d.tmp);
    const int nrhs = d.nrhs;
    const bool hit = (rowmask >> lane) & 1u;
    const int src = __popc(rowmask & ((1u << lane) - 1u));
    // L is constant: its loads go out before the flag wait
    T lv[J];
    const T* Lp = panels + panel_off + src;
#pragma unroll
    for (int j = 0; j < J; ++j) lv[j] = (hit && j0 + j < w) ? __ldg(Lp + (size_t)(j0 + j) * ld) : T(0);
    if (!ready) warp_wait(d.uflags + (size_t)src_unit * d.nslices + slice, epoch, status, lane);
    constexpr int PER = J * KW / 32;
    T xv[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int idx = lane + 32 * u, j = j0 + idx / KW, k = idx % KW;
        xv[u] = (j < w && k < kw) ? __ldcg(tmp + (size_t)(xcol + j) * nrhs + k0 + k) : T(0);
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int idx = lane + 32 * u;
        xs[idx / KW][idx % KW] = xv[u];
    }
    __syncwarp();
    const int jn = min(J, w - j0);  // warp-uniform
#pragma unroll
    for (int j = 0; j < J; ++j) {
        if (j >= jn) break;
        axpy_row<KW>(acc, lv[j], xs[j]);
    }
    __syncwarp();
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// One warp's blocks first, first + 8, ... < end of a lower-sweep block list,
// whole blocks. They go in groups of up to 32: lane k loads the descriptor
// of the group's k-th block and checks its source's flag (one round trip for
// the group), the descriptors are broadcast by shuffles, and the next
// block's L columns are prefetched into L2 while the current one is applied.
template <typename T, int KW>
__device__ __forceinline__ void lower_list(const SnSys& d, int first, int end, int slice, int k0, int kw,
                                           int epoch, int* status, int lane,
                                           T (*xs)[XsStride<T, KW>::value], T (&acc)[KW]) {
    const T* __restrict__ panels = static_cast<const T*>(d.panels);
    for (int g = first; g < end; g += 32 * kWarps) {
        const int mb = g + lane * kWarps;
        long long poff = 0;
        int ld = 0, xcol = 0, w = 0, nr = 0, srcu = 0;
        unsigned mask = 0;
        int ready = 1;
        if (mb < end) {
            const SnContrib& C = d.contribs[mb];
            poff = C.panel_off;
            ld = C.ld;
            xcol = C.xcol;
            w = C.w;
            nr = C.nr;
            srcu = C.src_unit;
            mask = C.rowmask;
            ready = dev::ld_acquire(d.uflags + (size_t)srcu * d.nslices + slice) >= epoch;
        }
        __syncwarp();  // orders the lanes' flag observations before every lane's loads
        const int cnt = min(32, (end - g + kWarps - 1) / kWarps);
        for (int k = 0; k < cnt; ++k) {
            if (k + 1 < cnt) {
                const long long np = __shfl_sync(0xffffffffu, poff, k + 1);
                const int nld = __shfl_sync(0xffffffffu, ld, k + 1);
                const int nw = __shfl_sync(0xffffffffu, w, k + 1);
                const int nnr = __shfl_sync(0xffffffffu, nr, k + 1);
                if (lane < nw) {
                    prefetch_l2(panels + np + (size_t)lane * nld);
                    prefetch_l2(panels + np + nnr - 1 + (size_t)lane * nld);
                }
            }
            lower_block<T, KW, kW>(d, __shfl_sync(0xffffffffu, poff, k), __shfl_sync(0xffffffffu, ld, k),
                                   __shfl_sync(0xffffffffu, xcol, k), __shfl_sync(0xffffffffu, w, k),
                                   __shfl_sync(0xffffffffu, srcu, k), __shfl_sync(0xffffffffu, mask, k),
                                   __shfl_sync(0xffffffffu, ready, k) != 0, 0, slice, k0, kw, epoch, status,
                                   lane, xs, acc);
        }
    }
}

// One warp's share of an upper-sweep block: rows [i0, i0 + J) of the 32-row
// block starting at row position p0 of the supernode, L[rows, unit]^T times
// x[rows], added into acc (lane = unit column).
template <typename T, int KW, int J>
__device__ __forceinline__ void upper_block(const SnSys& d, const SnUnit& U, int p0, int nr, int i0,
                                            int dep, int slice, int k0, int kw, int epoch,
                                            int* status, int lane, T (*xs)[XsStride<T, KW>::value], T (&acc)[KW]) {
    const T* __restrict__ panels = static_cast<const T*>(d.panels);
    const T* tmp = static_cast<const T*>(d.tmp);
    const int nrhs = d.nrhs;
    T lv[J];
    const T* Lp = panels + U.panel_col_off + p0 + i0 + (size_t)lane * U.ld;
#pragma unroll
    for (int i = 0; i < J; ++i) lv[i] = (lane < U.w && i0 + i < nr) ? __ldg(Lp + i) : T(0);
    const int myrow = (lane < J && i0 + lane < nr) ? d.sn_rows[U.rows_off + p0 + i0 + lane] : 0;
    if (dep >= 0) warp_wait(d.uflags + (size_t)dep * d.nslices + slice, epoch, status, lane);
    constexpr int PER = J * KW / 32;
    T xv[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int idx = lane + 32 * u, i = idx / KW, k = idx % KW;
        const int row = __shfl_sync(0xffffffffu, myrow, i);
        xv[u] = (i0 + i < nr && k < kw) ? __ldcg(tmp + (size_t)row * nrhs + k0 + k) : T(0);
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int idx = lane + 32 * u;
        xs[idx / KW][idx % KW] = xv[u];
    }
    __syncwarp();
    const int in = min(J, nr - i0);  // warp-uniform
#pragma unroll
    for (int i = 0; i < J; ++i) {
        if (i >= in) break;
        axpy_row<KW>(acc, lv[i], xs[i]);
    }
    __syncwarp();
}

template <class io, bool LOWER, int KW>
__global__ void __launch_bounds__(kT, 2) sn_sweep_kernel(SnSweepArgs a) {
    using T = typename io::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SnSmem<T, KW>& sm = *reinterpret_cast<SnSmem<T, KW>*>(smem_raw);
    if (a.skip && dev::ld_volatile(a.skip)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nitems = a.nitems;
    // every CTA reads the sweep's epoch before the last CTA out bumps it
    const int epoch = dev::ld_volatile(a.epoch);
    T (*xs)[XsStride<T, KW>::value] = sm.xs[warp];
    __shared__ int ticket, s_uidx, s_slice;
    __shared__ SnSys dsm;
    for (;;) {
        if (tid == 0) {
            const int it = atomicAdd(a.counters, 1);
            ticket = it;
            if (it < nitems) {
                if (a.item_sys) {
                    dsm = a.sys[a.item_sys[it]];
                    const int code = a.item_code[it];
                    if (code >= 0) {
                        s_uidx = code >> 3;
                        s_slice = code & 7;
                    } else {  // partial sum
                        s_uidx = ~(((-code) >> 3) - 1);
                        s_slice = (-code) & 7;
                    }
                } else {
                    dsm = a.sys0;
                    s_uidx = a.order[it / a.sys0.nslices];
                    s_slice = it % a.sys0.nslices;
                }
            }
        }
        __syncthreads();
        // thread 0 rewrites these only after the end-of-item barrier
        if (ticket >= nitems) break;
        const SnSys& d = dsm;
        const int uidx = s_uidx, slice = s_slice;
        T* tmp = static_cast<T*>(d.tmp);
        const int nrhs = d.nrhs;
        const int k0 = slice * KW;
        const int kw = min(KW, nrhs - k0);
        // a lower-sweep partial sum: the item is ~p
        const bool part = LOWER && uidx < 0;
        const SnPartial PS = part ? d.parts[~uidx] : SnPartial{};
        const SnUnit U = d.units[part ? PS.unit : uidx];
        const int w = U.w;
        // off the dependency chain: the unit's current right-hand side and
        // its inverse diagonal block go to shared memory first
        // the chain input: lower, the previous chunk of the supernode; upper,
        // the next one (both the neighbouring unit)
        const bool chain = !part && (LOWER ? U.pos0 > 0 : U.pos0 + w < U.sn_w);
        if (!part) {
            const T* __restrict__ dinv = static_cast<const T*>(d.dinv) + (size_t)uidx * 3 * kW * kW;
            for (int idx = tid; idx < kW * kW; idx += kT) sm.d[idx & 31][idx >> 5] = dinv[idx];
            if (chain) {
                const T* __restrict__ mc = dinv + (LOWER ? 1 : 2) * kW * kW;
                for (int idx = tid; idx < kW * kW; idx += kT) sm.m[idx & 31][idx >> 5] = mc[idx];
            }
            for (int idx = tid; idx < kW * KW; idx += kT) {
                const int i = idx / KW, k = idx % KW;
                sm.t[i][k] = (i < w && k < kw) ? tmp[(size_t)(U.c0 + i) * nrhs + k0 + k] : T(0);
            }
        }
        T acc[KW];
#pragma unroll
        for (int k = 0; k < KW; ++k) acc[k] = T(0);

        // Every block but the one on the dependency chain (lower: from the
        // previous chunk of the same supernode, listed last; upper: from the
        // next chunk) goes to a warp in turn; the chain block is folded into
        // the diagonal solve below.
        if (part) {
            lower_list<T, KW>(d, PS.contrib_begin + warp, PS.contrib_end, slice, k0, kw, epoch, a.status, lane,
                              xs, acc);
        } else if (LOWER) {
            // the unit's partial sums, one per warp in turn (slot row = lane)
            for (int q = U.part_begin + warp; q < U.part_end; q += kWarps) {
                warp_wait(d.uflags + (size_t)(d.n_units + q) * d.nslices + slice, epoch, a.status, lane);
                const T* ps = static_cast<const T*>(d.pbuf) + ((size_t)q * d.nslices + slice) * (kW * KW) + lane * KW;
#pragma unroll
                for (int k = 0; k < KW; ++k) acc[k] += __ldcg(ps + k);
            }
            const int nb = U.contrib_end - U.contrib_begin;
            const int nfree = chain ? nb - 1 : nb;  // the chain block is the list's last
            lower_list<T, KW>(d, U.contrib_begin + warp, U.contrib_begin + nfree, slice, k0, kw, epoch, a.status,
                              lane, xs, acc);
        } else {
            // block list: off-diagonal rows of the supernode in 32-row blocks,
            // highest rows first (they are solved first), each waiting for the
            // unit of its lowest row; then the later chunks of the supernode,
            // last chunk first, but the next one (the chain)
            const int wj = U.pos0 + w;                      // end of this unit's columns
            const int sn_w = U.sn_w;                        // supernode width
            const int nrb = (U.ld - sn_w + kW - 1) / kW;    // off-diagonal row blocks
            const int nlater = (sn_w - wj + kW - 1) / kW;   // later chunks
            const int nfree = nrb + nlater - (chain ? 1 : 0);
            for (int b = warp; b < nfree; b += kWarps) {
                int p0, nr, dep;
                if (b < nrb) {
                    p0 = sn_w + (nrb - 1 - b) * kW;
                    nr = min(kW, U.ld - p0);
                    dep = d.unit_of_row[d.sn_rows[U.rows_off + p0]];
                } else {
                    const int c = nlater - 1 - (b - nrb);  // later chunk index, last first
                    p0 = wj + c * kW;
                    nr = min(kW, sn_w - p0);
                    dep = uidx + 1 + c;
                }
                upper_block<T, KW, kW>(d, U, p0, nr, 0, dep, slice, k0, kw, epoch, a.status, lane, xs, acc);
            }
        }

        // fixed-order reduction of the warps' partial sums
#pragma unroll
        for (int k = 0; k < KW; ++k) xs[lane][k] = acc[k];
        __syncthreads();
        if (part) {  // the sum goes to the partial's slot, then its flag
            T* ps = static_cast<T*>(d.pbuf) + ((size_t)(~uidx) * d.nslices + slice) * (kW * KW);
            for (int idx = tid; idx < kW * KW; idx += kT) {
                const int i = idx / KW, k = idx % KW;
                T v = T(0);
#pragma unroll
                for (int ww = 0; ww < kWarps; ++ww) v += sm.xs[ww][i][k];
                ps[idx] = v;
            }
            __syncthreads();
            if (tid == 0) {
                dev::st_release(d.uflags + (size_t)(d.n_units + ~uidx) * d.nslices + slice, epoch);
            }
            continue;
        }
        for (int idx = tid; idx < kW * KW; idx += kT) {
            const int i = idx / KW, k = idx % KW;
            T s = T(0);
#pragma unroll
            for (int ww = 0; ww < kWarps; ++ww) s += sm.xs[ww][i][k];
            sm.t[i][k] -= s;
        }
        __syncthreads();
        // diagonal block: x = D^{-1} t (lower) or D^{-T} t (upper), lane =
        // row, RHS columns warp, warp + 8, ...; then, once the chain unit's
        // flag is seen, the chain term x -= M x_chain, x_chain (the
        // neighbouring unit's solution) broadcast from lane j by shuffles
        constexpr int KPW = (KW + kWarps - 1) / kWarps;  // RHS columns per warp
        T xv[KPW];
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = warp + q * kWarps;
            T v = T(0);
            if (k < kw) {
                if (LOWER) {
#pragma unroll 8
                    for (int j = 0; j < kW; ++j) v = fma(sm.d[lane][j], sm.t[j][k], v);
                } else {
#pragma unroll 8
                    for (int j = 0; j < kW; ++j) v = fma(sm.d[j][lane], sm.t[j][k], v);
                }
            }
            xv[q] = v;
        }
        if (chain && warp < kw) {
            const int cu = LOWER ? uidx - 1 : uidx + 1;                 // chain unit
            const int crow = LOWER ? U.c0 - kW : U.c0 + w;              // its first row
            const int cw = LOWER ? kW : min(kW, U.sn_w - (U.pos0 + w)); // its width
            warp_wait(d.uflags + (size_t)cu * d.nslices + slice, epoch, a.status, lane);
            T xc[KPW];
#pragma unroll
            for (int q = 0; q < KPW; ++q) {
                const int k = warp + q * kWarps;
                xc[q] = (k < kw && lane < cw) ? __ldcg(tmp + (size_t)(crow + lane) * nrhs + k0 + k) : T(0);
            }
#pragma unroll
            for (int q = 0; q < KPW; ++q) {
                if (warp + q * kWarps >= kw) break;  // warp-uniform
#pragma unroll 8
                for (int j = 0; j < kW; ++j) xv[q] = fma(-sm.m[lane][j], __shfl_sync(0xffffffffu, xc[q], j), xv[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = warp + q * kWarps;
            if (k < kw && lane < w) {
                tmp[(size_t)(U.c0 + lane) * nrhs + k0 + k] = xv[q];
                if (!LOWER) {
                    using TO = typename io::tout;
                    TO* out = static_cast<TO*>(d.out);
                    const size_t oo = (size_t)d.perm[U.c0 + lane] * nrhs + k0 + k;
                    if (io::accum) out[oo] += (TO)xv[q];
                    else out[oo] = (TO)xv[q];
                }
            }
        }
        // the barrier orders the CTA's writes before thread 0's release
        __syncthreads();
        if (tid == 0) {
            dev::st_release(d.uflags + (size_t)uidx * d.nslices + slice, epoch);
        }
    }
    // the last CTA out resets the ticket and advances the epoch for the next
    // launch (the launch boundary orders these writes)
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(a.counters + 1, 1) == (int)gridDim.x - 1) {
            a.counters[0] = 0;
            a.counters[1] = 0;
            *a.epoch = epoch + 1;
        }
    }
}

template <class io, bool LOWER, int KW>
cudaError_t launch_sn_kw(const SnSweepArgs& a, cudaStream_t stream) {
    using T = typename io::t;
    const void* fn = (const void*)sn_sweep_kernel<io, LOWER, KW>;
    const size_t smem = sizeof(SnSmem<T, KW>);
    int grid = 0;
    cudaError_t e = coop_grid(fn, kT, smem, &grid);  // resident CTAs: a persistent grid
    if (e != cudaSuccess) return e;
    if (grid > a.nitems) grid = a.nitems;
    sn_sweep_kernel<io, LOWER, KW><<<grid, kT, smem, stream>>>(a);
    return cudaGetLastError();
}

template <class io, bool LOWER>
cudaError_t launch_sn_io(const SnSweepArgs& a, cudaStream_t stream) {
    constexpr int wide = sizeof(typename io::t) == 8 ? 16 : 32;
    if (!a.wide && a.sys0.nrhs <= 8) return launch_sn_kw<io, LOWER, 8>(a, stream);
    return launch_sn_kw<io, LOWER, wide>(a, stream);
}

}  // namespace

int sn_slices(int nrhs, bool f64) {
    const int wide = f64 ? 16 : 32;
    return nrhs <= 8 ? 1 : (nrhs + wide - 1) / wide;
}

int sn_slice_width(int nrhs, bool f64, bool wide) {
    return (!wide && nrhs <= 8) ? 8 : (f64 ? 16 : 32);
}

size_t sn_pbuf_bytes(int nparts, int nrhs, bool f64, bool wide) {
    const int kw = sn_slice_width(nrhs, f64, wide);
    const int ns = (nrhs + kw - 1) / kw;
    return (size_t)nparts * ns * kChunk * kw * (f64 ? sizeof(double) : sizeof(float));
}

cudaError_t launch_sn_sweep(const SnSweepArgs& a, bool lower, SweepIO io, cudaStream_t stream) {
    if (a.nitems == 0) return cudaSuccess;
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
