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

#include <type_traits>

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

// Column quarters (lower sweep) or row quarters (upper sweep) of a block
// list, dealt to the 8 warps in equal contiguous shares (warp w: quarters
// [w Q / 8, (w + 1) Q / 8) of the list's Q = 4 * nblk), so that the warps of
// a CTA finish an item together whatever its number of blocks. A warp waits
// for a block's input once, at its first quarter of the block.
constexpr int kQ = 4, kJQ = kW / kQ;

template <typename T, int KW>
__device__ __forceinline__ void lower_quarters(const SnSys& d, int b0, int nblk, int warp, int slice, int k0,
                                               int kw, int epoch, int* status, int lane,
                                               T (*xs)[XsStride<T, KW>::value], T (&acc)[KW]) {
    const int total = nblk * kQ;
    const int u0 = warp * total / kWarps, u1 = (warp + 1) * total / kWarps;
    if (u0 >= u1) return;
    int cur = u0 / kQ;
    const int last = (u1 - 1) / kQ;
    SnContrib C = d.contribs[b0 + cur];
    SnContrib Cn = cur < last ? d.contribs[b0 + cur + 1] : C;  // the next block's descriptor, ahead
    bool waited = false;
    for (int u = u0; u < u1; ++u) {
        const int b = u / kQ, q = u % kQ;
        if (b != cur) {
            cur = b;
            C = Cn;
            waited = false;
            if (cur < last) Cn = d.contribs[b0 + cur + 1];
        }
        if (q * kJQ >= C.w) continue;  // warp-uniform
        lower_block<T, KW, kJQ>(d, C.panel_off, C.ld, C.xcol, C.w, C.src_unit, C.rowmask, waited, q * kJQ, slice,
                                k0, kw, epoch, status, lane, xs, acc);
        waited = true;
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

// Upper-sweep block list of unit `uidx` (off-diagonal 32-row blocks of the
// supernode, highest first, each final once the unit holding its first row
// is; then the later chunks of the supernode but the next, last first),
// dealt in row quarters as lower_quarters deals columns.
template <typename T, int KW>
__device__ __forceinline__ void upper_quarters(const SnSys& d, const SnUnit& U, int uidx, int nblk, int warp,
                                               int slice, int k0, int kw, int epoch, int* status, int lane,
                                               T (*xs)[XsStride<T, KW>::value], T (&acc)[KW]) {
    const int wj = U.pos0 + U.w, sn_w = U.sn_w;
    const int nrb = (U.ld - sn_w + kW - 1) / kW;   // off-diagonal row blocks
    const int nlater = (sn_w - wj + kW - 1) / kW;  // later chunks
    const int total = nblk * kQ;
    const int u0 = warp * total / kWarps, u1 = (warp + 1) * total / kWarps;
    int cur = -1, p0 = 0, nr = 0, dep = -1;
    bool waited = false;
    for (int u = u0; u < u1; ++u) {
        const int b = u / kQ, q = u % kQ;
        if (b != cur) {
            cur = b;
            waited = false;
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
        }
        if (q * kJQ >= nr) continue;  // warp-uniform
        upper_block<T, KW, kJQ>(d, U, p0, nr, q * kJQ, waited ? -1 : dep, slice, k0, kw, epoch, status, lane, xs,
                                acc);
        waited = true;
    }
}

// ---- wide FP64 RHS slices: a CTA-wide block pipeline ----------------------
//
// The CTA streams its item's blocks through S shared-memory stages with
// cp.async: while the 8 warps apply one block, the L and x blocks of the next
// S - 1 are in flight. Lane = RHS column k of the slice (FP64: two 16-lane
// groups, each taking half of the block's inner dimension); warp w owns 4
// destination rows (lower sweep) or unit columns (upper sweep), so a lane
// accumulates only rows present in the block and no reduction across warps
// is needed. Staged L blocks hold zeros beyond the block's extent, x blocks
// are stored transposed (x[k][j]) so that a lane reads its column with
// 16-byte loads.
template <typename T, int KW>
struct Wide {
    static constexpr int G = 32 / KW;                 // lane groups
    static constexpr int JR = kW / G;                 // inner indices per group
    static constexpr int V = 16 / (int)sizeof(T);     // elements per 16 bytes
    static constexpr int LS = kW + V;                 // row stride of a staged L block
    static constexpr int XS = kW + V;                 // row stride of a staged x block
    static constexpr int S = sizeof(T) == 4 ? 4 : 3;  // pipeline stages
};

template <typename T, int KW>
struct SnStage {
    __align__(16) T l[kW][Wide<T, KW>::LS];  // lower: l[i][j] (block row, source column); upper: l[j][i]
    __align__(16) T x[KW][Wide<T, KW>::XS];  // x[k][j], transposed
    unsigned mask;                           // lower: the block's row mask
    int ext;                                 // lower: source columns; upper: block rows
};

template <typename T, int KW>
struct SnSmemWide {
    SnStage<T, KW> st[Wide<T, KW>::S];
    T t[kW][KW + 1];
    T d[kW][kW + 1];
    T m[kW][kW + 1];
};

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// acc[r] += sum over the group's inner range of l_row[i] * xr[i] (16-byte loads of l_row).
template <typename T, int JR>
__device__ __forceinline__ T dot_row(const T* l_row, const T (&xr)[JR], T acc) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < JR; i += 4) {
            const float4 v = *reinterpret_cast<const float4*>(l_row + i);
            acc = fmaf(v.x, xr[i], acc);
            acc = fmaf(v.y, xr[i + 1], acc);
            acc = fmaf(v.z, xr[i + 2], acc);
            acc = fmaf(v.w, xr[i + 3], acc);
        }
    } else {
#pragma unroll
        for (int i = 0; i < JR; i += 2) {
            const double2 v = *reinterpret_cast<const double2*>(l_row + i);
            acc = fma(v.x, xr[i], acc);
            acc = fma(v.y, xr[i + 1], acc);
        }
    }
    return acc;
}

template <typename T, int JR>
__device__ __forceinline__ void load_col(const T* src, T (&xr)[JR]) {
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < JR; i += 4) {
            const float4 v = *reinterpret_cast<const float4*>(src + i);
            xr[i] = v.x; xr[i + 1] = v.y; xr[i + 2] = v.z; xr[i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < JR; i += 2) {
            const double2 v = *reinterpret_cast<const double2*>(src + i);
            xr[i] = v.x; xr[i + 1] = v.y;
        }
    }
}

// The S-stage pipeline over blocks 0..nblk-1: issue(b, stage) starts block
// b's copies into a stage (all threads), compute(b, stage) applies it.
template <int S, class Issue, class Compute>
__device__ __forceinline__ void pipeline(int nblk, Issue issue, Compute compute) {
#pragma unroll 1
    for (int b = 0; b < S - 1; ++b) {
        if (b < nblk) issue(b, b % S);
        cp_async_commit();
    }
#pragma unroll 1
    for (int b = 0; b < nblk; ++b) {
        cp_async_wait<S - 2>();  // this thread's copies of block b have landed
        __syncthreads();         // everyone's have, and every warp is done with block b - 1
        if (b + S - 1 < nblk) issue(b + S - 1, (b + S - 1) % S);
        cp_async_commit();
        compute(b, b % S);
    }
    cp_async_wait<0>();
}

// Lower sweep, wide slices: contribution blocks [b0, b1), whose sources
// have taken earlier tickets (a block waits for its source's flag before its
// x copy is issued). acc[r] += (L_block x_source)[row 4 * warp + r][k]. Lane
// k of each warp keeps a window of 32 block descriptors (lane j: block
// 32 * n + j) with their flags checked, broadcast by shuffles.
template <typename T, int KW>
__device__ __forceinline__ void lower_wide(const SnSys& d, SnSmemWide<T, KW>& sm, int b0, int b1, int slice, int k0,
                                           int kw, int epoch, int* status, int tid, int lane, int warp,
                                           T (&acc)[4]) {
    using C = Wide<T, KW>;
    const T* __restrict__ panels = static_cast<const T*>(d.panels);
    const T* tmp = static_cast<const T*>(d.tmp);
    const int nrhs = d.nrhs;
    int wbase = -1;
    long long poff = 0;
    int ld = 0, xcol = 0, w = 0, nr = 0, srcu = 0, ready = 1;
    unsigned mask = 0;
    auto issue = [&](int b, int s) {
        SnStage<T, KW>& st = sm.st[s];
        if ((b & ~31) != wbase) {  // next window
            wbase = b & ~31;
            const int mb = b0 + wbase + lane;
            if (mb < b1) {
                const SnContrib& c = d.contribs[mb];
                poff = c.panel_off; ld = c.ld; xcol = c.xcol; w = c.w; nr = c.nr; srcu = c.src_unit;
                mask = c.rowmask;
                ready = dev::ld_acquire(d.uflags + (size_t)srcu * d.nslices + slice) >= epoch;
            }
            __syncwarp();  // orders the lanes' flag observations before every lane's copies
        }
        const int q = b & 31;
        const long long bp = __shfl_sync(0xffffffffu, poff, q);
        const int bld = __shfl_sync(0xffffffffu, ld, q), bx = __shfl_sync(0xffffffffu, xcol, q);
        const int bw = __shfl_sync(0xffffffffu, w, q), bnr = __shfl_sync(0xffffffffu, nr, q);
        const int bs = __shfl_sync(0xffffffffu, srcu, q), br = __shfl_sync(0xffffffffu, ready, q);
        const unsigned bm = __shfl_sync(0xffffffffu, mask, q);
        if (tid == 0) {
            st.mask = bm;
            st.ext = bw;
        }
        for (int idx = tid; idx < kW * kW; idx += kT) {  // l[i][j], zero beyond the source columns
            const int i = idx & 31, j = idx >> 5;
            if (i < bnr) {
                if (j < bw) cp_async_elem(&st.l[i][j], panels + bp + (size_t)j * bld + i);
                else st.l[i][j] = T(0);
            }
        }
        if (!br) warp_wait(d.uflags + (size_t)bs * d.nslices + slice, epoch, status, lane);
        for (int idx = tid; idx < kW * KW; idx += kT) {  // x[k][j] = x_source[j][k], zero beyond
            const int k = idx % KW, j = idx / KW;
            if (j < bw) {
                if (k < kw) cp_async_elem(&st.x[k][j], tmp + (size_t)(bx + j) * nrhs + k0 + k);
            } else {
                st.x[k][j] = T(0);
            }
        }
    };
    auto compute = [&](int, int s) {
        const SnStage<T, KW>& st = sm.st[s];
        const unsigned bm = st.mask;
        const unsigned rows4 = (bm >> (4 * warp)) & 0xFu;
        if (!rows4) return;                  // warp-uniform
        const int k = lane % KW, h = lane / KW;
        if (h * C::JR >= st.ext) return;     // this group's source columns are all beyond the block
        T xr[C::JR];
        load_col<T, C::JR>(&st.x[k][h * C::JR], xr);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (!((rows4 >> r) & 1u)) continue;
            const int i = __popc(bm & ((1u << (4 * warp + r)) - 1u));
            acc[r] = dot_row<T, C::JR>(&st.l[i][h * C::JR], xr, acc[r]);
        }
    };
    pipeline<C::S>(b1 - b0, issue, compute);
}

// Upper sweep, wide slices: blocks 0..nblk-1 of the unit's list (off-
// diagonal 32-row blocks, highest first, then the later chunks but the next,
// last first), each waiting for its flag before its x copy is issued.
// acc[r] += (L_block^T x_block)[unit column 4 * warp + r][k].
template <typename T, int KW>
__device__ __forceinline__ void upper_wide(const SnSys& d, SnSmemWide<T, KW>& sm, const SnUnit& U, int uidx,
                                           int nblk, int slice, int k0, int kw, int epoch, int* status, int tid,
                                           int lane, int warp, T (&acc)[4]) {
    using C = Wide<T, KW>;
    const T* __restrict__ panels = static_cast<const T*>(d.panels);
    const T* tmp = static_cast<const T*>(d.tmp);
    const int nrhs = d.nrhs;
    const int w = U.w, wj = U.pos0 + w, sn_w = U.sn_w, sn_c0 = U.c0 - U.pos0;
    const int nrb = (U.ld - sn_w + kW - 1) / kW;
    const int nlater = (sn_w - wj + kW - 1) / kW;
    int wbase = -1, p0 = 0, nr = 0, ready = 1, dep = 0;
    auto issue = [&](int b, int s) {
        SnStage<T, KW>& st = sm.st[s];
        if ((b & ~31) != wbase) {  // next window
            wbase = b & ~31;
            const int mb = wbase + lane;
            if (mb < nblk) {
                if (mb < nrb) {
                    p0 = sn_w + (nrb - 1 - mb) * kW;
                    nr = min(kW, U.ld - p0);
                    dep = d.unit_of_row[d.sn_rows[U.rows_off + p0]];
                } else {
                    const int c = nlater - 1 - (mb - nrb);
                    p0 = wj + c * kW;
                    nr = min(kW, sn_w - p0);
                    dep = uidx + 1 + c;
                }
                ready = dev::ld_acquire(d.uflags + (size_t)dep * d.nslices + slice) >= epoch;
            }
            __syncwarp();
        }
        const int q = b & 31;
        const int bp0 = __shfl_sync(0xffffffffu, p0, q), bnr = __shfl_sync(0xffffffffu, nr, q);
        const int bdep = __shfl_sync(0xffffffffu, dep, q), br = __shfl_sync(0xffffffffu, ready, q);
        if (tid == 0) st.ext = bnr;
        for (int idx = tid; idx < kW * kW; idx += kT) {  // l[j][i] = L[block row i, unit column j]
            const int i = idx & 31, j = idx >> 5;
            if (j < w) {
                if (i < bnr) cp_async_elem(&st.l[j][i], panels + U.panel_col_off + (size_t)j * U.ld + bp0 + i);
                else st.l[j][i] = T(0);
            }
        }
        if (!br) warp_wait(d.uflags + (size_t)bdep * d.nslices + slice, epoch, status, lane);
        for (int idx = tid; idx < kW * KW; idx += kT) {  // x[k][i] = x[row of block row i][k]
            const int k = idx % KW, i = idx / KW;
            if (i < bnr) {
                if (k < kw) {
                    const int pos = bp0 + i;
                    const int row = pos < sn_w ? sn_c0 + pos : d.sn_rows[U.rows_off + pos];
                    cp_async_elem(&st.x[k][i], tmp + (size_t)row * nrhs + k0 + k);
                }
            } else {
                st.x[k][i] = T(0);
            }
        }
    };
    auto compute = [&](int, int s) {
        const SnStage<T, KW>& st = sm.st[s];
        if (4 * warp >= w) return;           // warp-uniform
        const int k = lane % KW, h = lane / KW;
        if (h * C::JR >= st.ext) return;     // this group's rows are all beyond the block
        T xr[C::JR];
        load_col<T, C::JR>(&st.x[k][h * C::JR], xr);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (4 * warp + r >= w) break;
            acc[r] = dot_row<T, C::JR>(&st.l[4 * warp + r][h * C::JR], xr, acc[r]);
        }
    };
    pipeline<C::S>(nblk, issue, compute);
}

// FP64 wide slices (16 RHS columns) use the CTA-wide block pipeline and 3
// CTAs per SM: FP64 arithmetic is slow enough on this GPU that skipping the
// rows a block does not have pays for the pipeline. Otherwise each warp takes
// its own blocks (lane = row).
template <class io, int KW>
constexpr bool kPipelined = sizeof(typename io::t) == 8 && KW >= 16;
template <class io, int KW>
using SnSmemOf = std::conditional_t<kPipelined<io, KW>, SnSmemWide<typename io::t, KW>, SnSmem<typename io::t, KW>>;

// QUART: every block list dealt in balanced quarters (FP32, several 32-wide
// slices of one system), known at compile time. (3 CTAs per SM was measured
// slower for it: more tickets held by waiting CTAs.)
template <class io, bool LOWER, int KW, bool QUART>
__global__ void __launch_bounds__(kT, (kPipelined<io, KW> ? 3 : 2)) sn_sweep_kernel(SnSweepArgs a) {
    using T = typename io::t;
    constexpr bool WIDE = kPipelined<io, KW>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SnSmemOf<io, KW>& sm = *reinterpret_cast<SnSmemOf<io, KW>*>(smem_raw);
    if (a.skip && dev::ld_volatile(a.skip)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nitems = a.nitems;
    // every CTA reads the sweep's epoch before the last CTA out bumps it
    const int epoch = dev::ld_volatile(a.epoch);
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
                // L2 loads: no value of an unsolved row enters L1 (the wide
                // path's cp.async x copies read through L1)
                sm.t[i][k] = (i < w && k < kw) ? __ldcg(tmp + (size_t)(U.c0 + i) * nrhs + k0 + k) : T(0);
            }
        }
        // Every block but the one on the dependency chain (lower: from the
        // previous chunk of the same supernode, listed last; upper: from the
        // next chunk) is applied here; the chain block is folded into the
        // diagonal solve below.
        const int nfree = part ? PS.contrib_end - PS.contrib_begin
                          : LOWER ? (U.contrib_end - U.contrib_begin) - (chain ? 1 : 0)  // chain block: the list's last
                                  : (U.ld - U.sn_w + kW - 1) / kW + (U.sn_w - (U.pos0 + w) + kW - 1) / kW -
                                        (chain ? 1 : 0);
        if constexpr (WIDE) {
            // warp w owns rows (lower) / unit columns (upper) 4w .. 4w + 3;
            // lane k < KW ends with the sums of RHS column k
            T acc[4] = {T(0), T(0), T(0), T(0)};
            if (LOWER) {
                const int b0 = part ? PS.contrib_begin : U.contrib_begin;
                lower_wide<T, KW>(d, sm, b0, b0 + nfree, slice, k0, kw, epoch, a.status, tid, lane, warp, acc);
            } else {
                upper_wide<T, KW>(d, sm, U, uidx, nfree, slice, k0, kw, epoch, a.status, tid, lane, warp, acc);
            }
            if constexpr (Wide<T, KW>::G == 2) {
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], 16);
            }
            const int k = lane % KW;
            const bool lead = lane < KW;
            if (LOWER && !part) {  // the unit's partial sums
                for (int q = U.part_begin; q < U.part_end; ++q) {
                    warp_wait(d.uflags + (size_t)(d.n_units + q) * d.nslices + slice, epoch, a.status, lane);
                    const T* ps = static_cast<const T*>(d.pbuf) + ((size_t)q * d.nslices + slice) * (kW * KW);
                    if (lead) {
#pragma unroll
                        for (int r = 0; r < 4; ++r) acc[r] += __ldcg(ps + (4 * warp + r) * KW + k);
                    }
                }
            }
            if (part) {  // the sum goes to the partial's slot, then its flag
                T* ps = static_cast<T*>(d.pbuf) + ((size_t)(~uidx) * d.nslices + slice) * (kW * KW);
                if (lead) {
#pragma unroll
                    for (int r = 0; r < 4; ++r) ps[(4 * warp + r) * KW + k] = acc[r];
                }
                __syncthreads();
                if (tid == 0) dev::st_release(d.uflags + (size_t)(d.n_units + ~uidx) * d.nslices + slice, epoch);
                continue;
            }
            __syncthreads();  // the staged t is complete
            if (lead) {
#pragma unroll
                for (int r = 0; r < 4; ++r) sm.t[4 * warp + r][k] -= acc[r];
            }
            __syncthreads();
        } else {
            T (*xs)[XsStride<T, KW>::value] = sm.xs[warp];
            T acc[KW];
#pragma unroll
            for (int k = 0; k < KW; ++k) acc[k] = T(0);
            // several 32-wide slices (throughput bound): blocks dealt in
            // balanced quarters; otherwise (latency bound): whole blocks,
            // round robin
            const bool kQuarters = QUART || (KW >= 32 && d.nslices > 1);
            if (part) {
                if (kQuarters)
                    lower_quarters<T, KW>(d, PS.contrib_begin, nfree, warp, slice, k0, kw, epoch, a.status, lane,
                                          xs, acc);
                else
                    lower_list<T, KW>(d, PS.contrib_begin + warp, PS.contrib_end, slice, k0, kw, epoch, a.status,
                                      lane, xs, acc);
            } else if (LOWER) {
                // the unit's partial sums, one per warp in turn (slot row = lane)
                for (int q = U.part_begin + warp; q < U.part_end; q += kWarps) {
                    warp_wait(d.uflags + (size_t)(d.n_units + q) * d.nslices + slice, epoch, a.status, lane);
                    const T* ps =
                        static_cast<const T*>(d.pbuf) + ((size_t)q * d.nslices + slice) * (kW * KW) + lane * KW;
#pragma unroll
                    for (int k = 0; k < KW; ++k) acc[k] += __ldcg(ps + k);
                }
                if (kQuarters)
                    lower_quarters<T, KW>(d, U.contrib_begin, nfree, warp, slice, k0, kw, epoch, a.status, lane, xs,
                                          acc);
                else
                    lower_list<T, KW>(d, U.contrib_begin + warp, U.contrib_begin + nfree, slice, k0, kw, epoch,
                                      a.status, lane, xs, acc);
            } else if (kQuarters) {
                upper_quarters<T, KW>(d, U, uidx, nfree, warp, slice, k0, kw, epoch, a.status, lane, xs, acc);
            } else {
                // off-diagonal rows of the supernode in 32-row blocks, highest
                // rows first (they are solved first), each waiting for the unit
                // of its lowest row; then the later chunks of the supernode, last
                // chunk first, but the next one (the chain); round robin
                const int wj = U.pos0 + w;                      // end of this unit's columns
                const int sn_w = U.sn_w;                        // supernode width
                const int nrb = (U.ld - sn_w + kW - 1) / kW;    // off-diagonal row blocks
                const int nlater = (sn_w - wj + kW - 1) / kW;   // later chunks
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
                if (tid == 0) dev::st_release(d.uflags + (size_t)(d.n_units + ~uidx) * d.nslices + slice, epoch);
                continue;
            }
            for (int idx = tid; idx < kW * KW; idx += kT) {
                const int i = idx / KW, k = idx % KW;
                T v = T(0);
#pragma unroll
                for (int ww = 0; ww < kWarps; ++ww) v += sm.xs[ww][i][k];
                sm.t[i][k] -= v;
            }
            __syncthreads();
        }
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

template <class io, bool LOWER, int KW, bool QUART = false>
cudaError_t launch_sn_kw(const SnSweepArgs& a, cudaStream_t stream) {
    const void* fn = (const void*)sn_sweep_kernel<io, LOWER, KW, QUART>;
    const size_t smem = sizeof(SnSmemOf<io, KW>);
    int grid = 0;
    cudaError_t e = coop_grid(fn, kT, smem, &grid);  // resident CTAs: a persistent grid
    if (e != cudaSuccess) return e;
    if (grid > a.nitems) grid = a.nitems;
    sn_sweep_kernel<io, LOWER, KW, QUART><<<grid, kT, smem, stream>>>(a);
    return cudaGetLastError();
}

template <class io, bool LOWER>
cudaError_t launch_sn_io(const SnSweepArgs& a, cudaStream_t stream) {
    constexpr int wide = sizeof(typename io::t) == 8 ? 16 : 32;
    if (!a.wide && a.sys0.nrhs <= 8) return launch_sn_kw<io, LOWER, 8>(a, stream);
    if constexpr (sizeof(typename io::t) == 4)
        if (!a.sys && a.sys0.nslices > 1) return launch_sn_kw<io, LOWER, wide, true>(a, stream);
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
