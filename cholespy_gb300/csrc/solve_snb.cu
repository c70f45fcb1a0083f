// Bulk-copy supernodal sweeps for many right-hand sides (sm_103a, FP32).
//
// Same work decomposition as solve_sn.cu (units of <= 32 columns of the
// top-region supernodes, atomic tickets in estimated-start order, epoch-
// valued unit flags, the chain block folded into the diagonal solve), shaped
// for 12..128 RHS (multiples of 4):
//
// * One work item = one unit and every RHS column, so each L block is read
//   once per solve instead of once per 32-column slice. Long lower-sweep
//   block lists can be split into partial-sum items (plan.cpp,
//   build_snb_lower) that the unit adds in a fixed order.
// * L blocks are pre-expanded 32 x 32 tiles (zero outside the block's rows
//   and columns): lower sweep, one per contribution block, [source
//   column][unit row]; upper sweep, one per off-diagonal block of the
//   unit's supernode, [block row][unit column]. The rows of a tile that the
//   block has (its source columns / block rows) are one bulk copy.
// * A producer warp takes the tickets (running up to one item ahead of the
//   consumers through two descriptor slots) and streams each item's blocks
//   through a 4-stage shared-memory ring with cp.async.bulk: per block,
//   once the source unit's flag is set, the L tile and the block's rows of
//   the work array, one bulk copy per run of consecutive rows, completing on
//   the stage's mbarrier. Descriptors and flags are read 32 blocks at a time
//   (one round trip per window). Eight consumer warps apply each stage
//   (thread = one RHS column and 16 (or 8) unit rows / columns, 4-row groups
//   the block lacks skipped; every output has one owner, so there is no
//   reduction across warps and no CTA-wide barrier per block) and release
//   it on the stage's second mbarrier.
// * After the last block: t' = t - sum, x = E t' (E = D^-1 lower, D^-T
//   upper), then x -= M2 x_2 for the chunk two before (lower) / after
//   (upper) in the unit's supernode (its block is the list's last; the
//   producer streams the tile M2 = E L_block instead of L_block, so it needs
//   no product by E), then, once the chain unit's flag is set, x -= M
//   x_chain with the chain rows brought into shared memory in one round
//   trip. The x rows go to the work array (and, upper sweep, through perm to
//   the output) and one release store publishes the unit. So E t' waits
//   only on chunks three or more back, and after the chain wait a unit does
//   one load and one 32 x 32 product.
// Reference: the same sweeps as kernels/kernels.cu:64-202 (solve_lower /
// solve_upper), with the per-row flag waits of the reference replaced by one
// flag per unit.
//
// Every wait is bounded (device.cuh, bulk.cuh). Results are deterministic:
// each output is summed by one thread over the item's blocks in list order.
#include <cuda_runtime.h>

#include "bulk.cuh"
#include "device.cuh"
#include "launch.h"
#include "solve_snb.h"
#include "tcgen05.cuh"

namespace gbchol {

namespace {

constexpr int kCW = 8;                    // consumer warps
constexpr int kThreads = (kCW + 1) * 32;  // + one producer warp
constexpr int kTile = 32 * 32;
// Ring geometry: KB block rows per stage (lower sweep with CUDA-core
// consumers: groups of up to 64 source columns; otherwise 32) and S stages:
// 4 of 32 rows, or 2 of 64 rows or with the tensor-core operand buffers (two
// CTAs per SM in every case).
template <bool LOWER, bool TC>
struct SnbRing {
    static constexpr int KB = (LOWER && !TC) ? 64 : 32;
    static constexpr int S = (TC || KB == 64) ? 2 : 4;
};

template <int SW, int KB>
struct SnbStage {
    float l[KB][32];   // L tile rows (lower: source columns; upper: block rows)
    float x[KB * SW];  // the block's rows of the work array, row stride = the RHS count
};

// Tensor-core operands of one block (canonical K-major layout, tcgen05.cuh):
// A = the block's work-array rows transposed (128 RHS columns x 32), B = the
// L tile (32 unit rows / columns x 32), each split into TF32 high and low
// parts.
template <bool TC>
struct SnbTc {};
template <>
struct SnbTc<true> {
    // 128-byte alignment (the descriptors need 16): coarser padding would
    // push the CTA past two per SM
    __align__(128) float a_hi[128 * 32];
    __align__(128) float a_lo[128 * 32];
    __align__(128) float b_hi[32 * 32];
    __align__(128) float b_lo[32 * 32];
    uint64_t mma_done;  // one phase per block: its MMAs have completed
    uint32_t tmem;      // accumulator: 128 lanes x 32 columns
};

template <int SW, bool LOWER, bool TC>
struct SnbSmem {
    static constexpr int kStages = SnbRing<LOWER, TC>::S;
    SnbStage<SW, SnbRing<LOWER, TC>::KB> st[kStages];
    float t[32][SW];   // t' = t - sum of the blocks (right-hand side of the diagonal solve)
    float e[32][32];   // e[j][i] = E[i][j]
    float m[32][32];   // m[j][i] = M[i][j] (the chain block folded into the diagonal solve)
    uint64_t full[kStages], empty[kStages];
    uint64_t item_full[2], item_empty[2];  // the two item-descriptor slots
    SnUnit item_unit[2];
    int item_v[2], item_valid[2], item_slice[2];
    int ext[kStages];        // rows of the stage's x block (lower: source columns, upper: block rows)
    unsigned mask[kStages];  // unit rows (lower) / columns (upper) the block has
    SnbTc<TC> tc;
};

template <typename TO, bool ACCUM>
struct SnbIO {
    using tout = TO;
    static constexpr bool accum = ACCUM;
};

// RR consecutive floats of shared memory (16-, 8- or 4-byte aligned by the
// consumers' row mapping), in one load.
template <int RR>
__device__ __forceinline__ void load_rows(const float* p, float (&v)[RR]) {
    if constexpr (RR == 4) {
        const float4 q = *reinterpret_cast<const float4*>(p);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else if constexpr (RR == 2) {
        const float2 q = *reinterpret_cast<const float2*>(p);
        v[0] = q.x; v[1] = q.y;
    } else {
        v[0] = p[0];
    }
}

// Item geometry shared by the producer and the consumers.
struct SnbItem {
    bool part, chain;
    int uidx, tile0, nblk;
};

template <bool LOWER>
__device__ __forceinline__ SnbItem snb_item(const SnbArgs& a, int v, const SnUnit& U) {
    SnbItem it;
    // a lower-sweep partial sum (item ~p): blocks summed into a slot
    it.part = LOWER && v < 0;
    it.uidx = it.part ? a.parts[~v].unit : v;
    // the chain input: lower, the previous chunk of the supernode (its block
    // is the last of the list); upper, the next one (not listed)
    it.chain = !it.part && (LOWER ? U.pos0 > 0 : U.pos0 + U.w < U.sn_w);
    if (it.part) {
        it.tile0 = a.parts[~v].contrib_begin;
        it.nblk = a.parts[~v].contrib_end - it.tile0;
    } else if (LOWER) {
        it.tile0 = a.unit_info[(size_t)it.uidx * 4];
        it.nblk = a.unit_info[(size_t)it.uidx * 4 + 1] - it.tile0;
    } else {
        it.tile0 = a.up_begin[it.uidx];
        it.nblk = a.up_begin[it.uidx + 1] - it.tile0;
    }
    return it;
}

// Whether the item's last block is the folded second block (tile M2 from
// a.fold2, applied after the diagonal solve's product).
template <bool LOWER>
__device__ __forceinline__ bool snb_folds2(const SnbArgs& a, const SnbItem& it, const SnUnit& U) {
    return !it.part && a.fold >= 2 && (LOWER ? snb_fold2_lo(U) : snb_fold2_up(U));
}

// The consumers' conversion of one landed stage into the tensor-core
// operands: A(k, j) = x[j][k] (RHS column k, block row j), B(n, j) =
// tile[j][n], each value v as hi = tf32(v), lo = tf32(v - hi); zero past the
// block's `ext` rows and the RHS count. Thread t: A for RHS column t % 128
// and row groups t / 128 + 2q; B for unit row / column t % 32 and row group t / 32.
template <int SW>
__device__ __forceinline__ void snb_split(const SnbStage<SW, 32>& st, SnbTc<true>& tb, int ext, int nrhs, int tid) {
    const int ka = tid & 127;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int jg = (tid >> 7) + 2 * q;  // rows 4 jg .. 4 jg + 3
        float4 hi, lo;
        float* h = &hi.x;
        float* l = &lo.x;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = 4 * jg + u;
            const float v = (j < ext && ka < nrhs) ? st.x[j * nrhs + ka] : 0.f;
            h[u] = tc::to_tf32(v);
            l[u] = tc::to_tf32(v - h[u]);
        }
        const int off = (ka >> 3) * 256 + jg * 32 + (ka & 7) * 4;  // floats: SBO 1024 B, LBO 128 B
        *reinterpret_cast<float4*>(&tb.a_hi[off]) = hi;
        *reinterpret_cast<float4*>(&tb.a_lo[off]) = lo;
    }
    {
        const int nb = tid & 31, jg = tid >> 5;
        float4 hi, lo;
        float* h = &hi.x;
        float* l = &lo.x;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = 4 * jg + u;
            const float v = j < ext ? st.l[j][nb] : 0.f;
            h[u] = tc::to_tf32(v);
            l[u] = tc::to_tf32(v - h[u]);
        }
        const int off = (nb >> 3) * 256 + jg * 32 + (nb & 7) * 4;
        *reinterpret_cast<float4*>(&tb.b_hi[off]) = hi;
        *reinterpret_cast<float4*>(&tb.b_lo[off]) = lo;
    }
}

// One block on the tensor cores (one thread): D += A_lo B_hi + A_hi B_lo +
// A_hi B_hi over K = 32 in steps of 8 (3 x 4 MMAs of 128 x 32 x 8).
__device__ __forceinline__ void snb_mma(SnbTc<true>& tb, bool first) {
    constexpr uint32_t idesc = tc::idesc_tf32(128, 32);
    const float* as[3] = {tb.a_lo, tb.a_hi, tb.a_hi};
    const float* bs[3] = {tb.b_hi, tb.b_lo, tb.b_hi};
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const uint64_t ad = tc::smem_desc(as[p] + ks * 64, 128, 1024);
            const uint64_t bd = tc::smem_desc(bs[p] + ks * 64, 128, 1024);
            tc::mma_tf32(tb.tmem, ad, bd, idesc, (first && p == 0 && ks == 0) ? 0u : 1u);
        }
    }
    tc::commit(&tb.mma_done);
}

template <class io, bool LOWER, int SW, bool TC>
__global__ void __launch_bounds__(kThreads, 2) snb_sweep_kernel(SnbArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SnbSmem<SW, LOWER, TC>& sm = *reinterpret_cast<SnbSmem<SW, LOWER, TC>*>(smem_raw);
    constexpr int kStages = SnbRing<LOWER, TC>::S;
    if (a.skip && dev::ld_volatile(a.skip)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // every CTA reads the sweep's epoch before the last CTA out bumps it
    const int epoch = dev::ld_volatile(a.epoch);
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            bulk::mbar_init(&sm.full[s], 1);
            bulk::mbar_init(&sm.empty[s], kCW);
        }
        for (int s = 0; s < 2; ++s) {
            bulk::mbar_init(&sm.item_full[s], 1);
            bulk::mbar_init(&sm.item_empty[s], kCW);
        }
        if constexpr (TC) bulk::mbar_init(&sm.tc.mma_done, 1);
        bulk::fence_mbar_init();
    }
    if constexpr (TC) {
        if (warp == 0) tc::alloc(&sm.tc.tmem, 32);
        tc::fence_before_sync();
    }
    __syncthreads();
    if constexpr (TC) tc::fence_after_sync();
    const int nrhs = a.nrhs;                       // columns of one item (its slice)
    const int ld = a.ld > 0 ? a.ld : nrhs;         // row stride of the work array
    const int ns = a.nslices;
    if (warp == kCW) {
        // ---- producer: tickets, then the item's blocks into the stage ring
        uint32_t gs = 0;  // ring stages used so far
        for (uint32_t n = 0;; ++n) {
            const int slot = (int)(n & 1);
            int tk = 0;
            if (lane == 0) tk = atomicAdd(a.counters, 1);
            tk = __shfl_sync(0xffffffffu, tk, 0);
            const bool valid = tk < a.nitems;
            // tickets: the slices of an item are consecutive
            const int v = valid ? a.order[tk / ns] : 0;
            const int slice = tk % ns;
            if (lane == 0) {
                if (n >= 2) bulk::mbar_wait(&sm.item_empty[slot], ((n >> 1) - 1) & 1, a.status);
                sm.item_valid[slot] = valid ? 1 : 0;
                if (valid) {
                    sm.item_v[slot] = v;
                    sm.item_slice[slot] = slice;
                    sm.item_unit[slot] = a.units[v >= 0 ? v : a.parts[~v].unit];
                }
                bulk::mbar_arrive(&sm.item_full[slot]);
            }
            if (!valid) break;
            const int* uf = a.uflags + (size_t)slice * a.flag_stride;  // the slice's flags
            const float* xs = a.tmp + (size_t)slice * nrhs;            // the slice's first column
            const SnUnit U = a.units[v >= 0 ? v : a.parts[~v].unit];
            const SnbItem it = snb_item<LOWER>(a, v, U);
            const unsigned umask = U.w == 32 ? 0xffffffffu : (1u << U.w) - 1u;
            const bool f2 = snb_folds2<LOWER>(a, it, U);  // the last block's tile is M2
            // blocks in windows of 32: lane j reads the descriptor of the
            // window's j-th block and checks its source's flag (one round
            // trip for the window); the descriptors are broadcast by shuffles
            for (int w0 = 0; w0 < it.nblk; w0 += 32) {
                const int cnt = min(32, it.nblk - w0);
                int src_j = 0, xcol_j = 0, w_j = 0, first_j = 0, ready_j = 1;
                unsigned mask_j = 0;
                if (lane < cnt) {
                    const int t = it.tile0 + w0 + lane;
                    if (LOWER) {
                        const SnbGroup& G = a.groups[t];
                        src_j = G.src_unit;
                        xcol_j = G.xcol;
                        w_j = G.cols;
                        first_j = G.first;
                        mask_j = G.rowmask;
                    } else {
                        src_j = a.up_dep[t];
                    }
                    ready_j = dev::ld_acquire(uf + src_j) >= epoch;
                }
                // upper: the rows of the window's first block (later blocks'
                // rows are read one block ahead)
                int row_next = LOWER ? -1 : a.up_rows[(size_t)(it.tile0 + w0) * 32 + lane];
                __syncwarp();  // orders the lanes' flag observations before every lane's copies
                for (int q = 0; q < cnt; ++q) {
                    const uint32_t g = gs + (uint32_t)(w0 + q);
                    const int s = (int)(g % kStages);
                    const int t = it.tile0 + w0 + q;
                    const int src = __shfl_sync(0xffffffffu, src_j, q);
                    const int ready = __shfl_sync(0xffffffffu, ready_j, q);
                    int row, rows_l = 0, tile = t;
                    unsigned mask;
                    if (LOWER) {
                        // a group: contiguous work-array rows and tile rows, one copy each
                        row = __shfl_sync(0xffffffffu, xcol_j, q);
                        rows_l = __shfl_sync(0xffffffffu, w_j, q);
                        tile = __shfl_sync(0xffffffffu, first_j, q);
                        mask = __shfl_sync(0xffffffffu, mask_j, q);
                    } else {
                        row = row_next;
                        if (q + 1 < cnt) row_next = a.up_rows[(size_t)(t + 1) * 32 + lane];
                        mask = umask;
                    }
                    // upper: the block's rows are a prefix of the lanes; runs of
                    // consecutive work-array rows go in one bulk copy each (with
                    // column slices a row's columns are not contiguous with the
                    // next row's: one copy per row)
                    int rows, run = 0;
                    bool start;
                    if (ld != nrhs) {
                        if (LOWER) {
                            rows = rows_l;
                        } else {
                            rows = __popc(__ballot_sync(0xffffffffu, row >= 0));
                        }
                        start = false;
                    } else if (LOWER) {
                        rows = rows_l;
                        start = lane == 0;
                        run = rows;
                    } else {
                        const unsigned have = __ballot_sync(0xffffffffu, row >= 0);
                        rows = __popc(have);
                        const int prev = __shfl_up_sync(0xffffffffu, row, 1);
                        start = row >= 0 && (lane == 0 || prev != row - 1);
                        const unsigned later = __ballot_sync(0xffffffffu, start) & ~((2u << lane) - 1u);
                        run = (later ? __ffs(later) - 1 : rows) - lane;  // rows in my run (if start)
                    }
                    if (lane == 0) {
                        if (g >= kStages) {
                            const uint32_t par = ((g / kStages) - 1) & 1;
                            bulk::mbar_wait(&sm.empty[s], par, a.status);
                            // the stage's previous copies have landed (normally
                            // long since: its consumers waited for them)
                            bulk::mbar_wait(&sm.full[s], par, a.status, false);
                        }
                        if (!ready) dev::wait_geq(uf + src, epoch, a.status);
                        sm.ext[s] = rows;
                        sm.mask[s] = mask;
                        bulk::mbar_arrive_expect_tx(&sm.full[s], (uint32_t)(rows * (32 + nrhs) * 4));
                    }
                    __syncwarp();
                    // the source rows were published under the flag: order the
                    // bulk (async-proxy) reads after its acquire
                    bulk::fence_proxy_async_global();
                    const float* ltile = (f2 && w0 + q == it.nblk - 1)
                                             ? a.fold2 + ((size_t)it.uidx * 2 + (LOWER ? 0 : 1)) * kTile
                                             : (LOWER ? a.lo_tiles : a.up_tiles) + (size_t)tile * kTile;
                    // the tile's first `rows` rows: the rest is zero and unread
                    if (lane == 0) bulk::copy_g2s(&sm.st[s].l[0][0], ltile, (uint32_t)rows * 32 * 4, &sm.full[s]);
                    if (start)
                        bulk::copy_g2s(&sm.st[s].x[(LOWER ? 0 : lane) * nrhs], xs + (size_t)row * ld,
                                       (uint32_t)(run * nrhs) * 4, &sm.full[s]);
                    if (ld != nrhs) {  // one copy per row: lower, rows row .. row + rows - 1; upper, lane's row
                        if (LOWER) {
                            for (int i = lane; i < rows; i += 32)
                                bulk::copy_g2s(&sm.st[s].x[i * nrhs], xs + (size_t)(row + i) * ld,
                                               (uint32_t)nrhs * 4, &sm.full[s]);
                        } else if (row >= 0) {
                            bulk::copy_g2s(&sm.st[s].x[lane * nrhs], xs + (size_t)row * ld, (uint32_t)nrhs * 4,
                                           &sm.full[s]);
                        }
                    }
                }
            }
            gs += (uint32_t)it.nblk;
        }
        // no bulk copy may still be landing when the CTA exits (they complete
        // by themselves; this matters only after an abandoned wait)
        if (lane == 0) {
            for (int s = 0; s < kStages; ++s) {
                if ((uint32_t)s >= gs) break;
                const uint32_t last = gs - 1 - (uint32_t)((gs - 1 - (uint32_t)s) % kStages);  // last use of s
                bulk::mbar_wait(&sm.full[s], (last / kStages) & 1, a.status, false);
            }
        }
    } else {
        // ---- consumers: thread = 4 consecutive RHS columns (k4 .. k4 + 3)
        // x RR unit rows (lower) / columns (upper); warp w owns rows 4w ..
        // 4w + 3 (with 64 / 32 columns, the warp's 2 / 4 lane groups take
        // 2 / 1 rows each), so a warp skips a block without rows in its group
        constexpr int KG = SW / 4;        // RHS groups of 4: 32, 16 or 8
        constexpr int RR = KG / 8;        // rows per thread: 4, 2 or 1
        const int kg = lane % KG;
        const int k4 = 4 * kg;
        const int r0 = 4 * warp + (lane / KG) * RR;
        const bool kin = k4 < nrhs;       // nrhs is a multiple of 4: all four columns or none
        uint32_t gs = 0;   // ring stages consumed so far
        uint32_t tcg = 0;  // blocks multiplied on the tensor cores so far (phases of mma_done)
        for (uint32_t n = 0;; ++n) {
            const int slot = (int)(n & 1);
            bulk::mbar_wait(&sm.item_full[slot], (n >> 1) & 1, a.status);
            if (!sm.item_valid[slot]) break;
            const int v = sm.item_v[slot];
            const SnUnit U = sm.item_unit[slot];
            const int slice = sm.item_slice[slot];
            int* uf = a.uflags + (size_t)slice * a.flag_stride;  // the slice's flags
            float* xs = a.tmp + (size_t)slice * nrhs;            // the slice's first column
            float* pbs = a.pbuf + (size_t)slice * (a.flag_stride - a.n_units) * 32 * nrhs;  // its partial slots
            __syncwarp();
            if (lane == 0) bulk::mbar_arrive(&sm.item_empty[slot]);  // the descriptor has been read
            const SnbItem it = snb_item<LOWER>(a, v, U);
            const int uidx = it.uidx, w = U.w;
            // the unit's current right-hand side (my rows, my columns)
            float4 tv[RR];
#pragma unroll
            for (int r = 0; r < RR; ++r) {
                const int i = r0 + r;
                tv[r] = (!it.part && i < w && kin)
                            ? __ldcg(reinterpret_cast<const float4*>(xs + (size_t)(U.c0 + i) * ld + k4))
                            : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            // E and M to shared memory (read after the consumers' barrier
            // below; the previous item's readers passed its last barrier)
            const bool f2 = snb_folds2<LOWER>(a, it, U);
            const int nreg = it.nblk - (f2 ? 1 : 0);  // blocks before the folded one
            if (!it.part) {
                const float* dv = a.dinv + (size_t)uidx * 3 * kTile;
                const float* mc = dv + (LOWER ? 1 : 2) * kTile;
                for (int idx = tid; idx < kTile; idx += kCW * 32) {
                    // dv[i + 32 j] = D^-1[i][j]
                    if (LOWER) (&sm.e[0][0])[idx] = dv[idx];
                    else sm.e[idx & 31][idx >> 5] = dv[idx];
                    if (it.chain) (&sm.m[0][0])[idx] = mc[idx];
                }
            }
            float4 acc[RR];
#pragma unroll
            for (int r = 0; r < RR; ++r) acc[r] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int b = 0; b < nreg; ++b) {
                const uint32_t g = gs + (uint32_t)b;
                const int s = (int)(g % kStages);
                bulk::mbar_wait(&sm.full[s], (g / kStages) & 1, a.status);
                if constexpr (TC) {
                    // the previous block's MMAs have read the operand buffers
                    if (tcg > 0) bulk::mbar_wait(&sm.tc.mma_done, (tcg - 1) & 1, a.status);
                    snb_split<SW>(sm.st[s], sm.tc, sm.ext[s], nrhs, tid);
                    tc::fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) bulk::mbar_arrive(&sm.empty[s]);  // the stage is free again
                    bulk::named_sync(1, kCW * 32);
                    if (tid == 0) {
                        tc::fence_after_sync();
                        snb_mma(sm.tc, b == 0);
                    }
                    ++tcg;
                    continue;
                }
                const int ext = sm.ext[s];
                // the warp's 4 rows (columns): a block without any is skipped
                const bool mine = ((sm.mask[s] >> (4 * warp)) & 0xFu) != 0 && kin;
                const auto& st = sm.st[s];
                if (mine) {
                    auto step = [&](int j) {
                        const float4 xv = *reinterpret_cast<const float4*>(&st.x[j * nrhs + k4]);
                        float lr[RR];
                        load_rows<RR>(&st.l[j][r0], lr);
#pragma unroll
                        for (int r = 0; r < RR; ++r) {
                            acc[r].x = fmaf(lr[r], xv.x, acc[r].x);
                            acc[r].y = fmaf(lr[r], xv.y, acc[r].y);
                            acc[r].z = fmaf(lr[r], xv.z, acc[r].z);
                            acc[r].w = fmaf(lr[r], xv.w, acc[r].w);
                        }
                    };
                    int j = 0;
                    for (; j + 4 <= ext; j += 4) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) step(j + u);
                    }
                    for (; j < ext; ++j) step(j);
                }
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&sm.empty[s]);
            }
            gs += (uint32_t)nreg;
            if constexpr (TC) {
                // the accumulator (lane = RHS column, 16 columns = unit rows
                // per warp) goes through shared memory into this mapping
                if (nreg > 0) {
                    bulk::mbar_wait(&sm.tc.mma_done, (tcg - 1) & 1, a.status);
                    tc::fence_after_sync();
                    float t16[16];
                    const int kk = 32 * (warp & 3) + lane, rr0 = 16 * (warp >> 2);
                    tc::ld16(sm.tc.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)rr0, t16);
                    tc::fence_before_sync();  // ordered before the next item's MMAs (barriers below)
#pragma unroll
                    for (int r = 0; r < 16; ++r) sm.t[rr0 + r][kk] = t16[r];
                    bulk::named_sync(1, kCW * 32);
#pragma unroll
                    for (int r = 0; r < RR; ++r) acc[r] = *reinterpret_cast<const float4*>(&sm.t[r0 + r][k4]);
                    bulk::named_sync(1, kCW * 32);
                }
            }
            if (it.part) {  // the sum goes to the partial's slot, then its flag
                float* ps = pbs + (size_t)(~v) * 32 * nrhs;
                if (kin) {
#pragma unroll
                    for (int r = 0; r < RR; ++r) *reinterpret_cast<float4*>(ps + (r0 + r) * nrhs + k4) = acc[r];
                }
                bulk::named_sync(1, kCW * 32);
                if (tid == 0) dev::st_release(uf + a.n_units + ~v, epoch);
                continue;
            }
            if (LOWER) {  // the unit's partial sums, in a fixed order
                const int pb = a.unit_info[(size_t)uidx * 4 + 2], pe = a.unit_info[(size_t)uidx * 4 + 3];
                for (int q = pb; q < pe; ++q) {
                    if (lane == 0) dev::wait_geq(uf + a.n_units + q, epoch, a.status);
                    __syncwarp();
                    const float* ps = pbs + (size_t)q * 32 * nrhs;
                    if (kin) {
#pragma unroll
                        for (int r = 0; r < RR; ++r) {
                            const float4 p4 = __ldcg(reinterpret_cast<const float4*>(ps + (r0 + r) * nrhs + k4));
                            acc[r].x += p4.x; acc[r].y += p4.y; acc[r].z += p4.z; acc[r].w += p4.w;
                        }
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < RR; ++r)
                *reinterpret_cast<float4*>(&sm.t[r0 + r][k4 < SW ? k4 : 0]) =
                    make_float4(tv[r].x - acc[r].x, tv[r].y - acc[r].y, tv[r].z - acc[r].z, tv[r].w - acc[r].w);
            bulk::named_sync(1, kCW * 32);
            // x = E t' (my rows, my columns). E is triangular (lower: D^-1,
            // upper: D^-T), so the warp's rows 4 warp .. 4 warp + 3 need only
            // j <= 4 warp + 3 (lower) / j >= 4 warp (upper)
            float4 xv[RR];
#pragma unroll
            for (int r = 0; r < RR; ++r) xv[r] = make_float4(0.f, 0.f, 0.f, 0.f);
            const int ej0 = LOWER ? 0 : 4 * warp, ej1 = LOWER ? 4 * warp + 4 : 32;
#pragma unroll 4
            for (int j = ej0; j < ej1; ++j) {
                const float4 tj = *reinterpret_cast<const float4*>(&sm.t[j][k4 < SW ? k4 : 0]);
                float ev4[RR];
                load_rows<RR>(&sm.e[j][r0], ev4);
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    const float ev = ev4[r];
                    xv[r].x = fmaf(ev, tj.x, xv[r].x);
                    xv[r].y = fmaf(ev, tj.y, xv[r].y);
                    xv[r].z = fmaf(ev, tj.z, xv[r].z);
                    xv[r].w = fmaf(ev, tj.w, xv[r].w);
                }
            }
            // x -= M x_c for the chain chunk c (unit cu, work-array rows crow ..
            // crow + cw - 1): once its flag is set, its rows replace t' in
            // shared memory (every consumer has finished reading t')
            auto fold = [&](int cu, int crow, int cw, const float (&mt)[32][32]) {
                // one poller: its acquire and the barrier order every
                // consumer's loads after the chain unit's release (eight
                // pollers would wait for the slowest one's round trip)
                if (tid == 0) dev::wait_geq(uf + cu, epoch, a.status);
                bulk::named_sync(1, kCW * 32);
                const int q4 = nrhs >> 2;  // 16-byte pieces per row
                constexpr int kSteps = SW / 32;  // 32 rows x SW columns over the consumer threads
                float4 xc[kSteps];
#pragma unroll
                for (int st = 0; st < kSteps; ++st) {
                    const int f = tid + st * kCW * 32, j = f / q4;
                    xc[st] = (f < 32 * q4 && j < cw)
                                 ? __ldcg(reinterpret_cast<const float4*>(xs + (size_t)(crow + j) * ld) + (f - j * q4))
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int st = 0; st < kSteps; ++st) {
                    const int f = tid + st * kCW * 32, j = f / q4;
                    if (f < 32 * q4) *reinterpret_cast<float4*>(&sm.t[j][4 * (f - j * q4)]) = xc[st];
                }
                bulk::named_sync(1, kCW * 32);
                if (kin) {
#pragma unroll 4
                    for (int j = 0; j < 32; ++j) {
                        const float4 xj = *reinterpret_cast<const float4*>(&sm.t[j][k4 < SW ? k4 : 0]);
                        float mv4[RR];
                        load_rows<RR>(&mt[j][r0], mv4);
#pragma unroll
                        for (int r = 0; r < RR; ++r) {
                            const float mv = mv4[r];
                            xv[r].x = fmaf(-mv, xj.x, xv[r].x);
                            xv[r].y = fmaf(-mv, xj.y, xv[r].y);
                            xv[r].z = fmaf(-mv, xj.z, xv[r].z);
                            xv[r].w = fmaf(-mv, xj.w, xv[r].w);
                        }
                    }
                }
            };
            if (f2) {  // the folded block: x -= M2 x_2 from its stage
                const uint32_t g = gs++;
                const int s = (int)(g % kStages);
                bulk::mbar_wait(&sm.full[s], (g / kStages) & 1, a.status);
                const int ext = sm.ext[s];
                const auto& st = sm.st[s];
                if (((sm.mask[s] >> (4 * warp)) & 0xFu) != 0 && kin) {
                    for (int j = 0; j < ext; ++j) {
                        const float4 xj = *reinterpret_cast<const float4*>(&st.x[j * nrhs + k4]);
                        float mv4[RR];
                        load_rows<RR>(&st.l[j][r0], mv4);
#pragma unroll
                        for (int r = 0; r < RR; ++r) {
                            const float mv = mv4[r];
                            xv[r].x = fmaf(-mv, xj.x, xv[r].x);
                            xv[r].y = fmaf(-mv, xj.y, xv[r].y);
                            xv[r].z = fmaf(-mv, xj.z, xv[r].z);
                            xv[r].w = fmaf(-mv, xj.w, xv[r].w);
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) bulk::mbar_arrive(&sm.empty[s]);
            }
            if (it.chain) {  // the chain unit: lower, the previous chunk; upper, the next one
                if (LOWER) fold(uidx - 1, U.c0 - 32, 32, sm.m);
                else fold(uidx + 1, U.c0 + w, min(32, U.sn_w - (U.pos0 + w)), sm.m);
            }
            if (kin) {
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    const int i = r0 + r;
                    if (i < w) *reinterpret_cast<float4*>(xs + (size_t)(U.c0 + i) * ld + k4) = xv[r];
                }
            }
            // the barrier orders the consumers' writes before the release
            bulk::named_sync(1, kCW * 32);
            if (tid == 0) dev::st_release(uf + uidx, epoch);
        }
        if constexpr (TC) {
            // every MMA has completed before the accumulator is freed (the
            // consumers waited for each item's last one; this matters only
            // after an abandoned wait)
            if (tid == 0 && tcg > 0) bulk::mbar_wait(&sm.tc.mma_done, (tcg - 1) & 1, a.status, false);
        }
    }
    __syncthreads();
    if constexpr (TC) {
        tc::fence_after_sync();
        if (warp == 0) tc::dealloc(sm.tc.tmem, 32);
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

template <class io, bool LOWER, int SW, bool TC>
cudaError_t launch_snb(const SnbArgs& a, cudaStream_t stream) {
    const void* fn = (const void*)snb_sweep_kernel<io, LOWER, SW, TC>;
    const size_t smem = sizeof(SnbSmem<SW, LOWER, TC>);
    int grid = 0;
    cudaError_t e = coop_grid(fn, kThreads, smem, &grid);  // resident CTAs: a persistent grid
    if (e != cudaSuccess) return e;
    if (grid > a.nitems) grid = a.nitems;
    snb_sweep_kernel<io, LOWER, SW, TC><<<grid, kThreads, smem, stream>>>(a);
    return cudaGetLastError();
}

template <class io>
cudaError_t launch_snb_io(const SnbArgs& a, bool lower, cudaStream_t stream) {
    if (a.tensor_cores)
        return lower ? launch_snb<io, true, 128, true>(a, stream) : launch_snb<io, false, 128, true>(a, stream);
    if (snb_width(a.nrhs) == 32)
        return lower ? launch_snb<io, true, 32, false>(a, stream) : launch_snb<io, false, 32, false>(a, stream);
    if (snb_width(a.nrhs) == 64)
        return lower ? launch_snb<io, true, 64, false>(a, stream) : launch_snb<io, false, 64, false>(a, stream);
    return lower ? launch_snb<io, true, 128, false>(a, stream) : launch_snb<io, false, 128, false>(a, stream);
}

// Lower tiles: warp per contribution block, lane = unit row i; tile[j][i] =
// L[row i, source column j] (the block's rows are the set bits of its row
// mask, in order).
__global__ void expand_lower_kernel(const SnContrib* __restrict__ contribs, int64_t n,
                                    const float* __restrict__ panels, float* __restrict__ tiles) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < n; b += nw) {
        const SnContrib C = contribs[b];
        const bool has = (C.rowmask >> lane) & 1u;
        const int ci = __popc(C.rowmask & ((1u << lane) - 1u));
        float* out = tiles + b * kTile;
        for (int j = 0; j < 32; ++j)
            out[j * 32 + lane] = (has && j < C.w) ? panels[C.panel_off + (int64_t)j * C.ld + ci] : 0.f;
    }
}

// Upper tiles: warp per block, lane = block row i; tile[i][c] = L[row i,
// unit column c] = panels[src + c * ld + i].
__global__ void expand_upper_kernel(const int64_t* __restrict__ src, const int32_t* __restrict__ ld,
                                    const int32_t* __restrict__ nrw, int64_t n, const float* __restrict__ panels,
                                    float* __restrict__ tiles) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < n; b += nw) {
        const int nr = nrw[b] & 0xffff, w = nrw[b] >> 16;
        const int64_t s0 = src[b];
        const int l = ld[b];
        float* out = tiles + b * kTile;
        for (int c = 0; c < 32; ++c)
            out[lane * 32 + c] = (lane < nr && c < w) ? panels[s0 + (int64_t)c * l + lane] : 0.f;
    }
}

// The top rows' part of the solution, out[perm[row]] = (or +=) tmp[row],
// after the upper sweep (one CTA per unit, coalesced along each row).
template <class io>
__global__ void __launch_bounds__(256) scatter_kernel(const SnUnit* __restrict__ units, const int32_t* __restrict__ perm,
                                                      const float* __restrict__ tmp, void* out_, int nrhs,
                                                      const int* skip) {
    if (skip && dev::ld_volatile(skip)) return;
    using TO = typename io::tout;
    TO* out = static_cast<TO*>(out_);
    const SnUnit U = units[blockIdx.x];
    for (int idx = threadIdx.x; idx < U.w * nrhs; idx += blockDim.x) {
        const int i = idx / nrhs, k = idx - i * nrhs;
        const size_t oo = (size_t)perm[U.c0 + i] * nrhs + k;
        const TO v = (TO)tmp[(size_t)(U.c0 + i) * nrhs + k];
        if (io::accum) out[oo] += v;
        else out[oo] = v;
    }
}

template <class io>
cudaError_t launch_scatter_io(const SnbArgs& a, int nunits, cudaStream_t stream) {
    scatter_kernel<io><<<nunits, 256, 0, stream>>>(a.units, a.perm, a.tmp, a.out, a.nrhs, a.skip);
    return cudaGetLastError();
}

int expand_grid(int64_t n) {
    const int64_t blocks = (n * 32 + 255) / 256;
    return (int)(blocks < 4096 ? (blocks > 0 ? blocks : 1) : 4096);
}

}  // namespace

cudaError_t launch_snb_sweep(const SnbArgs& a, bool lower, SweepIO io, cudaStream_t stream) {
    if (a.nitems == 0) return cudaSuccess;
    if (!snb_supported(a.nrhs)) return cudaErrorInvalidValue;
    switch (io) {
        case SweepIO::F32: return launch_snb_io<SnbIO<float, false>>(a, lower, stream);
        case SweepIO::F32_MIXED: return launch_snb_io<SnbIO<double, false>>(a, lower, stream);
        case SweepIO::F32_REFINE: return launch_snb_io<SnbIO<double, true>>(a, lower, stream);
        default: return cudaErrorInvalidValue;  // FP64 solves use solve_sn.cu
    }
}

cudaError_t launch_snb_scatter(const SnbArgs& a, int nunits, SweepIO io, cudaStream_t stream) {
    if (nunits == 0) return cudaSuccess;
    switch (io) {
        case SweepIO::F32: return launch_scatter_io<SnbIO<float, false>>(a, nunits, stream);
        case SweepIO::F32_MIXED: return launch_scatter_io<SnbIO<double, false>>(a, nunits, stream);
        case SweepIO::F32_REFINE: return launch_scatter_io<SnbIO<double, true>>(a, nunits, stream);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_snb_expand_lower(const SnContrib* contribs, int64_t n, const float* panels, float* tiles,
                                    cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    expand_lower_kernel<<<expand_grid(n), 256, 0, stream>>>(contribs, n, panels, tiles);
    return cudaGetLastError();
}

cudaError_t launch_snb_expand_upper(const int64_t* src, const int32_t* ld, const int32_t* nrw, int64_t n,
                                    const float* panels, float* tiles, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    expand_upper_kernel<<<expand_grid(n), 256, 0, stream>>>(src, ld, nrw, n, panels, tiles);
    return cudaGetLastError();
}

}  // namespace gbchol
