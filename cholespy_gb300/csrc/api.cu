// C ABI of gbchol (include/gbchol.h): solver handle, factor upload, level
// analysis, solves and refinement.
//
// Host-side counterpart of the reference's CholeskySolver<Float>
// (src/cholesky_solver.h:22-99, src/cholesky_solver.cpp:152-486) and of the
// CUDA driver shim (src/cuda_driver.cpp): this library links the CUDA
// runtime directly and shares the primary context with PyTorch.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "grad.h"
#include "prep.h"
#include "solver_impl.h"

using namespace gbchol;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace gbchol {
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
}  // namespace gbchol

namespace {

// Validates a CSC factor: diagonal first and positive-free of structure
// errors (sorted strictly increasing rows, all rows in [col, n)).
int validate_factor(int32_t n, const int32_t* perm, const int32_t* colptr, const int32_t* rowidx) {
    if (n < 0) return fail(GBCHOL_EINVAL, "Invalid factor: negative size.");
    std::vector<char> seen((size_t)n, 0);
    for (int32_t k = 0; k < n; ++k) {
        if (perm[k] < 0 || perm[k] >= n || seen[perm[k]])
            return fail(GBCHOL_EINVAL, "Invalid factor: perm is not a permutation.");
        seen[perm[k]] = 1;
    }
    if (colptr[0] != 0) return fail(GBCHOL_EINVAL, "Invalid factor: colptr[0] != 0.");
    for (int32_t j = 0; j < n; ++j) {
        int32_t s = colptr[j], e = colptr[j + 1];
        if (e <= s) return fail(GBCHOL_EINVAL, "Invalid factor: empty column (missing diagonal).");
        if (rowidx[s] != j) return fail(GBCHOL_EINVAL, "Invalid factor: diagonal must come first.");
        for (int32_t k = s + 1; k < e; ++k)
            if (rowidx[k] <= rowidx[k - 1] || rowidx[k] >= n)
                return fail(GBCHOL_EINVAL, "Invalid factor: row indices must be sorted and < n.");
    }
    return GBCHOL_OK;
}

// Fundamental supernodes of a factor pattern (for statistics and the
// supernodal kernels): column j+1 continues j's supernode when it is j's
// only child and has j's structure minus j.
void detect_supernodes(Factor& F) {
    const int32_t n = F.n;
    F.parent.assign((size_t)n, -1);
    std::vector<int32_t> nchild((size_t)n, 0);
    for (int32_t j = 0; j < n; ++j) {
        if (F.colptr[j + 1] - F.colptr[j] > 1) {
            F.parent[j] = F.rowidx[F.colptr[j] + 1];
            nchild[F.parent[j]]++;
        }
    }
    F.sn_start.assign(1, 0);
    for (int32_t j = 1; j < n; ++j) {
        int32_t cp = F.colptr[j] - F.colptr[j - 1], cc = F.colptr[j + 1] - F.colptr[j];
        bool merge = F.parent[j - 1] == j && cp == cc + 1 && nchild[j] == 1;
        if (!merge) F.sn_start.push_back(j);
    }
    F.sn_start.push_back(n);
}

// Host counting sort of rows by level, stable in row id: the `levels` array
// of the reference (src/cholesky_solver.cpp:349-367).
void sort_by_level(const std::vector<int32_t>& lev, int32_t max_lvl, std::vector<int32_t>& order) {
    const int32_t n = (int32_t)lev.size();
    std::vector<int32_t> ptr((size_t)max_lvl + 2, 0);
    for (int32_t i = 0; i < n; ++i) ptr[(size_t)lev[i] + 1]++;
    for (int32_t l = 0; l <= max_lvl; ++l) ptr[(size_t)l + 1] += ptr[l];
    order.resize((size_t)n);
    for (int32_t i = 0; i < n; ++i) order[ptr[lev[i]]++] = i;
}

// Elimination-tree level candidates: height (L) or depth (L^T) of every
// node, with parent(j) = first off-diagonal row of column j of L.
void tree_levels(const Factor& F, bool lower, std::vector<int32_t>& lev) {
    const int32_t n = F.n;
    std::vector<int32_t> parent((size_t)n, -1);
    for (int32_t j = 0; j < n; ++j)
        if (F.colptr[j + 1] - F.colptr[j] > 1) parent[j] = F.rowidx[F.colptr[j] + 1];
    lev.assign((size_t)n, 0);
    if (lower) {
        for (int32_t j = 0; j < n; ++j)
            if (parent[j] >= 0) lev[parent[j]] = std::max(lev[parent[j]], lev[j] + 1);
    } else {
        for (int32_t j = n - 1; j >= 0; --j)
            if (parent[j] >= 0) lev[j] = lev[parent[j]] + 1;
    }
}

int analyze_triangle(gbchol_solver* h, Triangle& t, bool lower) {
    const int32_t n = h->n;
    DevBuf<int32_t> lev;
    CUDA_TRY(lev.alloc((size_t)n));
    // fast path: etree candidates verified on the GPU against every nonzero
    const char* force = std::getenv("GBCHOL_SYNCFREE_ANALYSIS");
    bool verified = false;
    if (!(force && force[0] == '1')) {
        tree_levels(h->F, lower, t.row_levels);
        CUDA_TRY(cudaMemcpy(lev.p, t.row_levels.data(), sizeof(int32_t) * (size_t)n,
                            cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemset(h->max_lvl.p, 0, sizeof(int32_t)));
        // both triangles are checked on L's columns (the upper triangle's rows)
        CUDA_TRY(launch_level_verify(lower, n, h->upper.rowptr.p, h->upper.cols.p, lev.p, h->max_lvl.p, nullptr));
        int32_t mism = 1;
        CUDA_TRY(cudaMemcpy(&mism, h->max_lvl.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
        verified = mism == 0;
        if (verified) {
            t.max_lvl = 0;
            for (int32_t v : t.row_levels) t.max_lvl = std::max(t.max_lvl, v);
        }
    }
    t.general_kernel = !verified;
    if (!verified) {
        if (lower && !t.rowptr.p) {
            // L in CSR (cholmod_transpose, :252): columns ascending, diagonal
            // last; the general kernel walks rows
            std::vector<int32_t> rp, ci;
            std::vector<double> none;
            transpose_columns(n, h->F.colptr, h->F.rowidx, nullptr, nullptr, rp, ci, none);
            CUDA_TRY(t.rowptr.upload(rp.data(), rp.size()));
            CUDA_TRY(t.cols.upload(ci.data(), ci.size()));
        }
        CUDA_TRY(cudaMemset(h->max_lvl.p, 0, sizeof(int32_t)));
        int ep = h->next_epoch(nullptr);
        CUDA_TRY(launch_level_analysis(lower, n, t.rowptr.p, t.cols.p, lev.p, h->flags.p, ep,
                                       h->max_lvl.p, h->status.p, nullptr));
        CUDA_TRY(cudaDeviceSynchronize());
        int32_t st = 0;
        CUDA_TRY(cudaMemcpy(&st, h->status.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (st != 0) {
            cudaMemset(h->status.p, 0, sizeof(int32_t));
            return fail(GBCHOL_ETIMEOUT, "Level analysis: a device-side wait expired (malformed factor?).");
        }
        t.row_levels.resize((size_t)n);
        CUDA_TRY(cudaMemcpy(t.row_levels.data(), lev.p, sizeof(int32_t) * (size_t)n,
                            cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(&t.max_lvl, h->max_lvl.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
    }
    sort_by_level(t.row_levels, t.max_lvl, t.order_h);
    CUDA_TRY(t.order.upload(t.order_h.data(), (size_t)n));
    return GBCHOL_OK;
}

template <typename T>
cudaError_t upload_cast(DevBuf<T>& dst, const std::vector<double>& src) {
    std::vector<T> tmp(src.size());
    const int64_t cnt = (int64_t)src.size();
#pragma omp parallel for schedule(static) if (cnt >= ((int64_t)1 << 20))
    for (int64_t k = 0; k < cnt; ++k) tmp[k] = (T)src[k];
    return dst.upload(tmp.data(), tmp.size());
}

// The bulk sweeps' tiles and schedule (FP32 factor, no 32-column partial
// sums), the tiles expanded on the device from the FP32 panels. Skipped (the
// solves then use the 32-column sweeps for every RHS count) when the tiles
// would take more than half of the free device memory.
int setup_snb(gbchol_solver* h) {
    const SolvePlan& P = h->plan;
    h->snb_ready = false;
    h->snb_lo_tiles.release();
    h->snb_up_tiles.release();
    if (!(h->store & GBCHOL_STORE_F32) || P.units.empty() || !P.parts.empty()) return GBCHOL_OK;
    if (const char* env = std::getenv("GBCHOL_BULK_MIN_RHS")) h->snb_min_rhs = std::atoi(env);
    if (const char* env = std::getenv("GBCHOL_BULK_TC")) h->snb_tc = std::atoi(env) != 0;
    if (const char* env = std::getenv("GBCHOL_BULK_SLICES")) h->snb_slices = std::atoi(env);
    SnbOptions so;
    if (const char* env = std::getenv("GBCHOL_BULK_FOLD")) so.fold = std::atoi(env);
    SnbUpperPlan B;
    build_snb_upper(P, B);
    if (const char* env = std::getenv("GBCHOL_BULK_KEEP")) so.keep = std::atoi(env);
    if (const char* env = std::getenv("GBCHOL_BULK_GROUP")) so.group = std::atoi(env);
    if (const char* env = std::getenv("GBCHOL_BULK_BLK_NS")) so.blk_ns = std::atoll(env);
    if (const char* env = std::getenv("GBCHOL_BULK_BASE_NS")) so.base_ns = std::atoll(env);
    so.max_cols = snb_group_cols(h->snb_tc || h->snb_tc_groups);
    if (const char* env = std::getenv("GBCHOL_BULK_ORDER")) so.order_by_finish = std::atoi(env) != 0;
    if (const char* env = std::getenv("GBCHOL_BULK_GROUP_COLS"))
        so.max_cols = std::min(so.max_cols, std::max(32, std::atoi(env)));
    SnbLowerPlan L;
    build_snb_lower(P, B, so, L);
    const size_t nlo = P.contribs.size(), nup = B.dep.size();
    const size_t bytes = (nlo + nup) * 32 * 32 * sizeof(float);
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (bytes > free_b / 2) return GBCHOL_OK;
    CUDA_TRY(h->snb_up_begin.upload(B.begin.data(), B.begin.size()));
    CUDA_TRY(h->snb_up_dep.upload(B.dep.data(), B.dep.size()));
    CUDA_TRY(h->snb_up_rows.upload(B.rows.data(), B.rows.size()));
    CUDA_TRY(h->snb_unit_info.upload(L.unit_info.data(), L.unit_info.size()));
    CUDA_TRY(h->snb_groups.upload(L.groups.data(), L.groups.size()));
    CUDA_TRY(h->snb_parts.upload(L.parts.data(), L.parts.size()));
    CUDA_TRY(h->snb_order_lo.upload(L.order_lo.data(), L.order_lo.size()));
    CUDA_TRY(h->snb_order_up.upload(L.order_up.data(), L.order_up.size()));
    h->snb_nparts = (int32_t)L.parts.size();
    h->snb_group_cols = so.max_cols;
    h->snb_fold = so.fold;
    // the folded tiles depend only on the factor: a rebuild for other group
    // widths (after the host copy was dropped) keeps the uploaded ones
    if (!P.fold2.empty()) CUDA_TRY(upload_cast(h->snb_fold2, P.fold2));
    // flags of the bulk partial sums follow the units', per column slice (up to 4)
    if (h->uflags.count < (P.units.size() + L.parts.size()) * 4) {
        CUDA_TRY(h->uflags.alloc((P.units.size() + L.parts.size()) * 4));
        CUDA_TRY(cudaMemset(h->uflags.p, 0, sizeof(int32_t) * h->uflags.count));
    }
    CUDA_TRY(h->snb_lo_tiles.alloc(std::max<size_t>(1, nlo) * 32 * 32));
    CUDA_TRY(h->snb_up_tiles.alloc(std::max<size_t>(1, nup) * 32 * 32));
    DevBuf<int64_t> src;
    DevBuf<int32_t> ld, nrw;
    CUDA_TRY(src.upload(B.src.data(), B.src.size()));
    CUDA_TRY(ld.upload(B.ld.data(), B.ld.size()));
    CUDA_TRY(nrw.upload(B.nrw.data(), B.nrw.size()));
    CUDA_TRY(launch_snb_expand_lower(h->contribs.p, (int64_t)nlo, h->pan32.p, h->snb_lo_tiles.p, 0));
    CUDA_TRY(launch_snb_expand_upper(src.p, ld.p, nrw.p, (int64_t)nup, h->pan32.p, h->snb_up_tiles.p, 0));
    CUDA_TRY(cudaDeviceSynchronize());
    h->snb_ready = true;
    return GBCHOL_OK;
}

// Uploads FP64 values and/or their FP32 copy: with both, the FP64 array goes
// up once and is cast on the device (the FP32 result equals the host cast).
cudaError_t upload_values(DevBuf<float>& d32, DevBuf<double>& d64, const std::vector<double>& src, bool f32,
                          bool f64) {
    if (!f64) return f32 ? upload_cast(d32, src) : cudaSuccess;
    cudaError_t e = d64.upload(src.data(), src.size());
    if (e != cudaSuccess || !f32) return e;
    e = d32.alloc(src.size());
    if (e != cudaSuccess) return e;
    e = cast_to_f32(d64.p, d32.p, (int64_t)src.size(), nullptr);
    return e != cudaSuccess ? e : cudaDeviceSynchronize();
}

// The leaf sweeps' wavefront (PlanOptions::leaf_group_rows, leaf_skew):
// the defaults, or GBCHOL_LEAF_GROUP_ROWS / GBCHOL_LEAF_SKEW.
void leaf_wavefront_options(PlanOptions& o) {
    o.leaf_group_rows = 0;
    o.leaf_skew = 0;
    if (const char* env = std::getenv("GBCHOL_LEAF_GROUP_ROWS")) o.leaf_group_rows = std::max(0, std::atoi(env));
    if (const char* env = std::getenv("GBCHOL_LEAF_SKEW")) o.leaf_skew = std::max(0, std::atoi(env));
    o.partial_last = true;
    if (const char* env = std::getenv("GBCHOL_PARTIAL_LAST")) o.partial_last = std::atoi(env) != 0;
}

// Builds the solve plan from the factor and the level orders and uploads it.
int setup_plan(gbchol_solver* h) {
    const Factor& F = h->F;
    const int32_t n = F.n;
    SolvePlan& P = h->plan;
    leaf_wavefront_options(h->plan_opt);
    if (const char* env = std::getenv("GBCHOL_UP_MERGE")) h->up_merge = std::atoi(env) != 0;
    try {
        build_plan(F, h->lower.order_h, h->upper.order_h, h->plan_opt, P);
    } catch (const std::exception& ex) {
        return fail(GBCHOL_EINTERNAL, std::string("solve plan: ") + ex.what());
    }
    const bool f32 = h->store & GBCHOL_STORE_F32, f64 = h->store & GBCHOL_STORE_F64;
    // lower leaf sweep: leaf rows + the leaf part of the top rows
    CUDA_TRY(h->lo_rowptr.upload(P.lo_rowptr.data(), P.lo_rowptr.size()));
    CUDA_TRY(h->lo_cols.upload(P.lo_cols.data(), P.lo_cols.size()));
    CUDA_TRY(h->lo_tasks.upload(P.lo_tasks.data(), P.lo_tasks.size()));
    CUDA_TRY(upload_values(h->lo_v32, h->lo_v64, P.lo_vals, f32, f64));
    // upper leaf sweep: top-row part (partial pass) and diagonal + leaf part
    CUDA_TRY(h->upt_rowptr.upload(P.upt_rowptr.data(), P.upt_rowptr.size()));
    CUDA_TRY(h->upt_cols.upload(P.upt_cols.data(), P.upt_cols.size()));
    CUDA_TRY(h->upt_tasks.upload(P.upt_tasks.data(), P.upt_tasks.size()));
    CUDA_TRY(upload_values(h->upt_v32, h->upt_v64, P.upt_vals, f32, f64));
    CUDA_TRY(h->up_rowptr.upload(P.upl_rowptr.data(), P.upl_rowptr.size()));
    CUDA_TRY(h->up_cols.upload(P.upl_cols.data(), P.upl_cols.size()));
    CUDA_TRY(upload_values(h->up_v32, h->up_v64, P.upl_vals, f32, f64));
    P.upt_vals.clear();
    P.upt_vals.shrink_to_fit();
    P.upl_vals.clear();
    P.upl_vals.shrink_to_fit();
    CUDA_TRY(h->up_tasks.upload(P.up_tasks.data(), P.up_tasks.size()));
    // top region
    CUDA_TRY(h->sn_rows.upload(P.sn_rows.data(), P.sn_rows.size()));
    CUDA_TRY(upload_values(h->pan32, h->pan64, P.panels, f32, f64));
    CUDA_TRY(h->units.upload(P.units.data(), P.units.size()));
    CUDA_TRY(h->order_lo.upload(P.unit_order_lo.data(), P.unit_order_lo.size()));
    CUDA_TRY(h->unit_of_row.upload(P.unit_of_row.data(), P.unit_of_row.size()));
    CUDA_TRY(h->order_up.upload(P.unit_order_up.data(), P.unit_order_up.size()));
    CUDA_TRY(upload_values(h->dinv32, h->dinv64, P.dinv, f32, f64));
    P.dinv.clear();
    P.dinv.shrink_to_fit();
    CUDA_TRY(h->counters.alloc(10));
    CUDA_TRY(cudaMemset(h->counters.p, 0, sizeof(int32_t) * 10));
    {
        // solve sweeps count epochs from 1 on the device; row flags start at
        // 0 (leaf rows) or INT_MAX (top rows, always ready for the row kernels)
        const int32_t one = 1;
        CUDA_TRY(h->dev_epoch.upload(&one, 1));
    }
    CUDA_TRY(h->contribs.upload(P.contribs.data(), P.contribs.size()));
    CUDA_TRY(h->parts.upload(P.parts.data(), P.parts.size()));
    // unit flags, then partial-sum flags; <= 8 RHS slices
    CUDA_TRY(h->uflags.alloc(std::max<size_t>(1, (P.units.size() + P.parts.size()) * 8)));
    CUDA_TRY(cudaMemset(h->uflags.p, 0, sizeof(int32_t) * h->uflags.count));
    if (int rc = setup_snb(h)) return rc;
    P.fold2.clear();
    P.fold2.shrink_to_fit();
    // row flags: top rows are always "ready" for the row kernels (they are
    // solved by the supernodal kernel in an earlier launch)
    h->flags_init.assign((size_t)n, 0);
    for (int32_t j = 0; j < n; ++j)
        if (P.row_top[j]) h->flags_init[j] = INT_MAX;
    CUDA_TRY(cudaMemcpy(h->flags.p, h->flags_init.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    P.panels.clear();
    P.panels.shrink_to_fit();
    P.lo_vals.clear();
    P.lo_vals.shrink_to_fit();
    // the analysis copies of the triangles are not used by the solves
    h->lower.v32.release(); h->lower.v64.release();
    h->upper.v32.release(); h->upper.v64.release();
    h->lower.rowptr.release(); h->lower.cols.release();
    h->upper.rowptr.release(); h->upper.cols.release();
    return GBCHOL_OK;
}

// Uploads the factor (both triangles) and runs the analysis.
int setup_device(gbchol_solver* h) {
    auto t0 = std::chrono::steady_clock::now();
    const Factor& F = h->F;
    const int32_t n = F.n;
    CUDA_TRY(cudaGetDevice(&h->device));
    CUDA_TRY(h->perm.upload(F.perm.data(), (size_t)n));
    CUDA_TRY(h->flags.alloc((size_t)std::max(n, 1)));
    CUDA_TRY(cudaMemset(h->flags.p, 0, sizeof(int32_t) * (size_t)std::max(n, 1)));
    CUDA_TRY(h->status.alloc(1));
    CUDA_TRY(cudaMemset(h->status.p, 0, sizeof(int32_t)));
    CUDA_TRY(h->max_lvl.alloc(1));
    // L^T in CSR is L in CSC (the reference's "upper" triangle, :280); L's
    // CSR is built only if the general analysis kernel has to run
    CUDA_TRY(h->upper.rowptr.upload(F.colptr.data(), (size_t)n + 1));
    CUDA_TRY(h->upper.cols.upload(F.rowidx.data(), F.rowidx.size()));
    if (n > 0) {
        int rc = analyze_triangle(h, h->lower, true);
        if (rc) return rc;
        rc = analyze_triangle(h, h->upper, false);
        if (rc) return rc;
        rc = setup_plan(h);
        if (rc) return rc;
    }
    CUDA_TRY(cudaDeviceSynchronize());
    h->t_analysis = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return GBCHOL_OK;
}

int check_store(int32_t store) {
    if ((store & ~(GBCHOL_STORE_F32 | GBCHOL_STORE_F64 | GBCHOL_STORE_A64)) != 0 ||
        (store & (GBCHOL_STORE_F32 | GBCHOL_STORE_F64)) == 0)
        return fail(GBCHOL_EINVAL, "Invalid storage flags.");
    return GBCHOL_OK;
}

int ensure_tmp(gbchol_solver* h, size_t bytes) {
    if (h->tmp.count >= bytes) return GBCHOL_OK;
    CUDA_TRY(h->tmp.alloc(bytes));
    return GBCHOL_OK;
}

int check_rhs(int32_t nrhs) {
    if (nrhs > GBCHOL_MAX_RHS) return fail(GBCHOL_EINVAL, "The number of RHS should be less than 128.");
    if (nrhs < 1) return fail(GBCHOL_EINVAL, "The number of RHS must be at least 1.");
    return GBCHOL_OK;
}

}  // namespace

int gbchol::row_chunk() {
    const char* e = std::getenv("GBCHOL_ROW_CHUNK");
    int c = e ? std::atoi(e) : 1;
    return c < 1 ? 1 : (c > 64 ? 64 : c);
}

namespace {
// Column slices of a bulk-sweep kind (3: two, 4: four), when nrhs splits into
// that many slices of a multiple of 4 columns; else 1.
int snb_kind_slices(int kind, int nrhs) {
    const int s = kind == 3 ? 2 : (kind == 4 ? 4 : 1);
    return (s > 1 && nrhs % (4 * s) == 0) ? s : 1;
}

// Supernodal kernel of a solve: 0 the 32-column sweeps, 1 the bulk sweeps,
// 2 the bulk sweeps on the tensor cores (tiles built for groups of <= 32
// columns), 3 / 4 the bulk sweeps with 2 / 4 column slices per unit. An
// autotuned choice for this RHS count wins over the defaults.
int sn_kind(const gbchol_solver* h, int nrhs, bool f32) {
    if (!f32 || !h->snb_ready || !snb_supported(nrhs)) return 0;
    const auto& t = h->tuned[nrhs];
    if (t.valid) {
        if (t.sn == 2 && h->snb_group_cols > 32) return 1;
        if (t.sn >= 3 && snb_kind_slices(t.sn, nrhs) == 1) return 1;
        return t.sn;
    }
    if (nrhs < h->snb_min_rhs) return 0;
    if (h->snb_tc && h->snb_group_cols <= 32) return 2;
    const int kind = h->snb_slices == 4 ? 4 : (h->snb_slices == 2 ? 3 : 1);
    return snb_kind_slices(kind, nrhs) > 1 ? kind : 1;
}
bool use_snb(const gbchol_solver* h, int nrhs, bool f32) { return sn_kind(h, nrhs, f32) != 0; }
}  // namespace

size_t gbchol::work_bytes(const gbchol_solver* h, int nrhs, bool f32) {
    const size_t es = f32 ? sizeof(float) : sizeof(double);
    const size_t x = ((size_t)std::max(h->n, 1) * nrhs * es + 255) / 256 * 256;
    if (use_snb(h, nrhs, f32))  // the bulk sweeps' partial-sum slots
        return x + (size_t)h->snb_nparts * 32 * nrhs * sizeof(float);
    return x + sn_pbuf_bytes((int)h->plan.parts.size(), nrhs, !f32, false);
}

// One full solve with the work array `work` (work_bytes: the permuted-space
// n x nrhs array of T, then the partial-sum slots): leaf rows (lower) -> top
// units (lower) -> top units (upper) -> leaf rows (upper). `in` is read
// through perm by the lower leaf kernel; `out` is written through perm by the
// upper kernels (the bulk sweeps' top rows by their scatter launch).
int gbchol::run_sweeps_with(gbchol_solver* h, bool f32, SweepIO io, int nrhs, const void* in,
                            void* out, const int* skip, void* work, cudaStream_t s) {
    const SolvePlan& P = h->plan;
    RowSys rs;
    rs.perm = h->perm.p;
    rs.tmp = work;
    rs.flags = h->flags.p;
    rs.nrhs = nrhs;
    RowSweepArgs lo;
    lo.sys0 = rs;
    lo.sys0.rowptr = h->lo_rowptr.p;
    lo.sys0.cols = h->lo_cols.p;
    lo.sys0.vals = f32 ? (const void*)h->lo_v32.p : (const void*)h->lo_v64.p;
    lo.sys0.in = in;
    lo.tasks = h->lo_tasks.p;
    lo.ntasks = (int)P.lo_tasks.size();
    lo.status = h->status.p;
    lo.skip = skip;
    lo.counters = h->counters.p;
    const auto& tune = h->tuned[nrhs];
    lo.chunk = tune.valid ? tune.chunk : row_chunk();
    lo.max_nrhs = nrhs;
    // 2..8 RHS: lanes over the RHS columns (16-lane groups taking alternate
    // nonzeros) unless tuned otherwise; measured on GB300 (FP32, lanes over
    // the nonzeros -> over the RHS): icosphere 7, 3 / 8 RHS 0.861 -> 0.769 /
    // 1.122 -> 0.792 ms; icosphere 6, 3 RHS 0.561 -> 0.425 ms; 64^3, 4 RHS
    // 2.708 -> 2.594 ms; 64x64 grid, 3 RHS 0.416 -> 0.255 ms (1 RHS: equal)
    lo.rhs_split = tune.valid ? tune.rhs_split : (nrhs >= 2 && nrhs <= 8 ? 1 : 0);
    lo.epoch = h->dev_epoch.p;
    CUDA_TRY(launch_row_sweep(lo, true, io, s));
    SnSweepArgs sn;
    sn.sys0.units = h->units.p;
    sn.sys0.contribs = h->contribs.p;
    sn.sys0.sn_rows = h->sn_rows.p;
    sn.sys0.panels = f32 ? (const void*)h->pan32.p : (const void*)h->pan64.p;
    sn.sys0.dinv = f32 ? (const void*)h->dinv32.p : (const void*)h->dinv64.p;
    sn.sys0.perm = h->perm.p;
    sn.sys0.tmp = work;
    sn.sys0.uflags = h->uflags.p;
    sn.sys0.unit_of_row = h->unit_of_row.p;
    sn.sys0.parts = h->parts.p;
    sn.sys0.pbuf = static_cast<unsigned char*>(work) +
                   ((size_t)h->n * nrhs * (f32 ? sizeof(float) : sizeof(double)) + 255) / 256 * 256;
    if (use_snb(h, nrhs, f32)) {
        // 12..128 RHS (multiples of 4): the bulk-copy supernodal sweeps (solve_snb.cu)
        SnbArgs b;
        b.units = h->units.p;
        b.contribs = h->contribs.p;
        b.lo_tiles = h->snb_lo_tiles.p;
        b.up_tiles = h->snb_up_tiles.p;
        b.up_begin = h->snb_up_begin.p;
        b.up_rows = h->snb_up_rows.p;
        b.up_dep = h->snb_up_dep.p;
        b.groups = h->snb_groups.p;
        b.unit_info = h->snb_unit_info.p;
        b.parts = h->snb_parts.p;
        b.pbuf = reinterpret_cast<float*>(sn.sys0.pbuf);
        b.n_units = (int)P.units.size();
        b.dinv = h->dinv32.p;
        b.fold2 = h->snb_fold2.p;
        b.fold = h->snb_fold;
        b.perm = h->perm.p;
        b.tmp = static_cast<float*>(work);
        b.uflags = h->uflags.p;
        const int kind = sn_kind(h, nrhs, f32);
        const int nsl = snb_kind_slices(kind, nrhs);  // column slices: independent items per unit
        b.nrhs = nrhs / nsl;
        b.ld = nrhs;
        b.nslices = nsl;
        b.flag_stride = (int)P.units.size() + h->snb_nparts;
        b.tensor_cores = kind == 2 ? 1 : 0;
        b.status = h->status.p;
        b.skip = skip;
        b.epoch = h->dev_epoch.p;
        b.nitems = ((int)P.units.size() + h->snb_nparts) * nsl;
        b.order = h->snb_order_lo.p;
        b.counters = h->counters.p + 2;
        CUDA_TRY(launch_snb_sweep(b, true, io, s));
        b.out = nullptr;  // the top rows' output is scattered afterwards, off the chain
        b.nitems = (int)P.units.size() * nsl;
        b.order = h->snb_order_up.p;
        b.counters = h->counters.p + 4;
        CUDA_TRY(launch_snb_sweep(b, false, io, s));
        b.out = out;
        b.nrhs = nrhs;  // the scatter covers every column
        b.ld = 0;
        b.nslices = 1;
        CUDA_TRY(launch_snb_scatter(b, (int)P.units.size(), io, s));
    } else {
        sn.sys0.n_units = (int)P.units.size();
        sn.sys0.nrhs = nrhs;
        sn.sys0.nslices = sn_slices(nrhs, !f32);
        sn.nitems = (int)P.unit_order_lo.size() * sn.sys0.nslices;
        sn.status = h->status.p;
        sn.skip = skip;
        sn.order = h->order_lo.p;
        sn.counters = h->counters.p + 2;
        sn.epoch = h->dev_epoch.p;
        CUDA_TRY(launch_sn_sweep(sn, true, io, s));
        sn.sys0.out = out;
        sn.nitems = (int)P.units.size() * sn.sys0.nslices;
        sn.order = h->order_up.p;
        sn.counters = h->counters.p + 4;
        CUDA_TRY(launch_sn_sweep(sn, false, io, s));
    }
    // the leaf rows' top-row terms (final after the supernodal sweeps):
    // summed first by each leaf row of the upper sweep, with no flag checks,
    // so they overlap the leaf chain's waits (GB300 FP32, with / without a
    // separate wait-free pass launch: icosphere 7 / 3 RHS 0.854 / 0.942 ms,
    // 64^3 / 16 RHS 2.94 / 3.06 ms, / 128 RHS 4.17 / 4.20 ms; the 256-system
    // batch 16.0 / 16.5 ms); GBCHOL_UP_MERGE=0 keeps the separate pass
    RowSweepArgs pt = lo;
    pt.sys0.rowptr = h->upt_rowptr.p;
    pt.sys0.cols = h->upt_cols.p;
    pt.sys0.vals = f32 ? (const void*)h->upt_v32.p : (const void*)h->upt_v64.p;
    pt.sys0.in = nullptr;
    pt.sys0.out = out;
    pt.tasks = h->upt_tasks.p;
    pt.ntasks = (int)P.upt_tasks.size();
    pt.counters = h->counters.p + 8;
    if (!h->up_merge) CUDA_TRY(launch_row_sweep(pt, false, io, s));
    RowSweepArgs up = pt;
    up.sys0.rowptr = h->up_rowptr.p;
    up.sys0.cols = h->up_cols.p;
    up.sys0.vals = f32 ? (const void*)h->up_v32.p : (const void*)h->up_v64.p;
    if (h->up_merge) {
        up.sys0.nw_rowptr = pt.sys0.rowptr;
        up.sys0.nw_cols = pt.sys0.cols;
        up.sys0.nw_vals = pt.sys0.vals;
    }
    up.tasks = h->up_tasks.p;
    up.ntasks = (int)P.up_tasks.size();
    up.counters = h->counters.p + 6;
    CUDA_TRY(launch_row_sweep(up, false, io, s));
    return GBCHOL_OK;
}

namespace {

int run_sweeps(gbchol_solver* h, bool f32, SweepIO io, int nrhs, const void* in, void* out,
               const int* skip, cudaStream_t s) {
    return run_sweeps_with(h, f32, io, nrhs, in, out, skip, h->tmp.p, s);
}

// Kernel launches of one run_sweeps call.
int sweep_launches(const gbchol_solver* h) {
    const SolvePlan& P = h->plan;
    return (P.lo_tasks.empty() ? 0 : 1) + (P.units.empty() ? 0 : 2) + (P.upt_tasks.empty() || h->up_merge ? 0 : 1) +
           (P.up_tasks.empty() ? 0 : 1);
}

}  // namespace

extern "C" {

const char* gbchol_last_error(void) { return g_last_error.c_str(); }

const char* gbchol_version(void) { return "gbchol 0.1.0 (sm_103a)"; }

}  // extern "C"

namespace {

// The rest of construction once the input is a sorted, duplicate-summed CSC
// (host arrays ii / jj: the input's index arrays, recorded for the cached
// refactorisation).
int create_from_csc(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj, int32_t matrix_type,
                    int32_t store, Csc& A, gbchol_handle* out);

}  // namespace

extern "C" {

int gbchol_create(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj,
                  const double* x, int32_t matrix_type, int32_t store, gbchol_handle* out) {
    if (!out) return fail(GBCHOL_EINVAL, "out must not be NULL.");
    *out = nullptr;
    if (int rc = check_store(store)) return rc;
    if (n_rows < 0) return fail(GBCHOL_EINVAL, "The number of rows must be non-negative.");
    if (nnz > 0 && (!ii || !jj || !x)) return fail(GBCHOL_EINVAL, "Null input array.");
    if (matrix_type != GBCHOL_COO && !ii) return fail(GBCHOL_EINVAL, "Null pointer array.");
    std::string err;
    Csc A;
    Status st = build_csc(n_rows, nnz, ii, jj, x, matrix_type, A, err);
    if (st != ST_OK) return fail(GBCHOL_EINVAL, err);
    return create_from_csc(n_rows, nnz, ii, jj, matrix_type, store, A, out);
}

int gbchol_create_device(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                         int32_t matrix_type, int32_t store, gbchol_handle* out) {
    if (!out) return fail(GBCHOL_EINVAL, "out must not be NULL.");
    *out = nullptr;
    if (int rc = check_store(store)) return rc;
    if (n_rows < 0) return fail(GBCHOL_EINVAL, "The number of rows must be non-negative.");
    if (nnz < 0 || nnz >= (int64_t)INT32_MAX) return fail(GBCHOL_EINVAL, "Number of nonzero entries out of range.");
    if (nnz > 0 && (!ii || !jj || !x)) return fail(GBCHOL_EINVAL, "Null input array.");
    if (matrix_type != GBCHOL_COO && matrix_type != GBCHOL_CSR && matrix_type != GBCHOL_CSC)
        return fail(GBCHOL_EINVAL, "Unknown matrix type.");
    if (matrix_type != GBCHOL_COO && !ii) return fail(GBCHOL_EINVAL, "Null pointer array.");
    // the index arrays on the host: the pointer array's check, and the record
    // of the input pattern for the cached refactorisation
    const size_t nii = matrix_type == GBCHOL_COO ? (size_t)nnz : (size_t)n_rows + 1;
    std::vector<int32_t> hi(nii), hj((size_t)nnz);
    if (nii) CUDA_TRY(cudaMemcpy(hi.data(), ii, nii * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (nnz) CUDA_TRY(cudaMemcpy(hj.data(), jj, (size_t)nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (matrix_type != GBCHOL_COO) {
        const std::string what = matrix_type == GBCHOL_CSR ? "Sparse CSR matrix" : "Sparse CSC matrix";
        bool ok = hi[0] == 0 && (int64_t)hi[n_rows] == nnz;
        for (int32_t k = 0; ok && k < n_rows; ++k) ok = hi[k + 1] >= hi[k];
        if (!ok) return fail(GBCHOL_EINVAL, what + ": Invalid pointer array.");
    }
    DeviceCsc D;
    int bad = 0;
    CUDA_TRY(device_csc(n_rows, nnz, ii, jj, x, matrix_type, D, &bad, nullptr));
    if (bad)
        return fail(GBCHOL_EINVAL, matrix_type == GBCHOL_COO   ? "Sparse COO matrix: index out of range."
                                   : matrix_type == GBCHOL_CSR ? "Sparse CSR matrix: index out of range."
                                                                : "Sparse CSC matrix: index out of range.");
    Csc A;
    A.n = n_rows;
    A.colptr.resize((size_t)n_rows + 1);
    A.rowidx.resize((size_t)D.nnz);
    A.vals.resize((size_t)D.nnz);
    cudaError_t e = cudaMemcpy(A.colptr.data(), D.colptr, A.colptr.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && D.nnz)
        e = cudaMemcpy(A.rowidx.data(), D.rowidx, A.rowidx.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && D.nnz)
        e = cudaMemcpy(A.vals.data(), D.vals, A.vals.size() * sizeof(double), cudaMemcpyDeviceToHost);
    D.release();
    CUDA_TRY(e);
    return create_from_csc(n_rows, nnz, hi.data(), hj.data(), matrix_type, store, A, out);
}

}  // extern "C"

namespace {

int create_from_csc(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj, int32_t matrix_type,
                    int32_t store, Csc& A, gbchol_handle* out) {
    std::unique_ptr<gbchol_solver> h(new (std::nothrow) gbchol_solver());
    if (!h) return fail(GBCHOL_ENOMEM, "Out of host memory.");
    h->n = n_rows;
    h->store = store;
    std::string err;
    Status st = ST_OK;
    auto t0 = std::chrono::steady_clock::now();
    FactorOptions opt;
    st = factorize(A, opt, h->F, err);
    h->t_factor = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st == ST_NOT_POSDEF) return fail(GBCHOL_ENOTPOSDEF, "Matrix is not positive definite!");
    if (st != ST_OK) return fail(st == ST_NOMEM ? GBCHOL_ENOMEM : GBCHOL_EINVAL, err);
    record_input(h->F, nnz, ii, jj, matrix_type);
    if (store & GBCHOL_STORE_A64) {
        Csc S;
        symmetric_from_lower(A, S);
        h->nnz_a = S.nnz();
        CUDA_TRY(h->a_rowptr.upload(S.colptr.data(), S.colptr.size()));
        CUDA_TRY(h->a_cols.upload(S.rowidx.data(), S.rowidx.size()));
        CUDA_TRY(h->a_vals.upload(S.vals.data(), S.vals.size()));
    }
    if (int rc = setup_device(h.get())) return rc;
    *out = h.release();
    return GBCHOL_OK;
}

// Numeric factor of new values on the same pattern: the old ordering is
// given to the factorisation, and the resulting pattern must be the old one.
int refactor_values(const Factor& old, int32_t n, int64_t nnz, const int32_t* ii, const int32_t* jj,
                    const double* x, int32_t matrix_type, int32_t threads, Csc& A, Factor& Fn) {
    if (nnz > 0 && (!ii || !jj || !x)) return fail(GBCHOL_EINVAL, "Null input array.");
    if (matrix_type != GBCHOL_COO && !ii) return fail(GBCHOL_EINVAL, "Null pointer array.");
    if ((int32_t)old.perm.size() != n) return fail(GBCHOL_ESTATE, "No factor to refactorise.");
    std::string err;
    Status st = ST_OK;
    // the input pattern the factor was made from: numeric phase only
    if (refactor_cached(old, nnz, ii, jj, x, matrix_type, threads, A, Fn.vals, Fn.flops, st, err)) {
        if (st == ST_NOT_POSDEF) return fail(GBCHOL_ENOTPOSDEF, "Matrix is not positive definite!");
        if (st != ST_OK) return fail(st == ST_NOMEM ? GBCHOL_ENOMEM : GBCHOL_EINVAL, err);
        return GBCHOL_OK;
    }
    st = build_csc(n, nnz, ii, jj, x, matrix_type, A, err);
    if (st != ST_OK) return fail(GBCHOL_EINVAL, err);
    FactorOptions opt;
    opt.threads = threads;
    opt.use_given_perm = true;
    opt.perm_in = old.perm.data();
    st = factorize(A, opt, Fn, err);
    if (st == ST_NOT_POSDEF) return fail(GBCHOL_ENOTPOSDEF, "Matrix is not positive definite!");
    if (st != ST_OK) return fail(st == ST_NOMEM ? GBCHOL_ENOMEM : GBCHOL_EINVAL, err);
    if (Fn.perm != old.perm || Fn.colptr != old.colptr || Fn.rowidx != old.rowidx || Fn.sn_start != old.sn_start)
        return fail(GBCHOL_EINVAL, "The sparsity pattern differs from the factor's: make a new solver.");
    return GBCHOL_OK;
}

}  // namespace

extern "C" {

int gbchol_refactorize(gbchol_handle h, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                       int32_t matrix_type) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (h->n == 0) return GBCHOL_OK;
    auto t0 = std::chrono::steady_clock::now();
    Csc A;
    Factor Fn;
    if (int rc = refactor_values(h->F, h->n, nnz, ii, jj, x, matrix_type, 0, A, Fn)) return rc;
    Csc S;
    if (h->store & GBCHOL_STORE_A64) {
        symmetric_from_lower(A, S);
        if (S.nnz() != h->nnz_a) return fail(GBCHOL_EINVAL, "The sparsity pattern differs from the solver's.");
    }
    h->t_factor = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    DeviceGuard g(h->device);
    CUDA_TRY(cudaDeviceSynchronize());  // no solve may still use the old values
    h->F.vals.swap(Fn.vals);
    if (h->store & GBCHOL_STORE_A64) CUDA_TRY(h->a_vals.upload(S.vals.data(), S.vals.size()));
    ++h->plan_gen;
    if (int rc = setup_plan(h)) return rc;
    CUDA_TRY(cudaDeviceSynchronize());
    return GBCHOL_OK;
}

int gbchol_factor_refactorize(gbchol_factor_handle f, int64_t nnz, const int32_t* ii, const int32_t* jj,
                              const double* x, int32_t matrix_type, int32_t threads) {
    if (!f) return fail(GBCHOL_EINVAL, "Null factor.");
    if (f->F.n == 0) return GBCHOL_OK;
    Csc A;
    Factor Fn;
    if (int rc = refactor_values(f->F, f->F.n, nnz, ii, jj, x, matrix_type, threads, A, Fn)) return rc;
    f->F.vals.swap(Fn.vals);
    return GBCHOL_OK;
}

int gbchol_factor_solve(gbchol_factor_handle f, int32_t precision, int32_t nrhs, const void* b, void* x,
                        int32_t threads) {
    if (!f) return fail(GBCHOL_EINVAL, "Null factor.");
    if (precision != 0 && precision != 1) return fail(GBCHOL_EINVAL, "precision must be 0 (float) or 1 (double).");
    if (nrhs < 0) return fail(GBCHOL_EINVAL, "The number of RHS must be non-negative.");
    if (threads < 0) return fail(GBCHOL_EINVAL, "threads must be non-negative.");
    if (f->F.n > 0 && nrhs > 0 && (!b || !x)) return fail(GBCHOL_EINVAL, "Null b or x.");
    try {
        std::call_once(f->cpu_once, [&] { cpu_plan(f->F, f->cpu, threads); });
        cpu_solve(f->F, f->cpu, precision, nrhs, b, x, threads);
    } catch (const std::bad_alloc&) {
        return fail(GBCHOL_ENOMEM, "Out of host memory.");
    }
    return GBCHOL_OK;
}

int gbchol_create_from_factor(int32_t n, const int32_t* perm, const int32_t* colptr,
                              const int32_t* rowidx, const double* vals, int32_t store,
                              gbchol_handle* out) {
    if (!out) return fail(GBCHOL_EINVAL, "out must not be NULL.");
    *out = nullptr;
    if (int rc = check_store(store & ~GBCHOL_STORE_A64)) return rc;
    if (n < 0 || !perm || !colptr || (n > 0 && (!rowidx || !vals)))
        return fail(GBCHOL_EINVAL, "Invalid factor arrays.");
    if (int rc = validate_factor(n, perm, colptr, rowidx)) return rc;
    std::unique_ptr<gbchol_solver> h(new (std::nothrow) gbchol_solver());
    if (!h) return fail(GBCHOL_ENOMEM, "Out of host memory.");
    h->n = n;
    h->store = store & ~GBCHOL_STORE_A64;
    Factor& F = h->F;
    F.n = n;
    F.perm.assign(perm, perm + n);
    F.colptr.assign(colptr, colptr + n + 1);
    F.rowidx.assign(rowidx, rowidx + colptr[n]);
    F.vals.assign(vals, vals + colptr[n]);
    detect_supernodes(F);
    if (int rc = setup_device(h.get())) return rc;
    *out = h.release();
    return GBCHOL_OK;
}

int gbchol_factorize(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj,
                     const double* x, int32_t matrix_type, int32_t threads,
                     gbchol_factor_handle* out) {
    if (!out) return fail(GBCHOL_EINVAL, "out must not be NULL.");
    *out = nullptr;
    if (n_rows < 0) return fail(GBCHOL_EINVAL, "The number of rows must be non-negative.");
    if (nnz > 0 && (!ii || !jj || !x)) return fail(GBCHOL_EINVAL, "Null input array.");
    if (matrix_type != GBCHOL_COO && !ii) return fail(GBCHOL_EINVAL, "Null pointer array.");
    std::unique_ptr<gbchol_host_factor> f(new (std::nothrow) gbchol_host_factor());
    if (!f) return fail(GBCHOL_ENOMEM, "Out of host memory.");
    std::string err;
    Csc A;
    Status st = build_csc(n_rows, nnz, ii, jj, x, matrix_type, A, err);
    if (st != ST_OK) return fail(GBCHOL_EINVAL, err);
    FactorOptions opt;
    opt.threads = threads;
    st = factorize(A, opt, f->F, err);
    if (st == ST_NOT_POSDEF) return fail(GBCHOL_ENOTPOSDEF, "Matrix is not positive definite!");
    if (st != ST_OK) return fail(st == ST_NOMEM ? GBCHOL_ENOMEM : GBCHOL_EINVAL, err);
    record_input(f->F, nnz, ii, jj, matrix_type);
    *out = f.release();
    return GBCHOL_OK;
}

int gbchol_factor_info(gbchol_factor_handle f, int32_t* n, int64_t* nnz_l, int32_t* n_supernodes,
                       double* flops) {
    if (!f) return fail(GBCHOL_EINVAL, "Null factor.");
    if (n) *n = f->F.n;
    if (nnz_l) *nnz_l = f->F.nnz();
    if (n_supernodes) *n_supernodes = f->F.sn_start.empty() ? 0 : (int32_t)f->F.sn_start.size() - 1;
    if (flops) *flops = f->F.flops;
    return GBCHOL_OK;
}

int gbchol_factor_export(gbchol_factor_handle f, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                         double* vals) {
    if (!f) return fail(GBCHOL_EINVAL, "Null factor.");
    const Factor& F = f->F;
    if (perm) std::copy(F.perm.begin(), F.perm.end(), perm);
    if (colptr) std::copy(F.colptr.begin(), F.colptr.end(), colptr);
    if (rowidx) std::copy(F.rowidx.begin(), F.rowidx.end(), rowidx);
    if (vals) std::copy(F.vals.begin(), F.vals.end(), vals);
    return GBCHOL_OK;
}

int gbchol_factor_free(gbchol_factor_handle f) {
    delete f;
    return GBCHOL_OK;
}

int gbchol_destroy(gbchol_handle h) {
    if (!h) return GBCHOL_OK;
    {
        DeviceGuard g(h->device);
        if (h->last_stream) cudaStreamSynchronize(h->last_stream);
        delete h;
    }
    return GBCHOL_OK;
}

int gbchol_replan(gbchol_handle h, int32_t min_top_width, int32_t part_keep, int32_t part_group) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (min_top_width < 1 || part_keep < 0 || part_group < 0)
        return fail(GBCHOL_EINVAL, "min_top_width must be >= 1, part_keep and part_group >= 0.");
    DeviceGuard g(h->device);
    CUDA_TRY(cudaDeviceSynchronize());  // no solve may still use the old plan's buffers
    h->plan_opt.min_top_width = min_top_width;
    h->plan_opt.part_keep = part_keep;
    h->plan_opt.part_group = part_group;
    ++h->plan_gen;
    if (h->n == 0) return GBCHOL_OK;
    if (int rc = setup_plan(h)) return rc;
    CUDA_TRY(cudaDeviceSynchronize());
    return GBCHOL_OK;
}

int gbchol_autotune(gbchol_handle h, int32_t precision, int32_t nrhs, const int32_t* candidates, int32_t count,
                    int32_t reps, int32_t* chosen) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (int rc = check_rhs(nrhs)) return rc;
    if (precision != 0 && precision != 1) return fail(GBCHOL_EINVAL, "precision must be 0 or 1.");
    const bool f32 = precision == 0;
    if (!(h->store & (f32 ? GBCHOL_STORE_F32 : GBCHOL_STORE_F64)))
        return fail(GBCHOL_ESTATE, f32 ? "This solver keeps no FP32 factor." : "This solver keeps no FP64 factor.");
    if (!candidates || count < 1 || count > 64) return fail(GBCHOL_EINVAL, "1 to 64 candidate widths are needed.");
    if (reps < 1 || reps > 100) return fail(GBCHOL_EINVAL, "reps must be in [1, 100].");
    for (int32_t c = 0; c < count; ++c)
        if (candidates[c] < 1) return fail(GBCHOL_EINVAL, "Candidate widths must be >= 1.");
    if (h->n == 0) {
        if (chosen) *chosen = h->plan_opt.min_top_width;
        return GBCHOL_OK;
    }
    DeviceGuard g(h->device);
    const size_t bytes = (size_t)h->n * nrhs * (f32 ? sizeof(float) : sizeof(double));
    DevBuf<unsigned char> b, x;
    CUDA_TRY(b.alloc(bytes));
    CUDA_TRY(x.alloc(bytes));
    CUDA_TRY(cudaMemset(b.p, 0, bytes));
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int rc = GBCHOL_OK;
    int32_t best = -1;
    float best_ms = 0.f;
    const PlanOptions keep = h->plan_opt;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        rc = fail(GBCHOL_ECUDA, "cudaEventCreate failed.");
    const SweepIO io = f32 ? SweepIO::F32 : SweepIO::F64;
    for (int32_t c = 0; c < count && rc == GBCHOL_OK; ++c) {
        if ((rc = gbchol_replan(h, candidates[c], keep.part_keep, keep.part_group))) break;
        if ((rc = ensure_tmp(h, work_bytes(h, nrhs, f32)))) break;
        for (int w = 0; w < 2 && rc == GBCHOL_OK; ++w) rc = run_sweeps(h, f32, io, nrhs, b.p, x.p, nullptr, s);
        if (rc) break;
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps && rc == GBCHOL_OK; ++r) rc = run_sweeps(h, f32, io, nrhs, b.p, x.p, nullptr, s);
        cudaEventRecord(e1, s);
        if (rc) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = fail(GBCHOL_ECUDA, "autotune: timing failed.");
            break;
        }
        h->last_stream = s;
        if ((rc = gbchol_check(h))) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (best < 0 || ms < best_ms) {
            best = candidates[c];
            best_ms = ms;
        }
    }
    h->last_stream = nullptr;
    if (rc == GBCHOL_OK && best != h->plan_opt.min_top_width)
        rc = gbchol_replan(h, best, keep.part_keep, keep.part_group);
    if (rc == GBCHOL_OK && chosen) *chosen = best;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

int gbchol_autotune_sweeps(gbchol_handle h, int32_t precision, int32_t nrhs, int32_t reps, int32_t* choice) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (int rc = check_rhs(nrhs)) return rc;
    if (precision != 0 && precision != 1) return fail(GBCHOL_EINVAL, "precision must be 0 or 1.");
    const bool f32 = precision == 0;
    if (!(h->store & (f32 ? GBCHOL_STORE_F32 : GBCHOL_STORE_F64)))
        return fail(GBCHOL_ESTATE, f32 ? "This solver keeps no FP32 factor." : "This solver keeps no FP64 factor.");
    if (reps < 1 || reps > 100) return fail(GBCHOL_EINVAL, "reps must be in [1, 100].");
    if (h->n == 0) {
        if (choice) *choice = 0;
        return GBCHOL_OK;
    }
    DeviceGuard g(h->device);
    // the tensor-core variant needs lower groups of <= 32 columns: rebuild
    // the bulk tiles for it first (the other variants run on them too)
    const bool bulk_ok = f32 && h->snb_ready && snb_supported(nrhs);
    if (bulk_ok && h->snb_group_cols > 32) {
        h->snb_tc_groups = true;
        CUDA_TRY(cudaDeviceSynchronize());
        if (int rc = setup_snb(h)) return rc;
    }
    const size_t bytes = (size_t)h->n * nrhs * (f32 ? sizeof(float) : sizeof(double));
    DevBuf<unsigned char> b, x;
    CUDA_TRY(b.alloc(bytes));
    CUDA_TRY(x.alloc(bytes));
    CUDA_TRY(cudaMemset(b.p, 0, bytes));
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int rc = GBCHOL_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        rc = fail(GBCHOL_ECUDA, "cudaEventCreate failed.");
    const SweepIO io = f32 ? SweepIO::F32 : SweepIO::F64;
    gbchol_solver::SweepTune best;
    float best_ms = 0.f;
    const int sn_max = bulk_ok ? 4 : 0;
    for (int sn = 0; sn <= sn_max && rc == GBCHOL_OK; ++sn) {
        if (sn >= 3 && snb_kind_slices(sn, nrhs) == 1) continue;  // no such column split
        for (int split = 0; split <= (nrhs <= 8 ? 1 : 0) && rc == GBCHOL_OK; ++split)
            for (int chunk : {1, 2, 4}) {
                if (rc != GBCHOL_OK) break;
                gbchol_solver::SweepTune t;
                t.valid = 1;
                t.sn = (int8_t)sn;
                t.rhs_split = (int8_t)split;
                t.chunk = (int8_t)chunk;
                h->tuned[nrhs] = t;
                if ((rc = ensure_tmp(h, work_bytes(h, nrhs, f32)))) break;
                for (int w = 0; w < 2 && rc == GBCHOL_OK; ++w) rc = run_sweeps(h, f32, io, nrhs, b.p, x.p, nullptr, s);
                if (rc) break;
                cudaEventRecord(e0, s);
                for (int r = 0; r < reps && rc == GBCHOL_OK; ++r)
                    rc = run_sweeps(h, f32, io, nrhs, b.p, x.p, nullptr, s);
                cudaEventRecord(e1, s);
                if (rc) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    rc = fail(GBCHOL_ECUDA, "autotune: timing failed.");
                    break;
                }
                h->last_stream = s;
                if ((rc = gbchol_check(h))) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (!best.valid || ms < best_ms) {
                    best = t;
                    best_ms = ms;
                }
            }
    }
    h->last_stream = nullptr;
    h->tuned[nrhs] = rc == GBCHOL_OK ? best : gbchol_solver::SweepTune{};
    if (rc == GBCHOL_OK && choice) *choice = best.sn | (best.rhs_split << 4) | (best.chunk << 8);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

int gbchol_reserve(gbchol_handle h, int32_t nrhs) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (int rc = check_rhs(nrhs)) return rc;
    DeviceGuard g(h->device);
    return ensure_tmp(h, std::max(work_bytes(h, nrhs, true), work_bytes(h, nrhs, false)));
}

int gbchol_solve(gbchol_handle h, int32_t precision, int32_t nrhs, const void* b, void* x,
                 void* stream) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (int rc = check_rhs(nrhs)) return rc;
    const bool f32 = precision == 0;
    if (precision != 0 && precision != 1) return fail(GBCHOL_EINVAL, "precision must be 0 or 1.");
    if (f32 && !(h->store & GBCHOL_STORE_F32))
        return fail(GBCHOL_ESTATE, "This solver keeps no FP32 factor.");
    if (!f32 && !(h->store & GBCHOL_STORE_F64))
        return fail(GBCHOL_ESTATE, "This solver keeps no FP64 factor.");
    if (h->n == 0) return GBCHOL_OK;
    if (!b || !x) return fail(GBCHOL_EINVAL, "Null b or x.");
    DeviceGuard g(h->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (int rc = ensure_tmp(h, work_bytes(h, nrhs, f32))) return rc;
    const SweepIO io = f32 ? SweepIO::F32 : SweepIO::F64;
    if (int rc = run_sweeps(h, f32, io, nrhs, b, x, nullptr, s)) return rc;
    h->last_stream = s;
    return GBCHOL_OK;
}

int gbchol_solve_refined(gbchol_handle h, int32_t nrhs, const double* b, double* x, double tol,
                         int32_t max_iter, void* stream, gbchol_refine_stats* stats) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (int rc = check_rhs(nrhs)) return rc;
    if ((h->store & (GBCHOL_STORE_F32 | GBCHOL_STORE_A64)) != (GBCHOL_STORE_F32 | GBCHOL_STORE_A64))
        return fail(GBCHOL_ESTATE, "Refinement needs the FP32 factor and the FP64 matrix.");
    if (max_iter < 0 || max_iter > 100) return fail(GBCHOL_EINVAL, "max_iter must be in [0, 100].");
    if (!(tol >= 0.0)) return fail(GBCHOL_EINVAL, "tol must be non-negative.");
    if (h->n == 0) {
        if (stats) *stats = gbchol_refine_stats{0, 1, 0.0};
        return GBCHOL_OK;
    }
    if (!b || !x) return fail(GBCHOL_EINVAL, "Null b or x.");
    if ((const void*)b == (const void*)x) return fail(GBCHOL_EINVAL, "b and x must not alias for refinement.");
    DeviceGuard g(h->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int n = h->n;
    if (int rc = ensure_tmp(h, work_bytes(h, nrhs, true))) return rc;
    if (h->r64.count < (size_t)n * nrhs) CUDA_TRY(h->r64.alloc((size_t)n * nrhs));
    const int grid = residual_grid(n);
    if (h->partials.count < (size_t)grid * 2 * nrhs) CUDA_TRY(h->partials.alloc((size_t)grid * 2 * GBCHOL_MAX_RHS));
    if (!h->rstate.p) CUDA_TRY(h->rstate.alloc(1));
    CUDA_TRY(cudaMemsetAsync(h->rstate.p, 0, sizeof(RefineState), s));
    // x0 = A32^{-1} b
    if (int rc = run_sweeps(h, true, SweepIO::F32_MIXED, nrhs, b, x, nullptr, s)) return rc;
    ResidualArgs ra;
    ra.n = n;
    ra.nrhs = nrhs;
    ra.rowptr = h->a_rowptr.p;
    ra.cols = h->a_cols.p;
    ra.vals = h->a_vals.p;
    ra.b = b;
    ra.x = x;
    ra.r = h->r64.p;
    ra.partials = h->partials.p;
    ra.state = h->rstate.p;
    ra.tol = tol;
    const int* conv = &h->rstate.p->converged;
    // Each step: r = b - A x (and the stop decision), d = A32^{-1} r, x += d.
    // Once converged, every later kernel returns at once.
    for (int it = 0; it <= max_iter; ++it) {
        ra.iter = it;
        ra.first = it == 0;
        CUDA_TRY(launch_residual(ra, grid, s));
        if (it == max_iter) break;
        if (int rc = run_sweeps(h, true, SweepIO::F32_REFINE, nrhs, h->r64.p, x, conv, s)) return rc;
    }
    h->last_stream = s;
    if (stats) {
        RefineState hs;
        CUDA_TRY(cudaMemcpyAsync(&hs, h->rstate.p, sizeof(RefineState), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        // A non-finite or too-large residual never counts as converged.
        const int conv_ok = hs.converged && hs.max_rel <= tol;
        stats->iterations = conv_ok ? hs.iterations : max_iter;
        stats->converged = conv_ok;
        stats->max_rel_residual = hs.max_rel;
    }
    return GBCHOL_OK;
}

int gbchol_grad_values(int32_t precision, int64_t nnz, int32_t nrhs, const int32_t* rows,
                       const int32_t* cols, const void* grad_b, const void* x, void* grad_vals,
                       int32_t out_precision, int32_t symmetric, void* stream) {
    if (nnz < 0 || nrhs < 1 || nrhs > GBCHOL_MAX_RHS) return fail(GBCHOL_EINVAL, "Invalid sizes.");
    if ((precision != 0 && precision != 1) || (out_precision != 0 && out_precision != 1))
        return fail(GBCHOL_EINVAL, "precision must be 0 or 1.");
    if (nnz > 0 && (!rows || !cols || !grad_b || !x || !grad_vals))
        return fail(GBCHOL_EINVAL, "Null array.");
    GradArgs a;
    a.nnz = nnz;
    a.nrhs = nrhs;
    a.symmetric = symmetric ? 1 : 0;
    a.rows = rows;
    a.cols = cols;
    a.grad_b = grad_b;
    a.x = x;
    a.grad_vals = grad_vals;
    CUDA_TRY(launch_grad_values(a, precision == 0, out_precision == 0, static_cast<cudaStream_t>(stream)));
    return GBCHOL_OK;
}

int gbchol_selftest_wait(int32_t wait_us, int32_t* status_out) {
    if (wait_us < 1 || wait_us > 2000000 || !status_out) return fail(GBCHOL_EINVAL, "Invalid arguments.");
    DevBuf<int32_t> buf;
    CUDA_TRY(buf.alloc(2));
    CUDA_TRY(cudaMemset(buf.p, 0, 2 * sizeof(int32_t)));
    CUDA_TRY(launch_selftest_wait(buf.p, buf.p + 1, (unsigned long long)wait_us * 1000ull, nullptr));
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemcpy(status_out, buf.p + 1, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return GBCHOL_OK;
}

int gbchol_get_info(gbchol_handle h, gbchol_info* out) {
    if (!h || !out) return fail(GBCHOL_EINVAL, "Null argument.");
    gbchol_info i{};
    i.n = h->n;
    i.device = h->device;
    i.nnz_a = h->nnz_a;
    i.nnz_l = h->F.nnz();
    i.levels_lower = h->n ? h->lower.max_lvl + 1 : 0;
    i.levels_upper = h->n ? h->upper.max_lvl + 1 : 0;
    i.n_supernodes = h->F.sn_start.empty() ? 0 : (int32_t)h->F.sn_start.size() - 1;
    int32_t mx = 0;
    for (size_t s = 0; s + 1 < h->F.sn_start.size(); ++s)
        mx = std::max(mx, h->F.sn_start[s + 1] - h->F.sn_start[s]);
    i.max_supernode = mx;
    i.factor_flops = h->F.flops;
    i.factor_seconds = h->t_factor;
    i.analysis_seconds = h->t_analysis;
    i.store = h->store;
    i.top_rows = h->plan.n_top_rows;
    i.top_units = (int32_t)h->plan.units.size();
    i.top_blocks = (int64_t)h->plan.contribs.size();
    i.launches_per_solve = sweep_launches(h);
    *out = i;
    return GBCHOL_OK;
}

int gbchol_get_levels(gbchol_handle h, int32_t lower, int32_t* row_levels, int32_t* order,
                      int32_t* max_lvl) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    const Triangle& t = lower ? h->lower : h->upper;
    if (row_levels) std::copy(t.row_levels.begin(), t.row_levels.end(), row_levels);
    if (order) std::copy(t.order_h.begin(), t.order_h.end(), order);
    if (max_lvl) *max_lvl = t.max_lvl;
    return GBCHOL_OK;
}

int gbchol_get_factor(gbchol_handle h, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                      double* vals) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    const Factor& F = h->F;
    if (perm) std::copy(F.perm.begin(), F.perm.end(), perm);
    if (colptr) std::copy(F.colptr.begin(), F.colptr.end(), colptr);
    if (rowidx) std::copy(F.rowidx.begin(), F.rowidx.end(), rowidx);
    if (vals) std::copy(F.vals.begin(), F.vals.end(), vals);
    return GBCHOL_OK;
}

int gbchol_check(gbchol_handle h) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    DeviceGuard g(h->device);
    CUDA_TRY(cudaStreamSynchronize(h->last_stream));
    int32_t st = 0;
    CUDA_TRY(cudaMemcpy(&st, h->status.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (st != 0) {
        CUDA_TRY(cudaMemset(h->status.p, 0, sizeof(int32_t)));
        CUDA_TRY(cudaDeviceSynchronize());
        return fail(GBCHOL_ETIMEOUT, "A device-side wait expired during a solve; results are invalid.");
    }
    return GBCHOL_OK;
}

}  // extern "C"
