// Solve plan: splits the factor into a leaf region (row-wise sweeps) and a
// top region (supernodal sweeps on dense panels), and lists the work units
// and dense contribution blocks of the supernodal sweeps.
//
// Top region: every fundamental supernode at least `min_top_width` columns
// wide, plus all its ancestors (so the region is closed upwards: a top
// supernode's off-diagonal rows are top rows). Its columns are stored as
// dense column-major panels of (columns + off-diagonal rows) x columns and
// cut into chunks of kChunk columns, one work unit each.
//
// Lower sweep (L y = b):   leaf rows solve row by row; each top row first
//   receives b minus its leaf-column terms (row kernel, "partial" task), then
//   each top unit pulls the dense blocks L[unit rows, source chunk] of every
//   source chunk whose rows hit it and solves its diagonal block.
// Upper sweep (L^T x = y): each top unit subtracts L[below rows, unit]^T x
//   over the rows below its diagonal block (all top rows, solved earlier),
//   then solves its diagonal block; the leaf rows follow row by row.
#include "plan.h"

#include <algorithm>
#include <climits>
#include <stdexcept>

namespace gbchol {

void build_plan(const Factor& F, const std::vector<int32_t>& lower_order,
                const std::vector<int32_t>& upper_order, const PlanOptions& opt, SolvePlan& P) {
    const int32_t n = F.n;
    P = SolvePlan();
    P.n = n;
    P.sn_start = F.sn_start;
    const int32_t nsn = (int32_t)P.sn_start.size() - 1;
    std::vector<int32_t> sn_of((size_t)n);
    for (int32_t s = 0; s < nsn; ++s)
        for (int32_t j = P.sn_start[s]; j < P.sn_start[s + 1]; ++j) sn_of[j] = s;
    std::vector<int32_t> sn_parent((size_t)nsn, -1);
    for (int32_t s = 0; s < nsn; ++s) {
        int32_t last = P.sn_start[s + 1] - 1;
        int32_t p = F.colptr[last + 1] - F.colptr[last] > 1 ? F.rowidx[F.colptr[last] + 1] : -1;
        sn_parent[s] = p >= 0 ? sn_of[p] : -1;
    }
    // ---- top region: wide supernodes and their ancestors -------------------
    P.sn_top.assign((size_t)nsn, 0);
    for (int32_t s = 0; s < nsn; ++s)
        if (P.sn_start[s + 1] - P.sn_start[s] >= opt.min_top_width) P.sn_top[s] = 1;
    for (int32_t s = 0; s < nsn; ++s)  // parents have larger indices (postorder)
        if (P.sn_top[s] && sn_parent[s] >= 0) P.sn_top[sn_parent[s]] = 1;
    P.row_top.assign((size_t)n, 0);
    for (int32_t j = 0; j < n; ++j) P.row_top[j] = P.sn_top[sn_of[j]];
    for (int32_t j = 0; j < n; ++j) P.n_top_rows += P.row_top[j];

    // ---- panels, row lists and units ---------------------------------------
    std::vector<int32_t> unit_of_col((size_t)n, -1);
    std::vector<int32_t> first_unit((size_t)nsn, -1), unit_count((size_t)nsn, 0);
    std::vector<int64_t> rows_off((size_t)nsn, -1), panel_off((size_t)nsn, -1);
    // offsets first, then the row lists and panels, one supernode per task
    std::vector<int32_t> tops;
    {
        int64_t nrows = 0, npan = 0;
        for (int32_t s = 0; s < nsn; ++s) {
            if (!P.sn_top[s]) continue;
            const int32_t f = P.sn_start[s], w = P.sn_start[s + 1] - f;
            const int64_t ld = F.colptr[f + 1] - F.colptr[f];
            rows_off[s] = nrows;
            panel_off[s] = npan;
            nrows += ld;
            npan += ld * w;
            tops.push_back(s);
        }
        P.sn_rows.resize((size_t)nrows);
        P.panels.resize((size_t)npan);  // zero: a panel column holds no rows above its diagonal
    }
    int mismatch = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t q = 0; q < tops.size(); ++q) {
        const int32_t s = tops[q];
        const int32_t f = P.sn_start[s], w = P.sn_start[s + 1] - f;
        const int32_t ld = F.colptr[f + 1] - F.colptr[f];
        std::copy(F.rowidx.begin() + F.colptr[f], F.rowidx.begin() + F.colptr[f + 1],
                  P.sn_rows.begin() + rows_off[s]);
        const int32_t* rows = P.sn_rows.data() + rows_off[s];
        bool ok = true;
        for (int32_t j = 0; j < w && ok; ++j) {
            const int32_t c = f + j;
            const int32_t cnt = F.colptr[c + 1] - F.colptr[c];
            if (cnt != ld - j) {
                ok = false;
                break;
            }
            double* dst = P.panels.data() + panel_off[s] + (int64_t)j * ld + j;
            for (int32_t t = 0; t < cnt; ++t) {
                if (F.rowidx[F.colptr[c] + t] != rows[j + t]) ok = false;
                dst[t] = F.vals[F.colptr[c] + t];
            }
        }
        if (!ok) {
#pragma omp atomic write
            mismatch = 1;
        }
    }
    if (mismatch) throw std::runtime_error("supernode structure mismatch");
    for (const int32_t s : tops) {
        const int32_t f = P.sn_start[s], l1 = P.sn_start[s + 1];
        const int32_t ld = F.colptr[f + 1] - F.colptr[f];
        first_unit[s] = (int32_t)P.units.size();
        for (int32_t c0 = f; c0 < l1; c0 += kChunk) {
            SnUnit u{};
            u.c0 = c0;
            u.w = std::min(kChunk, l1 - c0);
            u.ld = ld;
            u.pos0 = c0 - f;
            u.panel_col_off = panel_off[s] + (int64_t)(c0 - f) * ld;
            u.rows_off = rows_off[s];
            for (int32_t c = c0; c < c0 + u.w; ++c) unit_of_col[c] = (int32_t)P.units.size();
            P.units.push_back(u);
            unit_count[s]++;
        }
    }
    const int32_t nunits = (int32_t)P.units.size();
    for (int32_t s = 0; s < nsn; ++s) {
        if (!P.sn_top[s]) continue;
        for (int32_t k = 0; k < unit_count[s]; ++k)
            P.units[first_unit[s] + k].sn_w = P.sn_start[s + 1] - P.sn_start[s];
    }
    // lower-sweep contributions, gathered per destination unit in source order
    std::vector<std::vector<SnContrib>> per_unit((size_t)nunits);
    for (int32_t s = 0; s < nsn; ++s) {
        if (!P.sn_top[s]) continue;
        const int32_t f = P.sn_start[s], w = P.sn_start[s + 1] - f;
        const int32_t ld = P.units[first_unit[s]].ld;
        const int32_t* rows = P.sn_rows.data() + rows_off[s];
        for (int32_t k = 0; k < unit_count[s]; ++k) {
            const int32_t vu = first_unit[s] + k;
            const SnUnit& V = P.units[vu];
            // rows below V's diagonal block, grouped by destination unit
            int32_t p = V.pos0 + V.w;
            while (p < ld) {
                const int32_t dst = unit_of_col[rows[p]];
                if (dst < 0) throw std::runtime_error("top region not closed upwards");
                int32_t q = p + 1;
                while (q < ld && unit_of_col[rows[q]] == dst) ++q;
                SnContrib c{};
                c.panel_off = V.panel_col_off + p;
                c.rows_off = rows_off[s] + p;
                c.ld = ld;
                c.xcol = V.c0;
                c.nr = q - p;
                c.w = V.w;
                c.src_unit = vu;
                c.rowmask = 0;
                for (int32_t t = p; t < q; ++t) c.rowmask |= 1u << (rows[t] - P.units[dst].c0);
                per_unit[dst].push_back(c);
                p = q;
            }
        }
        (void)w;
    }
    // The list is in source order: descendants first, the earlier chunks of
    // the unit's own supernode last (the previous chunk, on the dependency
    // chain, is the very last). A long list keeps its last part_keep blocks
    // and cuts the rest into consecutive groups of about part_group blocks,
    // each summed by a partial-sum item.
    for (int32_t u = 0; u < nunits; ++u) {
        SnUnit& U = P.units[u];
        const int32_t b0 = (int32_t)P.contribs.size();
        P.contribs.insert(P.contribs.end(), per_unit[u].begin(), per_unit[u].end());
        const int32_t nb = (int32_t)per_unit[u].size();
        U.contrib_begin = b0;
        U.contrib_end = b0 + nb;
        U.part_begin = U.part_end = (int32_t)P.parts.size();
        const int32_t keep = std::max(opt.part_keep, 1);  // the chain block stays with the unit
        if (opt.part_group > 0 && nb > keep + opt.part_group) {
            const int32_t m = nb - keep;
            const int32_t ng = (m + opt.part_group - 1) / opt.part_group;
            for (int32_t g = 0; g < ng; ++g) {
                SnPartial q{};
                q.unit = u;
                q.contrib_begin = b0 + (int32_t)((int64_t)m * g / ng);
                q.contrib_end = b0 + (int32_t)((int64_t)m * (g + 1) / ng);
                P.parts.push_back(q);
            }
            U.contrib_begin = b0 + m;
            U.part_end = (int32_t)P.parts.size();
        }
    }

    // Per unit, three 32x32 column-major FP64 matrices (FP64 products, cast
    // once for the FP32 factor):
    //   Dinv  = D^{-1}, D the unit's diagonal block (forward substitution on
    //           the identity), so that its diagonal solve is one product;
    //   M_lo  = D^{-1} L[unit, previous chunk] (a unit that is not its
    //           supernode's first chunk) and
    //   M_up  = D^{-T} L[next chunk, unit]^T (not the last chunk): the block
    //           on the sweep's dependency chain folded into the diagonal
    //           solve, x = D^{-1} t' - M x_chain, so that after the chain
    //           wait a unit does one 32x32 product and no reduction.
    // The bulk sweeps fold one more block of the unit's own supernode (FP64
    // products like the above):
    //   M2_lo = D^{-1} L[unit, chunk two before] and
    //   M2_up = D^{-T} L[chunk two after, unit]^T.
    constexpr size_t kMat = (size_t)kChunk * kChunk;
    P.dinv.assign((size_t)nunits * 3 * kMat, 0.0);
    P.fold2.assign((size_t)nunits * 2 * kMat, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int32_t u = 0; u < nunits; ++u) {
        const SnUnit& U = P.units[u];
        const double* D = P.panels.data() + U.panel_col_off + U.pos0;  // D(i,j) = D[i + j*ld]
        double* X = P.dinv.data() + (size_t)u * 3 * kMat;             // X(i,j) = X[i + j*32]
        for (int32_t j = 0; j < U.w; ++j) {
            for (int32_t i = j; i < U.w; ++i) {
                double v = (i == j) ? 1.0 : 0.0;
                for (int32_t k = j; k < i; ++k) v -= D[i + (size_t)k * U.ld] * X[k + j * kChunk];
                X[i + j * kChunk] = v / D[i + (size_t)i * U.ld];
            }
        }
        if (U.pos0 > 0) {  // previous chunk: 32 columns, panel columns just before the unit's
            const double* Lp = P.panels.data() + U.panel_col_off - (int64_t)kChunk * U.ld + U.pos0;
            double* Mlo = X + kMat;
            for (int32_t j = 0; j < kChunk; ++j)
                for (int32_t i = 0; i < U.w; ++i) {
                    double v = 0.0;
                    for (int32_t m = 0; m <= i; ++m) v += X[i + m * kChunk] * Lp[m + (size_t)j * U.ld];
                    Mlo[i + j * kChunk] = v;
                }
        }
        const int32_t wn = std::min(kChunk, U.sn_w - (U.pos0 + U.w));  // next chunk's width
        if (wn > 0) {
            const double* Ln = P.panels.data() + U.panel_col_off + U.pos0 + U.w;  // Ln(j, m) = Ln[j + m*ld]
            double* Mup = X + 2 * kMat;
            for (int32_t j = 0; j < wn; ++j)
                for (int32_t i = 0; i < U.w; ++i) {
                    double v = 0.0;
                    for (int32_t m = i; m < U.w; ++m) v += X[m + i * kChunk] * Ln[j + (size_t)m * U.ld];
                    Mup[i + j * kChunk] = v;
                }
        }
        double* F2 = P.fold2.data() + (size_t)u * 2 * kMat;
        if (snb_fold2_lo(U)) {  // chunk two before: 32 columns, 64 to 33 panel columns before the unit's
            const double* Lp = P.panels.data() + U.panel_col_off - (int64_t)2 * kChunk * U.ld + U.pos0;
            for (int32_t j = 0; j < kChunk; ++j)
                for (int32_t i = 0; i < U.w; ++i) {
                    double v = 0.0;
                    for (int32_t m = 0; m <= i; ++m) v += X[i + m * kChunk] * Lp[m + (size_t)j * U.ld];
                    F2[i + j * kChunk] = v;
                }
        }
        if (snb_fold2_up(U)) {  // chunk two after (the unit is a full 32-column chunk)
            const int32_t p2 = U.pos0 + U.w + kChunk, wn2 = std::min(kChunk, U.sn_w - p2);
            const double* Ln = P.panels.data() + U.panel_col_off + p2;
            for (int32_t j = 0; j < wn2; ++j)
                for (int32_t i = 0; i < U.w; ++i) {
                    double v = 0.0;
                    for (int32_t m = i; m < U.w; ++m) v += X[m + i * kChunk] * Ln[j + (size_t)m * U.ld];
                    F2[kMat + i + j * kChunk] = v;
                }
        }
    }
    // Ticket order of the supernodal items. Each item's start is estimated
    // with a small cost model (per item: flag latency kLat, fixed cost kBase,
    // kBlk per round of 8 blocks, one block per warp) from the estimated
    // finish of the items it waits on: an item should start when its work
    // before its last wait is just done as that wait ends. The key is that
    // start, and at least one more than the key of every item it waits on, so
    // sorting by key is a topological order (a CTA only ever waits on items
    // with smaller tickets: the persistent kernels cannot deadlock).
    // Ordering by plain dependency level instead would hand tickets to items
    // whose inputs come from long, slow chains, idling CTAs that items on the
    // critical path need.
    {
        constexpr int64_t kLat = 1000, kBase = 2000, kBlk = 1500;  // ns
        const int32_t nparts = (int32_t)P.parts.size();
        struct Est {
            int64_t first = INT64_MAX, last = 0, key_dep = -1;
            void dep(int64_t fin, int64_t key) {
                first = std::min(first, fin + kLat);
                last = std::max(last, fin + kLat);
                key_dep = std::max(key_dep, key);
            }
            // returns the finish estimate, sets the key
            int64_t done(int64_t nblocks, int64_t& key) const {
                const int64_t rounds = std::max<int64_t>(1, (nblocks + 7) / 8);
                const int64_t f = first == INT64_MAX ? 0 : first;
                key = std::max({f, last - (rounds - 1) * kBlk, key_dep + 1});
                return std::max(std::max(key, last) + kBase + kBlk, key + kBase + kBlk * rounds);
            }
        };
        std::vector<int64_t> fin_u((size_t)nunits, 0), fin_p((size_t)nparts, 0);
        std::vector<int64_t> key_u((size_t)nunits, 0), key_p((size_t)nparts, 0), key_up((size_t)nunits, 0);
        for (int32_t u = 0; u < nunits; ++u) {  // sources precede their destinations
            const SnUnit& U = P.units[u];
            Est eu;
            for (int32_t q = U.part_begin; q < U.part_end; ++q) {
                Est eq;
                for (int32_t e = P.parts[q].contrib_begin; e < P.parts[q].contrib_end; ++e)
                    eq.dep(fin_u[P.contribs[e].src_unit], key_u[P.contribs[e].src_unit]);
                fin_p[q] = eq.done(P.parts[q].contrib_end - P.parts[q].contrib_begin, key_p[q]);
                eu.dep(fin_p[q], key_p[q]);
            }
            for (int32_t e = U.contrib_begin; e < U.contrib_end; ++e)
                eu.dep(fin_u[P.contribs[e].src_unit], key_u[P.contribs[e].src_unit]);
            fin_u[u] = eu.done((U.contrib_end - U.contrib_begin) + (U.part_end - U.part_begin), key_u[u]);
        }
        // upper sweep: each 32-row block of the supernode's off-diagonal rows
        // waits for the unit holding its first (lowest) row: those rows lie on
        // the etree path above the supernode, and in the upper sweep a higher
        // row is always solved before a lower one
        std::vector<int64_t> fin_up((size_t)nunits, 0);
        for (int32_t u = nunits - 1; u >= 0; --u) {
            const SnUnit& U = P.units[u];
            const int32_t* rows = P.sn_rows.data() + U.rows_off;
            Est eu;
            int64_t nb = 0;
            for (int32_t p = U.sn_w; p < U.ld; p += kChunk, ++nb) {
                const int32_t d = unit_of_col[rows[p]];
                eu.dep(fin_up[d], key_up[d]);
            }
            const int32_t nlater = (U.sn_w - (U.pos0 + U.w) + kChunk - 1) / kChunk;
            for (int32_t c = 0; c < nlater; ++c, ++nb) eu.dep(fin_up[u + 1 + c], key_up[u + 1 + c]);
            fin_up[u] = eu.done(nb, key_up[u]);
        }
        auto clamp32 = [](int64_t v) { return (int32_t)std::min<int64_t>(v, INT32_MAX); };
        P.unit_level_lo.resize((size_t)nunits);
        P.unit_level_up.resize((size_t)nunits);
        P.part_level_lo.resize((size_t)nparts);
        for (int32_t u = 0; u < nunits; ++u) {
            P.unit_level_lo[u] = clamp32(key_u[u]);
            P.unit_level_up[u] = clamp32(key_up[u]);
        }
        for (int32_t q = 0; q < nparts; ++q) P.part_level_lo[q] = clamp32(key_p[q]);
        const auto& lo = P.unit_level_lo;
        const auto& lp = P.part_level_lo;
        const auto& up = P.unit_level_up;
        P.unit_order_lo.resize((size_t)nunits + nparts);
        P.unit_order_up.resize((size_t)nunits);
        for (int32_t u = 0; u < nunits; ++u) P.unit_order_lo[u] = P.unit_order_up[u] = u;
        for (int32_t q = 0; q < nparts; ++q) P.unit_order_lo[nunits + q] = ~q;
        auto key_lo = [&](int32_t item) { return item >= 0 ? lo[item] : lp[~item]; };
        std::stable_sort(P.unit_order_lo.begin(), P.unit_order_lo.end(),
                         [&](int32_t a, int32_t b) { return key_lo(a) < key_lo(b); });
        std::stable_sort(P.unit_order_up.begin(), P.unit_order_up.end(),
                         [&](int32_t a, int32_t b) { return up[a] < up[b]; });
    }

    P.unit_of_row = unit_of_col;

    // ---- leaf region -------------------------------------------------------
    // CSR of the leaf columns of L (columns ascending, diagonal last): a leaf
    // row's whole row (an entry's row is an etree ancestor of its column, and
    // the ancestors of a top column are top) and the leaf-column terms of a
    // top row
    {
        std::vector<char> leaf_col((size_t)n);
        for (int32_t j = 0; j < n; ++j) leaf_col[j] = !P.row_top[j];
        transpose_columns(n, F.colptr, F.rowidx, F.vals.data(), leaf_col.data(), P.lo_rowptr, P.lo_cols,
                          P.lo_vals);
    }
    for (int32_t i = 0; i < n; ++i) P.max_row_len = std::max(P.max_row_len, P.lo_rowptr[i + 1] - P.lo_rowptr[i]);
    {
        // leaf rows by their level in L (= etree height: their dependencies
        // are all leaf rows); the partial task of a top row keyed one past
        // the highest leaf column it reads, so it runs as soon as its own
        // inputs are done (with opt.partial_last, after every leaf row)
        std::vector<int32_t> parent((size_t)n, -1), height((size_t)n, 0);
        for (int32_t j = 0; j < n; ++j)
            if (F.colptr[j + 1] - F.colptr[j] > 1) parent[j] = F.rowidx[F.colptr[j] + 1];
        for (int32_t j = 0; j < n; ++j)
            if (parent[j] >= 0) height[parent[j]] = std::max(height[parent[j]], height[j] + 1);
        int32_t maxh = 0;
        for (int32_t r : lower_order)
            if (!P.row_top[r]) {
                P.lo_tasks.push_back(r);
                P.lo_task_key.push_back(height[r]);
                maxh = std::max(maxh, height[r]);
            }
        for (int32_t i = 0; i < n; ++i)
            if (P.row_top[i]) {
                int32_t key = 0;
                for (int32_t k = P.lo_rowptr[i]; k < P.lo_rowptr[i + 1]; ++k)
                    key = std::max(key, height[P.lo_cols[k]] + 1);
                P.lo_tasks.push_back(~i);
                P.lo_task_key.push_back(opt.partial_last ? maxh + 1 : key);
            }
        if (!opt.partial_last) {  // one topological order: by key, leaf rows first within a key
            const size_t nt = P.lo_tasks.size();
            std::vector<int32_t> idx(nt);
            for (size_t t = 0; t < nt; ++t) idx[t] = (int32_t)t;
            std::stable_sort(idx.begin(), idx.end(),
                             [&](int32_t a, int32_t b) { return P.lo_task_key[a] < P.lo_task_key[b]; });
            std::vector<int32_t> tasks(nt), keys(nt);
            for (size_t t = 0; t < nt; ++t) {
                tasks[t] = P.lo_tasks[idx[t]];
                keys[t] = P.lo_task_key[idx[t]];
            }
            P.lo_tasks.swap(tasks);
            P.lo_task_key.swap(keys);
        }
        // the wavefront (the batch merges systems by lo_task_key, which stays
        // the level: any order within a level is topological)
        if (opt.leaf_group_rows > 0 && opt.leaf_skew > 0) {
            const size_t nt = P.lo_tasks.size();
            std::vector<int64_t> wkey(nt);
            for (size_t t = 0; t < nt; ++t) {
                const int32_t v = P.lo_tasks[t], row = v >= 0 ? v : ~v;
                wkey[t] = P.lo_task_key[t] + (int64_t)opt.leaf_skew * (row / opt.leaf_group_rows);
            }
            std::vector<int32_t> idx(nt);
            for (size_t t = 0; t < nt; ++t) idx[t] = (int32_t)t;
            std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return wkey[a] < wkey[b]; });
            std::vector<int32_t> tasks(nt), keys(nt);
            for (size_t t = 0; t < nt; ++t) {
                tasks[t] = P.lo_tasks[idx[t]];
                keys[t] = P.lo_task_key[idx[t]];
            }
            P.lo_tasks.swap(tasks);
            P.lo_task_key.swap(keys);
        }
    }
    // upper leaf sweep: order by depth below the top region (number of leaf
    // ancestors), so every leaf subtree advances one level per step whatever
    // the depth of the top node it hangs from
    {
        std::vector<int32_t> parent((size_t)n, -1), ldepth((size_t)n, 0);
        for (int32_t j = 0; j < n; ++j)
            if (F.colptr[j + 1] - F.colptr[j] > 1) parent[j] = F.rowidx[F.colptr[j] + 1];
        int32_t maxd = 0;
        for (int32_t j = n - 1; j >= 0; --j) {
            if (P.row_top[j]) continue;
            const int32_t p = parent[j];
            ldepth[j] = (p >= 0 && !P.row_top[p]) ? ldepth[p] + 1 : 0;
            maxd = std::max(maxd, ldepth[j]);
        }
        std::vector<int32_t> cnt((size_t)maxd + 2, 0);
        for (int32_t j = 0; j < n; ++j)
            if (!P.row_top[j]) cnt[(size_t)ldepth[j] + 1]++;
        for (int32_t d = 0; d <= maxd; ++d) cnt[(size_t)d + 1] += cnt[d];
        P.up_tasks.assign((size_t)cnt[(size_t)maxd + 1], 0);
        P.up_task_key.assign(P.up_tasks.size(), 0);
        for (int32_t j = 0; j < n; ++j)
            if (!P.row_top[j]) {
                P.up_task_key[cnt[ldepth[j]]] = ldepth[j];
                P.up_tasks[cnt[ldepth[j]]++] = j;
            }
        if (opt.leaf_group_rows > 0 && opt.leaf_skew > 0) {  // the wavefront, from the last group down
            const int64_t last = (n - 1) / opt.leaf_group_rows;
            const size_t nt = P.up_tasks.size();
            std::vector<int32_t> idx(nt);
            for (size_t t = 0; t < nt; ++t) idx[t] = (int32_t)t;
            auto wkey = [&](int32_t t) {
                return P.up_task_key[t] + (int64_t)opt.leaf_skew * (last - P.up_tasks[t] / opt.leaf_group_rows);
            };
            std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return wkey(a) < wkey(b); });
            std::vector<int32_t> tasks(nt), keys(nt);
            for (size_t t = 0; t < nt; ++t) {
                tasks[t] = P.up_tasks[idx[t]];
                keys[t] = P.up_task_key[idx[t]];
            }
            P.up_tasks.swap(tasks);
            P.up_task_key.swap(keys);
        }
    }
    (void)upper_order;
    // upper sweep: split every leaf column of L into its top-row entries and
    // its diagonal + leaf-row entries (top columns: both empty)
    P.upt_rowptr.assign((size_t)n + 1, 0);
    P.upl_rowptr.assign((size_t)n + 1, 0);
    for (int32_t j = 0; j < n; ++j) {
        int32_t nt = 0, nl = 0;
        if (!P.row_top[j]) {
            nl = 1;
            for (int32_t k = F.colptr[j] + 1; k < F.colptr[j + 1]; ++k)
                (P.row_top[F.rowidx[k]] ? nt : nl)++;
        }
        P.upt_rowptr[j + 1] = P.upt_rowptr[j] + nt;
        P.upl_rowptr[j + 1] = P.upl_rowptr[j] + nl;
        if (nt > 0) P.upt_tasks.push_back(~j);
    }
    P.upt_cols.resize((size_t)P.upt_rowptr[n]);
    P.upt_vals.resize((size_t)P.upt_rowptr[n]);
    P.upl_cols.resize((size_t)P.upl_rowptr[n]);
    P.upl_vals.resize((size_t)P.upl_rowptr[n]);
    for (int32_t j = 0; j < n; ++j) {
        if (P.row_top[j]) continue;
        int32_t dt = P.upt_rowptr[j], dl = P.upl_rowptr[j];
        for (int32_t k = F.colptr[j]; k < F.colptr[j + 1]; ++k) {
            const int32_t r = F.rowidx[k];
            if (k > F.colptr[j] && P.row_top[r]) {
                P.upt_cols[dt] = r;
                P.upt_vals[dt++] = F.vals[k];
            } else {
                P.upl_cols[dl] = r;
                P.upl_vals[dl++] = F.vals[k];
            }
        }
    }
}

void build_snb_upper(const SolvePlan& P, SnbUpperPlan& B) {
    const int32_t nunits = (int32_t)P.units.size();
    B.begin.assign((size_t)nunits + 1, 0);
    for (int32_t u = 0; u < nunits; ++u) {
        const SnUnit& U = P.units[u];
        const int32_t wj = U.pos0 + U.w;
        const int32_t nrb = (U.ld - U.sn_w + kChunk - 1) / kChunk;
        const int32_t nlater = (U.sn_w - wj + kChunk - 1) / kChunk;
        const int32_t chain = wj < U.sn_w ? 1 : 0;
        B.begin[u + 1] = B.begin[u] + nrb + nlater - chain;
    }
    const size_t nb = (size_t)B.begin[nunits];
    B.src.resize(nb);
    B.ld.resize(nb);
    B.nrw.resize(nb);
    B.dep.resize(nb);
    B.rows.assign(nb * kChunk, -1);
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t u = 0; u < nunits; ++u) {
        const SnUnit& U = P.units[u];
        const int32_t* srows = P.sn_rows.data() + U.rows_off;
        const int32_t wj = U.pos0 + U.w;
        const int32_t nrb = (U.ld - U.sn_w + kChunk - 1) / kChunk;
        const int32_t nlater = (U.sn_w - wj + kChunk - 1) / kChunk;
        for (int32_t b = 0; b < B.begin[u + 1] - B.begin[u]; ++b) {
            int32_t p0, nr, dep;
            if (b < nrb) {  // off-diagonal rows, highest block first
                p0 = U.sn_w + (nrb - 1 - b) * kChunk;
                nr = std::min(kChunk, U.ld - p0);
                dep = P.unit_of_row[srows[p0]];
            } else {        // later chunks of the supernode, last first (the one after next is last)
                const int32_t c = nlater - 1 - (b - nrb);
                p0 = wj + c * kChunk;
                nr = std::min(kChunk, U.sn_w - p0);
                dep = u + 1 + c;
            }
            const size_t t = (size_t)B.begin[u] + b;
            B.src[t] = U.panel_col_off + p0;
            B.ld[t] = U.ld;
            B.nrw[t] = nr | (U.w << 16);
            B.dep[t] = dep;
            for (int32_t i = 0; i < nr; ++i) B.rows[t * kChunk + i] = srows[p0 + i];
        }
    }
}

void build_snb_lower(const SolvePlan& P, const SnbUpperPlan& B, const SnbOptions& o, SnbLowerPlan& L) {
    const int32_t nunits = (int32_t)P.units.size();
    L.unit_info.assign((size_t)nunits * 4, 0);
    L.parts.clear();
    L.groups.clear();
    // estimated starts (as in build_plan): an item should start when its work
    // before its last wait is just done as that wait ends; the key is that
    // start and at least one more than the key of every item it waits on, so
    // sorting by key is a topological order
    struct Est {
        int64_t first = INT64_MAX, last = 0, key_dep = -1;
        void dep(int64_t fin, int64_t key, int64_t lat) {
            first = std::min(first, fin + lat);
            last = std::max(last, fin + lat);
            key_dep = std::max(key_dep, key);
        }
        int64_t done(int64_t nblocks, int64_t base, int64_t blk, int64_t& key) const {
            const int64_t f = first == INT64_MAX ? 0 : first;
            key = std::max({f, last - std::max<int64_t>(0, nblocks - 1) * blk, key_dep + 1});
            return std::max(std::max(key, last) + base + blk, key + base + blk * std::max<int64_t>(1, nblocks));
        }
    };
    std::vector<int64_t> fin_u((size_t)nunits, 0), key_u((size_t)nunits, 0);
    std::vector<int64_t> fin_p, key_p;
    for (int32_t u = 0; u < nunits; ++u) {  // sources precede their destinations
        const SnUnit& U = P.units[u];
        const int32_t chain = U.pos0 > 0 ? 1 : 0;
        // the chunk before the chain one (its block is the list's second to
        // last): with fold >= 2 a group of its own, the unit's last
        const int32_t f2 = (o.fold >= 2 && snb_fold2_lo(U)) ? 1 : 0;
        const int32_t end = U.contrib_end - chain - f2;
        const int32_t g0 = (int32_t)L.groups.size();
        const int32_t own_c0 = U.c0 - U.pos0;  // first column of the unit's supernode
        for (int32_t e = U.contrib_begin; e < end;) {
            const SnContrib& C = P.contribs[e];
            SnbGroup g{e, C.w, C.src_unit, C.xcol, C.rowmask};
            int32_t f = e + 1;
            const bool own = C.xcol >= own_c0 && C.xcol < U.c0;
            while (!own && f < end && P.contribs[f - 1].w == kChunk && P.contribs[f].rowmask == C.rowmask &&
                   P.contribs[f].src_unit == P.contribs[f - 1].src_unit + 1 &&
                   P.contribs[f].xcol == P.contribs[f - 1].xcol + kChunk && g.cols + P.contribs[f].w <= o.max_cols) {
                g.cols += P.contribs[f].w;
                g.src_unit = P.contribs[f].src_unit;
                ++f;
            }
            L.groups.push_back(g);
            e = f;
        }
        // the unit applies its groups in the order their sources are
        // estimated to finish (source order otherwise: the subtrees of a
        // separator run side by side, so their blocks would wait for each other)
        if (o.order_by_finish)
            std::stable_sort(L.groups.begin() + g0, L.groups.end(), [&](const SnbGroup& x, const SnbGroup& y) {
                return fin_u[x.src_unit] < fin_u[y.src_unit];
            });
        if (f2) {
            const SnContrib& C = P.contribs[end];
            L.groups.push_back(SnbGroup{end, C.w, C.src_unit, C.xcol, C.rowmask});
        }
        const int32_t ng_u = (int32_t)L.groups.size() - g0;
        int32_t first = g0;
        const int32_t pb = (int32_t)L.parts.size();
        const int32_t keep = std::max(o.keep, f2);  // the folded group stays with the unit
        if (o.group > 0 && ng_u > keep + o.group) {
            const int32_t split = g0 + ng_u - keep;  // the unit keeps groups [split, end)
            const int32_t np = (split - g0 + o.group - 1) / o.group;
            for (int32_t q = 0; q < np; ++q) {  // equal shares of the split-off groups
                SnPartial pp{};
                pp.unit = u;
                pp.contrib_begin = g0 + (int32_t)((int64_t)(split - g0) * q / np);
                pp.contrib_end = g0 + (int32_t)((int64_t)(split - g0) * (q + 1) / np);
                L.parts.push_back(pp);
            }
            first = split;
        }
        const int32_t pe = (int32_t)L.parts.size();
        L.unit_info[(size_t)u * 4] = first;
        L.unit_info[(size_t)u * 4 + 1] = (int32_t)L.groups.size();
        L.unit_info[(size_t)u * 4 + 2] = pb;
        L.unit_info[(size_t)u * 4 + 3] = pe;
        fin_p.resize((size_t)pe);
        key_p.resize((size_t)pe);
        Est eu;
        for (int32_t q = pb; q < pe; ++q) {
            Est eq;
            for (int32_t e = L.parts[q].contrib_begin; e < L.parts[q].contrib_end; ++e)
                eq.dep(fin_u[L.groups[e].src_unit], key_u[L.groups[e].src_unit], o.lat_ns);
            fin_p[q] = eq.done(L.parts[q].contrib_end - L.parts[q].contrib_begin, o.base_ns, o.blk_ns, key_p[q]);
            eu.dep(fin_p[q], key_p[q], o.lat_ns);
        }
        const int32_t ge = (int32_t)L.groups.size();
        for (int32_t e = first; e < ge; ++e) eu.dep(fin_u[L.groups[e].src_unit], key_u[L.groups[e].src_unit], o.lat_ns);
        if (chain) eu.dep(fin_u[u - 1], key_u[u - 1], o.lat_ns);  // the chain unit
        fin_u[u] = eu.done(ge - first + chain, o.base_ns, o.blk_ns, key_u[u]);
    }
    const int32_t nparts = (int32_t)L.parts.size();
    std::vector<int64_t> fin_up((size_t)nunits, 0), key_up((size_t)nunits, 0);
    for (int32_t u = nunits - 1; u >= 0; --u) {  // the upper sweep waits on later units
        const SnUnit& U = P.units[u];
        Est eu;
        for (int32_t t = B.begin[u]; t < B.begin[u + 1]; ++t) eu.dep(fin_up[B.dep[t]], key_up[B.dep[t]], o.lat_ns);
        if (U.pos0 + U.w < U.sn_w) eu.dep(fin_up[u + 1], key_up[u + 1], o.lat_ns);  // the chain unit
        fin_up[u] = eu.done(B.begin[u + 1] - B.begin[u], o.base_ns, o.blk_ns, key_up[u]);
    }
    L.order_lo.resize((size_t)nunits + nparts);
    for (int32_t u = 0; u < nunits; ++u) L.order_lo[u] = u;
    for (int32_t q = 0; q < nparts; ++q) L.order_lo[nunits + q] = ~q;
    auto key_lo = [&](int32_t item) { return item >= 0 ? key_u[item] : key_p[~item]; };
    std::stable_sort(L.order_lo.begin(), L.order_lo.end(),
                     [&](int32_t a, int32_t b) { return key_lo(a) < key_lo(b); });
    L.order_up.resize((size_t)nunits);
    for (int32_t u = 0; u < nunits; ++u) L.order_up[u] = u;
    std::stable_sort(L.order_up.begin(), L.order_up.end(),
                     [&](int32_t a, int32_t b) { return key_up[a] < key_up[b]; });
}

}  // namespace gbchol
