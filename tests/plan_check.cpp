// Host-side check of the solve plan (cholespy_gb300/csrc/host/plan.cpp): runs
// every sweep of a solve on the CPU in FP64, item by item in the order the
// GPU kernels hand out their tickets, and checks
//   - that every flag an item waits on belongs to an item with an earlier
//     ticket (the persistent kernels are deadlock-free only then) that wrote
//     the values the item reads,
//   - the partial-sum items of the lower sweep and the per-block waits of the
//     upper sweep,
//   - the solution against a plain column-oriented solve with the factor.
// Built and run by tests/test_plan.py. Exit status 0 = all cases pass.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "host.h"
#include "plan.h"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace gbchol;

namespace {

int errors = 0;
#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            if (errors < 10) std::printf("check failed: %s (line %d)\n", #c, __LINE__); \
            ++errors;                                                   \
        }                                                               \
    } while (0)

// Rows of L sorted by (level, row): the level orders the analysis produces.
std::vector<int32_t> level_order(int32_t n, const std::vector<int32_t>& rp, const std::vector<int32_t>& ci,
                                 bool lower) {
    std::vector<int32_t> lev((size_t)n, 0);
    int32_t mx = 0;
    for (int32_t t = 0; t < n; ++t) {
        const int32_t row = lower ? t : n - 1 - t;
        const int32_t lo = lower ? rp[row] : rp[row] + 1, hi = lower ? rp[row + 1] - 1 : rp[row + 1];
        int32_t l = 0;
        for (int32_t k = lo; k < hi; ++k) l = std::max(l, lev[ci[k]] + 1);
        lev[row] = l;
        mx = std::max(mx, l);
    }
    std::vector<int32_t> ord((size_t)n);
    for (int32_t i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return lev[a] < lev[b]; });
    return ord;
}

// One solve through the plan; returns the relative error against the plain solve.
double run_case(const Factor& F, const SolvePlan& P, int r) {
    const int32_t n = F.n;
    std::mt19937 g(7);
    std::normal_distribution<double> N;
    std::vector<double> b((size_t)n * r), tmp((size_t)n * r, 0.0), out((size_t)n * r, 0.0);
    for (auto& v : b) v = N(g);
    // reference: y = L^{-1} P b, x = P^T L^{-T} y
    std::vector<double> y((size_t)n * r);
    for (int32_t i = 0; i < n; ++i)
        for (int k = 0; k < r; ++k) y[(size_t)i * r + k] = b[(size_t)F.perm[i] * r + k];
    for (int32_t c = 0; c < n; ++c)
        for (int k = 0; k < r; ++k) {
            const double yc = y[(size_t)c * r + k] / F.vals[F.colptr[c]];
            y[(size_t)c * r + k] = yc;
            for (int32_t p = F.colptr[c] + 1; p < F.colptr[c + 1]; ++p) y[(size_t)F.rowidx[p] * r + k] -= F.vals[p] * yc;
        }
    std::vector<double> xr = y;
    for (int32_t c = n - 1; c >= 0; --c)
        for (int k = 0; k < r; ++k) {
            double v = xr[(size_t)c * r + k];
            for (int32_t p = F.colptr[c] + 1; p < F.colptr[c + 1]; ++p) v -= F.vals[p] * xr[(size_t)F.rowidx[p] * r + k];
            xr[(size_t)c * r + k] = v / F.vals[F.colptr[c]];
        }
    std::vector<double> ref((size_t)n * r);
    for (int32_t i = 0; i < n; ++i)
        for (int k = 0; k < r; ++k) ref[(size_t)F.perm[i] * r + k] = xr[(size_t)i * r + k];

    // ---- lower leaf rows (row kernel): leaf rows solve, top rows get partial terms
    std::vector<char> row_done((size_t)n, 0);
    for (int32_t task : P.lo_tasks) {
        const bool partial = task < 0;
        const int32_t row = partial ? ~task : task;
        CHECK(partial == (bool)P.row_top[row]);
        const int32_t s = P.lo_rowptr[row], e = P.lo_rowptr[row + 1];
        const int32_t hi = partial ? e : e - 1;
        for (int k = 0; k < r; ++k) {
            double acc = 0.0;
            for (int32_t p = s; p < hi; ++p) {
                const int32_t c = P.lo_cols[p];
                CHECK(!P.row_top[c] && row_done[c]);
                acc += P.lo_vals[p] * tmp[(size_t)c * r + k];
            }
            double v = b[(size_t)F.perm[row] * r + k] - acc;
            if (!partial) v /= P.lo_vals[e - 1];
            tmp[(size_t)row * r + k] = v;
        }
        if (!partial) row_done[row] = 1;
    }
    // ---- lower supernodal sweep, items in ticket order
    const int32_t nunits = (int32_t)P.units.size(), nparts = (int32_t)P.parts.size();
    std::vector<char> unit_done((size_t)nunits, 0), part_done((size_t)nparts, 0);
    std::vector<double> pbuf((size_t)nparts * kChunk * r, 0.0);
    CHECK((int32_t)P.unit_order_lo.size() == nunits + nparts);
    auto apply = [&](const SnUnit& U, const SnContrib& C, double* acc) {
        CHECK(C.src_unit >= 0 && C.src_unit < nunits && unit_done[C.src_unit]);
        CHECK(C.nr >= 1 && C.nr <= kChunk && C.w >= 1 && C.w <= kChunk);
        uint32_t mask = 0;
        for (int32_t i = 0; i < C.nr; ++i) {
            const int32_t pos = P.sn_rows[C.rows_off + i] - U.c0;
            CHECK(pos >= 0 && pos < U.w);
            if (pos < 0 || pos >= U.w) continue;
            mask |= 1u << pos;
            // the kernel's lane pos reads block row popc(mask below pos)
            CHECK(__builtin_popcount(C.rowmask & ((1u << pos) - 1u)) == i);
            for (int k = 0; k < r; ++k) {
                double s = 0.0;
                for (int32_t j = 0; j < C.w; ++j)
                    s += P.panels[C.panel_off + i + (size_t)j * C.ld] * tmp[(size_t)(C.xcol + j) * r + k];
                acc[(size_t)pos * r + k] += s;
            }
        }
        CHECK(mask == C.rowmask);
    };
    for (int32_t item : P.unit_order_lo) {
        if (item < 0) {
            const SnPartial& Q = P.parts[~item];
            CHECK(!part_done[~item]);
            const SnUnit& U = P.units[Q.unit];
            CHECK(Q.contrib_begin >= 0 && Q.contrib_begin < Q.contrib_end);
            for (int32_t e = Q.contrib_begin; e < Q.contrib_end; ++e) apply(U, P.contribs[e], &pbuf[(size_t)(~item) * kChunk * r]);
            part_done[~item] = 1;
            continue;
        }
        const SnUnit& U = P.units[item];
        CHECK(!unit_done[item]);
        std::vector<double> acc((size_t)kChunk * r, 0.0);
        for (int32_t q = U.part_begin; q < U.part_end; ++q) {
            CHECK(part_done[q] && P.parts[q].unit == item);
            for (size_t t = 0; t < acc.size(); ++t) acc[t] += pbuf[(size_t)q * kChunk * r + t];
        }
        for (int32_t e = U.contrib_begin; e < U.contrib_end; ++e) apply(U, P.contribs[e], acc.data());
        // the partial sums and the unit's own blocks cover its whole list
        if (U.part_begin < U.part_end) {
            CHECK(P.parts[U.part_end - 1].contrib_end == U.contrib_begin);
            for (int32_t q = U.part_begin + 1; q < U.part_end; ++q)
                CHECK(P.parts[q].contrib_begin == P.parts[q - 1].contrib_end);
        }
        for (int32_t i = 0; i < U.w; ++i) {
            CHECK(P.row_top[U.c0 + i]);
            for (int k = 0; k < r; ++k) tmp[(size_t)(U.c0 + i) * r + k] -= acc[(size_t)i * r + k];
        }
        for (int k = 0; k < r; ++k)
            for (int32_t j = 0; j < U.w; ++j) {
                const double xj = tmp[(size_t)(U.c0 + j) * r + k] / P.panels[U.panel_col_off + U.pos0 + j + (size_t)j * U.ld];
                tmp[(size_t)(U.c0 + j) * r + k] = xj;
                for (int32_t i = j + 1; i < U.w; ++i)
                    tmp[(size_t)(U.c0 + i) * r + k] -= P.panels[U.panel_col_off + U.pos0 + i + (size_t)j * U.ld] * xj;
            }
        unit_done[item] = 1;
    }
    for (int32_t u = 0; u < nunits; ++u) CHECK(unit_done[u]);
    {
        double m = 0.0, mm = 0.0;
        for (size_t q = 0; q < y.size(); ++q) {
            m = std::max(m, std::fabs(y[q] - tmp[q]));
            mm = std::max(mm, std::fabs(y[q]));
        }
        CHECK(m <= 1e-9 * mm);
    }
    // ---- upper supernodal sweep, items in ticket order; a block of rows may
    // read only rows whose unit finished, and it waits on one unit only
    std::vector<char> udone((size_t)nunits, 0), rdone((size_t)n, 0);
    CHECK((int32_t)P.unit_order_up.size() == nunits);
    for (int32_t u : P.unit_order_up) {
        const SnUnit& U = P.units[u];
        const int32_t* rows = P.sn_rows.data() + U.rows_off;
        // blocks and the one unit each waits on (as the kernel lists them)
        for (int32_t p0 = U.sn_w; p0 < U.ld; p0 += kChunk) {
            const int32_t dep = P.unit_of_row[rows[p0]];
            CHECK(dep > u && udone[dep]);
            for (int32_t p = p0; p < std::min(U.ld, p0 + kChunk); ++p) CHECK(rdone[rows[p]]);
        }
        const int32_t wj = U.pos0 + U.w;
        for (int32_t c = 0; wj + c * kChunk < U.sn_w; ++c) {
            CHECK(u + 1 + c < nunits && udone[u + 1 + c]);
            CHECK(P.units[u + 1 + c].c0 == U.c0 + U.w + c * kChunk);
        }
        std::vector<double> t((size_t)U.w * r);
        for (int32_t j = 0; j < U.w; ++j)
            for (int k = 0; k < r; ++k) t[(size_t)j * r + k] = tmp[(size_t)(U.c0 + j) * r + k];
        for (int32_t p = wj; p < U.ld; ++p)
            for (int32_t j = 0; j < U.w; ++j)
                for (int k = 0; k < r; ++k)
                    t[(size_t)j * r + k] -= P.panels[U.panel_col_off + p + (size_t)j * U.ld] * tmp[(size_t)rows[p] * r + k];
        for (int k = 0; k < r; ++k)
            for (int32_t j = U.w - 1; j >= 0; --j) {
                const double xj = t[(size_t)j * r + k] / P.panels[U.panel_col_off + U.pos0 + j + (size_t)j * U.ld];
                t[(size_t)j * r + k] = xj;
                for (int32_t i = 0; i < j; ++i)
                    t[(size_t)i * r + k] -= P.panels[U.panel_col_off + U.pos0 + j + (size_t)i * U.ld] * xj;
            }
        for (int32_t j = 0; j < U.w; ++j) {
            for (int k = 0; k < r; ++k) {
                tmp[(size_t)(U.c0 + j) * r + k] = t[(size_t)j * r + k];
                out[(size_t)F.perm[U.c0 + j] * r + k] = t[(size_t)j * r + k];
            }
            rdone[U.c0 + j] = 1;
        }
        udone[u] = 1;
    }
    // ---- upper leaf rows: top-row terms (no waits), then the chained pass
    for (int32_t task : P.upt_tasks) {
        const int32_t row = ~task;
        CHECK(row >= 0 && !P.row_top[row]);
        for (int k = 0; k < r; ++k) {
            double acc = 0.0;
            for (int32_t p = P.upt_rowptr[row]; p < P.upt_rowptr[row + 1]; ++p) {
                const int32_t c = P.upt_cols[p];
                CHECK(P.row_top[c] && rdone[c]);
                acc += P.upt_vals[p] * tmp[(size_t)c * r + k];
            }
            tmp[(size_t)row * r + k] -= acc;
        }
    }
    for (int32_t row : P.up_tasks) {
        const int32_t s = P.upl_rowptr[row], e = P.upl_rowptr[row + 1];
        CHECK(P.upl_cols[s] == row);
        for (int k = 0; k < r; ++k) {
            double acc = 0.0;
            for (int32_t p = s + 1; p < e; ++p) {
                const int32_t c = P.upl_cols[p];
                CHECK(rdone[c] && !P.row_top[c]);
                acc += P.upl_vals[p] * tmp[(size_t)c * r + k];
            }
            const double v = (tmp[(size_t)row * r + k] - acc) / P.upl_vals[s];
            tmp[(size_t)row * r + k] = v;
            out[(size_t)F.perm[row] * r + k] = v;
        }
        rdone[row] = 1;
    }
    for (int32_t i = 0; i < n; ++i) CHECK(rdone[i]);
    double m = 0.0, mm = 0.0;
    for (size_t q = 0; q < out.size(); ++q) {
        m = std::max(m, std::fabs(out[q] - ref[q]));
        mm = std::max(mm, std::fabs(ref[q]));
    }
    return m / mm;
}

// 2-D 5-point or 3-D 7-point grid Laplacian plus a diagonal shift (COO).
void grid(int dim, int k, std::vector<int32_t>& ii, std::vector<int32_t>& jj, std::vector<double>& xx) {
    auto id = [&](int a, int b, int c) { return dim == 3 ? (a * k + b) * k + c : a * k + b; };
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b)
            for (int c = 0; c < (dim == 3 ? k : 1); ++c) {
                const int i = id(a, b, c);
                ii.push_back(i); jj.push_back(i); xx.push_back(2.0 * dim + 0.1);
                const int nb[6][3] = {{a + 1, b, c}, {a - 1, b, c}, {a, b + 1, c}, {a, b - 1, c}, {a, b, c + 1}, {a, b, c - 1}};
                for (int t = 0; t < 2 * dim; ++t) {
                    const int A = nb[t][0], B = nb[t][1], C = nb[t][2];
                    if (A < 0 || A >= k || B < 0 || B >= k || C < 0 || C >= (dim == 3 ? k : 1)) continue;
                    ii.push_back(i); jj.push_back(id(A, B, C)); xx.push_back(-1.0);
                }
            }
}

}  // namespace

// transpose_columns against a plain serial transpose, on a random CSC large
// enough for the multi-threaded path, with and without a column filter and
// with 1, 3 and 8 threads: identical output every time.
bool check_transpose() {
    const int32_t n = 30000, per = 48;
    std::mt19937 g(11);
    std::vector<int32_t> colptr((size_t)n + 1, 0), rowidx;
    std::vector<double> vals;
    for (int32_t c = 0; c < n; ++c) {
        const int32_t m = (int32_t)(g() % (2 * per));
        std::vector<int32_t> rows;
        for (int32_t k = 0; k < m; ++k) rows.push_back((int32_t)(g() % n));
        std::sort(rows.begin(), rows.end());
        rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
        for (int32_t r : rows) {
            rowidx.push_back(r);
            vals.push_back((double)(g() % 1000) - 500.0);
        }
        colptr[c + 1] = (int32_t)rowidx.size();
    }
    std::vector<char> keep((size_t)n);
    for (auto& k : keep) k = (char)(g() % 3 != 0);
    bool ok = rowidx.size() >= ((size_t)1 << 20);
    for (const char* kc : {(const char*)nullptr, (const char*)keep.data()}) {
        // plain serial transpose
        std::vector<int32_t> p0((size_t)n + 1, 0), i0;
        std::vector<double> v0;
        for (int32_t c = 0; c < n; ++c)
            if (!kc || kc[c])
                for (int32_t k = colptr[c]; k < colptr[c + 1]; ++k) p0[rowidx[k] + 1]++;
        for (int32_t r = 0; r < n; ++r) p0[r + 1] += p0[r];
        i0.resize((size_t)p0[n]);
        v0.resize((size_t)p0[n]);
        std::vector<int32_t> nx(p0.begin(), p0.end() - 1);
        for (int32_t c = 0; c < n; ++c)
            if (!kc || kc[c])
                for (int32_t k = colptr[c]; k < colptr[c + 1]; ++k) {
                    i0[nx[rowidx[k]]] = c;
                    v0[nx[rowidx[k]]++] = vals[k];
                }
        for (int t : {1, 3, 8}) {
#ifdef _OPENMP
            omp_set_num_threads(t);
#endif
            std::vector<int32_t> p1, i1;
            std::vector<double> v1;
            transpose_columns(n, colptr, rowidx, vals.data(), kc, p1, i1, v1);
            ok = ok && p1 == p0 && i1 == i0 && v1 == v0;
            transpose_columns(n, colptr, rowidx, nullptr, kc, p1, i1, v1);
            ok = ok && p1 == p0 && i1 == i0 && v1.empty();
        }
    }
#ifdef _OPENMP
    omp_set_num_threads(omp_get_num_procs());
#endif
    std::printf("transpose_columns: %s\n", ok ? "ok" : "MISMATCH");
    return ok;
}

// The bulk sweeps' schedule (build_snb_upper / build_snb_lower): every item
// waits only on items with earlier tickets; a unit's groups are its
// contribution list without the chain block, in order, each a run of
// consecutive blocks from consecutive full chunks of one supernode (same row
// mask, contiguous source columns, so contiguous L tiles), waiting on the
// unit of its last chunk, and no larger than max_cols; its partial sums
// cover the start of its groups exactly; the upper blocks of a unit are the
// blocks of the 32-column sweep in its order.
int check_snb(const SolvePlan& P, const SnbOptions& o) {
    int bad = 0;
    SnbUpperPlan B;
    build_snb_upper(P, B);
    SnbLowerPlan L;
    build_snb_lower(P, B, o, L);
    const int32_t nu = (int32_t)P.units.size(), np = (int32_t)L.parts.size();
    if ((int32_t)L.order_lo.size() != nu + np || (int32_t)L.order_up.size() != nu) return 1;
    std::vector<int32_t> tu((size_t)nu, -1), tp((size_t)np, -1), tup((size_t)nu, -1);
    for (int32_t t = 0; t < nu + np; ++t) {
        const int32_t v = L.order_lo[t];
        if (v >= 0) tu[v] = t;
        else tp[~v] = t;
    }
    for (int32_t t = 0; t < nu; ++t) tup[L.order_up[t]] = t;
    int32_t gat = 0;
    for (int32_t u = 0; u < nu; ++u) {
        const SnUnit& U = P.units[u];
        const int32_t first = L.unit_info[(size_t)u * 4], gend = L.unit_info[(size_t)u * 4 + 1],
                      pb = L.unit_info[(size_t)u * 4 + 2], pe = L.unit_info[(size_t)u * 4 + 3];
        const int32_t chain = U.pos0 > 0 ? 1 : 0;
        // folded second block: the full block of the chunk two before (the
        // contribution list's second to last), the unit's last group; its
        // folded tile is D^{-1} L_block
        const int32_t f2 = (o.fold >= 2 && snb_fold2_lo(U)) ? 1 : 0;
        const int32_t gl = U.contrib_end - chain;  // end of the grouped blocks
        if (f2) {
            const SnContrib& C = P.contribs[U.contrib_end - 2];
            bad += C.src_unit != u - 2 || C.xcol != U.c0 - 2 * kChunk || C.w != kChunk || C.nr != U.w;
            const SnbGroup& G = L.groups[gend - 1];
            bad += gend <= first || G.first != U.contrib_end - 2 || G.cols != kChunk || G.src_unit != u - 2;
            const double* M2 = P.fold2.data() + (size_t)u * 2 * kChunk * kChunk;
            const double* D = P.panels.data() + U.panel_col_off + U.pos0;
            const double* Lb = P.panels.data() + U.panel_col_off - (int64_t)2 * kChunk * U.ld + U.pos0;
            for (int32_t i = 0; i < U.w; ++i)
                for (int32_t j = 0; j < kChunk; ++j) {
                    double v = 0.0;
                    for (int32_t m = 0; m <= i; ++m) v += D[i + (size_t)m * U.ld] * M2[m + j * kChunk];
                    bad += std::fabs(v - Lb[i + (size_t)j * U.ld]) > 1e-9 * (1.0 + std::fabs(Lb[i + (size_t)j * U.ld]));
                }
        }
        // the groups cover [contrib_begin, gl) exactly once (in any order: a
        // unit applies them by estimated source finish)
        std::vector<char> seen((size_t)(U.contrib_end - U.contrib_begin), 0);
        for (int32_t g = gat; g < gend; ++g) {
            const SnbGroup& G = L.groups[g];
            int32_t cols = 0, f = G.first;
            bad += G.first < U.contrib_begin || G.first >= gl;
            while (cols < G.cols && f >= U.contrib_begin && f < gl) {
                const SnContrib& C = P.contribs[f];
                bad += C.rowmask != G.rowmask || C.xcol != G.xcol + cols || seen[f - U.contrib_begin]++ != 0;
                if (cols + C.w < G.cols) bad += C.w != kChunk;
                cols += C.w;
                ++f;
            }
            bad += cols != G.cols || G.cols > std::max(o.max_cols, kChunk) || P.contribs[f - 1].src_unit != G.src_unit;
            bad += tu[G.src_unit] < 0 || tu[G.src_unit] >= tu[u];
        }
        for (int32_t e = U.contrib_begin; e < gl; ++e) bad += seen[e - U.contrib_begin] != 1;
        if (chain) bad += tu[u - 1] >= tu[u];
        int32_t at = gat;
        for (int32_t q = pb; q < pe; ++q) {
            bad += L.parts[q].unit != u || L.parts[q].contrib_begin != at ||
                   L.parts[q].contrib_end <= L.parts[q].contrib_begin;
            at = L.parts[q].contrib_end;
            bad += tp[q] < 0 || tp[q] >= tu[u];
            for (int32_t g = L.parts[q].contrib_begin; g < L.parts[q].contrib_end; ++g)
                bad += tu[L.groups[g].src_unit] >= tp[q];
        }
        bad += at != first || first > gend;
        gat = gend;
        const int32_t wj = U.pos0 + U.w, nrb = (U.ld - U.sn_w + kChunk - 1) / kChunk;
        const int32_t nlater = (U.sn_w - wj + kChunk - 1) / kChunk, uchain = wj < U.sn_w ? 1 : 0;
        const int32_t uf2 = snb_fold2_up(U) ? 1 : 0;
        bad += B.begin[u + 1] - B.begin[u] != nrb + nlater - uchain;
        if (uf2) {
            // the block of the chunk two after is the unit's last (the sweeps may fold it)
            bad += B.begin[u + 1] <= B.begin[u] || B.dep[B.begin[u + 1] - 1] != u + 2;
            // the folded tile is D^{-T} L[chunk two after, unit]^T: D^T M2 = L_block^T
            const int32_t p2 = wj + kChunk, wn2 = std::min(kChunk, U.sn_w - p2);
            const double* M2 = P.fold2.data() + ((size_t)u * 2 + 1) * kChunk * kChunk;
            const double* D = P.panels.data() + U.panel_col_off + U.pos0;
            const double* Ln = P.panels.data() + U.panel_col_off + p2;
            for (int32_t i = 0; i < U.w; ++i)
                for (int32_t j = 0; j < wn2; ++j) {
                    // (D^T M2)(i, j): D^T(i, m) = D(m, i), the lower triangle read transposed
                    double w2 = 0.0;
                    for (int32_t m = i; m < U.w; ++m) w2 += D[m + (size_t)i * U.ld] * M2[m + j * kChunk];
                    bad += std::fabs(w2 - Ln[j + (size_t)i * U.ld]) > 1e-9 * (1.0 + std::fabs(Ln[j + (size_t)i * U.ld]));
                }
        }
        for (int32_t t = B.begin[u]; t < B.begin[u + 1]; ++t) {
            bad += tup[B.dep[t]] >= tup[u];
            // later chunks of the supernode: not the chain one
            if (t - B.begin[u] >= nrb) bad += B.dep[t] < u + 1 + uchain;
            const int32_t nr = B.nrw[t] & 0xffff, w = B.nrw[t] >> 16;
            bad += nr < 1 || nr > kChunk || w != U.w;
            for (int32_t i = 0; i < kChunk; ++i) bad += (B.rows[(size_t)t * kChunk + i] >= 0) != (i < nr);
        }
        if (uchain) bad += tup[u + 1] >= tup[u];
    }
    bad += gat != (int32_t)L.groups.size();
    return bad;
}

int main() {
    if (!check_transpose()) return 1;
    // lgr, lskew: leaf-sweep wavefront (rows per group, skew; 0: level order);
    // early: the top rows' partial tasks keyed by their own inputs (not last)
    struct Case { int dim, k, minw, keep, group, lgr, lskew, early = 0; };
    const Case cases[] = {
        {2, 8, 1, 16, 32, 0, 0},  {2, 20, 4, 16, 32, 0, 0}, {2, 20, 8, 2, 3, 0, 0},   {2, 40, 1, 1, 2, 0, 0},
        {3, 8, 1, 2, 3, 0, 0},    {3, 14, 4, 16, 32, 0, 0}, {3, 14, 8, 4, 5, 0, 0},   {3, 18, 8, 16, 32, 0, 0},
        {3, 18, 8, 0, 0, 0, 0},   {3, 14, 100000, 16, 32, 0, 0}, {2, 40, 1, 0, 0, 0, 0}, {3, 14, 4, 0, 0, 0, 0},
        {2, 40, 4, 0, 0, 64, 2},  {3, 14, 4, 0, 0, 100, 3}, {3, 18, 8, 16, 32, 50, 1},
        {2, 40, 4, 0, 0, 0, 0, 1}, {3, 14, 4, 0, 0, 100, 3, 1},
    };
    int failed = 0;
    for (const Case& cs : cases) {
        std::vector<int32_t> ii, jj;
        std::vector<double> xx;
        grid(cs.dim, cs.k, ii, jj, xx);
        const int32_t n = cs.dim == 3 ? cs.k * cs.k * cs.k : cs.k * cs.k;
        Csc A;
        std::string err;
        if (build_csc(n, (int64_t)xx.size(), ii.data(), jj.data(), xx.data(), FMT_COO, A, err)) {
            std::printf("build_csc: %s\n", err.c_str());
            return 1;
        }
        Factor F;
        FactorOptions fo;
        if (factorize(A, fo, F, err)) {
            std::printf("factorize: %s\n", err.c_str());
            return 1;
        }
        std::vector<int32_t> rp, ci;
        std::vector<double> rv;
        transpose(n, F.colptr, F.rowidx, F.vals, rp, ci, rv);
        const auto lo = level_order(n, rp, ci, true), up = level_order(n, F.colptr, F.rowidx, false);
        SolvePlan P;
        PlanOptions po;
        po.min_top_width = cs.minw;
        po.part_keep = cs.keep;
        po.part_group = cs.group;
        po.leaf_group_rows = cs.lgr;
        po.leaf_skew = cs.lskew;
        po.partial_last = !cs.early;
        build_plan(F, lo, up, po, P);
        if (cs.group == 0) {  // the bulk schedule is built on plans without 32-column partial sums
            for (const SnbOptions& so : {SnbOptions{}, SnbOptions{2, 3, 32, false, 1000, 3000, 500},
                                         SnbOptions{0, 1, 128, true, 10, 10, 10}, SnbOptions{16, 0, 64, true, 1000, 5000, 9000, 1}}) {
                const int bad = check_snb(P, so);
                std::printf("%dD k=%d minw=%d bulk keep=%d group=%d fold=%d: checks failed %d %s\n", cs.dim, cs.k,
                            cs.minw, so.keep, so.group, so.fold, bad, bad ? "FAIL" : "ok");
                failed += bad != 0;
            }
        }
        for (int r : {1, 3}) {
            errors = 0;
            const double rel = run_case(F, P, r);
            const bool ok = errors == 0 && rel < 1e-10;
            std::printf("%dD k=%d minw=%d keep=%d group=%d r=%d: units %zu parts %zu rel err %.2e checks failed %d %s\n",
                        cs.dim, cs.k, cs.minw, cs.keep, cs.group, r, P.units.size(), P.parts.size(), rel, errors,
                        ok ? "ok" : "FAIL");
            failed += !ok;
        }
    }
    return failed ? 1 : 0;
}
