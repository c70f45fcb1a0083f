// Sparse input preparation (host). Same semantics as the reference's
// coo_to_csc / csr_to_csc / csc_sort_indices / csc_sum_duplicates
// (src/cholesky_solver.cpp:8-149): the result is a CSC matrix whose row
// indices are sorted inside each column and whose duplicate (row, col)
// entries are summed. Unlike the reference, every index is range-checked and
// the per-column sort is stable, so duplicates are summed in input order.
#include "host.h"

#include <algorithm>
#include <cstring>
#include <numeric>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace gbchol {

namespace {

int prep_threads(int64_t nnz) {
#ifdef _OPENMP
    if (nnz >= (int64_t)1 << 18) return std::max(1, std::min(omp_get_max_threads(), 64));
#endif
    (void)nnz;
    return 1;
}

// Counting-sort placement of (row, col, val) triples into columns, keeping
// input order inside a column. `row_of(e)` / `col_of(e)` give the entry e.
// Large inputs: contiguous chunks of entries count per column, and chunk t's
// entries of a column go after those of chunks < t, so the placement (and
// everything after it) is the same for any thread count.
template <class RowOf, class ColOf>
void place_by_column(int32_t n, int64_t nnz, RowOf row_of, ColOf col_of, const double* x,
                     Csc& out) {
    out.n = n;
    out.colptr.assign((size_t)n + 1, 0);
    out.rowidx.resize((size_t)nnz);
    out.vals.resize((size_t)nnz);
    const int nt = prep_threads(nnz);
    if (nt == 1) {
        for (int64_t e = 0; e < nnz; ++e) out.colptr[(size_t)col_of(e) + 1]++;
        for (int32_t c = 0; c < n; ++c) out.colptr[c + 1] += out.colptr[c];
        std::vector<int32_t> next(out.colptr.begin(), out.colptr.end() - 1);
        for (int64_t e = 0; e < nnz; ++e) {
            int32_t c = col_of(e);
            int32_t dst = next[c]++;
            out.rowidx[dst] = row_of(e);
            out.vals[dst] = x[e];
        }
        return;
    }
    std::vector<int32_t> cnt((size_t)nt * n, 0);  // entries per (chunk, column), then offsets
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        int32_t* ct = cnt.data() + (size_t)t * n;
        for (int64_t e = nnz * t / nt; e < nnz * (t + 1) / nt; ++e) ct[col_of(e)]++;
    }
    int32_t run = 0;
    for (int32_t c = 0; c < n; ++c) {
        out.colptr[c] = run;
        for (int t = 0; t < nt; ++t) {
            const int32_t k = cnt[(size_t)t * n + c];
            cnt[(size_t)t * n + c] = run;
            run += k;
        }
    }
    out.colptr[n] = run;
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        int32_t* next = cnt.data() + (size_t)t * n;
        for (int64_t e = nnz * t / nt; e < nnz * (t + 1) / nt; ++e) {
            int32_t dst = next[col_of(e)]++;
            out.rowidx[dst] = row_of(e);
            out.vals[dst] = x[e];
        }
    }
}

// Stable sort of column c's entries [start, end) by row index, then
// summation of equal rows (in their input order, from the first one); the
// merged entries are written from `w` on. Returns the merged count.
int32_t sort_sum_column(Csc& A, int32_t start, int32_t end, int32_t w,
                        std::vector<std::pair<int32_t, double>>& tmp) {
    bool sorted = true;
    for (int32_t k = start + 1; k < end; ++k)
        if (A.rowidx[k] < A.rowidx[k - 1]) { sorted = false; break; }
    if (!sorted) {
        tmp.resize((size_t)(end - start));
        for (int32_t k = start; k < end; ++k) tmp[k - start] = {A.rowidx[k], A.vals[k]};
        std::stable_sort(tmp.begin(), tmp.end(),
                         [](const auto& a, const auto& b) { return a.first < b.first; });
        for (int32_t k = start; k < end; ++k) {
            A.rowidx[k] = tmp[k - start].first;
            A.vals[k] = tmp[k - start].second;
        }
    }
    const int32_t w0 = w;
    int32_t k = start;
    while (k < end) {
        int32_t r = A.rowidx[k];
        double v = A.vals[k++];
        while (k < end && A.rowidx[k] == r) v += A.vals[k++];
        A.rowidx[w] = r;
        A.vals[w] = v;
        ++w;
    }
    return w - w0;
}

// Stable sort of each column by row index, then summation of equal rows.
// Large inputs: columns are sorted and merged in place in parallel, then
// compacted by the merged counts (same result as the serial pass).
void sort_and_sum(Csc& A) {
    const int32_t n = A.n;
    const int nt = prep_threads(A.nnz());
    if (nt == 1) {
        std::vector<std::pair<int32_t, double>> tmp;
        int32_t w = 0, start = 0;
        for (int32_t c = 0; c < n; ++c) {
            const int32_t end = A.colptr[c + 1];
            A.colptr[c] = w;
            w += sort_sum_column(A, start, end, w, tmp);
            start = end;
        }
        A.colptr[n] = w;
    } else {
        std::vector<int32_t> merged((size_t)n + 1, 0);
#pragma omp parallel num_threads(nt)
        {
            std::vector<std::pair<int32_t, double>> tmp;
#pragma omp for schedule(dynamic, 256)
            for (int32_t c = 0; c < n; ++c)
                merged[c + 1] = sort_sum_column(A, A.colptr[c], A.colptr[c + 1], A.colptr[c], tmp);
        }
        for (int32_t c = 0; c < n; ++c) merged[c + 1] += merged[c];
        // compaction: column c's merged entries move down from colptr[c] to
        // merged[c] <= colptr[c]; columns in order, so nothing is overwritten
        // before it is read
        for (int32_t c = 0; c < n; ++c) {
            const int32_t src = A.colptr[c], dst = merged[c], len = merged[c + 1] - merged[c];
            if (src != dst) {
                std::memmove(A.rowidx.data() + dst, A.rowidx.data() + src, sizeof(int32_t) * len);
                std::memmove(A.vals.data() + dst, A.vals.data() + src, sizeof(double) * len);
            }
        }
        A.colptr.swap(merged);
    }
    const int32_t w = A.colptr[n];
    A.rowidx.resize((size_t)w);
    A.vals.resize((size_t)w);
    A.rowidx.shrink_to_fit();
    A.vals.shrink_to_fit();
}

}  // namespace

Status build_csc(int32_t n, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                 int32_t fmt, Csc& out, std::string& err) {
    if (n < 0) { err = "The number of rows must be non-negative."; return ST_INVALID; }
    if (nnz < 0 || nnz >= (int64_t)INT32_MAX) {
        err = "Number of nonzero entries out of range.";
        return ST_INVALID;
    }
    if (fmt == FMT_COO) {
        for (int64_t e = 0; e < nnz; ++e) {
            if (ii[e] < 0 || ii[e] >= n || jj[e] < 0 || jj[e] >= n) {
                err = "Sparse COO matrix: index out of range.";
                return ST_INVALID;
            }
        }
        place_by_column(n, nnz, [&](int64_t e) { return ii[e]; },
                        [&](int64_t e) { return jj[e]; }, x, out);
    } else if (fmt == FMT_CSR || fmt == FMT_CSC) {
        const char* what = fmt == FMT_CSR ? "Sparse CSR matrix" : "Sparse CSC matrix";
        if (ii[0] != 0 || (int64_t)ii[n] != nnz) {
            err = std::string(what) + ": Invalid pointer array.";
            return ST_INVALID;
        }
        for (int32_t k = 0; k < n; ++k)
            if (ii[k + 1] < ii[k]) {
                err = std::string(what) + ": Invalid pointer array.";
                return ST_INVALID;
            }
        for (int64_t e = 0; e < nnz; ++e)
            if (jj[e] < 0 || jj[e] >= n) {
                err = std::string(what) + ": index out of range.";
                return ST_INVALID;
            }
        if (fmt == FMT_CSR) {
            // owner row of each entry
            std::vector<int32_t> rowof((size_t)nnz);
            for (int32_t r = 0; r < n; ++r)
                for (int32_t e = ii[r]; e < ii[r + 1]; ++e) rowof[e] = r;
            place_by_column(n, nnz, [&](int64_t e) { return rowof[e]; },
                            [&](int64_t e) { return jj[e]; }, x, out);
        } else {
            out.n = n;
            out.colptr.assign(ii, ii + n + 1);
            out.rowidx.assign(jj, jj + nnz);
            out.vals.assign(x, x + nnz);
        }
    } else {
        err = "Unknown matrix type.";
        return ST_INVALID;
    }
    sort_and_sum(out);
    return ST_OK;
}

void symmetric_from_lower(const Csc& A, Csc& S) {
    const int32_t n = A.n;
    S.n = n;
    S.colptr.assign((size_t)n + 1, 0);
    for (int32_t c = 0; c < n; ++c)
        for (int32_t k = A.colptr[c]; k < A.colptr[c + 1]; ++k) {
            int32_t r = A.rowidx[k];
            if (r < c) continue;
            S.colptr[c + 1]++;
            if (r != c) S.colptr[r + 1]++;
        }
    for (int32_t c = 0; c < n; ++c) S.colptr[c + 1] += S.colptr[c];
    S.rowidx.resize((size_t)S.colptr[n]);
    S.vals.resize((size_t)S.colptr[n]);
    std::vector<int32_t> next(S.colptr.begin(), S.colptr.end() - 1);
    // Visiting columns in increasing order keeps every column's rows sorted:
    // mirrored entries (c, r) with c < r arrive while scanning column c < r.
    for (int32_t c = 0; c < n; ++c)
        for (int32_t k = A.colptr[c]; k < A.colptr[c + 1]; ++k) {
            int32_t r = A.rowidx[k];
            if (r < c) continue;
            double v = A.vals[k];
            // entry (r, c) into column c
            int32_t d = next[c]++;
            S.rowidx[d] = r;
            S.vals[d] = v;
            if (r != c) {  // mirror (c, r) into column r
                int32_t d2 = next[r]++;
                S.rowidx[d2] = c;
                S.vals[d2] = v;
            }
        }
    // Column c receives mirrored rows (< c) interleaved with its own rows
    // (>= c); restore the sorted order.
    for (int32_t c = 0; c < n; ++c) {
        int32_t s = S.colptr[c], e = S.colptr[c + 1];
        bool sorted = true;
        for (int32_t k = s + 1; k < e; ++k)
            if (S.rowidx[k] < S.rowidx[k - 1]) { sorted = false; break; }
        if (sorted) continue;
        std::vector<std::pair<int32_t, double>> t((size_t)(e - s));
        for (int32_t k = s; k < e; ++k) t[k - s] = {S.rowidx[k], S.vals[k]};
        std::sort(t.begin(), t.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        for (int32_t k = s; k < e; ++k) { S.rowidx[k] = t[k - s].first; S.vals[k] = t[k - s].second; }
    }
}

void transpose_columns(int32_t n, const std::vector<int32_t>& colptr, const std::vector<int32_t>& rowidx,
                       const double* vals, const char* keep_col, std::vector<int32_t>& tptr,
                       std::vector<int32_t>& tidx, std::vector<double>& tvals) {
    const int64_t nnz = (int64_t)rowidx.size();
    int nt = 1;
#ifdef _OPENMP
    if (nnz >= (int64_t)1 << 20) nt = std::max(1, std::min(omp_get_max_threads(), 64));
#endif
    // contiguous column ranges of about nnz / nt entries, in column order: a
    // range's rows are filled after those of every earlier range, so columns
    // stay ascending within each row whatever the thread count
    std::vector<int32_t> c0((size_t)nt + 1, n);
    c0[0] = 0;
    for (int t = 1; t < nt; ++t) {
        const int32_t target = (int32_t)(nnz * t / nt);
        c0[t] = (int32_t)(std::lower_bound(colptr.begin(), colptr.end() - 1, target) - colptr.begin());
    }
    for (int t = 1; t <= nt; ++t) c0[t] = std::max(c0[t], c0[t - 1]);
    std::vector<int32_t> cnt((size_t)nt * n, 0);  // entries per (range, row)
#pragma omp parallel for num_threads(nt) schedule(static, 1) if (nt > 1)
    for (int t = 0; t < nt; ++t) {
        int32_t* ct = cnt.data() + (size_t)t * n;
        for (int32_t c = c0[t]; c < c0[t + 1]; ++c) {
            if (keep_col && !keep_col[c]) continue;
            for (int32_t k = colptr[c]; k < colptr[c + 1]; ++k) ct[rowidx[k]]++;
        }
    }
    tptr.assign((size_t)n + 1, 0);
    for (int32_t r = 0; r < n; ++r) {
        int32_t v = 0;
        for (int t = 0; t < nt; ++t) v += cnt[(size_t)t * n + r];
        tptr[r + 1] = tptr[r] + v;
    }
    // turn the counts into each range's first slot per row
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1)
    for (int32_t r = 0; r < n; ++r) {
        int32_t off = tptr[r];
        for (int t = 0; t < nt; ++t) {
            const int32_t v = cnt[(size_t)t * n + r];
            cnt[(size_t)t * n + r] = off;
            off += v;
        }
    }
    tidx.resize((size_t)tptr[n]);
    tvals.resize(vals ? (size_t)tptr[n] : 0);
#pragma omp parallel for num_threads(nt) schedule(static, 1) if (nt > 1)
    for (int t = 0; t < nt; ++t) {
        int32_t* next = cnt.data() + (size_t)t * n;
        for (int32_t c = c0[t]; c < c0[t + 1]; ++c) {
            if (keep_col && !keep_col[c]) continue;
            for (int32_t k = colptr[c]; k < colptr[c + 1]; ++k) {
                const int32_t d = next[rowidx[k]]++;
                tidx[d] = c;
                if (vals) tvals[d] = vals[k];
            }
        }
    }
}

void transpose(int32_t n, const std::vector<int32_t>& colptr, const std::vector<int32_t>& rowidx,
               const std::vector<double>& vals, std::vector<int32_t>& tptr,
               std::vector<int32_t>& tidx, std::vector<double>& tvals) {
    transpose_columns(n, colptr, rowidx, vals.empty() ? nullptr : vals.data(), nullptr, tptr, tidx, tvals);
}

}  // namespace gbchol
