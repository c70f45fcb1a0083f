/*
 * ORACLE — test infrastructure only. This is the CPU restatement of the
 * reference's GPU-solve path that the tests, __graft_entry__.smoke() and
 * bench.py's CPU-baseline legs use as the checker. Nothing in the product
 * (cholespy_gb300/) links or calls this code.
 *
 * What it restates (reference rgl-epfl/cholespy v2.2.2):
 *   oracle_build_csc      src/cholesky_solver.cpp:8-149   (COO/CSR->CSC, sort,
 *                                                          sum duplicates)
 *   oracle_levels         kernels/kernels.cu:8-60 (analysis_lower/upper) and
 *                         src/cholesky_solver.cpp:349-367 (counting sort)
 *   oracle_lower_f32/f64  kernels/kernels.cu:64-131 (solve_lower), same
 *                         per-row operation order: r = b[perm[row]];
 *                         r -= val*x[col] for the row's entries in CSR order
 *                         (fused multiply-add, as nvcc compiles it);
 *                         x[row] = r / diag (diag last in the row)
 *   oracle_upper_f32/f64  kernels/kernels.cu:133-202 (solve_upper): entries
 *                         walked from the row's end down to the entry after
 *                         the diagonal; writes tmp[row] and out[perm[row]]
 *   oracle_chol_*         the host factorisation the reference delegates to
 *                         CHOLMOD (src/cholesky_solver.cpp:200-297). CHOLMOD is
 *                         an absent submodule (ext/suitesparse-metis-for-windows,
 *                         no pinned version in this checkout); this restates
 *                         the published up-looking simplicial LL^T (Davis,
 *                         "Direct Methods for Sparse Linear Systems", 2006,
 *                         chapter 4) on a GIVEN permutation, so the product's
 *                         factor can be checked entry by entry.
 *   oracle_cpu_solve      cholmod_solve(CHOLMOD_A) as called by solve_cpu
 *                         (src/cholesky_solver.cpp:435-463): x = P^T L^-T L^-1 P b
 *                         in FP64, RHS columns split across pthreads.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ prep -- */

/* Returns the number of entries after duplicate summation, or -1 on a bad
 * index. colptr has n+1 entries, rowidx/vals room for nnz entries. */
int64_t oracle_build_csc(int32_t n, int64_t nnz, const int32_t* ii, const int32_t* jj,
                         const double* x, int32_t fmt, int32_t* colptr, int32_t* rowidx,
                         double* vals) {
    int64_t e;
    int32_t i;
    memset(colptr, 0, sizeof(int32_t) * (size_t)(n + 1));
    if (fmt == 2) { /* COO: coo_to_csc, :8-48 */
        for (e = 0; e < nnz; ++e) {
            if (ii[e] < 0 || ii[e] >= n || jj[e] < 0 || jj[e] >= n) return -1;
            colptr[jj[e]]++;
        }
        for (i = 0, e = 0; i < n; ++i) { int32_t t = colptr[i]; colptr[i] = (int32_t)e; e += t; }
        colptr[n] = (int32_t)nnz;
        for (e = 0; e < nnz; ++e) {
            int32_t c = jj[e], d = colptr[c]++;
            rowidx[d] = ii[e];
            vals[d] = x[e];
        }
        for (i = 0, e = 0; i <= n; ++i) { int32_t t = colptr[i]; colptr[i] = (int32_t)e; e = t; }
    } else if (fmt == 1) { /* CSR: csr_to_csc, :50-92 */
        for (e = 0; e < nnz; ++e) {
            if (jj[e] < 0 || jj[e] >= n) return -1;
            colptr[jj[e]]++;
        }
        for (i = 0, e = 0; i < n; ++i) { int32_t t = colptr[i]; colptr[i] = (int32_t)e; e += t; }
        colptr[n] = (int32_t)nnz;
        for (i = 0; i < n; ++i)
            for (e = ii[i]; e < ii[i + 1]; ++e) {
                int32_t c = jj[e], d = colptr[c]++;
                rowidx[d] = i;
                vals[d] = x[e];
            }
        for (i = 0, e = 0; i <= n; ++i) { int32_t t = colptr[i]; colptr[i] = (int32_t)e; e = t; }
    } else { /* CSC: used as given */
        for (e = 0; e < nnz; ++e) if (jj[e] < 0 || jj[e] >= n) return -1;
        memcpy(colptr, ii, sizeof(int32_t) * (size_t)(n + 1));
        memcpy(rowidx, jj, sizeof(int32_t) * (size_t)nnz);
        memcpy(vals, x, sizeof(double) * (size_t)nnz);
    }
    /* csc_sort_indices (:95-116), stable insertion sort per column */
    for (i = 0; i < n; ++i) {
        int32_t s = colptr[i], t = colptr[i + 1], a, b;
        for (a = s + 1; a < t; ++a) {
            int32_t r = rowidx[a];
            double v = vals[a];
            for (b = a - 1; b >= s && rowidx[b] > r; --b) {
                rowidx[b + 1] = rowidx[b];
                vals[b + 1] = vals[b];
            }
            rowidx[b + 1] = r;
            vals[b + 1] = v;
        }
    }
    /* csc_sum_duplicates (:119-149) */
    {
        int64_t w = 0;
        int32_t end = 0;
        for (i = 0; i < n; ++i) {
            int32_t j = end;
            end = colptr[i + 1];
            while (j < end) {
                int32_t r = rowidx[j];
                double v = vals[j++];
                while (j < end && rowidx[j] == r) v += vals[j++];
                rowidx[w] = r;
                vals[w] = v;
                ++w;
            }
            colptr[i + 1] = (int32_t)w;
        }
        return w;
    }
}

/* --------------------------------------------------------------- levels -- */

/* lower = 1: CSR of L (diagonal last), rows processed 0..n-1.
 * lower = 0: CSR of L^T (diagonal first), rows processed n-1..0.
 * row_levels[i] = level of row i, order = rows sorted by (level, row). */
void oracle_levels(int32_t n, const int32_t* rowptr, const int32_t* cols, int32_t lower,
                   int32_t* row_levels, int32_t* order, int32_t* max_lvl_out) {
    int32_t max_lvl = 0, t;
    for (t = 0; t < n; ++t) {
        int32_t row = lower ? t : n - 1 - t;
        int32_t s = rowptr[row], e = rowptr[row + 1] - 1, lvl = 0, k;
        if (lower) {
            for (k = s; k < e; ++k) {
                int32_t cl = row_levels[cols[k]];
                if (lvl <= cl) lvl = cl + 1;
            }
        } else {
            for (k = e; k > s; --k) {
                int32_t cl = row_levels[cols[k]];
                if (lvl <= cl) lvl = cl + 1;
            }
        }
        if (lvl > max_lvl) max_lvl = lvl;
        row_levels[row] = lvl;
    }
    /* counting sort, :349-367 */
    {
        int32_t nl = max_lvl + 1, i;
        int32_t* ptr = (int32_t*)calloc((size_t)nl + 1, sizeof(int32_t));
        for (i = 0; i < n; ++i) ptr[1 + row_levels[i]]++;
        for (i = 0; i < nl; ++i) ptr[i + 1] += ptr[i];
        for (i = 0; i < n; ++i) order[ptr[row_levels[i]]++] = i;
        free(ptr);
    }
    if (max_lvl_out) *max_lvl_out = max_lvl;
}

/* --------------------------------------------------------------- sweeps -- */

#define DEFINE_SWEEPS(T, SUF, FMA)                                                               \
    void oracle_lower_##SUF(int32_t n, int32_t nrhs, const int32_t* rowptr, const int32_t* cols,  \
                            const T* vals, const int32_t* order, const int32_t* perm, const T* b, \
                            T* tmp) {                                                            \
        int32_t t, k;                                                                            \
        for (t = 0; t < n; ++t) {                                                                \
            int32_t row = order[t], s = rowptr[row], e = rowptr[row + 1] - 1, i;                 \
            T diag = vals[e];                                                                    \
            for (k = 0; k < nrhs; ++k) {                                                         \
                T r = b[(int64_t)perm[row] * nrhs + k];                                          \
                for (i = s; i < e; ++i) r = FMA(-vals[i], tmp[(int64_t)cols[i] * nrhs + k], r);  \
                tmp[(int64_t)row * nrhs + k] = r / diag;                                         \
            }                                                                                    \
        }                                                                                        \
    }                                                                                            \
    void oracle_upper_##SUF(int32_t n, int32_t nrhs, const int32_t* rowptr, const int32_t* cols,  \
                            const T* vals, const int32_t* order, const int32_t* perm, T* tmp,     \
                            T* out) {                                                            \
        int32_t t, k;                                                                            \
        for (t = 0; t < n; ++t) {                                                                \
            int32_t row = order[t], s = rowptr[row], e = rowptr[row + 1] - 1, i;                 \
            T diag = vals[s];                                                                    \
            for (k = 0; k < nrhs; ++k) {                                                         \
                T r = tmp[(int64_t)row * nrhs + k];                                              \
                for (i = e; i > s; --i) r = FMA(-vals[i], tmp[(int64_t)cols[i] * nrhs + k], r);  \
                tmp[(int64_t)row * nrhs + k] = r / diag;                                         \
                out[(int64_t)perm[row] * nrhs + k] = r / diag;                                   \
            }                                                                                    \
        }                                                                                        \
    }

DEFINE_SWEEPS(float, f32, fmaf)
DEFINE_SWEEPS(double, f64, fma)

/* ------------------------------------------------- simplicial LL^T ------- */

/* Upper triangle of C = P A P^T by columns (rows <= column), from the
 * entries of A with row >= col (CHOLMOD stype = -1 reads only those).
 * Arrays are malloc'd; caller frees. */
static void permuted_upper(int32_t n, const int32_t* Ap, const int32_t* Ai, const double* Ax,
                           const int32_t* perm, int32_t** Cp_out, int32_t** Ci_out,
                           double** Cx_out) {
    int32_t* pinv = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t* Cp = (int32_t*)calloc((size_t)n + 1, sizeof(int32_t));
    int32_t c, k;
    for (k = 0; k < n; ++k) pinv[perm[k]] = k;
    for (c = 0; c < n; ++c)
        for (k = Ap[c]; k < Ap[c + 1]; ++k) {
            int32_t r = Ai[k];
            if (r < c) continue;
            int32_t pr = pinv[r], pc = pinv[c];
            Cp[(pr > pc ? pr : pc) + 1]++;
        }
    for (c = 0; c < n; ++c) Cp[c + 1] += Cp[c];
    int32_t* Ci = (int32_t*)malloc(sizeof(int32_t) * (size_t)(Cp[n] > 0 ? Cp[n] : 1));
    double* Cx = (double*)malloc(sizeof(double) * (size_t)(Cp[n] > 0 ? Cp[n] : 1));
    int32_t* nx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (c = 0; c < n; ++c) nx[c] = Cp[c];
    for (c = 0; c < n; ++c)
        for (k = Ap[c]; k < Ap[c + 1]; ++k) {
            int32_t r = Ai[k];
            if (r < c) continue;
            int32_t pr = pinv[r], pc = pinv[c];
            int32_t hi = pr > pc ? pr : pc, lo = pr > pc ? pc : pr;
            int32_t d = nx[hi]++;
            Ci[d] = lo;
            Cx[d] = Ax[k];
        }
    free(nx);
    free(pinv);
    *Cp_out = Cp;
    *Ci_out = Ci;
    *Cx_out = Cx;
}

/* Elimination tree of C from its upper triangle (Liu). */
static void etree_upper(int32_t n, const int32_t* Cp, const int32_t* Ci, int32_t* parent) {
    int32_t* anc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t k, p;
    for (k = 0; k < n; ++k) {
        parent[k] = -1;
        anc[k] = -1;
        for (p = Cp[k]; p < Cp[k + 1]; ++p) {
            int32_t i = Ci[p];
            while (i != -1 && i < k) {
                int32_t inext = anc[i];
                anc[i] = k;
                if (inext == -1) parent[i] = k;
                i = inext;
            }
        }
    }
    free(anc);
}

/* Symbolic: Lp (n+1) of L = chol(P A P^T). Returns nnz(L). */
int64_t oracle_chol_symbolic(int32_t n, const int32_t* Ap, const int32_t* Ai, const double* Ax,
                             const int32_t* perm, int32_t* Lp) {
    int32_t *Cp, *Ci, k, p;
    double* Cx;
    permuted_upper(n, Ap, Ai, Ax, perm, &Cp, &Ci, &Cx);
    int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t* mark = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int64_t* cnt = (int64_t*)calloc((size_t)(n > 0 ? n : 1), sizeof(int64_t));
    etree_upper(n, Cp, Ci, parent);
    for (k = 0; k < n; ++k) {
        mark[k] = k;
        cnt[k]++;
        for (p = Cp[k]; p < Cp[k + 1]; ++p) {
            int32_t i = Ci[p];
            for (; i < k && mark[i] != k; i = parent[i]) {
                mark[i] = k;
                cnt[i]++; /* L(k, i) != 0 */
            }
        }
    }
    Lp[0] = 0;
    for (k = 0; k < n; ++k) Lp[k + 1] = Lp[k] + (int32_t)cnt[k];
    int64_t nz = Lp[n];
    free(cnt);
    free(mark);
    free(parent);
    free(Cp);
    free(Ci);
    free(Cx);
    return nz;
}

/* Numeric up-looking LL^T. Returns 0, or k+1 if the k-th pivot is not
 * positive (CHOLMOD_NOT_POSDEF). */
int32_t oracle_chol_numeric(int32_t n, const int32_t* Ap, const int32_t* Ai, const double* Ax,
                            const int32_t* perm, const int32_t* Lp, int32_t* Li, double* Lx) {
    int32_t *Cp, *Ci, k, p;
    double* Cx;
    int32_t rc = 0;
    permuted_upper(n, Ap, Ai, Ax, perm, &Cp, &Ci, &Cx);
    size_t nn = (size_t)(n > 0 ? n : 1);
    int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * nn);
    int32_t* mark = (int32_t*)malloc(sizeof(int32_t) * nn);
    int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * nn);
    int32_t* path = (int32_t*)malloc(sizeof(int32_t) * nn);
    int32_t* next = (int32_t*)malloc(sizeof(int32_t) * nn);
    double* x = (double*)calloc(nn, sizeof(double));
    etree_upper(n, Cp, Ci, parent);
    for (k = 0; k < n; ++k) next[k] = Lp[k];
    for (k = 0; k < n; ++k) {
        /* pattern of row k of L: reach of C(0:k-1, k) in the etree */
        int32_t top = n;
        mark[k] = k;
        x[k] = 0.0;
        for (p = Cp[k]; p < Cp[k + 1]; ++p) {
            int32_t i = Ci[p], len = 0;
            x[i] += Cx[p];
            for (; i < k && mark[i] != k; i = parent[i]) {
                path[len++] = i;
                mark[i] = k;
            }
            while (len > 0) stack[--top] = path[--len];
        }
        double d = x[k];
        x[k] = 0.0;
        for (; top < n; ++top) {
            int32_t i = stack[top];
            double lki = x[i] / Lx[Lp[i]];
            x[i] = 0.0;
            for (p = Lp[i] + 1; p < next[i]; ++p) x[Li[p]] -= Lx[p] * lki;
            d -= lki * lki;
            p = next[i]++;
            Li[p] = k;
            Lx[p] = lki;
        }
        if (!(d > 0.0)) { rc = k + 1; break; }
        p = next[k]++;
        Li[p] = k;
        Lx[p] = sqrt(d);
    }
    free(x);
    free(next);
    free(path);
    free(stack);
    free(mark);
    free(parent);
    free(Cp);
    free(Ci);
    free(Cx);
    return rc;
}

/* ------------------------------------------------------------ CPU solve -- */

typedef struct {
    int32_t n, nrhs, k0, k1;
    const int32_t *perm, *Lp, *Li;
    const double *Lx, *b;
    double* x;
} solve_job;

static void* solve_worker(void* arg) {
    solve_job* j = (solve_job*)arg;
    int32_t n = j->n, nrhs = j->nrhs, k, c, p;
    double* y = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (k = j->k0; k < j->k1; ++k) {
        for (c = 0; c < n; ++c) y[c] = j->b[(int64_t)j->perm[c] * nrhs + k];
        for (c = 0; c < n; ++c) { /* L y = P b, column oriented */
            double yc = y[c] / j->Lx[j->Lp[c]];
            y[c] = yc;
            for (p = j->Lp[c] + 1; p < j->Lp[c + 1]; ++p) y[j->Li[p]] -= j->Lx[p] * yc;
        }
        for (c = n - 1; c >= 0; --c) { /* L^T z = y */
            double acc = y[c];
            for (p = j->Lp[c] + 1; p < j->Lp[c + 1]; ++p) acc -= j->Lx[p] * y[j->Li[p]];
            y[c] = acc / j->Lx[j->Lp[c]];
        }
        for (c = 0; c < n; ++c) j->x[(int64_t)j->perm[c] * nrhs + k] = y[c];
    }
    free(y);
    return NULL;
}

/* x = P^T L^-T L^-1 P b, FP64, (n, nrhs) row-major; RHS split over threads. */
void oracle_cpu_solve(int32_t n, int32_t nrhs, const int32_t* perm, const int32_t* Lp,
                      const int32_t* Li, const double* Lx, const double* b, double* x,
                      int32_t threads) {
    int32_t t, nt = threads < 1 ? 1 : threads;
    if (nt > nrhs) nt = nrhs;
    if (nt < 1) return;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    solve_job* jobs = (solve_job*)malloc(sizeof(solve_job) * (size_t)nt);
    for (t = 0; t < nt; ++t) {
        solve_job j = {n, nrhs, (int32_t)((int64_t)nrhs * t / nt), (int32_t)((int64_t)nrhs * (t + 1) / nt),
                       perm, Lp, Li, Lx, b, x};
        jobs[t] = j;
    }
    for (t = 1; t < nt; ++t) pthread_create(&th[t], NULL, solve_worker, &jobs[t]);
    solve_worker(&jobs[0]);
    for (t = 1; t < nt; ++t) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
}
