// Dense FP64 building blocks for the host multifrontal factorisation:
// packed, register-blocked GEMM (C -= A B^T), recursive TRSM and Cholesky.
// Written for the compiler's auto-vectoriser (no intrinsics, so the same
// source builds on x86-64 and aarch64).
#include "dense.h"

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace gbchol {
namespace dense {

namespace {

constexpr int MR = 8;
constexpr int NR = 4;
constexpr int64_t MC = 96;
constexpr int64_t NC = 192;
constexpr int64_t KC = 256;

// Pack A[i0:i0+mc, p0:p0+kc] into MR-row panels: panel q, step p at
// Ap[(q*kc + p)*MR + i].
void pack_a(int64_t mc, int64_t kc, const double* A, int64_t lda, double* Ap) {
    for (int64_t q = 0; q < mc; q += MR) {
        int64_t mr = std::min<int64_t>(MR, mc - q);
        double* dst = Ap + q * kc;
        for (int64_t p = 0; p < kc; ++p) {
            const double* src = A + q + p * lda;
            int64_t i = 0;
            for (; i < mr; ++i) dst[p * MR + i] = src[i];
            for (; i < MR; ++i) dst[p * MR + i] = 0.0;
        }
    }
}

// Pack B[j0:j0+nc, p0:p0+kc] (B is n x k, we need B^T) into NR panels:
// Bp[(q*kc + p)*NR + j] = B[q+j, p].
void pack_b(int64_t nc, int64_t kc, const double* B, int64_t ldb, double* Bp) {
    for (int64_t q = 0; q < nc; q += NR) {
        int64_t nr = std::min<int64_t>(NR, nc - q);
        double* dst = Bp + q * kc;
        for (int64_t p = 0; p < kc; ++p) {
            const double* src = B + q + p * ldb;
            int64_t j = 0;
            for (; j < nr; ++j) dst[p * NR + j] = src[j];
            for (; j < NR; ++j) dst[p * NR + j] = 0.0;
        }
    }
}

inline void micro_kernel(int64_t kc, const double* __restrict Ap, const double* __restrict Bp,
                         double* C, int64_t ldc, int64_t mr, int64_t nr) {
    double acc[NR][MR];
    for (int j = 0; j < NR; ++j)
        for (int i = 0; i < MR; ++i) acc[j][i] = 0.0;
    for (int64_t p = 0; p < kc; ++p) {
        const double* a = Ap + p * MR;
        const double* b = Bp + p * NR;
        for (int j = 0; j < NR; ++j) {
            const double bj = b[j];
            for (int i = 0; i < MR; ++i) acc[j][i] += a[i] * bj;
        }
    }
    if (mr == MR && nr == NR) {
        for (int j = 0; j < NR; ++j)
            for (int i = 0; i < MR; ++i) C[i + j * ldc] -= acc[j][i];
    } else {
        for (int64_t j = 0; j < nr; ++j)
            for (int64_t i = 0; i < mr; ++i) C[i + j * ldc] -= acc[j][i];
    }
}

// One (mc x nc) tile of C, all of k.
void gemm_tile(int64_t mc, int64_t nc, int64_t k, const double* A, int64_t lda, const double* B,
               int64_t ldb, double* C, int64_t ldc, double* Ap, double* Bp) {
    for (int64_t p0 = 0; p0 < k; p0 += KC) {
        int64_t kc = std::min(KC, k - p0);
        pack_a(mc, kc, A + p0 * lda, lda, Ap);
        pack_b(nc, kc, B + p0 * ldb, ldb, Bp);
        for (int64_t j = 0; j < nc; j += NR) {
            int64_t nr = std::min<int64_t>(NR, nc - j);
            for (int64_t i = 0; i < mc; i += MR) {
                int64_t mr = std::min<int64_t>(MR, mc - i);
                micro_kernel(kc, Ap + i * kc, Bp + j * kc, C + i + j * ldc, ldc, mr, nr);
            }
        }
    }
}

// Small products: plain loops beat packing.
void gemm_small(int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                int64_t ldb, double* C, int64_t ldc, bool lower_only) {
    for (int64_t j = 0; j < n; ++j) {
        double* c = C + j * ldc;
        int64_t i0 = lower_only ? std::min(j, m) : 0;
        for (int64_t p = 0; p < k; ++p) {
            const double b = B[j + p * ldb];
            if (b == 0.0) continue;
            const double* a = A + p * lda;
            for (int64_t i = i0; i < m; ++i) c[i] -= a[i] * b;
        }
    }
}

}  // namespace

void gemm_nt_sub(int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                 int64_t ldb, double* C, int64_t ldc, bool lower_only, int threads) {
    if (m <= 0 || n <= 0 || k <= 0) return;
    // small products, and thin ones (k <= 8: the rank-k update of a narrow
    // supernode), are column updates; the choice depends on the sizes only
    if (k <= 8 || m * n * k <= 32 * 32 * 32) {
        gemm_small(m, n, k, A, lda, B, ldb, C, ldc, lower_only);
        return;
    }
    const int64_t tm = (m + MC - 1) / MC, tn = (n + NC - 1) / NC;
    struct T { int64_t i0, j0; };
    std::vector<T> tiles;
    tiles.reserve((size_t)(tm * tn));
    for (int64_t jt = 0; jt < tn; ++jt)
        for (int64_t it = 0; it < tm; ++it) {
            int64_t i0 = it * MC, j0 = jt * NC;
            if (lower_only && i0 + MC <= j0) continue;  // strictly above diagonal
            tiles.push_back({i0, j0});
        }
    const double work = (double)m * (double)n * (double)k;
    int nt = threads;
    if (work < 4.0e6 || tiles.size() < 2) nt = 1;
    nt = std::max(1, std::min<int>(nt, (int)tiles.size()));
#pragma omp parallel num_threads(nt) if (nt > 1)
    {
        // packing buffers kept per thread (packing writes every entry it uses)
        static thread_local std::unique_ptr<double[]> Ap, Bp;
        if (!Ap) {
            Ap.reset(new double[(size_t)(MC * KC)]);
            Bp.reset(new double[(size_t)(NC * KC)]);
        }
#pragma omp for schedule(dynamic, 1)
        for (int64_t t = 0; t < (int64_t)tiles.size(); ++t) {
            int64_t i0 = tiles[t].i0, j0 = tiles[t].j0;
            int64_t mc = std::min(MC, m - i0), nc = std::min(NC, n - j0);
            gemm_tile(mc, nc, k, A + i0, lda, B + j0, ldb, C + i0 + j0 * ldc, ldc, Ap.get(), Bp.get());
        }
    }
}

namespace {

void trsm_base(int64_t m, int64_t n, const double* L, int64_t ldl, double* B, int64_t ldb) {
    for (int64_t j = 0; j < n; ++j) {
        double* bj = B + j * ldb;
        for (int64_t p = 0; p < j; ++p) {
            const double l = L[j + p * ldl];
            if (l == 0.0) continue;
            const double* bp = B + p * ldb;
            for (int64_t i = 0; i < m; ++i) bj[i] -= bp[i] * l;
        }
        const double d = L[j + j * ldl];
        for (int64_t i = 0; i < m; ++i) bj[i] /= d;
    }
}

void trsm_rec(int64_t m, int64_t n, const double* L, int64_t ldl, double* B, int64_t ldb,
              int threads) {
    if (n <= 32) {
        trsm_base(m, n, L, ldl, B, ldb);
        return;
    }
    int64_t n1 = (n / 2 + 7) / 8 * 8;
    if (n1 >= n) n1 = n / 2;
    int64_t n2 = n - n1;
    trsm_rec(m, n1, L, ldl, B, ldb, threads);
    // B2 -= B1 * L21^T  (L21 is n2 x n1 at L[n1, 0])
    gemm_nt_sub(m, n2, n1, B, ldb, L + n1, ldl, B + n1 * ldb, ldb, false, threads);
    trsm_rec(m, n2, L + n1 + n1 * ldl, ldl, B + n1 * ldb, ldb, threads);
}

}  // namespace

void trsm_right_lower_t(int64_t m, int64_t n, const double* L, int64_t ldl, double* B, int64_t ldb,
                        int threads) {
    if (m <= 0 || n <= 0) return;
    // Large solves: blocks of kCols columns, left to right. Each block of B is
    // solved against its diagonal block of L (rows independent, in fixed
    // 64-row pieces), then the columns to its right are updated by one large
    // GEMM, which spreads well over threads. The blocking depends on the sizes
    // only, so the results do not depend on the thread count.
    constexpr int64_t kCols = 256;
    if (n > 2 * kCols && (double)m * (double)n * (double)n > 6.4e7) {
        for (int64_t j0 = 0; j0 < n; j0 += kCols) {
            const int64_t nb = std::min(kCols, n - j0);
            trsm_right_lower_t(m, nb, L + j0 + j0 * ldl, ldl, B + j0 * ldb, ldb, threads);
            if (j0 + nb < n)
                gemm_nt_sub(m, n - j0 - nb, nb, B + j0 * ldb, ldb, L + (j0 + nb) + j0 * ldl, ldl,
                            B + (j0 + nb) * ldb, ldb, false, threads);
        }
        return;
    }
    // Rows of B are independent: solve them in fixed blocks of kRows rows
    // (a multiple of the micro-kernel's MR), spread over threads when large.
    // The blocks do not depend on the thread count, and neither do the results.
    constexpr int64_t kRows = 64;
    const int64_t chunks = (m + kRows - 1) / kRows;
    const double work = (double)m * (double)n * (double)n;
    const int nt = (threads > 1 && work > 8.0e6) ? (int)std::min<int64_t>(threads, chunks) : 1;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1) if (nt > 1)
    for (int64_t c = 0; c < chunks; ++c) {
        const int64_t r0 = c * kRows;
        trsm_rec(std::min(kRows, m - r0), n, L, ldl, B + r0, ldb, 1);
    }
}

int64_t potrf_lower(int64_t n, double* A, int64_t lda, int threads) {
    if (n <= 0) return -1;
    if (n <= 48) {
        for (int64_t j = 0; j < n; ++j) {
            double* aj = A + j * lda;
            for (int64_t p = 0; p < j; ++p) {
                const double l = A[j + p * lda];
                if (l == 0.0) continue;
                const double* ap = A + p * lda;
                for (int64_t i = j; i < n; ++i) aj[i] -= ap[i] * l;
            }
            const double d = aj[j];
            if (!(d > 0.0) || !std::isfinite(d)) return j;
            const double s = std::sqrt(d);
            aj[j] = s;
            for (int64_t i = j + 1; i < n; ++i) aj[i] /= s;
        }
        return -1;
    }
    int64_t n1 = (n / 2 + 7) / 8 * 8;
    if (n1 >= n) n1 = n / 2;
    int64_t n2 = n - n1;
    int64_t bad = potrf_lower(n1, A, lda, threads);
    if (bad >= 0) return bad;
    double* A21 = A + n1;
    double* A22 = A + n1 + n1 * lda;
    trsm_right_lower_t(n2, n1, A, lda, A21, lda, threads);
    gemm_nt_sub(n2, n2, n1, A21, lda, A21, lda, A22, lda, true, threads);
    bad = potrf_lower(n2, A22, lda, threads);
    return bad >= 0 ? bad + n1 : -1;
}

}  // namespace dense
}  // namespace gbchol
