// Dense FP64 kernels for the host multifrontal factorisation (column-major).
#pragma once
#include <cstdint>

namespace gbchol {
namespace dense {

// C[m x n] -= A[m x k] * B[n x k]^T. If lower_only, blocks of C strictly
// above the diagonal are skipped (SYRK use, A == B). `threads` <= 1 runs
// serially.
void gemm_nt_sub(int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                 int64_t ldb, double* C, int64_t ldc, bool lower_only, int threads);

// B[m x n] <- B * L^{-T}, L lower triangular n x n (diagonal used).
void trsm_right_lower_t(int64_t m, int64_t n, const double* L, int64_t ldl, double* B, int64_t ldb,
                        int threads);

// In-place lower Cholesky of A[n x n]. Returns the index of the first
// non-positive pivot, or -1 on success.
int64_t potrf_lower(int64_t n, double* A, int64_t lda, int threads);

}  // namespace dense
}  // namespace gbchol
