// Host-side sparse preparation, fill-reducing ordering and numeric LL^T
// factorisation. These stand in for the reference's host pipeline:
//   - COO/CSR/CSC -> sorted, duplicate-free CSC   (src/cholesky_solver.cpp:8-149)
//   - CHOLMOD simplicial LL^T with nested-dissection ordering
//     (src/cholesky_solver.cpp:200-297; CHOLMOD itself is an absent submodule)
// The output of factorize() is what the reference hands to its GPU code:
// the permutation Perm and the factor L in CSC form with sorted row indices and
// the diagonal first in each column (cholmod_factor_to_sparse).
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace gbchol {

enum MatrixFormat : int32_t { FMT_CSC = 0, FMT_CSR = 1, FMT_COO = 2 };

// Status codes shared with the C ABI (include/gbchol.h).
enum Status : int32_t {
    ST_OK = 0,
    ST_INVALID = 1,      // bad argument: maps to ValueError
    ST_NOT_POSDEF = 2,   // factorisation hit a non-positive pivot: ValueError
    ST_CUDA = 3,         // CUDA runtime error: RuntimeError
    ST_NOMEM = 4,        // allocation failure: RuntimeError
    ST_TIMEOUT = 5,      // a device-side wait ran out of budget: RuntimeError
    ST_STATE = 6,        // call not valid for this handle: RuntimeError
    ST_INTERNAL = 7,
};

struct Csc {
    int32_t n = 0;
    std::vector<int32_t> colptr;  // n+1
    std::vector<int32_t> rowidx;  // nnz, sorted within each column
    std::vector<double> vals;     // nnz
    int64_t nnz() const { return (int64_t)rowidx.size(); }
};

// Builds a CSC matrix with row indices sorted inside each column and
// duplicate entries summed (duplicates summed in input order). Validates all
// indices. Follows coo_to_csc / csr_to_csc / csc_sort_indices /
// csc_sum_duplicates (src/cholesky_solver.cpp:8-149).
Status build_csc(int32_t n, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                 int32_t fmt, Csc& out, std::string& err);

// Full symmetric matrix (both triangles, CSR == CSC since symmetric) built
// from the lower triangle of A (row >= col), which is the only part CHOLMOD
// reads for stype = -1 (src/cholesky_solver.cpp:211-220). Used by iterative
// refinement (residual b - A x) and by the gradient.
void symmetric_from_lower(const Csc& A, Csc& S);

// Nested-dissection fill-reducing ordering of the symmetric graph given in
// CSR adjacency form (no self loops). Returns perm with perm[k] = original
// vertex placed at position k (CHOLMOD Perm convention).
std::vector<int32_t> nested_dissection(int32_t n, const std::vector<int32_t>& xadj,
                                       const std::vector<int32_t>& adj);

// Symbolic analysis of a factorisation, kept so that new values on the same
// sparsity pattern are factorised without ordering, symbolic factorisation or
// input sorting again (numeric refactorisation).
struct SymbolicCache {
    int32_t n = 0;
    std::vector<int32_t> a_colptr, a_rowidx;  // A's CSC pattern (sorted, duplicates merged)
    std::vector<int32_t> amap;                // A's CSC entry -> position in the permuted lower CSC (-1: upper)
    std::vector<int32_t> cptr, crow;          // lower CSC of P A P^T (pattern)
    std::vector<int32_t> sn_parent, child_ptr, children;  // supernodal elimination tree
    // fronts of the numeric phase (relaxed amalgamation): chains of
    // supernodes, each the last child of the next, merged into one front with
    // explicit zeros; front f has columns [fr_col[f], fr_col[f+1]) and below
    // them the fr_nr[f] rows rowidx[fr_rpos[f]...] of its top supernode. L
    // keeps its own (simplicial) pattern.
    std::vector<int32_t> fr_col, fr_nr, fr_parent, fr_child_ptr, fr_children;
    std::vector<int64_t> fr_rpos;
    // the raw input the analysis was made for (empty if not recorded):
    int32_t fmt = -1;
    std::vector<int32_t> in_i, in_j;  // index arrays as given
    std::vector<int32_t> inmap;       // input entry -> position in A's CSC
};

struct Factor {
    int32_t n = 0;
    std::vector<int32_t> perm;    // perm[k] = original row at position k
    std::vector<int32_t> colptr;  // CSC of L: n+1
    std::vector<int32_t> rowidx;  // rows sorted, diagonal first
    std::vector<double> vals;
    std::vector<int32_t> parent;  // elimination tree of P A P^T (-1 = root)
    std::vector<int32_t> sn_start;// fundamental supernodes: columns [sn_start[s], sn_start[s+1])
    double flops = 0.0;           // numeric factorisation flop count
    std::shared_ptr<SymbolicCache> sym;  // set by factorize()
    int64_t nnz() const { return (int64_t)rowidx.size(); }
};

struct FactorOptions {
    int32_t threads = 0;          // 0 = all available
    bool use_given_perm = false;  // take perm from `perm_in` instead of ordering
    const int32_t* perm_in = nullptr;
};

// Symbolic + numeric LL^T of P A P^T, A given by its lower triangle (row >=
// col entries of `A`; the upper part is ignored like CHOLMOD stype = -1).
// Ordering: nested dissection followed by an elimination-tree postorder.
// Numeric: supernodal multifrontal with dense blocked kernels. Returns
// ST_NOT_POSDEF on a non-positive pivot (src/cholesky_solver.cpp:241-242).
Status factorize(const Csc& A, const FactorOptions& opt, Factor& F, std::string& err);

// Numeric phase of factorize on its symbolic analysis: cval holds the values
// of the lower CSC of P A P^T (pattern S.cptr / S.crow); the values of L go to
// vals_out (F's pattern). ST_NOT_POSDEF on a non-positive pivot.
Status numeric_factor(const Factor& F, const SymbolicCache& S, const std::vector<double>& cval, int32_t threads,
                      std::vector<double>& vals_out, double& flops_out, std::string& err);

// Records in F's symbolic analysis the raw input it was made from (index
// arrays and format, as given to build_csc), so that refactor_cached can
// recognise the same input pattern.
void record_input(Factor& F, int64_t nnz, const int32_t* ii, const int32_t* jj, int32_t fmt);

// Numeric refactorisation of F for new values x of the recorded input
// pattern: the duplicates are summed in input order exactly as build_csc does,
// the values are placed by the cached maps and factorised by numeric_factor.
// Returns false (nothing done) when F has no recorded input or the given
// index arrays / format differ from it. On true, `st` is the numeric status,
// A the matrix with the new values (CSC, as build_csc gives it) and vals_out /
// flops_out the new factor values.
bool refactor_cached(const Factor& F, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                     int32_t fmt, int32_t threads, Csc& A, std::vector<double>& vals_out, double& flops_out,
                     Status& st, std::string& err);

// Transpose of a CSC pattern+values (gives the CSR of L from its CSC); with
// empty `vals`, of the pattern alone. Indices ascend within each output row.
void transpose(int32_t n, const std::vector<int32_t>& colptr, const std::vector<int32_t>& rowidx,
               const std::vector<double>& vals, std::vector<int32_t>& tptr,
               std::vector<int32_t>& tidx, std::vector<double>& tvals);
// The same restricted to the columns c with keep_col[c] != 0 (all columns if
// keep_col is null); vals may be null (pattern only). Multi-threaded for
// large inputs, with results independent of the thread count.
void transpose_columns(int32_t n, const std::vector<int32_t>& colptr, const std::vector<int32_t>& rowidx,
                       const double* vals, const char* keep_col, std::vector<int32_t>& tptr,
                       std::vector<int32_t>& tidx, std::vector<double>& tvals);

// Structure of the host solve of a factor (cpu_solve.cpp), built once per
// factor pattern: it holds positions into the factor's arrays, not values, so
// a numeric refactorisation of the same pattern keeps it valid.
struct CpuSolvePlan {
    int32_t n = 0;
    std::vector<int32_t> sn_start;    // supernodes: columns [sn_start[s], sn_start[s+1])
    std::vector<int32_t> task_first;  // subtree tasks: supernodes [task_first[t], task_last[t]]
    std::vector<int32_t> task_last;
    std::vector<int64_t> task_cost;   // nnz(L) of a task's columns (tasks sorted by it, descending)
    std::vector<int32_t> top_sn;      // supernodes outside every task, ascending
    std::vector<int32_t> top_rows;    // their columns, ascending
    std::vector<int64_t> pt_ptr;      // per top row: its entries L(i, j) in task columns j
    std::vector<int32_t> pt_col;
    std::vector<int64_t> pt_pos;      // position of L(i, j) in rowidx / vals
    int32_t max_nr = 0;               // most off-diagonal rows of one supernode
};

void cpu_plan(const Factor& F, CpuSolvePlan& P, int32_t threads);

// Host solve x = P^T L^-T L^-1 P b in FP64 (the CPU-array solve of the
// reference, src/cholesky_solver.cpp:435-463). b and x are row-major
// (n, nrhs) arrays of float (precision 0) or double (1), read and rounded like
// the reference's copies in and out; they may alias. threads = 0 uses every
// host core; the result does not depend on the thread count.
void cpu_solve(const Factor& F, const CpuSolvePlan& P, int32_t precision, int32_t nrhs, const void* b, void* x,
               int32_t threads);

}  // namespace gbchol
