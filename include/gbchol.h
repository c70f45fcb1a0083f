/*
 * gbchol: GB300-native (sm_103a) sparse Cholesky solve path, C ABI.
 *
 * This is the drop-in boundary for the GPU solve path of cholespy
 * (rgl-epfl/cholespy v2.2.2). Every entry point takes plain pointers and
 * sizes; the Python edge (cholespy_gb300/_ffi.py) binds them with ctypes, and
 * any other host language can bind them the same way.
 *
 * Conventions
 *   - Every function returns a gbchol_status (0 = success). On failure the
 *     message is available from gbchol_last_error() (thread-local).
 *   - Device pointers are CUDA device (or managed) addresses on the device the
 *     solver was created on. "stream" is a cudaStream_t (NULL = legacy
 *     default stream, like the reference's stream 0).
 *   - Right-hand sides are row-major (n, nrhs) arrays: element (i, k) at
 *     i * nrhs + k (reference kernels/kernels.cu:87,114,120,189).
 *   - A solver is not thread-safe: calls on one handle must be serialised,
 *     and solves on one handle must not overlap on the GPU (they share the
 *     handle's scratch), like the reference (src/cholesky_solver.h:88-98).
 */
#ifndef GBCHOL_H
#define GBCHOL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbchol_solver* gbchol_handle;

typedef enum {
    GBCHOL_OK = 0,
    GBCHOL_EINVAL = 1,      /* invalid argument (Python: ValueError) */
    GBCHOL_ENOTPOSDEF = 2,  /* not positive definite (Python: ValueError) */
    GBCHOL_ECUDA = 3,       /* CUDA error (Python: RuntimeError) */
    GBCHOL_ENOMEM = 4,      /* allocation failure (Python: RuntimeError) */
    GBCHOL_ETIMEOUT = 5,    /* a bounded device-side wait expired (Python: RuntimeError) */
    GBCHOL_ESTATE = 6,      /* call not valid for this handle (Python: RuntimeError) */
    GBCHOL_EINTERNAL = 7
} gbchol_status;

/* Matrix formats: same values as cholespy.MatrixType (src/cholesky_solver.h:8-12). */
enum { GBCHOL_CSC = 0, GBCHOL_CSR = 1, GBCHOL_COO = 2 };

/* Storage flags for gbchol_create: which copies the solver keeps on the GPU. */
enum {
    GBCHOL_STORE_F32 = 1, /* FP32 factor: CholeskySolverF solves, and the inner solve of refinement */
    GBCHOL_STORE_F64 = 2, /* FP64 factor: plain CholeskySolverD solves */
    GBCHOL_STORE_A64 = 4  /* FP64 copy of A: residuals for refinement and the gradient pattern */
};

/* Maximum RHS count of one solve (src/cholesky_solver.cpp:418-420). */
#define GBCHOL_MAX_RHS 128

/* Message of the last failed call on this thread ("" if none). */
const char* gbchol_last_error(void);

/* Library version string. */
const char* gbchol_version(void);

/*
 * Factor A on the host and analyse the factor on the current CUDA device.
 * Replaces CholeskySolver<Float>::CholeskySolver (src/cholesky_solver.cpp:152-198)
 * with cpu = false, including factorize (:200-297) and both analyze_cuda
 * calls (:299-376). ii/jj/x are HOST arrays with the meaning of the
 * reference constructor (src/main.cpp:21-26): COO rows/cols, or CSR row
 * pointers/cols, or CSC col pointers/rows; x is always float64. Only the lower
 * triangle (row >= col) of A is used, as CHOLMOD does with stype = -1.
 * `store` is a mask of GBCHOL_STORE_* flags.
 */
int gbchol_create(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj,
                  const double* x, int32_t matrix_type, int32_t store, gbchol_handle* out);

/*
 * gbchol_create for inputs that already live on the current CUDA device
 * (ii, jj, x device pointers, same meaning as gbchol_create): the COO / CSR /
 * CSC -> sorted, duplicate-summed CSC conversion runs on the GPU (equal, bit
 * for bit, to gbchol_create's host conversion), then the CSC goes to the host
 * for the factorisation. The reference instead copies device inputs to the
 * host and converts them there (src/main.cpp:47-67,
 * src/cholesky_solver.cpp:8-149).
 */
int gbchol_create_device(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                         int32_t matrix_type, int32_t store, gbchol_handle* out);

/*
 * Analyse an existing factor (the hot-path boundary proper): perm[k] is the
 * original row at position k (CHOLMOD Perm), L is given in CSC with sorted
 * rows and the diagonal first in each column (cholmod_factor_to_sparse,
 * src/cholesky_solver.cpp:247-252). Uploads L and L^T and runs the level
 * analysis of both (analyze_cuda, src/cholesky_solver.cpp:299-376). Host
 * arrays. A is not known, so refinement and gradients are unavailable.
 */
int gbchol_create_from_factor(int32_t n, const int32_t* perm, const int32_t* colptr,
                              const int32_t* rowidx, const double* vals, int32_t store,
                              gbchol_handle* out);

/*
 * Host-only ordering + numeric LL^T (no GPU use): the replacement of
 * cholmod_analyze + cholmod_factorize with the reference's settings
 * (simplicial LL^T, nested dissection; src/cholesky_solver.cpp:200-243),
 * preceded by the input preparation of src/cholesky_solver.cpp:152-179.
 * threads = 0 uses every host core. Fails with GBCHOL_ENOTPOSDEF and
 * "Matrix is not positive definite!" like src/cholesky_solver.cpp:241-242.
 */
typedef struct gbchol_host_factor* gbchol_factor_handle;

int gbchol_factorize(int32_t n_rows, int64_t nnz, const int32_t* ii, const int32_t* jj,
                     const double* x, int32_t matrix_type, int32_t threads,
                     gbchol_factor_handle* out);

/* Sizes of a host factor: n, nnz(L), number of fundamental supernodes, flops. */
int gbchol_factor_info(gbchol_factor_handle f, int32_t* n, int64_t* nnz_l, int32_t* n_supernodes,
                       double* flops);

/* Copy a host factor out (CSC, diagonal first); any pointer may be NULL. */
int gbchol_factor_export(gbchol_factor_handle f, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                         double* vals);

int gbchol_factor_free(gbchol_factor_handle f);

/*
 * Numeric refactorisation of a host factor: new values for the same
 * sparsity pattern (n as before; any input format, duplicates summed). The
 * factor's ordering is reused (no new ordering); GBCHOL_EINVAL if the new
 * pattern gives another factor pattern, GBCHOL_ENOTPOSDEF if the new matrix
 * is not positive definite (the factor keeps its old values on any error).
 * With the very index arrays and format the factor was made from, the kept
 * symbolic analysis is reused and only the numeric phase runs (same result).
 * No counterpart in the reference (it refactors through a new solver).
 */
int gbchol_factor_refactorize(gbchol_factor_handle f, int64_t nnz, const int32_t* ii, const int32_t* jj,
                              const double* x, int32_t matrix_type, int32_t threads);

/*
 * x = A^{-1} b on HOST arrays with a host factor: the solve of solvers built
 * from CPU arrays. Replaces CholeskySolver<Float>::solve_cpu
 * (src/cholesky_solver.cpp:435-463), i.e. cholmod_solve(CHOLMOD_A) on the
 * reference's CPU-side factor (src/main.cpp:68-70, 83-91): b is read as FP64,
 * the solve runs in FP64 on the factor's values and x is rounded to the
 * arrays' type. precision 0 = float b/x, 1 = double b/x; row-major (n, nrhs);
 * any nrhs >= 0 (the reference's CPU path has no 128 limit); b and x may
 * alias. threads = 0 uses every host core; the result does not depend on the
 * thread count. The first call builds the solve's structure (kept until the
 * factor is freed; a refactorisation keeps it). Blocks until x is written.
 * Solves only read the factor, so several threads may solve with one factor
 * at once; a refactorisation must not overlap them.
 * This path never runs for CUDA arrays: those go through gbchol_solve.
 */
int gbchol_factor_solve(gbchol_factor_handle f, int32_t precision, int32_t nrhs, const void* b, void* x,
                        int32_t threads);

/* Free every device and host buffer of the solver (src/cholesky_solver.cpp:465-486). */
int gbchol_destroy(gbchol_handle h);

/*
 * x = A^{-1} b for nrhs right-hand sides, asynchronously on `stream`.
 * Replaces CholeskySolver<Float>::solve_cuda (src/cholesky_solver.cpp:415-432):
 * lower sweep tmp = L^{-1} b[perm], upper sweep x[perm] = L^{-T} tmp.
 * precision: 0 = FP32 (float b/x), 1 = FP64 (double b/x). b and x are device
 * pointers and may alias. nrhs outside 1..128 fails with GBCHOL_EINVAL and the
 * reference's message "The number of RHS should be less than 128.".
 */
int gbchol_solve(gbchol_handle h, int32_t precision, int32_t nrhs, const void* b, void* x,
                 void* stream);

/*
 * gbchol_solve for callers that cannot allocate GPU memory while solving:
 * real-time loops whose device memory is fixed up front, or hosts whose
 * allocator owns all device memory (a framework's caching allocator, a pool
 * the solver may not bypass). gbchol_solve may grow the solver's work array with cudaMalloc when
 * a call brings more RHS than any before; this call allocates nothing. Its
 * work array is a fixed 16 MiB file-scope device array that every GPU
 * loading the library holds until exit, so it fails with GBCHOL_EINVAL when
 * the solve's work array exceeds 16 MiB: n * nrhs * element size (4 bytes
 * FP32, 8 FP64), plus 32 * nrhs * element size (rounded up to the RHS slice
 * width) per partial sum of the supernodal lower sweep. The first
 * call on a device looks up the array's device address; make it before any
 * stream capture. The address is cached for the life of the process's
 * context on that device (no calls after cudaDeviceReset). All calls share the array, so calls that overlap on the
 * GPU race: serialise them. Same arguments and results as gbchol_solve.
 * No counterpart in the reference.
 */
int gbchol_solve_noalloc(gbchol_handle h, int32_t precision, int32_t nrhs, const void* b, void* x,
                         void* stream);

/* Statistics of one refined solve. */
typedef struct {
    int32_t iterations;       /* refinement steps taken (0 = FP32 solve was enough) */
    int32_t converged;        /* 1 if max relative residual <= tol */
    double max_rel_residual;  /* max over RHS of ||b - A x||_2 / ||b||_2 */
} gbchol_refine_stats;

/*
 * FP32-factor solve with FP64-residual iterative refinement: x0 = A32^{-1} b,
 * then r = b - A x in FP64 on the original A, d = A32^{-1} r, x += d (FP64),
 * until max_k ||r_k||/||b_k|| <= tol or max_iter steps. b, x: FP64 device
 * arrays (n, nrhs), may not alias. Needs GBCHOL_STORE_F32 | GBCHOL_STORE_A64.
 * The loop runs without host synchronisation (a device flag ends it); when
 * `stats` is non-NULL the call synchronises `stream` to fill it.
 * No counterpart in the reference.
 */
int gbchol_solve_refined(gbchol_handle h, int32_t nrhs, const double* b, double* x, double tol,
                         int32_t max_iter, void* stream, gbchol_refine_stats* stats);

/*
 * Gradient of a loss with respect to the stored entries of A, given the
 * backward-solve result grad_b = A^{-1} grad_x and the solution x (device
 * arrays (n, nrhs), FP32 if precision = 0 else FP64). rows/cols: device
 * arrays of the nnz entries' (row, col) in the original ordering. Writes
 * grad_vals (FP32 if out_precision = 0 else FP64), one value per entry:
 *   symmetric = 1: dL/dA of the symmetric matrix, -1/2 (gb_r x_c + gb_c x_r)
 *                  on off-diagonal entries, -gb_r x_r on the diagonal;
 *   symmetric = 0: the exact gradient of the lower-triangle-only forward
 *                  (entries above the diagonal get 0, below -(gb_r x_c + gb_c x_r)).
 * Sums over the RHS columns. No counterpart in the reference.
 */
int gbchol_grad_values(int32_t precision, int64_t nnz, int32_t nrhs, const int32_t* rows,
                       const int32_t* cols, const void* grad_b, const void* x, void* grad_vals,
                       int32_t out_precision, int32_t symmetric, void* stream);

/*
 * Failure-detection self-test: one device-side wait, bounded by `wait_us`
 * microseconds (1..2e6), on a flag that nothing sets. Stores the status word
 * the wait left (GBCHOL_ETIMEOUT expected) in *status_out; the context stays
 * usable. Every sync-free kernel uses the same bounded wait. No counterpart in
 * the reference (its waits are unbounded, kernels/kernels.cu:20-21).
 */
int gbchol_selftest_wait(int32_t wait_us, int32_t* status_out);

/* Solver facts. */
typedef struct {
    int32_t n;
    int32_t device;
    int64_t nnz_a;            /* nnz of the symmetric A kept (0 if not kept) */
    int64_t nnz_l;            /* nnz of L (diagonal included) */
    int32_t levels_lower;     /* number of levels of L   (max_lvl + 1) */
    int32_t levels_upper;     /* number of levels of L^T (max_lvl + 1) */
    int32_t n_supernodes;
    int32_t max_supernode;
    double factor_flops;
    double factor_seconds;    /* host factorisation time */
    double analysis_seconds;  /* device analysis time incl. uploads */
    int32_t store;
    int32_t top_rows;         /* rows solved by the supernodal kernels */
    int32_t top_units;        /* supernodal work units (<= 32 columns each) */
    int64_t top_blocks;       /* dense contribution blocks of the lower sweep */
    int32_t launches_per_solve;  /* kernel launches of one gbchol_solve */
} gbchol_info;

int gbchol_get_info(gbchol_handle h, gbchol_info* out);

/*
 * Copy the analysis results to host arrays of size n: row_levels[i] is the
 * level of row i and order[] the rows sorted by (level, row), which is the
 * `levels` array of the reference (src/cholesky_solver.cpp:315-367).
 * lower = 1 for L, 0 for L^T. max_lvl may be NULL.
 */
int gbchol_get_levels(gbchol_handle h, int32_t lower, int32_t* row_levels, int32_t* order,
                      int32_t* max_lvl);

/*
 * Copy the factor to host arrays: perm (n), colptr (n+1), rowidx and vals
 * (nnz_l), CSC with the diagonal first. Any pointer may be NULL.
 */
int gbchol_get_factor(gbchol_handle h, int32_t* perm, int32_t* colptr, int32_t* rowidx,
                      double* vals);

/*
 * Synchronise the solver's last stream and report the device-side status
 * word: GBCHOL_ETIMEOUT if a bounded wait expired in an earlier solve (the
 * word is then cleared).
 */
int gbchol_check(gbchol_handle h);

/*
 * Preallocate scratch for solves of up to nrhs right-hand sides so that later
 * solves allocate nothing (needed before capturing solves in a CUDA graph).
 */
int gbchol_reserve(gbchol_handle h, int32_t nrhs);

/*
 * Rebuild the solve plan with other tuning parameters: supernodes at least
 * min_top_width columns wide (and their ancestors) form the supernodal top
 * region (default 8); lower-sweep contribution lists longer than
 * part_keep + part_group keep their last part_keep blocks and hand the rest
 * to partial sums of about part_group blocks (defaults 16 and 0; 0: no
 * partial sums).
 * Results change only by rounding. Synchronises the device. A batch built
 * from this solver before the call refuses to solve (GBCHOL_ESTATE): build it
 * again. No counterpart in the reference.
 */
int gbchol_replan(gbchol_handle h, int32_t min_top_width, int32_t part_keep, int32_t part_group);

/*
 * Autotuner: for each of the `count` candidate widths, rebuild the plan with
 * that min_top_width (gbchol_replan, keeping the partial-sum settings), time
 * `reps` solves of nrhs right-hand sides in the given precision (0 FP32,
 * 1 FP64) after two warm-up solves, and keep the fastest plan; the chosen
 * width is written to *chosen (may be NULL). Allocates and frees its own
 * buffers and stream. No counterpart in the reference.
 */
int gbchol_autotune(gbchol_handle h, int32_t precision, int32_t nrhs, const int32_t* candidates, int32_t count,
                    int32_t reps, int32_t* chosen);

/*
 * Times the sweep variants on this solver's current plan for `nrhs` RHS of
 * the given precision (`reps` timed solves each, after two untimed ones)
 * and keeps the fastest for later solves of that RHS count: the
 * top-region kernel (0: 32-column RHS slices, 1: one work item per unit for
 * every RHS column, CUDA cores, 2: the same on the tensor cores, 3 / 4: one
 * work item per unit and column half / quarter (the RHS tile width); 1-4 only
 * for FP32 and 4..128 RHS in multiples of 4, 3 and 4 when the columns split
 * into multiples of 4), for <= 8 RHS whether
 * the row sweeps put their lanes over the RHS columns instead of the
 * nonzeros (threads per column), and the rows each row-sweep ticket takes
 * (1, 2 or 4: how many consecutive level-ordered rows are merged into one
 * task). *choice = kernel | rhs_split << 4 | rows_per_ticket << 8.
 * Allocates scratch and synchronises. No counterpart in the reference (its
 * launch shape is fixed, src/cholesky_solver.cpp:378-413).
 */
int gbchol_autotune_sweeps(gbchol_handle h, int32_t precision, int32_t nrhs, int32_t reps, int32_t* choice);

/*
 * Numeric refactorisation of a solver: new values of the same sparsity
 * pattern (same n and input format as at creation). Keeps the ordering, the
 * symbolic factor and the level analysis; recomputes the numeric factor on the
 * host (reusing the ordering, and the whole symbolic analysis when the index
 * arrays are those of the constructor) and uploads it with the solve plan.
 * Errors as gbchol_factor_refactorize; the solver keeps its old factor on any error.
 * Synchronises the device; batches built from this solver must be built
 * again. No counterpart in the reference, whose users build a new solver per
 * set of values.
 */
int gbchol_refactorize(gbchol_handle h, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                       int32_t matrix_type);

/*
 * Batched solves: `count` solvers (same device) solved together, system s
 * with nrhs[s] right-hand sides, by one persistent launch per sweep phase.
 * precision 0 = FP32, 1 = FP64 (every solver must keep that factor). The
 * solvers must outlive the batch. The batch owns its scratch, so a bound
 * batch solve allocates nothing and synchronises nothing: it can be
 * captured in a CUDA graph and replayed. No counterpart in the reference.
 */
typedef struct gbchol_batch_s* gbchol_batch;

int gbchol_batch_create(int32_t count, const gbchol_handle* solvers, const int32_t* nrhs,
                        int32_t precision, gbchol_batch* out);

/*
 * Schedule of a batch's row sweeps. Consecutive systems whose work arrays
 * (n_s x nrhs[s] values) fit group_bytes form a group, and group g's tasks
 * are ticketed `skew` dependency levels after group g - 1's (a wavefront: the
 * x values a leaf row gathers were written recently and are still in L2;
 * skew 0 runs the groups one after another). row_variant 1 uses two lane
 * modes (lanes over the nonzeros up to 8 RHS, over the RHS columns above);
 * 2 fits the mode to each system's RHS count. gbchol_batch_create uses
 * group_bytes = 8 MiB, skew = 4, row_variant = 2 (the 256-system benchmark
 * batch on GB300: 19.5 ms per batch with one group and two modes, 16.4 ms
 * with these), unless GBCHOL_BATCH_GROUP_MB, GBCHOL_BATCH_SKEW or
 * GBCHOL_BATCH_ROW_VARIANT say otherwise.
 */
typedef struct {
    int64_t group_bytes;  /* <= 0: one group */
    int32_t skew;         /* >= 0 */
    int32_t row_variant;  /* 1 or 2 */
} gbchol_batch_options;

int gbchol_batch_create_ex(int32_t count, const gbchol_handle* solvers, const int32_t* nrhs,
                           int32_t precision, const gbchol_batch_options* options, gbchol_batch* out);

/* Bind the device arrays of every system: bs[s], xs[s] are (n_s, nrhs[s]). */
int gbchol_batch_set_io(gbchol_batch b, const void* const* bs, void* const* xs);

/* x_s = A_s^{-1} b_s for every system, asynchronously on `stream`. */
int gbchol_batch_solve(gbchol_batch b, void* stream);

/* Kernel launches per batched solve, total nnz(L) and rows of the batch. */
int gbchol_batch_info(gbchol_batch b, int32_t* launches, int64_t* nnz_l, int64_t* rows);

/* Synchronise `stream` and report an expired device-side wait (GBCHOL_ETIMEOUT). */
int gbchol_batch_check(gbchol_batch b, void* stream);

int gbchol_batch_destroy(gbchol_batch b);

#ifdef __cplusplus
}
#endif

#endif /* GBCHOL_H */
