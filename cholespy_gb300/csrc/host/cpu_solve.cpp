// Solve on host arrays with a host factor: the path of solvers built from CPU
// arrays. Counterpart of the reference's CholeskySolver<Float>::solve_cpu
// (src/cholesky_solver.cpp:435-463): there b is copied into an FP64
// column-major array, cholmod_solve(CHOLMOD_A) computes x = P^T L^-T L^-1 P b
// on the simplicial LL^T factor, and x is rounded to the caller's type.
//
// The same FP64 arithmetic runs here as a supernodal, panel-blocked solve:
//   * supernodes: runs of consecutive columns whose patterns nest (column
//     j+1 = column j without row j), so that all columns of one supernode
//     share their rows below it; the values stay in the factor's CSC arrays,
//     where a supernode is a column-major trapezoid;
//   * the elimination tree is cut into subtree tasks (a task's columns form
//     a contiguous range of the postordered factor) and a top region (the
//     supernodes whose subtree holds more than 1/256 of nnz(L), plus their
//     ancestors);
//   * forward sweep: tasks in parallel, each scattering only into rows of its
//     own subtree; then every top row gathers the entries of its row of L
//     that lie in task columns (a row list built once per factor); then the
//     top supernodes in column order, each in panels of 64 columns: the
//     panel's triangular solve, then the update of every row below the panel
//     (intra-supernode rows and off-diagonal rows alike), in blocks of rows;
//   * backward sweep: the top supernodes in reverse (each column's dot
//     product with the rows below it, blocks of columns in parallel; then the
//     panels' triangles in reverse), then the tasks in parallel (they read
//     only finished ancestors);
//   * one-column supernodes (most of a mesh factor's) update rows directly
//     and take their backward dot product in place;
//   * right-hand sides in chunks of 16 (then 8, 4, 2, 1), each packed
//     row-major; the parallel phases run over (task or row block, chunk).
// Every value is summed in an order fixed by the factor and the RHS count, so
// results do not depend on the thread count.
#include <algorithm>
#include <cstring>
#include <memory>
#include <type_traits>

#include "host.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace gbchol {

namespace {

constexpr int32_t PB = 64;   // panel width of the blocked triangular solves
constexpr int32_t QB = 1024;  // rows per block of a panel's update
constexpr int32_t JB = 16;   // columns per block of a backward dot product
constexpr int WMAX = 16;     // widest RHS chunk

int host_threads(int32_t t) {
    if (t > 0) return t;
#ifdef _OPENMP
    return std::max(1, omp_get_max_threads());
#else
    return 1;
#endif
}

int thread_id() {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

struct Fac {
    const int32_t* cp;  // colptr
    const int32_t* ri;  // rowidx
    const double* v;    // values
};

// Chunk rows of W doubles (W even) as W/2 pairs in GCC vector types (SSE2 /
// NEON registers on both host architectures; no ISA-specific code). Written
// out so that the arithmetic runs along the RHS columns: left alone, the
// compiler's vectoriser paired values of different factor columns and reduced
// them with scalar adds, which ran at a third of this speed.
typedef double v2d __attribute__((vector_size(16)));

template <int W>
struct Row {
    v2d v[W / 2];
    static Row zero() {
        Row r;
        for (int c = 0; c < W / 2; ++c) r.v[c] = v2d{0.0, 0.0};
        return r;
    }
    static Row load(const double* p) {
        Row r;
        std::memcpy(r.v, p, sizeof(double) * W);
        return r;
    }
    void store(double* p) const { std::memcpy(p, v, sizeof(double) * W); }
    void add_scaled(double l, const double* y) {  // this += l * y
        const v2d s = {l, l};
        const Row yr = load(y);
        for (int c = 0; c < W / 2; ++c) v[c] += s * yr.v[c];
    }
    void sub_from(double* p) const {  // p -= this
        Row r = load(p);
        for (int c = 0; c < W / 2; ++c) r.v[c] -= v[c];
        r.store(p);
    }
    void sub_scaled_from(double* p, double l) const {  // p -= l * this
        const v2d s = {l, l};
        Row r = load(p);
        for (int c = 0; c < W / 2; ++c) r.v[c] -= s * v[c];
        r.store(p);
    }
};

// Column-block kernels on one RHS chunk Y (n rows of W doubles).
template <int W>
struct Kern {
    // Triangle of panel [p0, p1): y_j = y_j / L(j,j), then y_i -= L(i,j) y_j
    // for i in (j, p1).
    static void fwd_tri(const Fac& f, int32_t p0, int32_t p1, double* Y) {
        for (int32_t j = p0; j < p1; ++j) {
            const double* col = f.v + f.cp[j];
            double* yj = Y + (int64_t)j * W;
            const double d = col[0];
            if constexpr (W == 1) {
                yj[0] /= d;
                for (int32_t i = j + 1; i < p1; ++i) Y[i] -= col[i - j] * yj[0];
            } else {
                Row<W> y = Row<W>::load(yj);
                const v2d dv = {d, d};
                for (int c = 0; c < W / 2; ++c) y.v[c] /= dv;
                y.store(yj);
                for (int32_t i = j + 1; i < p1; ++i) y.sub_scaled_from(Y + (int64_t)i * W, col[i - j]);
            }
        }
    }

    // Rows q in [q0, q1) below panel [p0, p1) of a supernode ending at column
    // c1: below-row q is row p1 + q for q < c1 - p1, else R[q - (c1 - p1)],
    // and sits at offset (p1 - j) + q of column j. y_row -= sum_j L(row, j) y_j,
    // the sum taken over j ascending from zero into `acc`. One RHS: columns
    // outer, a vector update across rows; wider chunks: blocks of 8 columns,
    // rows outer (the same order of operations).
    static void fwd_rect(const Fac& f, const int32_t* R, int32_t c1, int32_t p0, int32_t p1, int32_t q0,
                         int32_t q1, double* Y, double* acc) {
        const int32_t nin = c1 - p1;
        const int32_t nq = q1 - q0;
        auto row_of = [&](int32_t qq) { return qq < nin ? p1 + qq : R[qq - nin]; };
        std::fill(acc, acc + (int64_t)nq * W, 0.0);
        if constexpr (W == 1) {
            for (int32_t j = p0; j < p1; ++j) {
                const double* lj = f.v + f.cp[j] + (p1 - j) + q0;
                const double yj = Y[j];
                for (int32_t q = 0; q < nq; ++q) acc[q] += lj[q] * yj;
            }
            for (int32_t q = 0; q < nq; ++q) Y[row_of(q0 + q)] -= acc[q];
        } else {
            for (int32_t kb = p0; kb < p1; kb += 8) {
                const int32_t nk = std::min(8, p1 - kb);
                const double* col[8];
                for (int32_t k = 0; k < nk; ++k) col[k] = f.v + f.cp[kb + k] + (p1 - kb - k) + q0;
                const double* yk = Y + (int64_t)kb * W;
                if (nk == 8) {
                    int32_t q = 0;
                    for (; q + 2 <= nq; q += 2) {  // two rows share each y load
                        Row<W> t0 = Row<W>::load(acc + (int64_t)q * W);
                        Row<W> t1 = Row<W>::load(acc + (int64_t)(q + 1) * W);
                        for (int k = 0; k < 8; ++k) {
                            const double l0 = col[k][q], l1 = col[k][q + 1];
                            const v2d s0 = {l0, l0}, s1 = {l1, l1};
                            const Row<W> y = Row<W>::load(yk + k * W);
                            for (int c = 0; c < W / 2; ++c) {
                                t0.v[c] += s0 * y.v[c];
                                t1.v[c] += s1 * y.v[c];
                            }
                        }
                        t0.store(acc + (int64_t)q * W);
                        t1.store(acc + (int64_t)(q + 1) * W);
                    }
                    for (; q < nq; ++q) {
                        Row<W> t = Row<W>::load(acc + (int64_t)q * W);
                        for (int k = 0; k < 8; ++k) t.add_scaled(col[k][q], yk + k * W);
                        t.store(acc + (int64_t)q * W);
                    }
                } else {
                    for (int32_t q = 0; q < nq; ++q) {
                        Row<W> t = Row<W>::load(acc + (int64_t)q * W);
                        for (int32_t k = 0; k < nk; ++k) t.add_scaled(col[k][q], yk + (int64_t)k * W);
                        t.store(acc + (int64_t)q * W);
                    }
                }
            }
            for (int32_t q = 0; q < nq; ++q) Row<W>::load(acc + (int64_t)q * W).sub_from(Y + (int64_t)row_of(q0 + q) * W);
        }
    }

    // y_j -= sum_{q < m} L(below q, j) z_q for j in [j0, j1), where below-row
    // q of column j sits at offset (base - j) + q. The sum over q is split
    // into partial sums (4 for one RHS, 2 for two, 1 for wider chunks) that
    // are combined in a fixed order; wider chunks take two columns at a time.
    static void bwd_dot(const Fac& f, int32_t base, int32_t j0, int32_t j1, int32_t m, const double* Z,
                        double* Y) {
        if constexpr (W == 1) {
            for (int32_t j = j0; j < j1; ++j) {
                const double* lj = f.v + f.cp[j] + (base - j);
                double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int32_t q = 0;
                for (; q + 4 <= m; q += 4) {
                    s0 += lj[q] * Z[q];
                    s1 += lj[q + 1] * Z[q + 1];
                    s2 += lj[q + 2] * Z[q + 2];
                    s3 += lj[q + 3] * Z[q + 3];
                }
                for (; q < m; ++q) s0 += lj[q] * Z[q];
                Y[j] -= (s0 + s1) + (s2 + s3);
            }
        } else {
            constexpr int NP = W == 2 ? 2 : 1;  // partial sums per column
            for (int32_t j = j0; j < j1; j += 2) {
                const bool two = j + 1 < j1;
                const double* la = f.v + f.cp[j] + (base - j);
                const double* lb = two ? f.v + f.cp[j + 1] + (base - j - 1) : la;
                Row<W> sa[NP], sb[NP];
                for (int p = 0; p < NP; ++p) sa[p] = sb[p] = Row<W>::zero();
                int32_t q = 0;
                for (; q + NP <= m; q += NP)
                    for (int p = 0; p < NP; ++p) {
                        const double* z = Z + (int64_t)(q + p) * W;
                        sa[p].add_scaled(la[q + p], z);
                        sb[p].add_scaled(lb[q + p], z);
                    }
                for (; q < m; ++q) {
                    const double* z = Z + (int64_t)q * W;
                    sa[0].add_scaled(la[q], z);
                    sb[0].add_scaled(lb[q], z);
                }
                for (int p = 1; p < NP; ++p)
                    for (int c = 0; c < W / 2; ++c) {
                        sa[0].v[c] += sa[p].v[c];
                        sb[0].v[c] += sb[p].v[c];
                    }
                sa[0].sub_from(Y + (int64_t)j * W);
                if (two) sb[0].sub_from(Y + (int64_t)(j + 1) * W);
            }
        }
    }

    // Triangle of panel [p0, p1), backward: y_j = (y_j - sum_{i in (j, p1)}
    // L(i,j) y_i) / L(j,j), j descending.
    static void bwd_tri(const Fac& f, int32_t p0, int32_t p1, double* Y) {
        for (int32_t j = p1 - 1; j >= p0; --j) {
            const double* col = f.v + f.cp[j];
            const double d = col[0];
            if constexpr (W == 1) {
                double a = 0;
                for (int32_t i = j + 1; i < p1; ++i) a += col[i - j] * Y[i];
                Y[j] = (Y[j] - a) / d;
            } else {
                Row<W> a = Row<W>::zero();
                for (int32_t i = j + 1; i < p1; ++i) a.add_scaled(col[i - j], Y + (int64_t)i * W);
                Row<W> y = Row<W>::load(Y + (int64_t)j * W);
                const v2d dv = {d, d};
                for (int c = 0; c < W / 2; ++c) y.v[c] = (y.v[c] - a.v[c]) / dv;
                y.store(Y + (int64_t)j * W);
            }
        }
    }
};

template <class Fn>
void with_width(int w, Fn&& fn) {
    switch (w) {
        case 16: fn(std::integral_constant<int, 16>{}); break;
        case 8: fn(std::integral_constant<int, 8>{}); break;
        case 4: fn(std::integral_constant<int, 4>{}); break;
        case 2: fn(std::integral_constant<int, 2>{}); break;
        default: fn(std::integral_constant<int, 1>{}); break;
    }
}

// Supernode s: columns [c0, c1), off-diagonal rows R[0..nr).
struct Sn {
    int32_t c0, c1;
    const int32_t* R;
    int32_t nr;
};

inline Sn sn_of(const CpuSolvePlan& P, const Fac& f, int32_t s) {
    Sn x;
    x.c0 = P.sn_start[s];
    x.c1 = P.sn_start[s + 1];
    const int32_t w = x.c1 - x.c0;
    x.R = f.ri + f.cp[x.c0] + w;
    x.nr = f.cp[x.c0 + 1] - f.cp[x.c0] - w;
    return x;
}

// Forward sweep of one supernode on one chunk, updating only below-rows up
// to `nr_eff` of R (the rows inside the caller's subtree).
template <int W>
void fwd_sn(const Fac& f, const Sn& s, int32_t nr_eff, double* Y, double* acc) {
    if (s.c1 - s.c0 == 1) {  // one column: y_j /= L(j,j), then y_r -= L(r,j) y_j straight into each row
        const double* col = f.v + f.cp[s.c0];
        double* yj = Y + (int64_t)s.c0 * W;
        if constexpr (W == 1) {
            const double y = yj[0] / col[0];
            yj[0] = y;
            for (int32_t q = 0; q < nr_eff; ++q) Y[s.R[q]] -= col[1 + q] * y;
        } else {
            Row<W> y = Row<W>::load(yj);
            const v2d dv = {col[0], col[0]};
            for (int c = 0; c < W / 2; ++c) y.v[c] /= dv;
            y.store(yj);
            for (int32_t q = 0; q < nr_eff; ++q) y.sub_scaled_from(Y + (int64_t)s.R[q] * W, col[1 + q]);
        }
        return;
    }
    for (int32_t p0 = s.c0; p0 < s.c1; p0 += PB) {
        const int32_t p1 = std::min(p0 + PB, s.c1);
        Kern<W>::fwd_tri(f, p0, p1, Y);
        const int32_t m = (s.c1 - p1) + nr_eff;
        for (int32_t q0 = 0; q0 < m; q0 += QB)
            Kern<W>::fwd_rect(f, s.R, s.c1, p0, p1, q0, std::min(q0 + QB, m), Y, acc);
    }
}

// Backward sweep of one supernode on one chunk; Z holds nr rows of W.
template <int W>
void bwd_sn(const Fac& f, const Sn& s, double* Y, double* Z) {
    if (s.c1 - s.c0 == 1) {  // one column: a dot product over its rows, read in place
        const double* col = f.v + f.cp[s.c0];
        if constexpr (W == 1) {
            double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            int32_t q = 0;
            for (; q + 4 <= s.nr; q += 4) {
                s0 += col[1 + q] * Y[s.R[q]];
                s1 += col[2 + q] * Y[s.R[q + 1]];
                s2 += col[3 + q] * Y[s.R[q + 2]];
                s3 += col[4 + q] * Y[s.R[q + 3]];
            }
            for (; q < s.nr; ++q) s0 += col[1 + q] * Y[s.R[q]];
            Y[s.c0] = (Y[s.c0] - ((s0 + s1) + (s2 + s3))) / col[0];
        } else {
            Row<W> a = Row<W>::zero(), b = Row<W>::zero();
            int32_t q = 0;
            for (; q + 2 <= s.nr; q += 2) {
                a.add_scaled(col[1 + q], Y + (int64_t)s.R[q] * W);
                b.add_scaled(col[2 + q], Y + (int64_t)s.R[q + 1] * W);
            }
            if (q < s.nr) a.add_scaled(col[1 + q], Y + (int64_t)s.R[q] * W);
            Row<W> y = Row<W>::load(Y + (int64_t)s.c0 * W);
            const v2d dv = {col[0], col[0]};
            for (int c = 0; c < W / 2; ++c) y.v[c] = (y.v[c] - (a.v[c] + b.v[c])) / dv;
            y.store(Y + (int64_t)s.c0 * W);
        }
        return;
    }
    if (s.nr > 0) {
        for (int32_t k = 0; k < s.nr; ++k) std::memcpy(Z + (int64_t)k * W, Y + (int64_t)s.R[k] * W, sizeof(double) * W);
        Kern<W>::bwd_dot(f, s.c1, s.c0, s.c1, s.nr, Z, Y);
    }
    const int32_t np = (s.c1 - s.c0 + PB - 1) / PB;
    for (int32_t pi = np - 1; pi >= 0; --pi) {
        const int32_t p0 = s.c0 + pi * PB, p1 = std::min(p0 + PB, s.c1);
        if (s.c1 > p1) Kern<W>::bwd_dot(f, p1, p0, p1, s.c1 - p1, Y + (int64_t)p1 * W, Y);
        Kern<W>::bwd_tri(f, p0, p1, Y);
    }
}

struct Chunk {
    int32_t col0, w;  // RHS columns [col0, col0 + w)
    double* Y;        // n x w, permuted order
    double* Z;        // max_nr x w: rows gathered for a supernode split across threads
};

template <typename T>
struct Io {
    const T* b;
    T* x;
    int32_t nrhs;
    const int32_t* perm;
    void load(const Chunk& ch, int32_t k0, int32_t k1) const {
        for (int32_t k = k0; k < k1; ++k) {
            const T* src = b + (int64_t)perm[k] * nrhs + ch.col0;
            double* dst = ch.Y + (int64_t)k * ch.w;
            for (int32_t c = 0; c < ch.w; ++c) dst[c] = (double)src[c];
        }
    }
    void store(const Chunk& ch, int32_t k0, int32_t k1) const {
        for (int32_t k = k0; k < k1; ++k) {
            T* dst = x + (int64_t)perm[k] * nrhs + ch.col0;
            const double* src = ch.Y + (int64_t)k * ch.w;
            for (int32_t c = 0; c < ch.w; ++c) dst[c] = (T)src[c];
        }
    }
};

// One top row i (ordinal t): y_i = b_i - sum over its task-column entries.
template <int W>
void top_gather(const CpuSolvePlan& P, const Fac& f, int32_t t, double* Y) {
    const int32_t i = P.top_rows[t];
    if constexpr (W == 1) {
        double a = 0;
        for (int64_t e = P.pt_ptr[t]; e < P.pt_ptr[t + 1]; ++e) a += f.v[P.pt_pos[e]] * Y[P.pt_col[e]];
        Y[i] -= a;
    } else {
        Row<W> a = Row<W>::zero();
        for (int64_t e = P.pt_ptr[t]; e < P.pt_ptr[t + 1]; ++e)
            a.add_scaled(f.v[P.pt_pos[e]], Y + (int64_t)P.pt_col[e] * W);
        a.sub_from(Y + (int64_t)i * W);
    }
}

template <typename T>
void solve_impl(const Factor& F, const CpuSolvePlan& P, int32_t nrhs, const T* b, T* x, int threads) {
    const int32_t n = F.n;
    const Fac f{F.colptr.data(), F.rowidx.data(), F.vals.data()};
    // RHS chunks: 8 wide, then the remainder as 4 + 2 + 1
    std::vector<Chunk> chunks;
    {
        int32_t c = 0;
        while (nrhs - c >= WMAX) { chunks.push_back({c, WMAX, nullptr, nullptr}); c += WMAX; }
        for (int w = WMAX / 2; w >= 1; w /= 2)
            if (nrhs - c >= w) { chunks.push_back({c, w, nullptr, nullptr}); c += w; }
    }
    // work arrays without value-initialisation: every row of Y is loaded from
    // b (task columns by their task, the others as top rows) and every scratch
    // entry is written before it is read
    std::unique_ptr<double[]> ybuf(new double[(size_t)n * nrhs]);
    std::unique_ptr<double[]> zbuf(new double[(size_t)std::max(P.max_nr, 1) * nrhs]);
    for (Chunk& ch : chunks) {
        ch.Y = ybuf.get() + (int64_t)n * ch.col0;
        ch.Z = zbuf.get() + (int64_t)std::max(P.max_nr, 1) * ch.col0;
    }
    const int32_t nc = (int32_t)chunks.size();
    const Io<T> io{b, x, nrhs, F.perm.data()};
    const int32_t ntask = (int32_t)P.task_first.size();
    const int32_t ntop = (int32_t)P.top_rows.size();
    // tiny systems: the parallel phases cost more than they save
    if ((double)F.nnz() * nrhs < 2e5) threads = 1;
    const int T_ = threads;
    // per thread: a panel update's accumulator and a supernode's gathered rows
    const int64_t zrows = std::max(P.max_nr, 1);
    std::unique_ptr<double[]> accbuf(new double[(size_t)T_ * QB * WMAX]);
    std::unique_ptr<double[]> zthr(new double[(size_t)T_ * zrows * WMAX]);

    auto task_cols = [&](int32_t t, int32_t& lo, int32_t& hi) {
        lo = P.sn_start[P.task_first[t]];
        hi = P.sn_start[P.task_last[t] + 1] - 1;
    };
    auto task_fwd = [&](int32_t t, const Chunk& ch, double* acc) {
        int32_t lo, hi;
        task_cols(t, lo, hi);
        io.load(ch, lo, hi + 1);
        with_width(ch.w, [&](auto Wc) {
            constexpr int W = decltype(Wc)::value;
            for (int32_t s = P.task_first[t]; s <= P.task_last[t]; ++s) {
                const Sn sn = sn_of(P, f, s);
                const int32_t nr_eff = (int32_t)(std::upper_bound(sn.R, sn.R + sn.nr, hi) - sn.R);
                fwd_sn<W>(f, sn, nr_eff, ch.Y, acc);
            }
        });
    };
    auto task_bwd = [&](int32_t t, const Chunk& ch, double* Z) {
        int32_t lo, hi;
        task_cols(t, lo, hi);
        with_width(ch.w, [&](auto Wc) {
            constexpr int W = decltype(Wc)::value;
            for (int32_t s = P.task_last[t]; s >= P.task_first[t]; --s) bwd_sn<W>(f, sn_of(P, f, s), ch.Y, Z);
        });
        io.store(ch, lo, hi + 1);
    };
    auto top_rows_fwd = [&](const Chunk& ch, int32_t t0, int32_t t1) {
        for (int32_t t = t0; t < t1; ++t) io.load(ch, P.top_rows[t], P.top_rows[t] + 1);
        with_width(ch.w, [&](auto Wc) {
            constexpr int W = decltype(Wc)::value;
            for (int32_t t = t0; t < t1; ++t) top_gather<W>(P, f, t, ch.Y);
        });
    };
    auto top_rows_store = [&](const Chunk& ch, int32_t t0, int32_t t1) {
        for (int32_t t = t0; t < t1; ++t) io.store(ch, P.top_rows[t], P.top_rows[t] + 1);
    };

    if (T_ == 1) {
        // one thread: each chunk through the whole solve
        double* acc = accbuf.get();
        double* Z = zthr.get();
        for (int32_t ci = 0; ci < nc; ++ci) {
            const Chunk& ch = chunks[(size_t)ci];
            for (int32_t t = 0; t < ntask; ++t) task_fwd(t, ch, acc);
            top_rows_fwd(ch, 0, ntop);
            with_width(ch.w, [&](auto Wc) {
                constexpr int W = decltype(Wc)::value;
                for (int32_t s : P.top_sn) {
                    const Sn sn = sn_of(P, f, s);
                    fwd_sn<W>(f, sn, sn.nr, ch.Y, acc);
                }
                for (auto it = P.top_sn.rbegin(); it != P.top_sn.rend(); ++it) bwd_sn<W>(f, sn_of(P, f, *it), ch.Y, Z);
            });
            for (int32_t t = 0; t < ntask; ++t) task_bwd(t, ch, Z);
            top_rows_store(ch, 0, ntop);
        }
        return;
    }

    // Several threads: tasks x chunks, then the top region with the work of
    // each large supernode split across threads (measured better balanced
    // than whole chunks per thread even when there are as many chunks as
    // threads).
    const int32_t nrb = (ntop + QB - 1) / QB;  // blocks of top rows
    const int64_t big = 1 << 16;                // supernode work worth a split across threads
    // Split sizes of a large supernode's steps: about four items per thread
    // (every row's and every column's sum is computed whole by one item, so
    // the split does not change the result).
    auto split = [&](int32_t len, int32_t lo_cap, int32_t hi_cap) {
        const int32_t want = (int32_t)(((int64_t)len * nc + 4LL * T_ - 1) / (4LL * T_));
        return std::max(lo_cap, std::min(hi_cap, want));
    };
    // Steps of the top region: a run of consecutive small supernodes (one
    // thread, one barrier) or one large supernode (split across threads).
    struct Step {
        int32_t a, b;  // top_sn[a, b)
        bool split;
    };
    std::vector<Step> steps;
    for (int32_t i = 0; i < (int32_t)P.top_sn.size(); ++i) {
        const Sn sn = sn_of(P, f, P.top_sn[i]);
        // (one-column supernodes have their own formulas: never split)
        const bool large = sn.c1 - sn.c0 > 1 && (int64_t)(sn.c1 - sn.c0) * (sn.c1 - sn.c0 + sn.nr) * nrhs >= big;
        if (!large && !steps.empty() && !steps.back().split && steps.back().b == i)
            steps.back().b = i + 1;
        else
            steps.push_back({i, i + 1, large});
    }
#pragma omp parallel num_threads(T_)
    {
        double* acc = accbuf.get() + (size_t)thread_id() * QB * WMAX;
        double* Z = zthr.get() + (size_t)thread_id() * zrows * WMAX;
#pragma omp for schedule(dynamic, 1)
        for (int64_t it = 0; it < (int64_t)ntask * nc; ++it) task_fwd((int32_t)(it / nc), chunks[(size_t)(it % nc)], acc);
#pragma omp for schedule(dynamic, 1)
        for (int64_t it = 0; it < (int64_t)nrb * nc; ++it) {
            const int32_t rb = (int32_t)(it / nc);
            top_rows_fwd(chunks[(size_t)(it % nc)], rb * QB, std::min(ntop, (rb + 1) * QB));
        }
        // forward over the top supernodes
        for (const Step& st : steps) {
            if (!st.split) {
#pragma omp master
                for (const Chunk& ch : chunks)
                    with_width(ch.w, [&](auto Wc) {
                        for (int32_t i = st.a; i < st.b; ++i) {
                            const Sn sn = sn_of(P, f, P.top_sn[i]);
                            fwd_sn<decltype(Wc)::value>(f, sn, sn.nr, ch.Y, acc);
                        }
                    });
#pragma omp barrier
                continue;
            }
            const Sn sn = sn_of(P, f, P.top_sn[st.a]);
            for (int32_t p0 = sn.c0; p0 < sn.c1; p0 += PB) {
                const int32_t p1 = std::min(p0 + PB, sn.c1);
                const int32_t m = (sn.c1 - p1) + sn.nr;
                const int32_t qb = split(m, 16, QB);
                const int32_t nqb = (m + qb - 1) / qb;
#pragma omp for schedule(static, 1)
                for (int32_t ci = 0; ci < nc; ++ci) {
                    const Chunk& ch = chunks[(size_t)ci];
                    with_width(ch.w, [&](auto Wc) { Kern<decltype(Wc)::value>::fwd_tri(f, p0, p1, ch.Y); });
                }
#pragma omp for schedule(dynamic, 1)
                for (int64_t it = 0; it < (int64_t)nqb * nc; ++it) {
                    const Chunk& ch = chunks[(size_t)(it % nc)];
                    const int32_t q0 = (int32_t)(it / nc) * qb;
                    with_width(ch.w, [&](auto Wc) {
                        Kern<decltype(Wc)::value>::fwd_rect(f, sn.R, sn.c1, p0, p1, q0, std::min(q0 + qb, m), ch.Y, acc);
                    });
                }
            }
        }
        // backward over the top supernodes
        for (auto sit = steps.rbegin(); sit != steps.rend(); ++sit) {
            const Step& st = *sit;
            if (!st.split) {
#pragma omp master
                for (const Chunk& ch : chunks)
                    with_width(ch.w, [&](auto Wc) {
                        for (int32_t i = st.b - 1; i >= st.a; --i)
                            bwd_sn<decltype(Wc)::value>(f, sn_of(P, f, P.top_sn[i]), ch.Y, Z);
                    });
#pragma omp barrier
                continue;
            }
            const Sn sn = sn_of(P, f, P.top_sn[st.a]);
            const int32_t ws = sn.c1 - sn.c0;
            if (sn.nr > 0) {
#pragma omp for schedule(static)
                for (int64_t it = 0; it < (int64_t)sn.nr * nc; ++it) {
                    const Chunk& ch = chunks[(size_t)(it % nc)];
                    const int32_t k = (int32_t)(it / nc);
                    std::memcpy(ch.Z + (int64_t)k * ch.w, ch.Y + (int64_t)sn.R[k] * ch.w, sizeof(double) * ch.w);
                }
                const int32_t jb = split(ws, 1, JB);
                const int32_t njb = (ws + jb - 1) / jb;
#pragma omp for schedule(dynamic, 1)
                for (int64_t it = 0; it < (int64_t)njb * nc; ++it) {
                    const Chunk& ch = chunks[(size_t)(it % nc)];
                    const int32_t j0 = sn.c0 + (int32_t)(it / nc) * jb;
                    with_width(ch.w, [&](auto Wc) {
                        Kern<decltype(Wc)::value>::bwd_dot(f, sn.c1, j0, std::min(j0 + jb, sn.c1), sn.nr, ch.Z, ch.Y);
                    });
                }
            }
            const int32_t np = (ws + PB - 1) / PB;
            for (int32_t pi = np - 1; pi >= 0; --pi) {
                const int32_t p0 = sn.c0 + pi * PB, p1 = std::min(p0 + PB, sn.c1);
                if (sn.c1 > p1) {
                    const int32_t jb = split(p1 - p0, 1, JB);
                    const int32_t njb = (p1 - p0 + jb - 1) / jb;
#pragma omp for schedule(dynamic, 1)
                    for (int64_t it = 0; it < (int64_t)njb * nc; ++it) {
                        const Chunk& ch = chunks[(size_t)(it % nc)];
                        const int32_t j0 = p0 + (int32_t)(it / nc) * jb;
                        with_width(ch.w, [&](auto Wc) {
                            Kern<decltype(Wc)::value>::bwd_dot(f, p1, j0, std::min(j0 + jb, p1), sn.c1 - p1,
                                                               ch.Y + (int64_t)p1 * ch.w, ch.Y);
                        });
                    }
                }
#pragma omp for schedule(static, 1)
                for (int32_t ci = 0; ci < nc; ++ci) {
                    const Chunk& ch = chunks[(size_t)ci];
                    with_width(ch.w, [&](auto Wc) { Kern<decltype(Wc)::value>::bwd_tri(f, p0, p1, ch.Y); });
                }
            }
        }
#pragma omp for schedule(dynamic, 1)
        for (int64_t it = 0; it < (int64_t)ntask * nc; ++it) task_bwd((int32_t)(it / nc), chunks[(size_t)(it % nc)], Z);
#pragma omp for schedule(static)
        for (int64_t it = 0; it < (int64_t)nrb * nc; ++it) {
            const int32_t rb = (int32_t)(it / nc);
            top_rows_store(chunks[(size_t)(it % nc)], rb * QB, std::min(ntop, (rb + 1) * QB));
        }
    }
}

}  // namespace

void cpu_plan(const Factor& F, CpuSolvePlan& P, int32_t threads) {
    const int32_t n = F.n;
    const int32_t* cp = F.colptr.data();
    const int32_t* ri = F.rowidx.data();
    P = CpuSolvePlan();
    P.n = n;
    if (n == 0) {
        P.sn_start.assign(1, 0);
        return;
    }
    const int nt = host_threads(threads);
    // supernodes: column j joins column j-1 when pattern(j) = pattern(j-1) \ {j-1}
    std::vector<char> joins((size_t)n, 0);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1024) if (nt > 1 && F.nnz() > (1 << 20))
    for (int32_t j = 1; j < n; ++j) {
        const int32_t a = cp[j - 1], la = cp[j] - a, bb = cp[j], lb = cp[j + 1] - bb;
        joins[j] = (lb == la - 1 && la >= 2 && ri[a + 1] == j &&
                    std::equal(ri + a + 1, ri + a + la, ri + bb))
                       ? 1
                       : 0;
    }
    P.sn_start.push_back(0);
    for (int32_t j = 1; j < n; ++j)
        if (!joins[j]) P.sn_start.push_back(j);
    P.sn_start.push_back(n);
    const int32_t nsn = (int32_t)P.sn_start.size() - 1;
    for (int32_t s = 0; s < nsn; ++s) {
        const int32_t c0 = P.sn_start[s], w = P.sn_start[s + 1] - c0;
        P.max_nr = std::max(P.max_nr, cp[c0 + 1] - cp[c0] - w);
    }
    // elimination tree (parent = first off-diagonal row), subtree sizes and
    // costs; a task needs the subtrees to be contiguous column ranges
    // (postorder), which is checked: min index of the subtree = j - size + 1
    // (parents come after their children, so column j is complete when reached)
    std::vector<int32_t> size((size_t)n, 1), minidx((size_t)n);
    std::vector<int64_t> cost((size_t)n, 0);
    bool post = true;
    for (int32_t j = 0; j < n; ++j) minidx[j] = j;
    for (int32_t j = 0; j < n; ++j) {
        cost[j] += cp[j + 1] - cp[j];
        if (minidx[j] != j - size[j] + 1) post = false;
        if (cp[j + 1] - cp[j] > 1) {
            const int32_t p = ri[cp[j] + 1];
            size[p] += size[j];
            cost[p] += cost[j];
            minidx[p] = std::min(minidx[p], minidx[j]);
        }
    }
    const int64_t total = F.nnz();
    const int64_t cut = std::max<int64_t>(total / 256, 4096);
    std::vector<char> in_task((size_t)nsn, 0);
    if (post) {
        std::vector<int32_t> sn_of_col((size_t)n);
        for (int32_t s = 0; s < nsn; ++s)
            for (int32_t j = P.sn_start[s]; j < P.sn_start[s + 1]; ++j) sn_of_col[j] = s;
        for (int32_t s = 0; s < nsn; ++s) {
            const int32_t e = P.sn_start[s + 1] - 1;  // last column
            if (cost[e] > cut) continue;
            // maximal: the parent supernode (cost of its last column) is above the cut
            const int32_t pe = cp[e + 1] - cp[e] > 1 ? ri[cp[e] + 1] : -1;
            if (pe >= 0 && cost[P.sn_start[sn_of_col[pe] + 1] - 1] <= cut) continue;
            const int32_t first = sn_of_col[e - size[e] + 1];
            P.task_first.push_back(first);
            P.task_last.push_back(s);
            P.task_cost.push_back(cost[e]);
            for (int32_t q = first; q <= s; ++q) in_task[q] = 1;
        }
        // largest tasks first
        std::vector<int32_t> ord(P.task_first.size());
        for (size_t i = 0; i < ord.size(); ++i) ord[i] = (int32_t)i;
        std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b2) { return P.task_cost[a] > P.task_cost[b2]; });
        std::vector<int32_t> tf, tl;
        std::vector<int64_t> tc;
        for (int32_t i : ord) {
            tf.push_back(P.task_first[i]);
            tl.push_back(P.task_last[i]);
            tc.push_back(P.task_cost[i]);
        }
        P.task_first.swap(tf);
        P.task_last.swap(tl);
        P.task_cost.swap(tc);
    }
    std::vector<int32_t> top_index((size_t)n, -1);
    for (int32_t s = 0; s < nsn; ++s) {
        if (in_task[s]) continue;
        P.top_sn.push_back(s);
        for (int32_t j = P.sn_start[s]; j < P.sn_start[s + 1]; ++j) {
            top_index[j] = (int32_t)P.top_rows.size();
            P.top_rows.push_back(j);
        }
    }
    // row lists of the top rows restricted to task columns (entries of a task
    // column below the task's last column), ascending column per row
    const int32_t ntop = (int32_t)P.top_rows.size();
    P.pt_ptr.assign((size_t)ntop + 1, 0);
    std::vector<int32_t> task_hi_of_col((size_t)n, -1);
    for (size_t t = 0; t < P.task_first.size(); ++t) {
        const int32_t lo = P.sn_start[P.task_first[t]], hi = P.sn_start[P.task_last[t] + 1] - 1;
        for (int32_t j = lo; j <= hi; ++j) task_hi_of_col[j] = hi;
    }
    // contiguous column ranges (in column order) count their entries per top
    // row, then fill: columns ascend within each row for any thread count
    const int ntp = F.nnz() > (1 << 22) ? nt : 1;
    std::vector<int32_t> c0((size_t)ntp + 1, n);
    c0[0] = 0;
    for (int t = 1; t < ntp; ++t)
        c0[t] = (int32_t)(std::lower_bound(F.colptr.begin(), F.colptr.end() - 1, (int32_t)(F.nnz() * t / ntp)) -
                          F.colptr.begin());
    for (int t = 1; t <= ntp; ++t) c0[t] = std::max(c0[t], c0[t - 1]);
    std::vector<int64_t> cnt((size_t)ntp * ntop, 0);
#pragma omp parallel for num_threads(ntp) schedule(static, 1) if (ntp > 1)
    for (int t = 0; t < ntp; ++t) {
        int64_t* ct = cnt.data() + (size_t)t * ntop;
        for (int32_t j = c0[t]; j < c0[t + 1]; ++j) {
            if (task_hi_of_col[j] < 0) continue;
            const int32_t *b0 = ri + cp[j], *b1 = ri + cp[j + 1];
            for (const int32_t* p = std::upper_bound(b0, b1, task_hi_of_col[j]); p < b1; ++p) ct[top_index[*p]]++;
        }
    }
    int64_t run = 0;
    for (int32_t r = 0; r < ntop; ++r) {
        P.pt_ptr[r] = run;
        for (int t = 0; t < ntp; ++t) {
            const int64_t k = cnt[(size_t)t * ntop + r];
            cnt[(size_t)t * ntop + r] = run;
            run += k;
        }
    }
    P.pt_ptr[ntop] = run;
    P.pt_col.resize((size_t)run);
    P.pt_pos.resize((size_t)run);
#pragma omp parallel for num_threads(ntp) schedule(static, 1) if (ntp > 1)
    for (int t = 0; t < ntp; ++t) {
        int64_t* next = cnt.data() + (size_t)t * ntop;
        for (int32_t j = c0[t]; j < c0[t + 1]; ++j) {
            if (task_hi_of_col[j] < 0) continue;
            const int32_t *b0 = ri + cp[j], *b1 = ri + cp[j + 1];
            for (const int32_t* p = std::upper_bound(b0, b1, task_hi_of_col[j]); p < b1; ++p) {
                const int64_t d = next[top_index[*p]]++;
                P.pt_col[d] = j;
                P.pt_pos[d] = p - ri;
            }
        }
    }
}

void cpu_solve(const Factor& F, const CpuSolvePlan& P, int32_t precision, int32_t nrhs, const void* b, void* x,
               int32_t threads) {
    if (F.n == 0 || nrhs <= 0) return;
    const int nt = host_threads(threads);
    if (precision == 0)
        solve_impl<float>(F, P, nrhs, (const float*)b, (float*)x, nt);
    else
        solve_impl<double>(F, P, nrhs, (const double*)b, (double*)x, nt);
}

}  // namespace gbchol
