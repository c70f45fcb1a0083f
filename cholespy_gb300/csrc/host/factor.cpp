// Symbolic and numeric sparse LL^T factorisation on the host.
//
// Replaces the reference's CHOLMOD calls (src/cholesky_solver.cpp:200-297):
// cholmod_analyze (ordering + symbolic) and cholmod_factorize (numeric, LL^T,
// simplicial). The exported factor has exactly the simplicial symbolic
// pattern (no explicit zeros) and is laid out like cholmod_factor_to_sparse:
// CSC, rows sorted, diagonal first in each column. Only the numeric phase
// works on amalgamated fronts (chains of supernodes merged with explicit
// zeros); each column of L is then read back at its own pattern (entries
// outside it are exact zeros: every product feeding them has a zero factor).
//
// Published methods followed (no CHOLMOD source used):
//   * elimination tree: Liu's algorithm with path compression
//     (J. W. H. Liu, "The role of elimination trees in sparse factorization",
//     SIAM J. Matrix Anal. Appl. 11, 1990);
//   * postorder of the elimination tree (same reference);
//   * row-subtree traversal for the pattern of L (Davis, "Direct Methods for
//     Sparse Linear Systems", SIAM 2006, section 4.2);
//   * fundamental supernodes (Liu, Ng & Peyton, SIAM J. Matrix Anal. Appl.
//     14, 1993);
//   * multifrontal numeric factorisation (Duff & Reid 1983; Liu, SIAM Review
//     34, 1992) with dense blocked kernels (dense.cpp), on fronts from relaxed
//     supernode amalgamation (Ashcraft & Grimes, ACM TOMS 15, 1989).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>

#include "dense.h"
#include "host.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace gbchol {

namespace {

int resolve_threads(int32_t t) {
    if (t > 0) return t;
#ifdef _OPENMP
    return std::max(1, omp_get_max_threads());
#else
    return 1;
#endif
}

// CSR pattern of the strictly lower triangle of P A P^T: row i lists the
// columns j < i with a structural entry. Also returns the CSC of the lower
// triangle with values (diagonal included) for numeric assembly.
// With `amap`, also records for every entry k of A its position in the
// lower CSC (-1 for entries above the diagonal).
void permuted_lower(const Csc& A, const std::vector<int32_t>& pinv, std::vector<int32_t>& rptr,
                    std::vector<int32_t>& rcol, std::vector<int32_t>& cptr,
                    std::vector<int32_t>& crow, std::vector<double>& cval,
                    std::vector<int32_t>* amap = nullptr) {
    const int32_t n = A.n;
    if (amap) amap->assign(A.rowidx.size(), -1);
    rptr.assign((size_t)n + 1, 0);
    cptr.assign((size_t)n + 1, 0);
    for (int32_t c = 0; c < n; ++c)
        for (int32_t k = A.colptr[c]; k < A.colptr[c + 1]; ++k) {
            int32_t r = A.rowidx[k];
            if (r < c) continue;  // upper part ignored (stype = -1)
            int32_t pr = pinv[r], pc = pinv[c];
            int32_t hi = std::max(pr, pc), lo = std::min(pr, pc);
            cptr[lo + 1]++;
            if (hi != lo) rptr[hi + 1]++;
        }
    for (int32_t i = 0; i < n; ++i) {
        rptr[i + 1] += rptr[i];
        cptr[i + 1] += cptr[i];
    }
    rcol.resize((size_t)rptr[n]);
    crow.resize((size_t)cptr[n]);
    cval.resize((size_t)cptr[n]);
    std::vector<int32_t> rn(rptr.begin(), rptr.end() - 1), cn(cptr.begin(), cptr.end() - 1);
    for (int32_t c = 0; c < n; ++c)
        for (int32_t k = A.colptr[c]; k < A.colptr[c + 1]; ++k) {
            int32_t r = A.rowidx[k];
            if (r < c) continue;
            int32_t pr = pinv[r], pc = pinv[c];
            int32_t hi = std::max(pr, pc), lo = std::min(pr, pc);
            int32_t d = cn[lo]++;
            crow[d] = hi;
            cval[d] = A.vals[k];
            if (amap) (*amap)[k] = d;
            if (hi != lo) rcol[rn[hi]++] = lo;
        }
}

// Liu's elimination tree from the strictly-lower CSR pattern.
std::vector<int32_t> etree(int32_t n, const std::vector<int32_t>& rptr,
                           const std::vector<int32_t>& rcol) {
    std::vector<int32_t> parent((size_t)n, -1), anc((size_t)n, -1);
    for (int32_t i = 0; i < n; ++i) {
        for (int32_t k = rptr[i]; k < rptr[i + 1]; ++k) {
            int32_t r = rcol[k];
            while (r != -1 && r < i) {
                int32_t nx = anc[r];
                anc[r] = i;
                if (nx == -1) { parent[r] = i; break; }
                r = nx;
            }
        }
    }
    return parent;
}

// Postorder of a forest: children visited in increasing index order.
std::vector<int32_t> postorder(const std::vector<int32_t>& parent) {
    const int32_t n = (int32_t)parent.size();
    std::vector<int32_t> head((size_t)n, -1), next((size_t)n, -1), post;
    post.reserve((size_t)n);
    for (int32_t j = n - 1; j >= 0; --j) {
        if (parent[j] == -1) continue;
        next[j] = head[parent[j]];
        head[parent[j]] = j;
    }
    std::vector<int32_t> stack;
    for (int32_t r = 0; r < n; ++r) {
        if (parent[r] != -1) continue;
        stack.push_back(r);
        while (!stack.empty()) {
            int32_t p = stack.back();
            int32_t c = head[p];
            if (c == -1) {
                stack.pop_back();
                post.push_back(p);
            } else {
                head[p] = next[c];
                stack.push_back(c);
            }
        }
    }
    return post;
}

}  // namespace

Status factorize(const Csc& A, const FactorOptions& opt, Factor& F, std::string& err) {
    const int32_t n = A.n;
    const int threads = resolve_threads(opt.threads);
    F = Factor();
    F.n = n;
    if (n == 0) {
        F.colptr.assign(1, 0);
        F.sn_start.assign(1, 0);
        return ST_OK;
    }

    // ---- ordering -------------------------------------------------------
    std::vector<int32_t> perm0;
    if (opt.use_given_perm) {
        perm0.assign(opt.perm_in, opt.perm_in + n);
        std::vector<char> seen((size_t)n, 0);
        for (int32_t k = 0; k < n; ++k) {
            if (perm0[k] < 0 || perm0[k] >= n || seen[perm0[k]]) {
                err = "Invalid permutation.";
                return ST_INVALID;
            }
            seen[perm0[k]] = 1;
        }
    } else {
        // adjacency of the symmetric graph from the strictly lower part
        std::vector<int32_t> xadj((size_t)n + 1, 0), adj;
        for (int32_t c = 0; c < n; ++c)
            for (int32_t k = A.colptr[c]; k < A.colptr[c + 1]; ++k) {
                int32_t r = A.rowidx[k];
                if (r <= c) continue;
                xadj[r + 1]++;
                xadj[c + 1]++;
            }
        for (int32_t i = 0; i < n; ++i) xadj[i + 1] += xadj[i];
        adj.resize((size_t)xadj[n]);
        std::vector<int32_t> nx(xadj.begin(), xadj.end() - 1);
        for (int32_t c = 0; c < n; ++c)
            for (int32_t k = A.colptr[c]; k < A.colptr[c + 1]; ++k) {
                int32_t r = A.rowidx[k];
                if (r <= c) continue;
                adj[nx[r]++] = c;
                adj[nx[c]++] = r;
            }
        perm0 = nested_dissection(n, xadj, adj);
    }
    std::vector<int32_t> pinv((size_t)n);
    for (int32_t k = 0; k < n; ++k) pinv[perm0[k]] = k;

    std::vector<int32_t> rptr, rcol, cptr, crow;
    std::vector<double> cval;
    permuted_lower(A, pinv, rptr, rcol, cptr, crow, cval);
    std::vector<int32_t> parent = etree(n, rptr, rcol);

    // ---- postorder and final permutation --------------------------------
    {
        std::vector<int32_t> post = postorder(parent);
        F.perm.resize((size_t)n);
        for (int32_t k = 0; k < n; ++k) F.perm[k] = perm0[post[k]];
        for (int32_t k = 0; k < n; ++k) pinv[F.perm[k]] = k;
    }
    auto sym = std::make_shared<SymbolicCache>();
    permuted_lower(A, pinv, rptr, rcol, cptr, crow, cval, &sym->amap);
    parent = etree(n, rptr, rcol);
    F.parent = parent;

    // ---- column counts of L by row subtrees -----------------------------
    // Rows are independent: each thread walks its rows' subtrees with its own
    // marks and counts, and the integer counts are summed.
    std::vector<int64_t> cnt((size_t)n, 1);  // diagonal
    {
        const int nt = (threads > 1 && n >= 32768) ? threads : 1;
        std::vector<std::vector<int32_t>> part((size_t)nt);
#pragma omp parallel num_threads(nt) if (nt > 1)
        {
#ifdef _OPENMP
            std::vector<int32_t>& pc = part[(size_t)omp_get_thread_num()];
#else
            std::vector<int32_t>& pc = part[0];
#endif
            pc.assign((size_t)n, 0);
            std::vector<int32_t> mk((size_t)n, -1);
#pragma omp for schedule(dynamic, 1024)
            for (int32_t i = 0; i < n; ++i) {
                mk[i] = i;
                for (int32_t k = rptr[i]; k < rptr[i + 1]; ++k) {
                    for (int32_t r = rcol[k]; mk[r] != i; r = parent[r]) {
                        pc[r]++;
                        mk[r] = i;
                    }
                }
            }
        }
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1)
        for (int32_t j = 0; j < n; ++j)
            for (int t = 0; t < nt; ++t) cnt[j] += part[(size_t)t][j];
    }
    int64_t total = 0;
    for (int32_t j = 0; j < n; ++j) total += cnt[j];
    if (total >= (int64_t)INT32_MAX) {
        err = "Factor too large: nnz(L) exceeds 2^31-1.";
        return ST_NOMEM;
    }
    F.colptr.resize((size_t)n + 1);
    F.colptr[0] = 0;
    for (int32_t j = 0; j < n; ++j) F.colptr[j + 1] = F.colptr[j] + (int32_t)cnt[j];

    // ---- fundamental supernodes -----------------------------------------
    std::vector<int32_t> nchild((size_t)n, 0);
    for (int32_t j = 0; j < n; ++j)
        if (parent[j] >= 0) nchild[parent[j]]++;
    F.sn_start.clear();
    F.sn_start.push_back(0);
    for (int32_t j = 1; j < n; ++j) {
        bool merge = parent[j - 1] == j && cnt[j - 1] == cnt[j] + 1 && nchild[j] == 1;
        if (!merge) F.sn_start.push_back(j);
    }
    F.sn_start.push_back(n);
    const int32_t nsn = (int32_t)F.sn_start.size() - 1;
    std::vector<int32_t> sn_of((size_t)n);
    for (int32_t s = 0; s < nsn; ++s)
        for (int32_t j = F.sn_start[s]; j < F.sn_start[s + 1]; ++j) sn_of[j] = s;
    std::vector<int32_t> sn_parent((size_t)nsn, -1), child_ptr((size_t)nsn + 1, 0);
    for (int32_t s = 0; s < nsn; ++s) {
        const int32_t last = F.sn_start[s + 1] - 1;
        if (parent[last] >= 0) {
            sn_parent[s] = sn_of[parent[last]];
            child_ptr[sn_parent[s] + 1]++;
        }
    }
    for (int32_t s = 0; s < nsn; ++s) child_ptr[s + 1] += child_ptr[s];
    std::vector<int32_t> children((size_t)child_ptr[nsn]);
    {
        std::vector<int32_t> nx(child_ptr.begin(), child_ptr.end() - 1);
        for (int32_t s = 0; s < nsn; ++s)  // children in increasing order
            if (sn_parent[s] >= 0) children[nx[sn_parent[s]]++] = s;
    }

    // ---- pattern of L by supernodes -------------------------------------
    // rows(s) = the supernode's columns, the rows of A below them and the
    // rows of its children's patterns below their own columns (all of which
    // lie at or below the supernode's first column); every column j of a
    // fundamental supernode holds the suffix of rows(s) from j on. The lists
    // are built in postorder (children first), then copied out per column in
    // parallel.
    std::vector<int64_t> sptr((size_t)nsn + 1, 0);
    for (int32_t s = 0; s < nsn; ++s) sptr[s + 1] = sptr[s] + cnt[F.sn_start[s]];
    std::vector<int32_t> srows((size_t)sptr[nsn]);
    {
        // Subtrees below a size cut are independent (a supernode needs only
        // its children's lists): they are built as parallel tasks, each with
        // its own marks, then the supernodes above the cut in order.
        std::vector<int64_t> sub((size_t)nsn);
        std::vector<int32_t> sfirst((size_t)nsn);
        for (int32_t s = 0; s < nsn; ++s) {
            sub[s] = sptr[s + 1] - sptr[s];
            sfirst[s] = s;
        }
        for (int32_t s = 0; s < nsn; ++s)
            if (sn_parent[s] >= 0) {
                sub[sn_parent[s]] += sub[s];
                sfirst[sn_parent[s]] = std::min(sfirst[sn_parent[s]], sfirst[s]);
            }
        const int64_t cut = threads > 1 ? std::max<int64_t>(sptr[nsn] / (8 * threads), 1 << 16) : -1;
        std::vector<int32_t> roots;
        std::vector<char> above((size_t)nsn, 0);
        for (int32_t s = 0; s < nsn; ++s) {
            above[s] = sub[s] > cut;
            if (sub[s] <= cut && (sn_parent[s] < 0 || sub[sn_parent[s]] > cut)) roots.push_back(s);
        }
        int bad = 0;
        // rows(s): its columns, A's rows below them, its children's rows below
        // their own columns; the rows after the columns sorted
        auto build = [&](int32_t s, std::vector<int32_t>& mk) {
            const int32_t f = F.sn_start[s], l1 = F.sn_start[s + 1];
            int32_t* out = srows.data() + sptr[s];
            int64_t len = 0;
            const int64_t cap = sptr[s + 1] - sptr[s];
            for (int32_t j = f; j < l1; ++j) {
                out[len++] = j;
                mk[j] = s;
            }
            auto add = [&](int32_t r) {
                if (mk[r] == s) return;
                mk[r] = s;
                if (len < cap) out[len] = r;
                ++len;
            };
            for (int32_t j = f; j < l1; ++j)
                for (int32_t k = cptr[j]; k < cptr[j + 1]; ++k) add(crow[k]);
            for (int32_t q = child_ptr[s]; q < child_ptr[s + 1]; ++q) {
                const int32_t c = children[q];
                const int32_t cw = F.sn_start[c + 1] - F.sn_start[c];
                for (int64_t k = sptr[c] + cw; k < sptr[c + 1]; ++k) add(srows[k]);
            }
            if (len != cap) return false;
            std::sort(out + (l1 - f), out + len);
            return true;
        };
        const int nt = threads > 1 && roots.size() > 1 ? threads : 1;
#pragma omp parallel num_threads(nt) if (nt > 1)
        {
            std::vector<int32_t> mk((size_t)n, -1);
#pragma omp for schedule(dynamic, 1)
            for (int64_t q = 0; q < (int64_t)roots.size(); ++q)
                for (int32_t s = sfirst[roots[q]]; s <= roots[q]; ++s)
                    if (!build(s, mk)) {
#pragma omp atomic write
                        bad = 1;
                    }
        }
        std::vector<int32_t> mk((size_t)n, -1);
        for (int32_t s = 0; s < nsn && !bad; ++s)
            if (above[s] && !build(s, mk)) bad = 1;
        if (bad) {
            err = "Internal error: supernodal pattern does not match the column counts.";
            return ST_INTERNAL;
        }
    }
    F.rowidx.resize((size_t)total);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64) if (threads > 1)
    for (int32_t s = 0; s < nsn; ++s) {
        const int32_t f = F.sn_start[s], l1 = F.sn_start[s + 1];
        for (int32_t j = f; j < l1; ++j)
            std::copy(srows.begin() + sptr[s] + (j - f), srows.begin() + sptr[s + 1],
                      F.rowidx.begin() + F.colptr[j]);
    }
    std::vector<int32_t>().swap(srows);

    // ---- fronts of the numeric phase (relaxed amalgamation) -------------
    // Supernode s joins its parent p's front when its columns end where p's
    // begin (s is p's last child) and the merged front stays narrow or adds
    // few explicit zeros: always up to 4 columns, up to 16 columns with at
    // most half zeros, up to 48 with at most 10%, any width with at most 5%
    // (the zeros of the merged trapezoid of columns against its rows). The
    // rule depends on the pattern only.
    {
        std::vector<int32_t> gstart((size_t)nsn);
        std::vector<int64_t> gnz((size_t)nsn, 0);
        std::vector<char> merged((size_t)nsn, 0);
        for (int32_t s = 0; s < nsn; ++s) {
            gstart[s] = F.sn_start[s];
            for (int32_t j = F.sn_start[s]; j < F.sn_start[s + 1]; ++j) gnz[s] += cnt[j];
        }
        for (int32_t s = 0; s < nsn; ++s) {
            const int32_t p = sn_parent[s];
            if (p < 0 || F.sn_start[s + 1] != F.sn_start[p]) continue;
            const int64_t wp = F.sn_start[p + 1] - F.sn_start[p];
            const int64_t w = F.sn_start[p + 1] - gstart[s];
            const int64_t fsz = w + (cnt[F.sn_start[p]] - wp);
            const double trap = (double)w * (double)fsz - 0.5 * (double)w * (double)(w - 1);
            const double zeros = trap - (double)(gnz[s] + gnz[p]);
            const double frac = zeros / trap;
            if (w <= 4 || (w <= 16 && frac <= 0.5) || (w <= 48 && frac <= 0.1) || frac <= 0.05) {
                merged[s] = 1;
                gstart[p] = gstart[s];
                gnz[p] += gnz[s];
            }
        }
        std::vector<int32_t> front_of((size_t)nsn, -1), top_of((size_t)nsn);
        for (int32_t s = nsn - 1; s >= 0; --s) top_of[s] = merged[s] ? top_of[sn_parent[s]] : s;
        for (int32_t s = 0; s < nsn; ++s)
            if (!merged[s]) {
                front_of[s] = (int32_t)sym->fr_nr.size();
                const int32_t w = F.sn_start[s + 1] - F.sn_start[s];
                sym->fr_col.push_back(gstart[s]);
                sym->fr_rpos.push_back((int64_t)F.colptr[F.sn_start[s]] + w);
                sym->fr_nr.push_back((int32_t)cnt[F.sn_start[s]] - w);
            }
        const int32_t nfr = (int32_t)sym->fr_nr.size();
        sym->fr_col.push_back(n);
        sym->fr_parent.assign((size_t)nfr, -1);
        sym->fr_child_ptr.assign((size_t)nfr + 1, 0);
        for (int32_t s = 0; s < nsn; ++s)
            if (!merged[s] && sn_parent[s] >= 0) {
                const int32_t f = front_of[s], pf = front_of[top_of[sn_parent[s]]];
                sym->fr_parent[f] = pf;
                sym->fr_child_ptr[pf + 1]++;
            }
        for (int32_t f = 0; f < nfr; ++f) sym->fr_child_ptr[f + 1] += sym->fr_child_ptr[f];
        sym->fr_children.resize((size_t)sym->fr_child_ptr[nfr]);
        std::vector<int32_t> nx(sym->fr_child_ptr.begin(), sym->fr_child_ptr.end() - 1);
        for (int32_t f = 0; f < nfr; ++f)  // children in increasing order
            if (sym->fr_parent[f] >= 0) sym->fr_children[nx[sym->fr_parent[f]]++] = f;
    }

    // ---- the symbolic analysis kept for refactorisations ---------------
    sym->n = n;
    sym->a_colptr = A.colptr;
    sym->a_rowidx = A.rowidx;
    sym->cptr = std::move(cptr);
    sym->crow = std::move(crow);
    sym->sn_parent = std::move(sn_parent);
    sym->child_ptr = std::move(child_ptr);
    sym->children = std::move(children);
    F.sym = sym;
    return numeric_factor(F, *sym, cval, threads, F.vals, F.flops, err);
}

Status numeric_factor(const Factor& F, const SymbolicCache& S, const std::vector<double>& cval, int32_t nthreads,
                      std::vector<double>& vals_out, double& flops_out, std::string& err) {
    const int32_t n = F.n;
    const int threads = resolve_threads(nthreads);
    const int32_t nsn = (int32_t)S.fr_nr.size();  // fronts
    const int64_t total = F.nnz();
    const std::vector<int32_t>& cptr = S.cptr;
    const std::vector<int32_t>& crow = S.crow;
    const std::vector<int32_t>& sn_parent = S.fr_parent;
    const std::vector<int32_t>& child_ptr = S.fr_child_ptr;
    const std::vector<int32_t>& children = S.fr_children;
    if (n == 0) {
        vals_out.clear();
        flops_out = 0.0;
        return ST_OK;
    }
    // ---- multifrontal numeric factorisation -----------------------------
    // On the fronts of the relaxed amalgamation (S.fr_*). Fronts whose
    // subtree holds more than 1/(4 threads) of the flops (a set closed
    // towards the roots) are factorised last, one after the other,
    // with multi-threaded dense kernels; every subtree hanging below that set
    // is an independent task, factorised by one thread. A finished front is
    // kept whole and handed to its parent: its trailing m x m block (leading
    // dimension Fsz) is the update. A parent adds its children's updates in
    // reverse child order, the order of a serial postorder stack, so results
    // do not depend on the thread count.
    vals_out.assign((size_t)total, 0.0);
    std::vector<double> sn_flops((size_t)nsn), sub_flops((size_t)nsn);
    std::vector<int32_t> first((size_t)nsn);  // first supernode of each subtree (postorder: contiguous)
    double total_flops = 0.0;
    for (int32_t s = 0; s < nsn; ++s) {
        const double w = S.fr_col[s + 1] - S.fr_col[s];
        const double m = S.fr_nr[s];
        sn_flops[s] = w * w * w / 3.0 + m * w * w + m * m * w;
        total_flops += sn_flops[s];
        sub_flops[s] = sn_flops[s];
        first[s] = s;
    }
    for (int32_t s = 0; s < nsn; ++s)
        if (sn_parent[s] >= 0) {
            sub_flops[sn_parent[s]] += sub_flops[s];
            first[sn_parent[s]] = std::min(first[sn_parent[s]], first[s]);
        }
    const double cut = threads > 1 ? total_flops / (4.0 * threads) : -1.0;
    std::vector<char> top((size_t)nsn, 0);
    for (int32_t s = 0; s < nsn; ++s) top[s] = sub_flops[s] > cut;

    // Front storage without value-initialisation: a front is first touched
    // by the (parallel, for large fronts) zeroing of its lower triangle, not
    // by a serial fill when it is allocated.
    struct Buf {
        std::unique_ptr<double[]> p;
        size_t cap = 0;
        double* data() { return p.get(); }
        const double* data() const { return p.get(); }
    };
    struct Front {
        int64_t fsz = 0, w = 0;
        Buf u;  // the whole front, column-major; the update is u[w.., w..]
    };
    std::vector<Front> upd((size_t)nsn);  // finished fronts waiting for their parent
    constexpr int64_t kParCols = 256;     // columns from which copies go parallel
    // per-thread scratch: row positions, and consumed fronts kept for reuse
    // (best fit by capacity, at most 8): a fresh multi-megabyte buffer per
    // front costs its page faults
    struct Work {
        std::vector<int32_t> relpos;
        std::vector<Buf> pool;
        void recycle(Buf& v) {
            if (v.cap == 0) return;
            pool.push_back(std::move(v));
            v = Buf();
            if (pool.size() > 8) {  // drop the smallest
                size_t k = 0;
                for (size_t i = 1; i < pool.size(); ++i)
                    if (pool[i].cap < pool[k].cap) k = i;
                pool.erase(pool.begin() + (std::ptrdiff_t)k);
            }
        }
        Buf take(size_t need) {
            Buf v;
            size_t best = pool.size();
            for (size_t i = 0; i < pool.size(); ++i)
                if (pool[i].cap >= need && (best == pool.size() || pool[i].cap < pool[best].cap)) best = i;
            if (best < pool.size()) {
                v = std::move(pool[best]);
                pool.erase(pool.begin() + (std::ptrdiff_t)best);
            } else {  // none fits: a new buffer, uninitialised
                v.p.reset(new double[need]);
                v.cap = need;
            }
            return v;
        }
    };
    std::vector<Work> work((size_t)threads);

    // Factorises supernode s with `dt` threads for its dense kernels and copies;
    // false if a pivot is not positive.
    auto factor_sn = [&](int32_t s, Work& wk, int dt) -> bool {
        if (wk.relpos.empty()) wk.relpos.assign((size_t)n, -1);
        int32_t* relpos = wk.relpos.data();
        const int32_t f = S.fr_col[s], l1 = S.fr_col[s + 1];
        const int64_t w = l1 - f;
        const int32_t* below = F.rowidx.data() + S.fr_rpos[s];  // rows below the front's columns
        const int64_t m = S.fr_nr[s];
        const int64_t Fsz = w + m;
        for (int64_t i = 0; i < w; ++i) relpos[f + i] = (int32_t)i;
        for (int64_t i = 0; i < m; ++i) relpos[below[i]] = (int32_t)(w + i);
        Buf front = wk.take((size_t)(Fsz * Fsz));
        double* fr = front.data();
        // only the lower triangle of a front is ever read (assembly, the dense
        // kernels and the update all stay on or below the diagonal): zero that
#pragma omp parallel for num_threads(dt) schedule(static) if (dt > 1 && Fsz >= kParCols)
        for (int64_t j = 0; j < Fsz; ++j) std::fill(fr + j * Fsz + j, fr + (j + 1) * Fsz, 0.0);
        // original entries of columns f..l1-1 (lower part)
        for (int32_t j = f; j < l1; ++j) {
            double* col = fr + (int64_t)(j - f) * Fsz;
            for (int32_t k = cptr[j]; k < cptr[j + 1]; ++k) col[relpos[crow[k]]] += cval[k];
        }
        // extend-add the children's updates, last child first
        for (int32_t q = child_ptr[s + 1] - 1; q >= child_ptr[s]; --q) {
            const int32_t c = children[q];
            Front& up = upd[c];
            const int32_t cw = (int32_t)up.w;
            const int32_t* crows = F.rowidx.data() + S.fr_rpos[c];
            const int64_t cm = up.fsz - cw, ld = up.fsz;
            const double* ub = up.u.data() + cw + cw * ld;  // update block (lower part)
#pragma omp parallel for num_threads(dt) schedule(dynamic, 16) if (dt > 1 && cm >= kParCols)
            for (int64_t jj = 0; jj < cm; ++jj) {
                double* dst = fr + (int64_t)relpos[crows[jj]] * Fsz;
                const double* src = ub + jj * ld;
                for (int64_t ii = jj; ii < cm; ++ii) dst[relpos[crows[ii]]] += src[ii];
            }
            wk.recycle(up.u);
            up = Front();
        }
        // partial dense factorisation of the front
        const int64_t bad = dense::potrf_lower(w, fr, Fsz, dt);
        bool ok = bad < 0;
        if (ok && m > 0) {
            dense::trsm_right_lower_t(m, w, fr, Fsz, fr + w, Fsz, dt);
            dense::gemm_nt_sub(m, m, w, fr + w, Fsz, fr + w, Fsz, fr + w + w * Fsz, Fsz, true, dt);
        }
        if (ok) {  // store the columns of L: each column's own pattern
            double* vals = vals_out.data();
            const int32_t* cp = F.colptr.data();
            const int32_t* ri = F.rowidx.data();
#pragma omp parallel for num_threads(dt) schedule(static) if (dt > 1 && w * Fsz >= kParCols * kParCols)
            for (int64_t j = 0; j < w; ++j) {
                double* dst = vals + cp[f + j];
                const int64_t len = cp[f + j + 1] - cp[f + j];
                const double* src = fr + j * Fsz;
                if (len == Fsz - j) {  // the column fills the front below its diagonal
                    for (int64_t i = 0; i < len; ++i) dst[i] = src[j + i];
                } else {
                    const int32_t* pr = ri + cp[f + j];
                    for (int64_t i = 0; i < len; ++i) dst[i] = src[relpos[pr[i]]];
                }
            }
        }
        for (int64_t i = 0; i < w; ++i) relpos[f + i] = -1;
        for (int64_t i = 0; i < m; ++i) relpos[below[i]] = -1;
        if (ok && m > 0 && sn_parent[s] >= 0) {
            upd[s].fsz = Fsz;
            upd[s].w = w;
            upd[s].u = std::move(front);  // the front itself carries the update
        } else {
            wk.recycle(front);
        }
        return ok;
    };

    // subtrees below the top set, largest first, one task each
    std::vector<int32_t> roots;
    for (int32_t s = 0; s < nsn; ++s)
        if (!top[s] && (sn_parent[s] < 0 || top[sn_parent[s]])) roots.push_back(s);
    std::stable_sort(roots.begin(), roots.end(),
                     [&](int32_t a, int32_t b) { return sub_flops[a] > sub_flops[b]; });
    int failed = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1) if (threads > 1 && roots.size() > 1)
    for (int64_t q = 0; q < (int64_t)roots.size(); ++q) {
#ifdef _OPENMP
        Work& wk = work[(size_t)omp_get_thread_num()];
#else
        Work& wk = work[0];
#endif
        const int32_t r = roots[q];
        for (int32_t s = first[r]; s <= r; ++s) {
            int stop;
#pragma omp atomic read
            stop = failed;
            if (stop) break;
            if (!factor_sn(s, wk, 1)) {
#pragma omp atomic write
                failed = 1;
                break;
            }
        }
    }
    if (!failed)
        for (int32_t s = 0; s < nsn; ++s)
            if (top[s] && !factor_sn(s, work[0], threads)) {
                failed = 1;
                break;
            }
    if (failed) {
        err = "Matrix is not positive definite!";
        return ST_NOT_POSDEF;
    }
    // reported: the flop count of the supernodal (unamalgamated) factorisation
    double flops = 0.0;
    for (size_t t = 0; t + 1 < F.sn_start.size(); ++t) {
        const double w = F.sn_start[t + 1] - F.sn_start[t];
        const double m = (double)(F.colptr[F.sn_start[t] + 1] - F.colptr[F.sn_start[t]]) - w;
        flops += w * w * w / 3.0 + m * w * w + m * m * w;
    }
    flops_out = flops;
    return ST_OK;
}

void record_input(Factor& F, int64_t nnz, const int32_t* ii, const int32_t* jj, int32_t fmt) {
    if (!F.sym) return;
    SymbolicCache& S = *F.sym;
    const int32_t n = F.n;
    const size_t ni = fmt == FMT_COO ? (size_t)nnz : (size_t)n + 1;
    S.fmt = fmt;
    S.in_i.assign(ii, ii + ni);
    S.in_j.assign(jj, jj + nnz);
    S.inmap.resize((size_t)nnz);
    // entry e of the input sits at (row, col) of A; its CSC position is found
    // in the (sorted, duplicate-free) column
    auto place = [&](int64_t e, int32_t r, int32_t c) {
        const int32_t* b0 = S.a_rowidx.data() + S.a_colptr[c];
        const int32_t* b1 = S.a_rowidx.data() + S.a_colptr[c + 1];
        S.inmap[e] = (int32_t)(std::lower_bound(b0, b1, r) - S.a_rowidx.data());
    };
    if (fmt == FMT_COO) {
        for (int64_t e = 0; e < nnz; ++e) place(e, ii[e], jj[e]);
    } else {
        for (int32_t o = 0; o < n; ++o)  // o owns entries ii[o]..ii[o+1]: a row (CSR) or a column (CSC)
            for (int32_t e = ii[o]; e < ii[o + 1]; ++e) {
                if (fmt == FMT_CSR) place(e, o, jj[e]);
                else place(e, jj[e], o);
            }
    }
}

bool refactor_cached(const Factor& F, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x,
                     int32_t fmt, int32_t threads, Csc& A, std::vector<double>& vals_out, double& flops_out,
                     Status& st, std::string& err) {
    if (!F.sym || F.sym->fmt < 0 || fmt != F.sym->fmt) return false;
    const SymbolicCache& S = *F.sym;
    const int32_t n = F.n;
    const size_t ni = fmt == FMT_COO ? (size_t)nnz : (size_t)n + 1;
    if (S.in_i.size() != ni || S.in_j.size() != (size_t)nnz) return false;
    if (ni && std::memcmp(ii, S.in_i.data(), ni * sizeof(int32_t)) != 0) return false;
    if (nnz && std::memcmp(jj, S.in_j.data(), (size_t)nnz * sizeof(int32_t)) != 0) return false;
    // duplicates summed in input order, from the first one on (as build_csc)
    A.n = n;
    A.colptr = S.a_colptr;
    A.rowidx = S.a_rowidx;
    A.vals.assign(S.a_rowidx.size(), 0.0);
    std::vector<char> seen(S.a_rowidx.size(), 0);
    for (int64_t e = 0; e < nnz; ++e) {
        const int32_t p = S.inmap[e];
        if (seen[p]) {
            A.vals[p] += x[e];
        } else {
            A.vals[p] = x[e];
            seen[p] = 1;
        }
    }
    std::vector<double> cval((size_t)S.cptr[n], 0.0);
    for (size_t k = 0; k < S.amap.size(); ++k)
        if (S.amap[k] >= 0) cval[(size_t)S.amap[k]] = A.vals[k];
    st = numeric_factor(F, S, cval, threads, vals_out, flops_out, err);
    return true;
}

}  // namespace gbchol
