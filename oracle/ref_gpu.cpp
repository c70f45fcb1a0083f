// ORACLE — test infrastructure only (never part of the product).
//
// Launches the reference's OWN GPU kernels (kernels/kernels.cu of
// rgl-epfl/cholespy v2.2.2, compiled from source into oracle/_ref/ by
// oracle/ref_build.py) with the reference's host protocol, restated here:
//   * analysis: src/cholesky_solver.cpp:299-376 (CSR uploads, one-thread
//     blocks over n rows, D2H of the levels, host counting sort :349-367);
//   * solve: src/cholesky_solver.cpp:378-432 (memset of the row flags and
//     the block ticket, n blocks of 128 threads, lower then upper sweep).
// It is used to compare the product's level analysis with the reference's own
// analysis kernels and to time the reference's GPU solve on the same factor.
// Inputs are validated first: the reference kernels wait without bound, so
// they only ever see well-formed factors here.
#include <cuda.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

bool ck(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "CUDA error");
    return false;
}

struct Tri {
    CUdeviceptr rows = 0, cols = 0, data = 0, levels = 0;
    std::vector<int32_t> lev, order;       // as produced by the reference's analysis kernel
    std::vector<int32_t> lev_seq, order_seq;  // the sequential definition of the same quantity
    int32_t max_lvl = 0, max_lvl_seq = 0;
};

// Counting sort of rows by level, stable in row id (src/cholesky_solver.cpp:349-367).
void sort_levels(const std::vector<int32_t>& lev, int32_t max_lvl, std::vector<int32_t>& order) {
    const int32_t n = (int32_t)lev.size();
    std::vector<int32_t> ptr(max_lvl + 2, 0);
    for (int32_t i = 0; i < n; ++i) ptr[1 + lev[i]]++;
    for (int32_t l = 0; l <= max_lvl; ++l) ptr[l + 1] += ptr[l];
    order.resize(n);
    for (int32_t i = 0; i < n; ++i) order[ptr[lev[i]]++] = i;
}

struct RefGpu {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction al = nullptr, au = nullptr, sl = nullptr, su = nullptr;
    int32_t n = 0;
    int dbl = 0;
    CUdeviceptr perm = 0, processed = 0, stack_id = 0, tmp = 0;
    int32_t tmp_nrhs = 0;
    Tri lo, up;
};

bool wait_stream(CUstream s, double limit_s) {
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        CUresult r = cuStreamQuery(s);
        if (r == CUDA_SUCCESS) return true;
        if (r != CUDA_ERROR_NOT_READY) return ck(r, "cuStreamQuery");
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > limit_s) {
            g_err = "reference kernel did not finish within the time limit";
            return false;
        }
    }
}

template <typename T>
bool upload(CUdeviceptr* d, const T* h, size_t n) {
    if (!ck(cuMemAlloc(d, (n ? n : 1) * sizeof(T)), "cuMemAlloc")) return false;
    return n == 0 || ck(cuMemcpyHtoD(*d, h, n * sizeof(T)), "cuMemcpyHtoD");
}

// analyze_cuda (src/cholesky_solver.cpp:299-376)
bool analyze(RefGpu* g, Tri& t, bool lower) {
    const int32_t n = g->n;
    CUdeviceptr level_ind = 0, max_lvl = 0;
    if (!ck(cuMemAlloc(&level_ind, n * sizeof(int)), "alloc")) return false;
    if (!ck(cuMemAlloc(&max_lvl, sizeof(int)), "alloc")) return false;
    ck(cuMemsetD32(level_ind, 0, n), "memset");
    ck(cuMemsetD8(g->processed, 0, n), "memset");
    ck(cuMemsetD32(max_lvl, 0, 1), "memset");
    int nn = n;
    void* args[] = {&nn, &max_lvl, &g->processed, &level_ind, &t.rows, &t.cols};
    if (!ck(cuLaunchKernel(lower ? g->al : g->au, n, 1, 1, 1, 1, 1, 0, 0, args, 0), "launch analysis"))
        return false;
    if (!wait_stream(0, 600.0)) return false;
    t.lev.resize(n);
    ck(cuMemcpyDtoH(t.lev.data(), level_ind, n * sizeof(int)), "DtoH");
    ck(cuMemcpyDtoH(&t.max_lvl, max_lvl, sizeof(int)), "DtoH");
    sort_levels(t.lev, t.max_lvl, t.order);
    // The reference's analysis kernels store row_levels[row] and then
    // analyzed_rows[row] with no fence between them (kernels/kernels.cu:
    // 28-29, 55-56), so a waiting row can observe the flag before the level
    // and read a stale 0. On GB300 this was observed to give some rows too
    // low a level. A too-low level can put a row ahead of its dependency in
    // the solve's ticket order, and the solve kernels wait without bound, so
    // the solves below are driven by the sequential definition of the same
    // levels instead (levels[] of the correct analysis; no change to the
    // kernels). The kernel's own output is kept for comparison.
    {
        std::vector<int32_t> rp(n + 1), ci;
        ck(cuMemcpyDtoH(rp.data(), t.rows, (n + 1) * sizeof(int)), "DtoH");
        ci.resize(rp[n]);
        if (rp[n]) ck(cuMemcpyDtoH(ci.data(), t.cols, rp[n] * sizeof(int)), "DtoH");
        t.lev_seq.assign(n, 0);
        t.max_lvl_seq = 0;
        for (int32_t k = 0; k < n; ++k) {
            const int32_t row = lower ? k : n - 1 - k;
            const int32_t s0 = rp[row], e0 = rp[row + 1];
            int32_t l = 0;
            for (int32_t q = lower ? s0 : s0 + 1; q < (lower ? e0 - 1 : e0); ++q)
                l = std::max(l, t.lev_seq[ci[q]] + 1);
            t.lev_seq[row] = l;
            t.max_lvl_seq = std::max(t.max_lvl_seq, l);
        }
        sort_levels(t.lev_seq, t.max_lvl_seq, t.order_seq);
    }
    bool ok = upload(&t.levels, t.order_seq.data(), n);
    cuMemFree(level_ind);
    cuMemFree(max_lvl);
    return ok;
}

void free_tri(Tri& t) {
    if (t.rows) cuMemFree(t.rows);
    if (t.cols) cuMemFree(t.cols);
    if (t.data) cuMemFree(t.data);
    if (t.levels) cuMemFree(t.levels);
}

}  // namespace

extern "C" {

const char* refgpu_last_error() { return g_err.c_str(); }

void refgpu_destroy(void* p) {
    RefGpu* g = static_cast<RefGpu*>(p);
    if (!g) return;
    cuCtxSynchronize();
    free_tri(g->lo);
    free_tri(g->up);
    if (g->perm) cuMemFree(g->perm);
    if (g->processed) cuMemFree(g->processed);
    if (g->stack_id) cuMemFree(g->stack_id);
    if (g->tmp) cuMemFree(g->tmp);
    if (g->mod) cuModuleUnload(g->mod);
    delete g;
}

// perm/colptr/rowidx/vals: the factor L in CSC (diagonal first), host arrays.
int refgpu_create(const char* cubin, int32_t n, const int32_t* perm, const int32_t* colptr,
                  const int32_t* rowidx, const double* vals, int32_t dbl, void** out) {
    *out = nullptr;
    // validate: diagonal first, sorted rows in range, permutation
    std::vector<char> seen(n, 0);
    for (int32_t k = 0; k < n; ++k) {
        if (perm[k] < 0 || perm[k] >= n || seen[perm[k]]) { g_err = "bad perm"; return 1; }
        seen[perm[k]] = 1;
    }
    for (int32_t j = 0; j < n; ++j) {
        if (colptr[j + 1] <= colptr[j] || rowidx[colptr[j]] != j) { g_err = "bad factor"; return 1; }
        for (int32_t k = colptr[j] + 1; k < colptr[j + 1]; ++k)
            if (rowidx[k] <= rowidx[k - 1] || rowidx[k] >= n) { g_err = "bad factor"; return 1; }
    }
    if (!ck(cuInit(0), "cuInit")) return 2;
    RefGpu* g = new RefGpu();
    g->n = n;
    g->dbl = dbl;
    CUdevice dev;
    CUcontext cur = nullptr;
    cuCtxGetCurrent(&cur);
    if (cur) {
        g->ctx = cur;
    } else {
        if (!ck(cuDeviceGet(&dev, 0), "cuDeviceGet") ||
            !ck(cuDevicePrimaryCtxRetain(&g->ctx, dev), "ctx") || !ck(cuCtxSetCurrent(g->ctx), "ctx")) {
            delete g;
            return 2;
        }
    }
    if (!ck(cuModuleLoad(&g->mod, cubin), "cuModuleLoad") ||
        !ck(cuModuleGetFunction(&g->al, g->mod, "analysis_lower"), "fn") ||
        !ck(cuModuleGetFunction(&g->au, g->mod, "analysis_upper"), "fn") ||
        !ck(cuModuleGetFunction(&g->sl, g->mod, dbl ? "solve_lower_double" : "solve_lower_float"), "fn") ||
        !ck(cuModuleGetFunction(&g->su, g->mod, dbl ? "solve_upper_double" : "solve_upper_float"), "fn")) {
        refgpu_destroy(g);
        return 2;
    }
    const int64_t nnz = colptr[n];
    // CSR of L (cholmod_transpose): columns ascending, diagonal last
    std::vector<int32_t> rp(n + 1, 0), ci(nnz);
    std::vector<double> rv(nnz);
    for (int64_t k = 0; k < nnz; ++k) rp[rowidx[k] + 1]++;
    for (int32_t i = 0; i < n; ++i) rp[i + 1] += rp[i];
    {
        std::vector<int32_t> nx(rp.begin(), rp.end() - 1);
        for (int32_t j = 0; j < n; ++j)
            for (int32_t k = colptr[j]; k < colptr[j + 1]; ++k) {
                int32_t d = nx[rowidx[k]]++;
                ci[d] = j;
                rv[d] = vals[k];
            }
    }
    bool ok = upload(&g->perm, perm, n) && upload(&g->lo.rows, rp.data(), n + 1) &&
              upload(&g->lo.cols, ci.data(), nnz) && upload(&g->up.rows, colptr, n + 1) &&
              upload(&g->up.cols, rowidx, nnz);
    if (ok) {
        if (dbl) {
            ok = upload(&g->lo.data, rv.data(), nnz) && upload(&g->up.data, vals, nnz);
        } else {  // FP64 -> FP32 cast on the host (src/cholesky_solver.cpp:257-271)
            std::vector<float> a(rv.begin(), rv.end()), b(vals, vals + nnz);
            ok = upload(&g->lo.data, a.data(), nnz) && upload(&g->up.data, b.data(), nnz);
        }
    }
    ok = ok && ck(cuMemAlloc(&g->processed, n ? n : 1), "alloc") && ck(cuMemAlloc(&g->stack_id, 4), "alloc");
    ok = ok && analyze(g, g->lo, true) && analyze(g, g->up, false);
    if (!ok) {
        refgpu_destroy(g);
        return 3;
    }
    *out = g;
    return 0;
}

// which = 0: the reference analysis kernel's output; 1: sequential definition.
int refgpu_levels(void* p, int32_t lower, int32_t which, int32_t* row_levels, int32_t* order,
                  int32_t* max_lvl) {
    RefGpu* g = static_cast<RefGpu*>(p);
    const Tri& t = lower ? g->lo : g->up;
    const std::vector<int32_t>& lev = which ? t.lev_seq : t.lev;
    const std::vector<int32_t>& ord = which ? t.order_seq : t.order;
    std::memcpy(row_levels, lev.data(), sizeof(int32_t) * g->n);
    std::memcpy(order, ord.data(), sizeof(int32_t) * g->n);
    *max_lvl = which ? t.max_lvl_seq : t.max_lvl;
    return 0;
}

// launch_kernel + solve_cuda (src/cholesky_solver.cpp:378-432); b and x are
// device pointers, asynchronous on `stream`.
int refgpu_solve(void* p, int32_t nrhs, uint64_t b, uint64_t x, uint64_t stream) {
    RefGpu* g = static_cast<RefGpu*>(p);
    CUstream s = reinterpret_cast<CUstream>(stream);
    if (nrhs > 128) { g_err = "The number of RHS should be less than 128."; return 1; }
    if (nrhs != g->tmp_nrhs) {
        if (g->tmp) cuMemFree(g->tmp);
        if (!ck(cuMemAlloc(&g->tmp, (size_t)nrhs * g->n * (g->dbl ? 8 : 4)), "alloc tmp")) return 2;
        g->tmp_nrhs = nrhs;
    }
    for (int pass = 0; pass < 2; ++pass) {
        const bool lower = pass == 0;
        Tri& t = lower ? g->lo : g->up;
        if (!ck(cuMemsetD8Async(g->processed, 0, g->n, s), "memset") ||
            !ck(cuMemsetD32Async(g->stack_id, 0, 1, s), "memset"))
            return 2;
        CUdeviceptr xarg = lower ? b : x;
        int nr = nrhs, nn = g->n;
        void* args[] = {&nr, &nn, &g->stack_id, &t.levels, &g->processed, &t.rows, &t.cols,
                        &t.data, &g->tmp, &xarg, &g->perm};
        if (!ck(cuLaunchKernel(lower ? g->sl : g->su, g->n, 1, 1, 128, 1, 1, 0, s, args, 0), "launch solve"))
            return 2;
    }
    return 0;
}

int refgpu_sync(double limit_s) { return wait_stream(0, limit_s) ? 0 : 1; }

}  // extern "C"
