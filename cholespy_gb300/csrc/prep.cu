// Construction input prep on the GPU (sm_103a): COO / CSR / CSC arrays that
// already live on the device become the sorted, duplicate-summed CSC the host
// factorisation takes, with the same result, bit for bit, as the host
// conversion (host/sparse_prep.cpp: build_csc). Reference: the host
// conversion of src/cholesky_solver.cpp:8-149 (coo_to_csc, csr_to_csc,
// duplicates summed), which the reference runs after copying device inputs
// to the host (src/main.cpp:47-67).
//
// Steps: each entry's (column, row); counts per column and their scan (the
// column pointers); placement into columns (any order, by atomic cursors);
// a sort of each column by (row, entry index), i.e. stable by row in input
// order; then, per column, duplicates summed from the first in input order
// (the host's left-to-right sum) and the merged columns compacted.
#include <cuda_runtime.h>

#include <cstdint>

#include "prep.h"

namespace gbchol {

namespace {

constexpr int kT = 256;

// (column, row) of entry e, and the range check. fmt: 0 CSC (ii = column
// pointers, jj = rows), 1 CSR (ii = row pointers, jj = columns), 2 COO.
__global__ void entry_kernel(int32_t n, int64_t nnz, const int32_t* __restrict__ ii, const int32_t* __restrict__ jj,
                             int32_t fmt, const int32_t* __restrict__ owner, int32_t* __restrict__ col,
                             int32_t* __restrict__ row, int32_t* __restrict__ cnt, int32_t* bad) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
        int32_t r, c;
        if (fmt == 2) {
            r = ii[e];
            c = jj[e];
        } else if (fmt == 1) {
            r = owner[e];
            c = jj[e];
        } else {
            r = jj[e];
            c = owner[e];
        }
        if (r < 0 || r >= n || c < 0 || c >= n) {
            atomicExch(bad, 1);
            r = 0;
            c = 0;
        }
        row[e] = r;
        col[e] = c;
        atomicAdd(cnt + c, 1);
    }
}

// owner[e] = k for e in [ptr[k], ptr[k + 1]) (the pointer array was checked
// on the host: ptr[0] = 0, non-decreasing, ptr[n] = nnz).
__global__ void owner_kernel(int32_t n, const int32_t* __restrict__ ptr, int32_t* __restrict__ owner) {
    const int32_t stride = gridDim.x * blockDim.x;
    for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
        for (int32_t e = ptr[k]; e < ptr[k + 1]; ++e) owner[e] = k;
}

// Exclusive scan of cnt[0..n) into ptr[0..n]: each CTA scans its chunk of
// kT entries and writes the chunk's total (scan_chunks), one CTA scans the
// totals in place (scan_totals, serial over groups of kT), and the chunk
// offsets are added (scan_add).
__device__ __forceinline__ int32_t block_incl_scan(int32_t v, int32_t* s) {
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kT; off <<= 1) {  // Hillis-Steele
        const int32_t t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    return s[threadIdx.x];
}

__global__ void scan_chunks(int32_t n, const int32_t* __restrict__ cnt, int32_t* __restrict__ ptr,
                            int32_t* __restrict__ totals) {
    __shared__ int32_t s[kT];
    const int32_t i = blockIdx.x * kT + threadIdx.x;
    const int32_t v = i < n ? cnt[i] : 0;
    const int32_t inc = block_incl_scan(v, s);
    if (i < n) ptr[i] = inc - v;
    if (threadIdx.x == kT - 1) totals[blockIdx.x] = inc;
}

__global__ void scan_totals(int32_t m, int32_t* __restrict__ totals, int32_t* __restrict__ grand) {
    __shared__ int32_t s[kT];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int32_t base = 0; base < m; base += kT) {
        const int32_t i = base + threadIdx.x;
        const int32_t v = i < m ? totals[i] : 0;
        const int32_t inc = block_incl_scan(v, s);
        if (i < m) totals[i] = carry + inc - v;  // exclusive offset of chunk i
        __syncthreads();
        if (threadIdx.x == kT - 1) carry += inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void scan_add(int32_t n, const int32_t* __restrict__ totals, int32_t* __restrict__ ptr) {
    const int32_t i = blockIdx.x * kT + threadIdx.x;
    if (i < n) ptr[i] += totals[blockIdx.x];
}

cudaError_t exclusive_scan(int32_t n, const int32_t* cnt, int32_t* ptr, int32_t* totals, cudaStream_t s) {
    const int32_t chunks = (n + kT - 1) / kT;
    if (chunks > 0) {
        scan_chunks<<<chunks, kT, 0, s>>>(n, cnt, ptr, totals);
        scan_totals<<<1, kT, 0, s>>>(chunks, totals, ptr + n);
        scan_add<<<chunks, kT, 0, s>>>(n, totals, ptr);
    } else {
        cudaMemsetAsync(ptr, 0, sizeof(int32_t), s);
    }
    return cudaGetLastError();
}

__global__ void place_kernel(int64_t nnz, const int32_t* __restrict__ col, const int32_t* __restrict__ ptr,
                             int32_t* __restrict__ cursor, int32_t* __restrict__ slot) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
        const int32_t c = col[e];
        slot[ptr[c] + atomicAdd(cursor + c, 1)] = (int32_t)e;
    }
}

// Column c: its entries sorted by (row, entry index) (insertion sort: the
// columns of a sparse matrix are short), then equal rows summed in that
// order; merged[c] = the column's distinct rows.
__global__ void sort_column_kernel(int32_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ row,
                                   int32_t* __restrict__ slot, int32_t* __restrict__ merged) {
    const int32_t stride = gridDim.x * blockDim.x;
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += stride) {
        const int32_t s = ptr[c], e = ptr[c + 1];
        for (int32_t k = s + 1; k < e; ++k) {
            const int32_t v = slot[k];
            const int32_t rv = row[v];
            int32_t m = k - 1;
            while (m >= s) {
                const int32_t u = slot[m];
                const int32_t ru = row[u];
                if (ru < rv || (ru == rv && u < v)) break;
                slot[m + 1] = u;
                --m;
            }
            slot[m + 1] = v;
        }
        int32_t d = 0;
        for (int32_t k = s; k < e; ++k)
            if (k == s || row[slot[k]] != row[slot[k - 1]]) ++d;
        merged[c] = d;
    }
}

__global__ void merge_kernel(int32_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ mptr,
                             const int32_t* __restrict__ row, const int32_t* __restrict__ slot,
                             const double* __restrict__ x, int32_t* __restrict__ out_row, double* __restrict__ out_val) {
    const int32_t stride = gridDim.x * blockDim.x;
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += stride) {
        const int32_t s = ptr[c], e = ptr[c + 1];
        int32_t w = mptr[c];
        int32_t k = s;
        while (k < e) {
            const int32_t r = row[slot[k]];
            double v = x[slot[k++]];
            while (k < e && row[slot[k]] == r) v += x[slot[k++]];
            out_row[w] = r;
            out_val[w] = v;
            ++w;
        }
    }
}

__global__ void cast_kernel(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) dst[k] = (float)src[k];
}

int grid_for(int64_t items) {
    const int64_t b = (items + kT - 1) / kT;
    return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

cudaError_t device_csc(int32_t n, int64_t nnz, const int32_t* ii, const int32_t* jj, const double* x, int32_t fmt,
                       DeviceCsc& out, int* bad_index, cudaStream_t s) {
    *bad_index = 0;
    out = DeviceCsc{};
    cudaError_t e = cudaSuccess;
    int32_t *col = nullptr, *row = nullptr, *cnt = nullptr, *ptr = nullptr, *slot = nullptr, *merged = nullptr,
            *owner = nullptr, *bad = nullptr, *totals = nullptr;
    auto cleanup = [&]() {
        cudaFree(col); cudaFree(row); cudaFree(cnt); cudaFree(ptr); cudaFree(slot); cudaFree(merged);
        cudaFree(owner); cudaFree(bad); cudaFree(totals);
    };
    const size_t ne = (size_t)(nnz > 0 ? nnz : 1), nn = (size_t)n + 1;
#define PREP_TRY(x_)              \
    do {                          \
        e = (x_);                 \
        if (e != cudaSuccess) {   \
            cleanup();            \
            out.release();        \
            return e;             \
        }                         \
    } while (0)
    PREP_TRY(cudaMalloc(&col, ne * 4));
    PREP_TRY(cudaMalloc(&row, ne * 4));
    PREP_TRY(cudaMalloc(&cnt, nn * 4));
    PREP_TRY(cudaMalloc(&ptr, nn * 4));
    PREP_TRY(cudaMalloc(&slot, ne * 4));
    PREP_TRY(cudaMalloc(&merged, nn * 4));
    PREP_TRY(cudaMalloc(&bad, 4));
    PREP_TRY(cudaMalloc(&totals, ((nn + kT - 1) / kT + 1) * 4));
    PREP_TRY(cudaMemsetAsync(cnt, 0, nn * 4, s));
    PREP_TRY(cudaMemsetAsync(bad, 0, 4, s));
    if (fmt != 2) {
        PREP_TRY(cudaMalloc(&owner, ne * 4));
        owner_kernel<<<grid_for(n), kT, 0, s>>>(n, ii, owner);
        PREP_TRY(cudaGetLastError());
    }
    entry_kernel<<<grid_for(nnz), kT, 0, s>>>(n, nnz, ii, jj, fmt, owner, col, row, cnt, bad);
    PREP_TRY(cudaGetLastError());
    PREP_TRY(cudaMemcpyAsync(bad_index, bad, 4, cudaMemcpyDeviceToHost, s));
    PREP_TRY(cudaStreamSynchronize(s));
    if (*bad_index) {
        cleanup();
        return cudaSuccess;
    }
    PREP_TRY(exclusive_scan(n, cnt, ptr, totals, s));
    PREP_TRY(cudaMemsetAsync(cnt, 0, nn * 4, s));  // placement cursors
    place_kernel<<<grid_for(nnz), kT, 0, s>>>(nnz, col, ptr, cnt, slot);
    PREP_TRY(cudaGetLastError());
    sort_column_kernel<<<grid_for(n), kT, 0, s>>>(n, ptr, row, slot, merged);
    PREP_TRY(cudaGetLastError());
    PREP_TRY(cudaMalloc(&out.colptr, nn * 4));
    PREP_TRY(exclusive_scan(n, merged, out.colptr, totals, s));
    PREP_TRY(cudaMemcpyAsync(&out.nnz, out.colptr + n, 4, cudaMemcpyDeviceToHost, s));
    PREP_TRY(cudaStreamSynchronize(s));
    PREP_TRY(cudaMalloc(&out.rowidx, (size_t)(out.nnz > 0 ? out.nnz : 1) * 4));
    PREP_TRY(cudaMalloc(&out.vals, (size_t)(out.nnz > 0 ? out.nnz : 1) * 8));
    merge_kernel<<<grid_for(n), kT, 0, s>>>(n, ptr, out.colptr, row, slot, x, out.rowidx, out.vals);
    PREP_TRY(cudaGetLastError());
    PREP_TRY(cudaStreamSynchronize(s));
#undef PREP_TRY
    cleanup();
    out.n = n;
    return cudaSuccess;
}

cudaError_t cast_to_f32(const double* src, float* dst, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    cast_kernel<<<grid_for(n), kT, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

void DeviceCsc::release() {
    cudaFree(colptr);
    cudaFree(rowidx);
    cudaFree(vals);
    colptr = rowidx = nullptr;
    vals = nullptr;
}

}  // namespace gbchol
