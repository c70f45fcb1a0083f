// gbchol_solve_noalloc: the solve of gbchol_solve for callers that must not
// allocate GPU memory while solving. No counterpart in the reference.
//
// Some callers can't call cudaMalloc at solve time: real-time or embedded
// loops whose device memory is fixed up front (an allocation there can stall
// or fail), and hosts whose allocator owns all device memory (a framework's
// caching allocator, or a memory pool the solver may not bypass). gbchol_solve may grow the solver's work array (cudaMalloc) when a
// call brings more right-hand sides than any call before; this entry point
// never allocates: its permuted-space work array is the file-scope device
// array below, of a fixed size, which every GPU that loads the library holds
// until the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (host code cannot use the array's name as a
// device pointer) and caches it per device. Make that first call before any
// stream capture. The cached address holds for the life of the process's
// context on that device; a process that calls cudaDeviceReset must not
// call this entry point afterwards.
//
// Sharing: every call (on any solver) uses the same array and leaves its
// last contents there. The solve writes every element it reads before
// reading it, so nothing needs clearing; but calls whose executions overlap
// on the GPU (other streams, other threads) race on the array and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "solver_impl.h"

using namespace gbchol;

namespace {

// Maximum work array (work_bytes): about n * nrhs * sizeof(element) bytes,
// plus the partial-sum slots of the supernodal lower sweep.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (cached).
int scratch_address(int dev, void** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(GBCHOL_EINVAL, "Device ordinal out of range.");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(GBCHOL_ECUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                          cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GBCHOL_OK;
}

}  // namespace

extern "C" {

int gbchol_solve_noalloc(gbchol_handle h, int32_t precision, int32_t nrhs, const void* b, void* x,
                         void* stream) {
    if (!h) return fail(GBCHOL_EINVAL, "Null handle.");
    if (nrhs > GBCHOL_MAX_RHS) return fail(GBCHOL_EINVAL, "The number of RHS should be less than 128.");
    if (nrhs < 1) return fail(GBCHOL_EINVAL, "The number of RHS must be at least 1.");
    if (precision != 0 && precision != 1) return fail(GBCHOL_EINVAL, "precision must be 0 or 1.");
    const bool f32 = precision == 0;
    if (!(h->store & (f32 ? GBCHOL_STORE_F32 : GBCHOL_STORE_F64)))
        return fail(GBCHOL_ESTATE, f32 ? "This solver keeps no FP32 factor." : "This solver keeps no FP64 factor.");
    const size_t bytes = work_bytes(h, nrhs, f32);
    if (bytes > kNoAllocScratchBytes)
        return fail(GBCHOL_EINVAL, "gbchol_solve_noalloc: the solve's work array (" + std::to_string(bytes) +
                                       " bytes) exceeds the 16 MiB static work array; use gbchol_solve.");
    if (h->n == 0) return GBCHOL_OK;
    if (!b || !x) return fail(GBCHOL_EINVAL, "Null b or x.");
    DeviceGuard g(h->device);
    void* work = nullptr;
    if (int rc = scratch_address(h->device, &work)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (int rc = run_sweeps_with(h, f32, f32 ? SweepIO::F32 : SweepIO::F64, nrhs, b, x, nullptr, work, s))
        return rc;
    h->last_stream = s;
    return GBCHOL_OK;
}

}  // extern "C"
