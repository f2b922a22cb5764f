// tbg_eigvalsh_noalloc: band energies of device-resident Hamiltonians with no
// device allocation, for callers that cannot call cudaMalloc (their own
// allocator owns the device memory, or cudaMalloc/cudaFree would synchronise a
// latency-critical loop).  The FP64 eigensolver kernel reduces its matrices in
// place, so it works on a copy of the caller's input held in the fixed static
// array below instead of on library-allocated scratch.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "tbgpu_internal.cuh"

namespace tbg {

int eig_values_f64_inplace(cudaStream_t st, int N, int64_t batch, zc* A, double* E);

namespace {

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TBG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
// Largest n with one n x n complex FP64 matrix in the array: floor(sqrt(bytes / 16)).
constexpr int64_t kMaxNoallocN = 1448;
static_assert(16ULL * kMaxNoallocN * kMaxNoallocN <= TBG_NOALLOC_SCRATCH_BYTES &&
                  16ULL * (kMaxNoallocN + 1) * (kMaxNoallocN + 1) > TBG_NOALLOC_SCRATCH_BYTES,
              "kMaxNoallocN follows the array size");
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Set-up, once per device, with that device current: the host-side name of the
// array is not a device address, so look the address up and keep it.  The
// address belongs to the device's primary context as it is when looked up; a
// cudaDeviceReset (which reloads the module) invalidates it, so the entry point
// is not for processes that reset a device they use it on.
int scratch_address(int dev, void** out) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return TBG_OK;
}

}  // namespace
}  // namespace tbg

extern "C" int tbg_eigvalsh_noalloc(int64_t n, int64_t nk, const double* H_d, double* E_d, void* stream) {
    using namespace tbg;
    // one matrix must fit the array: 16 n^2 <= TBG_NOALLOC_SCRATCH_BYTES, n <= 1448
    if (n < 1 || 16ULL * (unsigned long long)n * (unsigned long long)n > TBG_NOALLOC_SCRATCH_BYTES)
        return set_error(TBG_E_UNSUPPORTED, "tbg_eigvalsh_noalloc: n must be in [1, " +
                                                std::to_string(kMaxNoallocN) + "] (one matrix of " +
                                                std::to_string((unsigned long long)TBG_NOALLOC_SCRATCH_BYTES) +
                                                " bytes of scratch at most)");
    if (nk < 0) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_eigvalsh_noalloc: negative nk");
    if (nk == 0) return TBG_OK;
    if (!H_d || !E_d) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_eigvalsh_noalloc: null device pointer");
    const unsigned long long per = 16ULL * (unsigned long long)n * (unsigned long long)n;
    const unsigned long long cap = TBG_NOALLOC_SCRATCH_BYTES / per;
    if ((unsigned long long)nk > cap)
        return set_error(TBG_E_UNSUPPORTED,
                         "tbg_eigvalsh_noalloc: " + std::to_string(nk) + " matrices of size " + std::to_string(n) +
                             " need " + std::to_string(per * (unsigned long long)nk) +
                             " bytes of scratch; the fixed array holds " +
                             std::to_string((unsigned long long)TBG_NOALLOC_SCRATCH_BYTES) + " bytes (at most " +
                             std::to_string(cap) + " matrices of this size per call)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return set_error(TBG_E_UNSUPPORTED, "device index out of range");
    void* scratch = nullptr;
    int rc = scratch_address(dev, &scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemcpyAsync(scratch, H_d, per * (unsigned long long)nk, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "tbg_eigvalsh_noalloc: copy into scratch");
    return eig_values_f64_inplace(st, (int)n, nk, static_cast<zc*>(scratch), E_d);
}
