// FMA throughput probe for the FP64 and FP32 SIMT pipes (roofline denominators).

#include <cuda_runtime.h>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

template <typename T>
__global__ void fma_loop_kernel(int iters, T seed, T* out) {
    T a0 = seed + threadIdx.x, a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T m = T(0.999999), c = T(1e-7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
            a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
        }
    }
    const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == T(-12345.0)) out[0] = s;  // keep the loop alive
}

template <typename T>
int time_fma(double* tflops) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    T* out = nullptr;
    TBG_CUDA(cudaMalloc(&out, sizeof(T)));
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_loop_kernel<T><<<blocks, threads>>>(64, T(1), out);  // warm-up
    cudaEventRecord(e0);
    fma_loop_kernel<T><<<blocks, threads>>>(iters, T(1), out);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    count_launch(2);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_error(e, "fma_loop_kernel");
    const double flops = 2.0 * 32.0 * iters * (double)blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return TBG_OK;
}

}  // namespace
}  // namespace tbg

extern "C" int tbg_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
    int rc = TBG_OK;
    if (fp64_tflops && (rc = tbg::time_fma<double>(fp64_tflops))) return rc;
    if (fp32_tflops && (rc = tbg::time_fma<float>(fp32_tflops))) return rc;
    return TBG_OK;
}
