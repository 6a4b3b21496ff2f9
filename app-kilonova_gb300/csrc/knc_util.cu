// knc_util.cu — FP64 throughput probe.
//
// The HBM and BF16 roofline denominators are measured outside this library;
// the plain FP64 stage is bound by the FP64 pipe instead, so the library
// measures that ceiling itself: independent FMA chains, explicit fma() so
// the count does not depend on contraction flags, timed with CUDA events.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/knc.h"

namespace {

constexpr int CHAINS = 8;
constexpr int ITERS = 2048;

__global__ void fp64_fma_kernel(double* out, double b, double c) {
    double a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = (double)(threadIdx.x + k) * 1e-3;
    for (int it = 0; it < ITERS; ++it) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    if (s == 1.2345) out[threadIdx.x] = s;   // never true; keeps the chains live
}

}  // namespace

extern "C" int knc_measure_fp64_peak(double* gflops) {
    if (!gflops) return KNC_ERR_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return KNC_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return KNC_ERR_CUDA;
    double* out = nullptr;
    if (cudaMalloc(&out, 1024 * sizeof(double)) != cudaSuccess) return KNC_ERR_CUDA;
    const int threads = 256;
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        fp64_fma_kernel<<<blocks, threads>>>(out, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * CHAINS * (double)ITERS * threads * (double)blocks;
        if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e9);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t err = cudaGetLastError();
    cudaFree(out);
    if (err != cudaSuccess) return KNC_ERR_CUDA;
    *gflops = best;
    return KNC_OK;
}
