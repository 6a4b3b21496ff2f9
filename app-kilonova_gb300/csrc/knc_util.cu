// knc_util.cu — FP64 throughput probe.
//
// The HBM and BF16 roofline denominators are measured outside this library;
// the plain FP64 stage is bound by the FP64 pipe instead, so the library
// measures that ceiling itself: independent FMA chains, explicit fma() so
// the count does not depend on contraction flags, timed with CUDA events.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/knc.h"
#include "knc_bits.cuh"

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

__global__ void conversions_kernel(const double* in, int64_t n, double* out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double x = in[k];
    const float hw = __double2float_rn(x);
    out[4 * k + 0] = (double)knc::d2f_rn(x);
    out[4 * k + 1] = (double)hw;
    out[4 * k + 2] = knc::f2d(hw);
    out[4 * k + 3] = knc::half_exact(x);
}

}  // namespace

extern "C" int knc_test_conversions(const double* in, int64_t n, double* out) {
    if (!in || !out || n <= 0) return KNC_ERR_INVALID_ARGUMENT;
    double *d_in = nullptr, *d_out = nullptr;
    if (cudaMalloc(&d_in, n * 8) != cudaSuccess) return KNC_ERR_OUT_OF_MEMORY;
    if (cudaMalloc(&d_out, n * 32) != cudaSuccess) {
        cudaFree(d_in);
        return KNC_ERR_OUT_OF_MEMORY;
    }
    cudaError_t e = cudaMemcpy(d_in, in, n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        conversions_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_in, n, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, n * 32, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    return e == cudaSuccess ? KNC_OK : KNC_ERR_CUDA;
}

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
