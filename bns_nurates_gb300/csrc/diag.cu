// Diagnostics: the FP64 and FP32 fused-multiply-add rates of the current
// device, the denominators of the pipe rooflines of the opacity kernels (the
// plain path is FP64-bound, the mixed path's double-float work FP32-bound).
//
// Every thread runs 8 independent FMA chains; the grid covers every SM
// several times over.  Rate = 2 x FMA count / elapsed (CUDA events).

#include <cuda_runtime.h>

#include "../../include/bns_nurates_gb300.h"

namespace {

__global__ void dfma_chains(double* out, double b, double c, int64_t iters)
{
    double a0 = threadIdx.x * 1e-3, a1 = a0 + 1., a2 = a0 + 2., a3 = a0 + 3.;
    double a4 = a0 + 4., a5 = a0 + 5., a6 = a0 + 6., a7 = a0 + 7.;
    for (int64_t i = 0; i < iters; ++i)
    {
        a0 = fma(a0, b, c);
        a1 = fma(a1, b, c);
        a2 = fma(a2, b, c);
        a3 = fma(a3, b, c);
        a4 = fma(a4, b, c);
        a5 = fma(a5, b, c);
        a6 = fma(a6, b, c);
        a7 = fma(a7, b, c);
    }
    const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 12345.678)
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ffma_chains(float* out, float b, float c, int64_t iters)
{
    float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    for (int64_t i = 0; i < iters; ++i)
    {
        a0 = fmaf(a0, b, c);
        a1 = fmaf(a1, b, c);
        a2 = fmaf(a2, b, c);
        a3 = fmaf(a3, b, c);
        a4 = fmaf(a4, b, c);
        a5 = fmaf(a5, b, c);
        a6 = fmaf(a6, b, c);
        a7 = fmaf(a7, b, c);
    }
    const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 12345.678f)
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace

extern "C" int bnsn_fp32_peak_probe(int64_t iters, double* tflops)
{
    if (!tflops || iters < 1)
        return BNSN_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return BNSN_ERR_NO_DEVICE;
    const int threads = 256, blocks = sms * 8;
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * threads * blocks) != cudaSuccess)
        return BNSN_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    ffma_chains<<<blocks, threads>>>(out, 0.9999999f, 1e-7f, iters / 10 + 1); // warm-up
    cudaEventRecord(e0);
    ffma_chains<<<blocks, threads>>>(out, 0.9999999f, 1e-7f, iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess)
        return BNSN_ERR_CUDA;
    *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) / 1e12;
    return BNSN_OK;
}

extern "C" int bnsn_fp64_peak_probe(int64_t iters, double* tflops)
{
    if (!tflops || iters < 1)
        return BNSN_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return BNSN_ERR_NO_DEVICE;
    const int threads = 256, blocks = sms * 8;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess)
        return BNSN_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_chains<<<blocks, threads>>>(out, 0.9999999, 1e-7, iters / 10 + 1); // warm-up
    cudaEventRecord(e0);
    dfma_chains<<<blocks, threads>>>(out, 0.9999999, 1e-7, iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess)
        return BNSN_ERR_CUDA;
    *tflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) / 1e12;
    return BNSN_OK;
}
