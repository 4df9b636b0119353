// FMA-throughput probe: the measured denominator of the ERI kernels' roofline (FP64 and FP32 CUDA-core
// pipes; the bandwidth and tensor peaks of the pool do not bound these kernels).  The FP64 tensor-core
// probe (DMMA, mma.sync m8n8k4 f64: Blackwell's tcgen05 has no f64 kind) measures the only FP64 matrix
// path against the FP64 FMA pipe, for the Hermite-to-Cartesian contraction decision.
#include "hfgpu.h"

#include <cuda_runtime.h>

namespace
{
template <typename T> __global__ void fma_loop(T* out, int iters, T a, T b)
{
    T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i)
    {
        x0 = x0 * a + b;
        x1 = x1 * a + b;
        x2 = x2 * a + b;
        x3 = x3 * a + b;
        x4 = x4 * a + b;
        x5 = x5 * a + b;
        x6 = x6 * a + b;
        x7 = x7 * a + b;
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == T(12345.678))
        out[blockIdx.x * blockDim.x + threadIdx.x] = s; // never true; keeps the loop alive
}

// Four independent m8n8k4 f64 accumulator chains per warp.
__global__ void dmma_loop(double* out, int iters, double a, double b)
{
    double c[4][2];
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        c[k][0] = threadIdx.x * 1e-3 + k;
        c[k][1] = c[k][0] + 0.5;
    }
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                         : "+d"(c[k][0]), "+d"(c[k][1])
                         : "d"(a), "d"(b));
    }
    const double s = (c[0][0] + c[0][1]) + (c[1][0] + c[1][1]) + (c[2][0] + c[2][1]) + (c[3][0] + c[3][1]);
    if (s == 12345.678)
        out[blockIdx.x * blockDim.x + threadIdx.x] = s; // never true; keeps the loop alive
}

double run_dmma(int device, int iters)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess)
        return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dmma_loop<<<blocks, threads>>>(out, iters / 10, 0.999999, 1e-7);
    cudaEventRecord(e0);
    dmma_loop<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f)
        return -1.0;
    const double flops = 2.0 * 8 * 8 * 4 * 4.0 * iters * static_cast<double>(blocks) * (threads / 32);
    return flops / (ms * 1e-3) / 1e12;
}

template <typename T> double run(int device, int iters)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess)
        return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_loop<T><<<blocks, threads>>>(out, iters / 10, T(0.999999), T(1e-7));
    cudaEventRecord(e0);
    fma_loop<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f)
        return -1.0;
    const double flops = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads;
    return flops / (ms * 1e-3) / 1e12;
}
} // namespace

extern "C" int hfg_measure_fma_peak(int device, int fp64, double* tflops)
{
    if (!tflops)
        return HFG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess)
        return HFG_ERR_CUDA;
    const double r = fp64 ? run<double>(device, 1 << 14) : run<float>(device, 1 << 17);
    if (r <= 0)
        return HFG_ERR_CUDA;
    *tflops = r;
    return HFG_OK;
}

extern "C" int hfg_measure_dmma_peak(int device, double* tflops)
{
    if (!tflops)
        return HFG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess)
        return HFG_ERR_CUDA;
    const double r = run_dmma(device, 1 << 12);
    if (r <= 0)
        return HFG_ERR_CUDA;
    *tflops = r;
    return HFG_OK;
}
