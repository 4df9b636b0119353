// hfg_boys_eval: the device Boys function of the ERI kernels (boys.cuh), evaluated on an array of T values,
// for known-answer tests against the reference's Boys::calculateBoys (src/Boys.cpp:14-71) and the
// convergent series.  Same code path as the class kernels: the slice of the requested top order is staged
// in shared memory and boys_eval<L, Real> fills F_0 .. F_L.
#include "boys.cuh"
#include "hfgpu.h"

#include <cuda_runtime.h>

#include <vector>

namespace
{
template <int L, typename Real>
__global__ void boys_eval_kernel(const double* __restrict__ T, long long n, const Real* __restrict__ slice_g,
                                 double* __restrict__ F)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* slice = reinterpret_cast<Real*>(smem_raw);
    constexpr int kVals = hfg::BoysGrid<Real>::kPoints * hfg::BoysGrid<Real>::kRow;
    for (int i = threadIdx.x; i < kVals; i += blockDim.x) slice[i] = slice_g[i];
    __syncthreads();
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        Real f[L + 1];
        hfg::boys_eval<L, Real>(static_cast<Real>(T[i]), slice, f);
#pragma unroll
        for (int m = 0; m <= L; ++m) F[i * (L + 1) + m] = static_cast<double>(f[m]);
    }
}

template <typename Real> cudaError_t launch_boys(int L, const double* T, long long n, const Real* slice, double* F)
{
    const size_t smem = sizeof(Real) * hfg::BoysGrid<Real>::kPoints * hfg::BoysGrid<Real>::kRow;
    const int blocks  = static_cast<int>(n / 256 + 1 < 1024 ? n / 256 + 1 : 1024);
    switch (L)
    {
#define HFG_BOYS_CASE(LL)                                                                                              \
    case LL: boys_eval_kernel<LL, Real><<<blocks, 256, smem>>>(T, n, slice, F); break;
        HFG_BOYS_CASE(0) HFG_BOYS_CASE(1) HFG_BOYS_CASE(2) HFG_BOYS_CASE(3) HFG_BOYS_CASE(4)
        HFG_BOYS_CASE(5) HFG_BOYS_CASE(6) HFG_BOYS_CASE(7) HFG_BOYS_CASE(8) HFG_BOYS_CASE(9)
#undef HFG_BOYS_CASE
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename Real> int run(int device, int L, long long n, const double* T, double* F)
{
    if (cudaSetDevice(device) != cudaSuccess)
        return HFG_ERR_CUDA;
    const std::vector<Real> slice = hfg::boys_slice_host<Real>(L);
    double *dT = nullptr, *dF = nullptr;
    Real* dS   = nullptr;
    int rc     = HFG_OK;
    const size_t nF = static_cast<size_t>(n) * (L + 1);
    if (cudaMalloc(&dT, sizeof(double) * n) != cudaSuccess || cudaMalloc(&dF, sizeof(double) * nF) != cudaSuccess ||
        cudaMalloc(&dS, sizeof(Real) * slice.size()) != cudaSuccess)
        rc = HFG_ERR_NOMEM;
    if (rc == HFG_OK && (cudaMemcpy(dT, T, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
                         cudaMemcpy(dS, slice.data(), sizeof(Real) * slice.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
                         launch_boys<Real>(L, dT, n, dS, dF) != cudaSuccess ||
                         cudaMemcpy(F, dF, sizeof(double) * nF, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = HFG_ERR_CUDA;
    cudaFree(dT);
    cudaFree(dF);
    cudaFree(dS);
    return rc;
}
} // namespace

extern "C" int hfg_boys_eval(int device, int m_max, int fp32, long long n, const double* T, double* F)
{
    if (m_max < 0 || m_max > hfg::kMaxLt + 1 || n <= 0 || !T || !F)
        return HFG_ERR_INVALID;
    for (long long i = 0; i < n; ++i)
        if (!(T[i] >= 0.0) || !(T[i] < 1e300))
            return HFG_ERR_INVALID;
    return fp32 ? run<float>(device, m_max, n, T, F) : run<double>(device, m_max, n, T, F);
}
