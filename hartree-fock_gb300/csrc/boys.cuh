// Boys function F_m(T) for the ERI kernels.
//
// Same scheme as the reference (src/Boys.cpp:14-71, after Weiss & Ochsenfeld, J. Comput. Chem. 36,
// 1390 (2015)): tabulate F_m on a uniform T grid, obtain F at an off-grid T by a Taylor expansion
// about a grid point using dF_m/dT = -F_{m+1}, then fill the lower orders by recursion; for T > 30 the
// asymptotic form F_0 = sqrt(pi/T)/2, F_{m+1} = (m+1/2) F_m / T.
//
// GB300 adaptation: the reference's grid (600,001 points x 34 orders of FP64 = 163 MB, 3 Taylor
// terms) cannot live in shared memory.  Here each kernel stages a class-specific slice in shared
// memory: only the K orders F_L .. F_{L+K-1} that the Taylor expansion of the top order needs (lower
// orders come from the downward recursion F_{m-1} = (2T F_m + e^{-T}) / (2m-1), stable for all T), each
// pre-divided by k!, plus e^{-T_i} so that e^{-T} = e^{-T_i} e^{-d} needs only a short series:
//
//            step h   Taylor terms K   points        slice size (L fixed)
//   FP64     0.05     7                601 (+1)      602 x 8 doubles = 38.5 KB
//   FP32     0.10     5                301 (+1)      302 x 6 floats  =  7.2 KB
//
// Nearest-point expansion keeps |d| <= h/2, so the truncation error is below (h/2)^K / K! relative:
// 1.2e-15 (FP64) and 2.6e-9 (FP32).
#pragma once

#include "hfg_common.cuh"

#include <cmath>
#include <vector>

namespace hfg
{
template <typename Real> struct BoysGrid;
template <> struct BoysGrid<double>
{
    static constexpr double kStep    = 0.05;
    static constexpr double kInvStep = 20.0;
    static constexpr int kTerms      = 7;
    static constexpr int kPoints     = 602;
    static constexpr int kRow        = kTerms + 1; // K scaled orders + e^{-T_i}
};
template <> struct BoysGrid<float>
{
    static constexpr double kStep    = 0.1;
    static constexpr double kInvStep = 10.0;
    static constexpr int kTerms      = 5;
    static constexpr int kPoints     = 302;
    static constexpr int kRow        = kTerms + 1;
};
constexpr double kBoysAsymptotic = 30.0;
constexpr double kSqrtPiBy2      = 0.88622692545275801365; // sqrt(pi)/2

// Host: F_m(T) from the convergent series F_m(T) = e^{-T}/2 * sum_i T^i / ((m+1/2)(m+3/2)...(m+i+1/2)),
// summed in long double until the terms stop changing the sum.
inline long double boys_series_host(int m, long double T)
{
    long double term = 1.0L / (m + 0.5L), sum = term;
    for (int i = 1; i < 2000; ++i)
    {
        term *= T / (m + i + 0.5L);
        const long double s2 = sum + term;
        if (s2 == sum)
            break;
        sum = s2;
    }
    return sum * std::exp(-T) / 2.0L;
}

// Host: the slice a class of total angular momentum L needs, row-major [point][kRow].
template <typename Real> std::vector<Real> boys_slice_host(int L)
{
    using G = BoysGrid<Real>;
    std::vector<Real> out(static_cast<size_t>(G::kPoints) * G::kRow);
    for (int i = 0; i < G::kPoints; ++i)
    {
        const long double Ti = i * static_cast<long double>(G::kStep);
        long double kfact    = 1.0L;
        for (int k = 0; k < G::kTerms; ++k)
        {
            if (k > 0)
                kfact *= k;
            out[static_cast<size_t>(i) * G::kRow + k] = static_cast<Real>(boys_series_host(L + k, Ti) / kfact);
        }
        out[static_cast<size_t>(i) * G::kRow + G::kTerms] = static_cast<Real>(std::exp(-Ti));
    }
    return out;
}

// 1/k! for the e^x series.
__host__ __device__ constexpr double inv_fact(int k)
{
    double f = 1.0;
    for (int i = 2; i <= k; ++i) f *= i;
    return 1.0 / f;
}
// y = t + magic rounds t to an integer held in the low bits of y: 1.5 * 2^52 (double), 1.5 * 2^23 (float).
template <typename Real> constexpr double kRoundMagic = 0.0;
template <> constexpr double kRoundMagic<double> = 6755399441055744.0;
template <> constexpr double kRoundMagic<float>  = 12582912.0;
template <typename Real> constexpr int kRoundMagicLow = 0;
template <> constexpr int kRoundMagicLow<double> = 0;          // low 32 bits of 1.5*2^52 are zero
template <> constexpr int kRoundMagicLow<float>  = 0x400000;   // mantissa of 1.5*2^23

#ifdef __CUDACC__
__device__ __forceinline__ int bits_low(double y) { return __double2loint(y); }
__device__ __forceinline__ int bits_low(float y) { return __float_as_int(y) & 0x7fffff; }
__device__ __forceinline__ double hfg_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float hfg_rsqrt(float x) { return rsqrtf(x); }

// F[0..L] at T from the staged slice (shared memory) of this class.
template <int L, typename Real> __device__ __forceinline__ void boys_eval(Real T, const Real* __restrict__ slice, Real* F)
{
    using G = BoysGrid<Real>;
    if (T > Real(kBoysAsymptotic))
    {
        const Real r    = hfg_rsqrt(T);
        const Real invT = r * r;
        F[0]            = Real(kSqrtPiBy2) * r;
#pragma unroll
        for (int m = 0; m < L; ++m) F[m + 1] = (Real(m) + Real(0.5)) * invT * F[m];
        return;
    }
    // Nearest grid point without a float->int conversion: adding 1.5*2^52 leaves round(T/h) in the low
    // mantissa bits (T is finite and >= 0 here; the clamp keeps a corrupt T inside the slice).
    const Real y  = T * Real(G::kInvStep) + Real(kRoundMagic<Real>);
    const int pt  = max(0, min(static_cast<int>(bits_low(y) - kRoundMagicLow<Real>), G::kPoints - 1));
    const Real x  = (y - Real(kRoundMagic<Real>)) * Real(G::kStep) - T; // T_i - T
    const Real* g = slice + pt * G::kRow;
    Real f        = g[G::kTerms - 1];
#pragma unroll
    for (int k = G::kTerms - 2; k >= 0; --k) f = f * x + g[k];
    F[L] = f;
    if constexpr (L > 0)
    {
        // e^{-T} = e^{-T_i} * e^{x}, x = T_i - T, |x| <= h/2: series to the same order as the Taylor part.
        Real ex = Real(inv_fact(G::kTerms));
#pragma unroll
        for (int k = G::kTerms - 1; k >= 0; --k) ex = ex * x + Real(inv_fact(k));
        const Real e    = g[G::kTerms] * ex;
        const Real twoT = T + T;
#pragma unroll
        for (int m = L; m >= 1; --m) F[m - 1] = (twoT * F[m] + e) * Real(1.0 / (2 * m - 1));
    }
}
#endif
} // namespace hfg
