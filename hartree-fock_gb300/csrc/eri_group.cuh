// Primitive-parallel form of the fused ERI + J/K kernel for low angular momentum, contracted classes.
//
// The thread-per-quartet form walks a quartet's npp_bra x npp_ket primitive quartets serially, one
// dependent load + Boys + recursion chain after the other; for the small (ss|ss) .. (pp|ps) classes that
// is latency-bound.  Here a group of g lanes (a power of two, chosen per round from the quartet's
// primitive-quartet count) shares one quartet: lane r of the group evaluates primitive quartets
// r, r+g, r+2g, ... independently, the group sums its integrals with shuffles, and one lane digests.
// The lists are ordered by bra pair and ket primitive count, so the quartets of a warp have about the
// same primitive count and the groups stay busy.  Same arithmetic per primitive quartet as eri_jk.cuh.
#pragma once

#include "eri_jk.cuh"

namespace hfg
{
#ifdef __CUDACC__
// One primitive quartet's contribution to the contracted integrals acc[NAB*NCD] (no angular factors).
template <int LA, int LB, int LC, int LD, typename Real>
__device__ __forceinline__ void eval_prim_quartet(const Real* __restrict__ rb, const Real* __restrict__ rk,
                                                  const Real* __restrict__ slice, Real* acc)
{
    constexpr int LAB = LA + LB, L = LAB + LC + LD;
    constexpr int NAB = ncart(LA) * ncart(LB), NCD = ncart(LC) * ncart(LD);
    constexpr int HAB = nherm(LAB), HL = nherm(L);
    const Real p = rb[0], q = rk[0];
    const Real X = rb[1] - rk[1], Y = rb[2] - rk[2], Z = rb[3] - rk[3];
    const Real rs   = hfg_rsqrt(p + q);
    const Real rho  = (p * q) * (rs * rs);
    const Real pref = (rb[4] * rk[4]) * rs;
    const Real T    = rho * (X * X + Y * Y + Z * Z);
    Real F[L + 1];
    boys_eval<L, Real>(T, slice, F);
    Real Fs[L + 1];
    {
        const Real m2r = Real(-2) * rho;
        Real w         = pref;
#pragma unroll
        for (int n = 0; n <= L; ++n)
        {
            Fs[n] = w * F[n];
            w *= m2r;
        }
    }
    Real R[HL];
    hermite_R<L, Real>(Fs, X, Y, Z, R);
    Real G[HAB * NCD];
    static_for<0, NCD>(
        [&](auto KL)
        {
            constexpr int kl   = decltype(KL)::value;
            constexpr int lx   = e3_len(LC, LD, kl, 0), ly = e3_len(LC, LD, kl, 1), lz = e3_len(LC, LD, kl, 2);
            constexpr int eoff = kPairHeader + e3_offset(LC, LD, kl);
            static_for<0, HAB>(
                [&](auto TUV)
                {
                    constexpr int h = decltype(TUV)::value;
                    constexpr int t = htuv(h, LAB, 0), u = htuv(h, LAB, 1), v = htuv(h, LAB, 2);
                    Real s          = Real(0);
                    static_for<0, lx * ly * lz>(
                        [&](auto EE)
                        {
                            constexpr int e   = decltype(EE)::value;
                            constexpr int tau = e % lx, nu = (e / lx) % ly, phi = e / (lx * ly);
                            const Real rr     = R[hidx(t + tau, u + nu, v + phi, L)];
                            const Real term   = (LC + LD == 0) ? rr : rk[eoff + e] * rr;
                            if constexpr (((tau + nu + phi) & 1) != 0)
                                s -= term;
                            else
                                s += term;
                        });
                    G[h * NCD + kl] = s;
                });
        });
    static_for<0, NAB>(
        [&](auto IJ)
        {
            constexpr int ij   = decltype(IJ)::value;
            constexpr int lx   = e3_len(LA, LB, ij, 0), ly = e3_len(LA, LB, ij, 1), lz = e3_len(LA, LB, ij, 2);
            constexpr int eoff = kPairHeader + e3_offset(LA, LB, ij);
#pragma unroll
            for (int kl = 0; kl < NCD; ++kl)
            {
                Real s = Real(0);
                static_for<0, lx * ly * lz>(
                    [&](auto EE)
                    {
                        constexpr int e = decltype(EE)::value;
                        constexpr int t = e % lx, u = (e / lx) % ly, v = e / (lx * ly);
                        const Real gg   = G[hidx(t, u, v, LAB) * NCD + kl];
                        s += (LA + LB == 0) ? gg : rb[eoff + e] * gg;
                    });
                acc[ij * NCD + kl] += s;
            }
        });
}

template <int LA, int LB, int LC, int LD, typename Real, bool UHF>
__global__ void __launch_bounds__(128) jk_class_group_kernel(const Quartet* __restrict__ list,
                                                             const unsigned long long* __restrict__ count, FockView v,
                                                             const Real* __restrict__ boys_slice)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* slice                = reinterpret_cast<Real*>(smem_raw);
    const unsigned long long n = *count;
    if (static_cast<unsigned long long>(blockIdx.x) * blockDim.x >= n)
        return;
    stage_boys<Real>(boys_slice, slice);
    constexpr int N = ncart(LA) * ncart(LB) * ncart(LC) * ncart(LD);
    constexpr int SB = pp_stride(LA, LB), SK = pp_stride(LC, LD);
    const Real* tb = static_cast<const Real*>(v.pptab[pair_class(LA, LB)]);
    const Real* tk = static_cast<const Real*>(v.pptab[pair_class(LC, LD)]);
    const int lane = threadIdx.x & 31;
    const unsigned long long warps = static_cast<unsigned long long>(gridDim.x) * (blockDim.x >> 5);
    // Each warp owns windows of 32 consecutive list entries.
    for (unsigned long long w0 = (static_cast<unsigned long long>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32;
         w0 < n; w0 += warps * 32)
    {
        const unsigned long long wend = min(n, w0 + 32);
        unsigned long long j = w0;
        while (j < wend)
        {
            // Group size from the round's first quartet: next power of two >= its primitive quartets.
            int P0 = 1;
            if (lane == 0)
            {
                const Quartet q0 = list[j];
                P0 = v.pairs[q0.bra].npp * v.pairs[q0.ket].npp;
            }
            P0 = __shfl_sync(0xffffffffu, P0, 0);
            int g = 1;
            while (g < P0 && g < 32) g <<= 1;
            const int sub = lane / g, r = lane % g;
            const unsigned long long qi = j + sub;
            const bool active = qi < wend;
            Real acc[N];
#pragma unroll
            for (int x = 0; x < N; ++x) acc[x] = Real(0);
            PairRec bra {}, ket {};
            Quartet qt {};
            if (active)
            {
                qt  = list[qi];
                bra = v.pairs[qt.bra];
                ket = v.pairs[qt.ket];
                const int P = bra.npp * ket.npp;
                for (int t = r; t < P; t += g)
                {
                    const int ib = t / ket.npp, ik = t - ib * ket.npp;
                    eval_prim_quartet<LA, LB, LC, LD, Real>(tb + static_cast<size_t>(bra.pp_off + ib) * SB,
                                                            tk + static_cast<size_t>(ket.pp_off + ik) * SK, slice, acc);
                }
            }
            for (int off = g >> 1; off > 0; off >>= 1)
#pragma unroll
                for (int x = 0; x < N; ++x) acc[x] += __shfl_xor_sync(0xffffffffu, acc[x], off);
            if (active && r == 0)
            {
                if (v.store != nullptr)
                {
                    static_for<0, N>(
                        [&](auto E)
                        {
                            constexpr int e  = decltype(E)::value;
                            constexpr int NB = ncart(LB), NC = ncart(LC), ND = ncart(LD), NCD = NC * ND;
                            constexpr double an = ang_norm(LA, e / NCD / NB) * ang_norm(LB, (e / NCD) % NB)
                                                * ang_norm(LC, (e % NCD) / ND) * ang_norm(LD, e % ND);
                            v.store[qi * N + e] = double(acc[e]) * an;
                        });
                }
                else
                    digest_quartet<LA, LB, LC, LD, Real, UHF>(bra, ket, qt.bra == qt.ket, acc, v);
            }
            j += 32 / g;
        }
    }
}
#endif
} // namespace hfg
