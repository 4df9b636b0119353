// Fused McMurchie-Davidson ERI evaluation + J/K digestion for one shell-quartet class.
//
// Reference counterpart: IntegralEngine::electronRepulsion (src/IntegralEngine.cpp:731-992) fused with
// the digestion loop of SCF::buildFockMatrixDirect (src/SCF.cpp:630-711).
//
// One thread evaluates one surviving shell quartet (ab|cd) of class (LA LB | LC LD), LA >= LB,
// LC >= LD, with every loop over Cartesian components, Hermite indices and expansion coefficients
// unrolled at compile time (static_for), so the R, G and ERI arrays are register arrays.  The
// contraction order per quartet:
//
//   for each bra primitive pair:   G[tuv][kl] = sum_{ket prims} sum_{tau nu phi} (-1)^{tau+nu+phi}
//                                               E^{kl}_{tau nu phi} R_{t+tau, u+nu, v+phi}
//                                  ERI[ij][kl] += sum_{tuv} E^{ij}_{tuv} G[tuv][kl]
//
// with R^n_{000} = pref * (-2 rho)^n F_n (the Boys values carry the whole primitive prefactor
// 2 pi^{5/2} / (p q sqrt(p+q)) * K_ab K_cd * coefficients * radial norms).  The 3-D Hermite tables
// E^{ij}_{tuv} of each primitive pair are precomputed once per engine (they depend only on the pair),
// which removes the per-quartet E recursion of the reference (IntegralEngine.cpp:805-820).
//
// Digestion: with s = (a==b ? 1/2 : 1)(c==d ? 1/2 : 1)(ab==cd ? 1/2 : 1) and v = s*(ij|kl),
//   X[i,j] += 2 v dDt[k,l]    X[k,l] += 2 v dDt[i,j]
//   Y[i,k] += v dDs[j,l]      Y[i,l] += v dDs[j,k]    Y[j,k] += v dDs[i,l]    Y[j,l] += v dDs[i,k]
// and afterwards J = X + X^T, K = Y + Y^T.  This covers every permutation of every unique integral once,
// which is what the reference's AO-level symmetry factors (SCF.cpp:665-707) achieve; the reference's
// AO-level skip |(ij|kl)| < SCHWARTZ_THRESH (SCF.cpp:669-671) is applied to the same contracted values.
// Per-quartet partial sums are formed in registers and added to X/Y once per quartet.
#pragma once

#include "boys.cuh"
#include "hfg_common.cuh"

namespace hfg
{
constexpr double kTwoPi25 = 34.98683665524972497; // 2 pi^{5/2}

// Device view of everything a class kernel needs.
struct FockView
{
    const PairRec* pairs;
    const void* pptab[kNumPairClasses]; // per pair class: primitive-pair records (Real of the kernel)
    // Per pair class: the same records field-major, value f of primitive slot s at [f * kfs + s].  Slots
    // follow the sorted class lists, so consecutive kets of a list read consecutive addresses.
    const void* ksoa[kNumPairClasses];
    long long kfs[kNumPairClasses];
    const void* Dt;                     // dD_tot   (double for FP64 kernels, float for FP32 kernels)
    const void* Da;                     // dD_alpha
    const void* Db;                     // dD_beta (UHF)
    double* X;                          // J accumulator (J = X + X^T)
    double* Ya;                         // K_alpha accumulator
    double* Yb;                         // K_beta accumulator (UHF)
    const long long* mat_off;           // per molecule: offset of its n x n block in the packed matrices
    const int* mat_ld;                  // per molecule: n
    double ao_thr;                      // AO-level skip threshold (SCHWARTZ_THRESH)
    float ao_thr_f;                     // the same threshold for the FP32 kernels
    double* store;                      // if set: write the quartets' integrals here instead of digesting
};

__device__ constexpr double ang_norm(int l, int c)
{
    const int i = cart_exp(l, c, 0), j = cart_exp(l, c, 1), k = cart_exp(l, c, 2);
    const int d = dfact_odd(2 * i - 1) * dfact_odd(2 * j - 1) * dfact_odd(2 * k - 1);
    return d == 1 ? 1.0 : (d == 3 ? 0.57735026918962576451 : (d == 9 ? 1.0 / 3.0 : (d == 15 ? 0.25819888974716112568 : 1.0)));
}

// Enumerates Hermite triples of total degree <= L by descending degree: k-th entry's hidx(., ., ., L).
__host__ __device__ constexpr int herm_desc(int k, int L)
{
    int n = 0;
    for (int d = L; d >= 0; --d)
        for (int v = 0; v <= d; ++v)
            for (int u = 0; u <= d - v; ++u)
            {
                if (n == k)
                    return hidx(d - u - v, u, v, L);
                ++n;
            }
    return 0;
}

// R^0_{tuv} for t+u+v <= L into R[hidx(t,u,v,L)], from Fs[n] = pref (-2 rho)^n F_n, in place,
// level by level (IntegralEngine.cpp:1082-1162 computes the same recursion in a dense 4-D buffer).
template <int L, typename Real>
__device__ __forceinline__ void hermite_R(const Real* Fs, Real X, Real Y, Real Z, Real* R)
{
    R[0] = Fs[L];
    static_for<0, L>(
        [&](auto NN)
        {
            constexpr int n = L - 1 - decltype(NN)::value;
            static_for<0, nherm(L)>(
                [&](auto KK)
                {
                    constexpr int h = herm_desc(decltype(KK)::value, L);
                    constexpr int t = htuv(h, L, 0), u = htuv(h, L, 1), v = htuv(h, L, 2);
                    constexpr int d = t + u + v;
                    if constexpr (d >= 1 && d <= L - n)
                    {
                        if constexpr (t > 0)
                        {
                            if constexpr (t >= 2)
                                R[h] = X * R[hidx(t - 1, u, v, L)] + Real(t - 1) * R[hidx(t - 2, u, v, L)];
                            else
                                R[h] = X * R[hidx(t - 1, u, v, L)];
                        }
                        else if constexpr (u > 0)
                        {
                            if constexpr (u >= 2)
                                R[h] = Y * R[hidx(t, u - 1, v, L)] + Real(u - 1) * R[hidx(t, u - 2, v, L)];
                            else
                                R[h] = Y * R[hidx(t, u - 1, v, L)];
                        }
                        else
                        {
                            if constexpr (v >= 2)
                                R[h] = Z * R[hidx(t, u, v - 1, L)] + Real(v - 1) * R[hidx(t, u, v - 2, L)];
                            else
                                R[h] = Z * R[hidx(t, u, v - 1, L)];
                        }
                    }
                });
            R[0] = Fs[n];
        });
}

// Field f of one primitive-pair record: records stored whole (AoS) or field-major (SoA, stride fs).
template <typename Real, bool SoA> struct RecRef
{
    const Real* __restrict__ p;
    long long fs;
    __device__ __forceinline__ Real operator[](int f) const
    {
        if constexpr (SoA)
            return p[f * fs];
        else
            return p[f];
    }
};

// Contracted Cartesian integrals of one quartet (without the angular normalisation factors), for the ket
// components kl in [KL0, KL1) (all of them by default): acc[ij * (KL1 - KL0) + kl - KL0].  KSoA: the ket
// table tk is field-major with field stride kfs.
template <int LA, int LB, int LC, int LD, typename Real, bool KSoA = false, int KL0 = 0,
          int KL1 = ncart(LC) * ncart(LD)>
__device__ __forceinline__ void eval_quartet(const PairRec& bra, const PairRec& ket, const Real* __restrict__ tb,
                                             const Real* __restrict__ tk, const Real* __restrict__ slice,
                                             Real* acc, long long kfs = 0)
{
    constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
    constexpr int NAB = ncart(LA) * ncart(LB), NCD = KL1 - KL0;
    constexpr int HAB = nherm(LAB), HL = nherm(L);
    constexpr int SB = pp_stride(LA, LB), SK = pp_stride(LC, LD);
#pragma unroll
    for (int x = 0; x < NAB * NCD; ++x) acc[x] = Real(0);

    for (int ib = 0; ib < bra.npp; ++ib)
    {
        const Real* __restrict__ rb = tb + static_cast<size_t>(bra.pp_off + ib) * SB;
        const Real p = rb[0], Px = rb[1], Py = rb[2], Pz = rb[3], Wab = rb[4];
        Real G[HAB * NCD];
#pragma unroll
        for (int x = 0; x < HAB * NCD; ++x) G[x] = Real(0);

        for (int ik = 0; ik < ket.npp; ++ik)
        {
            const RecRef<Real, KSoA> rk {KSoA ? tk + (ket.kslot + static_cast<long long>(ik) * ket.kstep)
                                              : tk + static_cast<size_t>(ket.pp_off + ik) * SK,
                                         kfs};
            const Real q = rk[0];
            const Real X = Px - rk[1], Y = Py - rk[2], Z = Pz - rk[3];
            const Real rs   = hfg_rsqrt(p + q);
            const Real rho  = (p * q) * (rs * rs);
            const Real pref = (Wab * rk[4]) * rs;
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

            static_for<KL0, KL1>(
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
                            G[h * NCD + (kl - KL0)] += s;
                        });
                });
        }

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
                            const Real gg = G[hidx(t, u, v, LAB) * NCD + kl];
                            s += (LA + LB == 0) ? gg : rb[eoff + e] * gg;
                        });
                    acc[ij * NCD + kl] += s;
                }
            });
    }
}

// Widening to double for the FP64 accumulators without the FP64 pipe (GB300 runs float -> double
// conversions there, at 1/64 of the FP32 rate): the IEEE-754 fields are moved with integer operations.
// Exact for normal numbers and zero; float subnormals (< 1.2e-38) become zero; infinities and NaNs keep
// their class.
__device__ __forceinline__ double widen(float x)
{
    const unsigned u                 = __float_as_uint(x);
    const unsigned e                 = (u >> 23) & 0xffu;
    const unsigned long long sign    = static_cast<unsigned long long>(u & 0x80000000u) << 32;
    const unsigned long long de      = e == 0xffu ? 0x7ffull : static_cast<unsigned long long>(e + 896u);
    const unsigned long long normal  = sign | (de << 52) | (static_cast<unsigned long long>(u & 0x7fffffu) << 29);
    return __longlong_as_double(static_cast<long long>(e == 0u ? sign : normal));
}
__device__ __forceinline__ double widen(double x) { return x; }

template <typename Real> __device__ __forceinline__ Real ao_threshold(const FockView& v)
{
    if constexpr (sizeof(Real) == 4)
        return v.ao_thr_f;
    else
        return v.ao_thr;
}

template <typename Real> __device__ __forceinline__ Real ldD(const void* p, long long i)
{
    return static_cast<const Real*>(p)[i];
}

// Density values one quartet's digestion reads: dD_tot over (cd) and (ab); per spin, the exchange
// partners (bd), (bc), (ad), (ac).
template <int LA, int LB, int LC, int LD, typename Real, bool UHF> struct DigestD
{
    static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    static constexpr int NS = UHF ? 2 : 1;
    static constexpr int kCount = NA * NB + NC * ND + NS * (NB * ND + NB * NC + NA * ND + NA * NC);
    // FP32 kernels (memory-latency bound) load them before the primitive loop, so the loads overlap the
    // integral evaluation, when they fit in about 40 registers; FP64 kernels (FP64-pipe bound) right
    // before the digestion.
    static constexpr bool kEarly = sizeof(Real) == 4 && kCount <= 40;
    Real Dcd[NC * ND], Dab[NA * NB];
    Real Dbd[NS][NB * ND], Dbc[NS][NB * NC], Dad[NS][NA * ND], Dac[NS][NA * NC];
};

template <int LA, int LB, int LC, int LD, typename Real, bool UHF>
__device__ __forceinline__ void load_digest_d(const PairRec& bra, const PairRec& ket, const FockView& v,
                                              DigestD<LA, LB, LC, LD, Real, UHF>& d)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    const long long off = v.mat_off[bra.mol];
    const int n         = v.mat_ld[bra.mol];
    const int a0 = bra.ao1, b0 = bra.ao2, c0 = ket.ao1, d0 = ket.ao2;
    auto at = [&](int r, int c) -> long long { return off + r + static_cast<long long>(c) * n; };
#pragma unroll
    for (int k = 0; k < NC; ++k)
#pragma unroll
        for (int l = 0; l < ND; ++l) d.Dcd[k * ND + l] = ldD<Real>(v.Dt, at(c0 + k, d0 + l));
#pragma unroll
    for (int i = 0; i < NA; ++i)
#pragma unroll
        for (int j = 0; j < NB; ++j) d.Dab[i * NB + j] = ldD<Real>(v.Dt, at(a0 + i, b0 + j));
#pragma unroll
    for (int spin = 0; spin < (UHF ? 2 : 1); ++spin)
    {
        const void* Ds = spin == 0 ? v.Da : v.Db;
#pragma unroll
        for (int j = 0; j < NB; ++j)
        {
#pragma unroll
            for (int l = 0; l < ND; ++l) d.Dbd[spin][j * ND + l] = ldD<Real>(Ds, at(b0 + j, d0 + l));
#pragma unroll
            for (int k = 0; k < NC; ++k) d.Dbc[spin][j * NC + k] = ldD<Real>(Ds, at(b0 + j, c0 + k));
        }
#pragma unroll
        for (int i = 0; i < NA; ++i)
        {
#pragma unroll
            for (int l = 0; l < ND; ++l) d.Dad[spin][i * ND + l] = ldD<Real>(Ds, at(a0 + i, d0 + l));
#pragma unroll
            for (int k = 0; k < NC; ++k) d.Dac[spin][i * NC + k] = ldD<Real>(Ds, at(a0 + i, c0 + k));
        }
    }
}

// Ket components kl in [KL0, KL1) that touch ket Cartesian index k (of shell c) or l (of shell d).
template <int ND, int KL0, int KL1> __host__ __device__ constexpr bool chunk_has_k(int k)
{
    for (int kl = KL0; kl < KL1; ++kl)
        if (kl / ND == k)
            return true;
    return false;
}
template <int ND, int KL0, int KL1> __host__ __device__ constexpr bool chunk_has_l(int l)
{
    for (int kl = KL0; kl < KL1; ++kl)
        if (kl % ND == l)
            return true;
    return false;
}

// Digestion of one evaluated quartet into X, Ya (, Yb), with its density values already loaded; acc holds
// the integrals of the ket components kl in [KL0, KL1) (all of them by default), and only the output
// elements those components reach are added.
// bra_warp: every lane of the warp calls this together and all active lanes hold the same bra pair;
// the bra's Coulomb block X_ab is then summed over the warp and added once (inactive lanes pass
// active = false and acc = 0).  Otherwise each active lane adds its own.
template <int LA, int LB, int LC, int LD, typename Real, bool UHF, int KL0 = 0, int KL1 = ncart(LC) * ncart(LD)>
__device__ __forceinline__ void digest_loaded(const PairRec& bra, const PairRec& ket, bool same_pair, const Real* acc,
                                              const FockView& v, const DigestD<LA, LB, LC, LD, Real, UHF>& d,
                                              bool active, bool bra_warp)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, CH = KL1 - KL0;
    const long long off = v.mat_off[bra.mol];
    const int n         = v.mat_ld[bra.mol];
    const Real s   = (bra.same ? Real(0.5) : Real(1)) * (ket.same ? Real(0.5) : Real(1)) * (same_pair ? Real(0.5) : Real(1));
    const Real thr = ao_threshold<Real>(v);
    const int a0 = bra.ao1, b0 = bra.ao2, c0 = ket.ao1, d0 = ket.ao2;
    auto at = [&](int r, int c) -> long long { return off + r + static_cast<long long>(c) * n; };

    Real Jab[NAB], Jcd[CH];
#pragma unroll
    for (int x = 0; x < NAB; ++x) Jab[x] = Real(0);
#pragma unroll
    for (int x = 0; x < CH; ++x) Jcd[x] = Real(0);

    constexpr int nspin = UHF ? 2 : 1;
#pragma unroll
    for (int spin = 0; spin < nspin; ++spin)
    {
        Real Kac[NA * NC], Kad[NA * ND], Kbc[NB * NC], Kbd[NB * ND];
#pragma unroll
        for (int x = 0; x < NA * NC; ++x) Kac[x] = Real(0);
#pragma unroll
        for (int x = 0; x < NA * ND; ++x) Kad[x] = Real(0);
#pragma unroll
        for (int x = 0; x < NB * NC; ++x) Kbc[x] = Real(0);
#pragma unroll
        for (int x = 0; x < NB * ND; ++x) Kbd[x] = Real(0);

        static_for<0, NA>(
            [&](auto I)
            {
                constexpr int i = decltype(I)::value;
                static_for<0, NB>(
                    [&](auto Jx)
                    {
                        constexpr int j = decltype(Jx)::value;
                        static_for<KL0, KL1>(
                            [&](auto KLx)
                            {
                                constexpr int kl = decltype(KLx)::value;
                                constexpr int k = kl / ND, l = kl % ND;
                                constexpr Real an = Real(ang_norm(LA, i) * ang_norm(LB, j) * ang_norm(LC, k)
                                                         * ang_norm(LD, l));
                                const Real eri = acc[(i * NB + j) * CH + (kl - KL0)] * an;
                                const Real w   = (fabs(eri) < thr) ? Real(0) : s * eri;
                                if (spin == 0)
                                {
                                    Jab[i * NB + j] += w * d.Dcd[k * ND + l];
                                    Jcd[kl - KL0] += w * d.Dab[i * NB + j];
                                }
                                Kac[i * NC + k] += w * d.Dbd[spin][j * ND + l];
                                Kad[i * ND + l] += w * d.Dbc[spin][j * NC + k];
                                Kbc[j * NC + k] += w * d.Dad[spin][i * ND + l];
                                Kbd[j * ND + l] += w * d.Dac[spin][i * NC + k];
                            });
                    });
            });
        if (active)
        {
            double* Y = spin == 0 ? v.Ya : v.Yb;
            static_for<0, NA>(
                [&](auto I)
                {
                    constexpr int i = decltype(I)::value;
                    static_for<0, NC>(
                        [&](auto Kx)
                        {
                            constexpr int k = decltype(Kx)::value;
                            if constexpr (chunk_has_k<ND, KL0, KL1>(k))
                                atomicAdd(Y + at(a0 + i, c0 + k), widen(Kac[i * NC + k]));
                        });
                    static_for<0, ND>(
                        [&](auto Lx)
                        {
                            constexpr int l = decltype(Lx)::value;
                            if constexpr (chunk_has_l<ND, KL0, KL1>(l))
                                atomicAdd(Y + at(a0 + i, d0 + l), widen(Kad[i * ND + l]));
                        });
                });
            static_for<0, NB>(
                [&](auto Jx)
                {
                    constexpr int j = decltype(Jx)::value;
                    static_for<0, NC>(
                        [&](auto Kx)
                        {
                            constexpr int k = decltype(Kx)::value;
                            if constexpr (chunk_has_k<ND, KL0, KL1>(k))
                                atomicAdd(Y + at(b0 + j, c0 + k), widen(Kbc[j * NC + k]));
                        });
                    static_for<0, ND>(
                        [&](auto Lx)
                        {
                            constexpr int l = decltype(Lx)::value;
                            if constexpr (chunk_has_l<ND, KL0, KL1>(l))
                                atomicAdd(Y + at(b0 + j, d0 + l), widen(Kbd[j * ND + l]));
                        });
                });
        }
    }
    if (bra_warp)
    {
        // Warp sum of the bra block, then one atomic per element from lane 0.
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int x = 0; x < NAB; ++x)
        {
            Real t = Jab[x];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0)
                atomicAdd(v.X + at(a0 + x / NB, b0 + x % NB), widen(Real(2) * t));
        }
    }
    else if (active)
    {
#pragma unroll
        for (int i = 0; i < NA; ++i)
#pragma unroll
            for (int j = 0; j < NB; ++j) atomicAdd(v.X + at(a0 + i, b0 + j), widen(Real(2) * Jab[i * NB + j]));
    }
    if (active)
    {
#pragma unroll
        for (int x = 0; x < CH; ++x)
            atomicAdd(v.X + at(c0 + (KL0 + x) / ND, d0 + (KL0 + x) % ND), widen(Real(2) * Jcd[x]));
    }
}

// Digestion of one evaluated quartet by one lane on its own.
template <int LA, int LB, int LC, int LD, typename Real, bool UHF>
__device__ __forceinline__ void digest_quartet(const PairRec& bra, const PairRec& ket, bool same_pair, const Real* acc,
                                               const FockView& v)
{
    DigestD<LA, LB, LC, LD, Real, UHF> d;
    load_digest_d<LA, LB, LC, LD, Real, UHF>(bra, ket, v, d);
    digest_loaded<LA, LB, LC, LD, Real, UHF>(bra, ket, same_pair, acc, v, d, true, false);
}

// Stage this class's Boys slice in shared memory.
template <typename Real> __device__ __forceinline__ void stage_boys(const Real* __restrict__ g, Real* s)
{
    constexpr int n = BoysGrid<Real>::kPoints * BoysGrid<Real>::kRow;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = g[i];
    __syncthreads();
}

// One launch processes the whole surviving list of one class; the list length is read on the device
// (written by the list builder), so a build needs no host round trip between kernels.
template <int LA, int LB, int LC, int LD, typename Real, bool UHF>
__global__ void __launch_bounds__(128) jk_class_kernel(const Quartet* __restrict__ list,
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
    const Real* tb      = static_cast<const Real*>(v.pptab[pair_class(LA, LB)]);
    const Real* tk      = static_cast<const Real*>(v.ksoa[pair_class(LC, LD)]);
    const long long kfs = v.kfs[pair_class(LC, LD)];
    using DD   = DigestD<LA, LB, LC, LD, Real, UHF>;
    const int lane = threadIdx.x & 31;
    // Warp-uniform iteration (every lane runs the same trip count, inactive lanes past the end), so that
    // the digestion may sum the bra block over the warp.
    for (unsigned long long base = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u);
         base < n; base += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
    {
        const unsigned long long q = base + lane;
        const bool active          = q < n;
        const Quartet qt           = list[active ? q : base];
        const PairRec bra          = v.pairs[qt.bra];
        const PairRec ket          = v.pairs[qt.ket];
        DD d;
        if (v.store == nullptr && DD::kEarly)
            load_digest_d<LA, LB, LC, LD, Real, UHF>(bra, ket, v, d);
        Real acc[N];
        if (active)
            eval_quartet<LA, LB, LC, LD, Real, true>(bra, ket, tb, tk, slice, acc, kfs);
        else
        {
#pragma unroll
            for (int x = 0; x < N; ++x) acc[x] = Real(0);
        }
        if (v.store != nullptr)
        {
            if (active)
                static_for<0, N>(
                    [&](auto E)
                    {
                        constexpr int e  = decltype(E)::value;
                        constexpr int NB = ncart(LB), NC = ncart(LC), ND = ncart(LD), NCD = NC * ND;
                        constexpr double an = ang_norm(LA, e / NCD / NB) * ang_norm(LB, (e / NCD) % NB)
                                            * ang_norm(LC, (e % NCD) / ND) * ang_norm(LD, e % ND);
                        v.store[q * N + e] = double(acc[e]) * an;
                    });
            continue;
        }
        if (!DD::kEarly)
            load_digest_d<LA, LB, LC, LD, Real, UHF>(bra, ket, v, d);
        const unsigned bra0 = __shfl_sync(0xffffffffu, qt.bra, 0);
        const bool bra_warp = __all_sync(0xffffffffu, qt.bra == bra0);
        digest_loaded<LA, LB, LC, LD, Real, UHF>(bra, ket, qt.bra == qt.ket, acc, v, d, active, bra_warp);
    }
}

// Ket-chunked thread form: one thread per (shell quartet, chunk of CH ket Cartesian components).  For the
// d-containing classes a thread cannot hold a whole quartet's G[HAB][NCD] and ERI[NAB][NCD] in registers;
// restricted to CH ket components the thread keeps R, G[HAB][CH] and ERI[NAB][CH] in registers, with every
// loop unrolled at compile time, and digests the integrals of its chunk (the bra Coulomb block summed over
// the warp as in the thread form; the exchange and ket Coulomb elements its chunk reaches).  Each chunk
// is its own launch over the whole list (jk_class_chunk_kernel<..., KL0, KL1>), so that every SM runs one
// chunk's unrolled code at a time: with the chunks of a quartet in neighbouring blocks of one launch the
// resident blocks of an SM ran different chunk bodies and stalled on instruction fetch (ncu: 30 cycles
// per issued instruction).  Each chunk recomputes the Boys values and R of its quartet: for FP32, where
// these are cheap next to the two Hermite transforms, that buys full lanes and no shared-memory round
// trips; the list and the records are re-read per chunk from L2.
template <int LA, int LB, int LC, int LD, typename Real, bool UHF, int KL0, int KL1>
__device__ __forceinline__ void chunk_body(const Quartet* __restrict__ list, unsigned long long n, const FockView& v,
                                           const Real* __restrict__ slice, unsigned qb, unsigned nqb)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, NCD = NC * ND, CH = KL1 - KL0;
    const Real* tb      = static_cast<const Real*>(v.pptab[pair_class(LA, LB)]);
    const Real* tk      = static_cast<const Real*>(v.ksoa[pair_class(LC, LD)]);
    const long long kfs = v.kfs[pair_class(LC, LD)];
    using DD       = DigestD<LA, LB, LC, LD, Real, UHF>;
    const int lane = threadIdx.x & 31;
    for (unsigned long long base = static_cast<unsigned long long>(qb) * blockDim.x + (threadIdx.x & ~31u); base < n;
         base += static_cast<unsigned long long>(nqb) * blockDim.x)
    {
        const unsigned long long q = base + lane;
        const bool active          = q < n;
        const Quartet qt           = list[active ? q : base];
        const PairRec bra          = v.pairs[qt.bra];
        const PairRec ket          = v.pairs[qt.ket];
        Real acc[NAB * CH];
        if (active)
            eval_quartet<LA, LB, LC, LD, Real, true, KL0, KL1>(bra, ket, tb, tk, slice, acc, kfs);
        else
        {
#pragma unroll
            for (int x = 0; x < NAB * CH; ++x) acc[x] = Real(0);
        }
        if (v.store != nullptr)
        {
            if (active)
                static_for<0, NAB>(
                    [&](auto IJ)
                    {
                        constexpr int ij = decltype(IJ)::value;
                        static_for<KL0, KL1>(
                            [&](auto KLx)
                            {
                                constexpr int kl = decltype(KLx)::value;
                                constexpr double an = ang_norm(LA, ij / NB) * ang_norm(LB, ij % NB) *
                                                      ang_norm(LC, kl / ND) * ang_norm(LD, kl % ND);
                                v.store[q * (NAB * NCD) + ij * NCD + kl] = double(acc[ij * CH + (kl - KL0)]) * an;
                            });
                    });
            continue;
        }
        DD d;
        load_digest_d<LA, LB, LC, LD, Real, UHF>(bra, ket, v, d); // values the chunk does not read are never loaded
        const unsigned bra0 = __shfl_sync(0xffffffffu, qt.bra, 0);
        const bool bra_warp = __all_sync(0xffffffffu, qt.bra == bra0);
        digest_loaded<LA, LB, LC, LD, Real, UHF, KL0, KL1>(bra, ket, qt.bra == qt.ket, acc, v, d, active, bra_warp);
    }
}

// Chunks of CH ket components of a (LC LD) ket.
template <int LC, int LD, int CH> __host__ __device__ constexpr int num_chunks()
{
    return (ncart(LC) * ncart(LD) + CH - 1) / CH;
}

// One chunk, ket components [KL0, KL1), of every quartet of the list.
template <int LA, int LB, int LC, int LD, typename Real, bool UHF, int KL0, int KL1>
__global__ void __launch_bounds__(128) jk_class_chunk_kernel(const Quartet* __restrict__ list,
                                                             const unsigned long long* __restrict__ count, FockView v,
                                                             const Real* __restrict__ boys_slice)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* slice                = reinterpret_cast<Real*>(smem_raw);
    const unsigned long long n = *count;
    if (static_cast<unsigned long long>(blockIdx.x) * blockDim.x >= n)
        return;
    stage_boys<Real>(boys_slice, slice);
    chunk_body<LA, LB, LC, LD, Real, UHF, KL0, KL1>(list, n, v, slice, blockIdx.x, gridDim.x);
}

// Digestion of stored integrals (the stored-integral SCF): integral blocks written once in store mode
// (row-major [ij][kl] per quartet, angular factors included) are digested with full densities every
// build.  Ket-chunked like jk_class_chunk_kernel so that the integrals and partial sums of a thread stay
// in registers: a thread digests ket components [KL0, KL1) of one quartet.
template <int LA, int LB, int LC, int LD, bool UHF, int KL0, int KL1>
__device__ __forceinline__ void stored_body(const Quartet* __restrict__ list, unsigned long long n, const FockView& v,
                                            const double* __restrict__ store, unsigned qb, unsigned nqb)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, NCD = NC * ND, CH = KL1 - KL0;
    using DD       = DigestD<LA, LB, LC, LD, double, UHF>;
    const int lane = threadIdx.x & 31;
    for (unsigned long long base = static_cast<unsigned long long>(qb) * blockDim.x + (threadIdx.x & ~31u); base < n;
         base += static_cast<unsigned long long>(nqb) * blockDim.x)
    {
        const unsigned long long q = base + lane;
        const bool active          = q < n;
        const Quartet qt           = list[active ? q : base];
        const PairRec bra          = v.pairs[qt.bra];
        const PairRec ket          = v.pairs[qt.ket];
        double acc[NAB * CH];
        const double* __restrict__ blk = store + (active ? q : base) * static_cast<unsigned long long>(NAB * NCD);
        static_for<0, NAB>(
            [&](auto IJ)
            {
                constexpr int ij = decltype(IJ)::value;
                static_for<KL0, KL1>(
                    [&](auto KLx)
                    {
                        constexpr int kl = decltype(KLx)::value;
                        // The digestion multiplies by the angular factors again.
                        constexpr double inv_an = 1.0 / (ang_norm(LA, ij / NB) * ang_norm(LB, ij % NB) *
                                                         ang_norm(LC, kl / ND) * ang_norm(LD, kl % ND));
                        acc[ij * CH + (kl - KL0)] = active ? blk[ij * NCD + kl] * inv_an : 0.0;
                    });
            });
        DD d;
        load_digest_d<LA, LB, LC, LD, double, UHF>(bra, ket, v, d);
        const unsigned bra0 = __shfl_sync(0xffffffffu, qt.bra, 0);
        const bool bra_warp = __all_sync(0xffffffffu, qt.bra == bra0);
        digest_loaded<LA, LB, LC, LD, double, UHF, KL0, KL1>(bra, ket, qt.bra == qt.ket, acc, v, d, active, bra_warp);
    }
}

// Ket components per thread of the stored digestion: at most 36 integrals per thread.
template <int LA, int LB, int LC, int LD> __host__ __device__ constexpr int stored_chunk()
{
    constexpr int NAB = ncart(LA) * ncart(LB), NCD = ncart(LC) * ncart(LD);
    constexpr int c   = 36 / NAB > 0 ? 36 / NAB : 1;
    return c < NCD ? c : NCD;
}

template <int LA, int LB, int LC, int LD, bool UHF>
__global__ void __launch_bounds__(128) jk_stored_kernel(const Quartet* __restrict__ list, unsigned long long n,
                                                        FockView v, const double* __restrict__ store)
{
    constexpr int NCD = ncart(LC) * ncart(LD), CH = stored_chunk<LA, LB, LC, LD>(), NCH = num_chunks<LC, LD, CH>();
    const unsigned qb = blockIdx.x / NCH, nqb = gridDim.x / NCH;
    const int chunk   = static_cast<int>(blockIdx.x % NCH);
    if (qb >= nqb || static_cast<unsigned long long>(qb) * blockDim.x >= n)
        return;
    static_for<0, NCH>(
        [&](auto C)
        {
            constexpr int c = decltype(C)::value;
            if (chunk == c)
                stored_body<LA, LB, LC, LD, UHF, c * CH, (c * CH + CH < NCD ? c * CH + CH : NCD)>(list, n, v, store, qb,
                                                                                                nqb);
        });
}

} // namespace hfg
