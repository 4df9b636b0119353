// Warp-cooperative fused ERI + J/K digestion for shell-quartet classes with many Cartesian components
// (the d-containing classes), where one thread cannot hold the quartet's Hermite and integral arrays
// in registers.
//
// One warp evaluates one quartet.  The scalar part of a primitive quartet (T, the prefactor, Boys
// F_0..F_L) is computed for 32 primitive quartets at once, one per lane (the FP64 pipe pays per warp
// instruction, so a scalar computed by every lane for the same primitive quartet would cost as much as
// 32 distinct ones), and the data-parallel parts are spread over the lanes through shared memory:
//   * R^n_{tuv}: level by level (n = L-1 .. 0), every entry of a level computed by some lane from the
//     previous level (ping-pong buffers), the recursion of src/IntegralEngine.cpp:1082-1162;
//   * G[tuv][kl] (ket Hermite -> Cartesian, summed over ket primitives): each lane owns entries;
//   * ERI[ij][kl] (bra Hermite -> Cartesian): each lane owns entries, accumulated in registers;
//   * digestion: each lane owns complete output elements of the J/K partial blocks (sum over the
//     quartet's integrals), so every output element gets exactly one global atomic per quartet.
// The numerical content is identical to the thread-per-quartet kernel (eri_jk.cuh).
#pragma once

#include "eri_jk.cuh"

#include <cuda_runtime.h>

namespace hfg
{
// Lookup tables for the runtime loops of the warp kernel, built once by the engine.
struct WarpTables
{
    // Recursion steps per total L (0..kMaxLt), entries in ascending degree order, hidx(.,L) layout:
    // x = dst, y = src1, z = src2 (-1 if absent), w = axis | (coef << 2).
    // (Totals up to kMaxLt + 1: the gradient needs one order more than the Fock build.)
    int4 rtab[kMaxLt + 2][nherm(kMaxLt + 1)];
    // The integer coefficient of each step as a double (no int -> double conversion on the FP64 pipe).
    double rcoef[kMaxLt + 2][nherm(kMaxLt + 1)];
    // (t,u,v) of the h-th Hermite index for total L: t | u << 8 | v << 16.
    int htuv[kMaxLt + 2][nherm(kMaxLt + 1)];
    // hidx(t,u,v,L) from the cube index (t*(L+1)+u)*(L+1)+v.
    short cube[kMaxLt + 2][(kMaxLt + 2) * (kMaxLt + 2) * (kMaxLt + 2)];
    // Per pair class and Cartesian pair ij: x,y,z = lengths of the 1-D Hermite ranges, w = offset of
    // the ij block inside the primitive-pair record (including the header).
    int4 e3[kNumPairClasses][ncart(kMaxL) * ncart(kMaxL)];
};

inline void build_warp_tables(WarpTables& T)
{
    for (int L = 0; L <= kMaxLt + 1; ++L)
    {
        int k = 0;
        for (int d = 0; d <= L; ++d)
            for (int v = 0; v <= d; ++v)
                for (int u = 0; u <= d - v; ++u)
                {
                    const int t = d - u - v;
                    int4 r;
                    r.x = hidx(t, u, v, L);
                    int ax, c;
                    if (t > 0)
                    {
                        ax = 0;
                        c  = t - 1;
                        r.y = hidx(t - 1, u, v, L);
                        r.z = c > 0 ? hidx(t - 2, u, v, L) : -1;
                    }
                    else if (u > 0)
                    {
                        ax = 1;
                        c  = u - 1;
                        r.y = hidx(t, u - 1, v, L);
                        r.z = c > 0 ? hidx(t, u - 2, v, L) : -1;
                    }
                    else if (v > 0)
                    {
                        ax = 2;
                        c  = v - 1;
                        r.y = hidx(t, u, v - 1, L);
                        r.z = c > 0 ? hidx(t, u, v - 2, L) : -1;
                    }
                    else
                    {
                        ax = 0;
                        c  = 0;
                        r.y = -1;
                        r.z = -1;
                    }
                    r.w             = ax | (c << 2);
                    T.rcoef[L][k]   = c;
                    T.rtab[L][k++] = r;
                }
        for (int h = 0; h < nherm(L); ++h)
            T.htuv[L][h] = htuv(h, L, 0) | (htuv(h, L, 1) << 8) | (htuv(h, L, 2) << 16);
        const int S = L + 1;
        for (int t = 0; t <= L; ++t)
            for (int u = 0; u <= L; ++u)
                for (int v = 0; v <= L; ++v)
                    T.cube[L][(t * S + u) * S + v] = static_cast<short>(t + u + v <= L ? hidx(t, u, v, L) : -1);
    }
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        const int l1 = pair_class_l1(pc), l2 = pair_class_l2(pc);
        for (int ij = 0; ij < ncart(l1) * ncart(l2); ++ij)
            T.e3[pc][ij] = make_int4(e3_len(l1, l2, ij, 0), e3_len(l1, l2, ij, 1), e3_len(l1, l2, ij, 2),
                                     kPairHeader + e3_offset(l1, l2, ij));
    }
}

#ifdef __CUDACC__
template <int LA, int LB, int LC, int LD, typename Real> struct WarpLayout
{
    static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    static constexpr int NAB = NA * NB, NCD = NC * ND;
    static constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
    static constexpr int HAB = nherm(LAB), HL = nherm(L);
    // Per-warp shared scratch (in Real units): two R levels, G, the digested integrals, and the scalar
    // part (X, Y, Z, scaled Boys values) of a batch of 32 primitive quartets.
    static constexpr int kR   = 2 * HL;
    static constexpr int kG   = HAB * NCD;
    static constexpr int kE   = NAB * NCD;
    static constexpr int kPb  = 32 * (L + 4);
    static constexpr int kPerWarp = ((kR + kG + kE + kPb + 1) / 2) * 2;
    static constexpr int kAcc     = (NAB * NCD + 31) / 32;
};

constexpr int kWarpKernelWarps = 4;

template <int LA, int LB, int LC, int LD, typename Real, bool UHF>
__global__ void __launch_bounds__(32 * kWarpKernelWarps)
    jk_class_warp_kernel(const Quartet* __restrict__ list, const unsigned long long* __restrict__ count, FockView v,
                         const Real* __restrict__ boys_slice, const WarpTables* __restrict__ tabs)
{
    using W = WarpLayout<LA, LB, LC, LD, Real>;
    constexpr int NA = W::NA, NB = W::NB, NC = W::NC, ND = W::ND, NAB = W::NAB, NCD = W::NCD;
    constexpr int LAB = W::LAB, L = W::L, HAB = W::HAB, HL = W::HL;
    constexpr int SB = pp_stride(LA, LB), SK = pp_stride(LC, LD), S = L + 1;
    constexpr int PCB = pair_class(LA, LB), PCK = pair_class(LC, LD);

    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* slice = reinterpret_cast<Real*>(smem_raw);
    const unsigned long long n = *count;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (static_cast<unsigned long long>(blockIdx.x) * kWarpKernelWarps >= n)
        return;
    stage_boys<Real>(boys_slice, slice);
    Real* wbase = slice + BoysGrid<Real>::kPoints * BoysGrid<Real>::kRow + wib * W::kPerWarp;
    Real* Rbuf0 = wbase;
    Real* Rbuf1 = wbase + HL;
    Real* Gs    = wbase + 2 * HL;
    Real* Es    = Gs + W::kG;
    Real* Pb    = Es + W::kE;

    const Real* tb = static_cast<const Real*>(v.pptab[PCB]);
    const Real* tk = static_cast<const Real*>(v.pptab[PCK]);

    for (unsigned long long q = static_cast<unsigned long long>(blockIdx.x) * kWarpKernelWarps + wib; q < n;
         q += static_cast<unsigned long long>(gridDim.x) * kWarpKernelWarps)
    {
        const Quartet qt  = list[q];
        const PairRec bra = v.pairs[qt.bra];
        const PairRec ket = v.pairs[qt.ket];
        Real acc[W::kAcc];
#pragma unroll
        for (int m = 0; m < W::kAcc; ++m) acc[m] = Real(0);

        // Primitive quartets t = ib * npk + ik in batches of 32: lane j of a batch computes the scalar
        // part of quartet base + j (T, prefactor, Boys) into the warp's buffer Pb, then the warp walks
        // the batch, running the distributed recursion and contractions on one primitive quartet at a time.
        const int npk = ket.npp, P = bra.npp * npk;
        for (int base = 0; base < P; base += 32)
        {
            __syncwarp(); // the previous batch's reads of Pb are done
            {
                const int t = base + lane;
                if (t < P)
                {
                    const int ib = t / npk, ik = t - ib * npk;
                    const Real* __restrict__ rb = tb + static_cast<size_t>(bra.pp_off + ib) * SB;
                    const Real* __restrict__ rk = tk + static_cast<size_t>(ket.pp_off + ik) * SK;
                    const Real p = rb[0], qq = rk[0];
                    const Real X = rb[1] - rk[1], Y = rb[2] - rk[2], Z = rb[3] - rk[3];
                    const Real rs   = hfg_rsqrt(p + qq);
                    const Real rho  = (p * qq) * (rs * rs);
                    const Real pref = (rb[4] * rk[4]) * rs;
                    const Real T    = rho * (X * X + Y * Y + Z * Z);
                    Real F[L + 1];
                    boys_eval<L, Real>(T, slice, F);
                    Pb[0 * 32 + lane] = X;
                    Pb[1 * 32 + lane] = Y;
                    Pb[2 * 32 + lane] = Z;
                    const Real m2r = Real(-2) * rho;
                    Real w         = pref;
#pragma unroll
                    for (int k = 0; k <= L; ++k)
                    {
                        Pb[(3 + k) * 32 + lane] = w * F[k];
                        w *= m2r;
                    }
                }
            }
            __syncwarp();
            const int nb = min(32, P - base);
            for (int j = 0; j < nb; ++j)
            {
                const int t = base + j, ib = t / npk, ik = t - ib * npk;
                const Real X = Pb[0 * 32 + j], Y = Pb[1 * 32 + j], Z = Pb[2 * 32 + j];
                const Real* __restrict__ rk = tk + static_cast<size_t>(ket.pp_off + ik) * SK;
                // R recursion, level n+1 in `src`, level n into `dst`.
                Real* src = Rbuf0;
                Real* dst = Rbuf1;
                if (lane == 0)
                    src[0] = Pb[(3 + L) * 32 + j];
                __syncwarp();
#pragma unroll
                for (int lev = L - 1; lev >= 0; --lev)
                {
                    const int cnt = nherm(L - lev);
                    for (int k = 1 + lane; k < cnt; k += 32)
                    {
                        const int4 r  = tabs->rtab[L][k];
                        const int ax  = r.w & 3, c = r.w >> 2;
                        const Real xa = ax == 0 ? X : (ax == 1 ? Y : Z);
                        Real val      = xa * src[r.y];
                        if (c > 0)
                        {
                            if constexpr (sizeof(Real) == 8)
                                val = fma(tabs->rcoef[L][k], src[r.z], val);
                            else
                                val = fmaf(Real(c), src[r.z], val);
                        }
                        dst[r.x] = val;
                    }
                    if (lane == 0)
                        dst[0] = Pb[(3 + lev) * 32 + j];
                    __syncwarp();
                    Real* tmp = src;
                    src       = dst;
                    dst       = tmp;
                }
                const Real* R = src; // level 0
                // G[tuv][kl] (+)= sum (-1)^{tau+nu+phi} E^{kl}_{tau nu phi} R_{t+tau,u+nu,v+phi}; entries are
                // lane-owned, restarted at the first ket primitive of every bra primitive.
                for (int e = lane; e < W::kG; e += 32)
                {
                    const int h = e / NCD, kl = e % NCD;
                    const int tuv = tabs->htuv[LAB][h];
                    const int tt = tuv & 255, u = (tuv >> 8) & 255, vv = tuv >> 16;
                    const int4 el = tabs->e3[PCK][kl];
                    Real s = Real(0);
                    int x  = el.w;
                    for (int phi = 0; phi < el.z; ++phi)
                        for (int nu = 0; nu < el.y; ++nu)
                            for (int tau = 0; tau < el.x; ++tau, ++x)
                            {
                                // The sign rides on the coefficient, so the term is one FMA.
                                const Real ek = ((tau + nu + phi) & 1) ? -rk[x] : rk[x];
                                s = fma(ek, R[tabs->cube[L][((tt + tau) * S + (u + nu)) * S + (vv + phi)]], s);
                            }
                    Gs[e] = (ik == 0 ? Real(0) : Gs[e]) + s;
                }
                __syncwarp();
                if (ik == npk - 1)
                {
                    // ERI[ij][kl] += sum_tuv E^{ij}_{tuv} G[tuv][kl] for bra primitive ib.
                    const Real* __restrict__ rb = tb + static_cast<size_t>(bra.pp_off + ib) * SB;
#pragma unroll
                    for (int m = 0; m < W::kAcc; ++m)
                    {
                        const int e = lane + 32 * m;
                        if (e < NAB * NCD)
                        {
                            const int ij = e / NCD, kl = e % NCD;
                            const int4 el = tabs->e3[PCB][ij];
                            Real s = Real(0);
                            int x  = el.w;
                            for (int vv = 0; vv < el.z; ++vv)
                                for (int u = 0; u < el.y; ++u)
                                    for (int tt = 0; tt < el.x; ++tt, ++x)
                                        s += rb[x] * Gs[tabs->cube[LAB][(tt * (LAB + 1) + u) * (LAB + 1) + vv] * NCD + kl];
                            acc[m] += s;
                        }
                    }
                    __syncwarp();
                }
            }
        }

        if (v.store != nullptr)
        {
#pragma unroll
            for (int m = 0; m < W::kAcc; ++m)
            {
                const int e = lane + 32 * m;
                if (e < NAB * NCD)
                {
                    const int ij = e / NCD, kl = e % NCD;
                    const double an = ang_norm(LA, ij / NB) * ang_norm(LB, ij % NB) * ang_norm(LC, kl / ND) * ang_norm(LD, kl % ND);
                    v.store[q * (NAB * NCD) + e] = double(acc[m]) * an;
                }
            }
            continue;
        }
        // Angular normalisation, AO-level skip and degeneracy factor, then into shared memory.
        const Real sdeg = (bra.same ? Real(0.5) : Real(1)) * (ket.same ? Real(0.5) : Real(1)) * (qt.bra == qt.ket ? Real(0.5) : Real(1));
        const Real athr = ao_threshold<Real>(v);
#pragma unroll
        for (int m = 0; m < W::kAcc; ++m)
        {
            const int e = lane + 32 * m;
            if (e < NAB * NCD)
            {
                const int ij = e / NCD, kl = e % NCD;
                const int i = ij / NB, j = ij % NB, k = kl / ND, l = kl % ND;
                const Real an = Real(ang_norm(LA, i) * ang_norm(LB, j) * ang_norm(LC, k) * ang_norm(LD, l));
                const Real eri = acc[m] * an;
                Es[e]          = (fabs(eri) < athr) ? Real(0) : sdeg * eri;
            }
        }
        __syncwarp();

        const long long off = v.mat_off[bra.mol];
        const int nld       = v.mat_ld[bra.mol];
        const int a0 = bra.ao1, b0 = bra.ao2, c0 = ket.ao1, d0 = ket.ao2;
        auto at = [&](int r, int c) -> long long { return off + r + static_cast<long long>(c) * nld; };
        // J blocks.
        for (int o = lane; o < NAB + NCD; o += 32)
        {
            Real s = Real(0);
            if (o < NAB)
            {
                for (int kl = 0; kl < NCD; ++kl) s += Es[o * NCD + kl] * ldD<Real>(v.Dt, at(c0 + kl / ND, d0 + kl % ND));
                atomicAdd(v.X + at(a0 + o / NB, b0 + o % NB), widen(Real(2) * s));
            }
            else
            {
                const int kl = o - NAB;
                for (int ij = 0; ij < NAB; ++ij) s += Es[ij * NCD + kl] * ldD<Real>(v.Dt, at(a0 + ij / NB, b0 + ij % NB));
                atomicAdd(v.X + at(c0 + kl / ND, d0 + kl % ND), widen(Real(2) * s));
            }
        }
        // K blocks: ac, ad, bc, bd.
        constexpr int nspin = UHF ? 2 : 1;
        for (int spin = 0; spin < nspin; ++spin)
        {
            const void* Ds = spin == 0 ? v.Da : v.Db;
            double* Yo     = spin == 0 ? v.Ya : v.Yb;
            constexpr int nK = NA * NC + NA * ND + NB * NC + NB * ND;
            for (int o = lane; o < nK; o += 32)
            {
                Real s = Real(0);
                if (o < NA * NC)
                {
                    const int i = o / NC, k = o % NC;
                    for (int j = 0; j < NB; ++j)
                        for (int l = 0; l < ND; ++l)
                            s += Es[(i * NB + j) * NCD + k * ND + l] * ldD<Real>(Ds, at(b0 + j, d0 + l));
                    atomicAdd(Yo + at(a0 + i, c0 + k), widen(s));
                }
                else if (o < NA * NC + NA * ND)
                {
                    const int r = o - NA * NC, i = r / ND, l = r % ND;
                    for (int j = 0; j < NB; ++j)
                        for (int k = 0; k < NC; ++k)
                            s += Es[(i * NB + j) * NCD + k * ND + l] * ldD<Real>(Ds, at(b0 + j, c0 + k));
                    atomicAdd(Yo + at(a0 + i, d0 + l), widen(s));
                }
                else if (o < NA * NC + NA * ND + NB * NC)
                {
                    const int r = o - NA * NC - NA * ND, j = r / NC, k = r % NC;
                    for (int i = 0; i < NA; ++i)
                        for (int l = 0; l < ND; ++l)
                            s += Es[(i * NB + j) * NCD + k * ND + l] * ldD<Real>(Ds, at(a0 + i, d0 + l));
                    atomicAdd(Yo + at(b0 + j, c0 + k), widen(s));
                }
                else
                {
                    const int r = o - NA * NC - NA * ND - NB * NC, j = r / ND, l = r % ND;
                    for (int i = 0; i < NA; ++i)
                        for (int k = 0; k < NC; ++k)
                            s += Es[(i * NB + j) * NCD + k * ND + l] * ldD<Real>(Ds, at(a0 + i, c0 + k));
                    atomicAdd(Yo + at(b0 + j, d0 + l), widen(s));
                }
            }
        }
        __syncwarp();
    }
}
#endif
} // namespace hfg
