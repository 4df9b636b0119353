// Adjoint two-electron part of the analytic nuclear gradient (no counterpart in the reference, which has
// no gradients; the differentiated integrals are those of src/IntegralEngine.cpp:731-992).
//
//   dE_2e/dX = 1/2 sum_{ijkl} d(ij|kl)/dX Gamma_ijkl,
//   Gamma_ijkl = Dt_ij Dt_kl - 1/2 sum_s (Ds_ik Ds_jl + Ds_il Ds_jk)        (s = alpha, beta)
//
// summed over unique shell quartets with the degeneracy factor s_q (1/2 per equal pair, as in the
// Fock build): dE/dX = 4 sum_q s_q sum_{ijkl in q} Gamma_ijkl d(ij|kl)/dX.
//
// Centre derivatives in McMurchie-Davidson form: d/dA_x of a primitive pair distribution has Hermite
// coefficients  DA^{ij}_t = 2a E^{i+1,j}_t - i E^{i-1,j}_t  (x factor; y and z factors unchanged), likewise
// DB with b and j, DC/DD on the ket.  The kernels never form derivative integrals; in two passes over
// the primitive quartets of a shell quartet
//   bra-outer: G[tuv][kl]  = sum_{ket prims} sum_{tau nu phi} (-1)^{tau+nu+phi} E^{kl}_{tau nu phi} R_{t+tau,..}
//              (t+u+v <= l_ab + 1), then once per bra primitive pair
//              y[ij][tuv]  = sum_kl Gamma_ijkl G[tuv][kl]          -> g_A += DA . y,  g_B += DB . y
//   ket-outer: X[ij][tuv'] = sum_{bra prims} sum_{tuv} E^{ij}_{tuv} R_{t+tau,..}   (tau+nu+phi <= l_cd + 1),
//              then once per ket primitive pair
//              h[kl][tuv'] = sum_ij Gamma_ijkl X[ij][tuv']         -> g_C += (-1)^{..} DC . h
// and g_D = -(g_A + g_B + g_C) (translational invariance): the Gamma contractions run once per primitive
// pair, not once per primitive quartet, at the price of evaluating R twice.  E/R tables are recomputed here, nothing from
// the forward build is stored.  FP64, or FP32 for the small-bound quartets of a mixed-precision gradient
// (FP64 accumulation).  One group of lanes per quartet (GradLayout::kGroup: 4 to 32 lanes by
// class size; the groups of a warp work independently, synchronised by group masks).
#pragma once

#include "eri_warp.cuh"

namespace hfg
{
// Per-primitive-pair gradient record for pair class (l1, l2): [0] a, [1] b, then for each axis the 1-D
// Hermite table E[i][j][t], i <= l1+1, j <= l2+1, t <= l1+l2+2 (dense).
__host__ __device__ constexpr int g1d_size(int l1, int l2) { return (l1 + 2) * (l2 + 2) * (l1 + l2 + 3); }
__host__ __device__ constexpr int g_stride(int l1, int l2)
{
    const int s = 2 + 3 * g1d_size(l1, l2);
    return s + (s & 1);
}

struct GradView
{
    const PairRec* pairs;
    const void* pptab[kNumPairClasses]; // forward records (p, P, W, ...), Real of the kernel
    const void* gtab[kNumPairClasses];  // gradient records, Real of the kernel
    const void* Dt;                     // densities, Real of the kernel
    const void* Da;
    const void* Db;
    int n;                  // nao
    const int* shell_atom;  // per shell
    double* grad;           // [natom][3]
};

#ifdef __CUDACC__
template <int LA, int LB, int LC, int LD> struct GradLayout
{
    static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    static constexpr int NAB = NA * NB, NCD = NC * ND;
    static constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD + 1;
    static constexpr int HAB1 = nherm(LAB + 1), HCD1 = nherm(LCD + 1), HL = nherm(L);
    static constexpr int kR = 2 * HL, kG = HAB1 * NCD, kX = NAB * HCD1, kGam = NAB * NCD;
    // Lanes per quartet: a power of two from 4 to 32, about a quarter of the larger per-quartet work array,
    // so that the small classes do not leave most of a warp idle; a warp holds 32 / kGroup quartets.
    static constexpr int kWork  = kG > kX ? kG : kX;
    static constexpr int kGroup = kWork <= 16 ? 4 : kWork <= 32 ? 8 : kWork <= 64 ? 16 : 32;
    // Per-primitive-quartet scalars (P - Q and the scaled Boys values F_0..F_L), computed by the group's
    // lanes for kGroup primitive quartets at once (one each) instead of by every lane for each.
    static constexpr int kScal = L + 4, kS = kGroup * kScal;
    static constexpr int kPerGroup = ((kR + kG + kX + kGam + kS + 1) / 2) * 2;
    static constexpr int kPerWarp  = kPerGroup * (32 / kGroup);
};

constexpr int kGradWarps = 2;

// Angular normalisation factor of component c of l in the kernel's precision (integer tests and selects
// only: no double arithmetic in the FP32 kernels).
template <typename Real> __device__ __forceinline__ Real ang_norm_r(int l, int c)
{
    const int i = cart_exp(l, c, 0), j = cart_exp(l, c, 1), k = cart_exp(l, c, 2);
    const int d = dfact_odd(2 * i - 1) * dfact_odd(2 * j - 1) * dfact_odd(2 * k - 1);
    return d == 1 ? Real(1) : (d == 3 ? Real(0.57735026918962576451) : (d == 9 ? Real(1.0 / 3.0) : (d == 15 ? Real(0.25819888974716112568) : Real(1))));
}

template <typename Real> __device__ __forceinline__ Real e1(const Real* T, int l2, int l12, int i, int j, int t)
{
    // T: one axis of a gradient record, dense [i][j][t] with extents (l1+2, l2+2, l12+3)
    return T[(i * (l2 + 2) + j) * (l12 + 3) + t];
}

template <int LA, int LB, int LC, int LD, typename Real>
__global__ void __launch_bounds__(32 * kGradWarps)
    grad_class_kernel(const Quartet* __restrict__ list, unsigned long long n, GradView v,
                      const Real* __restrict__ boys_slice, const WarpTables* __restrict__ tabs)
{
    using W = GradLayout<LA, LB, LC, LD>;
    constexpr int NB = W::NB, ND = W::ND, NAB = W::NAB, NCD = W::NCD;
    constexpr int LAB = W::LAB, LCD = W::LCD, L = W::L, HAB1 = W::HAB1, HCD1 = W::HCD1, HL = W::HL;
    constexpr int SB = pp_stride(LA, LB), SK = pp_stride(LC, LD);
    constexpr int GB = g_stride(LA, LB), GK = g_stride(LC, LD);
    constexpr int PCB = pair_class(LA, LB), PCK = pair_class(LC, LD);
    constexpr int S = L + 1;
    constexpr int G1B = g1d_size(LA, LB), G1K = g1d_size(LC, LD);

    constexpr int GS = W::kGroup, NG = 32 / GS; // lanes per quartet, quartets per warp
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* slice = reinterpret_cast<Real*>(smem_raw);
    const int wl = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int lane = wl % GS, grp = wl / GS; // lane within the quartet's group, group within the warp
    const unsigned gmask = (GS == 32) ? 0xffffffffu : (((1u << GS) - 1u) << (grp * GS));
    if (static_cast<unsigned long long>(blockIdx.x) * kGradWarps * NG >= n)
        return;
    stage_boys<Real>(boys_slice, slice);
    Real* wbase = slice + BoysGrid<Real>::kPoints * BoysGrid<Real>::kRow + wib * W::kPerWarp + grp * W::kPerGroup;
    Real* Rbuf0 = wbase;
    Real* Rbuf1 = wbase + HL;
    Real* Gs    = wbase + 2 * HL;
    Real* Xs    = Gs + W::kG;
    Real* Gam   = Xs + W::kX;
    Real* Sb    = Gam + W::kGam; // kGroup rows of kScal scalars
    constexpr int kScal = W::kScal;
    const Real* Dt = static_cast<const Real*>(v.Dt);
    const Real* Da = static_cast<const Real*>(v.Da);
    const Real* Db = static_cast<const Real*>(v.Db);

    for (unsigned long long q = (static_cast<unsigned long long>(blockIdx.x) * kGradWarps + wib) * NG + grp; q < n;
         q += static_cast<unsigned long long>(gridDim.x) * kGradWarps * NG)
    {
        const Quartet qt  = list[q];
        const PairRec bra = v.pairs[qt.bra];
        const PairRec ket = v.pairs[qt.ket];
        const int a0 = bra.ao1, b0 = bra.ao2, c0 = ket.ao1, d0 = ket.ao2;
        const int n = v.n;
        const Real sdeg = Real(4) * (bra.same ? Real(0.5) : Real(1)) * (ket.same ? Real(0.5) : Real(1)) * (qt.bra == qt.ket ? Real(0.5) : Real(1));
        // Gamma (with the angular normalisation of the four components and the degeneracy factor).
        for (int e = lane; e < NAB * NCD; e += GS)
        {
            const int ij = e / NCD, kl = e % NCD;
            const int i = ij / NB, j = ij % NB, k = kl / ND, l = kl % ND;
            const long long I = a0 + i, J = b0 + j, K = c0 + k, Lx = d0 + l;
            auto D = [&](const Real* M, long long r, long long c) { return M[r + c * n]; };
            const Real g = D(Dt, I, J) * D(Dt, K, Lx) -
                             Real(0.5) * (D(Da, I, K) * D(Da, J, Lx) + D(Da, I, Lx) * D(Da, J, K) +
                                    D(Db, I, K) * D(Db, J, Lx) + D(Db, I, Lx) * D(Db, J, K));
            Gam[e] = sdeg * ang_norm_r<Real>(LA, i) * ang_norm_r<Real>(LB, j) * ang_norm_r<Real>(LC, k) * ang_norm_r<Real>(LD, l) * g;
        }
        __syncwarp(gmask);
        Real gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};

        // The scalars of one primitive quartet into a row of the group's buffer: P - Q, then
        // Fs[n] = pref (-2 rho)^n F_n.  Each lane fills its own row, for a different primitive quartet.
        auto prim_scalars = [&](const Real* rb, const Real* rk, Real* row)
        {
            const Real p = rb[0], qq = rk[0];
            const Real X = rb[1] - rk[1], Y = rb[2] - rk[2], Z = rb[3] - rk[3];
            const Real rs   = hfg_rsqrt(p + qq);
            const Real rho  = (p * qq) * (rs * rs);
            const Real pref = (rb[4] * rk[4]) * rs;
            const Real T    = rho * (X * X + Y * Y + Z * Z);
            Real F[L + 1];
            boys_eval<L, Real>(T, slice, F);
            row[0] = X;
            row[1] = Y;
            row[2] = Z;
            const Real m2r = Real(-2) * rho;
            Real w         = pref;
#pragma unroll
            for (int k = 0; k <= L; ++k)
            {
                row[3 + k] = w * F[k];
                w *= m2r;
            }
        };
        // R^0_{tuv} of one buffered primitive quartet into one of the group's two R buffers (levels in
        // parallel over the group's lanes); returns the buffer that holds it.
        auto group_R = [&](const Real* row) -> const Real*
        {
            const Real X = row[0], Y = row[1], Z = row[2];
            const Real* Fs = row + 3;
            Real* src = Rbuf0;
            Real* dst = Rbuf1;
            if (lane == 0)
                src[0] = Fs[L];
            __syncwarp(gmask);
#pragma unroll
            for (int lev = L - 1; lev >= 0; --lev)
            {
                const int cnt = nherm(L - lev);
                for (int k = 1 + lane; k < cnt; k += GS)
                {
                    const int4 r  = tabs->rtab[L][k];
                    const int ax  = r.w & 3, c = r.w >> 2;
                    const Real xa = ax == 0 ? X : (ax == 1 ? Y : Z);
                    Real val    = xa * src[r.y];
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
                    dst[0] = Fs[lev];
                __syncwarp(gmask);
                Real* t = src;
                src       = dst;
                dst       = t;
            }
            return src;
        };

        // Bra-outer pass (centres A, B): G[tuv][kl] (t+u+v <= LAB+1) summed over the ket primitives of one
        // bra primitive pair, then contracted with Gamma and the bra's derivative coefficients once per bra
        // primitive pair.
        for (int ib = 0; ib < bra.npp; ++ib)
        {
            const Real* __restrict__ rb = static_cast<const Real*>(v.pptab[PCB]) + static_cast<size_t>(bra.pp_off + ib) * SB;
            const Real* __restrict__ gb = static_cast<const Real*>(v.gtab[PCB]) + static_cast<size_t>(bra.pp_off + ib) * GB;
            const Real aexp = gb[0], bexp = gb[1];
            for (int e = lane; e < HAB1 * NCD; e += GS) Gs[e] = Real(0);
            for (int ik = 0; ik < ket.npp; ++ik)
            {
                const int j = ik % GS;
                if (j == 0)
                {
                    // The next GS ket primitives' scalars, one per lane.
                    if (ik + lane < ket.npp)
                        prim_scalars(rb, static_cast<const Real*>(v.pptab[PCK]) + static_cast<size_t>(ket.pp_off + ik + lane) * SK,
                                     Sb + lane * kScal);
                    __syncwarp(gmask);
                }
                // The ket's 3-D Hermite coefficients E^{kl}_{tau nu phi} from its forward record (one DFMA per
                // term; products of the 1-D tables would cost a DMUL more on the FP64 pipe).
                const Real* __restrict__ rk = static_cast<const Real*>(v.pptab[PCK]) + static_cast<size_t>(ket.pp_off + ik) * SK;
                const Real* R = group_R(Sb + j * kScal);
                auto Ridx = [&](int t, int u, int w_) { return R[tabs->cube[L][(t * S + u) * S + w_]]; };
                for (int e = lane; e < HAB1 * NCD; e += GS)
                {
                    const int h = e / NCD, kl = e % NCD;
                    const int tuv = tabs->htuv[LAB + 1][h];
                    const int t = tuv & 255, u = (tuv >> 8) & 255, w_ = tuv >> 16;
                    const int4 g3 = tabs->e3[PCK][kl]; // 1-D range lengths, offset in the record
                    const Real* E3 = rk + g3.w;
                    Real s   = Real(0);
                    int idx  = 0;
                    for (int ph = 0; ph < g3.z; ++ph)
                        for (int nu = 0; nu < g3.y; ++nu)
                            for (int ta = 0; ta < g3.x; ++ta, ++idx)
                            {
                                const Real ek = (LCD == 0) ? Real(1) : E3[idx];
                                s = fma(((ta + nu + ph) & 1) ? -ek : ek, Ridx(t + ta, u + nu, w_ + ph), s);
                            }
                    Gs[e] += s;
                }
                __syncwarp(gmask); // G read R; the next primitive quartet overwrites the R buffers
            }
            for (int e = lane; e < NAB * HAB1; e += GS)
            {
                const int ij = e / HAB1, h = e % HAB1;
                Real y = Real(0);
                for (int kl = 0; kl < NCD; ++kl) y += Gam[ij * NCD + kl] * Gs[h * NCD + kl];
                if (y == Real(0))
                    continue;
                const int tuv = tabs->htuv[LAB + 1][h];
                const int tt[3] = {tuv & 255, (tuv >> 8) & 255, tuv >> 16};
                const int i = ij / NB, j = ij % NB;
                const int ie[3] = {cart_exp(LA, i, 0), cart_exp(LA, i, 1), cart_exp(LA, i, 2)};
                const int je[3] = {cart_exp(LB, j, 0), cart_exp(LB, j, 1), cart_exp(LB, j, 2)};
                const Real* E[3] = {gb + 2, gb + 2 + G1B, gb + 2 + 2 * G1B};
                Real f[3], dA[3], dB[3];
                for (int x = 0; x < 3; ++x)
                {
                    const int t = tt[x];
                    f[x]  = (t <= ie[x] + je[x]) ? e1(E[x], LB, LAB, ie[x], je[x], t) : Real(0);
                    dA[x] = Real(2) * aexp * e1(E[x], LB, LAB, ie[x] + 1, je[x], t) -
                            (ie[x] > 0 ? ie[x] * e1(E[x], LB, LAB, ie[x] - 1, je[x], t) : Real(0));
                    dB[x] = Real(2) * bexp * e1(E[x], LB, LAB, ie[x], je[x] + 1, t) -
                            (je[x] > 0 ? je[x] * e1(E[x], LB, LAB, ie[x], je[x] - 1, t) : Real(0));
                }
                gA[0] += y * dA[0] * f[1] * f[2];
                gA[1] += y * f[0] * dA[1] * f[2];
                gA[2] += y * f[0] * f[1] * dA[2];
                gB[0] += y * dB[0] * f[1] * f[2];
                gB[1] += y * f[0] * dB[1] * f[2];
                gB[2] += y * f[0] * f[1] * dB[2];
            }
            __syncwarp(gmask); // the contraction read Gs before the next bra primitive pair clears it
        }

        // Ket-outer pass (centre C): X[ij][tuv'] (tau+nu+phi <= LCD+1) summed over the bra primitives of one
        // ket primitive pair, then contracted once per ket primitive pair.
        for (int ik = 0; ik < ket.npp; ++ik)
        {
            const Real* __restrict__ rk = static_cast<const Real*>(v.pptab[PCK]) + static_cast<size_t>(ket.pp_off + ik) * SK;
            const Real* __restrict__ gk = static_cast<const Real*>(v.gtab[PCK]) + static_cast<size_t>(ket.pp_off + ik) * GK;
            const Real cexp = gk[0];
            for (int e = lane; e < NAB * HCD1; e += GS) Xs[e] = Real(0);
            for (int ib = 0; ib < bra.npp; ++ib)
            {
                const int j = ib % GS;
                if (j == 0)
                {
                    // The next GS bra primitives' scalars, one per lane.
                    if (ib + lane < bra.npp)
                        prim_scalars(static_cast<const Real*>(v.pptab[PCB]) + static_cast<size_t>(bra.pp_off + ib + lane) * SB, rk,
                                     Sb + lane * kScal);
                    __syncwarp(gmask);
                }
                // The bra's 3-D Hermite coefficients from its forward record, as for the ket in the first pass.
                const Real* __restrict__ rb = static_cast<const Real*>(v.pptab[PCB]) + static_cast<size_t>(bra.pp_off + ib) * SB;
                const Real* R = group_R(Sb + j * kScal);
                auto Ridx = [&](int t, int u, int w_) { return R[tabs->cube[L][(t * S + u) * S + w_]]; };
                for (int e = lane; e < NAB * HCD1; e += GS)
                {
                    const int ij = e / HCD1, h = e % HCD1;
                    const int tuv = tabs->htuv[LCD + 1][h];
                    const int ta = tuv & 255, nu = (tuv >> 8) & 255, ph = tuv >> 16;
                    const int4 g3 = tabs->e3[PCB][ij];
                    const Real* E3 = rb + g3.w;
                    Real s  = Real(0);
                    int idx = 0;
                    for (int w_ = 0; w_ < g3.z; ++w_)
                        for (int u = 0; u < g3.y; ++u)
                            for (int t = 0; t < g3.x; ++t, ++idx)
                                s = fma((LAB == 0) ? Real(1) : E3[idx], Ridx(t + ta, u + nu, w_ + ph), s);
                    Xs[e] += s;
                }
                __syncwarp(gmask);
            }
            for (int e = lane; e < NCD * HCD1; e += GS)
            {
                const int kl = e / HCD1, h = e % HCD1;
                Real hv = Real(0);
                for (int ij = 0; ij < NAB; ++ij) hv += Gam[ij * NCD + kl] * Xs[ij * HCD1 + h];
                if (hv == Real(0))
                    continue;
                const int tuv = tabs->htuv[LCD + 1][h];
                const int tt[3] = {tuv & 255, (tuv >> 8) & 255, tuv >> 16};
                if ((tt[0] + tt[1] + tt[2]) & 1)
                    hv = -hv;
                const int k = kl / ND, l = kl % ND;
                const int ke[3] = {cart_exp(LC, k, 0), cart_exp(LC, k, 1), cart_exp(LC, k, 2)};
                const int le[3] = {cart_exp(LD, l, 0), cart_exp(LD, l, 1), cart_exp(LD, l, 2)};
                const Real* E[3] = {gk + 2, gk + 2 + G1K, gk + 2 + 2 * G1K};
                Real f[3], dC[3];
                for (int x = 0; x < 3; ++x)
                {
                    const int t = tt[x];
                    f[x]  = (t <= ke[x] + le[x]) ? e1(E[x], LD, LCD, ke[x], le[x], t) : Real(0);
                    dC[x] = Real(2) * cexp * e1(E[x], LD, LCD, ke[x] + 1, le[x], t) -
                            (ke[x] > 0 ? ke[x] * e1(E[x], LD, LCD, ke[x] - 1, le[x], t) : Real(0));
                }
                gC[0] += hv * dC[0] * f[1] * f[2];
                gC[1] += hv * f[0] * dC[1] * f[2];
                gC[2] += hv * f[0] * f[1] * dC[2];
            }
            __syncwarp(gmask);
        }
        for (int x = 0; x < 3; ++x)
            for (int o = GS / 2; o > 0; o >>= 1)
            {
                gA[x] += __shfl_down_sync(gmask, gA[x], o, GS);
                gB[x] += __shfl_down_sync(gmask, gB[x], o, GS);
                gC[x] += __shfl_down_sync(gmask, gC[x], o, GS);
            }
        if (lane == 0)
        {
            const int ta = v.shell_atom[bra.sh1], tb = v.shell_atom[bra.sh2];
            const int tc = v.shell_atom[ket.sh1], td = v.shell_atom[ket.sh2];
            for (int x = 0; x < 3; ++x)
            {
                atomicAdd(v.grad + 3 * ta + x, widen(gA[x]));
                atomicAdd(v.grad + 3 * tb + x, widen(gB[x]));
                atomicAdd(v.grad + 3 * tc + x, widen(gC[x]));
                atomicAdd(v.grad + 3 * td + x, widen(-(gA[x] + gB[x] + gC[x])));
            }
        }
        __syncwarp(gmask);
    }
}

// Thread-per-quartet form of the gradient for the small classes: every loop over Cartesian components and
// Hermite indices unrolled at compile time, the per-quartet arrays in registers.  Two passes over the
// primitive quartets:
//   bra-outer:  Gs[tuv][kl] = sum_{ket prims} sum_{tau nu phi} (-1)^{tau+nu+phi} E^{kl}_{tau nu phi} R_{t+tau,..}
//               (t+u+v <= l_ab + 1) accumulates over the ket primitives of one bra primitive pair; then
//               y[ij][tuv] = sum_kl Gamma_ijkl Gs[tuv][kl] once per bra primitive pair, and
//               g_A += DA . y,  g_P += E . y(t+1)  (d/dA + d/dB = d/dP: the R index shifted by one);
//   ket-outer:  Hs[tuv'][ij] = sum_{bra prims} sum_tuv E^{ij}_{tuv} R_{t+tau,..} (tau+nu+phi <= l_cd + 1),
//               h = sum_ij Gamma_ijkl Hs once per ket primitive pair, g_C += (-1)^{..} DC . h;
// g_B = g_P - g_A and g_D = -(g_P + g_C).  The Gamma contraction runs once per primitive pair instead of
// once per primitive quartet; every term whose Hermite index lies outside the non-zero range of its
// coefficients is dropped at compile time.  Warp-uniform iteration: when the 32 quartets of a warp share
// the bra pair (bra-sorted lists), g_A and g_B are summed over the warp and added once.
template <int LA, int LB, int LC, int LD> struct GradThread
{
    static constexpr int NAB = ncart(LA) * ncart(LB), NCD = ncart(LC) * ncart(LD);
    static constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD + 1;
    static constexpr int HAB1 = nherm(LAB + 1), HCD1 = nherm(LCD + 1);
    // Values a thread holds at the peak of either pass (Gamma, R, and the pass's accumulator array).
    static constexpr int kPass1 = NAB * NCD + nherm(L) + HAB1 * NCD;
    static constexpr int kPass2 = NAB * NCD + nherm(L) + HCD1 * NAB;
    static constexpr int kValues = kPass1 > kPass2 ? kPass1 : kPass2;
};

template <int LA, int LB, int LC, int LD, typename Real>
__global__ void __launch_bounds__(128)
    grad_thread_kernel(const Quartet* __restrict__ list, unsigned long long n, GradView v, const Real* __restrict__ boys_slice)
{
    using W = GradThread<LA, LB, LC, LD>;
    constexpr int NB = ncart(LB), ND = ncart(LD), NAB = W::NAB, NCD = W::NCD;
    constexpr int LAB = W::LAB, LCD = W::LCD, L = W::L, HAB1 = W::HAB1, HCD1 = W::HCD1;
    constexpr int SB = pp_stride(LA, LB), SK = pp_stride(LC, LD);
    constexpr int GB = g_stride(LA, LB), GK = g_stride(LC, LD);
    constexpr int PCB = pair_class(LA, LB), PCK = pair_class(LC, LD);
    constexpr int G1B = g1d_size(LA, LB), G1K = g1d_size(LC, LD);
    // 1-D Hermite coefficient E[i][j][t] of a gradient record's axis table (extents l1+2, l2+2, l1+l2+3).
    constexpr int XB = (LB + 2) * (LAB + 3), YB = LAB + 3, XK = (LD + 2) * (LCD + 3), YK = LCD + 3;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* slice = reinterpret_cast<Real*>(smem_raw);
    if (static_cast<unsigned long long>(blockIdx.x) * blockDim.x >= n)
        return;
    stage_boys<Real>(boys_slice, slice);
    const Real* __restrict__ tbf = static_cast<const Real*>(v.pptab[PCB]);
    const Real* __restrict__ tkf = static_cast<const Real*>(v.pptab[PCK]);
    const Real* __restrict__ tbg = static_cast<const Real*>(v.gtab[PCB]);
    const Real* __restrict__ tkg = static_cast<const Real*>(v.gtab[PCK]);
    const Real* Dt = static_cast<const Real*>(v.Dt);
    const Real* Da = static_cast<const Real*>(v.Da);
    const Real* Db = static_cast<const Real*>(v.Db);
    const int lane = threadIdx.x & 31;

    for (unsigned long long base = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u);
         base < n; base += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
    {
        const unsigned long long q = base + lane;
        const bool active          = q < n;
        const Quartet qt           = list[active ? q : base];
        const PairRec bra          = v.pairs[qt.bra];
        const PairRec ket          = v.pairs[qt.ket];
        Real gA[3] = {0, 0, 0}, gP[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
        if (active)
        {
            const int nn = v.n;
            const long long a0 = bra.ao1, b0 = bra.ao2, c0 = ket.ao1, d0 = ket.ao2;
            const Real sdeg = Real(4) * (bra.same ? Real(0.5) : Real(1)) * (ket.same ? Real(0.5) : Real(1)) *
                              (qt.bra == qt.ket ? Real(0.5) : Real(1));
            Real Gam[NAB * NCD];
            static_for<0, NAB * NCD>(
                [&](auto EE)
                {
                    constexpr int e = decltype(EE)::value;
                    constexpr int ij = e / NCD, kl = e % NCD;
                    constexpr int i = ij / NB, j = ij % NB, k = kl / ND, l = kl % ND;
                    constexpr Real an = Real(ang_norm(LA, i) * ang_norm(LB, j) * ang_norm(LC, k) * ang_norm(LD, l));
                    const long long I = a0 + i, J = b0 + j, K = c0 + k, Lx = d0 + l;
                    auto D = [&](const Real* M, long long r, long long c) { return M[r + c * nn]; };
                    const Real g = D(Dt, I, J) * D(Dt, K, Lx) -
                                   Real(0.5) * (D(Da, I, K) * D(Da, J, Lx) + D(Da, I, Lx) * D(Da, J, K) +
                                                D(Db, I, K) * D(Db, J, Lx) + D(Db, I, Lx) * D(Db, J, K));
                    Gam[e] = (sdeg * an) * g;
                });

            // R^0_{tuv}, t+u+v <= L, of one primitive quartet.
            auto prim_R = [&](const Real* rb, const Real* rk, Real* R)
            {
                const Real p = rb[0], qq = rk[0];
                const Real X = rb[1] - rk[1], Y = rb[2] - rk[2], Z = rb[3] - rk[3];
                const Real rs   = hfg_rsqrt(p + qq);
                const Real rho  = (p * qq) * (rs * rs);
                const Real pref = (rb[4] * rk[4]) * rs;
                const Real T    = rho * (X * X + Y * Y + Z * Z);
                Real F[L + 1];
                boys_eval<L, Real>(T, slice, F);
                Real Fs[L + 1];
                const Real m2r = Real(-2) * rho;
                Real w         = pref;
#pragma unroll
                for (int m = 0; m <= L; ++m)
                {
                    Fs[m] = w * F[m];
                    w *= m2r;
                }
                hermite_R<L, Real>(Fs, X, Y, Z, R);
            };

            // Bra-outer pass: centres A and P.
            for (int ib = 0; ib < bra.npp; ++ib)
            {
                const Real* __restrict__ rb = tbf + static_cast<size_t>(bra.pp_off + ib) * SB;
                Real Gs[HAB1 * NCD];
#pragma unroll
                for (int x = 0; x < HAB1 * NCD; ++x) Gs[x] = Real(0);
                for (int ik = 0; ik < ket.npp; ++ik)
                {
                    const Real* __restrict__ rk = tkf + static_cast<size_t>(ket.pp_off + ik) * SK;
                    Real R[nherm(L)];
                    prim_R(rb, rk, R);
                    static_for<0, NCD>(
                        [&](auto KL)
                        {
                            constexpr int kl   = decltype(KL)::value;
                            constexpr int lx   = e3_len(LC, LD, kl, 0), ly = e3_len(LC, LD, kl, 1), lz = e3_len(LC, LD, kl, 2);
                            constexpr int eoff = kPairHeader + e3_offset(LC, LD, kl);
                            static_for<0, HAB1>(
                                [&](auto H)
                                {
                                    constexpr int h = decltype(H)::value;
                                    constexpr int t = htuv(h, LAB + 1, 0), u = htuv(h, LAB + 1, 1), w_ = htuv(h, LAB + 1, 2);
                                    Real s = Real(0);
                                    static_for<0, lx * ly * lz>(
                                        [&](auto EE)
                                        {
                                            constexpr int e   = decltype(EE)::value;
                                            constexpr int tau = e % lx, nu = (e / lx) % ly, phi = e / (lx * ly);
                                            const Real rr   = R[hidx(t + tau, u + nu, w_ + phi, L)];
                                            const Real term = (LCD == 0) ? rr : rk[eoff + e] * rr;
                                            if constexpr (((tau + nu + phi) & 1) != 0)
                                                s -= term;
                                            else
                                                s += term;
                                        });
                                    Gs[h * NCD + kl] += s;
                                });
                        });
                }
                const Real* __restrict__ gb = tbg + static_cast<size_t>(bra.pp_off + ib) * GB;
                const Real a2 = Real(2) * gb[0];
                const Real* Ex = gb + 2;
                const Real* Ey = Ex + G1B;
                const Real* Ez = Ey + G1B;
                static_for<0, NAB>(
                    [&](auto IJ)
                    {
                        constexpr int ij = decltype(IJ)::value;
                        constexpr int i = ij / NB, j = ij % NB;
                        constexpr int ix = cart_exp(LA, i, 0), iy = cart_exp(LA, i, 1), iz = cart_exp(LA, i, 2);
                        constexpr int jx = cart_exp(LB, j, 0), jy = cart_exp(LB, j, 1), jz = cart_exp(LB, j, 2);
                        static_for<0, HAB1>(
                            [&](auto H)
                            {
                                constexpr int h = decltype(H)::value;
                                constexpr int t = htuv(h, LAB + 1, 0), u = htuv(h, LAB + 1, 1), w_ = htuv(h, LAB + 1, 2);
                                constexpr bool inx = t <= ix + jx + 1 && u <= iy + jy && w_ <= iz + jz;
                                constexpr bool iny = t <= ix + jx && u <= iy + jy + 1 && w_ <= iz + jz;
                                constexpr bool inz = t <= ix + jx && u <= iy + jy && w_ <= iz + jz + 1;
                                if constexpr (inx || iny || inz)
                                {
                                    Real y = Real(0);
#pragma unroll
                                    for (int kl = 0; kl < NCD; ++kl) y += Gam[ij * NCD + kl] * Gs[h * NCD + kl];
                                    // E^{ij} along each axis at the index of this term, and its A derivative.
                                    auto e1 = [](const Real* T, int ii, int jj, int tt, int XS, int YS) { return T[ii * XS + jj * YS + tt]; };
                                    auto dA = [&](const Real* T, int ii, int jj, int tt)
                                    {
                                        Real r = a2 * e1(T, ii + 1, jj, tt, XB, YB);
                                        if (ii > 0 && tt <= ii - 1 + jj)
                                            r -= Real(ii) * e1(T, ii - 1, jj, tt, XB, YB);
                                        return r;
                                    };
                                    const Real fx = t <= ix + jx ? e1(Ex, ix, jx, t, XB, YB) : Real(0);
                                    const Real fy = u <= iy + jy ? e1(Ey, iy, jy, u, XB, YB) : Real(0);
                                    const Real fz = w_ <= iz + jz ? e1(Ez, iz, jz, w_, XB, YB) : Real(0);
                                    if constexpr (inx)
                                    {
                                        const Real yz = y * fy * fz;
                                        gA[0] += yz * dA(Ex, ix, jx, t);
                                        if constexpr (t >= 1)
                                            gP[0] += yz * e1(Ex, ix, jx, t - 1, XB, YB);
                                    }
                                    if constexpr (iny)
                                    {
                                        const Real xz = y * fx * fz;
                                        gA[1] += xz * dA(Ey, iy, jy, u);
                                        if constexpr (u >= 1)
                                            gP[1] += xz * e1(Ey, iy, jy, u - 1, XB, YB);
                                    }
                                    if constexpr (inz)
                                    {
                                        const Real xy = y * fx * fy;
                                        gA[2] += xy * dA(Ez, iz, jz, w_);
                                        if constexpr (w_ >= 1)
                                            gP[2] += xy * e1(Ez, iz, jz, w_ - 1, XB, YB);
                                    }
                                }
                            });
                    });
            }

            // Ket-outer pass: centre C.
            for (int ik = 0; ik < ket.npp; ++ik)
            {
                const Real* __restrict__ rk = tkf + static_cast<size_t>(ket.pp_off + ik) * SK;
                Real Hs[HCD1 * NAB];
#pragma unroll
                for (int x = 0; x < HCD1 * NAB; ++x) Hs[x] = Real(0);
                for (int ib = 0; ib < bra.npp; ++ib)
                {
                    const Real* __restrict__ rb = tbf + static_cast<size_t>(bra.pp_off + ib) * SB;
                    Real R[nherm(L)];
                    prim_R(rb, rk, R);
                    static_for<0, NAB>(
                        [&](auto IJ)
                        {
                            constexpr int ij   = decltype(IJ)::value;
                            constexpr int lx   = e3_len(LA, LB, ij, 0), ly = e3_len(LA, LB, ij, 1), lz = e3_len(LA, LB, ij, 2);
                            constexpr int eoff = kPairHeader + e3_offset(LA, LB, ij);
                            static_for<0, HCD1>(
                                [&](auto H)
                                {
                                    constexpr int h   = decltype(H)::value;
                                    constexpr int tau = htuv(h, LCD + 1, 0), nu = htuv(h, LCD + 1, 1), phi = htuv(h, LCD + 1, 2);
                                    Real s = Real(0);
                                    static_for<0, lx * ly * lz>(
                                        [&](auto EE)
                                        {
                                            constexpr int e = decltype(EE)::value;
                                            constexpr int t = e % lx, u = (e / lx) % ly, w_ = e / (lx * ly);
                                            const Real rr = R[hidx(t + tau, u + nu, w_ + phi, L)];
                                            s += (LAB == 0) ? rr : rb[eoff + e] * rr;
                                        });
                                    Hs[h * NAB + ij] += s;
                                });
                        });
                }
                const Real* __restrict__ gk = tkg + static_cast<size_t>(ket.pp_off + ik) * GK;
                const Real c2 = Real(2) * gk[0];
                const Real* Ex = gk + 2;
                const Real* Ey = Ex + G1K;
                const Real* Ez = Ey + G1K;
                static_for<0, NCD>(
                    [&](auto KL)
                    {
                        constexpr int kl = decltype(KL)::value;
                        constexpr int k = kl / ND, l = kl % ND;
                        constexpr int kx = cart_exp(LC, k, 0), ky = cart_exp(LC, k, 1), kz = cart_exp(LC, k, 2);
                        constexpr int lx = cart_exp(LD, l, 0), ly = cart_exp(LD, l, 1), lz = cart_exp(LD, l, 2);
                        static_for<0, HCD1>(
                            [&](auto H)
                            {
                                constexpr int h   = decltype(H)::value;
                                constexpr int tau = htuv(h, LCD + 1, 0), nu = htuv(h, LCD + 1, 1), phi = htuv(h, LCD + 1, 2);
                                constexpr bool inx = tau <= kx + lx + 1 && nu <= ky + ly && phi <= kz + lz;
                                constexpr bool iny = tau <= kx + lx && nu <= ky + ly + 1 && phi <= kz + lz;
                                constexpr bool inz = tau <= kx + lx && nu <= ky + ly && phi <= kz + lz + 1;
                                if constexpr (inx || iny || inz)
                                {
                                    Real hv = Real(0);
#pragma unroll
                                    for (int ij = 0; ij < NAB; ++ij) hv += Gam[ij * NCD + kl] * Hs[h * NAB + ij];
                                    if constexpr (((tau + nu + phi) & 1) != 0)
                                        hv = -hv;
                                    auto e1 = [](const Real* T, int ii, int jj, int tt) { return T[ii * XK + jj * YK + tt]; };
                                    auto dC = [&](const Real* T, int ii, int jj, int tt)
                                    {
                                        Real r = c2 * e1(T, ii + 1, jj, tt);
                                        if (ii > 0 && tt <= ii - 1 + jj)
                                            r -= Real(ii) * e1(T, ii - 1, jj, tt);
                                        return r;
                                    };
                                    const Real fx = tau <= kx + lx ? e1(Ex, kx, lx, tau) : Real(0);
                                    const Real fy = nu <= ky + ly ? e1(Ey, ky, ly, nu) : Real(0);
                                    const Real fz = phi <= kz + lz ? e1(Ez, kz, lz, phi) : Real(0);
                                    if constexpr (inx)
                                        gC[0] += hv * fy * fz * dC(Ex, kx, lx, tau);
                                    if constexpr (iny)
                                        gC[1] += hv * fx * fz * dC(Ey, ky, ly, nu);
                                    if constexpr (inz)
                                        gC[2] += hv * fx * fy * dC(Ez, kz, lz, phi);
                                }
                            });
                    });
            }
        }
        // g_B = g_P - g_A, g_D = -(g_P + g_C); the bra atoms' terms summed over the warp when it shares the bra.
        const unsigned bra0 = __shfl_sync(0xffffffffu, qt.bra, 0);
        const bool bra_warp = __all_sync(0xffffffffu, qt.bra == bra0);
        Real gB[3], gD[3];
#pragma unroll
        for (int x = 0; x < 3; ++x)
        {
            gB[x] = gP[x] - gA[x];
            gD[x] = -(gP[x] + gC[x]);
        }
        const int ta = v.shell_atom[bra.sh1], tb = v.shell_atom[bra.sh2];
        if (bra_warp)
        {
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                {
                    gA[x] += __shfl_xor_sync(0xffffffffu, gA[x], o);
                    gB[x] += __shfl_xor_sync(0xffffffffu, gB[x], o);
                }
        }
        if (bra_warp ? lane == 0 : active)
#pragma unroll
            for (int x = 0; x < 3; ++x)
            {
                atomicAdd(v.grad + 3 * ta + x, widen(gA[x]));
                atomicAdd(v.grad + 3 * tb + x, widen(gB[x]));
            }
        if (active)
        {
            const int tc = v.shell_atom[ket.sh1], td = v.shell_atom[ket.sh2];
#pragma unroll
            for (int x = 0; x < 3; ++x)
            {
                atomicAdd(v.grad + 3 * tc + x, widen(gC[x]));
                atomicAdd(v.grad + 3 * td + x, widen(gD[x]));
            }
        }
    }
}
#endif
} // namespace hfg
