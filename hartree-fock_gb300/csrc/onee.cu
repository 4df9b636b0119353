// One-electron integrals S, T, V and the one-electron part of the nuclear gradient on the GPU, FP64.
//
// Reference counterparts: IntegralEngine::overlap / kinetic / nuclearAttraction and the *Matrix drivers
// (src/IntegralEngine.cpp:78-368).  McMurchie-Davidson as in the host code (host_onee.cpp,
// host_grad.cpp): per primitive pair the 1-D Hermite tables E^{ij}_t (ket index up to l_b + 2 for the
// kinetic integral, bra up to l_a + 1 for the centre derivative), S = (pi/p)^{3/2} K E^x_0 E^y_0 E^z_0,
// T through overlaps with the ket exponent shifted by +-2, V = -(2 pi / p) K sum_C Z_C sum_tuv E R_tuv(P-C).
//
// Layout of the work: one warp per shell pair (oriented l_a >= l_b, one kernel per pair class so that the
// Hermite recursion is unrolled at compile time).  Per primitive pair the three 1-D tables are built in the
// warp's shared memory, the lanes split the nuclei (each lane sums Z_C R_tuv(P - C) over its nuclei, then a
// butterfly sum over the warp), and then split the integrals of the shell pair.  Gradient: the lanes split
// the integrals for the overlap and kinetic derivatives, the Hermite indices for the density-weighted
// Hermite tables, and the nuclei for the nuclear-attraction derivative; the operator-centre terms go to a
// per-block copy of the gradient in shared memory, added to the global gradient once per block.
#include "eri_jk.cuh"
#include "hfgpu.h"
#include "onee.h"

#include <cuda_runtime.h>

namespace hfg
{
namespace
{
constexpr int kOneeWarps = 4;
constexpr double kPi     = 3.14159265358979323846;

// 1-D Hermite table of one axis for i <= I, j <= J: E[(i * (J + 1) + j) * (I + J + 1) + t].
template <int I, int J> __device__ __forceinline__ void hermite_axis_dev(double p, double PA, double PB, double* E)
{
    constexpr int TT = I + J + 1;
    for (int k = 0; k < (I + 1) * (J + 1) * TT; ++k) E[k] = 0.0;
    const double h = 0.5 / p;
    E[0]           = 1.0;
    for (int i = 0; i <= I; ++i)
        for (int j = 0; j <= J; ++j)
        {
            if (i == 0 && j == 0)
                continue;
            const bool up_i   = i > 0;
            const int pi      = up_i ? i - 1 : i, pj = up_i ? j : j - 1;
            const double X    = up_i ? PA : PB;
            const double* src = E + (pi * (J + 1) + pj) * TT;
            double* dst       = E + (i * (J + 1) + j) * TT;
            for (int t = 0; t <= i + j; ++t)
            {
                double v = 0.0;
                if (t <= pi + pj)
                    v += X * src[t];
                if (t >= 1)
                    v += h * src[t - 1];
                if (t + 1 <= pi + pj)
                    v += (t + 1) * src[t + 1];
                dst[t] = v;
            }
        }
}

struct PrimPair
{
    double a, b, p, ip, K, cprod, P[3], PA[3], PB[3];
};

__device__ __forceinline__ PrimPair prim_pair(const OneeBasis& B, int sa, int sb, int pa, int pb)
{
    PrimPair q;
    const double* A  = B.centers + 3 * sa;
    const double* Bc = B.centers + 3 * sb;
    q.a              = B.alpha[B.prim_off[sa] + pa];
    q.b              = B.alpha[B.prim_off[sb] + pb];
    q.p              = q.a + q.b;
    q.ip             = 1.0 / q.p;
    double AB2       = 0.0;
    for (int x = 0; x < 3; ++x)
    {
        q.P[x]  = (q.a * A[x] + q.b * Bc[x]) * q.ip;
        q.PA[x] = q.P[x] - A[x];
        q.PB[x] = q.P[x] - Bc[x];
        AB2 += (A[x] - Bc[x]) * (A[x] - Bc[x]);
    }
    q.K     = exp(-q.a * q.b * q.ip * AB2);
    q.cprod = B.coeff[B.prim_off[sa] + pa] * B.coeff[B.prim_off[sb] + pb];
    return q;
}

// R_tuv(p, P - C) for t+u+v <= L (hidx(t,u,v,L) layout) of one nucleus at C.
template <int L>
__device__ __forceinline__ void nuclear_R(const double* P, double p, const double4& C, const double* __restrict__ slice,
                                          double* R)
{
    const double X = P[0] - C.x, Y = P[1] - C.y, Z = P[2] - C.z;
    double F[L + 1], Fs[L + 1];
    boys_eval<L, double>(p * (X * X + Y * Y + Z * Z), slice, F);
    double f = 1.0;
#pragma unroll
    for (int m = 0; m <= L; ++m)
    {
        Fs[m] = f * F[m];
        f *= -2.0 * p;
    }
    hermite_R<L, double>(Fs, X, Y, Z, R);
}

template <int LA, int LB>
__global__ void __launch_bounds__(32 * kOneeWarps) stv_kernel(const int2* __restrict__ pairs, int npairs, OneeBasis B,
                                                              const double4* __restrict__ nuc, int natom, int n,
                                                              const double* __restrict__ boys_slice, double* S,
                                                              double* T, double* V)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), L = LA + LB, H = nherm(L);
    constexpr int I = LA, J = LB + 2, TT = I + J + 1, AX = (I + 1) * (J + 1) * TT;
    constexpr int kSlice = BoysGrid<double>::kPoints * BoysGrid<double>::kRow;
    constexpr int M      = (NA * NB + 31) / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* slice = reinterpret_cast<double*>(smem_raw);
    for (int i = threadIdx.x; i < kSlice; i += blockDim.x) slice[i] = boys_slice[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    double* E  = slice + kSlice + wib * (3 * AX + H);
    double* Rs = E + 3 * AX; // the warp's sum over nuclei of Z_C R_tuv(P - C)
    for (int k = blockIdx.x * kOneeWarps + wib; k < npairs; k += gridDim.x * kOneeWarps)
    {
        const int sa = pairs[k].x, sb = pairs[k].y;
        double s_acc[M] = {}, t_acc[M] = {}, v_acc[M] = {};
        for (int pa = 0; pa < B.nprim[sa]; ++pa)
            for (int pb = 0; pb < B.nprim[sb]; ++pb)
            {
                const PrimPair q = prim_pair(B, sa, sb, pa, pb);
                // Same skip as the host code: K below 1e-30 adds nothing representable.
                if (q.K < 1e-30)
                    continue;
                __syncwarp();
                if (lane < 3)
                    hermite_axis_dev<I, J>(q.p, q.PA[lane], q.PB[lane], E + lane * AX);
                double Rsum[H];
#pragma unroll
                for (int h = 0; h < H; ++h) Rsum[h] = 0.0;
                for (int c = lane; c < natom; c += 32)
                {
                    const double4 C = nuc[c];
                    double R[H];
                    nuclear_R<L>(q.P, q.p, C, slice, R);
#pragma unroll
                    for (int h = 0; h < H; ++h) Rsum[h] += C.w * R[h];
                }
#pragma unroll
                for (int h = 0; h < H; ++h)
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) Rsum[h] += __shfl_xor_sync(0xffffffffu, Rsum[h], o);
                if (lane == 0)
#pragma unroll
                    for (int h = 0; h < H; ++h) Rs[h] = Rsum[h];
                __syncwarp();
                const double prefS = pow(kPi * q.ip, 1.5) * q.K;
                const double prefV = 2.0 * kPi * q.ip * q.K;
                auto e1 = [&](int ax, int i, int j, int t) { return E[ax * AX + (i * (J + 1) + j) * TT + t]; };
#pragma unroll
                for (int m = 0; m < M; ++m)
                {
                    const int e = lane + 32 * m;
                    if (e >= NA * NB)
                        continue;
                    const int i = e / NB, j = e % NB;
                    const int ix = cart_exp(LA, i, 0), iy = cart_exp(LA, i, 1), iz = cart_exp(LA, i, 2);
                    const int jx = cart_exp(LB, j, 0), jy = cart_exp(LB, j, 1), jz = cart_exp(LB, j, 2);
                    const double w = B.norms[B.norm_off[sa] + pa * NA + i] * B.norms[B.norm_off[sb] + pb * NB + j] * q.cprod;
                    const double ex = e1(0, ix, jx, 0), ey = e1(1, iy, jy, 0), ez = e1(2, iz, jz, 0);
                    s_acc[m] += w * prefS * ex * ey * ez;
                    const double t1 = q.b * (2 * (jx + jy + jz) + 3) * ex * ey * ez;
                    const double t2 = -2.0 * q.b * q.b *
                                      (e1(0, ix, jx + 2, 0) * ey * ez + ex * e1(1, iy, jy + 2, 0) * ez + ex * ey * e1(2, iz, jz + 2, 0));
                    double t3 = 0.0;
                    if (jx >= 2)
                        t3 -= jx * (jx - 1) * e1(0, ix, jx - 2, 0) * ey * ez;
                    if (jy >= 2)
                        t3 -= jy * (jy - 1) * ex * e1(1, iy, jy - 2, 0) * ez;
                    if (jz >= 2)
                        t3 -= jz * (jz - 1) * ex * ey * e1(2, iz, jz - 2, 0);
                    t_acc[m] += w * prefS * (t1 + t2 + 0.5 * t3);
                    double vs = 0.0;
                    for (int vv = 0; vv <= iz + jz; ++vv)
                        for (int u = 0; u <= iy + jy; ++u)
                            for (int t = 0; t <= ix + jx; ++t)
                                vs += e1(0, ix, jx, t) * e1(1, iy, jy, u) * e1(2, iz, jz, vv) * Rs[hidx(t, u, vv, L)];
                    v_acc[m] -= w * prefV * vs;
                }
            }
#pragma unroll
        for (int m = 0; m < M; ++m)
        {
            const int e = lane + 32 * m;
            if (e >= NA * NB)
                continue;
            const long long r = B.ao_off[sa] + e / NB, c = B.ao_off[sb] + e % NB;
            S[r + c * n] = S[c + r * n] = s_acc[m];
            T[r + c * n] = T[c + r * n] = t_acc[m];
            V[r + c * n] = V[c + r * n] = v_acc[m];
        }
    }
}

template <int LA, int LB> cudaError_t launch_stv(const OneeLaunch& c)
{
    constexpr int I = LA, J = LB + 2, TT = I + J + 1, AX = (I + 1) * (J + 1) * TT;
    const size_t smem =
        sizeof(double) * (BoysGrid<double>::kPoints * BoysGrid<double>::kRow + kOneeWarps * (3 * AX + nherm(LA + LB)));
    auto kern     = stv_kernel<LA, LB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess)
        return e;
    const int need = (c.npairs + kOneeWarps - 1) / kOneeWarps;
    const int grid = need < c.num_sms * 8 ? need : c.num_sms * 8;
    kern<<<grid > 0 ? grid : 1, 32 * kOneeWarps, smem, c.stream>>>(c.pairs, c.npairs, c.basis, c.nuc, c.natom, c.n,
                                                                   static_cast<const double*>(c.boys_slice), c.S, c.T,
                                                                   c.V);
    return cudaGetLastError();
}

// One-electron gradient of every pair (sa, sb) of one pair class (host_grad.cpp restated for one warp per
// pair): pair weight 2 off the diagonal, centre derivatives 2a phi_{i+1} - i phi_{i-1}; S and T depend on
// A - B only; the operator centre of V gets dR_tuv(P - C)/dC = -R_{tuv + 1_x}.
template <int LA, int LB>
__global__ void __launch_bounds__(32 * kOneeWarps)
    stv_grad_kernel(const int2* __restrict__ pairs, int npairs, OneeBasis B, const double4* __restrict__ nuc, int natom,
                    int n, const double* __restrict__ boys_slice, const double* __restrict__ D,
                    const double* __restrict__ W, const int* __restrict__ shell_atom, double* grad, int block_grad)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NAB = NA * NB;
    constexpr int Lt = LA + LB + 1, L2 = Lt + 1, H = nherm(Lt);
    constexpr int I = LA + 1, J = LB + 2, TT = I + J + 1, AX = (I + 1) * (J + 1) * TT;
    constexpr int kPerWarp = 3 * AX + 7 * H + 2 * NAB;
    constexpr int kSlice   = BoysGrid<double>::kPoints * BoysGrid<double>::kRow;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* slice = reinterpret_cast<double*>(smem_raw);
    double* gblk  = slice + kSlice + kOneeWarps * kPerWarp; // the block's copy of the gradient (block_grad)
    for (int i = threadIdx.x; i < kSlice; i += blockDim.x) slice[i] = boys_slice[i];
    if (block_grad)
        for (int i = threadIdx.x; i < 3 * natom; i += blockDim.x) gblk[i] = 0.0;
    __syncthreads();
    double* gout   = block_grad ? gblk : grad;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    double* E   = slice + kSlice + wib * kPerWarp;
    double* ED  = E + 3 * AX;  // [H]      sum_ij wD_ij E^{ij}_tuv
    double* DA  = ED + H;      // [3][H]   with the bra centre derivative
    double* DB  = DA + 3 * H;  // [3][H]   with the ket centre derivative
    double* wDs = DB + 3 * H;  // [NAB]    w D_ij of this primitive pair
    double* wWs = wDs + NAB;   // [NAB]    w W_ij
    for (int k = blockIdx.x * kOneeWarps + wib; k < npairs; k += gridDim.x * kOneeWarps)
    {
        const int sa = pairs[k].x, sb = pairs[k].y;
        const int atA = shell_atom[sa], atB = shell_atom[sb];
        const double pair_w = sa == sb ? 1.0 : 2.0;
        double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
        for (int pa = 0; pa < B.nprim[sa]; ++pa)
            for (int pb = 0; pb < B.nprim[sb]; ++pb)
            {
                const PrimPair q = prim_pair(B, sa, sb, pa, pb);
                if (q.K < 1e-30)
                    continue;
                __syncwarp();
                if (lane < 3)
                    hermite_axis_dev<I, J>(q.p, q.PA[lane], q.PB[lane], E + lane * AX);
                for (int e = lane; e < NAB; e += 32)
                {
                    const int i = e / NB, j = e % NB;
                    const long long mu = B.ao_off[sa] + i, nu = B.ao_off[sb] + j;
                    const double w = pair_w * B.norms[B.norm_off[sa] + pa * NA + i] *
                                     B.norms[B.norm_off[sb] + pb * NB + j] * q.cprod;
                    wDs[e] = w * D[mu + nu * n];
                    wWs[e] = w * W[mu + nu * n];
                }
                __syncwarp();
                const double prefS = pow(kPi * q.ip, 1.5) * q.K;
                const double prefV = 2.0 * kPi * q.ip * q.K;
                auto e1 = [&](int ax, int i, int j, int t) -> double {
                    return (i < 0 || j < 0 || t > i + j) ? 0.0 : E[ax * AX + (i * (J + 1) + j) * TT + t];
                };
                auto ovl = [&](const int* i, const int* j) {
                    return prefS * e1(0, i[0], j[0], 0) * e1(1, i[1], j[1], 0) * e1(2, i[2], j[2], 0);
                };
                auto kin = [&](const int* i, const int* j) {
                    if (i[0] < 0 || i[1] < 0 || i[2] < 0)
                        return 0.0;
                    double t2 = 0.0, t3 = 0.0;
                    for (int x = 0; x < 3; ++x)
                    {
                        int jp[3] = {j[0], j[1], j[2]};
                        jp[x] += 2;
                        t2 += ovl(i, jp);
                        if (j[x] >= 2)
                        {
                            int jm[3] = {j[0], j[1], j[2]};
                            jm[x] -= 2;
                            t3 -= j[x] * (j[x] - 1) * ovl(i, jm);
                        }
                    }
                    return q.b * (2 * (j[0] + j[1] + j[2]) + 3) * ovl(i, j) - 2.0 * q.b * q.b * t2 + 0.5 * t3;
                };
                // Overlap and kinetic derivatives, lanes over the integrals of the pair.
                for (int e = lane; e < NAB; e += 32)
                {
                    const int ci = e / NB, cj = e % NB;
                    const int i0[3] = {cart_exp(LA, ci, 0), cart_exp(LA, ci, 1), cart_exp(LA, ci, 2)};
                    const int j0[3] = {cart_exp(LB, cj, 0), cart_exp(LB, cj, 1), cart_exp(LB, cj, 2)};
                    for (int x = 0; x < 3; ++x)
                    {
                        int ip1[3] = {i0[0], i0[1], i0[2]}, im1[3] = {i0[0], i0[1], i0[2]};
                        ip1[x] += 1;
                        im1[x] -= 1;
                        const double dS = 2 * q.a * ovl(ip1, j0) - (i0[x] > 0 ? i0[x] * ovl(im1, j0) : 0.0);
                        const double dT = 2 * q.a * kin(ip1, j0) - (i0[x] > 0 ? i0[x] * kin(im1, j0) : 0.0);
                        const double g  = wDs[e] * dT - wWs[e] * dS;
                        gA[x] += g;
                        gB[x] -= g;
                    }
                }
                // Density-weighted Hermite tables, lanes over the Hermite indices.
                for (int h = lane; h < H; h += 32)
                {
                    const int tt[3] = {htuv(h, Lt, 0), htuv(h, Lt, 1), htuv(h, Lt, 2)};
                    double ed = 0.0, da[3] = {0, 0, 0}, db[3] = {0, 0, 0};
                    for (int e = 0; e < NAB; ++e)
                    {
                        const double wd = wDs[e];
                        if (wd == 0.0)
                            continue;
                        const int ci = e / NB, cj = e % NB;
                        const int i0[3] = {cart_exp(LA, ci, 0), cart_exp(LA, ci, 1), cart_exp(LA, ci, 2)};
                        const int j0[3] = {cart_exp(LB, cj, 0), cart_exp(LB, cj, 1), cart_exp(LB, cj, 2)};
                        double f[3], fa[3], fb[3];
                        for (int x = 0; x < 3; ++x)
                        {
                            f[x]  = e1(x, i0[x], j0[x], tt[x]);
                            fa[x] = 2 * q.a * e1(x, i0[x] + 1, j0[x], tt[x]) -
                                    (i0[x] > 0 ? i0[x] * e1(x, i0[x] - 1, j0[x], tt[x]) : 0.0);
                            fb[x] = 2 * q.b * e1(x, i0[x], j0[x] + 1, tt[x]) -
                                    (j0[x] > 0 ? j0[x] * e1(x, i0[x], j0[x] - 1, tt[x]) : 0.0);
                        }
                        ed += wd * f[0] * f[1] * f[2];
                        da[0] += wd * fa[0] * f[1] * f[2];
                        da[1] += wd * f[0] * fa[1] * f[2];
                        da[2] += wd * f[0] * f[1] * fa[2];
                        db[0] += wd * fb[0] * f[1] * f[2];
                        db[1] += wd * f[0] * fb[1] * f[2];
                        db[2] += wd * f[0] * f[1] * fb[2];
                    }
                    ED[h] = ed;
                    for (int x = 0; x < 3; ++x)
                    {
                        DA[x * H + h] = da[x];
                        DB[x * H + h] = db[x];
                    }
                }
                __syncwarp();
                // Nuclear-attraction derivative, lanes over the nuclei.
                for (int c = lane; c < natom; c += 32)
                {
                    const double4 C = nuc[c];
                    double R[nherm(L2)];
                    nuclear_R<L2>(q.P, q.p, C, slice, R);
                    double sa3[3] = {0, 0, 0}, sb3[3] = {0, 0, 0}, sc3[3] = {0, 0, 0};
                    static_for<0, H>(
                        [&](auto Hh)
                        {
                            constexpr int h = decltype(Hh)::value;
                            constexpr int t = htuv(h, Lt, 0), u = htuv(h, Lt, 1), v = htuv(h, Lt, 2);
                            const double r0 = R[hidx(t, u, v, L2)];
#pragma unroll
                            for (int x = 0; x < 3; ++x)
                            {
                                sa3[x] += DA[x * H + h] * r0;
                                sb3[x] += DB[x * H + h] * r0;
                            }
                            const double ed = ED[h];
                            sc3[0] -= ed * R[hidx(t + 1, u, v, L2)];
                            sc3[1] -= ed * R[hidx(t, u + 1, v, L2)];
                            sc3[2] -= ed * R[hidx(t, u, v + 1, L2)];
                        });
                    const double zc = -C.w * prefV;
#pragma unroll
                    for (int x = 0; x < 3; ++x)
                    {
                        gA[x] += zc * sa3[x];
                        gB[x] += zc * sb3[x];
                        atomicAdd(gout + 3 * c + x, zc * sc3[x]);
                    }
                }
            }
#pragma unroll
        for (int x = 0; x < 3; ++x)
        {
            double a = gA[x], b = gB[x];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
                a += __shfl_xor_sync(0xffffffffu, a, o);
                b += __shfl_xor_sync(0xffffffffu, b, o);
            }
            if (lane == 0)
            {
                atomicAdd(gout + 3 * atA + x, a);
                atomicAdd(gout + 3 * atB + x, b);
            }
        }
    }
    if (block_grad)
    {
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * natom; i += blockDim.x)
            if (gblk[i] != 0.0)
                atomicAdd(grad + i, gblk[i]);
    }
}

// Per-block copies of the gradient in shared memory up to this many atoms (48 KB of doubles).
constexpr int kBlockGradAtoms = 2048;

template <int LA, int LB> cudaError_t launch_stv_grad(const OneeLaunch& c)
{
    constexpr int NAB = ncart(LA) * ncart(LB), H = nherm(LA + LB + 1);
    constexpr int I = LA + 1, J = LB + 2, TT = I + J + 1, AX = (I + 1) * (J + 1) * TT;
    const int block_grad = c.natom <= kBlockGradAtoms ? 1 : 0;
    const size_t smem    = sizeof(double) * (BoysGrid<double>::kPoints * BoysGrid<double>::kRow +
                                          kOneeWarps * (3 * AX + 7 * H + 2 * NAB) + (block_grad ? 3 * c.natom : 0));
    auto kern     = stv_grad_kernel<LA, LB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess)
        return e;
    const int need = (c.npairs + kOneeWarps - 1) / kOneeWarps;
    const int grid = need < c.num_sms * 4 ? need : c.num_sms * 4;
    kern<<<grid > 0 ? grid : 1, 32 * kOneeWarps, smem, c.stream>>>(c.pairs, c.npairs, c.basis, c.nuc, c.natom, c.n,
                                                                   static_cast<const double*>(c.boys_slice), c.D, c.W,
                                                                   c.shell_atom, c.grad, block_grad);
    return cudaGetLastError();
}
} // namespace

cudaError_t launch_one_electron(int pc, const OneeLaunch& c)
{
    if (c.npairs == 0)
        return cudaSuccess;
    switch (pc)
    {
    case 0: return launch_stv<0, 0>(c);
    case 1: return launch_stv<1, 0>(c);
    case 2: return launch_stv<1, 1>(c);
    case 3: return launch_stv<2, 0>(c);
    case 4: return launch_stv<2, 1>(c);
    case 5: return launch_stv<2, 2>(c);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_one_electron_grad(int pc, const OneeLaunch& c)
{
    if (c.npairs == 0)
        return cudaSuccess;
    switch (pc)
    {
    case 0: return launch_stv_grad<0, 0>(c);
    case 1: return launch_stv_grad<1, 0>(c);
    case 2: return launch_stv_grad<1, 1>(c);
    case 3: return launch_stv_grad<2, 0>(c);
    case 4: return launch_stv_grad<2, 1>(c);
    case 5: return launch_stv_grad<2, 2>(c);
    default: return cudaErrorInvalidValue;
    }
}
} // namespace hfg
