// One-electron, overlap (energy-weighted density) and nuclear-repulsion parts of the analytic nuclear
// gradient, FP64 on the host (OpenMP over shell pairs).  The reference program has no gradient; the
// integrals differentiated are its own S, T, V (src/IntegralEngine.cpp:78-368) and V_nn
// (src/Molecule.cpp:80-89).
//
//   dE/dX = sum_{mn} D_mn d(T+V)_mn/dX - sum_{mn} W_mn dS_mn/dX + dV_nn/dX + (two-electron part, GPU)
//
// with D the total density, W the total energy-weighted density.  A Cartesian Gaussian's centre
// derivative is d/dA_x phi_i = 2a phi_{i+1_x} - i_x phi_{i-1_x} (same normalisation factor), so each
// derivative integral is a combination of integrals with the bra (or ket) exponent shifted by one.
// S and T depend on A - B only (dS/dB = -dS/dA); the operator centre C of V gets
// dV_C/dC = -(dV_C/dA + dV_C/dB).
#include "hfgpu.h"
#include "hfg_common.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace hfg
{
void host_boys_eval(int L, double T, double* F); // host_onee.cpp

namespace
{
constexpr int kGI = kMaxL + 2; // bra exponent range (l + 1)
constexpr int kGJ = kMaxL + 3; // ket exponent range (l + 2 for the kinetic integral)
constexpr int kGT = kGI + kGJ;

struct Axis
{
    double E[kGI][kGJ][kGT];
};

void hermite_axis_g(int l1, int l2, double p, double PA, double PB, Axis& A)
{
    std::memset(&A, 0, sizeof(A));
    const double h = 0.5 / p;
    A.E[0][0][0]   = 1.0;
    for (int i = 0; i <= l1; ++i)
        for (int j = 0; j <= l2; ++j)
        {
            if (i == 0 && j == 0)
                continue;
            const bool up_i = i > 0;
            const int pi = up_i ? i - 1 : i, pj = up_i ? j : j - 1;
            const double X = up_i ? PA : PB;
            for (int t = 0; t <= i + j; ++t)
            {
                double v = 0.0;
                if (t <= pi + pj)
                    v += X * A.E[pi][pj][t];
                if (t >= 1)
                    v += h * A.E[pi][pj][t - 1];
                if (t + 1 <= pi + pj)
                    v += (t + 1) * A.E[pi][pj][t + 1];
                A.E[i][j][t] = v;
            }
        }
}

void boys_host(int L, double T, double* F) { host_boys_eval(L, T, F); }
} // namespace
} // namespace hfg

extern "C" int hfg_gradient_one_electron(const hfg_basis* b, const int* shell_atom, int natom, const int* Z,
                                         const double* xyz, const double* D, const double* W, double* grad)
{
    using namespace hfg;
    if (!b || !shell_atom || !Z || !xyz || !D || !W || !grad || natom <= 0)
        return HFG_ERR_INVALID;
    const int ns = b->nshells;
    const size_t N = static_cast<size_t>(b->nao);
    // Nuclear repulsion.
    for (int i = 0; i < natom; ++i)
        for (int j = 0; j < natom; ++j)
        {
            if (i == j)
                continue;
            double d[3], r2 = 0.0;
            for (int k = 0; k < 3; ++k)
            {
                d[k] = xyz[3 * i + k] - xyz[3 * j + k];
                r2 += d[k] * d[k];
            }
            const double f = static_cast<double>(Z[i] * Z[j]) / (r2 * std::sqrt(r2));
            for (int k = 0; k < 3; ++k) grad[3 * i + k] -= f * d[k];
        }
    std::vector<double> gsum(static_cast<size_t>(3) * natom, 0.0);
#pragma omp parallel
    {
        std::vector<double> g(static_cast<size_t>(3) * natom, 0.0);
        constexpr int kS = 2 * kMaxL + 3;           // cube side for Lt + 1 <= 2 l_max + 2
        std::vector<double> lev(static_cast<size_t>(kS) * kS * kS * kS);
#pragma omp for schedule(dynamic, 4)
        for (long long k = 0; k < static_cast<long long>(ns) * ns; ++k)
        {
            const int sa = static_cast<int>(k / ns), sb = static_cast<int>(k % ns);
            if (sb < sa)
                continue; // (sb, sa) contributes the same as (sa, sb): factor 2 below
            const double pair_w = (sa == sb) ? 1.0 : 2.0;
            const int la = b->l[sa], lb = b->l[sb], na = ncart(la), nb = ncart(lb);
            const int atA = shell_atom[sa], atB = shell_atom[sb];
            const double* A = b->centers + 3 * sa;
            const double* B = b->centers + 3 * sb;
            const double AB2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
            const int Lt = la + lb + 1; // R needed up to la + lb + 1
            for (int pa = 0; pa < b->nprim_sh[sa]; ++pa)
                for (int pb = 0; pb < b->nprim_sh[sb]; ++pb)
                {
                    const double aa = b->alpha[b->prim_off[sa] + pa], bb = b->alpha[b->prim_off[sb] + pb];
                    const double p = aa + bb, ip = 1.0 / p;
                    double P[3], PA[3], PB[3];
                    for (int x = 0; x < 3; ++x)
                    {
                        P[x]  = (aa * A[x] + bb * B[x]) * ip;
                        PA[x] = P[x] - A[x];
                        PB[x] = P[x] - B[x];
                    }
                    const double K = std::exp(-aa * bb * ip * AB2);
                    // K below 1e-30 contributes nothing representable (the derivative adds at most a factor
                    // 2a to the bound of the one-electron integrals, which skip at the same K).
                    if (K < 1e-30)
                        continue;
                    Axis E[3];
                    for (int x = 0; x < 3; ++x) hermite_axis_g(la + 1, lb + 2, p, PA[x], PB[x], E[x]);
                    const double cprod = b->coeff[b->prim_off[sa] + pa] * b->coeff[b->prim_off[sb] + pb];
                    const double prefS = std::pow(M_PI * ip, 1.5) * K;
                    const double prefV = 2.0 * M_PI * ip * K;
                    auto e3 = [&](const int* i, const int* j, int t, int u, int v) {
                        if (i[0] < 0 || i[1] < 0 || i[2] < 0 || j[0] < 0 || j[1] < 0 || j[2] < 0)
                            return 0.0;
                        if (t > i[0] + j[0] || u > i[1] + j[1] || v > i[2] + j[2])
                            return 0.0;
                        return E[0].E[i[0]][j[0]][t] * E[1].E[i[1]][j[1]][u] * E[2].E[i[2]][j[2]][v];
                    };
                    auto ovl = [&](const int* i, const int* j) { return prefS * e3(i, j, 0, 0, 0); };
                    auto kin = [&](const int* i, const int* j) {
                        if (i[0] < 0 || i[1] < 0 || i[2] < 0 || j[0] < 0 || j[1] < 0 || j[2] < 0)
                            return 0.0;
                        const double s0 = ovl(i, j);
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
                        return bb * (2 * (j[0] + j[1] + j[2]) + 3) * s0 - 2.0 * bb * bb * t2 + 0.5 * t3;
                    };
                    // Hermite-space densities: ED[tuv] = sum_ij wD_ij E^{ij}_tuv, and the centre-derivative
                    // versions DA[x][tuv], DB[x][tuv] (2a E^{i+1_x,j} - i_x E^{i-1_x,j}, likewise for j).
                    double ED[kS * kS * kS] = {}, DA[3][kS * kS * kS] = {}, DB[3][kS * kS * kS] = {};
                    for (int ci = 0; ci < na; ++ci)
                    {
                        const int i0[3] = {cart_exp(la, ci, 0), cart_exp(la, ci, 1), cart_exp(la, ci, 2)};
                        const size_t mu = static_cast<size_t>(b->ao_off[sa] + ci);
                        const double nA = b->norms[b->norm_off[sa] + pa * na + ci];
                        for (int cj = 0; cj < nb; ++cj)
                        {
                            const int j0[3] = {cart_exp(lb, cj, 0), cart_exp(lb, cj, 1), cart_exp(lb, cj, 2)};
                            const size_t nu = static_cast<size_t>(b->ao_off[sb] + cj);
                            const double w  = pair_w * b->norms[b->norm_off[sb] + pb * nb + cj] * nA * cprod;
                            const double wD = w * D[mu + nu * N], wW = w * W[mu + nu * N];
                            for (int x = 0; x < 3; ++x)
                            {
                                int ip1[3] = {i0[0], i0[1], i0[2]}, im1[3] = {i0[0], i0[1], i0[2]};
                                ip1[x] += 1;
                                im1[x] -= 1;
                                const double dS_A = 2 * aa * ovl(ip1, j0) - i0[x] * ovl(im1, j0);
                                const double dT_A = 2 * aa * kin(ip1, j0) - i0[x] * kin(im1, j0);
                                g[3 * atA + x] += wD * dT_A - wW * dS_A;
                                g[3 * atB + x] -= wD * dT_A - wW * dS_A;
                            }
                            if (wD == 0.0)
                                continue;
                            for (int t = 0; t <= Lt; ++t)
                                for (int u = 0; u <= Lt - t; ++u)
                                    for (int v = 0; v <= Lt - t - u; ++v)
                                    {
                                        const int h = (t * kS + u) * kS + v;
                                        ED[h] += wD * e3(i0, j0, t, u, v);
                                        for (int x = 0; x < 3; ++x)
                                        {
                                            int ip1[3] = {i0[0], i0[1], i0[2]}, im1[3] = {i0[0], i0[1], i0[2]};
                                            int jp1[3] = {j0[0], j0[1], j0[2]}, jm1[3] = {j0[0], j0[1], j0[2]};
                                            ip1[x] += 1;
                                            im1[x] -= 1;
                                            jp1[x] += 1;
                                            jm1[x] -= 1;
                                            DA[x][h] += wD * (2 * aa * e3(ip1, j0, t, u, v) - i0[x] * e3(im1, j0, t, u, v));
                                            DB[x][h] += wD * (2 * bb * e3(i0, jp1, t, u, v) - j0[x] * e3(i0, jm1, t, u, v));
                                        }
                                    }
                        }
                    }
                    // Per nucleus: R_tuv(p, P - C) up to Lt + 1 (the operator derivative raises t, u or v).
                    const int L2 = Lt + 1, S2 = L2 + 1;
                    auto at = [&](int t, int u, int v, int n) -> double& { return lev[((static_cast<size_t>(n) * S2 + t) * S2 + u) * S2 + v]; };
                    for (int c = 0; c < natom; ++c)
                    {
                        const double PC[3] = {P[0] - xyz[3 * c], P[1] - xyz[3 * c + 1], P[2] - xyz[3 * c + 2]};
                        double F[2 * kMaxL + 4];
                        boys_host(L2, p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]), F);
                        double f = 1.0;
                        for (int n = 0; n <= L2; ++n)
                        {
                            at(0, 0, 0, n) = f * F[n];
                            f *= -2.0 * p;
                        }
                        for (int n = L2 - 1; n >= 0; --n)
                            for (int d = 1; d <= L2 - n; ++d)
                                for (int v = 0; v <= d; ++v)
                                    for (int u = 0; u <= d - v; ++u)
                                    {
                                        const int t = d - u - v;
                                        double r;
                                        if (t > 0)
                                            r = PC[0] * at(t - 1, u, v, n + 1) + (t > 1 ? (t - 1) * at(t - 2, u, v, n + 1) : 0.0);
                                        else if (u > 0)
                                            r = PC[1] * at(t, u - 1, v, n + 1) + (u > 1 ? (u - 1) * at(t, u - 2, v, n + 1) : 0.0);
                                        else
                                            r = PC[2] * at(t, u, v - 1, n + 1) + (v > 1 ? (v - 1) * at(t, u, v - 2, n + 1) : 0.0);
                                        at(t, u, v, n) = r;
                                    }
                        const double zc = -Z[c] * prefV; // V_C = -Z_C (2 pi / p) K sum E R
                        double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
                        for (int t = 0; t <= Lt; ++t)
                            for (int u = 0; u <= Lt - t; ++u)
                                for (int v = 0; v <= Lt - t - u; ++v)
                                {
                                    const int h = (t * kS + u) * kS + v;
                                    const double r0 = at(t, u, v, 0);
                                    for (int x = 0; x < 3; ++x)
                                    {
                                        gA[x] += DA[x][h] * r0;
                                        gB[x] += DB[x][h] * r0;
                                    }
                                    // dR_tuv(P - C)/dC = -R_{tuv + 1_x}
                                    if (ED[h] != 0.0)
                                    {
                                        gC[0] -= ED[h] * at(t + 1, u, v, 0);
                                        gC[1] -= ED[h] * at(t, u + 1, v, 0);
                                        gC[2] -= ED[h] * at(t, u, v + 1, 0);
                                    }
                                }
                        for (int x = 0; x < 3; ++x)
                        {
                            g[3 * atA + x] += zc * gA[x];
                            g[3 * atB + x] += zc * gB[x];
                            g[3 * c + x] += zc * gC[x];
                        }
                    }
                }
        }
#pragma omp critical(hfg_grad_reduce)
        for (size_t q = 0; q < g.size(); ++q) gsum[q] += g[q];
    }
    for (size_t q = 0; q < gsum.size(); ++q) grad[q] += gsum[q];
    return HFG_OK;
}
