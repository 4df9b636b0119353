// One-electron integrals S, T, V on the host in FP64 (McMurchie-Davidson), OpenMP over shell pairs.
//
// Reference counterparts: IntegralEngine::overlap / kinetic / nuclearAttraction and the *Matrix
// drivers (src/IntegralEngine.cpp:78-368).  The same formulas: Hermite expansion of the pair product,
// S = (pi/p)^{3/2} K E^x_0 E^y_0 E^z_0, the kinetic integral through overlaps with the ket exponent
// shifted by +-2 per axis, and V = -(2 pi/p) K sum_C Z_C sum_tuv E_t E_u E_v R_tuv(p, P-C).  Normalisation
// factors are applied per primitive and component as the reference does.  These stay FP64.
#include "hfgpu.h"
#include "hfg_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace hfg
{
namespace
{
// Host Boys function: nearest-point Taylor expansion (7 terms) on a 0.05 grid, downward recursion,
// asymptotic form above T = 30 -- the same scheme as the device kernels (boys.cuh).
struct HostBoys
{
    static constexpr double kStep = 0.05;
    static constexpr int kTerms = 7, kOrders = 2 * kMaxL + 3 + kTerms, kPoints = 602; // L <= 2 l_max + 2
    std::vector<double> g; // [point][order], orders 0..kOrders-1
    HostBoys() : g(static_cast<size_t>(kPoints) * kOrders)
    {
        for (int i = 0; i < kPoints; ++i)
        {
            const long double T = i * static_cast<long double>(kStep);
            for (int m = 0; m < kOrders; ++m)
            {
                long double term = 1.0L / (m + 0.5L), sum = term;
                for (int k = 1; k < 2000; ++k)
                {
                    term *= T / (m + k + 0.5L);
                    const long double s2 = sum + term;
                    if (s2 == sum)
                        break;
                    sum = s2;
                }
                g[static_cast<size_t>(i) * kOrders + m] = static_cast<double>(sum * std::exp(-T) / 2.0L);
            }
        }
    }
    void eval(int L, double T, double* F) const
    {
        if (T > 30.0)
        {
            F[0] = 0.88622692545275801365 / std::sqrt(T);
            for (int m = 0; m < L; ++m) F[m + 1] = (m + 0.5) * F[m] / T;
            return;
        }
        const int pt = std::min(kPoints - 1, std::max(0, static_cast<int>(T / kStep + 0.5)));
        const double x = pt * kStep - T;
        const double* row = &g[static_cast<size_t>(pt) * kOrders];
        double f = 0.0, xk = 1.0, kf = 1.0;
        for (int k = 0; k < kTerms; ++k)
        {
            if (k > 0)
            {
                xk *= x;
                kf *= k;
            }
            f += row[L + k] * xk / kf;
        }
        F[L] = f;
        const double e = std::exp(-T);
        for (int m = L; m >= 1; --m) F[m - 1] = (2.0 * T * F[m] + e) / (2 * m - 1);
    }
};

const HostBoys& host_boys()
{
    static const HostBoys b;
    return b;
}
} // namespace

// F_0..F_L(T) on the host, L <= 2 l_max + 2 (used by the gradient code as well).
void host_boys_eval(int L, double T, double* F) { host_boys().eval(L, T, F); }

namespace
{

constexpr int kE1 = kMaxL + 3; // ket exponent range up to l + 2 for the kinetic integral

void hermite_axis(int l1, int l2, double p, double PA, double PB, double E[kMaxL + 1][kE1][2 * kMaxL + 4])
{
    std::memset(E, 0, sizeof(double) * (kMaxL + 1) * kE1 * (2 * kMaxL + 4));
    const double h = 0.5 / p;
    E[0][0][0]     = 1.0;
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
                    v += X * E[pi][pj][t];
                if (t >= 1)
                    v += h * E[pi][pj][t - 1];
                if (t + 1 <= pi + pj)
                    v += (t + 1) * E[pi][pj][t + 1];
                E[i][j][t] = v;
            }
        }
}
} // namespace
} // namespace hfg

extern "C" int hfg_one_electron(const hfg_basis* b, int natom, const int* Z, const double* xyz, double* S, double* T,
                                double* V)
{
    using namespace hfg;
    if (!b || !S || !T || !V || (natom > 0 && (!Z || !xyz)) || b->nshells <= 0)
        return HFG_ERR_INVALID;
    for (int s = 0; s < b->nshells; ++s)
        if (b->l[s] < 0 || b->l[s] > kMaxL)
            return HFG_ERR_UNSUPPORTED;
    const int ns = b->nshells;
    const size_t N = static_cast<size_t>(b->nao);
    std::memset(S, 0, sizeof(double) * N * N);
    std::memset(T, 0, sizeof(double) * N * N);
    std::memset(V, 0, sizeof(double) * N * N);
    const HostBoys& boys = host_boys();
    std::vector<std::pair<int, int>> sp;
    for (int a = 0; a < ns; ++a)
        for (int c = a; c < ns; ++c) sp.emplace_back(a, c);

#pragma omp parallel for schedule(dynamic, 8)
    for (long long k = 0; k < static_cast<long long>(sp.size()); ++k)
    {
        const int sa = sp[k].first, sb = sp[k].second;
        const int la = b->l[sa], lb = b->l[sb], na = ncart(la), nb = ncart(lb);
        const double* A = b->centers + 3 * sa;
        const double* B = b->centers + 3 * sb;
        const double AB2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
        double s_blk[36] = {}, t_blk[36] = {}, v_blk[36] = {};
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
                // A primitive pair with K = exp(-ab/p |A-B|^2) below 1e-30 adds nothing representable to
                // any S, T or V element: the remaining factors (contraction and normalisation, kinetic
                // exponent powers, nuclear charges times Boys values) stay far below 1e16 for the s, p, d
                // shells of the supported basis sets.
                if (K < 1e-30)
                    continue;
                double E[3][kMaxL + 1][kE1][2 * kMaxL + 4];
                for (int x = 0; x < 3; ++x) hermite_axis(la, lb + 2, p, PA[x], PB[x], E[x]);
                const double cprod = b->coeff[b->prim_off[sa] + pa] * b->coeff[b->prim_off[sb] + pb];
                const double prefS = std::pow(M_PI * ip, 1.5) * K;
                const double prefV = 2.0 * M_PI * ip * K;
                // Nuclear attraction: sum_C Z_C R_tuv(p, P - C), accumulated over nuclei once per
                // primitive pair (the E coefficients do not depend on the nucleus).
                const int Lt = la + lb, S1 = Lt + 1;
                double Rsum[(2 * kMaxL + 1) * (2 * kMaxL + 1) * (2 * kMaxL + 1)] = {};
                double Rl[(2 * kMaxL + 1) * (2 * kMaxL + 1) * (2 * kMaxL + 1) * (2 * kMaxL + 1)];
                auto at = [&](int t, int u, int v, int n) -> double& { return Rl[((n * S1 + v) * S1 + u) * S1 + t]; };
                for (int c = 0; c < natom; ++c)
                {
                    const double PC[3] = {P[0] - xyz[3 * c], P[1] - xyz[3 * c + 1], P[2] - xyz[3 * c + 2]};
                    double F[2 * kMaxL + 1];
                    boys.eval(Lt, p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]), F);
                    double f = 1.0;
                    for (int n = 0; n <= Lt; ++n)
                    {
                        at(0, 0, 0, n) = f * F[n];
                        f *= -2.0 * p;
                    }
                    for (int n = Lt - 1; n >= 0; --n)
                        for (int d = 1; d <= Lt - n; ++d)
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
                    for (int v = 0; v <= Lt; ++v)
                        for (int u = 0; u <= Lt - v; ++u)
                            for (int t = 0; t <= Lt - u - v; ++t) Rsum[(v * S1 + u) * S1 + t] += Z[c] * at(t, u, v, 0);
                }
                for (int i = 0; i < na; ++i)
                {
                    const int ix = cart_exp(la, i, 0), iy = cart_exp(la, i, 1), iz = cart_exp(la, i, 2);
                    const double nA = b->norms[b->norm_off[sa] + pa * na + i];
                    for (int j = 0; j < nb; ++j)
                    {
                        const int jx = cart_exp(lb, j, 0), jy = cart_exp(lb, j, 1), jz = cart_exp(lb, j, 2);
                        const double nB = b->norms[b->norm_off[sb] + pb * nb + j];
                        const double w  = nA * nB * cprod;
                        const double ex = E[0][ix][jx][0], ey = E[1][iy][jy][0], ez = E[2][iz][jz][0];
                        s_blk[i * nb + j] += w * prefS * ex * ey * ez;
                        const double t1 = bb * (2 * (jx + jy + jz) + 3) * ex * ey * ez;
                        const double t2 = -2.0 * bb * bb *
                                          (E[0][ix][jx + 2][0] * ey * ez + ex * E[1][iy][jy + 2][0] * ez + ex * ey * E[2][iz][jz + 2][0]);
                        double t3 = 0.0;
                        if (jx >= 2)
                            t3 -= jx * (jx - 1) * E[0][ix][jx - 2][0] * ey * ez;
                        if (jy >= 2)
                            t3 -= jy * (jy - 1) * ex * E[1][iy][jy - 2][0] * ez;
                        if (jz >= 2)
                            t3 -= jz * (jz - 1) * ex * ey * E[2][iz][jz - 2][0];
                        t_blk[i * nb + j] += w * prefS * (t1 + t2 + 0.5 * t3);
                        double vs = 0.0;
                        for (int vv = 0; vv <= iz + jz; ++vv)
                            for (int u = 0; u <= iy + jy; ++u)
                                for (int t = 0; t <= ix + jx; ++t)
                                    vs += E[0][ix][jx][t] * E[1][iy][jy][u] * E[2][iz][jz][vv] * Rsum[(vv * S1 + u) * S1 + t];
                        v_blk[i * nb + j] -= w * prefV * vs;
                    }
                }
            }
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j)
            {
                const size_t r = static_cast<size_t>(b->ao_off[sa] + i), c = static_cast<size_t>(b->ao_off[sb] + j);
                S[r + c * N] = s_blk[i * nb + j];
                T[r + c * N] = t_blk[i * nb + j];
                V[r + c * N] = v_blk[i * nb + j];
                S[c + r * N] = s_blk[i * nb + j];
                T[c + r * N] = t_blk[i * nb + j];
                V[c + r * N] = v_blk[i * nb + j];
            }
    }
    return HFG_OK;
}
