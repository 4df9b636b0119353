/*
 * CPU oracle: a plain-C restatement of the reference program's direct-SCF two-electron path
 * (MalachiF1/Hartree-Fock).  TEST INFRASTRUCTURE ONLY -- the GPU product never links or calls it.
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark load it, as the checker.
 *
 * Every function follows one reference function, cited file:line (paths inside the reference tree):
 *
 *   orc_boys                 Boys::calculateBoys                src/Boys.cpp:14-71 (grid: 92-105, series: 74-89)
 *   pair_data                computePrimitivePairData           src/IntegralEngine.cpp:995-1022
 *   hermite_coeffs           computeHermiteCoeffs               src/IntegralEngine.cpp:1025-1079
 *   aux_integrals            computeAuxiliaryIntegrals          src/IntegralEngine.cpp:1082-1162
 *   orc_eri                  electronRepulsion (vector overload) src/IntegralEngine.cpp:731-992
 *   orc_schwartz             schwartzScreeningMatrix            src/IntegralEngine.cpp:695-728
 *   orc_fock_direct          SCF::buildFockMatrixDirect         src/SCF.cpp:523-744 (J/K part, no F_prev)
 *   orc_survivors            the screening predicates of        src/SCF.cpp:592-623
 *   orc_fock_direct_sample   the same build over a sample of bra shell pairs (CPU-baseline timing)
 *   orc_count_survivors      the number of quartets passing those predicates (to scale a sample)
 *   orc_one_electron         overlap/kinetic/nuclearAttraction  src/IntegralEngine.cpp:78-368
 *
 * The basis arrives as the structure of arrays that IntegralEngine builds (IntegralEngine.cpp:13-75):
 * per shell l, primitive count/offset, AO offset, norm-factor offset and centre; per primitive the
 * exponent and contraction coefficient; per primitive x AO the normalisation factor; per AO the
 * Cartesian exponents.  All arithmetic is FP64, as in the reference.  Angular momentum up to d (l<=2).
 *
 * Parity of this restatement is pinned against the reference itself, compiled from its own sources
 * (oracle/_ref, see oracle/Makefile.ref), and against golden fixtures generated from it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_L 2
#define ORC_MAX_LT (4 * ORC_MAX_L)            /* total L of a quartet */
#define ORC_MAX_NAO 6                          /* Cartesian d */
#define ORC_MAX_PRIM 16
#define ORC_EBUF ((ORC_MAX_L + 1) * (ORC_MAX_L + 1) * (2 * ORC_MAX_L + 2) / 2)
#define ORC_RDIM (ORC_MAX_LT + 1)

typedef struct
{
    int nshells, nao, nprim_total;
    const int* l;          /* [nshells] */
    const int* nprim;      /* [nshells] */
    const int* prim_off;   /* [nshells] */
    const int* ao_off;     /* [nshells] */
    const int* norm_off;   /* [nshells] */
    const double* centers; /* [nshells][3] */
    const double* alpha;   /* [nprim_total] */
    const double* coeff;   /* [nprim_total] */
    const double* norms;   /* [sum nprim*nao] */
    const int* am;         /* [nao][3] */
} orc_basis;

/* ------------------------------------------------------------------------------------------------
 * Boys function: Boys.hpp:5-9 (grid constants), Boys.cpp:14-105.
 * ----------------------------------------------------------------------------------------------*/
#define BOYS_STEP 5.0e-5
#define BOYS_GRID_MAX 30.0
#define BOYS_ORDERS 34 /* MAX_L + 2 */
#define BOYS_POINTS 600001
static const double SQRT_PI_BY_2 = 0.8862269254527579;
static const double TRANSITION_VALUES[83] = {
    0.00,  2.35,  2.35,  2.35,  2.35,  2.38,  2.82,  3.05,  3.72,  3.76,  4.01,  4.61,  4.92,  5.15,
    5.63,  6.02,  6.33,  6.83,  7.15,  7.43,  7.94,  8.27,  8.59,  8.88,  9.21,  9.84,  9.99,  10.40,
    10.71, 11.15, 11.54, 11.88, 12.37, 12.69, 13.21, 13.42, 13.81, 14.25, 14.65, 14.97, 15.31, 15.84,
    15.96, 16.22, 16.69, 17.15, 17.49, 17.92, 18.28, 18.61, 18.85, 19.18, 19.68, 19.94, 20.53, 20.73,
    21.25, 21.54, 21.89, 22.29, 22.72, 23.07, 23.44, 23.90, 24.17, 24.56, 24.85, 25.23, 25.63, 25.96,
    26.43, 26.78, 27.09, 27.56, 27.89, 28.27, 28.71, 29.00, 29.38, 29.84, 30.22, 30.56, 30.85};

static double* g_boys_grid = NULL;

/* Series of Boys.cpp:74-89: F_m(T) = exp(-T)/2 * sum_i T^i / ((m+1/2)(m+3/2)...(m+i+1/2)). */
double orc_boys_series(unsigned m, double T)
{
    double sum = 0.0, term = 1.0 / (m + 0.5);
    sum += term;
    for (int i = 1; i < 200; ++i)
    {
        term *= T / (m + i + 0.5);
        sum += term;
        if (fabs(term) < 1e-15)
            break;
    }
    return sum * exp(-T) / 2.0;
}

/* Grid of Boys.cpp:92-105 (the reference caches it on disk; here it is rebuilt in memory). */
static const double* boys_grid(void)
{
    if (g_boys_grid)
        return g_boys_grid;
#pragma omp critical(orc_boys_grid)
    {
        if (!g_boys_grid)
        {
            double* g = (double*)malloc(sizeof(double) * (size_t)(BOYS_POINTS + 1) * BOYS_ORDERS);
#pragma omp parallel for schedule(static)
            for (long i = 0; i <= BOYS_POINTS; ++i)
            {
                const double Ti = i * BOYS_STEP;
                for (int j = 0; j < BOYS_ORDERS; ++j) g[(size_t)i * BOYS_ORDERS + j] = orc_boys_series(j, Ti);
            }
            g_boys_grid = g;
        }
    }
    return g_boys_grid;
}

void orc_boys(unsigned m_max, double T, double* F)
{
    if (T > 30.0)
    {
        F[0]              = SQRT_PI_BY_2 / sqrt(T);
        const double invT = 1.0 / T;
        for (unsigned m = 0; m < m_max; ++m) F[m + 1] = (m + 0.5) * F[m] * invT;
        return;
    }
    const double* grid   = boys_grid();
    const size_t gi      = (size_t)(T / BOYS_STEP);
    const double dT      = T - gi * BOYS_STEP;
    const double half_d2 = 0.5 * dT * dT;
    if (m_max < 2)
    {
        const double* g = grid + gi * BOYS_ORDERS;
        F[0]            = g[0] - dT * g[1] + half_d2 * g[2];
        if (m_max == 1)
            F[1] = g[1] - dT * g[2] + half_d2 * g[3];
        return;
    }
    const double emt = exp(-T);
    if (T <= TRANSITION_VALUES[m_max])
    {
        const double* g = grid + gi * BOYS_ORDERS + m_max;
        F[m_max]        = g[0] - dT * g[1] + half_d2 * g[2];
        const double twoT = 2.0 * T;
        for (unsigned m = m_max; m >= 1; --m) F[m - 1] = (twoT * F[m] + emt) / (2 * (m - 1) + 1);
    }
    else
    {
        const double* g = grid + gi * BOYS_ORDERS;
        F[0]            = g[0] - dT * g[1] + half_d2 * g[2];
        const double inv2T = 1 / (2 * T);
        for (unsigned m = 0; m < m_max; ++m) F[m + 1] = ((2.0 * m + 1.0) * F[m] - emt) * inv2T;
    }
}

/* ------------------------------------------------------------------------------------------------
 * Primitive pair data, Hermite E and R recursion (IntegralEngine.cpp:995-1162, hpp:41-141).
 * ----------------------------------------------------------------------------------------------*/
typedef struct
{
    double p, K, P[3], PA[3], PB[3];
} pair_t;

static void pair_data(double a, const double* A, double b, const double* B, pair_t* out)
{
    const double p = a + b, oo_p = 1.0 / p;
    double AB2     = 0.0;
    for (int k = 0; k < 3; ++k)
    {
        out->P[k]  = (a * A[k] + b * B[k]) * oo_p;
        out->PA[k] = out->P[k] - A[k];
        out->PB[k] = out->P[k] - B[k];
        AB2 += (A[k] - B[k]) * (A[k] - B[k]);
    }
    out->p = p;
    out->K = exp(-a * b * oo_p * AB2);
}

/* Triangular E layout of IntegralEngine.hpp:68-99. */
static inline int e_index(int l2, int i, int j, int t)
{
    return i * (l2 + 1) * (i + l2 + 1) / 2 + (j * (i + 1)) + j * (j - 1) / 2 + t;
}

static void hermite_coeffs(int l1, int l2, double p, double PA, double PB, double* E)
{
    E[0]               = 1.0;
    const double oo_2p = 0.5 / p;
    for (int i = 1; i <= l1; ++i)
    {
        const double* Em = E + e_index(l2, i - 1, 0, 0);
        double* Ei       = E + e_index(l2, i, 0, 0);
        for (int t = i; t >= 0; --t)
        {
            double v = 0.0;
            if (t <= i - 1)
                v = PA * Em[t];
            if (t >= 1)
                v += oo_2p * Em[t - 1];
            if (t + 1 <= i - 1)
                v += (t + 1) * Em[t + 1];
            Ei[t] = v;
        }
    }
    for (int j = 1; j <= l2; ++j)
        for (int i = 0; i <= l1; ++i)
        {
            const double* Em = E + e_index(l2, i, j - 1, 0);
            double* Eij      = E + e_index(l2, i, j, 0);
            for (int t = i + j; t >= 0; --t)
            {
                double v = 0.0;
                if (t <= i + j - 1)
                    v = PB * Em[t];
                if (t >= 1)
                    v += oo_2p * Em[t - 1];
                if (t + 1 <= i + j - 1)
                    v += (t + 1) * Em[t + 1];
                Eij[t] = v;
            }
        }
}

/* Dense R layout of IntegralEngine.hpp:109-141: index t + u*S + v*S^2 + n*S^3 with S = L+1. */
static void aux_integrals(int L, double p, const double* PC, const double* F, double* R)
{
    const int su = L + 1, sv = su * su, sn = sv * su;
    double f = 1.0;
    for (int n = 0; n <= L; ++n)
    {
        R[n * sn] = f * F[n];
        f *= -2.0 * p;
    }
    for (int n = L - 1; n >= 0; --n)
    {
        const double* Rp = R + (n + 1) * sn;
        double* Rn       = R + n * sn;
        for (int t = 1; t <= L - n; ++t) Rn[t] = PC[0] * Rp[t - 1] + (t >= 2 ? (t - 1) * Rp[t - 2] : 0.0);
        for (int u = 1; u <= L - n; ++u)
            for (int t = 0; t <= L - n - u; ++t)
                Rn[t + u * su] = PC[1] * Rp[t + (u - 1) * su] + (u >= 2 ? (u - 1) * Rp[t + (u - 2) * su] : 0.0);
        for (int v = 1; v <= L - n; ++v)
            for (int u = 0; u <= L - n - v; ++u)
                for (int t = 0; t <= L - n - u - v; ++t)
                    Rn[t + u * su + v * sv] = PC[2] * Rp[t + u * su + (v - 1) * sv]
                                            + (v >= 2 ? (v - 1) * Rp[t + u * su + (v - 2) * sv] : 0.0);
    }
}

static inline int nao_of(int l) { return (l + 1) * (l + 2) / 2; }

/* ------------------------------------------------------------------------------------------------
 * Contracted shell quartet, row-major [a][b][c][d] (IntegralEngine.cpp:731-992).  Entries with j>i or
 * l>k (AO indices), and when a==c && b==d those with ij<kl, stay zero exactly as in the reference.
 * ----------------------------------------------------------------------------------------------*/
void orc_eri(const orc_basis* B, long sa, long sb, long sc, long sd, double* G)
{
    const int la = B->l[sa], lb = B->l[sb], lc = B->l[sc], ld = B->l[sd];
    const int na = nao_of(la), nb = nao_of(lb), nc = nao_of(lc), nd = nao_of(ld);
    const int npa = B->nprim[sa], npb = B->nprim[sb], npc = B->nprim[sc], npd = B->nprim[sd];
    const int L = la + lb + lc + ld;
    const int ncd = npc * npd;
    const int nG = na * nb * nc * nd;
    memset(G, 0, sizeof(double) * nG);

    pair_t cdp[ORC_MAX_PRIM * ORC_MAX_PRIM];
    double Ecd[ORC_MAX_PRIM * ORC_MAX_PRIM][3][ORC_EBUF];
    const double* C = B->centers + 3 * sc;
    const double* D = B->centers + 3 * sd;
    for (int pc = 0; pc < npc; ++pc)
        for (int pd = 0; pd < npd; ++pd)
        {
            const int idx = pc * npd + pd;
            pair_data(B->alpha[B->prim_off[sc] + pc], C, B->alpha[B->prim_off[sd] + pd], D, &cdp[idx]);
            for (int k = 0; k < 3; ++k) hermite_coeffs(lc, ld, cdp[idx].p, cdp[idx].PA[k], cdp[idx].PB[k], Ecd[idx][k]);
        }

    const double* A  = B->centers + 3 * sa;
    const double* Bc = B->centers + 3 * sb;
    const int ao_a = B->ao_off[sa], ao_b = B->ao_off[sb], ao_c = B->ao_off[sc], ao_d = B->ao_off[sd];
    const int same_pair = (sa == sc && sb == sd);
    double Eab[3][ORC_EBUF];
    double F[ORC_RDIM];
    double R[ORC_RDIM * ORC_RDIM * ORC_RDIM * ORC_RDIM];
    double prim[ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO];
    const int su = L + 1, sv = su * su;
    const double two_pi_25 = 2.0 * pow(M_PI, 2.5);

    for (int pa = 0; pa < npa; ++pa)
    {
        const double ca     = B->coeff[B->prim_off[sa] + pa];
        const double* normA = B->norms + B->norm_off[sa] + pa * na;
        for (int pb = 0; pb < npb; ++pb)
        {
            const double cb     = B->coeff[B->prim_off[sb] + pb];
            const double* normB = B->norms + B->norm_off[sb] + pb * nb;
            pair_t ab;
            pair_data(B->alpha[B->prim_off[sa] + pa], A, B->alpha[B->prim_off[sb] + pb], Bc, &ab);
            for (int k = 0; k < 3; ++k) hermite_coeffs(la, lb, ab.p, ab.PA[k], ab.PB[k], Eab[k]);

            for (int icd = 0; icd < ncd; ++icd)
            {
                const pair_t* cd = &cdp[icd];
                const int pc = icd / npd, pd = icd % npd;
                const double pref = (two_pi_25 / (ab.p * cd->p * sqrt(ab.p + cd->p))) * ab.K * cd->K;
                const double delta = (ab.p * cd->p) / (ab.p + cd->p);
                double PQ[3] = {ab.P[0] - cd->P[0], ab.P[1] - cd->P[1], ab.P[2] - cd->P[2]};
                const double T = delta * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
                orc_boys((unsigned)L, T, F);
                aux_integrals(L, delta, PQ, F, R);

                /* 6-deep Hermite sum per AO quartet (IntegralEngine.cpp:847-939). */
                for (int a = 0; a < na; ++a)
                {
                    const int i = ao_a + a;
                    const int* am1 = B->am + 3 * i;
                    for (int b = 0; b < nb; ++b)
                    {
                        const int j = ao_b + b;
                        if (j > i)
                            continue;
                        const int bigI = i * (i + 1) / 2 + j;
                        const int* am2 = B->am + 3 * j;
                        const double* Exab = Eab[0] + e_index(lb, am1[0], am2[0], 0);
                        const double* Eyab = Eab[1] + e_index(lb, am1[1], am2[1], 0);
                        const double* Ezab = Eab[2] + e_index(lb, am1[2], am2[2], 0);
                        for (int c = 0; c < nc; ++c)
                        {
                            const int k = ao_c + c;
                            const int* am3 = B->am + 3 * k;
                            for (int d = 0; d < nd; ++d)
                            {
                                const int l = ao_d + d;
                                if (l > k)
                                    continue;
                                const int bigK = k * (k + 1) / 2 + l;
                                if (same_pair && bigI < bigK)
                                    continue;
                                const int* am4 = B->am + 3 * l;
                                const double* Excd = Ecd[icd][0] + e_index(ld, am3[0], am4[0], 0);
                                const double* Eycd = Ecd[icd][1] + e_index(ld, am3[1], am4[1], 0);
                                const double* Ezcd = Ecd[icd][2] + e_index(ld, am3[2], am4[2], 0);
                                const int l12 = am1[0] + am2[0], l34 = am3[0] + am4[0];
                                const int m12 = am1[1] + am2[1], m34 = am3[1] + am4[1];
                                const int n12 = am1[2] + am2[2], n34 = am3[2] + am4[2];
                                double acc = 0.0;
                                for (int v1 = 0; v1 <= n12; ++v1)
                                {
                                    double sv2 = 0.0;
                                    for (int v2 = 0; v2 <= n34; ++v2)
                                    {
                                        double su1 = 0.0;
                                        for (int u1 = 0; u1 <= m12; ++u1)
                                        {
                                            double su2 = 0.0;
                                            for (int u2 = 0; u2 <= m34; ++u2)
                                            {
                                                const double* Ruv = R + (u1 + u2) * su + (v1 + v2) * sv;
                                                double st1 = 0.0;
                                                for (int t1 = 0; t1 <= l12; ++t1)
                                                {
                                                    double st2 = 0.0;
                                                    for (int t2 = 0; t2 <= l34; ++t2)
                                                    {
                                                        const double sgn = ((t2 + u2 + v2) & 1) ? -1.0 : 1.0;
                                                        st2 += sgn * Excd[t2] * Ruv[t1 + t2];
                                                    }
                                                    st1 += Exab[t1] * st2;
                                                }
                                                su2 += Eycd[u2] * st1;
                                            }
                                            su1 += Eyab[u1] * su2;
                                        }
                                        sv2 += Ezcd[v2] * su1;
                                    }
                                    acc += Ezab[v1] * sv2;
                                }
                                prim[((a * nb + b) * nc + c) * nd + d] = acc;
                            }
                        }
                    }
                }

                /* Contraction with coefficients and normalisation (IntegralEngine.cpp:941-988). */
                const double cc = B->coeff[B->prim_off[sc] + pc], cdd = B->coeff[B->prim_off[sd] + pd];
                const double* normC = B->norms + B->norm_off[sc] + pc * nc;
                const double* normD = B->norms + B->norm_off[sd] + pd * nd;
                const double cprod = ca * cb * cc * cdd;
                for (int a = 0; a < na; ++a)
                {
                    const int i = ao_a + a;
                    for (int b = 0; b < nb; ++b)
                    {
                        const int j = ao_b + b;
                        if (j > i)
                            continue;
                        const int bigI = i * (i + 1) / 2 + j;
                        for (int c = 0; c < nc; ++c)
                        {
                            const int k = ao_c + c;
                            for (int d = 0; d < nd; ++d)
                            {
                                const int l = ao_d + d;
                                if (l > k)
                                    continue;
                                if (same_pair && bigI < k * (k + 1) / 2 + l)
                                    continue;
                                const int idx = ((a * nb + b) * nc + c) * nd + d;
                                G[idx] += normA[a] * normB[b] * normC[c] * normD[d] * cprod * pref * prim[idx];
                            }
                        }
                    }
                }
            }
        }
    }
}

/* Q(a,b) = sqrt(max_ab (ab|ab)) over the diagonal of each shell pair (IntegralEngine.cpp:695-728). */
void orc_schwartz(const orc_basis* B, double* Q)
{
    const int ns = B->nshells;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < ns; ++i)
    {
        double G[ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO];
        for (int j = 0; j <= i; ++j)
        {
            const int ni = nao_of(B->l[i]), nj = nao_of(B->l[j]);
            orc_eri(B, i, j, i, j, G);
            double mx = 0.0;
            for (int a = 0; a < ni; ++a)
                for (int b = 0; b < nj; ++b)
                {
                    const double v = G[a * (nj * ni * nj + nj) + b * (ni * nj + 1)];
                    mx = v > mx ? v : mx;
                }
            Q[(size_t)j + (size_t)i * ns] = sqrt(mx);
            Q[(size_t)i + (size_t)j * ns] = sqrt(mx);
        }
    }
}

/* Shell-pair maxima of |dD| (SCF.cpp:544-575); M is nshells x nshells, symmetric. */
static void shell_max(const orc_basis* B, const double* dD, double* M)
{
    const int ns = B->nshells, n = B->nao;
    for (int s1 = 0; s1 < ns; ++s1)
        for (int s2 = 0; s2 <= s1; ++s2)
        {
            double mx = 0.0;
            for (int a = B->ao_off[s1]; a < B->ao_off[s1] + nao_of(B->l[s1]); ++a)
                for (int b = B->ao_off[s2]; b < B->ao_off[s2] + nao_of(B->l[s2]); ++b)
                {
                    const double v = fabs(dD[(size_t)a + (size_t)b * n]);
                    mx = v > mx ? v : mx;
                }
            M[(size_t)s1 + (size_t)s2 * ns] = mx;
            M[(size_t)s2 + (size_t)s1 * ns] = mx;
        }
}

static inline double max2(double a, double b) { return a > b ? a : b; }

/* The Schwartz and density predicates of SCF.cpp:602-623 for canonical (a>=b, c>=d, ab>=cd). */
static inline int quartet_survives(int ns, const double* Q, const double* Mt, const double* Ma, const double* Mb,
                                   long a, long b, long c, long d, double sthr, double dthr)
{
    if (Q[a + b * ns] * Q[c + d * ns] < sthr)
        return 0;
    double md = max2(max2(2 * Mt[a + b * ns], 2 * Mt[c + d * ns]),
                     max2(max2(Ma[a + c * ns], Ma[a + d * ns]), max2(Ma[b + c * ns], Ma[b + d * ns])));
    if (Mb)
        md = max2(md, max2(max2(Mb[a + c * ns], Mb[a + d * ns]), max2(Mb[b + c * ns], Mb[b + d * ns])));
    return md >= dthr;
}

/* Canonical surviving quartets (a,b,c,d) in the reference's loop order; returns the count and writes up
 * to `cap` of them into out[4*i..]. */
long orc_survivors(const orc_basis* B, const double* Q, const double* dDtot, const double* dDa, const double* dDb,
                   double sthr, double dthr, int* out, long cap)
{
    const int ns = B->nshells;
    double* Mt = (double*)malloc(sizeof(double) * ns * ns);
    double* Ma = (double*)malloc(sizeof(double) * ns * ns);
    double* Mb = dDb ? (double*)malloc(sizeof(double) * ns * ns) : NULL;
    shell_max(B, dDtot, Mt);
    shell_max(B, dDa, Ma);
    if (Mb)
        shell_max(B, dDb, Mb);
    long count = 0;
    for (long a = 0; a < ns; ++a)
        for (long b = 0; b <= a; ++b)
            for (long c = 0; c <= a; ++c)
                for (long d = 0; d <= c; ++d)
                {
                    if (a * (a + 1) / 2 + b < c * (c + 1) / 2 + d)
                        continue;
                    if (!quartet_survives(ns, Q, Mt, Ma, Mb, a, b, c, d, sthr, dthr))
                        continue;
                    if (out && count < cap)
                    {
                        out[4 * count + 0] = (int)a;
                        out[4 * count + 1] = (int)b;
                        out[4 * count + 2] = (int)c;
                        out[4 * count + 3] = (int)d;
                    }
                    ++count;
                }
    free(Mt);
    free(Ma);
    free(Mb);
    return count;
}

/* J[dD_tot], K_alpha[dD_alpha] (and K_beta[dD_beta] when dDb != NULL) as SCF::buildFockMatrixDirect
 * forms them (SCF.cpp:523-728): canonical shell-quartet loop with Schwartz and density screening,
 * the reference ERI block, the AO-level |eri| < schwartz_thr skip, the symmetry-factor digestion
 * into the upper triangle, then the upper triangle mirrored.  Matrices are column-major n x n.
 * Returns the number of surviving shell quartets. */
/* Digestion of one ERI block into thread-local J/K (SCF.cpp:637-711): each canonical AO quartet
 * (ij|kl), i>=j, k>=l, ij>=kl, adds its distinct permutations into the upper triangle (row <= column). */
static void digest_block(const orc_basis* B, long a, long b, long c, long d, const double* G, const double* dDtot,
                         const double* dDa, const double* dDb, double sthr, double* Jp, double* Kap, double* Kbp)
{
    const size_t N = (size_t)B->nao;
    const int na = nao_of(B->l[a]), nb = nao_of(B->l[b]), nc = nao_of(B->l[c]), nd = nao_of(B->l[d]);
    for (int A = 0; A < na; ++A)
    {
        const size_t i = A + B->ao_off[a];
        for (int Bq = 0; Bq < nb; ++Bq)
        {
            const size_t j = Bq + B->ao_off[b];
            if (j > i)
                continue;
            for (int C = 0; C < nc; ++C)
            {
                const size_t k = C + B->ao_off[c];
                const size_t lmax = (i == k) ? j : k;
                for (int Dq = 0; Dq < nd; ++Dq)
                {
                    const size_t l = Dq + B->ao_off[d];
                    if (l > lmax)
                        continue;
                    const double eri = G[((A * nb + Bq) * nc + C) * nd + Dq];
                    if (fabs(eri) < sthr)
                        continue;
                    const size_t ji = j + i * N, lk = l + k * N, li = l + i * N, kj = k + j * N;
                    const size_t lj = l + j * N, ki = k + i * N;
                    const double f_kl = (k == l) ? 1.0 : 2.0, f_ij = (i == j) ? 1.0 : 2.0;
                    Jp[ji] += f_kl * dDtot[lk] * eri;
                    Jp[lk] += ((l != j || k != i) ? 1.0 : 0.0) * f_ij * dDtot[ji] * eri;
                    const double f_jk = (j == k) ? 2.0 : 1.0;
                    const double f_jl = (j == l && i != k) ? 2.0 : 1.0;
                    const double f_ik = (i == k && j != l) ? 2.0 : 1.0;
                    const size_t x1 = i < k ? i + k * N : ki;
                    const size_t x2 = j < l ? j + l * N : lj;
                    const size_t x3 = j < k ? j + k * N : kj;
                    const double w1 = (x1 != li) ? f_ik : 0.0;
                    const double w2 = (x2 != li && x2 != x1) ? f_jl : 0.0;
                    const double w3 = (x3 != li && x3 != x1 && x3 != x2) ? f_jk : 0.0;
                    Kap[li] += dDa[kj] * eri;
                    Kap[x1] += w1 * dDa[lj] * eri;
                    Kap[x2] += w2 * dDa[ki] * eri;
                    Kap[x3] += w3 * dDa[li] * eri;
                    if (Kbp)
                    {
                        Kbp[li] += dDb[kj] * eri;
                        Kbp[x1] += w1 * dDb[lj] * eri;
                        Kbp[x2] += w2 * dDb[ki] * eri;
                        Kbp[x3] += w3 * dDb[li] * eri;
                    }
                }
            }
        }
    }
}

static void mirror_upper(size_t N, double* J, double* Ka, double* Kb)
{
    /* selfadjointView<Upper>: mirror the upper triangle (row <= column) into the lower one. */
    for (size_t c = 0; c < N; ++c)
        for (size_t r = c + 1; r < N; ++r)
        {
            J[r + c * N] = J[c + r * N];
            Ka[r + c * N] = Ka[c + r * N];
            if (Kb)
                Kb[r + c * N] = Kb[c + r * N];
        }
}

/* J[dD_tot], K_alpha[dD_alpha] (and K_beta[dD_beta] when dDb != NULL) as SCF::buildFockMatrixDirect
 * forms them (SCF.cpp:523-728): canonical shell-quartet loop (collapse(4), dynamic 32) with Schwartz and
 * density screening, the reference ERI block, the AO-level |eri| < schwartz_thr skip, the symmetry-factor
 * digestion into thread-local upper triangles, a critical-section reduction, then the upper triangle
 * mirrored.  Matrices are column-major n x n.  Returns the number of surviving shell quartets. */
long orc_fock_direct(const orc_basis* B, const double* Q, const double* dDtot, const double* dDa, const double* dDb,
                     double sthr, double dthr, double* J, double* Ka, double* Kb)
{
    const int ns = B->nshells;
    const size_t N = (size_t)B->nao;
    double* Mt = (double*)malloc(sizeof(double) * ns * ns);
    double* Ma = (double*)malloc(sizeof(double) * ns * ns);
    double* Mb = dDb ? (double*)malloc(sizeof(double) * ns * ns) : NULL;
    shell_max(B, dDtot, Mt);
    shell_max(B, dDa, Ma);
    if (Mb)
        shell_max(B, dDb, Mb);
    memset(J, 0, sizeof(double) * N * N);
    memset(Ka, 0, sizeof(double) * N * N);
    if (Kb)
        memset(Kb, 0, sizeof(double) * N * N);
    long survivors = 0;

#pragma omp parallel reduction(+ : survivors)
    {
        double* Jp  = (double*)calloc(N * N, sizeof(double));
        double* Kap = (double*)calloc(N * N, sizeof(double));
        double* Kbp = Kb ? (double*)calloc(N * N, sizeof(double)) : NULL;
        double G[ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO];
        const long ns4 = (long)ns * ns * ns * ns;
#pragma omp for schedule(dynamic, 32) nowait
        for (long q = 0; q < ns4; ++q)
        {
            const long a = q / ((long)ns * ns * ns), b = (q / ((long)ns * ns)) % ns, c = (q / ns) % ns, d = q % ns;
            if (b > a || d > c || a * (a + 1) / 2 + b < c * (c + 1) / 2 + d)
                continue;
            if (!quartet_survives(ns, Q, Mt, Ma, Mb, a, b, c, d, sthr, dthr))
                continue;
            ++survivors;
            orc_eri(B, a, b, c, d, G);
            digest_block(B, a, b, c, d, G, dDtot, dDa, dDb, sthr, Jp, Kap, Kbp);
        }
#pragma omp critical(orc_fock_reduce)
        {
            for (size_t x = 0; x < N * N; ++x)
            {
                J[x] += Jp[x];
                Ka[x] += Kap[x];
                if (Kb)
                    Kb[x] += Kbp[x];
            }
        }
        free(Jp);
        free(Kap);
        free(Kbp);
    }
    mirror_upper(N, J, Ka, Kb);
    free(Mt);
    free(Ma);
    free(Mb);
    return survivors;
}

/* The same build restricted to the ordered bra pairs (a, b) flagged in bra_mask[a * ns + b]: a bounded
 * sample of one build, used to time the CPU baseline on workloads whose full build takes too long on a
 * CPU.  For each sampled bra the whole ket range (c, d) in [0, ns)^2 is scanned with the skip tests of the
 * full build's nShells^4 loop (SCF.cpp:592-600), so that a sample of a fraction f of the ordered bra pairs
 * costs f of the full build, scan included.  Returns the surviving quartets evaluated. */
long orc_fock_direct_sample(const orc_basis* B, const double* Q, const double* dDtot, const double* dDa,
                            const double* dDb, double sthr, double dthr, const unsigned char* bra_mask, double* J,
                            double* Ka, double* Kb)
{
    const int ns = B->nshells;
    const size_t N = (size_t)B->nao;
    double* Mt = (double*)malloc(sizeof(double) * ns * ns);
    double* Ma = (double*)malloc(sizeof(double) * ns * ns);
    double* Mb = dDb ? (double*)malloc(sizeof(double) * ns * ns) : NULL;
    shell_max(B, dDtot, Mt);
    shell_max(B, dDa, Ma);
    if (Mb)
        shell_max(B, dDb, Mb);
    memset(J, 0, sizeof(double) * N * N);
    memset(Ka, 0, sizeof(double) * N * N);
    if (Kb)
        memset(Kb, 0, sizeof(double) * N * N);
    const long npairs = (long)ns * ns;
    long nsel = 0;
    for (long p = 0; p < npairs; ++p) nsel += bra_mask[p] ? 1 : 0;
    long* sel = (long*)malloc(sizeof(long) * (nsel > 0 ? nsel : 1));
    nsel = 0;
    for (long p = 0; p < npairs; ++p)
        if (bra_mask[p])
            sel[nsel++] = p;
    long survivors = 0;
#pragma omp parallel reduction(+ : survivors)
    {
        double* Jp  = (double*)calloc(N * N, sizeof(double));
        double* Kap = (double*)calloc(N * N, sizeof(double));
        double* Kbp = Kb ? (double*)calloc(N * N, sizeof(double)) : NULL;
        double G[ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO * ORC_MAX_NAO];
        /* The sampled bras' slices of the full build's flat index q = ((a ns + b) ns + c) ns + d, walked with
         * the same schedule and decoding as orc_fock_direct. */
        const long ns2 = (long)ns * ns, ns3 = ns2 * ns;
#pragma omp for schedule(dynamic, 32) nowait
        for (long t = 0; t < nsel * ns2; ++t)
        {
            const long q = sel[t / ns2] * ns2 + t % ns2;
            const long a = q / ns3, b = (q / ns2) % ns, c = (q / ns) % ns, d = q % ns;
            {
                if (b > a || d > c || a * (a + 1) / 2 + b < c * (c + 1) / 2 + d)
                    continue;
                if (!quartet_survives(ns, Q, Mt, Ma, Mb, a, b, c, d, sthr, dthr))
                    continue;
                ++survivors;
                orc_eri(B, a, b, c, d, G);
                digest_block(B, a, b, c, d, G, dDtot, dDa, dDb, sthr, Jp, Kap, Kbp);
            }
        }
#pragma omp critical(orc_fock_reduce_sample)
        {
            for (size_t x = 0; x < N * N; ++x)
            {
                J[x] += Jp[x];
                Ka[x] += Kap[x];
                if (Kb)
                    Kb[x] += Kbp[x];
            }
        }
        free(Jp);
        free(Kap);
        free(Kbp);
    }
    mirror_upper(N, J, Ka, Kb);
    free(sel);
    free(Mt);
    free(Ma);
    free(Mb);
    return survivors;
}


/* Number of canonical quartets surviving the predicates of SCF.cpp:602-623, without the O(nshells^4)
 * scan: pairs sorted by Q descending, for each bra pair only the ket pairs of the Schwartz prefix are
 * tested.  Used to scale a sampled CPU build to the full build. */
static const double* g_sortQ;
static int cmp_q_desc(const void* x, const void* y)
{
    const double a = g_sortQ[*(const long*)x], b = g_sortQ[*(const long*)y];
    return a > b ? -1 : (a < b ? 1 : 0);
}

long orc_count_survivors(const orc_basis* B, const double* Q, const double* dDtot, const double* dDa, const double* dDb,
                         double sthr, double dthr)
{
    const int ns = B->nshells;
    const long np = (long)ns * (ns + 1) / 2;
    long* ord = (long*)malloc(sizeof(long) * np);
    double* qp = (double*)malloc(sizeof(double) * np);
    int* pa = (int*)malloc(sizeof(int) * np);
    int* pb = (int*)malloc(sizeof(int) * np);
    long k = 0;
    for (int a = 0; a < ns; ++a)
        for (int b = 0; b <= a; ++b, ++k)
        {
            pa[k] = a;
            pb[k] = b;
            qp[k] = Q[a + (size_t)b * ns];
            ord[k] = k;
        }
    g_sortQ = qp;
    qsort(ord, (size_t)np, sizeof(long), cmp_q_desc);
    double* Mt = (double*)malloc(sizeof(double) * ns * ns);
    double* Ma = (double*)malloc(sizeof(double) * ns * ns);
    double* Mb = dDb ? (double*)malloc(sizeof(double) * ns * ns) : NULL;
    shell_max(B, dDtot, Mt);
    shell_max(B, dDa, Ma);
    if (Mb)
        shell_max(B, dDb, Mb);
    long total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (long i = 0; i < np; ++i)
    {
        const long pi = ord[i];
        for (long j = 0; j <= i; ++j)
        {
            const long pj = ord[j];
            if (qp[pi] * qp[pj] < sthr)
                break;
            /* canonical orientation is irrelevant for the predicate (it is symmetric) */
            if (quartet_survives(ns, Q, Mt, Ma, Mb, pa[pi], pb[pi], pa[pj], pb[pj], sthr, dthr))
                ++total;
        }
    }
    free(ord);
    free(qp);
    free(pa);
    free(pb);
    free(Mt);
    free(Ma);
    free(Mb);
    return total;
}

/* ------------------------------------------------------------------------------------------------
 * One-electron integrals S, T, V (IntegralEngine.cpp:78-368), used to check the host's FP64 S/T/V.
 * ----------------------------------------------------------------------------------------------*/
void orc_one_electron(const orc_basis* B, int natom, const int* Z, const double* xyz, double* S, double* T, double* V)
{
    const int ns = B->nshells;
    const size_t N = (size_t)B->nao;
    memset(S, 0, sizeof(double) * N * N);
    memset(T, 0, sizeof(double) * N * N);
    memset(V, 0, sizeof(double) * N * N);
#pragma omp parallel for schedule(dynamic, 1)
    for (int sa = 0; sa < ns; ++sa)
        for (int sb = sa; sb < ns; ++sb)
        {
            const int la = B->l[sa], lb = B->l[sb], na = nao_of(la), nb = nao_of(lb);
            const double* A = B->centers + 3 * sa;
            const double* Bc = B->centers + 3 * sb;
            for (int pa = 0; pa < B->nprim[sa]; ++pa)
                for (int pb = 0; pb < B->nprim[sb]; ++pb)
                {
                    const double aa = B->alpha[B->prim_off[sa] + pa], ab_ = B->alpha[B->prim_off[sb] + pb];
                    pair_t pr;
                    pair_data(aa, A, ab_, Bc, &pr);
                    /* E tables with l2+2 for the kinetic term (IntegralEngine.cpp:178-180). */
                    double Es[3][(ORC_MAX_L + 1) * (ORC_MAX_L + 3) * (2 * ORC_MAX_L + 4) / 2];
                    double Ev[3][ORC_EBUF];
                    for (int k = 0; k < 3; ++k)
                    {
                        hermite_coeffs(la, lb + 2, pr.p, pr.PA[k], pr.PB[k], Es[k]);
                        hermite_coeffs(la, lb, pr.p, pr.PA[k], pr.PB[k], Ev[k]);
                    }
                    const double cprod = B->coeff[B->prim_off[sa] + pa] * B->coeff[B->prim_off[sb] + pb];
                    const double prefS = pow(M_PI / pr.p, 1.5) * pr.K;
                    const double prefV = (2.0 * M_PI / pr.p) * pr.K;
                    const int lk = lb + 2;
                    for (int a = 0; a < na; ++a)
                    {
                        const int i = B->ao_off[sa] + a;
                        const int *m1 = B->am + 3 * i;
                        const double nA = B->norms[B->norm_off[sa] + pa * na + a];
                        for (int b = 0; b < nb; ++b)
                        {
                            const int j = B->ao_off[sb] + b;
                            const int *m2 = B->am + 3 * j;
                            const double nB = B->norms[B->norm_off[sb] + pb * nb + b];
                            const double w = nA * nB * cprod;
                            const double ex = Ev[0][e_index(lb, m1[0], m2[0], 0)];
                            const double ey = Ev[1][e_index(lb, m1[1], m2[1], 0)];
                            const double ez = Ev[2][e_index(lb, m1[2], m2[2], 0)];
                            S[(size_t)i + (size_t)j * N] += w * prefS * ex * ey * ez;
                            /* Kinetic (IntegralEngine.cpp:214-234) with the l2+2 tables. */
                            const double kx = Es[0][e_index(lk, m1[0], m2[0], 0)];
                            const double ky = Es[1][e_index(lk, m1[1], m2[1], 0)];
                            const double kz = Es[2][e_index(lk, m1[2], m2[2], 0)];
                            double t1 = ab_ * (2 * (m2[0] + m2[1] + m2[2]) + 3) * kx * ky * kz;
                            double t2 = -2.0 * ab_ * ab_
                                      * (Es[0][e_index(lk, m1[0], m2[0] + 2, 0)] * ky * kz
                                         + kx * Es[1][e_index(lk, m1[1], m2[1] + 2, 0)] * kz
                                         + kx * ky * Es[2][e_index(lk, m1[2], m2[2] + 2, 0)]);
                            double t3 = 0.0;
                            if (m2[0] >= 2)
                                t3 -= m2[0] * (m2[0] - 1) * Es[0][e_index(lk, m1[0], m2[0] - 2, 0)] * ky * kz;
                            if (m2[1] >= 2)
                                t3 -= m2[1] * (m2[1] - 1) * kx * Es[1][e_index(lk, m1[1], m2[1] - 2, 0)] * kz;
                            if (m2[2] >= 2)
                                t3 -= m2[2] * (m2[2] - 1) * kx * ky * Es[2][e_index(lk, m1[2], m2[2] - 2, 0)];
                            t3 *= 0.5;
                            T[(size_t)i + (size_t)j * N] += w * prefS * (t1 + t2 + t3);
                        }
                    }
                    /* Nuclear attraction (IntegralEngine.cpp:314-352). */
                    const int Lt = la + lb;
                    double F[2 * ORC_MAX_L + 1];
                    double R[(2 * ORC_MAX_L + 1) * (2 * ORC_MAX_L + 1) * (2 * ORC_MAX_L + 1) * (2 * ORC_MAX_L + 1)];
                    const int su = Lt + 1, sv = su * su;
                    for (int at = 0; at < natom; ++at)
                    {
                        double PC[3] = {pr.P[0] - xyz[3 * at], pr.P[1] - xyz[3 * at + 1], pr.P[2] - xyz[3 * at + 2]};
                        const double Tb = pr.p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
                        orc_boys((unsigned)Lt, Tb, F);
                        aux_integrals(Lt, pr.p, PC, F, R);
                        for (int a = 0; a < na; ++a)
                        {
                            const int i = B->ao_off[sa] + a;
                            const int *m1 = B->am + 3 * i;
                            const double nA = B->norms[B->norm_off[sa] + pa * na + a];
                            for (int b = 0; b < nb; ++b)
                            {
                                const int j = B->ao_off[sb] + b;
                                const int *m2 = B->am + 3 * j;
                                const double nB = B->norms[B->norm_off[sb] + pb * nb + b];
                                const double* Ex = Ev[0] + e_index(lb, m1[0], m2[0], 0);
                                const double* Ey = Ev[1] + e_index(lb, m1[1], m2[1], 0);
                                const double* Ez = Ev[2] + e_index(lb, m1[2], m2[2], 0);
                                double sum = 0.0;
                                for (int v = 0; v <= m1[2] + m2[2]; ++v)
                                {
                                    double su_ = 0.0;
                                    for (int u = 0; u <= m1[1] + m2[1]; ++u)
                                    {
                                        double st = 0.0;
                                        for (int t = 0; t <= m1[0] + m2[0]; ++t) st += Ex[t] * R[t + u * su + v * sv];
                                        su_ += Ey[u] * st;
                                    }
                                    sum += Ez[v] * su_;
                                }
                                V[(size_t)i + (size_t)j * N] -= nA * nB * cprod * prefV * Z[at] * sum;
                            }
                        }
                    }
                }
        }
    for (size_t c = 0; c < N; ++c)
        for (size_t r = c + 1; r < N; ++r)
        {
            S[r + c * N] = S[c + r * N];
            T[r + c * N] = T[c + r * N];
            V[r + c * N] = V[c + r * N];
        }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
