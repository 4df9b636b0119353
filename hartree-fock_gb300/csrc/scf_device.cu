// Device-side pieces of the SCF iteration that the reference does on the host, so that one whole
// iteration (Fock build, DIIS, orbital step, energy and convergence measures) can be captured in a CUDA
// graph and replayed with a single host read-back per iteration.
//
//   DIIS::update                  src/DIIS.cpp:12-26   ring of at most DIIS_SIZE (F_alpha, F_beta, e) entries
//   DIIS::extrapolate             src/DIIS.cpp:28-72   bordered B c = (0, .., 0, -1), F = sum c_i F_i
//   SCF energy / convergence      src/SCF.cpp:81-91, 833-834
//
// The DIIS history lives in a ring of `cap` fixed slots (logical entry i, oldest first, in slot
// (head + i) % cap); B is kept per slot pair and only the newest row is recomputed.  The bordered system
// is solved by one thread with Gaussian elimination and complete pivoting in logical order, the same
// arithmetic as the host path.  Every reduction is two-pass with a fixed order, so replays are
// deterministic.
#include "scf_device.h"

#include <cmath>

namespace hfg
{
namespace
{
constexpr int kRedThreads = 256;

// Partial sums of x . y over blocks of the vector: part[blockIdx.y * gridDim.x + blockIdx.x], for up to
// gridDim.y vector pairs (x of pair k at xs[k], y at ys[k]).
__global__ void dot_partial_kernel(const double* const* __restrict__ xs, const double* const* __restrict__ ys, long long n,
                                   double* __restrict__ part)
{
    __shared__ double red[kRedThreads / 32];
    const double* x = xs[blockIdx.y];
    const double* y = ys[blockIdx.y];
    double s        = 0.0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        s = fma(x[i], y[i], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int w = 0; w < kRedThreads / 32; ++w) t += red[w];
        part[blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
}

// The B row of the newest DIIS slot from the partial dots of e_new with every slot.
__global__ void diis_brow_kernel(const double* __restrict__ part, int nblk, DiisState* st, double* __restrict__ B)
{
    const int k = threadIdx.x;
    const int cap = st->cap, nw = st->newest;
    if (k < cap)
    {
        double t = 0.0;
        for (int b = 0; b < nblk; ++b) t += part[k * nblk + b];
        B[nw * cap + k] = t;
        B[k * cap + nw] = t;
    }
}

// Advances the ring: the slot the next entry goes to (the oldest one once the ring is full).
__global__ void diis_advance_kernel(DiisState* st)
{
    if (st->count < st->cap)
    {
        st->newest = (st->head + st->count) % st->cap;
        ++st->count;
    }
    else
    {
        st->newest = st->head;
        st->head   = (st->head + 1) % st->cap;
    }
}

// dst[newest] = src for `nv` vectors of length n (slot arrays dst_k of stride `cap` pointers).
__global__ void diis_store_kernel(const DiisState* __restrict__ st, DiisSlots sl, const double* __restrict__ Fa,
                                  const double* __restrict__ Fb, const double* __restrict__ e, long long n)
{
    const int s = st->newest;
    double* fa = sl.Fa[s];
    double* fb = sl.Fb[s];
    double* es = sl.e[s];
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        fa[i] = Fa[i];
        fb[i] = Fb[i];
        es[i] = e[i];
    }
}

// Bordered system in logical order, Gaussian elimination with complete pivoting (as the host solve),
// coefficients per slot into st->coef (0 for empty slots), ||e_newest|| into sc->diis_error.
__global__ void diis_solve_kernel(DiisState* st, const double* __restrict__ B, ScfScalars* sc)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    constexpr int M = kDiisMaxSize + 1;
    const int m = st->count, cap = st->cap, n = m + 1;
    double A[M * M], b[M], y[M], x[M];
    int perm[M];
    auto at = [&](int i, int j) -> double& { return A[i + j * n]; };
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) at(i, j) = B[((st->head + i) % cap) * cap + (st->head + j) % cap];
    for (int i = 0; i < m; ++i)
    {
        at(m, i) = -1.0;
        at(i, m) = -1.0;
        b[i]     = 0.0;
    }
    at(m, m) = 0.0;
    b[m]     = -1.0;
    for (int i = 0; i < n; ++i) perm[i] = i;
    int rank = n;
    for (int k = 0; k < n; ++k)
    {
        int pi = k, pj = k;
        double best = 0.0;
        for (int j = k; j < n; ++j)
            for (int i = k; i < n; ++i)
                if (fabs(at(i, j)) > best)
                {
                    best = fabs(at(i, j));
                    pi   = i;
                    pj   = j;
                }
        if (best == 0.0)
        {
            rank = k;
            break;
        }
        for (int j = 0; j < n; ++j)
        {
            const double t = at(k, j);
            at(k, j)       = at(pi, j);
            at(pi, j)      = t;
        }
        {
            const double t = b[k];
            b[k]           = b[pi];
            b[pi]          = t;
        }
        for (int i = 0; i < n; ++i)
        {
            const double t = at(i, k);
            at(i, k)       = at(i, pj);
            at(i, pj)      = t;
        }
        {
            const int t = perm[k];
            perm[k]     = perm[pj];
            perm[pj]    = t;
        }
        for (int i = k + 1; i < n; ++i)
        {
            const double f = at(i, k) / at(k, k);
            for (int j = k; j < n; ++j) at(i, j) -= f * at(k, j);
            b[i] -= f * b[k];
        }
    }
    for (int k = 0; k < n; ++k) y[k] = 0.0;
    for (int k = rank - 1; k >= 0; --k)
    {
        double s = b[k];
        for (int j = k + 1; j < rank; ++j) s -= at(k, j) * y[j];
        y[k] = s / at(k, k);
    }
    for (int k = 0; k < n; ++k) x[perm[k]] = y[k];
    for (int s = 0; s < cap; ++s) st->coef[s] = 0.0;
    for (int i = 0; i < m; ++i) st->coef[(st->head + i) % cap] = x[i];
    sc->diis_error = sqrt(fmax(B[st->newest * cap + st->newest], 0.0));
}

// F = sum over slots coef[s] F_s, for both spins (empty slots hold zeros and have coefficient 0).
__global__ void diis_extrapolate_kernel(const DiisState* __restrict__ st, DiisSlots sl, double* __restrict__ Fa,
                                        double* __restrict__ Fb, long long n)
{
    const int cap = st->cap;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        double a = 0.0, bb = 0.0;
        for (int s = 0; s < cap; ++s)
        {
            const double c = st->coef[s];
            a  = fma(c, sl.Fa[s][i], a);
            bb = fma(c, sl.Fb[s][i], bb);
        }
        Fa[i] = a;
        Fb[i] = bb;
    }
}

// Energy E = 1/2 <Da, h + Fa> + 1/2 <Db, h + Fb>, dE = |E - E_prev|, dD = ||Dt - Dt_prev||_F from the
// partial sums of the three reductions (pairs 0, 1: energy terms, pair 2: the density difference).
__global__ void scf_scalars_kernel(const double* __restrict__ part, int nblk, ScfScalars* sc)
{
    if (threadIdx.x != 0)
        return;
    double t[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k)
        for (int b = 0; b < nblk; ++b) t[k] += part[k * nblk + b];
    const double E = 0.5 * t[0] + 0.5 * t[1];
    sc->delta_e    = fabs(E - sc->energy);
    sc->energy     = E;
    sc->delta_d    = sqrt(fmax(t[2], 0.0));
}

// w = h + F (energy operand) and d = Dt - Dt_prev (density change), elementwise.
__global__ void energy_operands_kernel(const double* __restrict__ h, const double* __restrict__ Fa,
                                       const double* __restrict__ Fb, const double* __restrict__ Dt,
                                       const double* __restrict__ Dtp, double* __restrict__ wa, double* __restrict__ wb,
                                       double* __restrict__ dd, long long n)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        wa[i] = h[i] + Fa[i];
        wb[i] = h[i] + Fb[i];
        dd[i] = Dt[i] - Dtp[i];
    }
}

inline int blocks_for(long long n, int num_sms)
{
    long long b = (n + kRedThreads - 1) / kRedThreads;
    const long long cap = static_cast<long long>(num_sms) * 4;
    return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}
} // namespace

int dot_blocks(int num_sms) { return num_sms * 2; }

cudaError_t diis_push(const DiisDevice& d, const double* Fa, const double* Fb, const double* e, long long n,
                      cudaStream_t s)
{
    diis_advance_kernel<<<1, 1, 0, s>>>(d.state);
    diis_store_kernel<<<blocks_for(n, d.num_sms), kRedThreads, 0, s>>>(d.state, d.slots, Fa, Fb, e, n);
    // Dots of e (now also in the newest slot) with every slot: pair k = (e, e_k).
    dot_partial_kernel<<<dim3(d.nblk, d.cap), kRedThreads, 0, s>>>(d.xs_e, d.ys_slots, n, d.part);
    diis_brow_kernel<<<1, 32, 0, s>>>(d.part, d.nblk, d.state, d.B);
    return cudaGetLastError();
}

cudaError_t diis_extrapolate(const DiisDevice& d, double* Fa, double* Fb, ScfScalars* sc, long long n, cudaStream_t s)
{
    diis_solve_kernel<<<1, 1, 0, s>>>(d.state, d.B, sc);
    diis_extrapolate_kernel<<<blocks_for(n, d.num_sms), kRedThreads, 0, s>>>(d.state, d.slots, Fa, Fb, n);
    return cudaGetLastError();
}

cudaError_t scf_measures(const MeasureDevice& m, long long n, cudaStream_t s)
{
    energy_operands_kernel<<<blocks_for(n, m.num_sms), kRedThreads, 0, s>>>(m.h, m.Fa, m.Fb, m.Dt, m.Dtp, m.wa, m.wb,
                                                                            m.dd, n);
    dot_partial_kernel<<<dim3(m.nblk, 3), kRedThreads, 0, s>>>(m.xs, m.ys, n, m.part);
    scf_scalars_kernel<<<1, 32, 0, s>>>(m.part, m.nblk, m.sc);
    return cudaGetLastError();
}
} // namespace hfg
