// Shared compile-time helpers for the direct-SCF Fock-build kernels.
//
// Conventions that follow the reference program (MalachiF1/Hartree-Fock):
//   * Cartesian components of a shell of angular momentum l are ordered with the x exponent
//     descending, then the y exponent descending (src/Basis.cpp:48-59):
//     p: x, y, z;  d: xx, xy, xz, yy, yz, zz.
//   * Matrices are column-major n x n FP64 (Eigen's default layout used throughout src/SCF.cpp).
//   * Hermite expansion of a Gaussian pair product (McMurchie-Davidson) as in
//     src/IntegralEngine.cpp:1025-1079; auxiliary integrals R^n_{tuv} as in :1082-1162.
#pragma once

#include <cstdint>
#include <type_traits>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace hfg
{
constexpr int kMaxL    = 2;                     // s, p, d shells
constexpr int kMaxLt   = 4 * kMaxL;             // total angular momentum of a shell quartet
constexpr int kNumPairClasses = (kMaxL + 1) * (kMaxL + 2) / 2;                  // (l1 >= l2)
constexpr int kNumQuartetClasses = kNumPairClasses * (kNumPairClasses + 1) / 2; // (bra >= ket)

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// Exponent of Cartesian component c (0-based, reference order) of angular momentum l along axis ax.
__host__ __device__ constexpr int cart_exp(int l, int c, int ax)
{
    int idx = 0;
    for (int i = l; i >= 0; --i)
        for (int j = l - i; j >= 0; --j)
        {
            if (idx == c)
                return ax == 0 ? i : (ax == 1 ? j : l - i - j);
            ++idx;
        }
    return 0;
}

// Pair class index of (l1, l2) with l1 >= l2: (0,0)=0, (1,0)=1, (1,1)=2, (2,0)=3, (2,1)=4, (2,2)=5.
__host__ __device__ constexpr int pair_class(int l1, int l2) { return l1 * (l1 + 1) / 2 + l2; }
__host__ __device__ constexpr int pair_class_l1(int pc)
{
    int l = 0;
    while ((l + 1) * (l + 2) / 2 <= pc) ++l;
    return l;
}
__host__ __device__ constexpr int pair_class_l2(int pc) { return pc - pair_class_l1(pc) * (pair_class_l1(pc) + 1) / 2; }
// Quartet class of (bra pair class >= ket pair class).
__host__ __device__ constexpr int quartet_class(int pb, int pk) { return pb * (pb + 1) / 2 + pk; }

// Hermite index (t,u,v), t+u+v <= L, laid out v-major, then u, then t.
__host__ __device__ constexpr int hidx(int t, int u, int v, int L)
{
    int idx = 0;
    for (int vv = 0; vv < v; ++vv)
    {
        const int m = L - vv;
        idx += (m + 1) * (m + 2) / 2;
    }
    const int m = L - v;
    for (int uu = 0; uu < u; ++uu) idx += (m - uu + 1);
    return idx + t;
}

// Inverse of hidx: component `ax` of the n-th Hermite triple for total L.
__host__ __device__ constexpr int htuv(int n, int L, int ax)
{
    for (int v = 0; v <= L; ++v)
        for (int u = 0; u <= L - v; ++u)
            for (int t = 0; t <= L - v - u; ++t)
                if (hidx(t, u, v, L) == n)
                    return ax == 0 ? t : (ax == 1 ? u : v);
    return 0;
}

// Full 3-D Hermite expansion table of a primitive pair (l1, l2): for each Cartesian component pair
// ij = i*ncart(l2)+j, the coefficients E^{ij}_{tuv} = Ex[ix,jx,t] Ey[iy,jy,u] Ez[iz,jz,v] for
// t <= ix+jx, u <= iy+jy, v <= iz+jz, stored contiguously (t fastest).
__host__ __device__ constexpr int e3_len(int l1, int l2, int ij, int ax)
{
    return cart_exp(l1, ij / ncart(l2), ax) + cart_exp(l2, ij % ncart(l2), ax) + 1;
}
__host__ __device__ constexpr int e3_size_of(int l1, int l2, int ij)
{
    return e3_len(l1, l2, ij, 0) * e3_len(l1, l2, ij, 1) * e3_len(l1, l2, ij, 2);
}
__host__ __device__ constexpr int e3_offset(int l1, int l2, int ij)
{
    int off = 0;
    for (int k = 0; k < ij; ++k) off += e3_size_of(l1, l2, k);
    return off;
}
__host__ __device__ constexpr int e3_total(int l1, int l2) { return e3_offset(l1, l2, ncart(l1) * ncart(l2)); }

// Per-primitive-pair record: [0] p, [1..3] P, [4] W = sqrt(2 pi^{5/2}) / p * exp(-ab/p |A-B|^2) * c_a c_b *
// radial normalisation of both primitives (so that W_ab W_cd / sqrt(p+q) is the whole primitive
// prefactor of an ERI), [5] 1/p, then e3_total(l1,l2) Hermite coefficients; padded to even.
constexpr int kPairHeader = 6;
__host__ __device__ constexpr int pp_stride(int l1, int l2)
{
    const int s = kPairHeader + e3_total(l1, l2);
    return s + (s & 1);
}

// Angular normalisation 1/sqrt((2i-1)!!(2j-1)!!(2k-1)!!) of a Cartesian component
// (the l-dependent factor of src/Basis.cpp:61-77).
__host__ __device__ constexpr int dfact_odd(int n) // (n)!! for odd n >= -1
{
    int r = 1;
    for (int k = n; k > 1; k -= 2) r *= k;
    return r;
}

// Compile-time loop: f(std::integral_constant<int, I>) for I in [B, E).
template <int B, int E, typename F> __host__ __device__ __forceinline__ void static_for(F&& f)
{
    if constexpr (B < E)
    {
        f(std::integral_constant<int, B> {});
        static_for<B + 1, E>(f);
    }
}

// Shell pair as seen by the kernels.  sh1 has l1 >= l2 (the pair is oriented that way).
struct PairRec
{
    int sh1, sh2;     // shell indices
    int ao1, ao2;     // first AO of each shell
    int pp_off;       // first primitive pair (index into the class's primitive-pair table)
    int npp;          // number of primitive pairs
    int mol;          // molecule (batch) index
    int same;         // 1 if sh1 == sh2
    int kslot, kstep; // field-major tables: primitive pair i at slot kslot + i * kstep
};

struct Quartet
{
    uint32_t bra, ket; // indices into a pair array (the sorted one for built lists); bra's class >= ket's class
};
} // namespace hfg
