// hfgpu engine: basis packing, Schwartz screening, device quartet lists, class dispatch and the C ABI.
//
// Reference counterparts (MalachiF1/Hartree-Fock):
//   IntegralEngine::IntegralEngine          src/IntegralEngine.cpp:13-75    -> hfg_create / pack_molecules
//   computePrimitivePairData/HermiteCoeffs  src/IntegralEngine.cpp:995-1079 -> pack_molecules (once per engine)
//   schwartzScreeningMatrix                 src/IntegralEngine.cpp:695-728  -> compute_schwartz
//   SCF::buildFockMatrixDirect              src/SCF.cpp:523-744             -> fock_direct
//
// Device data layout (HBM):
//   pairs       PairRec per shell pair (a >= b within a molecule), oriented so l(sh1) >= l(sh2), by pair
//               id and, after the Schwartz sort, in sorted-list order (spairs; the lists hold those indices)
//   pptab64/32  per pair class, primitive-pair records of pp_stride(l1,l2) values (p, P, W, 1/p, E3),
//               renumbered in sorted order after the sort, and a field-major copy (ksoa) for the thread
//               kernels' ket reads; primitive pairs below the screening bound are left out
//   cls_*       per pair class, pair ids sorted by (molecule, primitive-pair count desc, Q desc), with
//               their Q values and the segments of equal primitive-pair count
//   lists       per quartet class and precision, the surviving quartets (bra, ket) as sorted indices
//   matrices    per molecule n x n column-major blocks, concatenated (dD, X, Y, J, K)
//
// Streams: `stream` carries a build; mixed builds run the FP32 class kernels on stream2 concurrently with
// the FP64 ones (fork after the list build, join before the symmetrisation).
#include "engine.h"
#include "eri_grad.cuh"
#include "hfgpu.h"
#include "onee.h"
#include "persistent.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace hfg
{
namespace
{
thread_local std::string g_create_error;

struct HfgError : std::runtime_error
{
    int code;
    HfgError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define HFG_CUDA(call)                                                                                               \
    do                                                                                                               \
    {                                                                                                                \
        cudaError_t e_ = (call);                                                                                     \
        if (e_ != cudaSuccess)                                                                                       \
            throw HfgError(e_ == cudaErrorMemoryAllocation ? HFG_ERR_NOMEM : HFG_ERR_CUDA,                           \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                                      \
    } while (0)

template <typename T> struct DevBuf
{
    T* p     = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count)
    {
        if (count <= n && p)
            return;
        release();
        if (count == 0)
            return;
        HFG_CUDA(cudaMalloc(&p, sizeof(T) * count));
        n = count;
    }
    void upload(const std::vector<T>& v, cudaStream_t s)
    {
        alloc(v.size());
        if (!v.empty())
            HFG_CUDA(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    }
};

struct MolInfo
{
    int nshells, nao;
    int sh_off;         // first global shell
    long long mat_off;  // offset of its n x n block
    long long smax_off; // offset of its nshells x nshells shell-max block
};

// Host-side basis of one molecule (copied from the caller).
struct HostBasis
{
    std::vector<int> l, nprim, prim_off, ao_off, norm_off, am;
    std::vector<double> centers, alpha, coeff, norms, radial; // radial: coeff-free radial norm per primitive
    hfg_basis view {};
};
} // namespace
} // namespace hfg

struct hfg_engine
{
    int device  = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] {};
    // Mixed builds: the FP32 class kernels run on stream2 concurrently with the FP64 ones on `stream`, so
    // that FP64-pipe bound and FP32/memory-latency bound kernels share the SMs (each grid may be limited
    // to `overlap_share` of the resident blocks per SM; full grids measured best: (H2O)_64 mixed build
    // 697 ms serial, 632 ms overlapped at share 1, 734 / 809 / 923 ms at 0.67 / 0.5 / 0.34).
    // ev2: fork, join, FP32 start, FP32 end.
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev2[4] {};
    bool overlap = true;
    float overlap_share = 1.0f;   // FP64 class kernels' grids
    float overlap_share32 = 1.0f; // FP32 class kernels' grids
    std::string last_error;

    int nmol = 0;
    std::vector<hfg::MolInfo> mols;
    std::vector<hfg::HostBasis> basis;
    long long mat_total  = 0; // sum n_m^2
    long long smax_total = 0; // sum nshells_m^2
    int nshells_total    = 0;

    std::vector<hfg::PairRec> pairs;
    std::vector<int> pair_class_of;
    hfg::DevBuf<hfg::PairRec> d_pairs;
    // The pairs in sorted-list order (class by class; position k of class pc at cls_base[pc] + k): the
    // quartet lists hold these indices, so the kets of a warp read neighbouring records.
    std::vector<int> cls_base, spair_id;
    hfg::DevBuf<hfg::PairRec> d_spairs;
    hfg::DevBuf<double> d_pptab64[hfg::kNumPairClasses];
    hfg::DevBuf<float> d_pptab32[hfg::kNumPairClasses];
    // Field-major copies of the same records (thread kernels' ket reads), field stride kfs[pc].
    hfg::DevBuf<double> d_ksoa64[hfg::kNumPairClasses];
    hfg::DevBuf<float> d_ksoa32[hfg::kNumPairClasses];
    long long kfs[hfg::kNumPairClasses] {};
    // Host records in pack order: pair k's primitives start at record orig_off[k] of h_tab[class].
    std::vector<double> h_tab[hfg::kNumPairClasses];
    std::vector<int> orig_off;
    // Primitive-pair screening: per record the Coulomb self-repulsion bound sqrt((ab|ab)) of that one
    // primitive pair; a primitive pair takes part in the Fock build iff bound * max_cd Q_cd >= prim_thr.
    // Pair k keeps the primitive pairs keep_idx[keep_off[k] .. keep_off[k+1]) of its npp_full[k].
    double prim_thr = 1e-15;
    std::vector<double> h_qp[hfg::kNumPairClasses];
    std::vector<int> npp_full, keep_off, keep_idx;
    // Unscreened records in pack order (the nuclear gradient's derivative integrals use every primitive).
    hfg::DevBuf<double> d_pptab64_full[hfg::kNumPairClasses];
    hfg::DevBuf<float> d_pptab32_full[hfg::kNumPairClasses];
    hfg::DevBuf<hfg::PairRec> d_gspairs; // sorted order, npp_full, pp_off = orig_off
    hfg::DevBuf<long long> d_mat_off;
    hfg::DevBuf<int> d_mat_ld;
    hfg::DevBuf<long long> d_smax_off; // per molecule offset of its shell-max block
    hfg::DevBuf<int> d_nsh;            // per molecule shell count
    hfg::DevBuf<int> d_shnao;          // per pair: Cartesian counts of sh1, sh2
    hfg::DevBuf<hfg::WarpTables> d_tables;
    hfg::DevBuf<double> d_boys64[hfg::kMaxLt + 2];
    hfg::DevBuf<float> d_boys32[hfg::kMaxLt + 2];
    hfg::DevBuf<double> d_gtab[hfg::kNumPairClasses]; // gradient records (built on first use)
    hfg::DevBuf<float> d_gtab32[hfg::kNumPairClasses]; // their FP32 copies (mixed-precision gradient)
    bool have_gtab = false;
    hfg::DevBuf<int> d_shell_atom;
    hfg::DevBuf<double> d_grad;
    // One-electron integrals on the device (molecule 0): the basis arrays, the shell pairs per pair class
    // (oriented l1 >= l2), the nuclei, and scratch for W.
    bool have_onee = false;
    hfg::DevBuf<int> d_ob_int;    // l, nprim, prim_off, ao_off, norm_off (nshells each)
    hfg::DevBuf<double> d_ob_dbl; // centers (3 nshells), alpha, coeff, norms
    hfg::DevBuf<int2> d_ob_pairs[hfg::kNumPairClasses];
    int ob_npairs[hfg::kNumPairClasses] {};
    hfg::OneeBasis ob {};
    hfg::DevBuf<double4> d_nuc;
    hfg::DevBuf<double> d_W;
    hfg::DevBuf<int> d_shell_atom1;
    // Final state of the last hfg_scf_run (for hfg_gradient's backward call).
    std::vector<double> scf_Da, scf_Db, scf_W;
    bool scf_valid = false, scf_uhf = false;

    // Schwartz bounds per pair, and per pair class sorted lists.
    std::vector<double> Qpair;
    bool have_Q = false;
    std::vector<int> cls_ids[hfg::kNumPairClasses];
    std::vector<double> cls_Q[hfg::kNumPairClasses];
    // Segments of equal primitive-pair count: x = begin, y = end (positions in the class list), z = npp.
    std::vector<int4> cls_seg[hfg::kNumPairClasses];
    std::vector<int2> cls_molseg[hfg::kNumPairClasses]; // per molecule: [first, end) segment
    hfg::DevBuf<int> d_cls_ids[hfg::kNumPairClasses];
    hfg::DevBuf<double> d_cls_Q[hfg::kNumPairClasses];
    hfg::DevBuf<float> d_cls_Qf[hfg::kNumPairClasses]; // FP32 copy for the precision split
    hfg::DevBuf<int4> d_cls_seg[hfg::kNumPairClasses];
    hfg::DevBuf<int2> d_cls_sh[hfg::kNumPairClasses]; // (sh1, sh2) of each sorted position
    hfg::DevBuf<int2> d_cls_molseg[hfg::kNumPairClasses];
    hfg::DevBuf<unsigned> d_bra_cnt[hfg::kNumQuartetClasses];            // per bra pair: survivors (fp64, fp32)
    hfg::DevBuf<unsigned long long> d_bra_off[hfg::kNumQuartetClasses];  // per bra pair: list offsets
    hfg::DevBuf<unsigned long long> d_scan_tmp;

    // Quartet lists (capacity for the Schwartz threshold they were sized for).
    double cap_thr = -1.0;
    unsigned long long cap[hfg::kNumQuartetClasses] {};
    bool cap_mixed = false;
    hfg::DevBuf<hfg::Quartet> d_list[hfg::kNumQuartetClasses][2];
    hfg::DevBuf<unsigned long long> d_counts; // [qclass][prec] quartets, then [qclass][prec] prim quartets, then overflow
    std::vector<unsigned long long> h_counts;

    // Work matrices.
    hfg::DevBuf<double> d_dD[3];   // tot, alpha, beta (FP64)
    hfg::DevBuf<float> d_dDf[3];   // FP32 copies for the FP32 kernels
    hfg::DevBuf<double> d_acc[3];  // X, Ya, Yb
    hfg::DevBuf<double> d_out[3];  // J, Ka, Kb
    hfg::DevBuf<double> d_smax[3]; // shell-pair maxima of |dD|
    hfg::DevBuf<double> d_smax2;   // 2 * shell maxima of |dD_tot|
    hfg::DevBuf<double> d_store;
    hfg::DevBuf<hfg::Quartet> d_tmp_list;
    // Stored integrals (hfg_store_integrals): per quartet class the Schwartz survivors (sorted pair
    // indices) and their FP64 integral blocks, row-major [ij][kl] per quartet.
    double conv_thr = -1.0;
    unsigned long long conv_n[hfg::kNumQuartetClasses] {};
    hfg::DevBuf<hfg::Quartet> d_conv_list[hfg::kNumQuartetClasses];
    hfg::DevBuf<double> d_conv[hfg::kNumQuartetClasses];
    hfg::DevBuf<unsigned long long> d_tmp_count;

    // Kernel forms: the caller's setting per (class, precision), and the pick per (class, precision, UHF).
    int form_set[hfg::kNumQuartetClasses][2] {};
    int form_pick[hfg::kNumQuartetClasses][2][2] {};
    hfg::DevBuf<hfg::Quartet> d_tune_list;
    hfg::DevBuf<unsigned long long> d_tune_cnt;
    hfg::DevBuf<double> d_tune_acc[3];
    cudaEvent_t tune_ev[2] {};

    // CUDA-graph replay of whole builds (hfg_set_graph_mode): the graph of the last device-pointer
    // request, valid while the request key matches and no buffer it uses has been reallocated.
    bool graph_mode = false;
    // Persistent work-queue launch of the small classes (hfg_set_persistent) and its item counter.
    bool persistent = false;
    hfg::DevBuf<unsigned long long> d_pcounter;
    // Gradient kernels: the lane-group form for every class (hfg_set_gradient_form).
    bool grad_group_only = false;
    // Kernel-form autotuning on first use of a class (hfg_set_autotune); off: default forms only.
    bool autotune = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    struct GraphKey
    {
        int precision = -1, uhf = 0;
        double sthr = 0, dthr = 0, cutoff = 0;
        const void* ptr[6] {};
        bool operator==(const GraphKey& o) const
        {
            return precision == o.precision && uhf == o.uhf && sthr == o.sthr && dthr == o.dthr && cutoff == o.cutoff &&
                   std::equal(ptr, ptr + 6, o.ptr);
        }
    } graph_key;
    int graph_launches = 0;
    int graph_forms[hfg::kNumQuartetClasses][2] {};
    unsigned long long* h_counts_pin = nullptr; // pinned copy of d_counts written by the graph

    bool last_valid = false;
    int last_mixed  = 0;
};

namespace hfg
{
namespace
{
// ------------------------------------------------------------------------------------------------
// Small kernels.
// ------------------------------------------------------------------------------------------------
__global__ void to_float_kernel(const double* __restrict__ a, float* __restrict__ b, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = static_cast<float>(a[i]);
}

// nch contiguous chunks of `chunk` entries, chunk c starting at entry c * (n / nch) of list[0, n)
// (chunk <= n / nch), and their total count.
__global__ void sample_list_kernel(const Quartet* __restrict__ list, unsigned long long n, unsigned long long nch,
                                   unsigned long long chunk, Quartet* __restrict__ out, unsigned long long* __restrict__ count)
{
    const unsigned long long m = nch * chunk, step = n / nch;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < m;
         i += (unsigned long long)gridDim.x * blockDim.x)
        out[i] = list[(i / chunk) * step + i % chunk];
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *count = m;
}

// Shell-pair maxima of |dD| (SCF.cpp:544-575) for every molecule block, with exact integer operations
// on the bit patterns (|x| clears the sign bit; non-negative doubles order like their bits).  M2, when
// given, receives 2*M (exact).
__global__ void shell_max_kernel(const double* __restrict__ dD, const PairRec* __restrict__ pairs, int npairs,
                                 const long long* __restrict__ mat_off, const int* __restrict__ mat_ld,
                                 const long long* __restrict__ smax_off, const int* __restrict__ nsh,
                                 const int* __restrict__ sh_nao, double* __restrict__ M, double* __restrict__ M2)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < npairs; k += gridDim.x * blockDim.x)
    {
        const PairRec pr = pairs[k];
        const long long off = mat_off[pr.mol];
        const int n = mat_ld[pr.mol], ns = nsh[pr.mol];
        const int n1 = sh_nao[k * 2], n2 = sh_nao[k * 2 + 1];
        long long mx = 0;
        for (int j = 0; j < n2; ++j)
            for (int i = 0; i < n1; ++i)
                mx = max(mx, __double_as_longlong(dD[off + (pr.ao1 + i) + (long long)(pr.ao2 + j) * n]) & 0x7fffffffffffffffLL);
        const double v = __longlong_as_double(mx);
        const long long e1 = smax_off[pr.mol] + pr.sh1 + (long long)pr.sh2 * ns;
        const long long e2 = smax_off[pr.mol] + pr.sh2 + (long long)pr.sh1 * ns;
        M[e1] = v;
        M[e2] = v;
        if (M2)
        {
            const double v2 = 2.0 * v;
            M2[e1] = v2;
            M2[e2] = v2;
        }
    }
}

// The non-negative finite double with bit pattern b as a float, by integer operations (truncating; below
// FP32's normal range 0, above it +inf).  Monotone in b, so it narrows a maximum taken on the bit patterns.
__device__ __forceinline__ float narrow_nonneg(long long b)
{
    const int e = static_cast<int>(b >> 52); // biased exponent (the sign bit is clear)
    if (e < 897)
        return 0.0f;
    if (e > 1150)
        return __int_as_float(0x7f800000);
    return __int_as_float(((e - 896) << 23) | static_cast<int>((b >> 29) & 0x7fffff));
}

struct BuildArgs
{
    const int* ids1;
    const double* Q1;
    int n1;
    int base1, base2; // sorted-array index of position 0 of each class (what the lists hold)
    const double* Q2;
    const int2* sh2;     // (sh1, sh2) per ket position
    const int4* seg2;    // ket class segments (equal primitive-pair count, Q descending inside)
    const int2* molseg2; // per molecule: ket segment range
    bool same_class;
    const PairRec* pairs;
    const double* Mt;
    const double* Mt2; // 2 * Mt
    const double* Ma;
    const double* Mb; // null for RHF
    const float* Qf1;
    const float* Qf2;
    const long long* smax_off;
    const int* nsh;
    double sthr, dthr;
    float cutoff;
    int mixed;
    int pass;                      // 0: count per bra pair, 1: write at the scanned offsets
    unsigned* bra_cnt;             // [n1][2]
    const unsigned long long* bra_off; // [n1][2] exclusive offsets (pass 1)
    Quartet* out64;
    Quartet* out32;
    unsigned long long* prim64;
    unsigned long long* prim32;
    unsigned long long cap; // list capacity (the Schwartz-only count): writes beyond it are dropped
};

// Survival list of one quartet class in two deterministic passes, one warp per bra pair.  Ket
// candidates are visited segment by segment (segments of equal primitive-pair count, Q descending
// inside each), and inside a segment only the Schwartz prefix Q_i*Q_j >= thr is tested (the product is
// monotone in Q_j); the density predicate is that of SCF.cpp:610-623.  Pass 0 counts survivors per
// bra pair and precision, pass 1 writes them at scanned offsets in candidate order, so the list is
// ordered by bra pair and, inside a bra pair, by ket primitive count: a warp of the class kernels sees
// quartets of equal primitive counts.  FP32 / FP64 split by the quartet bound Q_i Q_j max|dD|.
__global__ void build_lists_kernel(BuildArgs a)
{
    const int lane = threadIdx.x & 31;
    const int i    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.n1)
        return;
    const int pid_i  = a.ids1[i];
    const double Qi  = a.Q1[i];
    const PairRec pi = a.pairs[pid_i];
    const int2 ms    = a.molseg2[pi.mol];
    const long long so = a.smax_off[pi.mol];
    const int ns = a.nsh[pi.mol];
    // The shell-max matrices are symmetric: index them so that the ket shell (which varies across the
    // lanes) is the contiguous one.  Every value here is >= 0, and for non-negative doubles the order of
    // the IEEE bit patterns is the numeric order, so the maxima and the density test run as exact 64-bit
    // integer operations (GB300's FP64 pipe is 1/64 of its FP32 rate); the Schwartz product stays FP64.
    auto bits = [](const double* m, long long i) { return __double_as_longlong(m[i]); };
    const int sa = pi.sh1, sb = pi.sh2;
    const long long dab = bits(a.Mt2, so + sa + (long long)sb * ns);
    const long long dthr = __double_as_longlong(a.dthr);
    const long long ra = so + (long long)sa * ns, rb2 = so + (long long)sb * ns;
    const float Qfi = a.Qf1[i];
    unsigned c64 = 0, c32 = 0;
    unsigned long long p64 = 0, p32 = 0;
    const unsigned long long o64 = a.pass ? a.bra_off[2 * i] : 0ull;
    const unsigned long long o32 = a.pass ? a.bra_off[2 * i + 1] : 0ull;
    for (int sidx = ms.x; sidx < ms.y; ++sidx)
    {
        const int4 seg = a.seg2[sidx];
        const int jb = seg.x;
        const int je = a.same_class ? min(seg.y, i + 1) : seg.y;
        if (jb >= je)
            continue;
        int lo = jb, hi = je;
        while (lo < hi)
        {
            const int mid = (lo + hi) >> 1;
            if (Qi * a.Q2[mid] < a.sthr)
                hi = mid;
            else
                lo = mid + 1;
        }
        const int jend = lo;
        for (int base = jb; base < jend; base += 32)
        {
            const int j = base + lane;
            bool s64 = false, s32 = false;
            if (j < jend)
            {
                const int2 scd = a.sh2[j];
                const int sc = scd.x, sd = scd.y;
                long long md = max(dab, bits(a.Mt2, so + sc + (long long)sd * ns));
                md = max(md, max(max(bits(a.Ma, ra + sc), bits(a.Ma, ra + sd)), max(bits(a.Ma, rb2 + sc), bits(a.Ma, rb2 + sd))));
                if (a.Mb)
                    md = max(md, max(max(bits(a.Mb, ra + sc), bits(a.Mb, ra + sd)), max(bits(a.Mb, rb2 + sc), bits(a.Mb, rb2 + sd))));
                if (md >= dthr)
                {
                    bool lowp = false;
                    if (a.mixed) // the FP32/FP64 split is this engine's own heuristic: evaluated in FP32
                        lowp = Qfi * a.Qf2[j] * narrow_nonneg(md) < a.cutoff;
                    s32 = lowp;
                    s64 = !lowp;
                }
            }
            const unsigned m64 = __ballot_sync(0xffffffffu, s64);
            const unsigned m32 = __ballot_sync(0xffffffffu, s32);
            const unsigned lt  = (1u << lane) - 1u;
            if (a.pass)
            {
                const Quartet qv {static_cast<uint32_t>(a.base1 + i), static_cast<uint32_t>(a.base2 + j)};
                const unsigned long long w64 = o64 + c64 + __popc(m64 & lt), w32 = o32 + c32 + __popc(m32 & lt);
                if (s64 && w64 < a.cap)
                    a.out64[w64] = qv;
                if (s32 && w32 < a.cap)
                    a.out32[w32] = qv;
            }
            c64 += __popc(m64);
            c32 += __popc(m32);
            const unsigned long long pp = (unsigned long long)pi.npp * seg.z;
            p64 += pp * __popc(m64);
            p32 += pp * __popc(m32);
        }
    }
    if (a.pass == 0 && lane == 0)
    {
        a.bra_cnt[2 * i]     = c64;
        a.bra_cnt[2 * i + 1] = c32;
        if (p64)
            atomicAdd(a.prim64, p64);
        if (p32)
            atomicAdd(a.prim32, p32);
    }
}

// Exclusive scan of the per-bra counts (two interleaved sequences, fp64 and fp32) in three steps:
// per-block scan, scan of the block totals (one block), add the block offsets.  The grand totals land
// in total[0..1] (the class kernels' list lengths).
constexpr int kScanBlock = 1024;
__global__ void scan_block_kernel(const unsigned* __restrict__ cnt, unsigned long long* __restrict__ off, int n,
                                  unsigned long long* __restrict__ block_tot)
{
    __shared__ unsigned long long warp_tot[2][32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 2; ++q)
    {
        unsigned long long v = i < n ? cnt[2 * i + q] : 0ull, x = v;
        for (int o = 1; o < 32; o <<= 1)
        {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o)
                x += y;
        }
        if (lane == 31)
            warp_tot[q][w] = x;
        __syncthreads();
        if (w == 0)
        {
            unsigned long long t = warp_tot[q][lane], tx = t;
            for (int o = 1; o < 32; o <<= 1)
            {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, tx, o);
                if (lane >= o)
                    tx += y;
            }
            warp_tot[q][lane] = tx - t; // exclusive warp offsets
            if (lane == 31)
                block_tot[2 * blockIdx.x + q] = tx;
        }
        __syncthreads();
        if (i < n)
            off[2 * i + q] = x - v + warp_tot[q][w];
        __syncthreads();
    }
}

__global__ void scan_tops_kernel(unsigned long long* __restrict__ block_tot, int nb, unsigned long long* __restrict__ total)
{
    if (threadIdx.x == 0)
        for (int q = 0; q < 2; ++q)
        {
            unsigned long long run = 0;
            for (int b = 0; b < nb; ++b)
            {
                const unsigned long long t = block_tot[2 * b + q];
                block_tot[2 * b + q] = run;
                run += t;
            }
            total[q] = run;
        }
}

__global__ void scan_add_kernel(unsigned long long* __restrict__ off, int n, const unsigned long long* __restrict__ block_tot)
{
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n)
    {
        off[2 * i] += block_tot[2 * blockIdx.x];
        off[2 * i + 1] += block_tot[2 * blockIdx.x + 1];
    }
}

// J = X + X^T, K = Y + Y^T over the concatenated molecule blocks.
__global__ void symmetrize_kernel(const double* __restrict__ X, double* __restrict__ J, const long long* __restrict__ mat_off,
                                  const int* __restrict__ mat_ld, int nmol, long long total)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    {
        int lo = 0, hi = nmol - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (mat_off[mid] <= e)
                lo = mid;
            else
                hi = mid - 1;
        }
        const long long off = mat_off[lo];
        const int n = mat_ld[lo];
        const long long loc = e - off;
        const int r = static_cast<int>(loc % n), c = static_cast<int>(loc / n);
        J[e] = X[e] + X[off + c + (long long)r * n];
    }
}

// Q(pair) = sqrt(max_ij (ij|ij)) from stored (P|P) blocks.
__global__ void schwartz_from_store_kernel(const double* __restrict__ store, const Quartet* __restrict__ list, int n,
                                           int nab, double* __restrict__ Qpair)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    {
        double mx = 0.0;
        for (int ij = 0; ij < nab; ++ij) mx = fmax(mx, store[(long long)k * nab * nab + ij * nab + ij]);
        Qpair[list[k].bra] = sqrt(mx);
    }
}

// ------------------------------------------------------------------------------------------------
// Host helpers.
// ------------------------------------------------------------------------------------------------
inline int grid_for(long long n, int threads, int num_sms)
{
    long long g = (n + threads - 1) / threads;
    const long long cap = static_cast<long long>(num_sms) * 16;
    if (g > cap)
        g = cap;
    return static_cast<int>(g < 1 ? 1 : g);
}

double ang_norm_host(int l, int c)
{
    const int i = cart_exp(l, c, 0), j = cart_exp(l, c, 1), k = cart_exp(l, c, 2);
    return 1.0 / std::sqrt(static_cast<double>(dfact_odd(2 * i - 1) * dfact_odd(2 * j - 1) * dfact_odd(2 * k - 1)));
}

void validate_and_copy(const hfg_basis& b, HostBasis& hb)
{
    if (b.nshells <= 0 || b.nao <= 0 || b.nprim <= 0 || !b.l || !b.nprim_sh || !b.prim_off || !b.ao_off ||
        !b.norm_off || !b.centers || !b.alpha || !b.coeff || !b.norms || !b.am)
        throw HfgError(HFG_ERR_INVALID, "basis: missing arrays or empty basis");
    hb.l.assign(b.l, b.l + b.nshells);
    hb.nprim.assign(b.nprim_sh, b.nprim_sh + b.nshells);
    hb.prim_off.assign(b.prim_off, b.prim_off + b.nshells);
    hb.ao_off.assign(b.ao_off, b.ao_off + b.nshells);
    hb.centers.assign(b.centers, b.centers + 3 * b.nshells);
    hb.alpha.assign(b.alpha, b.alpha + b.nprim);
    hb.coeff.assign(b.coeff, b.coeff + b.nprim);
    hb.radial.assign(b.nprim, 0.0);
    hb.norm_off.assign(b.norm_off, b.norm_off + b.nshells);
    hb.am.assign(b.am, b.am + 3 * b.nao);
    {
        size_t nn = 0;
        for (int s = 0; s < b.nshells; ++s)
        {
            if (b.l[s] < 0 || b.l[s] > kMaxL || b.nprim_sh[s] <= 0)
                break;
            nn = std::max(nn, static_cast<size_t>(b.norm_off[s]) + static_cast<size_t>(b.nprim_sh[s]) * ncart(b.l[s]));
        }
        hb.norms.assign(b.norms, b.norms + nn);
    }
    int ao = 0;
    for (int s = 0; s < b.nshells; ++s)
    {
        const int l = b.l[s];
        if (l < 0 || l > kMaxL)
            throw HfgError(HFG_ERR_UNSUPPORTED, "basis: angular momentum " + std::to_string(l) +
                                                    " above d (l <= 2) is not supported");
        if (b.nprim_sh[s] <= 0 || b.prim_off[s] < 0 || b.prim_off[s] + b.nprim_sh[s] > b.nprim)
            throw HfgError(HFG_ERR_BASIS, "basis: bad primitive range of shell " + std::to_string(s));
        if (b.ao_off[s] != ao)
            throw HfgError(HFG_ERR_BASIS, "basis: AO offsets are not contiguous at shell " + std::to_string(s));
        const int nc = ncart(l);
        for (int c = 0; c < nc; ++c)
            for (int ax = 0; ax < 3; ++ax)
                if (b.am[3 * (ao + c) + ax] != cart_exp(l, c, ax))
                    throw HfgError(HFG_ERR_BASIS, "basis: Cartesian order differs from the reference's at shell " +
                                                      std::to_string(s));
        for (int p = 0; p < b.nprim_sh[s]; ++p)
        {
            const double a = b.alpha[b.prim_off[s] + p];
            if (!(a > 0.0) || !std::isfinite(a) || !std::isfinite(b.coeff[b.prim_off[s] + p]))
                throw HfgError(HFG_ERR_BASIS, "basis: non-positive or non-finite exponent in shell " + std::to_string(s));
            // The reference's factor (src/Basis.cpp:69-73) is radial(alpha, l) * angular(component).
            const double rad = b.norms[b.norm_off[s] + p * nc + 0] / ang_norm_host(l, 0);
            for (int c = 0; c < nc; ++c)
            {
                const double want = rad * ang_norm_host(l, c);
                const double got  = b.norms[b.norm_off[s] + p * nc + c];
                if (!(std::fabs(got - want) <= 1e-12 * std::fabs(want)))
                    throw HfgError(HFG_ERR_BASIS, "basis: normalisation factors of shell " + std::to_string(s) +
                                                      " do not factor into radial x angular parts");
            }
            hb.radial[b.prim_off[s] + p] = rad;
        }
        for (int ax = 0; ax < 3; ++ax)
            if (!std::isfinite(b.centers[3 * s + ax]))
                throw HfgError(HFG_ERR_BASIS, "basis: non-finite centre of shell " + std::to_string(s));
        ao += nc;
    }
    if (ao != b.nao)
        throw HfgError(HFG_ERR_BASIS, "basis: nao does not match the shells");
    hb.view = hfg_basis {b.nshells, b.nao, b.nprim, hb.l.data(), hb.nprim.data(), hb.prim_off.data(), hb.ao_off.data(),
                         hb.norm_off.data(), hb.centers.data(), hb.alpha.data(), hb.coeff.data(), hb.norms.data(),
                         hb.am.data()};
}

// 1-D Hermite coefficients E^{ij}_t of one axis for i <= l1, j <= l2 (McMurchie-Davidson recurrences;
// the reference builds the same table in src/IntegralEngine.cpp:1025-1079).  E[i][j][t], K not included.
void hermite_1d(int l1, int l2, double p, double PA, double PB, double E[kMaxL + 1][kMaxL + 1][2 * kMaxL + 1])
{
    std::memset(E, 0, sizeof(double) * (kMaxL + 1) * (kMaxL + 1) * (2 * kMaxL + 1));
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

// Drops the captured build graph (a buffer it uses is about to change).
static void invalidate_graph(hfg_engine* e)
{
    if (e->graph_exec)
        cudaGraphExecDestroy(e->graph_exec);
    if (e->graph)
        cudaGraphDestroy(e->graph);
    e->graph_exec = nullptr;
    e->graph      = nullptr;
}

// Uploads the pairs and both layouts of the primitive-pair tables for the current pp_off numbering and
// the kept primitive pairs of every pair.
static void upload_pair_tables(hfg_engine* e)
{
    using namespace hfg;
    invalidate_graph(e);
    std::vector<size_t> total(kNumPairClasses, 0);
    for (size_t k = 0; k < e->pairs.size(); ++k) total[e->pair_class_of[k]] += e->pairs[k].npp;
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        const int stride      = pp_stride(pair_class_l1(pc), pair_class_l2(pc));
        const size_t ks       = std::max<size_t>(32, (total[pc] + 31) / 32 * 32);
        std::vector<double> aos(total[pc] * stride), soa(ks * stride, 0.0);
        for (size_t k = 0; k < e->pairs.size(); ++k)
        {
            if (e->pair_class_of[k] != pc)
                continue;
            const PairRec& pr = e->pairs[k];
            for (int i = 0; i < pr.npp; ++i)
            {
                const int idx     = e->keep_idx[e->keep_off[k] + i];
                const double* src = &e->h_tab[pc][static_cast<size_t>(e->orig_off[k] + idx) * stride];
                const size_t slot = static_cast<size_t>(pr.pp_off + i);
                std::copy(src, src + stride, &aos[slot * stride]);
                const size_t kslot = static_cast<size_t>(pr.kslot) + static_cast<size_t>(i) * pr.kstep;
                for (int f = 0; f < stride; ++f) soa[f * ks + kslot] = src[f];
            }
        }
        e->d_pptab64[pc].upload(aos, e->stream);
        e->d_pptab32[pc].upload(std::vector<float>(aos.begin(), aos.end()), e->stream);
        e->d_ksoa64[pc].upload(soa, e->stream);
        e->d_ksoa32[pc].upload(std::vector<float>(soa.begin(), soa.end()), e->stream);
        e->kfs[pc] = static_cast<long long>(ks);
    }
    e->d_pairs.upload(e->pairs, e->stream);
    std::vector<PairRec> sp(e->spair_id.size()), gp(e->spair_id.size());
    for (size_t k = 0; k < sp.size(); ++k)
    {
        const int id = e->spair_id[k];
        sp[k]        = e->pairs[id];
        gp[k]        = e->pairs[id];
        gp[k].npp    = e->npp_full[id];
        gp[k].pp_off = e->orig_off[id];
        gp[k].kslot  = e->orig_off[id];
        gp[k].kstep  = 1;
    }
    e->d_spairs.upload(sp, e->stream);
    e->d_gspairs.upload(gp, e->stream);
    HFG_CUDA(cudaStreamSynchronize(e->stream)); // the host vectors above die here
}

// Coulomb self-repulsion bound sqrt(max_ij (ab_ij|ab_ij)) of ONE primitive pair from its record (p, W,
// Hermite coefficients E^{ij}_{tuv}).  With P = Q and q = p the Hermite integrals are R_{tuv} =
// (t-1)!!(u-1)!!(v-1)!! (-p)^n / (2n+1) for even t, u, v (n = (t+u+v)/2) and 0 otherwise, and the
// prefactor is W^2 / sqrt(2p).  By the Cauchy-Schwarz inequality of the Coulomb metric, the primitive
// pair's share of any integral (ab|cd) is at most this bound times Q_cd.
static double prim_self_bound(int l1, int l2, const std::vector<double>& rec)
{
    using namespace hfg;
    const double p = rec[0], W = rec[4];
    double best    = 0.0;
    for (int ij = 0; ij < ncart(l1) * ncart(l2); ++ij)
    {
        const int lx = e3_len(l1, l2, ij, 0), ly = e3_len(l1, l2, ij, 1), lz = e3_len(l1, l2, ij, 2);
        const int off = kPairHeader + e3_offset(l1, l2, ij);
        double acc    = 0.0;
        for (int e1 = 0; e1 < lx * ly * lz; ++e1)
            for (int e2 = 0; e2 < lx * ly * lz; ++e2)
            {
                const int t = e1 % lx + e2 % lx, u = (e1 / lx) % ly + (e2 / lx) % ly, v = e1 / (lx * ly) + e2 / (lx * ly);
                if ((t | u | v) & 1)
                    continue;
                const int n = (t + u + v) / 2;
                const int t2 = e2 % lx + (e2 / lx) % ly + e2 / (lx * ly);
                const double r = dfact_odd(t - 1) * dfact_odd(u - 1) * dfact_odd(v - 1) * std::pow(-p, n) / (2 * n + 1);
                acc += ((t2 & 1) ? -1.0 : 1.0) * rec[off + e1] * rec[off + e2] * r;
            }
        const double an = ang_norm_host(l1, ij / ncart(l2)) * ang_norm_host(l2, ij % ncart(l2));
        best            = std::max(best, acc * an * an);
    }
    return std::sqrt(best) * std::fabs(W) / std::pow(2.0 * p, 0.25);
}

// Keeps, per pair, the primitive pairs whose bound times max Q reaches prim_thr (all if prim_thr is 0).
static void screen_primitives(hfg_engine* e)
{
    double qmax = 0.0;
    for (double q : e->Qpair) qmax = std::max(qmax, q);
    e->keep_off.assign(e->pairs.size() + 1, 0);
    e->keep_idx.clear();
    for (size_t k = 0; k < e->pairs.size(); ++k)
    {
        const std::vector<double>& qp = e->h_qp[e->pair_class_of[k]];
        for (int i = 0; i < e->npp_full[k]; ++i)
            if (!(e->prim_thr > 0.0) || qp[e->orig_off[k] + i] * qmax >= e->prim_thr)
                e->keep_idx.push_back(i);
        e->keep_off[k + 1] = static_cast<int>(e->keep_idx.size());
        e->pairs[k].npp    = e->keep_off[k + 1] - e->keep_off[k];
    }
}

// Builds pairs, primitive-pair tables and sorted class lists skeleton (without Q).
static void pack_molecules(hfg_engine* e)
{
    using namespace hfg;
    std::vector<std::vector<double>> tab(kNumPairClasses);
    std::vector<int> class_npp(kNumPairClasses, 0);
    for (int m = 0; m < e->nmol; ++m)
    {
        const HostBasis& b = e->basis[m];
        const int ns       = e->mols[m].nshells;
        for (int s1 = 0; s1 < ns; ++s1)
            for (int s2 = 0; s2 <= s1; ++s2)
            {
                int a = s1, bb = s2;
                if (b.l[bb] > b.l[a])
                    std::swap(a, bb);
                const int l1 = b.l[a], l2 = b.l[bb];
                const int pc = pair_class(l1, l2);
                PairRec pr {};
                pr.sh1    = a;
                pr.sh2    = bb;
                pr.ao1    = b.ao_off[a];
                pr.ao2    = b.ao_off[bb];
                pr.pp_off = class_npp[pc];
                pr.npp    = b.nprim[a] * b.nprim[bb];
                pr.mol    = m;
                pr.same   = (s1 == s2) ? 1 : 0;
                pr.kslot  = pr.pp_off;
                pr.kstep  = 1;
                const double* A = &b.centers[3 * a];
                const double* B = &b.centers[3 * bb];
                const double AB2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
                const int stride = pp_stride(l1, l2);
                for (int pa = 0; pa < b.nprim[a]; ++pa)
                    for (int pb = 0; pb < b.nprim[bb]; ++pb)
                    {
                        const double aa = b.alpha[b.prim_off[a] + pa], ab = b.alpha[b.prim_off[bb] + pb];
                        const double p = aa + ab, ip = 1.0 / p;
                        double P[3], PA[3], PB[3];
                        for (int k = 0; k < 3; ++k)
                        {
                            P[k]  = (aa * A[k] + ab * B[k]) * ip;
                            PA[k] = P[k] - A[k];
                            PB[k] = P[k] - B[k];
                        }
                        const double Kw = std::exp(-aa * ab * ip * AB2) * b.coeff[b.prim_off[a] + pa] *
                                          b.coeff[b.prim_off[bb] + pb] * b.radial[b.prim_off[a] + pa] *
                                          b.radial[b.prim_off[bb] + pb];
                        std::vector<double> rec(stride, 0.0);
                        rec[0] = p;
                        rec[1] = P[0];
                        rec[2] = P[1];
                        rec[3] = P[2];
                        rec[4] = std::sqrt(kTwoPi25) * ip * Kw;
                        rec[5] = ip;
                        double E[3][kMaxL + 1][kMaxL + 1][2 * kMaxL + 1];
                        for (int k = 0; k < 3; ++k) hermite_1d(l1, l2, p, PA[k], PB[k], E[k]);
                        int x = kPairHeader;
                        for (int ij = 0; ij < ncart(l1) * ncart(l2); ++ij)
                        {
                            const int ci = ij / ncart(l2), cj = ij % ncart(l2);
                            const int ix = cart_exp(l1, ci, 0), iy = cart_exp(l1, ci, 1), iz = cart_exp(l1, ci, 2);
                            const int jx = cart_exp(l2, cj, 0), jy = cart_exp(l2, cj, 1), jz = cart_exp(l2, cj, 2);
                            for (int v = 0; v <= iz + jz; ++v)
                                for (int u = 0; u <= iy + jy; ++u)
                                    for (int t = 0; t <= ix + jx; ++t)
                                        rec[x++] = E[0][ix][jx][t] * E[1][iy][jy][u] * E[2][iz][jz][v];
                        }
                        tab[pc].insert(tab[pc].end(), rec.begin(), rec.end());
                        e->h_qp[pc].push_back(prim_self_bound(l1, l2, rec));
                    }
                class_npp[pc] += pr.npp;
                e->orig_off.push_back(pr.pp_off);
                e->npp_full.push_back(pr.npp);
                e->pairs.push_back(pr);
                e->pair_class_of.push_back(pc);
            }
    }
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        e->h_tab[pc] = std::move(tab[pc]);
        e->d_pptab64_full[pc].upload(e->h_tab[pc], e->stream);
        e->d_pptab32_full[pc].upload(std::vector<float>(e->h_tab[pc].begin(), e->h_tab[pc].end()), e->stream);
    }
    e->keep_off.assign(e->pairs.size() + 1, 0);
    e->keep_idx.clear();
    for (size_t k = 0; k < e->pairs.size(); ++k)
    {
        for (int i = 0; i < e->npp_full[k]; ++i) e->keep_idx.push_back(i);
        e->keep_off[k + 1] = static_cast<int>(e->keep_idx.size());
    }
    upload_pair_tables(e);
    std::vector<long long> moff;
    std::vector<int> mld;
    for (const auto& mi : e->mols)
    {
        moff.push_back(mi.mat_off);
        mld.push_back(mi.nao);
    }
    e->d_mat_off.upload(moff, e->stream);
    e->d_mat_ld.upload(mld, e->stream);
    {
        std::vector<long long> so;
        std::vector<int> nsh;
        for (const auto& mi : e->mols)
        {
            so.push_back(mi.smax_off);
            nsh.push_back(mi.nshells);
        }
        std::vector<int> shnao(2 * e->pairs.size());
        for (size_t k = 0; k < e->pairs.size(); ++k)
        {
            const auto& b = e->basis[e->pairs[k].mol];
            shnao[2 * k]     = ncart(b.l[e->pairs[k].sh1]);
            shnao[2 * k + 1] = ncart(b.l[e->pairs[k].sh2]);
        }
        e->d_smax_off.upload(so, e->stream);
        e->d_nsh.upload(nsh, e->stream);
        e->d_shnao.upload(shnao, e->stream);
    }
    auto tables = std::make_unique<WarpTables>();
    build_warp_tables(*tables);
    e->d_tables.alloc(1);
    HFG_CUDA(cudaMemcpyAsync(e->d_tables.p, tables.get(), sizeof(WarpTables), cudaMemcpyHostToDevice, e->stream));
    for (int L = 0; L <= kMaxLt + 1; ++L)
    {
        e->d_boys64[L].upload(boys_slice_host<double>(L), e->stream);
        e->d_boys32[L].upload(boys_slice_host<float>(L), e->stream);
    }
    HFG_CUDA(cudaStreamSynchronize(e->stream));
}

static FockView base_view(hfg_engine* e, bool fp32)
{
    FockView v {};
    v.pairs = e->d_pairs.p;
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        v.pptab[pc] = fp32 ? static_cast<const void*>(e->d_pptab32[pc].p) : static_cast<const void*>(e->d_pptab64[pc].p);
        v.ksoa[pc]  = fp32 ? static_cast<const void*>(e->d_ksoa32[pc].p) : static_cast<const void*>(e->d_ksoa64[pc].p);
        v.kfs[pc]   = e->kfs[pc];
    }
    v.mat_off = e->d_mat_off.p;
    v.mat_ld  = e->d_mat_ld.p;
    return v;
}

static int qclass_of(int pb, int pk) { return quartet_class(std::max(pb, pk), std::min(pb, pk)); }

// Evaluates a list of quartets of one class in store mode (FP64) into d_store.
static void eval_store(hfg_engine* e, int qc, const std::vector<Quartet>& q)
{
    const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
    const int P2 = qc - P1 * (P1 + 1) / 2;
    const int nq = ncart(pair_class_l1(P1)) * ncart(pair_class_l2(P1)) * ncart(pair_class_l1(P2)) * ncart(pair_class_l2(P2));
    e->d_tmp_list.upload(q, e->stream);
    e->d_tmp_count.alloc(1);
    unsigned long long n = q.size();
    HFG_CUDA(cudaMemcpyAsync(e->d_tmp_count.p, &n, sizeof(n), cudaMemcpyHostToDevice, e->stream));
    e->d_store.alloc(q.size() * nq);
    ClassLaunch L {};
    L.list       = e->d_tmp_list.p;
    L.count_dev  = e->d_tmp_count.p;
    L.count_host = n;
    L.view       = base_view(e, false);
    L.view.store = e->d_store.p;
    L.view.ao_thr = 0.0;
    L.boys_slice = e->d_boys64[pair_class_l1(P1) + pair_class_l2(P1) + pair_class_l1(P2) + pair_class_l2(P2)].p;
    L.tables     = e->d_tables.p;
    L.fp32       = false;
    L.uhf        = false;
    L.stream     = e->stream;
    L.num_sms    = e->num_sms;
    HFG_CUDA(launch_class(qc, L));
}

static void compute_schwartz(hfg_engine* e)
{
    e->Qpair.assign(e->pairs.size(), 0.0);
    DevBuf<double> dQ;
    dQ.alloc(e->pairs.size());
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        std::vector<Quartet> q;
        for (size_t k = 0; k < e->pairs.size(); ++k)
            if (e->pair_class_of[k] == pc)
                q.push_back(Quartet {static_cast<uint32_t>(k), static_cast<uint32_t>(k)});
        if (q.empty())
            continue;
        eval_store(e, quartet_class(pc, pc), q);
        const int nab = ncart(pair_class_l1(pc)) * ncart(pair_class_l2(pc));
        schwartz_from_store_kernel<<<grid_for(q.size(), 128, e->num_sms), 128, 0, e->stream>>>(
            e->d_store.p, e->d_tmp_list.p, static_cast<int>(q.size()), nab, dQ.p);
        HFG_CUDA(cudaGetLastError());
        HFG_CUDA(cudaStreamSynchronize(e->stream));
    }
    HFG_CUDA(cudaMemcpyAsync(e->Qpair.data(), dQ.p, sizeof(double) * e->pairs.size(), cudaMemcpyDeviceToHost, e->stream));
    HFG_CUDA(cudaStreamSynchronize(e->stream));
    e->d_store.release();
}

// Sorts each pair class by (molecule, primitive-pair count descending, Q descending) and records the
// segments of equal primitive-pair count; uploads the class lists.
static void sort_classes(hfg_engine* e)
{
    screen_primitives(e);
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        auto& ids = e->cls_ids[pc];
        ids.clear();
        for (size_t k = 0; k < e->pairs.size(); ++k)
            if (e->pair_class_of[k] == pc)
                ids.push_back(static_cast<int>(k));
        std::stable_sort(ids.begin(), ids.end(), [&](int x, int y) {
            const PairRec &px = e->pairs[x], &py = e->pairs[y];
            if (px.mol != py.mol)
                return px.mol < py.mol;
            if (px.npp != py.npp)
                return px.npp > py.npp;
            return e->Qpair[x] > e->Qpair[y];
        });
        e->cls_Q[pc].resize(ids.size());
        for (size_t k = 0; k < ids.size(); ++k) e->cls_Q[pc][k] = e->Qpair[ids[k]];
        e->cls_seg[pc].clear();
        e->cls_molseg[pc].assign(e->nmol, make_int2(0, 0));
        size_t k = 0;
        for (int m = 0; m < e->nmol; ++m)
        {
            const int first = static_cast<int>(e->cls_seg[pc].size());
            while (k < ids.size() && e->pairs[ids[k]].mol == m)
            {
                const size_t b = k;
                const int npp  = e->pairs[ids[k]].npp;
                while (k < ids.size() && e->pairs[ids[k]].mol == m && e->pairs[ids[k]].npp == npp) ++k;
                e->cls_seg[pc].push_back(make_int4(static_cast<int>(b), static_cast<int>(k), npp, m));
            }
            e->cls_molseg[pc][m] = make_int2(first, static_cast<int>(e->cls_seg[pc].size()));
        }
        std::vector<int2> sh(ids.size());
        for (size_t k2 = 0; k2 < ids.size(); ++k2) sh[k2] = make_int2(e->pairs[ids[k2]].sh1, e->pairs[ids[k2]].sh2);
        e->d_cls_sh[pc].upload(sh, e->stream);
        e->d_cls_ids[pc].upload(ids, e->stream);
        e->d_cls_Q[pc].upload(e->cls_Q[pc], e->stream);
        {
            std::vector<float> qf(e->cls_Q[pc].begin(), e->cls_Q[pc].end());
            e->d_cls_Qf[pc].upload(qf, e->stream);
        }
        e->d_cls_seg[pc].upload(e->cls_seg[pc], e->stream);
        e->d_cls_molseg[pc].upload(e->cls_molseg[pc], e->stream);
    }
    HFG_CUDA(cudaStreamSynchronize(e->stream));
    // Renumber the primitive slots of every class in sorted-list order.  Whole records (pp_off) stay
    // contiguous per pair; in the field-major tables a segment of equal primitive count is stored
    // primitive-major, so the kets of a warp (neighbours in one segment) read neighbouring slots for
    // every primitive index.
    e->cls_base.assign(kNumPairClasses, 0);
    e->spair_id.clear();
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        e->cls_base[pc] = static_cast<int>(e->spair_id.size());
        e->spair_id.insert(e->spair_id.end(), e->cls_ids[pc].begin(), e->cls_ids[pc].end());
        int off = 0;
        for (const int4& seg : e->cls_seg[pc])
        {
            const int seg_off = off, len = seg.y - seg.x;
            for (int k = seg.x; k < seg.y; ++k)
            {
                PairRec& pr = e->pairs[e->cls_ids[pc][k]];
                pr.pp_off   = off;
                pr.kslot    = seg_off + (k - seg.x);
                pr.kstep    = len;
                off += pr.npp;
            }
        }
    }
    upload_pair_tables(e);
    e->have_Q  = true;
    e->cap_thr = -1.0; // capacities depend on Q
}

// Schwartz prefix of bra position i (class P1) inside ket segment seg (class P2).
static int prefix_end(const hfg_engine* e, int P1, int P2, size_t i, const int4& seg, double sthr)
{
    const int jb = seg.x;
    const int je = (P1 == P2) ? std::min(seg.y, static_cast<int>(i) + 1) : seg.y;
    int lo = jb, hi = std::max(jb, je);
    const double Qi = e->cls_Q[P1][i];
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (Qi * e->cls_Q[P2][mid] < sthr)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// Exact Schwartz-only survivor count per quartet class (an upper bound of any build's list).
static void size_lists(hfg_engine* e, double sthr, bool mixed)
{
    if (e->cap_thr == sthr && (!mixed || e->cap_mixed))
        return;
    invalidate_graph(e);
    for (int P1 = 0; P1 < kNumPairClasses; ++P1)
        for (int P2 = 0; P2 <= P1; ++P2)
        {
            const int qc = quartet_class(P1, P2);
            unsigned long long c = 0;
            for (size_t i = 0; i < e->cls_ids[P1].size(); ++i)
            {
                const int mol = e->pairs[e->cls_ids[P1][i]].mol;
                const int2 ms = e->cls_molseg[P2][mol];
                for (int sg = ms.x; sg < ms.y; ++sg)
                {
                    const int4& seg = e->cls_seg[P2][sg];
                    c += static_cast<unsigned long long>(std::max(0, prefix_end(e, P1, P2, i, seg, sthr) - seg.x));
                }
            }
            e->cap[qc] = c;
            e->d_list[qc][0].alloc(std::max<unsigned long long>(c, 1));
            if (mixed)
                e->d_list[qc][1].alloc(std::max<unsigned long long>(c, 1));
            e->d_bra_cnt[qc].alloc(2 * std::max<size_t>(e->cls_ids[P1].size(), 1));
            e->d_bra_off[qc].alloc(2 * std::max<size_t>(e->cls_ids[P1].size(), 1));
        }
    e->cap_thr   = sthr;
    e->cap_mixed = mixed;
}

// Screening and the survival lists of every quartet class from the densities already in d_dD[0..2]
// (the shell-pair maxima, then count pass, scan and write pass per class).  Returns the launches.
// graph: enqueue only (no host synchronisation); the counts go to the pinned buffer, checked after replay.
static int build_lists(hfg_engine* e, bool uhf, bool mixed, double sthr, double dthr, double cutoff, bool graph = false)
{
    cudaStream_t s  = e->stream;
    const int nspin = uhf ? 3 : 2;
    // Shell-pair maxima.
    for (int k = 0; k < nspin; ++k)
    {
        if (k == 0)
            e->d_smax2.alloc(e->smax_total);
        shell_max_kernel<<<grid_for(e->pairs.size(), 128, e->num_sms), 128, 0, s>>>(
            e->d_dD[k].p, e->d_pairs.p, static_cast<int>(e->pairs.size()), e->d_mat_off.p, e->d_mat_ld.p, e->d_smax_off.p,
            e->d_nsh.p, e->d_shnao.p, e->d_smax[k].p, k == 0 ? e->d_smax2.p : nullptr);
        HFG_CUDA(cudaGetLastError());
    }

    // Lists: count pass, scan, write pass, per quartet class.
    const int ncnt = kNumQuartetClasses * 2;
    e->d_counts.alloc(2 * ncnt + 1);
    HFG_CUDA(cudaMemsetAsync(e->d_counts.p, 0, sizeof(unsigned long long) * (2 * ncnt + 1), s));
    int launches = 0;
    size_t max_blocks = 1;
    for (int P1 = 0; P1 < kNumPairClasses; ++P1)
        max_blocks = std::max(max_blocks, (e->cls_ids[P1].size() + kScanBlock - 1) / kScanBlock);
    e->d_scan_tmp.alloc(2 * max_blocks);
    for (int pass = 0; pass < 2; ++pass)
        for (int P1 = 0; P1 < kNumPairClasses; ++P1)
            for (int P2 = 0; P2 <= P1; ++P2)
            {
                const int qc = quartet_class(P1, P2);
                if (e->cap[qc] == 0 || e->cls_ids[P1].empty() || e->cls_ids[P2].empty())
                    continue;
                BuildArgs a {};
                a.ids1 = e->d_cls_ids[P1].p;
                a.base1 = e->cls_base[P1];
                a.base2 = e->cls_base[P2];
                a.Q1   = e->d_cls_Q[P1].p;
                a.n1   = static_cast<int>(e->cls_ids[P1].size());
                a.Q2   = e->d_cls_Q[P2].p;
                a.sh2  = e->d_cls_sh[P2].p;
                a.seg2 = e->d_cls_seg[P2].p;
                a.molseg2 = e->d_cls_molseg[P2].p;
                a.same_class = P1 == P2;
                a.pairs = e->d_pairs.p;
                a.Mt = e->d_smax[0].p;
                a.Mt2 = e->d_smax2.p;
                a.Ma = e->d_smax[1].p;
                a.Mb = uhf ? e->d_smax[2].p : nullptr;
                a.Qf1 = e->d_cls_Qf[P1].p;
                a.Qf2 = e->d_cls_Qf[P2].p;
                a.smax_off = e->d_smax_off.p;
                a.nsh = e->d_nsh.p;
                a.sthr = sthr;
                a.dthr = dthr;
                a.cutoff = static_cast<float>(cutoff);
                a.mixed = mixed ? 1 : 0;
                a.pass = pass;
                a.bra_cnt = e->d_bra_cnt[qc].p;
                a.bra_off = e->d_bra_off[qc].p;
                a.out64 = e->d_list[qc][0].p;
                a.out32 = mixed ? e->d_list[qc][1].p : nullptr;
                a.prim64 = e->d_counts.p + ncnt + 2 * qc;
                a.prim32 = e->d_counts.p + ncnt + 2 * qc + 1;
                a.cap = e->cap[qc];
                const long long threads = static_cast<long long>(a.n1) * 32;
                build_lists_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, s>>>(a);
                HFG_CUDA(cudaGetLastError());
                ++launches;
                if (pass == 0)
                {
                    const int nb = (a.n1 + kScanBlock - 1) / kScanBlock;
                    scan_block_kernel<<<nb, kScanBlock, 0, s>>>(e->d_bra_cnt[qc].p, e->d_bra_off[qc].p, a.n1,
                                                                e->d_scan_tmp.p);
                    scan_tops_kernel<<<1, 32, 0, s>>>(e->d_scan_tmp.p, nb, e->d_counts.p + 2 * qc);
                    scan_add_kernel<<<nb, kScanBlock, 0, s>>>(e->d_bra_off[qc].p, a.n1, e->d_scan_tmp.p);
                    HFG_CUDA(cudaGetLastError());
                    launches += 3;
                }
            }
    if (graph)
        return launches + nspin;
    e->h_counts.assign(2 * ncnt + 1, 0);
    HFG_CUDA(cudaMemcpyAsync(e->h_counts.data(), e->d_counts.p, sizeof(unsigned long long) * (2 * ncnt + 1),
                             cudaMemcpyDeviceToHost, s));
    HFG_CUDA(cudaEventRecord(e->ev[2], s));
    HFG_CUDA(cudaStreamSynchronize(s));
    for (int qc = 0; qc < kNumQuartetClasses; ++qc)
        if (e->h_counts[2 * qc] > e->cap[qc] || e->h_counts[2 * qc + 1] > e->cap[qc])
            throw HfgError(HFG_ERR_OVERFLOW, "fock: quartet list overflow");

    return launches + nspin;
}

// Kernel form autotuner.  A class whose list has at least kTuneMin quartets and more than one compiled
// form runs each form on a sample of its real list (same densities, thresholds and Boys slice; scratch
// accumulators), once to warm up and kTuneReps times timed with events; the fastest form is kept.  The
// sample is kTuneChunks contiguous runs spread over the list: contiguous, because neighbouring quartets
// share their bra pair (which sets the digestion's atomic traffic), and spread, because the list is
// ordered by primitive count.  At most kTuneSample quartets, several waves of the largest grid.
constexpr unsigned long long kTuneMin    = 1ull << 16;
constexpr unsigned long long kTuneSample = 1ull << 21;
constexpr unsigned long long kTuneChunks = 16;
constexpr int kTuneReps                  = 2;

int pick_form(hfg_engine* e, int qc, int prec, bool uhf, const ClassLaunch& base, double* ms_tune)
{
    const int set = e->form_set[qc][prec];
    if (set != 0)
        return set;
    int& pick = e->form_pick[qc][prec][uhf ? 1 : 0];
    if (pick != 0)
        return pick;
    const unsigned mask = class_form_mask(qc, prec == 1);
    if ((mask & (mask - 1)) == 0) // a single form
    {
        for (int f = 1; f < 32; ++f)
            if (mask == (1u << f))
                pick = f;
        return pick;
    }
    const unsigned long long n = base.count_host;
    if (n < kTuneMin || !e->autotune)
        return 0; // too small to time, or tuning off: the default form runs and the class stays untuned
    const auto t0 = std::chrono::steady_clock::now();
    const unsigned long long nch   = n <= kTuneSample ? 1 : kTuneChunks;
    const unsigned long long chunk = n <= kTuneSample ? n : kTuneSample / kTuneChunks;
    const unsigned long long m     = nch * chunk;
    cudaStream_t s = base.stream;
    e->d_tune_list.alloc(m);
    e->d_tune_cnt.alloc(1);
    for (int k = 0; k < 3; ++k)
    {
        e->d_tune_acc[k].alloc(e->mat_total);
        HFG_CUDA(cudaMemsetAsync(e->d_tune_acc[k].p, 0, sizeof(double) * e->mat_total, s));
    }
    if (!e->tune_ev[0])
        for (auto& ev : e->tune_ev) HFG_CUDA(cudaEventCreate(&ev));
    sample_list_kernel<<<grid_for(static_cast<long long>(m), 256, e->num_sms), 256, 0, s>>>(base.list, n, nch, chunk,
                                                                                              e->d_tune_list.p, e->d_tune_cnt.p);
    HFG_CUDA(cudaGetLastError());
    ClassLaunch t = base;
    t.list        = e->d_tune_list.p;
    t.count_dev   = e->d_tune_cnt.p;
    t.count_host  = m;
    t.view.X      = e->d_tune_acc[0].p;
    t.view.Ya     = e->d_tune_acc[1].p;
    t.view.Yb     = e->d_tune_acc[2].p;
    float best    = 0.f;
    for (int f = 1; f < 32; ++f)
    {
        if (!((mask >> f) & 1u))
            continue;
        t.form = f;
        HFG_CUDA(launch_class(qc, t));
        HFG_CUDA(cudaEventRecord(e->tune_ev[0], s));
        for (int rep = 0; rep < kTuneReps; ++rep) HFG_CUDA(launch_class(qc, t));
        HFG_CUDA(cudaEventRecord(e->tune_ev[1], s));
        HFG_CUDA(cudaEventSynchronize(e->tune_ev[1]));
        float ms = 0.f;
        HFG_CUDA(cudaEventElapsedTime(&ms, e->tune_ev[0], e->tune_ev[1]));
        if (pick == 0 || ms < best)
        {
            best = ms;
            pick = f;
        }
    }
    *ms_tune += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return pick;
}

// Enqueues one build on the engine stream.  Eager (graph == false): timing events, list lengths read
// back after the list build, only non-empty classes launched, forms tuned on first use.  Graph: nothing
// that needs the host (no read-back, no tuning): every class with a non-empty capacity is launched
// with the grid of its capacity (the kernels read their list lengths on the device, so surplus blocks
// exit at once), and the counts are copied to pinned memory for the host to read after the replay.
static int enqueue_build(hfg_engine* e, const hfg_fock_request& r, bool graph, int form_ran[][2], double* ms_tune)
{
    const bool mixed   = r.precision == HFG_PRECISION_MIXED;
    const bool uhf     = r.unrestricted != 0;
    const long long N2 = e->mat_total;
    cudaStream_t s     = e->stream;
    const int nspin    = uhf ? 3 : 2;
    const double* src[3] = {r.dD_tot, r.dD_alpha, r.dD_beta};
    if (!graph)
        HFG_CUDA(cudaEventRecord(e->ev[0], s));
    for (int k = 0; k < nspin; ++k)
    {
        HFG_CUDA(cudaMemcpyAsync(e->d_dD[k].p, src[k], sizeof(double) * N2,
                                 r.device_pointers ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        HFG_CUDA(cudaMemsetAsync(e->d_acc[k].p, 0, sizeof(double) * N2, s));
        if (mixed)
        {
            to_float_kernel<<<grid_for(N2, 256, e->num_sms), 256, 0, s>>>(e->d_dD[k].p, e->d_dDf[k].p, N2);
            HFG_CUDA(cudaGetLastError());
        }
    }
    if (!graph)
        HFG_CUDA(cudaEventRecord(e->ev[1], s));

    int launches = nspin * (mixed ? 2 : 1) +
                   build_lists(e, uhf, mixed, r.schwartz_threshold, r.density_threshold, r.fp32_cutoff, graph);

    // Class kernels: FP64 lists on `s`; FP32 lists on stream2 concurrently when overlapping, else after.
    const bool overlap = mixed && e->overlap;
    if (overlap)
    {
        HFG_CUDA(cudaEventRecord(e->ev2[0], s));
        HFG_CUDA(cudaStreamWaitEvent(e->stream2, e->ev2[0], 0));
    }
    auto make_view = [&](int prec) {
        FockView v  = base_view(e, prec == 1);
        v.pairs     = e->d_spairs.p;
        v.Dt        = prec == 1 ? static_cast<const void*>(e->d_dDf[0].p) : e->d_dD[0].p;
        v.Da        = prec == 1 ? static_cast<const void*>(e->d_dDf[1].p) : e->d_dD[1].p;
        v.Db        = prec == 1 ? static_cast<const void*>(e->d_dDf[2].p) : e->d_dD[2].p;
        v.X         = e->d_acc[0].p;
        v.Ya        = e->d_acc[1].p;
        v.Yb        = e->d_acc[2].p;
        v.ao_thr    = r.schwartz_threshold;
        v.ao_thr_f  = static_cast<float>(r.schwartz_threshold);
        return v;
    };
    // Persistent mode: one work-queue launch for the small classes of both precisions on `s` (it runs
    // beside the FP32 classes on stream2); those classes are skipped below.
    const bool persist = e->persistent;
    auto in_queue = [&](int qc) {
        return persist && (qc == kPersistentClasses[0] || qc == kPersistentClasses[1] || qc == kPersistentClasses[2] ||
                           qc == kPersistentClasses[3]);
    };
    if (persist)
    {
        if (!graph)
            HFG_CUDA(cudaEventRecord(e->ev[3], s));
        PersistentArgs pa {};
        bool any = false;
        for (int seg = 0; seg < kPersistentSegments; ++seg)
        {
            const int prec = seg / 4, qc = kPersistentClasses[seg % 4];
            if ((prec == 1 && !mixed) || e->cap[qc] == 0 || (!graph && e->h_counts[2 * qc + prec] == 0))
                continue;
            const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
            const int P2 = qc - P1 * (P1 + 1) / 2;
            const int L  = pair_class_l1(P1) + pair_class_l2(P1) + pair_class_l1(P2) + pair_class_l2(P2);
            pa.list[seg]  = e->d_list[qc][prec].p;
            pa.count[seg] = e->d_counts.p + 2 * qc + prec;
            pa.slice[seg] = prec == 1 ? static_cast<const void*>(e->d_boys32[L].p) : e->d_boys64[L].p;
            form_ran[qc][prec] = kFormPersistent;
            any = true;
        }
        if (any)
        {
            pa.view[0] = make_view(0);
            pa.view[1] = make_view(mixed ? 1 : 0);
            e->d_pcounter.alloc(1);
            pa.counter = e->d_pcounter.p;
            HFG_CUDA(launch_persistent(pa, uhf, s, e->num_sms));
            ++launches;
        }
    }
    for (int prec = 0; prec < (mixed ? 2 : 1); ++prec)
    {
        cudaStream_t ps = (overlap && prec == 1) ? e->stream2 : s;
        if (!graph && !(persist && prec == 0))
            HFG_CUDA(cudaEventRecord(overlap && prec == 1 ? e->ev2[2] : e->ev[3 + prec], ps));
        for (int qc = kNumQuartetClasses - 1; qc >= 0; --qc)
        {
            const unsigned long long n = graph ? e->cap[qc] : e->h_counts[2 * qc + prec];
            if (n == 0 || in_queue(qc))
                continue;
            const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
            const int P2 = qc - P1 * (P1 + 1) / 2;
            const int L  = pair_class_l1(P1) + pair_class_l2(P1) + pair_class_l1(P2) + pair_class_l2(P2);
            ClassLaunch c {};
            c.list       = e->d_list[qc][prec].p;
            c.count_dev  = e->d_counts.p + 2 * qc + prec;
            c.count_host = n;
            c.view       = base_view(e, prec == 1);
            c.view.pairs = e->d_spairs.p;
            c.view.Dt    = prec == 1 ? static_cast<const void*>(e->d_dDf[0].p) : e->d_dD[0].p;
            c.view.Da    = prec == 1 ? static_cast<const void*>(e->d_dDf[1].p) : e->d_dD[1].p;
            c.view.Db    = prec == 1 ? static_cast<const void*>(e->d_dDf[2].p) : e->d_dD[2].p;
            c.view.X     = e->d_acc[0].p;
            c.view.Ya    = e->d_acc[1].p;
            c.view.Yb    = e->d_acc[2].p;
            c.view.ao_thr = r.schwartz_threshold;
            c.view.ao_thr_f = static_cast<float>(r.schwartz_threshold);
            c.boys_slice = prec == 1 ? static_cast<const void*>(e->d_boys32[L].p) : e->d_boys64[L].p;
            c.tables     = e->d_tables.p;
            c.fp32       = prec == 1;
            c.uhf        = uhf;
            c.stream     = ps;
            c.num_sms    = e->num_sms;
            c.share      = overlap ? (prec == 1 ? e->overlap_share32 : e->overlap_share) : 1.f;
            if (graph)
            {
                const int set  = e->form_set[qc][prec];
                const int pick = e->form_pick[qc][prec][uhf ? 1 : 0];
                c.form         = set != 0 ? set : pick;
            }
            else
                c.form = pick_form(e, qc, prec, uhf, c, ms_tune);
            HFG_CUDA(launch_class(qc, c));
            form_ran[qc][prec] = c.form != 0 ? c.form : class_default_form(qc, prec == 1);
            launches += class_launches(qc, prec == 1, c.form);
        }
        if (!graph && overlap && prec == 1)
            HFG_CUDA(cudaEventRecord(e->ev2[3], ps));
        if (!graph && overlap && prec == 0)
            HFG_CUDA(cudaEventRecord(e->ev[4], s)); // end of the FP64 kernels
    }
    if (overlap)
    {
        HFG_CUDA(cudaEventRecord(e->ev2[1], e->stream2));
        HFG_CUDA(cudaStreamWaitEvent(s, e->ev2[1], 0));
    }
    if (!graph)
        HFG_CUDA(cudaEventRecord(e->ev[5], s));
    double* outs[3] = {r.J, r.K_alpha, r.K_beta};
    for (int k = 0; k < nspin; ++k)
    {
        symmetrize_kernel<<<grid_for(N2, 256, e->num_sms), 256, 0, s>>>(e->d_acc[k].p, e->d_out[k].p, e->d_mat_off.p,
                                                                          e->d_mat_ld.p, e->nmol, N2);
        HFG_CUDA(cudaGetLastError());
        ++launches;
    }
    if (!graph)
        HFG_CUDA(cudaEventRecord(e->ev[6], s));
    for (int k = 0; k < nspin; ++k)
        HFG_CUDA(cudaMemcpyAsync(outs[k], e->d_out[k].p, sizeof(double) * N2,
                                 r.device_pointers ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    if (graph)
        HFG_CUDA(cudaMemcpyAsync(e->h_counts_pin, e->d_counts.p, sizeof(unsigned long long) * (4 * kNumQuartetClasses + 1),
                                 cudaMemcpyDeviceToHost, s));
    return launches;
}

static void fill_stats(hfg_engine* e, bool uhf, int launches, int form_ran[][2], double ms_tune, hfg_fock_stats* st)
{
    const int ncnt = kNumQuartetClasses * 2;
    std::memset(st, 0, sizeof(*st));
    for (int qc = 0; qc < kNumQuartetClasses; ++qc)
    {
        st->quartets_fp64[qc]      = e->h_counts[2 * qc];
        st->quartets_fp32[qc]      = e->h_counts[2 * qc + 1];
        st->prim_quartets_fp64[qc] = e->h_counts[ncnt + 2 * qc];
        st->prim_quartets_fp32[qc] = e->h_counts[ncnt + 2 * qc + 1];
        st->flops_fp64 += flops_per_prim_quartet(qc) * st->prim_quartets_fp64[qc] +
                          flops_per_quartet_digest(qc, uhf) * st->quartets_fp64[qc];
        st->flops_fp32 += flops_per_prim_quartet(qc) * st->prim_quartets_fp32[qc] +
                          flops_per_quartet_digest(qc, uhf) * st->quartets_fp32[qc];
        st->form_fp64[qc] = st->quartets_fp64[qc] ? form_ran[qc][0] : 0;
        st->form_fp32[qc] = st->quartets_fp32[qc] ? form_ran[qc][1] : 0;
    }
    st->kernel_launches = launches;
    st->ms_tune         = ms_tune;
}

static void fock_direct(hfg_engine* e, const hfg_fock_request& r, hfg_fock_stats* st)
{
    if (!(r.schwartz_threshold >= 0.0) || !(r.density_threshold >= 0.0) || !std::isfinite(r.schwartz_threshold) ||
        !std::isfinite(r.density_threshold))
        throw HfgError(HFG_ERR_INVALID, "fock: thresholds must be finite and >= 0");
    if (!r.dD_tot || !r.dD_alpha || !r.J || !r.K_alpha || (r.unrestricted && (!r.dD_beta || !r.K_beta)))
        throw HfgError(HFG_ERR_INVALID, "fock: missing matrix pointer");
    if (r.precision != HFG_PRECISION_FP64 && r.precision != HFG_PRECISION_MIXED)
        throw HfgError(HFG_ERR_INVALID, "fock: unknown precision mode");
    const bool mixed = r.precision == HFG_PRECISION_MIXED;
    const bool uhf   = r.unrestricted != 0;
    if (!e->have_Q)
    {
        compute_schwartz(e);
        sort_classes(e);
    }
    size_lists(e, r.schwartz_threshold, mixed);
    const long long N2 = e->mat_total;
    cudaStream_t s     = e->stream;
    for (int k = 0; k < 3; ++k)
    {
        e->d_dD[k].alloc(N2);
        e->d_acc[k].alloc(N2);
        e->d_out[k].alloc(N2);
        e->d_smax[k].alloc(e->smax_total);
        if (mixed && !e->d_dDf[k].p)
        {
            invalidate_graph(e);
            e->d_dDf[k].alloc(N2);
        }
    }
    e->d_smax2.alloc(e->smax_total);
    const int ncnt = kNumQuartetClasses * 2;
    const bool use_graph = e->graph_mode && r.device_pointers;
    hfg_engine::GraphKey key;
    key.precision = r.precision;
    key.uhf       = uhf ? 1 : 0;
    key.sthr      = r.schwartz_threshold;
    key.dthr      = r.density_threshold;
    key.cutoff    = mixed ? r.fp32_cutoff : 0.0;
    const void* ptrs[6] = {r.dD_tot, r.dD_alpha, uhf ? r.dD_beta : nullptr, r.J, r.K_alpha, uhf ? r.K_beta : nullptr};
    std::copy(ptrs, ptrs + 6, key.ptr);

    if (use_graph && e->graph_exec && key == e->graph_key)
    {
        // Replay.
        HFG_CUDA(cudaEventRecord(e->ev[1], s));
        HFG_CUDA(cudaGraphLaunch(e->graph_exec, s));
        HFG_CUDA(cudaEventRecord(e->ev[6], s));
        HFG_CUDA(cudaStreamSynchronize(s));
        e->h_counts.assign(e->h_counts_pin, e->h_counts_pin + 2 * ncnt + 1);
        for (int qc = 0; qc < kNumQuartetClasses; ++qc)
            if (e->h_counts[2 * qc] > e->cap[qc] || e->h_counts[2 * qc + 1] > e->cap[qc])
                throw HfgError(HFG_ERR_OVERFLOW, "fock: quartet list overflow");
        e->last_valid = true;
        e->last_mixed = mixed ? 1 : 0;
        if (st)
        {
            fill_stats(e, uhf, e->graph_launches, e->graph_forms, 0.0, st);
            float ms = 0.f;
            HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[1], e->ev[6]));
            st->ms_total = ms; // the split into lists / FP64 / FP32 is not timed inside a graph
        }
        return;
    }

    int form_ran[kNumQuartetClasses][2] {};
    double ms_tune = 0.0;
    const int launches = enqueue_build(e, r, false, form_ran, &ms_tune);
    HFG_CUDA(cudaStreamSynchronize(s));
    e->last_valid = true;
    e->last_mixed = mixed ? 1 : 0;
    if (st)
    {
        fill_stats(e, uhf, launches, form_ran, ms_tune, st);
        float ms = 0.f;
        HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[1], e->ev[6]));
        st->ms_total = ms;
        HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[1], e->ev[2]));
        st->ms_lists = ms;
        HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[3], mixed ? e->ev[4] : e->ev[5]));
        st->ms_eri_fp64 = ms;
        if (mixed)
        {
            // Overlapped: the FP32 kernels' own span on stream2 (it overlaps the FP64 span).
            if (e->overlap)
                HFG_CUDA(cudaEventElapsedTime(&ms, e->ev2[2], e->ev2[3]));
            else
                HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[4], e->ev[5]));
            st->ms_eri_fp32 = ms;
            if (e->overlap)
            {
                HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[3], e->ev[5]));
                st->ms_eri_both = ms;
            }
        }
    }
    if (use_graph)
    {
        // Capture the same build for the next calls with this key (forms are tuned by now).
        invalidate_graph(e);
        if (!e->h_counts_pin)
            HFG_CUDA(cudaMallocHost(&e->h_counts_pin, sizeof(unsigned long long) * (2 * ncnt + 1)));
        int forms[kNumQuartetClasses][2] {};
        double unused = 0.0;
        HFG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        int glaunches = 0;
        try
        {
            glaunches = enqueue_build(e, r, true, forms, &unused);
        }
        catch (...)
        {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g)
                cudaGraphDestroy(g);
            throw;
        }
        HFG_CUDA(cudaStreamEndCapture(s, &e->graph));
        HFG_CUDA(cudaGraphInstantiate(&e->graph_exec, e->graph, 0));
        e->graph_key      = key;
        e->graph_launches = glaunches;
        std::memcpy(e->graph_forms, forms, sizeof(forms));
    }
}

// Stored-integral path (the reference's conventional SCF): IntegralEngine::electronRepulsionTensor
// (src/IntegralEngine.cpp:635-692) evaluates every shell quartet that survives Schwartz screening once;
// here the survivors come from the list builder with the density test switched off (threshold 0 passes
// every candidate), and each class list is evaluated in store mode into its own FP64 buffer.
static void store_integrals(hfg_engine* e, double sthr, size_t* bytes_out)
{
    if (!(sthr >= 0.0) || !std::isfinite(sthr))
        throw HfgError(HFG_ERR_INVALID, "store_integrals: threshold must be finite and >= 0");
    if (!e->have_Q)
    {
        compute_schwartz(e);
        sort_classes(e);
    }
    size_lists(e, sthr, false);
    const long long N2 = e->mat_total;
    for (int k = 0; k < 3; ++k)
    {
        e->d_dD[k].alloc(N2);
        e->d_acc[k].alloc(N2);
        e->d_out[k].alloc(N2);
        e->d_smax[k].alloc(e->smax_total);
        HFG_CUDA(cudaMemsetAsync(e->d_dD[k].p, 0, sizeof(double) * N2, e->stream));
    }
    e->d_smax2.alloc(e->smax_total);
    build_lists(e, false, false, sthr, 0.0, 0.0); // density threshold 0: Schwartz survivors only
    size_t bytes = 0;
    for (int qc = 0; qc < kNumQuartetClasses; ++qc)
    {
        const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
        const int P2 = qc - P1 * (P1 + 1) / 2;
        const size_t nq = ncart(pair_class_l1(P1)) * ncart(pair_class_l2(P1)) * ncart(pair_class_l1(P2)) * ncart(pair_class_l2(P2));
        bytes += e->h_counts[2 * qc] * (nq * sizeof(double) + sizeof(Quartet));
    }
    size_t free_b = 0, total_b = 0;
    HFG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (bytes > free_b / 10 * 8)
        throw HfgError(HFG_ERR_NOMEM, "store_integrals: the stored integrals need " + std::to_string(bytes >> 20) +
                                          " MiB, more than 80% of the free device memory; use the direct build");
    for (int qc = 0; qc < kNumQuartetClasses; ++qc)
    {
        const unsigned long long n = e->h_counts[2 * qc];
        e->conv_n[qc] = n;
        if (n == 0)
            continue;
        const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
        const int P2 = qc - P1 * (P1 + 1) / 2;
        const int L  = pair_class_l1(P1) + pair_class_l2(P1) + pair_class_l1(P2) + pair_class_l2(P2);
        const size_t nq = ncart(pair_class_l1(P1)) * ncart(pair_class_l2(P1)) * ncart(pair_class_l1(P2)) * ncart(pair_class_l2(P2));
        e->d_conv_list[qc].alloc(n);
        HFG_CUDA(cudaMemcpyAsync(e->d_conv_list[qc].p, e->d_list[qc][0].p, sizeof(Quartet) * n, cudaMemcpyDeviceToDevice,
                                 e->stream));
        e->d_conv[qc].alloc(n * nq);
        ClassLaunch c {};
        c.list       = e->d_conv_list[qc].p;
        c.count_dev  = e->d_counts.p + 2 * qc;
        c.count_host = n;
        c.view       = base_view(e, false);
        c.view.pairs = e->d_spairs.p;
        c.view.store = e->d_conv[qc].p;
        c.view.ao_thr = 0.0;
        c.boys_slice = e->d_boys64[L].p;
        c.tables     = e->d_tables.p;
        c.stream     = e->stream;
        c.num_sms    = e->num_sms;
        c.form       = class_default_form(qc, false);
        HFG_CUDA(launch_class(qc, c));
    }
    HFG_CUDA(cudaStreamSynchronize(e->stream));
    e->conv_thr = sthr;
    e->last_valid = false; // the lists of the last direct build were overwritten
    if (bytes_out)
        *bytes_out = bytes;
}

// SCF::buildFockMatrix (src/SCF.cpp:233-521): J[D], K[D] of the FULL densities from the stored integrals,
// with the AO-level skip |(ij|kl)| < SCHWARTZ_THRESH of the reference's loop.  The request's dD fields
// carry the full densities here.
static void fock_conventional(hfg_engine* e, const hfg_fock_request& r, hfg_fock_stats* st)
{
    if (e->conv_thr < 0.0)
        throw HfgError(HFG_ERR_INVALID, "fock_conventional: no stored integrals (call hfg_store_integrals first)");
    if (!r.dD_tot || !r.dD_alpha || !r.J || !r.K_alpha || (r.unrestricted && (!r.dD_beta || !r.K_beta)))
        throw HfgError(HFG_ERR_INVALID, "fock: missing matrix pointer");
    const bool uhf     = r.unrestricted != 0;
    const long long N2 = e->mat_total;
    const int nspin    = uhf ? 3 : 2;
    cudaStream_t s     = e->stream;
    const double* src[3] = {r.dD_tot, r.dD_alpha, r.dD_beta};
    HFG_CUDA(cudaEventRecord(e->ev[1], s));
    for (int k = 0; k < nspin; ++k)
    {
        HFG_CUDA(cudaMemcpyAsync(e->d_dD[k].p, src[k], sizeof(double) * N2,
                                 r.device_pointers ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        HFG_CUDA(cudaMemsetAsync(e->d_acc[k].p, 0, sizeof(double) * N2, s));
    }
    int launches = 0;
    for (int qc = kNumQuartetClasses - 1; qc >= 0; --qc)
    {
        if (e->conv_n[qc] == 0)
            continue;
        StoredLaunch L {};
        L.list        = e->d_conv_list[qc].p;
        L.count       = e->conv_n[qc];
        L.store       = e->d_conv[qc].p;
        L.view        = base_view(e, false);
        L.view.pairs  = e->d_spairs.p;
        L.view.Dt     = e->d_dD[0].p;
        L.view.Da     = e->d_dD[1].p;
        L.view.Db     = e->d_dD[2].p;
        L.view.X      = e->d_acc[0].p;
        L.view.Ya     = e->d_acc[1].p;
        L.view.Yb     = e->d_acc[2].p;
        L.view.ao_thr = r.schwartz_threshold;
        L.uhf         = uhf;
        L.stream      = s;
        L.num_sms     = e->num_sms;
        HFG_CUDA(launch_stored(qc, L));
        ++launches;
    }
    double* outs[3] = {r.J, r.K_alpha, r.K_beta};
    for (int k = 0; k < nspin; ++k)
    {
        symmetrize_kernel<<<grid_for(N2, 256, e->num_sms), 256, 0, s>>>(e->d_acc[k].p, e->d_out[k].p, e->d_mat_off.p,
                                                                          e->d_mat_ld.p, e->nmol, N2);
        HFG_CUDA(cudaGetLastError());
        ++launches;
    }
    HFG_CUDA(cudaEventRecord(e->ev[6], s));
    for (int k = 0; k < nspin; ++k)
        HFG_CUDA(cudaMemcpyAsync(outs[k], e->d_out[k].p, sizeof(double) * N2,
                                 r.device_pointers ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    HFG_CUDA(cudaStreamSynchronize(s));
    if (st)
    {
        std::memset(st, 0, sizeof(*st));
        for (int qc = 0; qc < kNumQuartetClasses; ++qc)
        {
            st->quartets_fp64[qc] = e->conv_n[qc];
            st->form_fp64[qc]     = e->conv_n[qc] ? HFG_FORM_THREAD : 0;
        }
        st->kernel_launches = launches;
        float ms = 0.f;
        HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[1], e->ev[6]));
        st->ms_total = ms;
    }
}

// Device copies of molecule 0's basis and its shell pairs per pair class (once per engine).
static void upload_onee(hfg_engine* e)
{
    if (e->have_onee)
        return;
    if (e->nmol != 1)
        throw HfgError(HFG_ERR_INVALID, "one-electron integrals: the engine must hold exactly one molecule");
    const HostBasis& b = e->basis[0];
    const int ns       = static_cast<int>(b.l.size());
    std::vector<int> ints;
    for (const auto* v : {&b.l, &b.nprim, &b.prim_off, &b.ao_off, &b.norm_off}) ints.insert(ints.end(), v->begin(), v->end());
    std::vector<double> dbl;
    for (const auto* v : {&b.centers, &b.alpha, &b.coeff, &b.norms}) dbl.insert(dbl.end(), v->begin(), v->end());
    e->d_ob_int.upload(ints, e->stream);
    e->d_ob_dbl.upload(dbl, e->stream);
    const int* ip    = e->d_ob_int.p;
    const double* dp = e->d_ob_dbl.p;
    e->ob = OneeBasis {ip, ip + ns, ip + 2 * ns, ip + 3 * ns, ip + 4 * ns, dp, dp + 3 * ns, dp + 3 * ns + b.alpha.size(),
                       dp + 3 * ns + b.alpha.size() + b.coeff.size()};
    std::vector<std::vector<int2>> cls(kNumPairClasses);
    for (int s1 = 0; s1 < ns; ++s1)
        for (int s2 = 0; s2 <= s1; ++s2)
        {
            int a = s1, c = s2;
            if (b.l[c] > b.l[a])
                std::swap(a, c);
            cls[pair_class(b.l[a], b.l[c])].push_back(make_int2(a, c));
        }
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        e->d_ob_pairs[pc].upload(cls[pc], e->stream);
        e->ob_npairs[pc] = static_cast<int>(cls[pc].size());
    }
    HFG_CUDA(cudaStreamSynchronize(e->stream)); // the host vectors die here
    e->have_onee = true;
}

static void upload_nuclei(hfg_engine* e, int natom, const int* Z, const double* xyz)
{
    std::vector<double4> nuc(natom);
    for (int a = 0; a < natom; ++a) nuc[a] = make_double4(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2], static_cast<double>(Z[a]));
    e->d_nuc.upload(nuc, e->stream);
    HFG_CUDA(cudaStreamSynchronize(e->stream)); // the host vector dies here
}

// IntegralEngine::overlapMatrix / kineticMatrix / nuclearAttractionMatrix (src/IntegralEngine.cpp:78-368) on
// the device: S, T, V (n x n column-major, device pointers), FP64.
void one_electron_device(hfg_engine* e, int natom, const int* Z, const double* xyz, double* S, double* T, double* V)
{
    upload_onee(e);
    upload_nuclei(e, natom, Z, xyz);
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        OneeLaunch L {};
        L.pairs      = e->d_ob_pairs[pc].p;
        L.npairs     = e->ob_npairs[pc];
        L.basis      = e->ob;
        L.nuc        = e->d_nuc.p;
        L.natom      = natom;
        L.n          = e->mols[0].nao;
        L.boys_slice = e->d_boys64[pair_class_l1(pc) + pair_class_l2(pc)].p;
        L.S          = S;
        L.T          = T;
        L.V          = V;
        L.stream     = e->stream;
        L.num_sms    = e->num_sms;
        HFG_CUDA(launch_one_electron(pc, L));
    }
}

// One-electron part of the gradient on the device: sum D d(T + V)/dX - W dS/dX added into the device array
// grad (natom x 3); D (total density) and W (energy-weighted density) are device pointers.
static void gradient_one_electron_device(hfg_engine* e, const std::vector<int>& shell_atom, int natom, const int* Z,
                                         const double* xyz, const double* D, const double* W, double* grad)
{
    upload_onee(e);
    upload_nuclei(e, natom, Z, xyz);
    e->d_shell_atom1.upload(shell_atom, e->stream);
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        OneeLaunch L {};
        L.pairs      = e->d_ob_pairs[pc].p;
        L.npairs     = e->ob_npairs[pc];
        L.basis      = e->ob;
        L.nuc        = e->d_nuc.p;
        L.natom      = natom;
        L.n          = e->mols[0].nao;
        L.boys_slice = e->d_boys64[pair_class_l1(pc) + pair_class_l2(pc) + 2].p;
        L.D          = D;
        L.W          = W;
        L.shell_atom = e->d_shell_atom1.p;
        L.grad       = grad;
        L.stream     = e->stream;
        L.num_sms    = e->num_sms;
        HFG_CUDA(launch_one_electron_grad(pc, L));
    }
    HFG_CUDA(cudaStreamSynchronize(e->stream)); // shell_atom belongs to the caller
}

// Shell -> atom from the shell centres (a shell sits on the nucleus with the same coordinates).
static std::vector<int> shell_atoms(const hfg_engine* e, int natom, const double* xyz)
{
    const auto& hb = e->basis[0];
    std::vector<int> shell_atom(hb.l.size(), -1);
    for (size_t sh = 0; sh < hb.l.size(); ++sh)
    {
        for (int a = 0; a < natom; ++a)
            if (hb.centers[3 * sh] == xyz[3 * a] && hb.centers[3 * sh + 1] == xyz[3 * a + 1] &&
                hb.centers[3 * sh + 2] == xyz[3 * a + 2])
            {
                shell_atom[sh] = a;
                break;
            }
        if (shell_atom[sh] < 0)
            throw HfgError(HFG_ERR_INVALID, "gradient: a shell centre matches no nucleus");
    }
    return shell_atom;
}

const hfg_basis* engine_basis(const hfg_engine* e)
{
    return (e && e->nmol == 1) ? &e->basis[0].view : nullptr;
}

void engine_set_error(hfg_engine* e, const std::string& msg)
{
    if (e)
        e->last_error = msg;
}

// Gradient records per primitive pair (same order as the forward tables): a, b and the 1-D Hermite
// tables E[i][j][t] up to (l1+1, l2+1) of the three axes.
static void build_grad_tables(hfg_engine* e)
{
    if (e->have_gtab)
        return;
    std::vector<std::vector<double>> tab(kNumPairClasses);
    for (size_t k = 0; k < e->pairs.size(); ++k)
    {
        const PairRec& pr = e->pairs[k];
        const int pc = e->pair_class_of[k];
        const HostBasis& b = e->basis[pr.mol];
        const int l1 = b.l[pr.sh1], l2 = b.l[pr.sh2];
        const int stride = g_stride(l1, l2), n1 = g1d_size(l1, l2);
        const int pp_off = e->orig_off[k]; // unscreened pack-order layout
        if (tab[pc].size() < static_cast<size_t>(pp_off + e->npp_full[k]) * stride)
            tab[pc].resize(static_cast<size_t>(pp_off + e->npp_full[k]) * stride, 0.0);
        const double* A = &b.centers[3 * pr.sh1];
        const double* B = &b.centers[3 * pr.sh2];
        int idx = 0;
        for (int pa = 0; pa < b.nprim[pr.sh1]; ++pa)
            for (int pb = 0; pb < b.nprim[pr.sh2]; ++pb, ++idx)
            {
                const double aa = b.alpha[b.prim_off[pr.sh1] + pa], ab = b.alpha[b.prim_off[pr.sh2] + pb];
                const double p = aa + ab, ip = 1.0 / p, h = 0.5 * ip;
                double* rec = &tab[pc][static_cast<size_t>(pp_off + idx) * stride];
                rec[0] = aa;
                rec[1] = ab;
                for (int ax = 0; ax < 3; ++ax)
                {
                    const double P = (aa * A[ax] + ab * B[ax]) * ip, PA = P - A[ax], PB = P - B[ax];
                    double* E = rec + 2 + ax * n1;
                    auto at = [&](int i, int j, int t) -> double& { return E[(i * (l2 + 2) + j) * (l1 + l2 + 3) + t]; };
                    at(0, 0, 0) = 1.0;
                    for (int i = 0; i <= l1 + 1; ++i)
                        for (int j = 0; j <= l2 + 1; ++j)
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
                                    v += X * at(pi, pj, t);
                                if (t >= 1)
                                    v += h * at(pi, pj, t - 1);
                                if (t + 1 <= pi + pj)
                                    v += (t + 1) * at(pi, pj, t + 1);
                                at(i, j, t) = v;
                            }
                        }
                }
            }
    }
    for (int pc = 0; pc < kNumPairClasses; ++pc)
    {
        e->d_gtab[pc].upload(tab[pc], e->stream);
        e->d_gtab32[pc].upload(std::vector<float>(tab[pc].begin(), tab[pc].end()), e->stream);
    }
    HFG_CUDA(cudaStreamSynchronize(e->stream));
    e->have_gtab = true;
}

// Two-electron part of the nuclear gradient on the device (eri_grad.cuh) for the densities in
// d_dD[0..2] (total, alpha, beta); adds into grad[3*natom] (host).  mixed: quartets whose bound
// Q_ab Q_cd max|D| is below `cutoff` run in the FP32 kernels (the Fock build's split), the rest in FP64;
// every contribution accumulates in FP64.  Returns the device milliseconds.
static double gradient_two_electron(hfg_engine* e, const std::vector<int>& shell_atom, int natom, bool uhf,
                                    double sthr, double dthr, bool mixed, double cutoff, double* grad)
{
    cudaStream_t s = e->stream;
    build_grad_tables(e);
    e->d_shell_atom.upload(shell_atom, s);
    e->d_grad.alloc(static_cast<size_t>(3) * natom);
    HFG_CUDA(cudaMemsetAsync(e->d_grad.p, 0, sizeof(double) * 3 * natom, s));
    const long long N2 = e->mat_total;
    if (mixed)
        for (int k = 0; k < 3; ++k)
        {
            if (!e->d_dDf[k].p)
            {
                invalidate_graph(e);
                e->d_dDf[k].alloc(N2);
            }
            to_float_kernel<<<grid_for(N2, 256, e->num_sms), 256, 0, s>>>(e->d_dD[k].p, e->d_dDf[k].p, N2);
            HFG_CUDA(cudaGetLastError());
        }
    size_lists(e, sthr, mixed);
    build_lists(e, uhf, mixed, sthr, dthr, cutoff);
    GradView v[2] {};
    for (int prec = 0; prec < (mixed ? 2 : 1); ++prec)
    {
        GradView& g = v[prec];
        g.pairs     = e->d_gspairs.p;
        for (int pc = 0; pc < kNumPairClasses; ++pc)
        {
            g.pptab[pc] = prec ? static_cast<const void*>(e->d_pptab32_full[pc].p) : e->d_pptab64_full[pc].p;
            g.gtab[pc]  = prec ? static_cast<const void*>(e->d_gtab32[pc].p) : e->d_gtab[pc].p;
        }
        g.Dt = prec ? static_cast<const void*>(e->d_dDf[0].p) : e->d_dD[0].p;
        g.Da = prec ? static_cast<const void*>(e->d_dDf[1].p) : e->d_dD[1].p;
        g.Db = uhf ? (prec ? static_cast<const void*>(e->d_dDf[2].p) : e->d_dD[2].p) : g.Da;
        g.n          = e->mols[0].nao;
        g.shell_atom = e->d_shell_atom.p;
        g.grad       = e->d_grad.p;
    }
    HFG_CUDA(cudaEventRecord(e->ev[6], s));
    for (int prec = 0; prec < (mixed ? 2 : 1); ++prec)
        for (int qc = kNumQuartetClasses - 1; qc >= 0; --qc)
        {
            const unsigned long long n = e->h_counts[2 * qc + prec];
            if (n == 0)
                continue;
            const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
            const int P2 = qc - P1 * (P1 + 1) / 2;
            const int L  = pair_class_l1(P1) + pair_class_l2(P1) + pair_class_l1(P2) + pair_class_l2(P2);
            const void* slice = prec ? static_cast<const void*>(e->d_boys32[L + 1].p) : e->d_boys64[L + 1].p;
            GradLaunch g {e->d_list[qc][prec].p, n, v[prec], slice, e->d_tables.p, s, e->num_sms, prec == 1, e->grad_group_only};
            HFG_CUDA(launch_grad(qc, g));
        }
    HFG_CUDA(cudaEventRecord(e->ev[7], s));
    std::vector<double> g(static_cast<size_t>(3) * natom);
    HFG_CUDA(cudaMemcpyAsync(g.data(), e->d_grad.p, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, s));
    HFG_CUDA(cudaStreamSynchronize(s));
    for (size_t k = 0; k < g.size(); ++k) grad[k] += g[k];
    float ms = 0.f;
    HFG_CUDA(cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]));
    return ms;
}

// Enqueues one device-pointer Fock build on the engine stream without any host synchronisation, for a
// caller that captures it into its own CUDA graph (the SCF iteration graph).  The build must have run
// eagerly once with the same precision, spin case and Schwartz threshold (forms tuned, lists sized,
// buffers allocated).  The list lengths land in pinned memory; engine_check_counts reads them after the
// graph has run.  Returns the kernel launches enqueued; throws like the other engine calls.
int engine_enqueue_fock(hfg_engine* e, const hfg_fock_request& r)
{
    if (!r.device_pointers)
        throw HfgError(HFG_ERR_INVALID, "fock: a captured build needs device pointers");
    if (!e->have_Q || e->cap_thr != r.schwartz_threshold || (r.precision == HFG_PRECISION_MIXED && !e->cap_mixed) ||
        !e->h_counts_pin)
        throw HfgError(HFG_ERR_INVALID, "fock: a captured build needs an eager build with the same request first");
    int forms[kNumQuartetClasses][2] {};
    double unused = 0.0;
    return enqueue_build(e, r, true, forms, &unused);
}

// Allocates what a captured build writes to on the host (before any capture begins).
void engine_prepare_capture(hfg_engine* e)
{
    if (!e->h_counts_pin)
        HFG_CUDA(cudaMallocHost(&e->h_counts_pin, sizeof(unsigned long long) * (4 * kNumQuartetClasses + 1)));
}

// After a graph holding engine_enqueue_fock has run (and the stream is synchronised): the list-overflow
// check and the survivor counts of that build.
void engine_check_counts(hfg_engine* e, bool mixed)
{
    const int ncnt = kNumQuartetClasses * 2;
    e->h_counts.assign(e->h_counts_pin, e->h_counts_pin + 2 * ncnt + 1);
    for (int qc = 0; qc < kNumQuartetClasses; ++qc)
        if (e->h_counts[2 * qc] > e->cap[qc] || e->h_counts[2 * qc + 1] > e->cap[qc])
            throw HfgError(HFG_ERR_OVERFLOW, "fock: quartet list overflow");
    e->last_valid = true;
    e->last_mixed = mixed ? 1 : 0;
}

// The engine-call guard for host code outside this file: runs f, maps engine exceptions to HFG codes.
int engine_guarded(hfg_engine* e, const std::function<void()>& f)
{
    try
    {
        f();
        return HFG_OK;
    }
    catch (const HfgError& x)
    {
        e->last_error = x.what();
        return x.code;
    }
    catch (const std::bad_alloc&)
    {
        e->last_error = "host allocation failed";
        return HFG_ERR_NOMEM;
    }
    catch (const std::exception& x)
    {
        e->last_error = x.what();
        return HFG_ERR_INVALID;
    }
}

void engine_store_scf_state(hfg_engine* e, const double* Da, const double* Db, const double* W, bool uhf)
{
    const size_t N2 = static_cast<size_t>(e->mols[0].nao) * e->mols[0].nao;
    e->scf_Da.assign(Da, Da + N2);
    e->scf_Db.assign(Db, Db + N2);
    e->scf_W.assign(W, W + N2);
    e->scf_uhf   = uhf;
    e->scf_valid = true;
}

// Work model (per primitive quartet of class (la lb|lc ld), L = sum): the R recursion (one FMA per
// R^n_tuv), the ket and bra Hermite->Cartesian transforms with dense Hermite blocks, scaling and Boys;
// per shell quartet the digestion FMAs (RHF: 2 J + 4 K per integral; UHF adds 4 K_beta).
double flops_per_prim_quartet(int qc)
{
    const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
    const int P2 = qc - P1 * (P1 + 1) / 2;
    const int la = pair_class_l1(P1), lb = pair_class_l2(P1), lc = pair_class_l1(P2), ld = pair_class_l2(P2);
    const int L = la + lb + lc + ld;
    const double nab = ncart(la) * ncart(lb), ncd = ncart(lc) * ncart(ld);
    const double hab = nherm(la + lb), hcd = nherm(lc + ld);
    const double cL4 = (L + 1.0) * (L + 2.0) * (L + 3.0) * (L + 4.0) / 24.0;
    return 2.0 * cL4 + 2.0 * hab * ncd * hcd + 2.0 * nab * ncd * hab + 2.0 * nab * ncd + (2.0 * (L + 1) + 10.0);
}

double flops_per_quartet_digest(int qc, bool uhf)
{
    const int P1 = [&] { int p = 0; while ((p + 1) * (p + 2) / 2 <= qc) ++p; return p; }();
    const int P2 = qc - P1 * (P1 + 1) / 2;
    const double n = ncart(pair_class_l1(P1)) * ncart(pair_class_l2(P1)) * ncart(pair_class_l1(P2)) * ncart(pair_class_l2(P2));
    return (uhf ? 20.0 : 12.0) * n;
}
} // namespace hfg


// ------------------------------------------------------------------------------------------------
// Allocation-free shell-quartet block.  hfg_eri_block grows a device buffer for every request and
// frees it afterwards, and cudaFree synchronises the whole device; callers that must not allocate or
// free device memory per request (a process that runs under a fixed device-memory budget once its
// engine exists, or a pipeline whose other streams must not be stalled by an implicit device-wide
// synchronisation) use hfg_eri_block_noalloc instead.  Its scratch -- the one-entry quartet list, the
// list length and the output block -- lives in this file-scope device array; every GPU that loads the
// library holds it until the process exits.
// ------------------------------------------------------------------------------------------------
namespace hfg
{
namespace
{
constexpr size_t kNoAllocScratchBytes = 16384;         // stated maximum
constexpr size_t kNoAllocBlockOffset  = 256;           // Quartet at 0, count at 8, block from 256
constexpr size_t kNoAllocMaxBlock     = (kNoAllocScratchBytes - kNoAllocBlockOffset) / sizeof(double); // 2016 values
static __device__ __align__(256) unsigned char hfg_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up once per device, with that device
// current; the host-side symbol itself is not a device address).
void* noalloc_scratch(int device)
{
    if (device < 0 || device >= kMaxDevices)
        throw HfgError(HFG_ERR_INVALID, "hfg_eri_block_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device])
    {
        void* ptr = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&ptr, hfg_noalloc_scratch);
        if (rc != cudaSuccess || ptr == nullptr)
            throw HfgError(HFG_ERR_CUDA, std::string("hfg_eri_block_noalloc: cudaGetSymbolAddress failed: ") +
                                             cudaGetErrorString(rc));
        g_noalloc_ptr[device] = ptr;
    }
    return g_noalloc_ptr[device];
}
} // namespace
} // namespace hfg
// ------------------------------------------------------------------------------------------------
// C ABI.
// ------------------------------------------------------------------------------------------------
using hfg::HfgError;

template <typename F> static int guarded(hfg_engine* e, F&& f)
{
    try
    {
        f();
        return HFG_OK;
    }
    catch (const HfgError& x)
    {
        if (e)
            e->last_error = x.what();
        else
            hfg::g_create_error = x.what();
        return x.code;
    }
    catch (const std::bad_alloc&)
    {
        if (e)
            e->last_error = "host allocation failed";
        return HFG_ERR_NOMEM;
    }
    catch (const std::exception& x)
    {
        if (e)
            e->last_error = x.what();
        else
            hfg::g_create_error = x.what();
        return HFG_ERR_INVALID;
    }
}

extern "C" {

const char* hfg_version(void) { return "hfgpu 0.1 (sm_103a)"; }

int hfg_create_batch(const hfg_basis* bases, int nmol, int device, hfg_engine** out)
{
    if (!out || !bases || nmol <= 0)
    {
        hfg::g_create_error = "hfg_create: null argument or empty batch";
        return HFG_ERR_INVALID;
    }
    *out = nullptr;
    auto e = std::make_unique<hfg_engine>();
    const int rc = guarded(nullptr, [&] {
        int ndev = 0;
        HFG_CUDA(cudaGetDeviceCount(&ndev));
        if (device < 0 || device >= ndev)
            throw HfgError(HFG_ERR_INVALID, "hfg_create: device index out of range");
        e->device = device;
        HFG_CUDA(cudaSetDevice(device));
        HFG_CUDA(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device));
        HFG_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        HFG_CUDA(cudaStreamCreateWithFlags(&e->stream2, cudaStreamNonBlocking));
        for (auto& ev : e->ev) HFG_CUDA(cudaEventCreate(&ev));
        for (auto& ev : e->ev2) HFG_CUDA(cudaEventCreate(&ev));
        e->nmol = nmol;
        e->basis.resize(nmol);
        long long mat = 0, smax = 0;
        int sh = 0;
        for (int m = 0; m < nmol; ++m)
        {
            hfg::validate_and_copy(bases[m], e->basis[m]);
            hfg::MolInfo mi {};
            mi.nshells  = bases[m].nshells;
            mi.nao      = bases[m].nao;
            mi.sh_off   = sh;
            mi.mat_off  = mat;
            mi.smax_off = smax;
            e->mols.push_back(mi);
            mat += static_cast<long long>(mi.nao) * mi.nao;
            smax += static_cast<long long>(mi.nshells) * mi.nshells;
            sh += mi.nshells;
        }
        e->mat_total     = mat;
        e->smax_total    = smax;
        e->nshells_total = sh;
        hfg::pack_molecules(e.get());
    });
    if (rc != HFG_OK)
    {
        if (e->stream)
        {
            cudaStreamDestroy(e->stream);
            e->stream = nullptr;
        }
        if (e->stream2)
        {
            cudaStreamDestroy(e->stream2);
            e->stream2 = nullptr;
        }
        return rc;
    }
    *out = e.release();
    return HFG_OK;
}

int hfg_create(const hfg_basis* basis, int device, hfg_engine** out) { return hfg_create_batch(basis, 1, device, out); }

void hfg_destroy(hfg_engine* e)
{
    if (!e)
        return;
    cudaSetDevice(e->device);
    if (e->stream)
        cudaStreamSynchronize(e->stream);
    hfg::invalidate_graph(e);
    if (e->h_counts_pin)
        cudaFreeHost(e->h_counts_pin);
    for (auto& ev : e->ev)
        if (ev)
            cudaEventDestroy(ev);
    for (auto& ev : e->tune_ev)
        if (ev)
            cudaEventDestroy(ev);
    for (auto& ev : e->ev2)
        if (ev)
            cudaEventDestroy(ev);
    if (e->stream2)
    {
        cudaStreamSynchronize(e->stream2);
        cudaStreamDestroy(e->stream2);
    }
    if (e->stream)
        cudaStreamDestroy(e->stream);
    delete e;
}

const char* hfg_last_error(const hfg_engine* e) { return e ? e->last_error.c_str() : hfg::g_create_error.c_str(); }

void* hfg_stream(hfg_engine* e) { return e ? static_cast<void*>(e->stream) : nullptr; }

int hfg_schwartz(hfg_engine* e, double* Q)
{
    if (!e || !Q)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        if (!e->have_Q)
        {
            hfg::compute_schwartz(e);
            hfg::sort_classes(e);
        }
        std::vector<long long> qoff(e->nmol, 0);
        long long acc = 0;
        for (int m = 0; m < e->nmol; ++m)
        {
            qoff[m] = acc;
            acc += static_cast<long long>(e->mols[m].nshells) * e->mols[m].nshells;
        }
        std::fill(Q, Q + acc, 0.0);
        for (size_t k = 0; k < e->pairs.size(); ++k)
        {
            const auto& p = e->pairs[k];
            const int ns  = e->mols[p.mol].nshells;
            Q[qoff[p.mol] + p.sh1 + static_cast<long long>(p.sh2) * ns] = e->Qpair[k];
            Q[qoff[p.mol] + p.sh2 + static_cast<long long>(p.sh1) * ns] = e->Qpair[k];
        }
    });
}

int hfg_set_primitive_threshold(hfg_engine* e, double threshold)
{
    if (!e)
        return HFG_ERR_INVALID;
    if (!(threshold >= 0.0) || !std::isfinite(threshold))
    {
        e->last_error = "set_primitive_threshold: threshold must be finite and >= 0";
        return HFG_ERR_INVALID;
    }
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        e->prim_thr = threshold;
        if (e->have_Q)
            hfg::sort_classes(e); // re-screens, re-sorts and re-uploads the tables
    });
}

int hfg_set_schwartz(hfg_engine* e, const double* Q)
{
    if (!e || !Q)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        e->Qpair.assign(e->pairs.size(), 0.0);
        long long acc = 0;
        std::vector<long long> qoff(e->nmol, 0);
        for (int m = 0; m < e->nmol; ++m)
        {
            qoff[m] = acc;
            acc += static_cast<long long>(e->mols[m].nshells) * e->mols[m].nshells;
        }
        for (size_t k = 0; k < e->pairs.size(); ++k)
        {
            const auto& p = e->pairs[k];
            const int ns  = e->mols[p.mol].nshells;
            // The reference reads Q(a, b) with a >= b (SCF.cpp:606); take that element.
            const int a = std::max(p.sh1, p.sh2), b = std::min(p.sh1, p.sh2);
            const double v = Q[qoff[p.mol] + a + static_cast<long long>(b) * ns];
            if (!(v >= 0.0) || !std::isfinite(v))
                throw HfgError(HFG_ERR_INVALID, "hfg_set_schwartz: Q must be finite and >= 0");
            e->Qpair[k] = v;
        }
        hfg::sort_classes(e);
    });
}

int hfg_fock_direct(hfg_engine* e, const hfg_fock_request* req, hfg_fock_stats* stats)
{
    if (!e || !req)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        hfg::fock_direct(e, *req, stats);
    });
}

int hfg_store_integrals(hfg_engine* e, double schwartz_threshold, size_t* bytes)
{
    if (!e)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        hfg::store_integrals(e, schwartz_threshold, bytes);
    });
}

int hfg_fock_conventional(hfg_engine* e, const hfg_fock_request* req, hfg_fock_stats* stats)
{
    if (!e || !req)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        hfg::fock_conventional(e, *req, stats);
    });
}

int hfg_set_kernel_form(hfg_engine* e, int qclass, int fp32, int form)
{
    if (!e)
        return HFG_ERR_INVALID;
    if (qclass < -1 || qclass >= hfg::kNumQuartetClasses || (fp32 != 0 && fp32 != 1) || form < HFG_FORM_AUTO ||
        form > HFG_FORM_CHUNK)
    {
        e->last_error = "set_kernel_form: class, precision or form out of range";
        return HFG_ERR_INVALID;
    }
    const int lo = qclass < 0 ? 0 : qclass, hi = qclass < 0 ? hfg::kNumQuartetClasses : qclass + 1;
    hfg::invalidate_graph(e); // a captured build holds the old forms
    for (int qc = lo; qc < hi; ++qc)
    {
        const bool ok = form == HFG_FORM_AUTO || ((hfg::class_form_mask(qc, fp32 != 0) >> form) & 1u);
        if (!ok)
        {
            if (qclass >= 0)
            {
                e->last_error = "set_kernel_form: form not compiled for this class and precision";
                return HFG_ERR_UNSUPPORTED;
            }
            e->form_set[qc][fp32] = HFG_FORM_AUTO;
            continue;
        }
        e->form_set[qc][fp32] = form;
        if (form == HFG_FORM_AUTO)
            e->form_pick[qc][fp32][0] = e->form_pick[qc][fp32][1] = 0;
    }
    return HFG_OK;
}

int hfg_set_precision_overlap(hfg_engine* e, int on, double share)
{
    if (!e)
        return HFG_ERR_INVALID;
    if (!(share > 0.0 && share <= 1.0))
    {
        e->last_error = "set_precision_overlap: share must be in (0, 1]";
        return HFG_ERR_INVALID;
    }
    hfg::invalidate_graph(e);
    e->overlap       = on != 0;
    e->overlap_share   = static_cast<float>(share);
    e->overlap_share32 = static_cast<float>(share);
    return HFG_OK;
}

int hfg_set_precision_shares(hfg_engine* e, double share_fp64, double share_fp32)
{
    if (!e)
        return HFG_ERR_INVALID;
    if (!(share_fp64 > 0.0 && share_fp64 <= 1.0) || !(share_fp32 > 0.0 && share_fp32 <= 1.0))
    {
        e->last_error = "set_precision_shares: shares must be in (0, 1]";
        return HFG_ERR_INVALID;
    }
    hfg::invalidate_graph(e);
    e->overlap_share   = static_cast<float>(share_fp64);
    e->overlap_share32 = static_cast<float>(share_fp32);
    return HFG_OK;
}

int hfg_set_persistent(hfg_engine* e, int on)
{
    if (!e)
        return HFG_ERR_INVALID;
    hfg::invalidate_graph(e);
    e->persistent = on != 0;
    return HFG_OK;
}

int hfg_set_autotune(hfg_engine* e, int on)
{
    if (!e)
        return HFG_ERR_INVALID;
    e->autotune = on != 0;
    return HFG_OK;
}

int hfg_set_gradient_form(hfg_engine* e, int group_only)
{
    if (!e)
        return HFG_ERR_INVALID;
    e->grad_group_only = group_only != 0;
    return HFG_OK;
}

int hfg_set_graph_mode(hfg_engine* e, int on)
{
    if (!e)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        e->graph_mode = on != 0;
        if (!e->graph_mode)
            hfg::invalidate_graph(e);
    });
}

int hfg_kernel_forms(hfg_engine* e, int fp32, int unrestricted, int* forms, unsigned* available)
{
    if (!e || !forms || (fp32 != 0 && fp32 != 1))
        return HFG_ERR_INVALID;
    for (int qc = 0; qc < hfg::kNumQuartetClasses; ++qc)
    {
        const int set = e->form_set[qc][fp32];
        forms[qc]     = set != 0 ? set : e->form_pick[qc][fp32][unrestricted ? 1 : 0];
        if (available)
            available[qc] = hfg::class_form_mask(qc, fp32 != 0);
    }
    return HFG_OK;
}

int hfg_survivors(hfg_engine* e, int* quartets, long long cap, long long* count)
{
    if (!e || !count)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        if (!e->last_valid)
            throw HfgError(HFG_ERR_INVALID, "hfg_survivors: no Fock build yet");
        HFG_CUDA(cudaSetDevice(e->device));
        std::vector<std::array<int, 5>> all;
        for (int qc = 0; qc < hfg::kNumQuartetClasses; ++qc)
            for (int prec = 0; prec < 2; ++prec)
            {
                const unsigned long long n = e->h_counts[2 * qc + prec];
                if (n == 0)
                    continue;
                std::vector<hfg::Quartet> q(n);
                HFG_CUDA(cudaMemcpy(q.data(), e->d_list[qc][prec].p, sizeof(hfg::Quartet) * n, cudaMemcpyDeviceToHost));
                for (const auto& x : q)
                {
                    const auto& P = e->pairs[e->spair_id[x.bra]];
                    const auto& K = e->pairs[e->spair_id[x.ket]];
                    int a = std::max(P.sh1, P.sh2), b = std::min(P.sh1, P.sh2);
                    int c = std::max(K.sh1, K.sh2), d = std::min(K.sh1, K.sh2);
                    const long long ab = static_cast<long long>(a) * (a + 1) / 2 + b;
                    const long long cd = static_cast<long long>(c) * (c + 1) / 2 + d;
                    if (ab < cd)
                    {
                        std::swap(a, c);
                        std::swap(b, d);
                    }
                    all.push_back({P.mol, a, b, c, d});
                }
            }
        std::sort(all.begin(), all.end());
        *count = static_cast<long long>(all.size());
        if (quartets)
            for (long long k = 0; k < std::min<long long>(cap, *count); ++k)
                for (int j = 0; j < 4; ++j) quartets[4 * k + j] = all[k][j + 1];
    });
}

int hfg_gradient(hfg_engine* e, const hfg_gradient_request* r, double* grad, double* ms_two_electron)
{
    if (!e || !r || !grad || r->natom <= 0 || !r->Z || !r->xyz)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        if (e->nmol != 1)
            throw HfgError(HFG_ERR_INVALID, "hfg_gradient: the engine must hold exactly one molecule");
        if (r->precision != HFG_PRECISION_FP64 && r->precision != HFG_PRECISION_MIXED)
            throw HfgError(HFG_ERR_INVALID, "hfg_gradient: unknown precision mode");
        if (r->precision == HFG_PRECISION_MIXED && !(r->fp32_cutoff >= 0.0 && std::isfinite(r->fp32_cutoff)))
            throw HfgError(HFG_ERR_INVALID, "hfg_gradient: fp32_cutoff must be finite and >= 0");
        HFG_CUDA(cudaSetDevice(e->device));
        const int n = e->mols[0].nao;
        const size_t N2 = static_cast<size_t>(n) * n;
        const bool use_last = r->D_alpha == nullptr;
        if (use_last && !e->scf_valid)
            throw HfgError(HFG_ERR_INVALID, "hfg_gradient: no densities given and no SCF run on this engine");
        const bool uhf = use_last ? e->scf_uhf : (r->unrestricted != 0);
        const double* Da = use_last ? e->scf_Da.data() : r->D_alpha;
        const double* Db = use_last ? e->scf_Db.data() : (uhf ? r->D_beta : r->D_alpha);
        const double* W  = use_last ? e->scf_W.data() : r->W;
        if (!Db || !W)
            throw HfgError(HFG_ERR_INVALID, "hfg_gradient: missing D_beta or W");
        const std::vector<int> shell_atom = hfg::shell_atoms(e, r->natom, r->xyz);
        std::vector<double> Dt(N2);
        for (size_t k = 0; k < N2; ++k) Dt[k] = Da[k] + Db[k];
        for (int k = 0; k < 3; ++k)
        {
            e->d_dD[k].alloc(N2);
            e->d_smax[k].alloc(e->smax_total);
        }
        if (!e->have_Q)
        {
            hfg::compute_schwartz(e);
            hfg::sort_classes(e);
        }
        HFG_CUDA(cudaMemcpyAsync(e->d_dD[0].p, Dt.data(), sizeof(double) * N2, cudaMemcpyHostToDevice, e->stream));
        HFG_CUDA(cudaMemcpyAsync(e->d_dD[1].p, Da, sizeof(double) * N2, cudaMemcpyHostToDevice, e->stream));
        HFG_CUDA(cudaMemcpyAsync(e->d_dD[2].p, Db, sizeof(double) * N2, cudaMemcpyHostToDevice, e->stream));
        std::fill(grad, grad + 3 * r->natom, 0.0);
        const double ms = hfg::gradient_two_electron(e, shell_atom, r->natom, true, r->schwartz_threshold,
                                                     r->density_threshold, r->precision == HFG_PRECISION_MIXED,
                                                     r->fp32_cutoff, grad);
        if (ms_two_electron)
            *ms_two_electron = ms;
        e->last_valid = false; // the lists now hold the gradient's quartets
        // Nuclear repulsion (src/Molecule.cpp:80-89 differentiated) on the host; the one-electron and overlap
        // parts on the device, with the total density still in d_dD[0].
        const int na = r->natom;
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < na; ++j)
            {
                if (i == j)
                    continue;
                double d[3], r2 = 0.0;
                for (int k = 0; k < 3; ++k)
                {
                    d[k] = r->xyz[3 * i + k] - r->xyz[3 * j + k];
                    r2 += d[k] * d[k];
                }
                const double f = static_cast<double>(r->Z[i] * r->Z[j]) / (r2 * std::sqrt(r2));
                for (int k = 0; k < 3; ++k) grad[3 * i + k] -= f * d[k];
            }
        e->d_W.alloc(N2);
        HFG_CUDA(cudaMemcpyAsync(e->d_W.p, W, sizeof(double) * N2, cudaMemcpyHostToDevice, e->stream));
        HFG_CUDA(cudaMemsetAsync(e->d_grad.p, 0, sizeof(double) * 3 * na, e->stream));
        hfg::gradient_one_electron_device(e, shell_atom, na, r->Z, r->xyz, e->d_dD[0].p, e->d_W.p, e->d_grad.p);
        std::vector<double> g1(static_cast<size_t>(3) * na);
        HFG_CUDA(cudaMemcpyAsync(g1.data(), e->d_grad.p, sizeof(double) * g1.size(), cudaMemcpyDeviceToHost, e->stream));
        HFG_CUDA(cudaStreamSynchronize(e->stream));
        for (size_t k = 0; k < g1.size(); ++k) grad[k] += g1[k];
    });
}

int hfg_one_electron_gpu(hfg_engine* e, int natom, const int* Z, const double* xyz, double* S, double* T, double* V)
{
    if (!e || natom <= 0 || !Z || !xyz || !S || !T || !V)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        if (e->nmol != 1)
            throw HfgError(HFG_ERR_INVALID, "hfg_one_electron_gpu: the engine must hold exactly one molecule");
        const size_t N2 = static_cast<size_t>(e->mols[0].nao) * e->mols[0].nao;
        hfg::DevBuf<double> d;
        d.alloc(3 * N2);
        hfg::one_electron_device(e, natom, Z, xyz, d.p, d.p + N2, d.p + 2 * N2);
        HFG_CUDA(cudaMemcpyAsync(S, d.p, sizeof(double) * N2, cudaMemcpyDeviceToHost, e->stream));
        HFG_CUDA(cudaMemcpyAsync(T, d.p + N2, sizeof(double) * N2, cudaMemcpyDeviceToHost, e->stream));
        HFG_CUDA(cudaMemcpyAsync(V, d.p + 2 * N2, sizeof(double) * N2, cudaMemcpyDeviceToHost, e->stream));
        HFG_CUDA(cudaStreamSynchronize(e->stream));
    });
}

int hfg_gradient_one_electron_gpu(hfg_engine* e, int natom, const int* Z, const double* xyz, const double* D,
                                  const double* W, double* grad)
{
    if (!e || natom <= 0 || !Z || !xyz || !D || !W || !grad)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        if (e->nmol != 1)
            throw HfgError(HFG_ERR_INVALID, "hfg_gradient_one_electron_gpu: the engine must hold exactly one molecule");
        const std::vector<int> shell_atom = hfg::shell_atoms(e, natom, xyz);
        const size_t N2 = static_cast<size_t>(e->mols[0].nao) * e->mols[0].nao;
        hfg::DevBuf<double> d;
        d.alloc(2 * N2 + 3 * static_cast<size_t>(natom));
        HFG_CUDA(cudaMemcpyAsync(d.p, D, sizeof(double) * N2, cudaMemcpyHostToDevice, e->stream));
        HFG_CUDA(cudaMemcpyAsync(d.p + N2, W, sizeof(double) * N2, cudaMemcpyHostToDevice, e->stream));
        HFG_CUDA(cudaMemsetAsync(d.p + 2 * N2, 0, sizeof(double) * 3 * natom, e->stream));
        hfg::gradient_one_electron_device(e, shell_atom, natom, Z, xyz, d.p, d.p + N2, d.p + 2 * N2);
        std::vector<double> g1(static_cast<size_t>(3) * natom);
        HFG_CUDA(cudaMemcpyAsync(g1.data(), d.p + 2 * N2, sizeof(double) * g1.size(), cudaMemcpyDeviceToHost, e->stream));
        HFG_CUDA(cudaStreamSynchronize(e->stream));
        for (size_t k = 0; k < g1.size(); ++k) grad[k] += g1[k];
    });
}

int hfg_eri_block_noalloc(hfg_engine* e, int a, int b, int c, int d, double* out)
{
    if (!e || !out || e->nmol != 1)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        const int ns = e->mols[0].nshells;
        if (a < 0 || b < 0 || c < 0 || d < 0 || a >= ns || b >= ns || c >= ns || d >= ns)
            throw HfgError(HFG_ERR_INVALID, "hfg_eri_block_noalloc: shell index out of range");
        const auto& hb = e->basis[0];
        const int na = hfg::ncart(hb.l[a]), nb = hfg::ncart(hb.l[b]), nc = hfg::ncart(hb.l[c]), nd = hfg::ncart(hb.l[d]);
        const size_t nblk = static_cast<size_t>(na) * nb * nc * nd;
        if (nblk > hfg::kNoAllocMaxBlock)
            throw HfgError(HFG_ERR_INVALID, "hfg_eri_block_noalloc: block of " + std::to_string(nblk) +
                                                " values exceeds the scratch maximum of " +
                                                std::to_string(hfg::kNoAllocMaxBlock));
        unsigned char* scratch = static_cast<unsigned char*>(hfg::noalloc_scratch(e->device));
        auto pair_id = [&](int x, int y) { const int hi = std::max(x, y), lo = std::min(x, y); return hi * (hi + 1) / 2 + lo; };
        const int pb = pair_id(a, b), pk = pair_id(c, d);
        const int cb = e->pair_class_of[pb], ck = e->pair_class_of[pk];
        int bra = pb, ket = pk;
        if (cb < ck)
            std::swap(bra, ket);
        const int qc = hfg::qclass_of(cb, ck);
        const int P1 = std::max(cb, ck), P2 = std::min(cb, ck);
        // The one-entry list and its length: written fresh by every call (nothing accumulates in the
        // scratch; the kernel overwrites every value of the block).
        struct Head
        {
            hfg::Quartet q;
            unsigned long long n;
        } head {hfg::Quartet {static_cast<uint32_t>(bra), static_cast<uint32_t>(ket)}, 1ull};
        HFG_CUDA(cudaMemcpyAsync(scratch, &head, sizeof(head), cudaMemcpyHostToDevice, e->stream));
        hfg::ClassLaunch L {};
        L.list        = reinterpret_cast<const hfg::Quartet*>(scratch);
        L.count_dev   = reinterpret_cast<const unsigned long long*>(scratch + offsetof(Head, n));
        L.count_host  = 1;
        L.view        = hfg::base_view(e, false);
        L.view.store  = reinterpret_cast<double*>(scratch + hfg::kNoAllocBlockOffset);
        L.view.ao_thr = 0.0;
        L.boys_slice  = e->d_boys64[hfg::pair_class_l1(P1) + hfg::pair_class_l2(P1) + hfg::pair_class_l1(P2) +
                                   hfg::pair_class_l2(P2)].p;
        L.tables      = e->d_tables.p;
        L.stream      = e->stream;
        L.num_sms     = e->num_sms;
        HFG_CUDA(hfg::launch_class(qc, L));
        double blk[hfg::kNoAllocMaxBlock];
        HFG_CUDA(cudaMemcpyAsync(blk, scratch + hfg::kNoAllocBlockOffset, sizeof(double) * nblk, cudaMemcpyDeviceToHost,
                                 e->stream));
        HFG_CUDA(cudaStreamSynchronize(e->stream));
        const auto& B = e->pairs[bra];
        const auto& K = e->pairs[ket];
        const int n2 = hfg::ncart(hb.l[B.sh2]), n3 = hfg::ncart(hb.l[K.sh1]), n4 = hfg::ncart(hb.l[K.sh2]);
        const int sh[4] = {a, b, c, d};
        const bool swap_pairs = (bra != pb);
        const int p0 = swap_pairs ? 2 : 0, p1 = swap_pairs ? 0 : 2;
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j)
                for (int k = 0; k < nc; ++k)
                    for (int l = 0; l < nd; ++l)
                    {
                        const int cc[4] = {i, j, k, l};
                        int comp[4];
                        auto place = [&](int sa_, int sb_, const hfg::PairRec& pr, int* dst) {
                            const bool direct = (sh[sa_] == pr.sh1 && sh[sb_] == pr.sh2);
                            dst[0] = direct ? cc[sa_] : cc[sb_];
                            dst[1] = direct ? cc[sb_] : cc[sa_];
                        };
                        place(p0, p0 + 1, B, comp);
                        place(p1, p1 + 1, K, comp + 2);
                        out[((i * nb + j) * nc + k) * nd + l] = blk[((comp[0] * n2 + comp[1]) * n3 + comp[2]) * n4 + comp[3]];
                    }
    });
}

int hfg_eri_block(hfg_engine* e, int a, int b, int c, int d, double* out)
{
    if (!e || !out || e->nmol != 1)
        return HFG_ERR_INVALID;
    return guarded(e, [&] {
        HFG_CUDA(cudaSetDevice(e->device));
        const int ns = e->mols[0].nshells;
        if (a < 0 || b < 0 || c < 0 || d < 0 || a >= ns || b >= ns || c >= ns || d >= ns)
            throw HfgError(HFG_ERR_INVALID, "hfg_eri_block: shell index out of range");
        auto pair_id = [&](int x, int y) -> int {
            const int hi = std::max(x, y), lo = std::min(x, y);
            // pairs are generated in (s1 desc-major) order: s1 = 0.., s2 = 0..s1
            return hi * (hi + 1) / 2 + lo;
        };
        const int pb = pair_id(a, b), pk = pair_id(c, d);
        const int cb = e->pair_class_of[pb], ck = e->pair_class_of[pk];
        int bra = pb, ket = pk;
        if (cb < ck)
            std::swap(bra, ket);
        const int qc = hfg::qclass_of(cb, ck);
        hfg::eval_store(e, qc, {hfg::Quartet {static_cast<uint32_t>(bra), static_cast<uint32_t>(ket)}});
        const auto& B = e->pairs[bra];
        const auto& K = e->pairs[ket];
        const auto& hb = e->basis[0];
        const int n1 = hfg::ncart(hb.l[B.sh1]), n2 = hfg::ncart(hb.l[B.sh2]), n3 = hfg::ncart(hb.l[K.sh1]), n4 = hfg::ncart(hb.l[K.sh2]);
        std::vector<double> blk(static_cast<size_t>(n1) * n2 * n3 * n4);
        HFG_CUDA(cudaMemcpyAsync(blk.data(), e->d_store.p, sizeof(double) * blk.size(), cudaMemcpyDeviceToHost, e->stream));
        HFG_CUDA(cudaStreamSynchronize(e->stream));
        // blk is [B.sh1][B.sh2][K.sh1][K.sh2]; permute into [a][b][c][d].
        const int na = hfg::ncart(hb.l[a]), nb = hfg::ncart(hb.l[b]), nc = hfg::ncart(hb.l[c]), nd = hfg::ncart(hb.l[d]);
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < nb; ++j)
                for (int k = 0; k < nc; ++k)
                    for (int l = 0; l < nd; ++l)
                    {
                        // Map (shell, component) pairs of the request to the stored orientation.
                        int comp[4];
                        const int sh[4] = {a, b, c, d}, cc[4] = {i, j, k, l};
                        const bool swap_pairs = (bra != pb);
                        const int p0 = swap_pairs ? 2 : 0, p1 = swap_pairs ? 0 : 2;
                        // bra pair holds request slots p0, p0+1
                        auto place = [&](int slot_a, int slot_b, const hfg::PairRec& pr, int* dst) {
                            if (sh[slot_a] == pr.sh1 && (sh[slot_b] == pr.sh2))
                            {
                                dst[0] = cc[slot_a];
                                dst[1] = cc[slot_b];
                            }
                            else
                            {
                                dst[0] = cc[slot_b];
                                dst[1] = cc[slot_a];
                            }
                        };
                        place(p0, p0 + 1, B, comp);
                        place(p1, p1 + 1, K, comp + 2);
                        out[((i * nb + j) * nc + k) * nd + l] = blk[((comp[0] * n2 + comp[1]) * n3 + comp[2]) * n4 + comp[3]];
                    }
        e->d_store.release();
    });
}

} // extern "C"
