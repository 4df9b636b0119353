// Persistent form of the Fock build for the small shell-quartet classes: ONE launch works through the
// quartet lists of (ss|ss), (ps|ss), (ps|ps) and (pp|ss), FP64 and FP32 together, as a work queue.
//
// Work items are blocks of 128 consecutive quartets of one list.  The items of the eight lists (four
// classes x two precisions, FP64 first, the heavier quartets early) form one index range; every block
// takes the next item with an atomic counter and runs the thread-per-quartet code of that class
// (eri_jk.cuh: eval_quartet + digestion with the warp-summed bra block) on it, until the range is used
// up.  Nothing waits on another block: a block that finds the counter past the end returns.  The list
// lengths are read on the device, so the launch is the same in a captured graph.  The Boys slices are
// read from global memory (L1-resident) because the items of one block change class.
//
// Only these four classes are in the queue: their thread kernels fit in 126 registers (FP64), so the
// merged kernel keeps four 128-thread blocks per SM; the classes with more work per quartet keep their
// own launches.
#include "engine.h"
#include "persistent.h"

namespace hfg
{
namespace
{
template <int LA, int LB, int LC, int LD, typename Real, bool UHF>
__device__ __forceinline__ void run_item(const Quartet* __restrict__ list, unsigned long long n, unsigned long long start,
                                         const FockView& v, const Real* __restrict__ slice)
{
    constexpr int N = ncart(LA) * ncart(LB) * ncart(LC) * ncart(LD);
    const unsigned long long base = start + (threadIdx.x & ~31u);
    if (base >= n)
        return; // whole warps only: the digestion's warp sums need every lane of the warp
    const int lane              = threadIdx.x & 31;
    const unsigned long long q  = base + lane;
    const bool active           = q < n;
    const Real* tb              = static_cast<const Real*>(v.pptab[pair_class(LA, LB)]);
    const Real* tk              = static_cast<const Real*>(v.ksoa[pair_class(LC, LD)]);
    const long long kfs         = v.kfs[pair_class(LC, LD)];
    const Quartet qt            = list[active ? q : base];
    const PairRec bra           = v.pairs[qt.bra];
    const PairRec ket           = v.pairs[qt.ket];
    using DD = DigestD<LA, LB, LC, LD, Real, UHF>;
    DD d;
    if (DD::kEarly)
        load_digest_d<LA, LB, LC, LD, Real, UHF>(bra, ket, v, d);
    Real acc[N];
    if (active)
        eval_quartet<LA, LB, LC, LD, Real, true>(bra, ket, tb, tk, slice, acc, kfs);
    else
    {
#pragma unroll
        for (int x = 0; x < N; ++x) acc[x] = Real(0);
    }
    if (!DD::kEarly)
        load_digest_d<LA, LB, LC, LD, Real, UHF>(bra, ket, v, d);
    const unsigned bra0 = __shfl_sync(0xffffffffu, qt.bra, 0);
    const bool bra_warp = __all_sync(0xffffffffu, qt.bra == bra0);
    digest_loaded<LA, LB, LC, LD, Real, UHF>(bra, ket, qt.bra == qt.ket, acc, v, d, active, bra_warp);
}

template <bool UHF> __global__ void __launch_bounds__(128) jk_persistent_kernel(PersistentArgs a)
{
    __shared__ unsigned long long seg_end[kPersistentSegments];
    __shared__ unsigned long long item;
    if (threadIdx.x == 0)
    {
        unsigned long long acc = 0;
        for (int s = 0; s < kPersistentSegments; ++s)
        {
            acc += a.count[s] ? (*a.count[s] + 127) / 128 : 0;
            seg_end[s] = acc;
        }
    }
    __syncthreads();
    const unsigned long long total = seg_end[kPersistentSegments - 1];
    for (;;)
    {
        if (threadIdx.x == 0)
            item = atomicAdd(a.counter, 1ull);
        __syncthreads();
        const unsigned long long i = item;
        __syncthreads(); // every thread has read `item` before thread 0 takes the next one
        if (i >= total)
            break;
        int s = 0;
        while (i >= seg_end[s]) ++s;
        const unsigned long long start = (i - (s > 0 ? seg_end[s - 1] : 0ull)) * 128ull;
        const unsigned long long n     = *a.count[s];
        const Quartet* L = a.list[s];
        switch (s)
        {
        case 0: run_item<0, 0, 0, 0, double, UHF>(L, n, start, a.view[0], static_cast<const double*>(a.slice[0])); break;
        case 1: run_item<1, 0, 0, 0, double, UHF>(L, n, start, a.view[0], static_cast<const double*>(a.slice[1])); break;
        case 2: run_item<1, 0, 1, 0, double, UHF>(L, n, start, a.view[0], static_cast<const double*>(a.slice[2])); break;
        case 3: run_item<1, 1, 0, 0, double, UHF>(L, n, start, a.view[0], static_cast<const double*>(a.slice[3])); break;
        case 4: run_item<0, 0, 0, 0, float, UHF>(L, n, start, a.view[1], static_cast<const float*>(a.slice[4])); break;
        case 5: run_item<1, 0, 0, 0, float, UHF>(L, n, start, a.view[1], static_cast<const float*>(a.slice[5])); break;
        case 6: run_item<1, 0, 1, 0, float, UHF>(L, n, start, a.view[1], static_cast<const float*>(a.slice[6])); break;
        default: run_item<1, 1, 0, 0, float, UHF>(L, n, start, a.view[1], static_cast<const float*>(a.slice[7])); break;
        }
    }
}
} // namespace

cudaError_t launch_persistent(const PersistentArgs& a, bool uhf, cudaStream_t stream, int num_sms)
{
    auto kern  = uhf ? jk_persistent_kernel<true> : jk_persistent_kernel<false>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
    if (e != cudaSuccess)
        return e;
    e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess)
        return e;
    kern<<<num_sms * (per_sm > 0 ? per_sm : 1), 128, 0, stream>>>(a);
    return cudaGetLastError();
}
} // namespace hfg
