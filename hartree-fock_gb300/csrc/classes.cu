// Kernel instantiations and launchers of ONE shell-quartet class.  The build compiles this file three
// times per class, -DHFG_QCLASS=<0..20> -DHFG_PART=<0..2>: part 0 the FP64 Fock kernels (and the form
// mask), part 1 the FP32 Fock kernels, part 2 the gradient kernels, so that the 63 units compile in
// parallel and the largest class does not serialise the build.
#include "engine.h"
#include "eri_grad.cuh"
#include "eri_group.cuh"

#ifndef HFG_QCLASS
#error "compile with -DHFG_QCLASS=<quartet class>"
#endif
#ifndef HFG_PART
#error "compile with -DHFG_PART=<0: FP64 Fock kernels, 1: FP32 Fock kernels, 2: gradient kernels>"
#endif

namespace hfg
{
namespace
{
constexpr int QC = HFG_QCLASS;
constexpr int bra_class()
{
    int p = 0;
    while ((p + 1) * (p + 2) / 2 <= QC) ++p;
    return p;
}
constexpr int P1 = bra_class();
constexpr int P2 = QC - P1 * (P1 + 1) / 2;
constexpr int LA = pair_class_l1(P1), LB = pair_class_l2(P1), LC = pair_class_l1(P2), LD = pair_class_l2(P2);
constexpr int NAB = ncart(LA) * ncart(LB), NCD = ncart(LC) * ncart(LD);
constexpr int L   = LA + LB + LC + LD;
// Kernel form per class and precision, from the ptxas footprint of the thread-per-quartet form
// (sm_103a, -O3): thread-per-quartet where its stack frame stays at or below ~1.2 KB, the
// warp-cooperative form for the larger d classes.
//   FP64 warp: (dp|pp) (dp|ds) (dp|dp) (dd|ps) (dd|pp) (dd|ds) (dd|dp) (dd|dd)   = classes 12-14, 16-20
//   FP32 warp: (dp|dp) (dd|pp) (dd|ds) (dd|dp) (dd|dd)                           = classes 14, 17-20
constexpr bool warp_form(bool fp32)
{
    return fp32 ? (QC == 14 || QC >= 17) : (QC == 12 || QC == 13 || QC == 14 || QC >= 16);
}
// The primitive-parallel group form exists for the small, contracted classes (L <= 3, <= 27 integrals).
constexpr bool kGroup = (L <= 3) && (NAB * NCD <= 27);
// FP32 classes whose thread form sits at the 255-register limit ((dp|ps), (dp|pp), (dp|ds), (dd|ps): one or
// two blocks per SM) also compile the warp form, and the autotuner times both.
constexpr bool dual_form(bool fp32) { return fp32 && (QC == 11 || QC == 12 || QC == 13 || QC == 16); }
// Ket-chunked thread form (FP32 d classes): ket components per thread, chosen so that R, G[HAB][CH] and
// ERI[NAB][CH] stay in registers (HL + (HAB + NAB) * CH floats well below 255); 0 = not compiled.
//   (dp|pp) (dp|ds): 3   (dp|dp): 2   (dd|ps) (dd|pp) (dd|ds) (dd|dp): 1
constexpr int chunk_width(bool fp32)
{
    if (!fp32)
        return 0;
    return (QC == 12 || QC == 13) ? 3 : QC == 14 ? 2 : (QC >= 16 && QC <= 19) ? 1 : 0;
}
// The form a launch with form 0 runs (before or without autotuning): the chunked form where the tuner
// keeps it at full size ((H2O)_64/6-31G**: (dp|pp), (dp|ds), (dp|dp), (dd|pp), (dd|ds), (dd|dp) in FP32),
// else warp or thread.
constexpr int default_form(bool fp32)
{
    return (fp32 && (QC == 12 || QC == 13 || QC == 14 || (QC >= 17 && QC <= 19))) ? kFormChunk
                                                                                   : (warp_form(fp32) ? kFormWarp : kFormThread);
}
constexpr unsigned form_mask(bool fp32)
{
    return (warp_form(fp32) || dual_form(fp32) ? (1u << kFormWarp) : 0u) |
           (!warp_form(fp32) || dual_form(fp32) ? (1u << kFormThread) : 0u) | (kGroup ? (1u << kFormGroup) : 0u) |
           (chunk_width(fp32) > 0 ? (1u << kFormChunk) : 0u);
}

// Resident blocks per SM a grid may take: the occupancy limit times the share, at least one.
inline unsigned long long resident(int per_sm, float share)
{
    const int r = static_cast<int>(static_cast<float>(per_sm > 0 ? per_sm : 1) * share);
    return static_cast<unsigned long long>(r > 0 ? r : 1);
}

template <typename Real, bool UHF> cudaError_t launch_t(const ClassLaunch& c)
{
    constexpr bool kWarpForm = warp_form(sizeof(Real) == 4);
    if (c.count_host == 0)
        return cudaSuccess;
    const int form = c.form == 0 ? default_form(sizeof(Real) == 4) : c.form;
    if (!((form_mask(sizeof(Real) == 4) >> form) & 1u))
        return cudaErrorInvalidValue;
    const size_t slice_bytes = sizeof(Real) * BoysGrid<Real>::kPoints * BoysGrid<Real>::kRow;
    if constexpr (kGroup)
    {
        if (form == kFormGroup)
        {
            auto kern         = jk_class_group_kernel<LA, LB, LC, LD, Real, UHF>;
            const size_t smem = slice_bytes;
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess)
                return e;
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
            if (e != cudaSuccess)
                return e;
            const unsigned long long need = (c.count_host + 127) / 128; // 4 warps x 32-quartet windows
            const unsigned long long cap  = static_cast<unsigned long long>(c.num_sms) * resident(per_sm, c.share);
            kern<<<static_cast<unsigned>(need < cap ? need : cap), 128, smem, c.stream>>>(
                c.list, c.count_dev, c.view, static_cast<const Real*>(c.boys_slice));
            return cudaGetLastError();
        }
    }
    constexpr int kChunk = chunk_width(sizeof(Real) == 4);
    if constexpr (kChunk > 0)
    {
        if (form == kFormChunk)
        {
            // One launch per chunk of kChunk ket components, each over the whole list.
            constexpr int nch = num_chunks<LC, LD, kChunk>();
            cudaError_t err   = cudaSuccess;
            static_for<0, nch>(
                [&](auto C)
                {
                    constexpr int k0 = decltype(C)::value * kChunk;
                    constexpr int k1 = k0 + kChunk < NCD ? k0 + kChunk : NCD;
                    if (err != cudaSuccess)
                        return;
                    auto kern         = jk_class_chunk_kernel<LA, LB, LC, LD, Real, UHF, k0, k1>;
                    const size_t smem = slice_bytes;
                    err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
                    if (err != cudaSuccess)
                        return;
                    int per_sm = 0;
                    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
                    if (err != cudaSuccess)
                        return;
                    const unsigned long long need = (c.count_host + 127) / 128;
                    const unsigned long long cap  = static_cast<unsigned long long>(c.num_sms) * resident(per_sm, c.share);
                    kern<<<static_cast<unsigned>(need < cap ? need : cap), 128, smem, c.stream>>>(
                        c.list, c.count_dev, c.view, static_cast<const Real*>(c.boys_slice));
                    err = cudaGetLastError();
                });
            return err;
        }
    }
    constexpr bool kHasWarp = kWarpForm || dual_form(sizeof(Real) == 4);
    constexpr bool kHasThread = !kWarpForm || dual_form(sizeof(Real) == 4);
    if constexpr (kHasWarp)
    {
        if (form == kFormWarp)
        {
            using W             = WarpLayout<LA, LB, LC, LD, Real>;
            const size_t smem   = slice_bytes + sizeof(Real) * W::kPerWarp * kWarpKernelWarps;
            auto kern           = jk_class_warp_kernel<LA, LB, LC, LD, Real, UHF>;
            cudaError_t e       = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess)
                return e;
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kWarpKernelWarps, smem);
            if (e != cudaSuccess)
                return e;
            const unsigned long long need = (c.count_host + kWarpKernelWarps - 1) / kWarpKernelWarps;
            const unsigned long long cap  = static_cast<unsigned long long>(c.num_sms) * resident(per_sm, c.share);
            const unsigned grid           = static_cast<unsigned>(need < cap ? need : cap);
            kern<<<grid, 32 * kWarpKernelWarps, smem, c.stream>>>(c.list, c.count_dev, c.view,
                                                                  static_cast<const Real*>(c.boys_slice), c.tables);
            return cudaGetLastError();
        }
    }
    if constexpr (kHasThread)
    {
        if (form == kFormThread)
        {
            auto kern           = jk_class_kernel<LA, LB, LC, LD, Real, UHF>;
            const size_t smem   = slice_bytes;
            cudaError_t e       = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess)
                return e;
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
            if (e != cudaSuccess)
                return e;
            const unsigned long long need = (c.count_host + 127) / 128;
            const unsigned long long cap  = static_cast<unsigned long long>(c.num_sms) * resident(per_sm, c.share);
            const unsigned grid           = static_cast<unsigned>(need < cap ? need : cap);
            kern<<<grid, 128, smem, c.stream>>>(c.list, c.count_dev, c.view, static_cast<const Real*>(c.boys_slice));
            return cudaGetLastError();
        }
    }
    return cudaErrorInvalidValue;
}
} // namespace

#define HFG_CAT2(a, b) a##b
#define HFG_CAT(a, b) HFG_CAT2(a, b)

#if HFG_PART == 0
cudaError_t HFG_CAT(launch_class64_, HFG_QCLASS)(const ClassLaunch& c)
{
    return c.uhf ? launch_t<double, true>(c) : launch_t<double, false>(c);
}

cudaError_t HFG_CAT(launch_stored_, HFG_QCLASS)(const StoredLaunch& c)
{
    if (c.count == 0)
        return cudaSuccess;
    constexpr int nch = num_chunks<LC, LD, stored_chunk<LA, LB, LC, LD>()>();
    auto kern = c.uhf ? jk_stored_kernel<LA, LB, LC, LD, true> : jk_stored_kernel<LA, LB, LC, LD, false>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
    if (e != cudaSuccess)
        return e;
    const unsigned long long need = (c.count + 127) / 128;
    unsigned long long cap = static_cast<unsigned long long>(c.num_sms) * (per_sm > 0 ? per_sm : 1) / nch;
    if (cap < 1)
        cap = 1;
    const unsigned long long qblocks = need < cap ? need : cap;
    kern<<<static_cast<unsigned>(qblocks * nch), 128, 0, c.stream>>>(c.list, c.count, c.view, c.store);
    return cudaGetLastError();
}

// Bits 0-15: compiled forms; 16-23: the default form; 24-31: kernel launches of one chunk-form launch.
unsigned HFG_CAT(class_form_mask_, HFG_QCLASS)(bool fp32)
{
    const unsigned nch = chunk_width(fp32) > 0 ? static_cast<unsigned>((NCD + chunk_width(fp32) - 1) / chunk_width(fp32)) : 0u;
    return form_mask(fp32) | (static_cast<unsigned>(default_form(fp32)) << 16) | (nch << 24);
}
#elif HFG_PART == 1
cudaError_t HFG_CAT(launch_class32_, HFG_QCLASS)(const ClassLaunch& c)
{
    return c.uhf ? launch_t<float, true>(c) : launch_t<float, false>(c);
}
#else
namespace
{
// Thread-per-quartet gradient form where the per-thread arrays fit in registers (GradThread::kValues: at
// most 72 doubles or 160 floats):
//   FP64: (ss|ss) (ps|ss) (ps|ps) (pp|ss) (ds|ss);  FP32: also (pp|ps) (ds|ps) (dp|ss).
template <typename Real> constexpr bool grad_thread_form()
{
    return GradThread<LA, LB, LC, LD>::kValues <= (sizeof(Real) == 8 ? 72 : 160);
}

template <typename Real> cudaError_t launch_grad_thread(const GradLaunch& c)
{
    const size_t smem = sizeof(Real) * BoysGrid<Real>::kPoints * BoysGrid<Real>::kRow;
    auto kern         = grad_thread_kernel<LA, LB, LC, LD, Real>;
    cudaError_t e     = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
    if (e != cudaSuccess)
        return e;
    const unsigned long long need = (c.count + 127) / 128;
    const unsigned long long cap  = static_cast<unsigned long long>(c.num_sms) * (per_sm > 0 ? per_sm : 1);
    kern<<<static_cast<unsigned>(need < cap ? need : cap), 128, smem, c.stream>>>(c.list, c.count, c.view,
                                                                                static_cast<const Real*>(c.boys_slice));
    return cudaGetLastError();
}

template <typename Real> cudaError_t launch_grad_t(const GradLaunch& c)
{
    if constexpr (grad_thread_form<Real>())
        if (!c.group_form)
            return launch_grad_thread<Real>(c);
    using W           = GradLayout<LA, LB, LC, LD>;
    const size_t smem = sizeof(Real) * (BoysGrid<Real>::kPoints * BoysGrid<Real>::kRow + W::kPerWarp * kGradWarps);
    auto kern         = grad_class_kernel<LA, LB, LC, LD, Real>;
    cudaError_t e     = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kGradWarps, smem);
    if (e != cudaSuccess)
        return e;
    constexpr unsigned long long per_block = kGradWarps * (32 / W::kGroup); // quartets in flight per block
    const unsigned long long need = (c.count + per_block - 1) / per_block;
    const unsigned long long cap  = static_cast<unsigned long long>(c.num_sms) * (per_sm > 0 ? per_sm : 1);
    kern<<<static_cast<unsigned>(need < cap ? need : cap), 32 * kGradWarps, smem, c.stream>>>(
        c.list, c.count, c.view, static_cast<const Real*>(c.boys_slice), c.tables);
    return cudaGetLastError();
}
} // namespace

cudaError_t HFG_CAT(launch_grad_, HFG_QCLASS)(const GradLaunch& c)
{
    if (c.count == 0)
        return cudaSuccess;
    return c.fp32 ? launch_grad_t<float>(c) : launch_grad_t<double>(c);
}
#endif
} // namespace hfg
