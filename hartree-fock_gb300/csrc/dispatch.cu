// Tables of the per-class launchers (three translation units per class, see classes.cu): FP64 and FP32
// Fock kernels, gradient kernels, and the compiled-form masks.
#include "engine.h"
#include "eri_grad.cuh"

namespace hfg
{
#define HFG_DECL(c)                                                                                                    \
    cudaError_t launch_class64_##c(const ClassLaunch&);                                                               \
    cudaError_t launch_class32_##c(const ClassLaunch&);                                                               \
    cudaError_t launch_grad_##c(const GradLaunch&);                                                                   \
    cudaError_t launch_stored_##c(const StoredLaunch&);                                                               \
    unsigned class_form_mask_##c(bool);
HFG_DECL(0) HFG_DECL(1) HFG_DECL(2) HFG_DECL(3) HFG_DECL(4) HFG_DECL(5) HFG_DECL(6) HFG_DECL(7) HFG_DECL(8)
HFG_DECL(9) HFG_DECL(10) HFG_DECL(11) HFG_DECL(12) HFG_DECL(13) HFG_DECL(14) HFG_DECL(15) HFG_DECL(16)
HFG_DECL(17) HFG_DECL(18) HFG_DECL(19) HFG_DECL(20)
#undef HFG_DECL

static const ClassLauncher kLaunch64[kNumQuartetClasses] = {
    launch_class64_0, launch_class64_1, launch_class64_2, launch_class64_3, launch_class64_4, launch_class64_5,
    launch_class64_6, launch_class64_7, launch_class64_8, launch_class64_9, launch_class64_10, launch_class64_11,
    launch_class64_12, launch_class64_13, launch_class64_14, launch_class64_15, launch_class64_16, launch_class64_17,
    launch_class64_18, launch_class64_19, launch_class64_20};
static const ClassLauncher kLaunch32[kNumQuartetClasses] = {
    launch_class32_0, launch_class32_1, launch_class32_2, launch_class32_3, launch_class32_4, launch_class32_5,
    launch_class32_6, launch_class32_7, launch_class32_8, launch_class32_9, launch_class32_10, launch_class32_11,
    launch_class32_12, launch_class32_13, launch_class32_14, launch_class32_15, launch_class32_16, launch_class32_17,
    launch_class32_18, launch_class32_19, launch_class32_20};

static const decltype(&launch_grad_0) kGrad[kNumQuartetClasses] = {
    launch_grad_0,  launch_grad_1,  launch_grad_2,  launch_grad_3,  launch_grad_4,  launch_grad_5,  launch_grad_6,
    launch_grad_7,  launch_grad_8,  launch_grad_9,  launch_grad_10, launch_grad_11, launch_grad_12, launch_grad_13,
    launch_grad_14, launch_grad_15, launch_grad_16, launch_grad_17, launch_grad_18, launch_grad_19, launch_grad_20};

static const decltype(&launch_stored_0) kStored[kNumQuartetClasses] = {
    launch_stored_0,  launch_stored_1,  launch_stored_2,  launch_stored_3,  launch_stored_4,  launch_stored_5,
    launch_stored_6,  launch_stored_7,  launch_stored_8,  launch_stored_9,  launch_stored_10, launch_stored_11,
    launch_stored_12, launch_stored_13, launch_stored_14, launch_stored_15, launch_stored_16, launch_stored_17,
    launch_stored_18, launch_stored_19, launch_stored_20};

cudaError_t launch_stored(int qclass, const StoredLaunch& L)
{
    if (qclass < 0 || qclass >= kNumQuartetClasses)
        return cudaErrorInvalidValue;
    return kStored[qclass](L);
}

cudaError_t launch_grad(int qclass, const GradLaunch& L)
{
    if (qclass < 0 || qclass >= kNumQuartetClasses)
        return cudaErrorInvalidValue;
    return kGrad[qclass](L);
}

cudaError_t launch_class(int qclass, const ClassLaunch& L)
{
    if (qclass < 0 || qclass >= kNumQuartetClasses)
        return cudaErrorInvalidValue;
    return L.fp32 ? kLaunch32[qclass](L) : kLaunch64[qclass](L);
}

static unsigned (*const kMask[kNumQuartetClasses])(bool) = {
    class_form_mask_0,  class_form_mask_1,  class_form_mask_2,  class_form_mask_3,  class_form_mask_4,
    class_form_mask_5,  class_form_mask_6,  class_form_mask_7,  class_form_mask_8,  class_form_mask_9,
    class_form_mask_10, class_form_mask_11, class_form_mask_12, class_form_mask_13, class_form_mask_14,
    class_form_mask_15, class_form_mask_16, class_form_mask_17, class_form_mask_18, class_form_mask_19,
    class_form_mask_20};

// The class TUs return the compiled-form mask in bits 0-15, the default form in bits 16-23 and the
// kernel launches of the chunk form (one per chunk) in bits 24-31.
unsigned class_form_mask(int qclass, bool fp32)
{
    return (qclass >= 0 && qclass < kNumQuartetClasses) ? (kMask[qclass](fp32) & 0xffffu) : 0u;
}

int class_default_form(int qclass, bool fp32)
{
    return (qclass >= 0 && qclass < kNumQuartetClasses) ? static_cast<int>((kMask[qclass](fp32) >> 16) & 0xffu) : 0;
}

int class_launches(int qclass, bool fp32, int form)
{
    if (qclass < 0 || qclass >= kNumQuartetClasses)
        return 0;
    const unsigned m = kMask[qclass](fp32);
    if (form == 0)
        form = static_cast<int>((m >> 16) & 0xffu);
    return form == kFormChunk ? static_cast<int>((m >> 24) & 0xffu) : 1;
}

} // namespace hfg
