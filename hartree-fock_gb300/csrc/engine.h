// Internal engine state and the per-class launcher interface.
#pragma once

#include "hfg_common.cuh"
#include "eri_warp.cuh"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace hfg
{
// Launches the class kernel of one quartet class for one list.
struct ClassLaunch
{
    const Quartet* list;
    const unsigned long long* count_dev;
    unsigned long long count_host;
    FockView view;
    const void* boys_slice; // slice of the class's total L, Real of the precision
    const WarpTables* tables;
    bool fp32;
    bool uhf;
    cudaStream_t stream;
    int num_sms;
    int form; // 0: the class's default form, else one of kFormThread / kFormWarp / kFormGroup / kFormChunk
    float share = 1.f; // fraction of the resident blocks per SM the grid may take (concurrent precisions)
};
// Kernel forms of a class kernel (eri_jk.cuh, eri_warp.cuh, eri_group.cuh).
constexpr int kFormThread = 1, kFormWarp = 2, kFormGroup = 3, kFormChunk = 4;
constexpr int kFormPersistent = 5; // reported in the stats only: the class ran in the persistent work queue
using ClassLauncher = cudaError_t (*)(const ClassLaunch&);
// Defined in classes.cu (one translation unit per quartet class).
cudaError_t launch_class(int qclass, const ClassLaunch& L);
// Bit f set: form f is compiled for this class and precision.
unsigned class_form_mask(int qclass, bool fp32);
// The form a launch with form == 0 runs.
int class_default_form(int qclass, bool fp32);
// Kernel launches one launch_class call makes in the given form (0: the default form).
int class_launches(int qclass, bool fp32, int form);

// Digestion of one class's stored integrals (the stored-integral SCF).
struct StoredLaunch
{
    const Quartet* list;
    unsigned long long count;
    const double* store;
    FockView view;
    bool uhf;
    cudaStream_t stream;
    int num_sms;
};
cudaError_t launch_stored(int qclass, const StoredLaunch& L);

struct GradView;
struct GradLaunch
{
    const Quartet* list;
    unsigned long long count;
    const GradView& view;
    const void* boys_slice; // slice for total L + 1, Real of the kernel
    const WarpTables* tables;
    cudaStream_t stream;
    int num_sms;
    bool fp32;
    bool group_form; // the lane-group kernel for every class (else the thread form where it is compiled)
};
cudaError_t launch_grad(int qclass, const GradLaunch& L);

// Work model: algorithmic FLOPs of one primitive quartet and of one shell quartet's digestion.
double flops_per_prim_quartet(int qclass);
double flops_per_quartet_digest(int qclass, bool uhf);
} // namespace hfg
