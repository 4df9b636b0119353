// The persistent work-queue launch of the small classes (persistent.cu).
#pragma once

#include "eri_jk.cuh"

#include <cuda_runtime.h>

namespace hfg
{
// Segments of the work queue: (ss|ss), (ps|ss), (ps|ps), (pp|ss) in FP64, then the same in FP32.
constexpr int kPersistentSegments = 8;
constexpr int kPersistentClasses[4] = {0, 1, 2, 3}; // quartet classes in the queue

struct PersistentArgs
{
    const Quartet* list[kPersistentSegments];
    const unsigned long long* count[kPersistentSegments]; // device list lengths (null: segment empty)
    FockView view[2];                                     // FP64, FP32
    const void* slice[kPersistentSegments];               // Boys slices (global memory) of each segment's L
    unsigned long long* counter;                          // the queue's next item (reset by the launch)
};

// Resets the counter and launches one persistent grid (as many blocks as fit on the GPU at once).
cudaError_t launch_persistent(const PersistentArgs& a, bool uhf, cudaStream_t stream, int num_sms);
} // namespace hfg
