// Device-side DIIS and SCF convergence measures (scf_device.cu), used by the SCF driver (host_scf.cpp)
// so that a whole SCF iteration can be captured in one CUDA graph.
#pragma once

#include <cuda_runtime.h>

namespace hfg
{
constexpr int kDiisMaxSize = 16; // largest DIIS_SIZE the device path handles (the host path has no limit)

// Ring of DIIS entries: logical entry i (0 = oldest) is in slot (head + i) % cap; coef[s] after a solve.
struct DiisState
{
    int count, head, cap, newest;
    double coef[kDiisMaxSize];
};

struct DiisSlots
{
    double* Fa[kDiisMaxSize];
    double* Fb[kDiisMaxSize];
    double* e[kDiisMaxSize];
};

// The measures the host reads after every iteration (pinned copy).
struct ScfScalars
{
    double energy, delta_e, delta_d, diis_error;
};

struct DiisDevice
{
    DiisState* state;
    DiisSlots slots;
    double* B;                     // cap x cap, per slot pair
    const double* const* xs_e;     // [cap]: the new error vector (fixed buffer) for every pair
    const double* const* ys_slots; // [cap]: the slots' error vectors
    double* part;                  // cap x nblk partial sums
    int cap, nblk, num_sms;
};

struct MeasureDevice
{
    const double *h, *Fa, *Fb, *Dt, *Dtp;
    double *wa, *wb, *dd;          // scratch vectors of length n
    const double* const* xs;       // [3]: Da, Db, dd
    const double* const* ys;       // [3]: wa, wb, dd
    double* part;                  // 3 x nblk
    ScfScalars* sc;
    int nblk, num_sms;
};

int dot_blocks(int num_sms);
// Appends (Fa, Fb, e) to the ring (dropping the oldest entry when full) and updates B's newest row.
cudaError_t diis_push(const DiisDevice& d, const double* Fa, const double* Fb, const double* e, long long n,
                      cudaStream_t s);
// Solves for the coefficients and writes F = sum c_i F_i into Fa, Fb; ||e_newest|| into sc->diis_error.
cudaError_t diis_extrapolate(const DiisDevice& d, double* Fa, double* Fb, ScfScalars* sc, long long n, cudaStream_t s);
// sc->energy (and delta_e against the previous value), sc->delta_d.
cudaError_t scf_measures(const MeasureDevice& m, long long n, cudaStream_t s);
} // namespace hfg
