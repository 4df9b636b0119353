// Device one-electron integrals (onee.cu): launch interface used by the engine.
#pragma once

#include <cuda_runtime.h>

namespace hfg
{
// The basis of one molecule in device memory (the hfg_basis arrays).
struct OneeBasis
{
    const int *l, *nprim, *prim_off, *ao_off, *norm_off;
    const double *centers, *alpha, *coeff, *norms;
};

// One pair class's shell pairs (sa, sb) with l(sa) >= l(sb), each pair once.
struct OneeLaunch
{
    const int2* pairs;
    int npairs;
    OneeBasis basis;
    const double4* nuc; // x, y, z, Z per nucleus
    int natom;
    int n;                  // nao (column-major n x n outputs)
    const void* boys_slice; // FP64 Boys slice of total L = l(sa) + l(sb) (gradient: + 2)
    double *S, *T, *V;
    // Gradient (launch_one_electron_grad): densities and the natom x 3 output.
    const double *D, *W;
    const int* shell_atom;
    double* grad;
    cudaStream_t stream;
    int num_sms;
};

// S, T, V blocks of every pair of pair class pc (both triangles written).
cudaError_t launch_one_electron(int pc, const OneeLaunch& L);
// Adds sum D dT/dX + D dV/dX - W dS/dX of every pair of pair class pc into grad (atomic).
cudaError_t launch_one_electron_grad(int pc, const OneeLaunch& L);
} // namespace hfg
