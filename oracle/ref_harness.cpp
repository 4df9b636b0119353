// Test-only harness around the reference Hartree-Fock program (MalachiF1/Hartree-Fock).
//
// This translation unit is compiled together with the reference's own, unmodified sources
// (src/*.cpp, src/Symmetry/*.cpp) into oracle/_ref/libhfref.so by oracle/Makefile.ref.  It exposes,
// through a plain C ABI that Python's ctypes can load, the reference functions on the direct-SCF
// two-electron path, so that tests can compare the GPU engine against the reference's own numbers:
//
//   Boys::calculateBoys                     src/Boys.cpp:14-71
//   IntegralEngine::electronRepulsion       src/IntegralEngine.cpp:731-992  (std::vector overload)
//   IntegralEngine::schwartzScreeningMatrix src/IntegralEngine.cpp:695-728
//   SCF::buildFockMatrixDirect              src/SCF.cpp:523-744
//   SCF::run                                src/SCF.cpp:23-135
//
// It is test infrastructure: nothing in the product links it, and it only exists where the
// reference sources are available to compile.
#include <Eigen/Dense>

#include <cstring>
#include <filesystem>
#include <memory>
#include <string>
#include <unistd.h>
#include <vector>

// The harness needs the SCF object's private state (the density/Fock matrices and the private
// buildFockMatrixDirect); widen access for the reference headers included below only.
#define private public
#include "Boys.hpp"
#include "IntegralEngine.hpp"
#include "Input.hpp"
#include "Output.hpp"
#include "SCF.hpp"
#undef private

namespace
{
struct Session
{
    std::string workdir;
    std::string inputPath;
    std::shared_ptr<Output> output;
    std::unique_ptr<SCF> scf;
    std::string lastError;
};

thread_local std::string g_lastError;

// The reference reads "basis_sets/<name>.json" and caches "boys_grid.data" relative to the current
// directory; run those calls from the oracle work directory and restore the caller's directory.
struct CwdGuard
{
    std::filesystem::path saved;
    explicit CwdGuard(const std::string& dir) : saved(std::filesystem::current_path())
    {
        std::filesystem::current_path(dir);
    }
    ~CwdGuard() { std::filesystem::current_path(saved); }
};

void copyMat(const Eigen::MatrixXd& m, double* out)
{
    std::memcpy(out, m.data(), sizeof(double) * m.size());
}

Eigen::MatrixXd fromPtr(const double* p, size_t n)
{
    Eigen::MatrixXd m(n, n);
    std::memcpy(m.data(), p, sizeof(double) * n * n);
    return m;
}
} // namespace

extern "C" {

const char* ref_last_error() { return g_lastError.c_str(); }

// Parses an input file with the reference's Input class and builds (but does not run) an SCF object;
// initialize() is called so that S, T, V, X and the Schwartz matrix Q are available.
void* ref_open(const char* input_path, const char* workdir, const char* output_path)
{
    try
    {
        auto s       = std::make_unique<Session>();
        s->workdir   = workdir;
        s->inputPath = input_path;
        CwdGuard guard(s->workdir);
        Input input(s->inputPath);
        auto [molecule, options, basis] = input.read();
        s->output = std::make_shared<Output>(output_path);
        s->scf    = std::make_unique<SCF>(molecule, basis, options, s->output);
        s->scf->initialize(options.schwartzThreshold, options.direct);
        s->scf->computeInitialGuessDensity();
        return s.release();
    }
    catch (const std::exception& e)
    {
        g_lastError = e.what();
        return nullptr;
    }
}

void ref_close(void* h) { delete static_cast<Session*>(h); }

// sizes[0..7] = nShells, nAO, nPrimitives, nNormFactors, unrestricted, nOccAlpha, nOccBeta, nAtoms
int ref_info(void* h, long* sizes, double* nuclear_repulsion)
{
    auto* s          = static_cast<Session*>(h);
    const SCF& scf   = *s->scf;
    sizes[0]         = static_cast<long>(scf.basis.nShells);
    sizes[1]         = static_cast<long>(scf.basis.nAOs);
    sizes[2]         = static_cast<long>(scf.basis.nPrimitives);
    sizes[3]         = static_cast<long>(scf.basis.nNormFactors);
    sizes[4]         = scf.options.unrestricted ? 1 : 0;
    sizes[5]         = static_cast<long>(scf.occupiedCountAlpha);
    sizes[6]         = static_cast<long>(scf.occupiedCountBeta);
    sizes[7]         = static_cast<long>(scf.molecule->getGeometry().size());
    *nuclear_repulsion = scf.nuclearEnergy;
    return 0;
}

// Geometry after the reference's own preprocessing (centre of mass / symmetry reorientation).
int ref_geometry(void* h, int* Z, double* xyz)
{
    auto* s         = static_cast<Session*>(h);
    const auto& geo = s->scf->molecule->getGeometry();
    for (size_t i = 0; i < geo.size(); ++i)
    {
        Z[i]           = static_cast<int>(geo[i].atomicNumber);
        xyz[3 * i + 0] = geo[i].coords.x();
        xyz[3 * i + 1] = geo[i].coords.y();
        xyz[3 * i + 2] = geo[i].coords.z();
    }
    return 0;
}

// The structure-of-arrays basis held by IntegralEngine (IntegralEngine.cpp:13-75).
int ref_basis_soa(void* h, int* l, int* nprim, int* primOff, int* aoOff, int* normOff, double* centers, double* alpha,
                  double* coeff, double* norms, int* am)
{
    auto* s                 = static_cast<Session*>(h);
    const IntegralEngine& e = *s->scf->integralEngine;
    for (size_t i = 0; i < e.nShells; ++i)
    {
        l[i]               = e.lShell[i];
        nprim[i]           = e.nPrimitives[i];
        primOff[i]         = e.primitiveOffsets[i];
        aoOff[i]           = e.aoOffsets[i];
        normOff[i]         = e.normFactorOffsets[i];
        centers[3 * i + 0] = e.centers(0, i);
        centers[3 * i + 1] = e.centers(1, i);
        centers[3 * i + 2] = e.centers(2, i);
    }
    for (Eigen::Index i = 0; i < e.alpha.size(); ++i)
    {
        alpha[i] = e.alpha[i];
        coeff[i] = e.coeff[i];
    }
    for (Eigen::Index i = 0; i < e.normalizationFactors.size(); ++i) norms[i] = e.normalizationFactors[i];
    for (Eigen::Index i = 0; i < e.angularMomentum.cols(); ++i)
        for (int k = 0; k < 3; ++k) am[3 * i + k] = e.angularMomentum(k, i);
    return 0;
}

int ref_boys(unsigned m_max, double T, double* F)
{
    try
    {
        Boys::calculateBoys(m_max, T, std::span<double>(F, m_max + 1));
        return 0;
    }
    catch (const std::exception& e)
    {
        g_lastError = e.what();
        return -1;
    }
}

double ref_boys_analytical(unsigned m, double T) { return Boys::analyticalBoys(m, T); }

// One contracted shell-quartet block, row-major [a][b][c][d], with the reference's zero pattern.
int ref_eri(void* h, long a, long b, long c, long d, double* out)
{
    auto* s                 = static_cast<Session*>(h);
    const IntegralEngine& e = *s->scf->integralEngine;
    const auto& n           = e.getNAOsPerShell();
    std::vector<double> G(static_cast<size_t>(n[a] * n[b] * n[c] * n[d]), 0.0);
    e.electronRepulsion(a, b, c, d, G);
    std::memcpy(out, G.data(), sizeof(double) * G.size());
    return 0;
}

int ref_schwartz(void* h, double* Q)
{
    copyMat(static_cast<Session*>(h)->scf->Q, Q);
    return 0;
}

int ref_one_electron(void* h, double* S, double* T, double* V)
{
    auto* s = static_cast<Session*>(h);
    copyMat(s->scf->S, S);
    copyMat(s->scf->T, T);
    copyMat(s->scf->V, V);
    return 0;
}

// Core-Hamiltonian guess densities as computed by the reference (SCF.cpp:165-231).
int ref_guess(void* h, double* Da, double* Db)
{
    auto* s = static_cast<Session*>(h);
    copyMat(s->scf->D_alpha, Da);
    copyMat(s->scf->D_beta, Db);
    return 0;
}

// One call of SCF::buildFockMatrixDirect with caller-provided densities and previous Fock matrices.
// Returns F_alpha, F_beta = F_prev + J - K as the reference forms them (SCF.cpp:731-743).
int ref_fock_direct(void* h, const double* Da, const double* Db, const double* DaPrev, const double* DbPrev,
                    const double* FaPrev, const double* FbPrev, double* Fa, double* Fb)
{
    try
    {
        auto* s       = static_cast<Session*>(h);
        SCF& scf      = *s->scf;
        const size_t n = scf.basisCount;
        scf.D_alpha      = fromPtr(Da, n);
        scf.D_beta       = fromPtr(Db, n);
        scf.D_alpha_prev = fromPtr(DaPrev, n);
        scf.D_beta_prev  = fromPtr(DbPrev, n);
        scf.D_tot        = scf.D_alpha + scf.D_beta;
        scf.D_tot_prev   = scf.D_alpha_prev + scf.D_beta_prev;
        scf.F_alpha_prev = fromPtr(FaPrev, n);
        scf.F_beta_prev  = fromPtr(FbPrev, n);
        scf.buildFockMatrixDirect();
        copyMat(scf.F_alpha, Fa);
        copyMat(scf.F_beta, Fb);
        return 0;
    }
    catch (const std::exception& e)
    {
        g_lastError = e.what();
        return -1;
    }
}

// Full SCF::run on a fresh SCF object built from the same input.
// out[0] = electronic energy, out[1] = nuclear repulsion, out[2] = iterations performed.
int ref_scf_run(void* h, double* out, double* Da, double* Db, double* Fa, double* Fb)
{
    try
    {
        auto* s = static_cast<Session*>(h);
        CwdGuard guard(s->workdir);
        Input input(s->inputPath);
        auto [molecule, options, basis] = input.read();
        SCF scf(molecule, basis, options, s->output);
        scf.run();
        out[0] = scf.electronicEnergy;
        out[1] = scf.nuclearEnergy;
        out[2] = static_cast<double>(scf.iteration);
        copyMat(scf.D_alpha, Da);
        copyMat(scf.D_beta, Db);
        copyMat(scf.F_alpha, Fa);
        copyMat(scf.F_beta, Fb);
        return 0;
    }
    catch (const std::exception& e)
    {
        g_lastError = e.what();
        return -1;
    }
}

} // extern "C"
