// Direct SCF driver with the GPU Fock build; linear algebra stays FP64 on the device (cuBLAS/cuSOLVER).
//
// The semantics are those of the reference's SCF class (MalachiF1/Hartree-Fock):
//   SCF::initialize                    src/SCF.cpp:138-162   S, T, V, h = T + V, X = S^{-1/2} (Utils.cpp:117-138)
//   SCF::computeInitialGuessDensity    src/SCF.cpp:165-231   core guess, GUESS_MIX HOMO/LUMO rotation (UHF)
//   SCF::run                           src/SCF.cpp:23-135    iteration loop, DIIS, convergence test
//   SCF::buildFockMatrixDirect tail    src/SCF.cpp:731-743   F = F_prev + J[dD] - K[dD]  (incremental)
//   SCF::diagonalizeAndUpdate          src/SCF.cpp:747-835   damping, level shifting, densities, energy
//   DIIS::update / extrapolate         src/DIIS.cpp:12-72    B_ij = <e_i|e_j>, bordered system, sum c_i F_i
//   SCF::computeSpinSquared            src/SCF.cpp:838-845
// Only the two-electron build is replaced (hfg_fock_direct on device pointers).  The orbital
// eigenvectors come from cuSOLVER's syevd (ascending eigenvalues, as Eigen's SelfAdjointEigenSolver).
#include "hfgpu.h"
#include "scf_device.h"

#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <deque>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

struct hfg_engine;

namespace hfg
{
// Defined in engine.cu.
const hfg_basis* engine_basis(const hfg_engine* e);
void engine_set_error(hfg_engine* e, const std::string& msg);
void engine_store_scf_state(hfg_engine* e, const double* Da, const double* Db, const double* W, bool uhf);
int engine_enqueue_fock(hfg_engine* e, const hfg_fock_request& r);
void engine_prepare_capture(hfg_engine* e);
void engine_check_counts(hfg_engine* e, bool mixed);
int engine_guarded(hfg_engine* e, const std::function<void()>& f);
void one_electron_device(hfg_engine* e, int natom, const int* Z, const double* xyz, double* S, double* T, double* V);

namespace
{
struct ScfError : std::runtime_error
{
    int code;
    ScfError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess)
        throw ScfError(e == cudaErrorMemoryAllocation ? HFG_ERR_NOMEM : HFG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
void ck(cublasStatus_t e, const char* what)
{
    if (e != CUBLAS_STATUS_SUCCESS)
        throw ScfError(HFG_ERR_CUDA, std::string(what) + ": cublas status " + std::to_string(static_cast<int>(e)));
}
void ck(cusolverStatus_t e, const char* what)
{
    if (e != CUSOLVER_STATUS_SUCCESS)
        throw ScfError(HFG_ERR_CUDA, std::string(what) + ": cusolver status " + std::to_string(static_cast<int>(e)));
}

struct DMat
{
    double* p = nullptr;
    size_t n  = 0;
    DMat() = default;
    explicit DMat(size_t count) { alloc(count); }
    DMat(const DMat&) = delete;
    DMat& operator=(const DMat&) = delete;
    DMat(DMat&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; }
    ~DMat()
    {
        if (p)
            cudaFree(p);
    }
    void alloc(size_t count)
    {
        ck(cudaMalloc(&p, sizeof(double) * std::max<size_t>(count, 1)), "cudaMalloc");
        n = count;
    }
};

class Scf
{
  public:
    Scf(hfg_engine* e, const hfg_scf_options& o, int natom, const int* Z, const double* xyz, int charge, int mult)
        : eng_(e), o_(o)
    {
        const hfg_basis* b = engine_basis(e);
        if (!b)
            throw ScfError(HFG_ERR_INVALID, "scf: the engine must hold exactly one molecule");
        n_ = b->nao;
        long nel = -charge;
        for (int a = 0; a < natom; ++a) nel += Z[a];
        if (nel < 0 || mult < 1 || (nel + mult - 1) % 2 != 0)
            throw ScfError(HFG_ERR_INVALID, "scf: charge and multiplicity do not fit the electron count");
        nocc_a_ = static_cast<int>((nel + mult - 1) / 2);
        nocc_b_ = static_cast<int>((nel - mult + 1) / 2);
        if (nocc_a_ >= n_ || nocc_a_ < 1)
            throw ScfError(HFG_ERR_INVALID, "scf: occupied orbitals must be between 1 and nao - 1");
        uhf_ = o.unrestricted != 0;
        // Nuclear repulsion (src/Molecule.cpp:80-89).
        for (int i = 0; i < natom; ++i)
            for (int j = i + 1; j < natom; ++j)
            {
                const double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1], dz = xyz[3 * i + 2] - xyz[3 * j + 2];
                enuc_ += static_cast<double>(Z[i] * Z[j]) / std::sqrt(dx * dx + dy * dy + dz * dz);
            }
        s_ = static_cast<cudaStream_t>(hfg_stream(e));
        ck(cublasCreate(&cb_), "cublasCreate");
        ck(cublasSetStream(cb_, s_), "cublasSetStream");
        ck(cusolverDnCreate(&cs_), "cusolverDnCreate");
        ck(cusolverDnSetStream(cs_, s_), "cusolverDnSetStream");
        const size_t N2 = static_cast<size_t>(n_) * n_;
        for (DMat* m : {&S_, &X_, &h_, &Fa_, &Fb_, &Fap_, &Fbp_, &Da_, &Db_, &Dap_, &Dbp_, &Dt_, &Dtp_, &Ca_, &Cb_, &T1_,
                        &T2_, &J_, &Ka_, &Kb_, &dDt_, &dDa_, &dDb_, &e_})
            m->alloc(N2);
        wa_.alloc(n_);
        wb_.alloc(n_);
        ck(cudaMalloc(&info_, sizeof(int)), "cudaMalloc");
        int lw = 0;
        ck(cusolverDnDsyevd_bufferSize(cs_, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n_, T1_.p, n_, wa_.p, &lw),
           "syevd_bufferSize");
        work_.alloc(static_cast<size_t>(lw));
        lwork_ = lw;

        // One-electron part on the device (FP64): S, and h = T + V; X = S^{-1/2}.
        const int rc = engine_guarded(e, [&] { one_electron_device(e, natom, Z, xyz, S_.p, T1_.p, T2_.p); });
        if (rc != HFG_OK)
            throw ScfError(rc, std::string("scf: one-electron integrals failed: ") + hfg_last_error(e));
        add(h_, 1.0, T1_, 1.0, T2_);
        inverse_sqrt();
    }

    ~Scf()
    {
        free_device_iterations();
        if (info_)
            cudaFree(info_);
        if (cs_)
            cusolverDnDestroy(cs_);
        if (cb_)
            cublasDestroy(cb_);
    }

    // SCF.cpp:165-231.
    void guess()
    {
        copy(Fa_, h_);
        copy(Fap_, Fa_);
        eig_orth(Fa_, Ca_, wa_, false);
        zero(Dap_);
        density(Ca_, nocc_a_, Da_, 0.0);
        zero(Dbp_);
        if (uhf_)
        {
            if (o_.guess_mix > 0)
            {
                const double k = o_.guess_mix / 10.0, s = 1.0 / std::sqrt(1.0 + k * k);
                double* homo = Ca_.p + static_cast<size_t>(nocc_a_ - 1) * n_;
                double* lumo = Ca_.p + static_cast<size_t>(nocc_a_) * n_;
                // mixedHomo = s(homo + k lumo), mixedLumo = s(lumo - k homo)
                ck(cudaMemcpyAsync(T1_.p, homo, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s_), "copy");
                const double one = 1.0, kk = k, mk = -k;
                ck(cublasDaxpy(cb_, n_, &kk, lumo, 1, homo, 1), "axpy");
                ck(cublasDscal(cb_, n_, &s, homo, 1), "scal");
                ck(cublasDaxpy(cb_, n_, &mk, T1_.p, 1, lumo, 1), "axpy");
                ck(cublasDscal(cb_, n_, &s, lumo, 1), "scal");
                (void)one;
                density(Ca_, nocc_a_, Da_, 0.0);
            }
            copy(Fb_, h_);
            copy(Fbp_, Fb_);
            eig_orth(Fb_, Cb_, wb_, false);
            density(Cb_, nocc_b_, Db_, 0.0);
        }
        else
        {
            copy(Fb_, Fa_);
            copy(Fbp_, Fap_);
            copy(Cb_, Ca_);
            copy_vec(wb_, wa_);
            copy(Db_, Da_);
        }
        zero(Dtp_);
        add(Dt_, 1.0, Da_, 1.0, Db_);
        energy_ = electronic_energy();
        eig_host();
    }

    void run(hfg_scf_result& res)
    {
        const auto t0 = std::chrono::steady_clock::now();
        guess();
        if (o_.verbose)
            std::printf("%15s%15s%15s%15s\n", "Iteration", "dE", "dD", "DIIS Error");
        int it = 0;
        bool conv = false;
        // Device iterations (DIIS and the measures on the GPU) when the options allow a graph; the first
        // runs eagerly (it tunes the kernel forms and sizes the lists), the next is captured, and every
        // later one replays that graph.
        if (o_.direct == 0)
        {
            // SCF::initialize (SCF.cpp:157-159): the integrals are computed once before the iterations.
            const int rc = hfg_store_integrals(eng_, o_.schwartz_threshold, nullptr);
            if (rc != HFG_OK)
                throw ScfError(rc, std::string("scf: storing the integrals failed: ") + hfg_last_error(eng_));
        }
        const bool device_iter = o_.direct != 0 && o_.graph_iterations != 0 && o_.damp == 0 && !(o_.level_shift > 0) &&
                                 (!o_.use_diis || o_.diis_size <= kDiisMaxSize) && o_.full_rebuild_every == 0;
        if (device_iter)
            setup_device_iterations();
        for (it = 0; it < o_.max_iter; ++it)
        {
            if (device_iter)
                device_iteration(it);
            else
            {
                const double lastE = energy_;
                fock(it);
                if (o_.use_diis)
                {
                    diis_update();
                    diis_extrapolate();
                }
                diagonalize_update(it);
                dE_ = std::fabs(energy_ - lastE);
                add(T1_, 1.0, Dt_, -1.0, Dtp_);
                dD_ = nrm(T1_);
                if (o_.use_diis)
                    diis_err_ = hist_.empty() ? 0.0 : nrm(hist_.back().e);
            }
            if (o_.verbose)
                std::printf("%15d%15.5e%15.5e%15.5e\n", it + 1, dE_, dD_, diis_err_);
            if (dE_ < o_.energy_tol && dD_ < o_.density_tol && (!o_.use_diis || diis_err_ < o_.diis_tol))
            {
                conv = true;
                break;
            }
        }
        ck(cudaStreamSynchronize(s_), "sync");
        if (device_iter)
        {
            int info = 0;
            ck(cudaMemcpy(&info, info_, sizeof(int), cudaMemcpyDeviceToHost), "d2h");
            if (info != 0)
                throw ScfError(HFG_ERR_CUDA, "scf: syevd did not converge (info " + std::to_string(info) + ")");
            eig_host();
        }
        res.graph_replays = replays_;
        const auto t1 = std::chrono::steady_clock::now();
        res.e_electronic = energy_;
        res.e_nuclear    = enuc_;
        res.e_total      = energy_ + enuc_;
        res.iterations   = conv ? it + 1 : o_.max_iter;
        res.converged    = conv ? 1 : 0;
        res.delta_e      = dE_;
        res.delta_d      = dD_;
        res.diis_error   = diis_err_;
        res.ms_total     = std::chrono::duration<double, std::milli>(t1 - t0).count();
        res.ms_fock      = ms_fock_;
        res.fock_builds  = builds_;
        res.s_squared    = spin_squared();
    }

    // Hands the final densities and the energy-weighted density W = sum_s C_occ eps_occ C_occ^T to the
    // engine for a later hfg_gradient call (the backward half of the forward/backward pair).
    void store_state()
    {
        const size_t N2 = static_cast<size_t>(n_) * n_;
        std::vector<double> Da(N2), Db(N2), W(N2, 0.0), Wt(N2);
        auto wspin = [&](const DMat& C, const DMat& w, int nocc) {
            if (nocc == 0)
                return;
            copy(T1_, C);
            std::vector<double> eps(n_);
            ck(cudaMemcpyAsync(eps.data(), w.p, sizeof(double) * n_, cudaMemcpyDeviceToHost, s_), "d2h");
            ck(cudaStreamSynchronize(s_), "sync");
            for (int i = 0; i < nocc; ++i)
                ck(cublasDscal(cb_, n_, &eps[i], T1_.p + static_cast<size_t>(i) * n_, 1), "scal");
            gemm(CUBLAS_OP_N, CUBLAS_OP_T, n_, n_, nocc, 1.0, T1_.p, C.p, 0.0, T2_.p);
            ck(cudaMemcpyAsync(Wt.data(), T2_.p, sizeof(double) * N2, cudaMemcpyDeviceToHost, s_), "d2h");
            ck(cudaStreamSynchronize(s_), "sync");
            for (size_t k = 0; k < N2; ++k) W[k] += Wt[k];
        };
        wspin(Ca_, wa_, nocc_a_);
        if (uhf_)
            wspin(Cb_, wb_, nocc_b_);
        else
            for (size_t k = 0; k < N2; ++k) W[k] *= 2.0;
        ck(cudaMemcpyAsync(Da.data(), Da_.p, sizeof(double) * N2, cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaMemcpyAsync(Db.data(), Db_.p, sizeof(double) * N2, cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaStreamSynchronize(s_), "sync");
        engine_store_scf_state(eng_, Da.data(), Db.data(), W.data(), uhf_);
    }

    void download(double* Da, double* Db)
    {
        const size_t N2 = static_cast<size_t>(n_) * n_;
        if (Da)
            ck(cudaMemcpyAsync(Da, Da_.p, sizeof(double) * N2, cudaMemcpyDeviceToHost, s_), "d2h");
        if (Db)
            ck(cudaMemcpyAsync(Db, Db_.p, sizeof(double) * N2, cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaStreamSynchronize(s_), "sync");
    }

  private:
    struct Hist
    {
        DMat Fa, Fb, e;
    };

    hfg_engine* eng_;
    hfg_scf_options o_;
    int n_ = 0, nocc_a_ = 0, nocc_b_ = 0;
    bool uhf_ = false;
    double enuc_ = 0.0, energy_ = 0.0, dE_ = 0.0, dD_ = 0.0, diis_err_ = 0.0, ms_fock_ = 0.0, damp_ = 0.0;
    int builds_ = 0;
    bool ls_a_ = false, ls_b_ = false;
    std::vector<double> wa_h_, wb_h_;
    cudaStream_t s_ = nullptr;
    cublasHandle_t cb_ = nullptr;
    cusolverDnHandle_t cs_ = nullptr;
    DMat S_, X_, h_, Fa_, Fb_, Fap_, Fbp_, Da_, Db_, Dap_, Dbp_, Dt_, Dtp_, Ca_, Cb_, T1_, T2_, J_, Ka_, Kb_, dDt_, dDa_,
        dDb_, e_, wa_, wb_, work_;
    int lwork_ = 0;
    int* info_ = nullptr;
    std::deque<Hist> hist_;

    void up(DMat& d, const std::vector<double>& h)
    {
        ck(cudaMemcpyAsync(d.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s_), "h2d");
    }
    void copy(DMat& d, const DMat& s)
    {
        ck(cudaMemcpyAsync(d.p, s.p, sizeof(double) * static_cast<size_t>(n_) * n_, cudaMemcpyDeviceToDevice, s_), "d2d");
    }
    void copy_vec(DMat& d, const DMat& s)
    {
        ck(cudaMemcpyAsync(d.p, s.p, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s_), "d2d");
    }
    void zero(DMat& d) { ck(cudaMemsetAsync(d.p, 0, sizeof(double) * static_cast<size_t>(n_) * n_, s_), "memset"); }
    // d = a*A + b*B
    void add(DMat& d, double a, const DMat& A, double b, const DMat& B)
    {
        ck(cublasDgeam(cb_, CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, &a, A.p, n_, &b, B.p, n_, d.p, n_), "geam");
    }
    // C = alpha op(A) op(B) + beta C, inner dimension k
    void gemm(cublasOperation_t ta, cublasOperation_t tb, int m, int nn, int k, double alpha, const double* A,
              const double* B, double beta, double* C)
    {
        ck(cublasDgemm(cb_, ta, tb, m, nn, k, &alpha, A, n_, B, n_, &beta, C, n_), "gemm");
    }
    double dot(const DMat& A, const DMat& B)
    {
        double r = 0.0;
        ck(cublasDdot(cb_, n_ * n_, A.p, 1, B.p, 1, &r), "dot");
        return r;
    }
    double nrm(const DMat& A)
    {
        double r = 0.0;
        ck(cublasDnrm2(cb_, n_ * n_, A.p, 1, &r), "nrm2");
        return r;
    }
    // Symmetric eigen-decomposition in place: A -> eigenvectors, w ascending.
    void syevd(double* A, double* w)
    {
        ck(cusolverDnDsyevd(cs_, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n_, A, n_, w, work_.p, lwork_, info_),
           "syevd");
        int info = 0;
        ck(cudaMemcpyAsync(&info, info_, sizeof(int), cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaStreamSynchronize(s_), "sync");
        if (info != 0)
            throw ScfError(HFG_ERR_CUDA, "scf: syevd did not converge (info " + std::to_string(info) + ")");
    }
    // X = S^{-1/2} by eigen-decomposition, zero for non-positive eigenvalues (Utils.cpp:117-138).
    void inverse_sqrt()
    {
        copy(T1_, S_);
        syevd(T1_.p, wa_.p);
        std::vector<double> w(n_);
        ck(cudaMemcpyAsync(w.data(), wa_.p, sizeof(double) * n_, cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaStreamSynchronize(s_), "sync");
        // T2 = U diag(w^-1/2)
        copy(T2_, T1_);
        for (int i = 0; i < n_; ++i)
        {
            const double f = w[i] > 0 ? 1.0 / std::sqrt(w[i]) : 0.0;
            ck(cublasDscal(cb_, n_, &f, T2_.p + static_cast<size_t>(i) * n_, 1), "scal");
        }
        gemm(CUBLAS_OP_N, CUBLAS_OP_T, n_, n_, n_, 1.0, T2_.p, T1_.p, 0.0, X_.p);
    }
    // F' = X^T F X (+ level shift), eigenvectors C = X C', eigenvalues w (SCF.cpp:764-791).
    void eig_orth(const DMat& F, DMat& C, DMat& w, bool shift, const DMat* Cprev = nullptr, int nocc = 0)
    {
        gemm(CUBLAS_OP_T, CUBLAS_OP_N, n_, n_, n_, 1.0, X_.p, F.p, 0.0, T2_.p);
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, T2_.p, X_.p, 0.0, T1_.p);
        if (shift && Cprev)
        {
            // M = X S C_prev; F' += levelShift * M[:, nocc:] M[:, nocc:]^T
            gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, X_.p, S_.p, 0.0, T2_.p);
            gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, T2_.p, Cprev->p, 0.0, e_.p);
            const int nv = n_ - nocc;
            if (nv > 0)
                gemm(CUBLAS_OP_N, CUBLAS_OP_T, n_, n_, nv, o_.level_shift, e_.p + static_cast<size_t>(nocc) * n_,
                     e_.p + static_cast<size_t>(nocc) * n_, 1.0, T1_.p);
        }
        syevd(T1_.p, w.p);
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, X_.p, T1_.p, 0.0, C.p);
    }
    // D = (1 - c) C_occ C_occ^T + c D
    void density(const DMat& C, int nocc, DMat& D, double c)
    {
        if (nocc == 0)
        {
            const double f = c;
            ck(cublasDscal(cb_, n_ * n_, &f, D.p, 1), "scal");
            return;
        }
        gemm(CUBLAS_OP_N, CUBLAS_OP_T, n_, n_, nocc, 1.0 - c, C.p, C.p, c, D.p);
    }
    double electronic_energy()
    {
        add(T1_, 1.0, h_, 1.0, Fa_);
        double E = 0.5 * dot(Da_, T1_);
        add(T1_, 1.0, h_, 1.0, Fb_);
        E += 0.5 * dot(Db_, T1_);
        return E;
    }
    void eig_host()
    {
        wa_h_.resize(n_);
        wb_h_.resize(n_);
        ck(cudaMemcpyAsync(wa_h_.data(), wa_.p, sizeof(double) * n_, cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaMemcpyAsync(wb_h_.data(), wb_.p, sizeof(double) * n_, cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaStreamSynchronize(s_), "sync");
    }
    // SCF::buildFockMatrixDirect with the GPU build; F = F_prev + J - K (SCF.cpp:731-743).  DIRECT FALSE:
    // SCF::buildFockMatrix from the stored integrals, F = h + J[D] - K[D] (SCF.cpp:233-521).
    void fock(int it)
    {
        const bool conv = o_.direct == 0;
        const bool full = conv || (o_.full_rebuild_every > 0 && it > 0 && it % o_.full_rebuild_every == 0);
        if (full)
        {
            copy(dDt_, Dt_);
            copy(dDa_, Da_);
            copy(dDb_, Db_);
        }
        else
        {
            add(dDt_, 1.0, Dt_, -1.0, Dtp_);
            add(dDa_, 1.0, Da_, -1.0, Dap_);
            if (uhf_)
                add(dDb_, 1.0, Db_, -1.0, Dbp_);
        }
        hfg_fock_request r {};
        r.unrestricted       = uhf_ ? 1 : 0;
        r.precision          = o_.precision;
        r.device_pointers    = 1;
        r.schwartz_threshold = o_.schwartz_threshold;
        r.density_threshold  = o_.density_threshold;
        r.fp32_cutoff        = o_.fp32_cutoff;
        r.dD_tot             = dDt_.p;
        r.dD_alpha           = dDa_.p;
        r.dD_beta            = uhf_ ? dDb_.p : nullptr;
        r.J                  = J_.p;
        r.K_alpha            = Ka_.p;
        r.K_beta             = uhf_ ? Kb_.p : nullptr;
        hfg_fock_stats st {};
        const int rc = conv ? hfg_fock_conventional(eng_, &r, &st) : hfg_fock_direct(eng_, &r, &st);
        if (rc != HFG_OK)
            throw ScfError(rc, std::string("scf: Fock build failed: ") + hfg_last_error(eng_));
        ms_fock_ += st.ms_total;
        ++builds_;
        const DMat& base_a = full ? h_ : Fap_;
        add(Fa_, 1.0, base_a, 1.0, J_);
        add(Fa_, 1.0, Fa_, -1.0, Ka_);
        copy(Fap_, Fa_);
        if (uhf_)
        {
            const DMat& base_b = full ? h_ : Fbp_;
            add(Fb_, 1.0, base_b, 1.0, J_);
            add(Fb_, 1.0, Fb_, -1.0, Kb_);
            copy(Fbp_, Fb_);
        }
        else
        {
            copy(Fb_, Fa_);
            copy(Fbp_, Fap_);
        }
    }
    // e = F_a D_a S - S D_a F_a + (beta), history of at most diis_size entries (DIIS.cpp:12-26).
    void diis_update()
    {
        Hist h;
        h.Fa.alloc(static_cast<size_t>(n_) * n_);
        h.Fb.alloc(static_cast<size_t>(n_) * n_);
        h.e.alloc(static_cast<size_t>(n_) * n_);
        auto comm = [&](const DMat& F, const DMat& D, double beta) {
            gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, F.p, D.p, 0.0, T1_.p);
            gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, T1_.p, S_.p, 0.0, T2_.p);
            // h.e = beta * h.e + T2 - T2^T  (S D F = (F D S)^T for symmetric F, D, S)
            const double one = 1.0, mone = -1.0;
            ck(cublasDgeam(cb_, CUBLAS_OP_N, CUBLAS_OP_T, n_, n_, &one, T2_.p, n_, &mone, T2_.p, n_, T1_.p, n_), "geam");
            if (beta == 0.0)
                copy(h.e, T1_);
            else
                add(h.e, 1.0, h.e, 1.0, T1_);
        };
        comm(Fa_, Da_, 0.0);
        comm(Fb_, Db_, 1.0);
        copy(h.Fa, Fa_);
        copy(h.Fb, Fb_);
        if (static_cast<int>(hist_.size()) >= o_.diis_size)
            hist_.pop_front();
        hist_.push_back(std::move(h));
    }
    // Bordered B c = (0, .., 0, -1), F = sum c_i F_i (DIIS.cpp:28-72).
    void diis_extrapolate()
    {
        const int m = static_cast<int>(hist_.size());
        if (m == 0)
            return;
        std::vector<double> B(static_cast<size_t>(m + 1) * (m + 1), 0.0), rhs(m + 1, 0.0);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j <= i; ++j)
                B[i + j * (m + 1)] = B[j + i * (m + 1)] = dot(hist_[i].e, hist_[j].e);
        for (int i = 0; i < m; ++i) B[m + i * (m + 1)] = B[i + m * (m + 1)] = -1.0;
        B[m + m * (m + 1)] = 0.0;
        rhs[m]            = -1.0;
        const std::vector<double> c = solve(B, rhs, m + 1);
        zero(Fa_);
        zero(Fb_);
        for (int i = 0; i < m; ++i)
        {
            ck(cublasDaxpy(cb_, n_ * n_, &c[i], hist_[i].Fa.p, 1, Fa_.p, 1), "axpy");
            ck(cublasDaxpy(cb_, n_ * n_, &c[i], hist_[i].Fb.p, 1, Fb_.p, 1), "axpy");
        }
    }
    // Gaussian elimination with complete pivoting (stands in for Eigen's colPivHouseholderQr().solve()).
    static std::vector<double> solve(std::vector<double> A, std::vector<double> b, int n)
    {
        std::vector<int> perm(n);
        for (int i = 0; i < n; ++i) perm[i] = i;
        auto at = [&](int i, int j) -> double& { return A[i + static_cast<size_t>(j) * n]; };
        int rank = n;
        for (int k = 0; k < n; ++k)
        {
            int pi = k, pj = k;
            double best = 0.0;
            for (int j = k; j < n; ++j)
                for (int i = k; i < n; ++i)
                    if (std::fabs(at(i, j)) > best)
                    {
                        best = std::fabs(at(i, j));
                        pi   = i;
                        pj   = j;
                    }
            if (best == 0.0)
            {
                rank = k;
                break;
            }
            for (int j = 0; j < n; ++j) std::swap(at(k, j), at(pi, j));
            std::swap(b[k], b[pi]);
            for (int i = 0; i < n; ++i) std::swap(at(i, k), at(i, pj));
            std::swap(perm[k], perm[pj]);
            for (int i = k + 1; i < n; ++i)
            {
                const double f = at(i, k) / at(k, k);
                for (int j = k; j < n; ++j) at(i, j) -= f * at(k, j);
                b[i] -= f * b[k];
            }
        }
        std::vector<double> y(n, 0.0), x(n, 0.0);
        for (int k = rank - 1; k >= 0; --k)
        {
            double s = b[k];
            for (int j = k + 1; j < rank; ++j) s -= at(k, j) * y[j];
            y[k] = s / at(k, k);
        }
        for (int k = 0; k < n; ++k) x[perm[k]] = y[k];
        return x;
    }
    // SCF.cpp:747-835.
    void diagonalize_update(int it)
    {
        if (o_.damp > 0 && o_.max_damp_iter != 0 && o_.max_damp_iter > it && (dE_ > o_.stop_damp_thresh || it == 0))
            damp_ = o_.damp / 100.0;
        else
            damp_ = 0.0;
        if (o_.level_shift > 0 && it < o_.max_lshift_iter && (dE_ > o_.stop_lshift_thresh || it == 0))
        {
            ls_a_ = (wa_h_[nocc_a_] - wa_h_[nocc_a_ - 1]) < o_.lshift_gap_tol;
            ls_b_ = (nocc_b_ >= 1 ? (wb_h_[nocc_b_] - wb_h_[nocc_b_ - 1]) : 0.0) < o_.lshift_gap_tol;
        }
        else
        {
            ls_a_ = ls_b_ = false;
        }
        // alpha
        {
            DMat Cprev(static_cast<size_t>(n_) * n_);
            copy(Cprev, Ca_);
            eig_orth(Fa_, Ca_, wa_, ls_a_, &Cprev, nocc_a_);
        }
        copy(Dap_, Da_);
        density(Ca_, nocc_a_, Da_, damp_);
        copy(Dbp_, Db_);
        if (uhf_)
        {
            DMat Cprev(static_cast<size_t>(n_) * n_);
            copy(Cprev, Cb_);
            eig_orth(Fb_, Cb_, wb_, ls_b_, &Cprev, nocc_b_);
            density(Cb_, nocc_b_, Db_, damp_);
        }
        else
        {
            copy(Cb_, Ca_);
            copy_vec(wb_, wa_);
            copy(Db_, Da_);
        }
        copy(Dtp_, Dt_);
        add(Dt_, 1.0, Da_, 1.0, Db_);
        energy_ = electronic_energy();
        eig_host();
    }
    // ---- Device iterations (graph_iterations): DIIS, energy and convergence measures on the GPU ----------
    DMat ring_[3 * kDiisMaxSize];        // DIIS slots: F_alpha, F_beta, e
    DMat Bm_, part_, wsc_a_, wsc_b_, dd_; // B per slot pair, partial sums, energy operands, density change
    DiisState* dstate_   = nullptr;
    ScfScalars* dsc_     = nullptr;
    ScfScalars* hsc_     = nullptr; // pinned
    const double** dptr_ = nullptr; // device pointer tables: [cap] x_e, [cap] y_slots, [3] xs, [3] ys
    void* cublas_ws_     = nullptr;
    DiisDevice dd_dev_ {};
    MeasureDevice md_ {};
    cudaGraph_t seg_graph_[3] {};
    cudaGraphExec_t seg_exec_[3] {};
    bool graph_failed_ = false;
    int replays_                = 0;
    cudaEvent_t gev_[2] {};

    void setup_device_iterations()
    {
        const size_t N2 = static_cast<size_t>(n_) * n_;
        const int cap   = o_.use_diis ? o_.diis_size : 1;
        int sms = 0, dev = 0;
        ck(cudaGetDevice(&dev), "device");
        ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
        const int nblk = dot_blocks(sms);
        for (int k = 0; k < 3 * cap; ++k)
        {
            ring_[k].alloc(N2);
            ck(cudaMemsetAsync(ring_[k].p, 0, sizeof(double) * N2, s_), "memset");
        }
        Bm_.alloc(static_cast<size_t>(cap) * cap);
        ck(cudaMemsetAsync(Bm_.p, 0, sizeof(double) * cap * cap, s_), "memset");
        part_.alloc(static_cast<size_t>(std::max(cap, 3)) * nblk);
        wsc_a_.alloc(N2);
        wsc_b_.alloc(N2);
        dd_.alloc(N2);
        ck(cudaMalloc(&dstate_, sizeof(DiisState)), "cudaMalloc");
        ck(cudaMalloc(&dsc_, sizeof(ScfScalars)), "cudaMalloc");
        ck(cudaMallocHost(&hsc_, sizeof(ScfScalars)), "cudaMallocHost");
        ck(cudaMalloc(&dptr_, sizeof(double*) * (2 * cap + 6)), "cudaMalloc");
        DiisState st {};
        st.cap = cap;
        ck(cudaMemcpyAsync(dstate_, &st, sizeof(st), cudaMemcpyHostToDevice, s_), "h2d");
        std::vector<const double*> tab(2 * cap + 6);
        for (int k = 0; k < cap; ++k)
        {
            tab[k]       = e_.p; // the new error vector, built in e_ every iteration
            tab[cap + k] = ring_[2 * cap + k].p;
        }
        tab[2 * cap + 0] = Da_.p;
        tab[2 * cap + 1] = Db_.p;
        tab[2 * cap + 2] = dd_.p;
        tab[2 * cap + 3] = wsc_a_.p;
        tab[2 * cap + 4] = wsc_b_.p;
        tab[2 * cap + 5] = dd_.p;
        ck(cudaMemcpyAsync(dptr_, tab.data(), sizeof(double*) * tab.size(), cudaMemcpyHostToDevice, s_), "h2d");
        dd_dev_.state = dstate_;
        for (int k = 0; k < cap; ++k)
        {
            dd_dev_.slots.Fa[k] = ring_[k].p;
            dd_dev_.slots.Fb[k] = ring_[cap + k].p;
            dd_dev_.slots.e[k]  = ring_[2 * cap + k].p;
        }
        dd_dev_.B        = Bm_.p;
        dd_dev_.xs_e     = dptr_;
        dd_dev_.ys_slots = dptr_ + cap;
        dd_dev_.part     = part_.p;
        dd_dev_.cap      = cap;
        dd_dev_.nblk     = nblk;
        dd_dev_.num_sms  = sms;
        md_ = MeasureDevice {h_.p, Fa_.p, Fb_.p, Dt_.p, Dtp_.p, wsc_a_.p, wsc_b_.p, dd_.p, dptr_ + 2 * cap,
                             dptr_ + 2 * cap + 3, part_.p, dsc_, nblk, sms};
        // cuBLAS gets its own workspace, so that no call inside a capture allocates.
        const size_t ws = 32u << 20;
        ck(cudaMalloc(&cublas_ws_, ws), "cudaMalloc");
        ck(cublasSetWorkspace(cb_, cublas_ws_, ws), "cublasSetWorkspace");
        for (auto& ev : gev_) ck(cudaEventCreate(&ev), "event");
        engine_prepare_capture(eng_);
        // The guess's energy is the first "previous" energy of the measures.
        ck(scf_measures(md_, static_cast<long long>(N2), s_), "measures");
    }

    void free_device_iterations()
    {
        for (int k = 0; k < 3; ++k)
        {
            if (seg_exec_[k])
                cudaGraphExecDestroy(seg_exec_[k]);
            if (seg_graph_[k])
                cudaGraphDestroy(seg_graph_[k]);
        }
        for (auto& ev : gev_)
            if (ev)
                cudaEventDestroy(ev);
        if (dstate_)
            cudaFree(dstate_);
        if (dsc_)
            cudaFree(dsc_);
        if (hsc_)
            cudaFreeHost(hsc_);
        if (dptr_)
            cudaFree(dptr_);
        if (cublas_ws_)
            cudaFree(cublas_ws_);
    }

    // One iteration is enqueued as segments separated by the eigensolver calls, because cuSOLVER's syevd
    // refuses stream capture (and a refused capture leaves its handle unusable, so it is never attempted):
    //   segment 0   dD, the Fock build, F = F_prev + J - K, DIIS (device), F'_alpha = X^T F_alpha X
    //   syevd(F'_alpha)                                                                   (eager)
    //   segment 1   C_alpha, D_alpha; RHF: the beta copies, D_tot, the measures; UHF: F'_beta = X^T F_beta X
    //   UHF: syevd(F'_beta), segment 2   C_beta, D_beta, D_tot, the measures
    // No segment synchronises with the host, so from the second iteration on each one is captured once and
    // replayed (`capture`: enqueue into the capture that is open on the stream).
    void segment(int k, bool capture)
    {
        const long long N2 = static_cast<long long>(n_) * n_;
        if (k == 0)
        {
            add(dDt_, 1.0, Dt_, -1.0, Dtp_);
            add(dDa_, 1.0, Da_, -1.0, Dap_);
            if (uhf_)
                add(dDb_, 1.0, Db_, -1.0, Dbp_);
            hfg_fock_request r {};
            r.unrestricted       = uhf_ ? 1 : 0;
            r.precision          = o_.precision;
            r.device_pointers    = 1;
            r.schwartz_threshold = o_.schwartz_threshold;
            r.density_threshold  = o_.density_threshold;
            r.fp32_cutoff        = o_.fp32_cutoff;
            r.dD_tot             = dDt_.p;
            r.dD_alpha           = dDa_.p;
            r.dD_beta            = uhf_ ? dDb_.p : nullptr;
            r.J                  = J_.p;
            r.K_alpha            = Ka_.p;
            r.K_beta             = uhf_ ? Kb_.p : nullptr;
            if (capture)
            {
                ck(cudaEventRecord(gev_[0], s_), "event");
                const int rc = engine_guarded(eng_, [&] { engine_enqueue_fock(eng_, r); });
                if (rc != HFG_OK)
                    throw ScfError(rc, std::string("scf: Fock build failed: ") + hfg_last_error(eng_));
                ck(cudaEventRecord(gev_[1], s_), "event");
            }
            else
            {
                hfg_fock_stats st {};
                const int rc = hfg_fock_direct(eng_, &r, &st);
                if (rc != HFG_OK)
                    throw ScfError(rc, std::string("scf: Fock build failed: ") + hfg_last_error(eng_));
                ms_fock_ += st.ms_total;
            }
            add(Fa_, 1.0, Fap_, 1.0, J_);
            add(Fa_, 1.0, Fa_, -1.0, Ka_);
            copy(Fap_, Fa_);
            if (uhf_)
            {
                add(Fb_, 1.0, Fbp_, 1.0, J_);
                add(Fb_, 1.0, Fb_, -1.0, Kb_);
                copy(Fbp_, Fb_);
            }
            else
            {
                copy(Fb_, Fa_);
                copy(Fbp_, Fap_);
            }
            if (o_.use_diis)
            {
                // e = (F_a D_a S - S D_a F_a) + (beta) into e_, as diis_update does.
                const double one = 1.0, mone = -1.0;
                auto comm = [&](const DMat& F, const DMat& D, bool accumulate) {
                    gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, F.p, D.p, 0.0, T1_.p);
                    gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, T1_.p, S_.p, 0.0, T2_.p);
                    ck(cublasDgeam(cb_, CUBLAS_OP_N, CUBLAS_OP_T, n_, n_, &one, T2_.p, n_, &mone, T2_.p, n_, T1_.p, n_),
                       "geam");
                    if (accumulate)
                        add(e_, 1.0, e_, 1.0, T1_);
                    else
                        copy(e_, T1_);
                };
                comm(Fa_, Da_, false);
                comm(Fb_, Db_, true);
                ck(hfg::diis_push(dd_dev_, Fa_.p, Fb_.p, e_.p, N2, s_), "diis_push");
                ck(hfg::diis_extrapolate(dd_dev_, Fa_.p, Fb_.p, dsc_, N2, s_), "diis_extrapolate");
            }
            orth(Fa_); // F'_alpha into T1
            return;
        }
        // Orbital step (SCF.cpp:747-835 without damping and level shifting).
        const bool alpha = k == 1;
        DMat& C = alpha ? Ca_ : Cb_;
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, X_.p, T1_.p, 0.0, C.p);
        if (alpha)
        {
            copy(Dap_, Da_);
            density(Ca_, nocc_a_, Da_, 0.0);
            copy(Dbp_, Db_);
            if (uhf_)
            {
                orth(Fb_); // F'_beta into T1 for the next eigensolve
                return;
            }
            copy(Cb_, Ca_);
            copy_vec(wb_, wa_);
            copy(Db_, Da_);
        }
        else
            density(Cb_, nocc_b_, Db_, 0.0);
        copy(Dtp_, Dt_);
        add(Dt_, 1.0, Da_, 1.0, Db_);
        ck(scf_measures(md_, N2, s_), "measures");
        ck(cudaMemcpyAsync(hsc_, dsc_, sizeof(ScfScalars), cudaMemcpyDeviceToHost, s_), "d2h");
    }

    // T1 = X^T F X.
    void orth(const DMat& F)
    {
        gemm(CUBLAS_OP_T, CUBLAS_OP_N, n_, n_, n_, 1.0, X_.p, F.p, 0.0, T2_.p);
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, n_, n_, n_, 1.0, T2_.p, X_.p, 0.0, T1_.p);
    }

    // Eigenvectors of T1 in place, eigenvalues into w (its status is checked after the iterations).
    void eigensolve(DMat& w)
    {
        ck(cusolverDnDsyevd(cs_, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n_, T1_.p, n_, w.p, work_.p, lwork_,
                            info_),
           "syevd");
    }

    void read_measures()
    {
        ck(cudaStreamSynchronize(s_), "sync");
        energy_ = hsc_->energy;
        dE_     = hsc_->delta_e;
        dD_     = hsc_->delta_d;
        if (o_.use_diis)
            diis_err_ = hsc_->diis_error;
    }

    // Captures segment k (nothing of it runs); false if the capture was refused.
    bool capture_segment(int k)
    {
        ck(cudaStreamBeginCapture(s_, cudaStreamCaptureModeRelaxed), "begin capture");
        bool ok = true;
        try
        {
            segment(k, true);
        }
        catch (const ScfError&)
        {
            ok = false;
        }
        cudaGraph_t g       = nullptr;
        const cudaError_t e = cudaStreamEndCapture(s_, &g);
        if (ok && e == cudaSuccess && g && cudaGraphInstantiate(&seg_exec_[k], g, 0) == cudaSuccess)
        {
            seg_graph_[k] = g;
            return true;
        }
        if (g)
            cudaGraphDestroy(g);
        seg_exec_[k] = nullptr;
        cudaGetLastError(); // clear the refused capture's error state
        return false;
    }

    void device_iteration(int it)
    {
        ++builds_;
        const int nseg = uhf_ ? 3 : 2;
        if (it > 0 && !seg_exec_[0] && !graph_failed_)
            for (int k = 0; k < nseg && !graph_failed_; ++k)
                graph_failed_ = !capture_segment(k);
        const bool replay = !graph_failed_ && seg_exec_[0];
        for (int k = 0; k < nseg; ++k)
        {
            if (replay)
                ck(cudaGraphLaunch(seg_exec_[k], s_), "graph launch");
            else
                segment(k, false);
            if (k + 1 < nseg)
                eigensolve(k == 0 ? wa_ : wb_);
        }
        read_measures();
        if (replay)
        {
            const int rc = engine_guarded(eng_, [&] { engine_check_counts(eng_, o_.precision == HFG_PRECISION_MIXED); });
            if (rc != HFG_OK)
                throw ScfError(rc, std::string("scf: Fock build failed: ") + hfg_last_error(eng_));
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, gev_[0], gev_[1]) == cudaSuccess)
                ms_fock_ += ms;
            ++replays_;
        }
    }

    // <S^2> = Sz(Sz+1) + N_beta - |C_a,occ^T S C_b,occ|^2 (SCF.cpp:838-845).
    double spin_squared()
    {
        const double Sz = 0.5 * (nocc_a_ - nocc_b_);
        if (nocc_b_ == 0)
            return Sz * (Sz + 1.0);
        gemm(CUBLAS_OP_T, CUBLAS_OP_N, nocc_a_, n_, n_, 1.0, Ca_.p, S_.p, 0.0, T1_.p);
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, nocc_a_, nocc_b_, n_, 1.0, T1_.p, Cb_.p, 0.0, T2_.p);
        double s = 0.0;
        std::vector<double> M(static_cast<size_t>(n_) * nocc_b_);
        ck(cudaMemcpyAsync(M.data(), T2_.p, sizeof(double) * M.size(), cudaMemcpyDeviceToHost, s_), "d2h");
        ck(cudaStreamSynchronize(s_), "sync");
        for (int j = 0; j < nocc_b_; ++j)
            for (int i = 0; i < nocc_a_; ++i) s += M[i + static_cast<size_t>(j) * n_] * M[i + static_cast<size_t>(j) * n_];
        return Sz * (Sz + 1.0) + nocc_b_ - s;
    }
};

template <typename F> int scf_guarded(hfg_engine* e, F&& f)
{
    try
    {
        f();
        return HFG_OK;
    }
    catch (const ScfError& x)
    {
        engine_set_error(e, x.what());
        return x.code;
    }
    catch (const std::bad_alloc&)
    {
        engine_set_error(e, "host allocation failed");
        return HFG_ERR_NOMEM;
    }
    catch (const std::exception& x)
    {
        engine_set_error(e, x.what());
        return HFG_ERR_INVALID;
    }
}
} // namespace
} // namespace hfg

extern "C" {

void hfg_scf_default_options(hfg_scf_options* o, int multiplicity)
{
    if (!o)
        return;
    *o                    = hfg_scf_options {};
    o->max_iter           = 30;
    o->energy_tol         = 1e-6;
    o->density_tol        = 1e-6;
    o->use_diis           = 1;
    o->diis_size          = 6;
    o->diis_tol           = 1e-6;
    o->unrestricted       = multiplicity != 1 ? 1 : 0;
    o->guess_mix          = 0;
    o->damp               = 0;
    o->max_damp_iter      = o->max_iter;
    o->stop_damp_thresh   = 0.0;
    o->level_shift        = 0.0;
    o->lshift_gap_tol     = std::numeric_limits<double>::infinity();
    o->max_lshift_iter    = o->max_iter;
    o->stop_lshift_thresh = 0.0;
    o->schwartz_threshold = 1e-10;
    o->density_threshold  = 1e-10;
    o->precision          = HFG_PRECISION_FP64;
    o->fp32_cutoff        = 2e-4; // tuned on (H2O)_64 RHF/6-31G**: SCF |dE| 3.6e-8 Eh vs FP64 (1e-4: 6.0e-8, 3e-4: 1.2e-7)
    o->full_rebuild_every = 0;
    o->verbose            = 0;
    o->graph_iterations   = 0;
    o->direct             = 1;
}

int hfg_scf_run(hfg_engine* e, const hfg_scf_options* opt, int natom, const int* Z, const double* xyz, int charge,
                int multiplicity, hfg_scf_result* res, double* Da, double* Db)
{
    if (!e || !opt || !res || natom <= 0 || !Z || !xyz)
        return HFG_ERR_INVALID;
    if (opt->max_iter < 0 || opt->diis_size < 1 || opt->damp < 0 || opt->damp > 100 || opt->guess_mix < 0)
        return HFG_ERR_INVALID;
    return hfg::scf_guarded(e, [&] {
        *res = hfg_scf_result {};
        hfg::Scf scf(e, *opt, natom, Z, xyz, charge, multiplicity);
        scf.run(*res);
        scf.store_state();
        scf.download(Da, Db);
    });
}

int hfg_core_guess(hfg_engine* e, const hfg_scf_options* opt, int natom, const int* Z, const double* xyz, int charge,
                   int multiplicity, double* Da, double* Db)
{
    if (!e || !opt || natom <= 0 || !Z || !xyz)
        return HFG_ERR_INVALID;
    return hfg::scf_guarded(e, [&] {
        hfg::Scf scf(e, *opt, natom, Z, xyz, charge, multiplicity);
        scf.guess();
        scf.download(Da, Db);
    });
}
}
