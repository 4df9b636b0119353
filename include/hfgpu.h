/*
 * hfgpu -- GB300 direct-SCF two-electron (Fock-build) engine: C ABI.
 *
 * This is the drop-in boundary for the two-electron path of the reference Hartree-Fock program
 * (MalachiF1/Hartree-Fock).  The reference has no plugin API; its boundary is the C++ class API of
 * IntegralEngine and the private SCF::buildFockMatrixDirect.  Each entry point below names the
 * reference interface it replaces.  Plain pointers and sizes only; matrices are column-major
 * n x n FP64, exactly Eigen::MatrixXd's layout in the reference.
 *
 * Conventions: every function returns HFG_OK (0) or a negative HFG_ERR_* code and never aborts;
 * hfg_last_error() describes the last failure.  Calls on one engine are not thread-safe; the engine
 * keeps no caller pointer after a call returns.  Host-pointer calls synchronise before returning.
 */
#ifndef HFGPU_H
#define HFGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HFG_OK 0
#define HFG_ERR_INVALID -1     /* bad argument (null pointer, size, threshold) */
#define HFG_ERR_CUDA -2        /* CUDA runtime failure (message in hfg_last_error) */
#define HFG_ERR_BASIS -3       /* basis data inconsistent (offsets, normalisation factors) */
#define HFG_ERR_UNSUPPORTED -4 /* angular momentum above d, or a feature not built */
#define HFG_ERR_NOMEM -5       /* device or host allocation failed */
#define HFG_ERR_OVERFLOW -6    /* a quartet list exceeded its capacity (internal) */

#define HFG_PRECISION_FP64 0  /* every surviving quartet in FP64 */
#define HFG_PRECISION_MIXED 1 /* quartets with bound below fp32_cutoff in FP32, the rest in FP64 */

/* The basis as the reference's IntegralEngine holds it (src/IntegralEngine.cpp:13-75,
 * include/IntegralEngine.hpp:145-168): per shell l, primitive count and offsets, AO offset, offset of
 * its normalisation factors and centre (bohr); per primitive exponent and contraction coefficient;
 * per primitive x AO the normalisation factor (src/Basis.cpp:61-77); per AO the Cartesian exponents.
 * Cartesian order within a shell: x exponent descending, then y descending (src/Basis.cpp:48-59). */
typedef struct hfg_basis
{
    int nshells;
    int nao;
    int nprim;             /* total primitives */
    const int* l;          /* [nshells] */
    const int* nprim_sh;   /* [nshells] */
    const int* prim_off;   /* [nshells] */
    const int* ao_off;     /* [nshells] */
    const int* norm_off;   /* [nshells] */
    const double* centers; /* [nshells][3] */
    const double* alpha;   /* [nprim] */
    const double* coeff;   /* [nprim] */
    const double* norms;   /* [sum_s nprim_sh[s]*nao(l[s])] */
    const int* am;         /* [nao][3] */
} hfg_basis;

typedef struct hfg_engine hfg_engine;

/* One direct Fock build, SCF::buildFockMatrixDirect (src/SCF.cpp:523-744) without the final
 * F = F_prev + J - K, which the caller forms exactly as SCF.cpp:731-743 does.
 * Inputs are the density increments dD = D - D_prev.  Outputs are the full symmetric
 * J[dD_tot], K_alpha[dD_alpha] (and K_beta[dD_beta] when unrestricted).
 * For a batch engine every matrix is the concatenation of the molecules' n_m x n_m blocks. */
typedef struct hfg_fock_request
{
    int unrestricted;          /* 0: RHF (dD_beta and K_beta ignored), 1: UHF */
    int precision;             /* HFG_PRECISION_FP64 or HFG_PRECISION_MIXED */
    int device_pointers;       /* 1: all matrix pointers below are CUDA device pointers */
    double schwartz_threshold; /* SCHWARTZ_THRESH: shell quartet and AO-level skip (SCF.cpp:606, 670) */
    double density_threshold;  /* DENSITY_THRESH (SCF.cpp:610-623) */
    double fp32_cutoff;        /* MIXED: quartets with Q_ab Q_cd max|dD| below this run in FP32 */
    const double* dD_tot;      /* D_tot - D_tot_prev */
    const double* dD_alpha;    /* D_alpha - D_alpha_prev */
    const double* dD_beta;     /* D_beta - D_beta_prev (UHF) */
    double* J;
    double* K_alpha;
    double* K_beta; /* UHF */
} hfg_fock_request;

#define HFG_NUM_CLASSES 21 /* shell-quartet classes (la lb | lc ld) for s, p, d */

typedef struct hfg_fock_stats
{
    unsigned long long quartets_fp64[HFG_NUM_CLASSES]; /* surviving shell quartets per class */
    unsigned long long quartets_fp32[HFG_NUM_CLASSES];
    unsigned long long prim_quartets_fp64[HFG_NUM_CLASSES]; /* primitive quartets evaluated */
    unsigned long long prim_quartets_fp32[HFG_NUM_CLASSES];
    double flops_fp64;  /* algorithmic FP64 flops of the build (work model of the engine docs) */
    double flops_fp32;
    double ms_total;    /* device time of the build, list building to symmetrisation */
    double ms_lists;    /* device time of screening + list building */
    double ms_eri_fp64; /* device time of the FP64 class kernels */
    double ms_eri_fp32; /* device time of the FP32 class kernels */
    int kernel_launches;
    int form_fp64[HFG_NUM_CLASSES]; /* kernel form each class ran in (HFG_FORM_*; 0 = class not launched) */
    int form_fp32[HFG_NUM_CLASSES];
    double ms_tune;     /* host wall time spent timing kernel forms in this call (first use of a class only) */
    double ms_eri_both; /* mixed builds with overlapped precisions: the span of all class kernels (FP64 and FP32
                           run concurrently, so ms_eri_fp64 and ms_eri_fp32 overlap); 0 otherwise */
} hfg_fock_stats;

/* IntegralEngine::IntegralEngine(const BasisSet&) (include/IntegralEngine.hpp:11).  Packs the basis
 * into device tables (shell pairs, primitive-pair Hermite tables, Boys grids) on `device`. */
int hfg_create(const hfg_basis* basis, int device, hfg_engine** out);

/* A batch of independent molecules in one engine: their Fock builds run in one launch per class.
 * No reference counterpart (the reference handles one molecule per process). */
int hfg_create_batch(const hfg_basis* bases, int nmol, int device, hfg_engine** out);

void hfg_destroy(hfg_engine* engine);

/* Last error message of `engine` (or of the last failed create when engine is NULL). */
const char* hfg_last_error(const hfg_engine* engine);

/* IntegralEngine::schwartzScreeningMatrix (include/IntegralEngine.hpp:32, src/IntegralEngine.cpp:695-728):
 * Q(a,b) = sqrt(max (ab|ab)), nshells x nshells column-major (host pointer).  Batch engines write the
 * molecules' blocks one after another. */
int hfg_schwartz(hfg_engine* engine, double* Q);

/* Replace the engine's Schwartz matrix (host, same layout as hfg_schwartz), e.g. with the reference's
 * own Q so that quartet survival can be compared bit for bit. */
int hfg_set_schwartz(hfg_engine* engine, const double* Q);

/* Primitive-pair screening of the Fock build (no reference counterpart: the reference evaluates every
 * primitive pair of a surviving quartet, src/IntegralEngine.cpp:371-520).  A primitive pair ab enters
 * the build iff sqrt((ab|ab)) * max_cd Q_cd >= threshold, where (ab|ab) is that primitive pair's own
 * Coulomb self-repulsion: by the Cauchy-Schwarz inequality every dropped term of an integral is below
 * the threshold.  Default 1e-15; 0 keeps every primitive pair.  Schwartz bounds and the nuclear
 * gradient always use every primitive pair. */
int hfg_set_primitive_threshold(hfg_engine* engine, double threshold);

/* SCF::buildFockMatrixDirect (include/SCF.hpp:129, src/SCF.cpp:523-744); `stats` may be NULL. */
int hfg_fock_direct(hfg_engine* engine, const hfg_fock_request* req, hfg_fock_stats* stats);

/* IntegralEngine::electronRepulsionTensor (src/IntegralEngine.cpp:635-692), the stored-integral (DIRECT
 * FALSE) path: evaluates every shell quartet whose Schwartz product reaches `schwartz_threshold` once, in
 * FP64, and keeps the integral blocks in device memory (`bytes`, may be NULL, receives their size).  Fails
 * with HFG_ERR_NOMEM when they would need more than 80% of the free device memory. */
int hfg_store_integrals(hfg_engine* engine, double schwartz_threshold, size_t* bytes);

/* SCF::buildFockMatrix (src/SCF.cpp:233-521): J[D] and K[D] of the FULL densities from the stored
 * integrals (the request's dD_tot / dD_alpha / dD_beta carry D_tot, D_alpha, D_beta here), with the
 * reference's AO-level skip |(ij|kl)| < schwartz_threshold; the caller forms F = h + J - K as SCF.cpp:507-520
 * does.  Needs hfg_store_integrals first; `precision` and the density threshold are not used. */
int hfg_fock_conventional(hfg_engine* engine, const hfg_fock_request* req, hfg_fock_stats* stats);

/* Kernel forms of a class kernel.  THREAD: one thread per shell quartet.  WARP: one warp per quartet
 * (the large d classes).  GROUP: a power-of-two group of lanes per quartet, splitting its primitive
 * quartets (the small contracted classes, L <= 3).  AUTO: on the first build that runs the class with
 * enough quartets, every compiled form runs on an evenly spaced sample of the real list and the fastest
 * is kept for the life of the engine (per class, precision and RHF/UHF).
 * No reference counterpart: the reference has one CPU loop (src/SCF.cpp:592-728). */
#define HFG_FORM_AUTO 0
#define HFG_FORM_THREAD 1
#define HFG_FORM_WARP 2
#define HFG_FORM_GROUP 3
#define HFG_FORM_CHUNK 4 /* one thread per (quartet, chunk of ket Cartesian components): the FP32 d classes */
#define HFG_FORM_PERSISTENT 5 /* in hfg_fock_stats only: the class ran in the persistent work queue */
/* Set the form of class `qclass` (-1: every class) at precision `fp32` (0: FP64 kernels, 1: FP32
 * kernels).  HFG_FORM_AUTO forgets earlier timings; a form the class was not compiled in returns
 * HFG_ERR_UNSUPPORTED (with qclass -1 such classes keep AUTO). */
int hfg_set_kernel_form(hfg_engine* engine, int qclass, int fp32, int form);
/* Mixed builds run the FP32 class kernels on a second stream concurrently with the FP64 ones, each grid
 * limited to `share` (0 < share <= 1) of the resident blocks per SM, so that the FP64-pipe bound and
 * the FP32 / memory-latency bound kernels share the SMs.  On by default with share 1 (full grids).  No
 * reference counterpart. */
int hfg_set_precision_overlap(hfg_engine* engine, int on, double share);
/* The same limit set separately for the FP64 and the FP32 class kernels' grids (each in (0, 1]): the FP64
 * kernels keep the FP64 pipe busy with few warps per SM, so a smaller FP64 share leaves the rest of the SM
 * to the FP32 kernels running beside them.  No reference counterpart. */
int hfg_set_precision_shares(hfg_engine* engine, double share_fp64, double share_fp32);

/* CUDA-graph replay of Fock builds (no reference counterpart; the SCF driver calls hfg_fock_direct on
 * device pointers every iteration).  On: a device-pointer request runs eagerly once and is captured
 * with every class kernel at a fixed grid (the kernels read their list lengths on the device); later
 * requests with the same precision, spin case, thresholds, cutoff and matrix pointers replay the
 * graph as one launch.  Changing forms, thresholds or the Schwartz matrix drops the graph.  Replays
 * report ms_total but not its split into lists / FP64 / FP32.  Off by default; host-pointer requests
 * always run eagerly. */
int hfg_set_graph_mode(hfg_engine* engine, int on);

/* Persistent work-queue launch (no reference counterpart; the reference's loop is SCF.cpp:592-728): when on,
 * the quartet lists of (ss|ss), (ps|ss), (ps|ps) and (pp|ss), FP64 and FP32, are worked through by ONE
 * launch whose blocks take 128-quartet items from a shared counter (no block waits on another); the other
 * classes keep their own launches.  Off by default.  Builds with it on or off give the same matrices to
 * rounding (the digestion's atomics sum in a different order). */
int hfg_set_persistent(hfg_engine* engine, int on);

/* Kernel-form autotuning (no reference counterpart): on (default), the first build that runs a class with at
 * least 64k surviving quartets and more than one compiled form times the forms on a sample of its list and
 * keeps the fastest (hfg_kernel_forms reports the picks); off, every class not set by hfg_set_kernel_form
 * runs its default form, with no timing trials (reproducible launch sequences, e.g. under a profiler). */
int hfg_set_autotune(hfg_engine* engine, int on);

/* Gradient kernel form (no reference counterpart): 0 (default) runs the thread-per-quartet gradient kernel
 * for the classes whose per-quartet arrays fit in registers ((ss|ss) (ps|ss) (ps|ps) (pp|ss) (ds|ss) in
 * FP64, and (pp|ps) (ds|ps) (dp|ss) as well in FP32) and the lane-group kernel for the others; 1 runs the
 * lane-group kernel for every class.  Both give the same gradient to rounding. */
int hfg_set_gradient_form(hfg_engine* engine, int group_only);

/* Forms in use: forms[qc] for the given precision and spin case, 0 where AUTO has not decided yet.
 * `available` (may be NULL) receives the bit mask of compiled forms per class (bit f = form f). */
int hfg_kernel_forms(hfg_engine* engine, int fp32, int unrestricted, int forms[HFG_NUM_CLASSES],
                     unsigned available[HFG_NUM_CLASSES]);

/* The surviving canonical shell quartets (a >= b, c >= d, ab >= cd; the reference's loop indices,
 * SCF.cpp:592-623) of the last hfg_fock_direct call, sorted lexicographically, as 4 ints each.
 * Returns the count in *count; writes at most `cap` quartets (quartets may be NULL to query). */
int hfg_survivors(hfg_engine* engine, int* quartets, long long cap, long long* count);

/* IntegralEngine::electronRepulsion(a, b, c, d, std::vector<double>&) (include/IntegralEngine.hpp:26-28,
 * src/IntegralEngine.cpp:731-992): contracted block, row-major [a][b][c][d], full (no zero pattern). */
int hfg_eri_block(hfg_engine* engine, int a, int b, int c, int d, double* out);

/* Allocation-free variant of hfg_eri_block (no counterpart in the reference).  For callers that must not
 * allocate or free device memory per request -- a process that runs under a fixed device-memory budget
 * once its engine exists, or a pipeline whose other streams must not be stalled (hfg_eri_block grows a
 * device buffer per call and frees it, and cudaFree synchronises the whole device).  Same kernel and
 * result as hfg_eri_block (host output, row-major [a][b][c][d]); its scratch is a 16 KB file-scope
 * device array per GPU (held until the process exits), so one block may hold at most 2016 values
 * (every s/p/d block fits; larger requests fail with HFG_ERR_INVALID).  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device current: make that first
 * call before any stream capture.  The address is kept per device for the life of the process: after a
 * cudaDeviceReset the library must be reloaded before this entry point is used again.  Calls on one device
 * share the array: calls that overlap on the GPU (from several host threads or engines at once) race. */
int hfg_eri_block_noalloc(hfg_engine* engine, int a, int b, int c, int d, double* out);

/* The CUDA stream the engine launches on (a cudaStream_t), for callers that time or order work. */
void* hfg_stream(hfg_engine* engine);

/* ---------------------------------------------------------------------------------------------
 * Host side of the SCF (the reference's SCF driver semantics, src/SCF.cpp:23-231 and 747-835),
 * so that a caller can run a whole direct SCF with the GPU Fock build.
 * ------------------------------------------------------------------------------------------- */

/* IntegralEngine::overlapMatrix / kineticMatrix / nuclearAttractionMatrix (src/IntegralEngine.cpp:78-368):
 * S, T, V (FP64, host, column-major nao x nao) for the basis and nuclei Z at xyz (bohr). */
int hfg_one_electron(const hfg_basis* basis, int natom, const int* Z, const double* xyz, double* S, double* T,
                     double* V);

/* The same S, T, V computed on the GPU of `engine` (its single molecule's basis), FP64, host outputs.  The
 * SCF driver uses this device path. */
int hfg_one_electron_gpu(hfg_engine* engine, int natom, const int* Z, const double* xyz, double* S, double* T,
                         double* V);

/* SCFOptions (include/SCF.hpp:9-32) plus the engine's own knobs. */
typedef struct hfg_scf_options
{
    int max_iter;              /* MAX_ITER (30) */
    double energy_tol;         /* ENERGY_TOL (1e-6) */
    double density_tol;        /* DENSITY_TOL (1e-6), Frobenius norm of dD_tot */
    int use_diis;              /* DIIS (1) */
    int diis_size;             /* DIIS_SIZE (6) */
    double diis_tol;           /* DIIS_TOL (1e-6) */
    int unrestricted;          /* UNRESTRICTED (multiplicity != 1) */
    int guess_mix;             /* GUESS_MIX (0) */
    int damp;                  /* DAMP percentage (0) */
    int max_damp_iter;         /* MAX_DAMP_CYCLES (= max_iter) */
    double stop_damp_thresh;   /* STOP_DAMP_THRESH (0) */
    double level_shift;        /* LEVEL_SHIFT (0) */
    double lshift_gap_tol;     /* LSHIFT_GAP_TOL (infinity) */
    double max_lshift_iter;    /* MAX_LSHIFT_CYCLES (= max_iter) */
    double stop_lshift_thresh; /* STOP_LSHIFT_THRESH (0) */
    double schwartz_threshold; /* SCHWARTZ_THRESH (1e-10) */
    double density_threshold;  /* DENSITY_THRESH (1e-10) */
    int precision;             /* HFG_PRECISION_FP64 / HFG_PRECISION_MIXED */
    double fp32_cutoff;        /* FP32 cutoff of the mixed mode (2e-4) */
    int full_rebuild_every;    /* 0: incremental builds as the reference; k > 0: full build every k iterations */
    int verbose;               /* print the iteration table to stdout */
    int graph_iterations;      /* 1: every SCF iteration after the first replays CUDA graphs captured once: the Fock
                                  build, F update, DIIS on the device, X^T F X, the orbital update, energy and
                                  convergence measures, in segments around the eigensolver calls (cuSOLVER's syevd,
                                  which refuses capture, runs between them); one host read-back per iteration.
                                  Used when damping and level shifting are off and DIIS_SIZE <= 16; otherwise, or if
                                  a capture is refused, the same device iterations run eagerly. */
    int direct;                /* DIRECT (1).  0: the stored-integral SCF (SCF.cpp:233-521): integrals stored once by
                                  hfg_store_integrals, every Fock build F = h + J[D] - K[D] from them */
} hfg_scf_options;

typedef struct hfg_scf_result
{
    double e_electronic, e_nuclear, e_total;
    int iterations; /* SCF cycles run (the reference's final iteration index + 1) */
    int converged;
    double delta_e, delta_d, diis_error;
    double ms_total; /* wall time of the SCF (host clock), including the Fock builds */
    double ms_fock;  /* device time of the Fock builds */
    int fock_builds;
    double s_squared; /* <S^2> (UHF) */
    int graph_replays; /* iterations that ran as a replayed CUDA graph (graph_iterations) */
} hfg_scf_result;

/* The reference's defaults (SCF.hpp:9-32, Input.cpp:127-140) for a molecule of this multiplicity. */
void hfg_scf_default_options(hfg_scf_options* opt, int multiplicity);

/* SCF::SCF + SCF::run (src/SCF.cpp:13-135) for the single molecule of `engine`, whose nuclei are Z at xyz
 * (bohr, the basis centres' atoms) with total charge and multiplicity.  Density matrices of the last
 * iteration are written to D_alpha / D_beta (host, may be NULL). */
int hfg_scf_run(hfg_engine* engine, const hfg_scf_options* opt, int natom, const int* Z, const double* xyz,
                int charge, int multiplicity, hfg_scf_result* result, double* D_alpha, double* D_beta);

/* Core-Hamiltonian guess densities (src/SCF.cpp:165-231), host output. */
int hfg_core_guess(hfg_engine* engine, const hfg_scf_options* opt, int natom, const int* Z, const double* xyz,
                   int charge, int multiplicity, double* D_alpha, double* D_beta);

/* Analytic nuclear gradient (no reference counterpart: the reference has no gradients; checked against
 * central finite differences of its energy).  The backward half of the forward/backward pair whose
 * forward half is hfg_scf_run: with D_alpha == NULL the densities and energy-weighted density of the
 * last hfg_scf_run on this engine are used.  grad: natom x 3 (Eh/bohr).  Two-electron part on the GPU
 * (adjoint kernel, E/R tables recomputed), one-electron and overlap parts FP64 on the GPU, nuclear
 * repulsion on the host.  The engine must hold one molecule whose shell centres are the nuclei at xyz. */
typedef struct hfg_gradient_request
{
    int natom;
    const int* Z;
    const double* xyz;
    int unrestricted;
    const double* D_alpha; /* host, or NULL: use the last SCF's */
    const double* D_beta;  /* host (UHF; RHF: ignored, D_beta = D_alpha) */
    const double* W;       /* host: total energy-weighted density sum_s C_occ eps_occ C_occ^T */
    double schwartz_threshold;
    double density_threshold;
    int precision;      /* HFG_PRECISION_FP64, or HFG_PRECISION_MIXED: quartets whose bound Q_ab Q_cd max|D|
                           is below fp32_cutoff run in FP32 (FP64 accumulation), as in the Fock build */
    double fp32_cutoff;
} hfg_gradient_request;

int hfg_gradient(hfg_engine* engine, const hfg_gradient_request* req, double* grad, double* ms_two_electron);

/* One-electron and overlap parts of the gradient (sum D d(T+V)/dX - W dS/dX) on the GPU of `engine`, added
 * into grad (host, natom x 3); D is the total density, W the total energy-weighted density (host).
 * hfg_gradient uses this device path together with the nuclear-repulsion term. */
int hfg_gradient_one_electron_gpu(hfg_engine* engine, int natom, const int* Z, const double* xyz, const double* D,
                                  const double* W, double* grad);

/* One-electron, overlap (-W dS) and nuclear-repulsion parts of the gradient, added into grad (host CPU code,
 * FP64, OpenMP). */
int hfg_gradient_one_electron(const hfg_basis* basis, const int* shell_atom, int natom, const int* Z,
                              const double* xyz, const double* D, const double* W, double* grad);

/* Peak FMA throughput of this GPU measured by a register-only FMA loop (TFLOP/s, FP64 if fp64 != 0,
 * else FP32): the denominator of the ERI kernels' roofline. */
int hfg_measure_fma_peak(int device, int fp64, double* tflops);
/* FP64 tensor-core (DMMA m8n8k4) throughput of this GPU in TFLOP/s (no reference counterpart). */
int hfg_measure_dmma_peak(int device, double* tflops);

/* The device Boys function of the ERI kernels, F_0(T) .. F_m_max(T) for n values of T (host arrays; F is
 * n x (m_max + 1), row-major), evaluated on `device` by the same code the class kernels run (FP32 when
 * fp32 != 0): a known-answer check of Boys::calculateBoys (src/Boys.cpp:14-71).  m_max <= 9, T >= 0. */
int hfg_boys_eval(int device, int m_max, int fp32, long long n, const double* T, double* F);

/* Library version string. */
const char* hfg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HFGPU_H */
