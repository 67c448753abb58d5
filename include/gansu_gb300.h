/*
 * gansu_gb300.h - C ABI of the GB300-native Hartree-Fock hot path.
 *
 * Every entry point is plain C: host or device pointers, sizes, a CUDA stream
 * handle passed as void*, and an int status (HF_OK = 0).  No exception and no
 * C++ or torch type crosses this boundary.  Matrices are row-major N x N FP64
 * in device memory, symmetric, owned by the caller, exactly as the reference's
 * gansu::gpu free functions expect them (include/gpu_manager.hpp:34-109).
 *
 * The library is one shared object (libgansu_gb300.so) built for sm_103a.
 * There is no CPU fallback: on a machine without a usable GPU every compute
 * entry point returns HF_ERR_CUDA.
 */
#ifndef GANSU_GB300_H
#define GANSU_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
    HF_OK = 0,
    HF_ERR_INVALID_ARGUMENT = 1, /* bad size, null pointer, unsupported shell type */
    HF_ERR_CUDA = 2,             /* a CUDA runtime call failed (message: hf_last_error) */
    HF_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed */
    HF_ERR_NOT_CONVERGED = 4,    /* SCF hit maxiter */
    HF_ERR_SOLVER = 5,           /* cuSOLVER reported failure (info != 0) */
    HF_ERR_IO = 6,               /* basis / xyz file could not be read or parsed */
    HF_ERR_NOT_SPD = 7           /* metric not positive definite (RI) */
};

/* Last error message of the calling thread (never NULL). */
const char* hf_last_error(void);
/* Library version string. */
const char* hf_version(void);

/* ----------------------------------------------------------- input model */
/* Binary layout of gansu::PrimitiveShell (include/types.hpp:116-125). */
typedef struct {
    double exponent;
    double coefficient;
    double x, y, z;
    int shell_type;
    size_t basis_index;
    int atom_index;
} hf_primitive_shell;

/* Binary layout of gansu::Atom (include/types.hpp:131-135); coordinates in bohr. */
typedef struct {
    int atomic_number;
    double x, y, z;
} hf_atom;

typedef struct hf_molecule hf_molecule;

/* Replaces gansu::Molecular(xyz, gbs, charge, beta_to_alpha)
 * (include/molecular.hpp:56-109): parses the XYZ file (angstrom -> bohr,
 * src/parseXYZ.cpp:43-119) and the Gaussian basis file
 * (src/basis_set.cpp:32-124), expands primitive shells per atom and stably
 * sorts them by shell type (include/molecular.hpp:117-186). */
int hf_molecule_from_files(const char* xyz_path, const char* gbs_path, int charge, int beta_to_alpha,
                           hf_molecule** out);
/* Same from atoms already in bohr (the Molecular(atoms, gbs, ...) constructor). */
int hf_molecule_from_atoms(const hf_atom* atoms, int num_atoms, const char* gbs_path, int charge,
                           int beta_to_alpha, hf_molecule** out);
void hf_molecule_destroy(hf_molecule* mol);
/* Sizes: basis functions, primitive shells, atoms, electrons, alpha, beta. */
int hf_molecule_sizes(const hf_molecule* mol, int* num_basis, int* num_primitives, int* num_atoms,
                      int* num_electrons, int* num_alpha, int* num_beta);
/* Copies out the primitive shells (sorted by shell type), the CGTO
 * normalisation factors (num_basis doubles, reference convention including its
 * integer-division exponent for odd L) and the atoms. */
int hf_molecule_get(const hf_molecule* mol, hf_primitive_shell* prims, double* cgto_norm, hf_atom* atoms);

/* ---------------------------------------------------------------- engine */
/* An engine holds everything the Fock build needs on the device: contracted
 * shells rebuilt from the primitive list, shell pairs with their primitive
 * pair data and Schwarz bounds, the quartet work lists sorted by bound, the
 * Boys table and all SCF workspaces.  Creating it is the precomputation of the
 * reference's ERI plugin (ERI::precomputation, include/eri.hpp:36-63;
 * ERI_Direct::precomputation, src/eri.cu:323-347).  No allocation happens in
 * the per-iteration calls below. */
typedef struct hf_engine hf_engine;

/* Precision tier of the direct Fock build. */
enum {
    HF_PRECISION_FP64 = 0,  /* every surviving quartet in FP64 */
    HF_PRECISION_MIXED = 1  /* Q_ab*Q_cd*max|D| < mixed_threshold -> FP32 */
};

/* host arrays; prims must be sorted by shell type as hf_molecule_get returns them */
int hf_engine_create(const hf_primitive_shell* prims, int num_primitives, const double* cgto_norm, int num_basis,
                     const hf_atom* atoms, int num_atoms, double schwarz_threshold, hf_engine** out);
void hf_engine_destroy(hf_engine* eng);
/* Number of contracted shells and surviving contracted shell quartets. */
int hf_engine_stats(const hf_engine* eng, int* num_shells, long long* num_shell_pairs, long long* num_quartets);

/* Per quartet class (bra la,lb | ket lc,ld) counts accumulated by the direct
 * Fock builds since the last reset: primitive and contracted quartets evaluated
 * in each precision.  *num_classes receives the class count; arrays are filled
 * when max_classes >= *num_classes (class_l gets 4 ints per class).  No
 * reference counterpart: the flop model of the roofline uses these counts. */
int hf_engine_class_stats(hf_engine* eng, int max_classes, int* num_classes, int* class_l, long long* prim_fp64,
                          long long* prim_fp32, long long* contracted_fp64, long long* contracted_fp32);
int hf_engine_reset_stats(hf_engine* eng);
/* Bytes copied host -> device by hf_engine_create. */
int hf_engine_transfer_bytes(const hf_engine* eng, long long* h2d_bytes);
/* Number of CUDA kernels this library has launched in the process. */
long long hf_kernel_launch_count(void);
/* Diagnostic: sustained FMA throughput of the current GPU in TFLOP/s for
 * precision 0 (FP64) or 1 (FP32), the denominators of the integral-kernel
 * roofline. */
int hf_measure_fma_peak(int precision, double* tflops);

/* Replaces gansu::gpu::computeCoreHamiltonianMatrix (src/gpu_manager.cu:333-404):
 * S and H = T + V (point nuclei, charge = atomic number), device N x N. */
int hf_compute_core_hamiltonian(hf_engine* eng, double* d_overlap, double* d_core_hamiltonian, void* stream);

/* Replaces gansu::gpu::computeSchwarzUpperBounds (src/gpu_manager.cu:2154-2179):
 * primitive-pair bounds sqrt(max_comp (ab|ab)) as a dense host matrix
 * out[i*num_primitives + j] over the engine's primitive order. */
int hf_primitive_pair_bounds(hf_engine* eng, double* h_out);

/* Replaces gansu::gpu::computeERIMatrix (src/gpu_manager.cu:434-517): the full
 * N^4 tensor ((i*N+j)*N+k)*N+l in device memory, primitive-Schwarz screened.
 * For small molecules and parity tests only (N^4 doubles). */
int hf_compute_eri_matrix(hf_engine* eng, double* d_eri, void* stream);

/* Replaces gansu::gpu::computeFockMatrix_RHF (src/gpu_manager.cu:678-691):
 * F = H + sum_kl D_kl[(ij|kl) - 1/2 (ik|jl)] from a stored tensor. */
int hf_compute_fock_stored_rhf(const double* d_density, const double* d_core_hamiltonian, const double* d_eri,
                               double* d_fock, int num_basis, void* stream);

/* Replaces gansu::gpu::computeFockMatrix_Direct_RHF (src/gpu_manager.cu:2212-2227,
 * a stub that throws in the reference): Schwarz-screened McMurchie-Davidson
 * ERIs fused with the J/K contraction, no ERI tensor stored.
 * F = H + J - K/2. precision: HF_PRECISION_FP64 or HF_PRECISION_MIXED. */
int hf_compute_fock_direct_rhf(hf_engine* eng, const double* d_density, const double* d_core_hamiltonian,
                               double* d_fock, int precision, double mixed_threshold, void* stream);

/* Coulomb and exchange matrices J_ij = sum D_kl (ij|kl), K_ij = sum D_kl (ik|jl)
 * (the pieces of computeJMatrix/computeKMatrix, src/gpu_manager.cu:2327-2540). */
int hf_compute_jk_direct(hf_engine* eng, const double* d_density, double* d_J, double* d_K, int precision,
                         double mixed_threshold, void* stream);

/* Launch schedule of the direct Fock build (no
 * reference counterpart: the reference launches one kernel per class in turn,
 * src/gpu_manager.cu:2327-2540).  num_branches in 1..8: the quartet-class
 * launches run on that many streams forked from and joined back into the
 * caller's stream (1, the default: all on the caller's stream).  use_graph != 0:
 * each distinct build (same density and output pointers, precision and cuts) is
 * captured into a CUDA graph on its second call and replayed from then on (so is
 * the RHF loop's purification density, HF_EIGEN_PURIFICATION); the
 * graph reads the buffers at replay, so their contents may change between calls,
 * not their addresses.  On batch engines (hf_batch_rhf_scf) use_graph replays the
 * SCF iteration's purified density step and its Fock build instead. */
int hf_engine_set_fock_schedule(hf_engine* eng, int num_branches, int use_graph);

typedef struct {
    double build_ms_default;  /* one FP64 build under the default schedule */
    double build_ms_tuned;    /* the same build under the chosen schedule */
    int num_branches;         /* chosen branch count (1, 2, 4 or 8) */
    int num_class_pairs;      /* quartet class pairs with work */
    int num_caps_changed;     /* class-pair launches (FP64 and FP32 counted apart) whose grid cap differs from 16 blocks/SM */
} hf_autotune_report;

/* Autotuner of that schedule (no reference counterpart): on the caller's density
 * (device N x N; a batch engine's in its block layout), times every quartet class pair's FP64 and FP32 launch at grid
 * caps of 2..32 blocks per SM and keeps the fastest, then the branch count (1, 2,
 * 4 or 8, class pairs placed longest first on the least loaded branch) with the
 * fastest FP64 build.  The analytic gradient's class launches use the same
 * branches.  The choice stays with the engine; the class statistics
 * are reset.  Synchronises the stream.  report may be NULL. */
int hf_engine_autotune(hf_engine* eng, const double* d_density, hf_autotune_report* report, void* stream);

/* Applies a schedule chosen earlier (hf_engine_fock_schedule of a tuned engine
 * over the same molecule, e.g. kept in a file) without timing anything: per class
 * pair the grid caps (1..64 blocks per SM) of the FP64 and FP32 launches and the
 * branch (0..7, taken modulo the branch count); a NULL array restores that
 * default.  num_class_pairs must equal the engine's. */
int hf_engine_set_fock_grid_caps(hf_engine* eng, int num_class_pairs, const int* cap_fp64, const int* cap_fp32,
                                 const int* branch);

/* Graphs of the schedule (use_graph): Fock builds and RHF purifications captured
 * so far, and how many builds and purifications were replayed from them. */
int hf_engine_graph_stats(const hf_engine* eng, int* fock_graphs, int* purification_graphs, long long* replays);

/* The schedule in force: per class pair (engine order, *num_class_pairs of them,
 * arrays filled up to max_class_pairs, each may be NULL) the grid caps in blocks
 * per SM of its FP64 and FP32 launches and its branch. */
int hf_engine_fock_schedule(const hf_engine* eng, int max_class_pairs, int* num_class_pairs, int* cap_fp64,
                            int* cap_fp32, int* branch);

/* Replaces gansu::gpu::computeDIISErrorMatrix (src/gpu_manager.cu:1020-1067):
 * E = FDS - SDF, and X E X^T when include_transform != 0. */
int hf_compute_diis_error(hf_engine* eng, const double* d_overlap, const double* d_transform, const double* d_fock,
                          const double* d_density, double* d_error, int include_transform, void* stream);

/* Replaces gansu::gpu::computeFockMatrixDIIS (src/gpu_manager.cu:1078-1194):
 * B_ij = <e_i, e_j>, F = sum_i c_i F_i with the weights that minimise
 * |sum_i c_i e_i| subject to sum_i c_i = 1 (FP64, on the device).
 * num_prev in [2, 16]; d_errors/d_focks hold num_prev N x N matrices.
 * Where the reference's LU has no answer (an error vector that repeats
 * another, or a combination of others, to ~1e-7 relative: the bordered
 * matrix is singular), the repeated vector gets weight 0 and the minimiser
 * over the rest is used; an exactly zero error vector gets weight 1. */
int hf_compute_fock_diis(hf_engine* eng, const double* d_errors, const double* d_focks, double* d_new_fock,
                         int num_prev, void* stream);

/* Diagnostics of the last RHF purification (HF_EIGEN_PURIFICATION; no
 * reference counterpart): up to 16 words -- SP2 steps, tr(P) - nocc and
 * |tr(P) - |P|_F^2| after McWeeny, the SP2 stopping error, 1 if SP2 met its
 * stopping rule, McWeeny steps, a barrier-timeout flag, the grid barriers
 * passed, then (N <= 512, one launch) the microseconds from the launch's start
 * to the end of F' = X^T F X, P0, the SP2 steps, McWeeny, X P and D.  Zeros
 * before the first purification.  Synchronises. */
int hf_engine_purification_status(hf_engine* eng, double* h_out, int max_words);

/* The UHF Fock matrices of computeFockMatrix_UHF (src/gpu_manager.cu:707-731)
 * from separately built J and K of the two spin densities
 * (hf_compute_jk_direct): F_a = H + J_a + J_b - K_a, F_b = H + J_a + J_b - K_b. */
int hf_combine_uhf_fock(const double* d_core_hamiltonian, const double* d_j_a, const double* d_j_b,
                        const double* d_k_a, const double* d_k_b, double* d_fock_a, double* d_fock_b, int num_basis,
                        void* stream);

/* DIIS extrapolation that allocates nothing (no reference counterpart: the
 * reference's computeFockMatrixDIIS allocates on every call).  For callers
 * that cannot allocate device memory while an SCF step runs -- a CUDA graph
 * being recorded, an application whose device memory belongs to its own pool,
 * a thread that must not synchronise the device.  Same result as
 * hf_compute_fock_diis without an engine: F = sum_i c_i F_i from num_prev
 * (2..16) stored error/Fock pairs, N = num_basis.  Its scratch is a static
 * device array of 280 doubles held by every GPU that loads the library; the
 * first call on a device looks its address up (make that call before any
 * stream capture; after cudaDeviceReset the next call looks it up again).
 * Dependent error vectors are handled as in hf_compute_fock_diis.  Calls that
 * overlap on the GPU share the scratch and race: serialise them. */
int hf_compute_fock_diis_noalloc(const double* d_errors, const double* d_focks, double* d_new_fock, int num_prev,
                                 int num_basis, void* stream);

/* -------------------------------------------------------------------- RI */
/* Attaches the auxiliary basis of eri_method = ri: the primitives of
 * Molecular(atoms, auxiliary_gbsfilename) (src/rhf.cu:76-79; the ERI_RI
 * constructor, src/eri.cu:119-132), same layout and normalisation as the AO
 * primitives, auxiliary shells up to f.  Replaces any earlier auxiliary basis
 * and drops a B tensor built from it. */
int hf_engine_set_auxiliary_basis(hf_engine* eng, const hf_primitive_shell* aux_prims, int num_aux_primitives,
                                  const double* aux_cgto_norm, int num_aux_basis);

/* Replaces gpu::computeTwoCenterERIs (src/gpu_manager.cu:1963-2041): the RI
 * metric (P|Q), row-major naux x naux, screened by Q_P * Q_Q < thr. */
int hf_compute_two_center_eris(hf_engine* eng, double* d_metric, void* stream);

/* Replaces gpu::computeThreeCenterERIs (src/gpu_manager.cu:2048-2141):
 * (mu nu|P) at d_three_center[(P * N + mu) * N + nu] (both triangles),
 * screened by Q_mu_nu * Q_P < thr.  Allocates a packed temporary. */
int hf_compute_three_center_eris(hf_engine* eng, double* d_three_center, void* stream);

/* Replaces gpu::compute_RI_IntermediateMatrixB (src/gpu_manager.cu:1448-1526):
 * metric, Cholesky V = L L^T (HF_ERR_NOT_SPD if it fails), three-centre
 * integrals, B = L^-1 (mu nu|P).  B stays on the engine for the RI Fock
 * builds; when d_b_out is non-NULL it also receives B in the reference layout
 * [P][mu][nu] (naux * N * N doubles). */
int hf_compute_ri_intermediate_b(hf_engine* eng, double* d_b_out, void* stream);

/* Replaces gpu::computeFockMatrix_RI_RHF (src/gpu_manager.cu:1543-1632):
 * F = H + J - K/2 with J = sum_P B_P (B_P . D) and K = sum_P B_P D B_P^T for a
 * symmetric D (K from an eigen-factorisation of D).  Builds B on first use. */
int hf_compute_fock_ri_rhf(hf_engine* eng, const double* d_density, const double* d_core_hamiltonian,
                           double* d_fock, void* stream);

/* The J and K of hf_compute_fock_ri_rhf separately (N x N each). */
int hf_compute_jk_ri(hf_engine* eng, const double* d_density, double* d_J, double* d_K, void* stream);

/* Split-BF16 tensor-core GEMM (no reference counterpart: the tcgen05 building
 * block of the RI mixed tier, exposed for testing).  A is m x k, B is n x k,
 * row-major FP64; both are split into BF16 hi/lo planes and
 * A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T accumulates in FP32 in TMEM.
 * mode 0: C (m x n) = A B^T, stored through the BF16 hi/lo output planes;
 * mode 1: C (m x m) = A A^T (B unused; upper tiles, mirrored);
 * mode 2: C (m x m) = A B^T + B A^T.  Allocates temporaries; synchronises. */
int hf_split_bf16_matmul(const double* d_a, const double* d_b, double* d_c, int m, int n, int k, int mode,
                         void* stream);

/* ------------------------------------------------------------------- SCF */
typedef struct {
    int max_iter;                   /* reference default 100 */
    double convergence_threshold;   /* |dE| threshold, reference default 1e-6 */
    int diis_size;                  /* reference default 8 */
    int diis_include_transform;     /* reference default 0 */
    int precision;                  /* HF_PRECISION_FP64 / HF_PRECISION_MIXED */
    double mixed_threshold;         /* FP32 cut for Q_ab*Q_cd*max|dD| */
    int incremental;                /* 1: build G(dD) and accumulate (mixed tier) */
    int rebuild_every;              /* full rebuild period for the incremental build, 0 = never */
    int full_build_precision;       /* precision of full (non-incremental) builds under the mixed tier */
    int eigensolver;                /* HF_EIGEN_SYEVD, HF_EIGEN_SYEVJ or HF_EIGEN_PURIFICATION */
    int verbose;                    /* print per-iteration lines like the reference */
    int eri_method;                 /* HF_ERI_DIRECT, HF_ERI_RI or HF_ERI_STORED (eri_method = direct / ri / stored,
                                       src/rhf.cu:72-88) */
    double anchor_threshold;        /* mixed tier: low-precision full builds (direct: all quartets FP32; RI:
                                       split-BF16 K) while max|dD| >= this, then one FP64 build, then
                                       incremental builds; 0 = the first build is the FP64 one */
    int initial_guess;              /* HF_GUESS_CORE / _GWH / _DENSITY / _SAD (initial_guess = core / gwh /
                                       density / sad) */
    const double* guess_density_a;  /* HF_GUESS_DENSITY / HF_GUESS_SAD: device alpha-spin density (N x N;
                                       a batch engine: the block layout); RHF takes D_a + D_b */
    const double* guess_density_b;  /* beta-spin density, same layout; NULL for RHF means D_a is the total */
    const double* orthogonalizer;   /* NULL: X = U s^{-1/2} of S (src/hf.cu:171-243).  Otherwise a device N x N
                                       row-major X whose nonzero columns span the orbital space, e.g. the
                                       spherical-harmonic subspace of the Cartesian basis (no reference
                                       counterpart); the DIIS error is then X^T (FDS - SDF) X.
                                       Single-molecule SCFs only. */
    int convergence_method;         /* HF_CONV_DIIS, HF_CONV_DAMPING or HF_CONV_OPTIMAL_DAMPING
                                       (convergence_method = diis / damping / optimaldamping) */
    double damping_factor;          /* HF_CONV_DAMPING: F <- (1 - a) F_prev + a F (reference default 0.9) */
    int purification_max_steps;     /* HF_EIGEN_PURIFICATION: SP2 steps at most (0: 100 when N <= 512, else a
                                       fixed 50); a projector that has not converged within them fails the
                                       trace/idempotency check and the SCF reruns with syevd */
    double anchor_mixed_threshold;  /* mixed tier, direct builds: 0 = the anchor build is all FP64; > 0 = the
                                       anchor takes quartets with Q_ab*Q_cd*max|D| below this in FP32 */
    double incremental_drop;        /* incremental dD builds (direct): quartets whose Qs_ab*Qs_cd times the
                                       largest |dD| of the shell blocks they read is below this are left out
                                       (0: the Schwarz threshold); capped at 0.03 * convergence_threshold */
    double pre_anchor_drop;         /* mixed tier, direct builds before the anchor: quartets whose
                                       Qs_ab*Qs_cd*max|D| is below this are left out of those builds
                                       (0: 1e-6); the anchor and later builds are not affected */
} hf_scf_options;

/* Fock-matrix update between iterations (Convergence_RHF_DIIS / _Damping,
 * include/rhf.hpp:182-353; UHF and ROHF alike).  Optimal damping
 * (computeOptimalDampingFactor_RHF, src/gpu_manager.cu:898-963): with
 * s = Tr[F_old (D - D_old)], c = Tr[(F - F_old)(D - D_old)], a = 1 if
 * c <= -s/2, else -s/(2c); F and D are both damped.  Damping is RHF, UHF
 * (constant factor, as the reference) and ROHF; the batch SCF is DIIS only. */
enum {
    HF_CONV_DIIS = 0,
    HF_CONV_DAMPING = 1,
    HF_CONV_OPTIMAL_DAMPING = 2
};

/* Density from the Fock matrix inside the SCF loop.  The reference diagonalises
 * (computeCoefficientMatrix, src/gpu_manager.cu:529-599); purification gives the
 * same aufbau density when the HOMO-LUMO gap is open, without eigenvectors:
 * FP32 SP2 steps until their idempotency error stops shrinking, then FP64
 * McWeeny steps (N <= 512: the whole step is one launch); orbitals and orbital
 * energies come from one diagonalisation of the final Fock matrix.  Every
 * purified projector is checked (trace = number of occupied orbitals to 1e-6,
 * idempotency to 1e-8); if one fails (small or closed gap) the RHF SCF is
 * rerun with HF_EIGEN_SYEVD and hf_scf_result.eigensolver_used says so. */
enum {
    HF_EIGEN_SYEVD = 0,
    HF_EIGEN_SYEVJ = 1,
    HF_EIGEN_PURIFICATION = 2
};

/* Initial guess (InitialGuess_RHF_Core / _GWH / _Density / _SAD, include/rhf.hpp:378-588;
 * the UHF and ROHF classes of include/uhf.hpp and include/rohf.hpp).  DENSITY and SAD
 * start from the caller's densities (options.guess_density_a/_b); the SAD density is
 * the block-diagonal superposition of atomic densities that the host assembles
 * (read_density_from_sad, src/utils.cpp:21-56, or atomic RHF/ROHF solves).
 *   RHF   DENSITY: F = F(D_a + D_b);  SAD: F(D), C, D, F
 *   UHF   DENSITY = SAD: F(D_a, D_b), C, beta symmetry break, D, F
 *   ROHF  DENSITY = SAD: D_closed = 2 D_b, D_open = D_a - D_b, F, C, D, F */
enum {
    HF_GUESS_CORE = 0,     /* diagonalise H */
    HF_GUESS_GWH = 1,      /* diagonalise 1.75 S_pq (H_pp + H_qq) / 2 (src/gpu_kernels.cu:535-545) */
    HF_GUESS_DENSITY = 2,  /* the given density (initial_guess = density) */
    HF_GUESS_SAD = 3       /* the given superposition of atomic densities (initial_guess = sad) */
};

/* Two-electron backend of the SCF. */
enum {
    HF_ERI_DIRECT = 0,  /* fused direct J/K build every iteration */
    HF_ERI_RI = 1,      /* density fitting; needs hf_engine_set_auxiliary_basis */
    HF_ERI_STORED = 2   /* RHF only: the N^4 tensor computed once and kept with the engine, F from it
                           every iteration (ERI_Stored_RHF, the reference's default eri_method); FP64 */
};

typedef struct {
    double electronic_energy;       /* 1/2 sum D (H + F) */
    double nuclear_repulsion;
    double total_energy;
    int iterations;                 /* reference convention: iter_ at exit (src/hf.cu:297-300) */
    int converged;
    double fock_ms_total;           /* summed device time of the Fock builds */
    double scf_ms_total;            /* SCF loop (iterations only), CUDA events on the stream */
    double setup_ms;                /* core Hamiltonian + X + guess */
    double diag_ms_total;           /* F' = X^T F X, eigensolver, C = X C', density (loop) */
    double diis_ms_total;           /* DIIS error, B matrix, solve and extrapolation (loop) */
    long long fp64_quartets;        /* summed over all Fock builds */
    long long fp32_quartets;
    int eigensolver_used;           /* RHF: the eigensolver the SCF finished with (a purified density that
                                       fails its trace/idempotency checks reruns the SCF with HF_EIGEN_SYEVD) */
} hf_scf_result;

void hf_scf_options_default(hf_scf_options* opt);

/* Restricted HF SCF on the device (RHF::solve -> HF::single_point_energy,
 * src/hf.cu:245-314): X = U s^{-1/2} (s < 1e-6 -> 0), core-Hamiltonian guess,
 * DIIS as Convergence_RHF_DIIS (include/rhf.hpp:298-327), convergence on |dE|.
 * Optional outputs (device, may be NULL): final density, Fock, orbital energies,
 * coefficients. */
int hf_rhf_scf(hf_engine* eng, int num_electrons, const hf_scf_options* opt, hf_scf_result* result,
               double* d_density_out, double* d_fock_out, double* d_orbital_energies_out,
               double* d_coefficients_out);

/* Unrestricted HF on the device (UHF::solve, src/uhf.cu; Convergence_UHF_DIIS,
 * include/uhf.hpp:291-380): spin densities D_s = C_s,occ C_s,occ^T, Fock
 * F_a = H + J(D_a + D_b) - K(D_a) (and b), energy 1/2 sum[(D_a + D_b) H + D_a F_a
 * + D_b F_b], guess orbitals for both spins with the beta symmetry break of
 * InitialGuess_UHF::break_symmetry (include/uhf.hpp:429-436: the last basis
 * function's row and the last orbital's column of C_b zeroed), one DIIS ring per
 * spin on the same cyclic index, |dE| convergence.  Two direct J/K builds per
 * iteration.
 * Outputs (device, may be NULL): spin densities, and the orbital energies and
 * coefficients (row-major, orbitals as columns) of the diagonalisations that
 * produced them. */
int hf_uhf_scf(hf_engine* eng, int num_alpha, int num_beta, const hf_scf_options* opt, hf_scf_result* result,
               double* d_density_a_out, double* d_density_b_out, double* d_orbital_energies_a_out,
               double* d_orbital_energies_b_out, double* d_coefficients_a_out, double* d_coefficients_b_out);

/* Restricted open-shell HF on the device (ROHF::solve, src/rohf.cu; Fock build
 * computeFockMatrix_ROHF, src/gpu_manager.cu:733-817).  num_beta closed and
 * num_alpha - num_beta open orbitals; D_closed = 2 C_c C_c^T, D_open = C_o C_o^T;
 * F_c = H + J(D) - K(D_c)/2 - K(D_o)/2, F_o = (H + J(D) - K(D_c)/2 - K(D_o))/2
 * (D = D_c + D_o); the unified Fock matrix R in the MO basis from C^T F_c C and
 * C^T F_o C with the coupling constants coupling[6] = {A_cc, B_cc, A_oo, B_oo,
 * A_vv, B_vv} (NULL: Roothaan, src/rohf.cu:30-39), back to the AO basis as
 * S C R C^T S; energy 1/2 [<D_c, H + F_c> + <D_o, H> + 2 <D_o, F_o>]; DIIS on the
 * unified F with D.  Two direct J/K builds per iteration.  Outputs (device, may
 * be NULL): alpha = D_c/2 + D_o and beta = D_c/2 densities (export_density_matrix,
 * src/rohf.cu:288-315), orbital energies and coefficients of the last
 * diagonalised unified Fock matrix. */
int hf_rohf_scf(hf_engine* eng, int num_alpha, int num_beta, const double* coupling, const hf_scf_options* opt,
                hf_scf_result* result, double* d_density_a_out, double* d_density_b_out,
                double* d_orbital_energies_out, double* d_coefficients_out);

/* ---------------------------------------------------------------- batch */
/* One engine over many independent molecules (no reference counterpart: the
 * reference solves one molecule per HF object).  Molecule m is given as the
 * arrays hf_engine_create takes.  Shell pairs and quartets never mix
 * molecules; one launch per quartet class serves the whole batch.  Give
 * molecules of equal size (and electron count) next to each other: each run
 * of them is one group of batched linear algebra.  RI, the gradient and
 * hf_rhf_scf are single-molecule; a batch engine's J/K/F outputs use the
 * block layout (molecule m's N_m x N_m matrix after those of molecules < m). */
int hf_engine_create_batch(int num_molecules, const hf_primitive_shell* const* prims, const int* num_primitives,
                           const double* const* cgto_norm, const int* num_basis, const hf_atom* const* atoms,
                           const int* num_atoms, double schwarz_threshold, hf_engine** out);

/* RHF for every molecule of a batch engine, in lockstep iterations (replaces a
 * loop of RHF::solve, src/hf.cu:245-314; FP64).  results[m] holds molecule m's
 * energies and iteration count at its own convergence; batch_scf_ms (may be
 * NULL) the device time of the batch loop and batch_iterations (may be NULL)
 * its iteration count.  HF_ERR_NOT_CONVERGED if any molecule did not converge. */
int hf_batch_rhf_scf(hf_engine* eng, const int* num_electrons, const hf_scf_options* opt, hf_scf_result* results,
                     double* batch_scf_ms, int* batch_iterations);

/* ------------------------------------------------------------- gradient */
/* Energy-weighted density W = 2 sum_{i < num_occupied} eps_i C_i C_i^T from the
 * SCF's coefficients (row-major, orbitals as columns) and orbital energies.
 * No reference counterpart (the reference has no analytic gradient). */
int hf_energy_weighted_density(hf_engine* eng, const double* d_coefficients, const double* d_orbital_energies,
                               int num_occupied, double* d_out, void* stream);

/* Analytic RHF nuclear gradient dE/dR (3 * num_atoms doubles, host, bohr,
 * Eh/bohr) from the converged density D and energy-weighted density W:
 * sum D dH - sum W dS + derivative ERIs contracted with the two-particle
 * density (Hermite intermediates recomputed, FP64) + nuclear repulsion.
 * The backward half of the energy/gradient pair that feeds a geometry
 * optimiser (the reference only has an energy-only coordinate search,
 * include/builder.hpp:108-275).  gradient_ms (may be NULL) receives the
 * device time. */
int hf_rhf_gradient(hf_engine* eng, const double* d_density, const double* d_energy_weighted_density,
                    double* h_gradient, double* gradient_ms, void* stream);

/* Analytic RHF gradient of the RI (density-fitted) energy of eri_method = ri
 * (the energy of the reference's RI Fock build, src/gpu_manager.cu:1448-1632):
 * the one-electron and nuclear terms of hf_rhf_gradient plus derivative
 * three-centre integrals contracted with Gamma_P = c_P D - 1/2 D C_P D and
 * derivative metric integrals with gamma_PQ = c_P c_Q - 1/2 tr(C_P D C_Q D)
 * (c = V^-1 (T . D), C_P = sum_Q (V^-1)_PQ T_Q), formed from the occupied
 * orbitals d_coefficients[:, :num_occupied] (row-major N x N, the SCF's
 * coefficient output).  Needs hf_engine_set_auxiliary_basis.  FP64.  No
 * reference counterpart. */
int hf_rhf_gradient_ri(hf_engine* eng, const double* d_density, const double* d_energy_weighted_density,
                       const double* d_coefficients, int num_occupied, double* h_gradient, double* gradient_ms,
                       void* stream);

/* hf_rhf_gradient with the two-electron part split by bound: derivative
 * integrals of quartets with Qs_ab Qs_cd c_max^4 max|D|^2 >= mixed_threshold in
 * FP64, the rest in FP32 (FP32 Hermite tables and contraction, FP64 atomic
 * accumulation into the gradient).  No reference counterpart. */
int hf_rhf_gradient_mixed(hf_engine* eng, const double* d_density, const double* d_energy_weighted_density,
                          double mixed_threshold, double* h_gradient, double* gradient_ms, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GANSU_GB300_H */
