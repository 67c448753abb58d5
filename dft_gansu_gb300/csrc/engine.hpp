// Engine: everything the hot path needs, resident on the device.
#pragma once
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <array>
#include <utility>
#include <vector>

#include "engine_types.hpp"
#include "internal.hpp"
#include "md_math.cuh"

namespace gb {

constexpr int kNumPairClasses = (kMaxL + 1) * (kMaxL + 2) / 2;
constexpr int kNumClassPairs = kNumPairClasses * (kNumPairClasses + 1) / 2;
// per class pair and precision: {primitive quartets, contracted quartets}
constexpr int kCounterSlots = kNumClassPairs * 2 * 2;

struct Shell {
    int l, nprim, prim_off, bf, atom;  // bf: global first function (sum of the earlier molecules' N + local)
    int mol;                           // molecule of the shell (0 for a single-molecule engine)
    double x, y, z;
};

// Block layout of N x N matrices for one or several molecules: molecule m's
// matrix occupies [base[m], base[m] + n[m]^2) row-major; a single molecule is
// the plain N x N matrix.
struct BlockMap {
    const long long* base;  // nmol + 1 offsets
    const int* n;
    const int* bf0;         // first global function of each molecule
    int nmol;
    long long nelem;        // base[nmol]
};

#ifdef __CUDACC__
__device__ __forceinline__ int block_of(const BlockMap& M, long long k)
{
    int lo = 0, hi = M.nmol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (M.base[mid] <= k) lo = mid; else hi = mid - 1;
    }
    return lo;
}
#endif

// (la, lb) pair classes with la >= lb, ordered (0,0),(1,0),(1,1),(2,0),(2,1),(2,2)
struct PairClass {
    int la, lb;
    int begin, count;  // global pair index range
    std::vector<std::pair<int, int>> groups;  // (class-relative start, size) of equal primitive-pair count
    std::vector<int> group_mol;               // molecule of each group (groups never span molecules)
};

// One molecule of an engine's input (reference layouts: gansu::PrimitiveShell, gansu::Atom).
struct MolInput {
    const hf_primitive_shell* prims;
    int nprim;
    const double* cgto;
    int nbasis;
    const hf_atom* atoms;
    int natom;
};
int build_engine(const MolInput* mols, int nmol, double schwarz_threshold, hf_engine** out);

// bra class X >= ket class Y
struct ClassPair {
    int X, Y;
    int entry_begin, nentry;  // bra entries (global entry index range)
    long long n_survivors;    // contracted quartets passing the contracted bound test
};

// Device buffers of one mixed-precision plan (per Fock build).
struct MixedPlan {
    long long* off64 = nullptr;  // per class pair: nentry+1 (packed by entry_begin + class pair index)
    long long* off32 = nullptr;
    int* lo32 = nullptr;
};

struct RiState;  // ri.hpp

// Launch schedule of the direct Fock build (fock.cu).  The class-pair launches
// run on nbranch streams forked from and joined back to the caller's stream
// (1: all on the caller's stream); with use_graph every distinct build (same
// density and output pointers, precision and cuts) is captured into a CUDA
// graph on its second occurrence and replayed from then on.  cap64/cap32 are
// the grid caps (blocks per SM) of each class pair's FP64 and FP32 launches,
// chosen by hf_engine_autotune (0: kFockBlocksPerSm).
constexpr int kMaxBranches = 8;
constexpr int kFockBlocksPerSm = 16;
// upper bound on the primitive quartets of one work item (bra primitive range x ket
// primitive pairs) above which a bra's entry is split by primitive range
constexpr int kPrimPerItem = 64;
constexpr int kMaxFockGraphs = 16;
struct FockSchedule {
    int nbranch = 1;
    bool use_graph = false;
    std::vector<int> branch_of;     // per class pair (empty: round robin)
    std::vector<int> cap64, cap32;  // per class pair (empty: default)
    cudaStream_t branch[kMaxBranches] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kMaxBranches] = {};
    cudaStream_t capture = nullptr;  // graphs are captured on this stream (the caller's may be the legacy stream)
    struct Graph {
        const double* D;
        double *J, *K;
        int precision;
        double mixed_thr, drop;
        int uses;
        cudaGraphExec_t exec;  // null until the second use
        bool mixed;            // Engine::last_mixed after this build
        long long launches;    // kernels in the graph
    };
    std::vector<Graph> graphs;
    // the RHF loop's purification (scf.cu), captured and replayed the same way
    struct PurifyGraph {
        const double* F;
        double* D;
        int nocc;
        int max_steps;         // SP2 step limit of the options (part of the key)
        int uses;
        bool failed;           // the capture failed: this purification runs as ordinary launches
        cudaGraphExec_t exec;
        long long launches;
    };
    std::vector<PurifyGraph> purify;
    void* cublas_ws = nullptr;     // cuBLAS workspace while capturing (cuBLAS's own pool may allocate)
    long long graph_replays = 0;   // builds and purifications replayed from graphs
};
constexpr size_t kCublasCaptureWorkspace = size_t(16) << 20;

struct Engine {
    int num_basis = 0, num_shells = 0, num_atoms = 0, num_prims = 0;
    // molecules (a batch engine holds several; a plain engine one)
    int nmol = 1;
    std::vector<int> mol_bf0, mol_n, mol_atom0, mol_natom;
    std::vector<long long> mol_base;  // nmol + 1 block offsets of the block layout
    long long nelem = 0;              // elements of one block-layout matrix (N^2 for one molecule)
    long long* d_mol_base = nullptr;
    int* d_mol_n = nullptr;
    int* d_mol_bf0 = nullptr;
    int2* d_mol_atoms = nullptr;      // first atom, number of atoms
    int* d_shell_mol = nullptr;
    unsigned char* d_mol_active = nullptr;  // batches: set while a batch SCF runs (null otherwise)
    BlockMap block_map() const { return BlockMap{d_mol_base, d_mol_n, d_mol_bf0, nmol, nelem}; }
    double schwarz_threshold = 1e-12;
    double cgto_max = 1.0;

    std::vector<hf_primitive_shell> prims;  // as given (sorted by type)
    std::vector<double> cgto;
    std::vector<hf_atom> atoms;
    std::vector<Shell> shells;
    std::vector<double> scale;              // s_i = cgto_i * component factor
    std::vector<ShellPairDev> pairs;        // host copy
    std::vector<PrimPair64> pp64;
    std::vector<PairClass> pair_classes;
    std::vector<ClassPair> class_pairs;
    std::vector<int> entry_bra, entry_cnt;  // per (bra, ket group) entry
    std::vector<int> entry_lo0;              // class-relative first ket of the entry's group
    std::vector<int> entry_prim;             // bra primitive-pair range of the entry: first | (end << 16)
    std::vector<long long> off_static;      // per class pair, nentry+1 (packed: entry_begin + cp)
    long long total_survivors = 0;          // work items (a split bra counts once per entry)
    long long unique_quartets = 0;          // contracted quartets of the lists
    std::vector<double> prim_bound;         // per primitive of the input list pair (dense), filled lazily

    // device
    ShellPairDev* d_pairs = nullptr;
    PrimPair64* d_pp64 = nullptr;
    PrimPair32* d_pp32 = nullptr;
    double* d_boys64 = nullptr;
    float* d_boys32 = nullptr;
    double* d_scale = nullptr;
    double* d_atoms = nullptr;  // natom x 4: x, y, z, Z
    int* d_entry_bra = nullptr;
    int* d_entry_cnt = nullptr;
    int* d_entry_lo0 = nullptr;
    int* d_entry_prim = nullptr;
    double* d_pair_qs = nullptr;  // Qs per global pair (for the mixed plan)
    long long* d_off_static = nullptr;
    int* d_cp_meta = nullptr;     // per class pair: entry_begin | nentry | ket_base | off_base
    MixedPlan plan;
    double* d_Dp64 = nullptr;
    float* d_Dp32 = nullptr;
    double* d_Jp = nullptr;
    double* d_Kp = nullptr;
    float* d_Jp32 = nullptr;   // FP32-tier accumulators (FP32 accumulation)
    float* d_Kp32 = nullptr;
    bool last_mixed = false;   // whether the last build used the FP32 accumulators
    double* d_grad = nullptr;     // 3 * natom gradient accumulators (allocated on first use)
    int* d_shell_atom = nullptr;  // contracted shell -> atom
    long long* d_goff64 = nullptr;  // gradient work-item offsets (FP64 / FP32 lists)
    long long* d_goff32 = nullptr;
    int2* d_shell_info = nullptr;   // per shell: first basis function, number of components
    float* d_block_dmax = nullptr;  // per shell block max |D| of the density being built (mixed plan)
    double* d_eri = nullptr;     // stored N^4 ERI tensor of eri_method = stored (allocated on first use)
    double* d_scalar = nullptr;  // small scratch scalars (8 doubles)
    unsigned long long* d_counters = nullptr;  // [class pair][precision][prim, contracted]
    long long bytes_h2d = 0;                   // bytes uploaded by engine creation

    RiState* ri = nullptr;  // auxiliary basis and B tensor (RI), attached on request
    FockSchedule sched;     // launch schedule of the direct Fock build (fock.cu)

    cublasHandle_t cublas = nullptr;
    cusolverDnHandle_t cusolver = nullptr;
    int num_sms = 152;

    // SCF workspaces (allocated on first SCF call, reused)
    struct Scf {
        int n = 0, m = 0;
        double *S = nullptr, *H = nullptr, *X = nullptr, *F = nullptr, *D = nullptr, *Dprev = nullptr,
               *G = nullptr, *dD = nullptr, *C = nullptr, *W = nullptr, *eps = nullptr, *T1 = nullptr,
               *T2 = nullptr, *E = nullptr, *Es = nullptr, *Fs = nullptr, *work = nullptr, *diis = nullptr,
               *J = nullptr, *K = nullptr;
        int* info = nullptr;
        int lwork = 0, lwork_j = 0;
        double* work_j = nullptr;
        syevjInfo_t syevj_params = nullptr;
        float *P32a = nullptr, *P32b = nullptr, *P32c = nullptr;  // purification (FP32 SP2) buffers
        double *Qocc = nullptr, *Mocc = nullptr, *qwork = nullptr;  // occupied basis from the projector
        int* qinfo = nullptr;
        int qlwork = 0;
        double* pur = nullptr;  // purification status words, grid barrier and partial sums (purify.cu)
        size_t pur_doubles = 0;
    } scf;

    ~Engine();
};

// entry point tables implemented by the per-class objects
using FockLauncher = void (*)(bool fp32, const FockClassLaunch&, int grid, cudaStream_t);
using EriLauncher = void (*)(const FockClassLaunch&, const double* scale, double* eri, int grid, cudaStream_t);
FockLauncher fock_launcher(int la, int lb, int lc, int ld);
EriLauncher eri_launcher(int la, int lb, int lc, int ld);

// fock.cu
// mixed tier: drop threshold of the all-FP32 builds before the FP64 anchor (those
// builds only steer the density towards the anchor, which keeps the Schwarz set;
// on n-decane 6-31G* 1e-6 leaves out 10-30% of their quartets and changes neither
// the iteration count nor the converged energy beyond the convergence threshold)
constexpr double kPreAnchorDrop = 1e-6;

// drop > 0: under the mixed tier, quartets whose bound Qs_ab Qs_cd c_max^4 max|D| is
// below drop are skipped (default: the Schwarz threshold, or the FP32 cut if lower)
int build_jk(Engine& e, const double* d_D, double* d_J, double* d_K, int precision, double mixed_thr,
             cudaStream_t s, double drop = -1.0);
int finish_fock(Engine& e, const double* d_H, const double* d_J, const double* d_K, double* d_F, cudaStream_t s);
int scale_density(Engine& e, const double* d_D, bool want_fp32, cudaStream_t s);
// device split of the static quartet lists into FP64 prefix / FP32 rest (e.plan)
int mixed_plan(Engine& e, const double* d_D, double factor, bool square, double tau, double skip, cudaStream_t s);
// max |A| of every molecule's block (fock.cu)
int mol_absmax(Engine& e, const double* d_A, double* d_out, cudaStream_t s);
// batch build with per-molecule FP32 cuts and drop thresholds (fock.cu)
int build_jk_batch(Engine& e, const double* d_D, const double* d_mol_tau, const double* d_mol_skip,
                   double* d_mol_dmax, cudaStream_t s);
// the full ERI tensor ((i*N+j)*N+k)*N+l of a single-molecule engine (fock.cu)
int compute_eri_tensor(Engine& e, double* d_eri, cudaStream_t s);
// F = H + sum_kl D_kl [(ij|kl) - 1/2 (ik|jl)] from a stored tensor (fock.cu)
int stored_fock(const double* d_D, const double* d_H, const double* d_eri, double* d_F, int n, cudaStream_t s);
// releases the schedule's streams, events and graphs (fock.cu)
void schedule_release(FockSchedule& S);
// creates the schedule's branch streams and events on first use (fock.cu)
int schedule_streams(Engine& e);

#ifdef __CUDACC__
// Issues launch(c, stream) for every class pair with work: on s itself when the
// schedule has one branch, else on the branch streams, forked from s (an event
// recorded on s) and joined back into s, so s sees one ordered build either way.
template <class Launch>
int launch_class_pairs(Engine& e, cudaStream_t s, Launch&& launch)
{
    FockSchedule& S = e.sched;
    const int ncp = static_cast<int>(e.class_pairs.size());
    const int nb = std::max(1, std::min(S.nbranch, kMaxBranches));
    int st;
    if (nb == 1) {
        for (int c = 0; c < ncp; ++c)
            if (e.class_pairs[c].n_survivors > 0 && (st = launch(c, s))) return st;
        return HF_OK;
    }
    if ((st = schedule_streams(e))) return st;
    GB_CUDA_TRY(cudaEventRecord(S.fork, s));
    for (int b = 0; b < nb; ++b) GB_CUDA_TRY(cudaStreamWaitEvent(S.branch[b], S.fork, 0));
    for (int c = 0; c < ncp; ++c) {
        if (e.class_pairs[c].n_survivors == 0) continue;
        const int b = (c < static_cast<int>(S.branch_of.size()) ? S.branch_of[c] : c) % nb;
        if ((st = launch(c, S.branch[b]))) return st;
    }
    for (int b = 0; b < nb; ++b) {
        GB_CUDA_TRY(cudaEventRecord(S.join[b], S.branch[b]));
        GB_CUDA_TRY(cudaStreamWaitEvent(s, S.join[b], 0));
    }
    return HF_OK;
}
#endif

// one_electron.cu
int core_hamiltonian(Engine& e, double* d_S, double* d_H, cudaStream_t s);

// grad.cu
int energy_weighted_density(Engine& e, const double* d_C, const double* d_eps, int nocc, double* d_W, cudaStream_t s);
// d_C != nullptr: the two-electron part is the RI one (ri_grad.cu) from the occupied
// orbitals C[:, :nocc] (row-major, row stride ldc) instead of the four-centre one
int rhf_gradient(Engine& e, const double* d_D, const double* d_W, double* h_grad, cudaStream_t s, float* ms_out,
                 int precision = 0, double mixed_threshold = 0.0, const double* d_C = nullptr, int ldc = 0,
                 int nocc = 0);

// host MD helpers (engine.cu)
void host_boys_table(std::vector<double>& table);
double prim_pair_bound(int la, int lb, const PrimPair64& pp, double abx, double aby, double abz, const double* boys);
double aux_prim_bound(int l, const PrimPair64& q, const double* boys);  // unit partner, no CGTO factor
double scaled_coef(double c, double a, int L);
PrimPair64 make_prim_pair(double a, double ca, const double* A, double b, double cb, const double* B);

// ri.cu
void ri_destroy(RiState* r);

}  // namespace gb
