// Batched RHF over many independent molecules (no reference counterpart: the
// reference runs RHF::solve once per molecule, src/hf.cu:245-314).
//
// All molecules live in one engine (build_engine with several inputs): shell
// pairs and quartet work lists never mix molecules, and every N x N matrix of
// molecule m is a block of the block layout (BlockMap).  One SCF iteration for
// the whole batch is:
//   * per group of equal-size molecules (molecules are sorted by (N, nocc)):
//     F' = X^T F X, eigenvectors (cuSOLVER batched syev), C = X V, D = 2 C_occ C_occ^T
//     as strided-batched DGEMMs over the group's contiguous blocks;
//   * one Fock build over all molecules (the same class kernels and work lists
//     as a single molecule: one launch per quartet class covers the batch);
//   * per-molecule energies in one kernel, read back once;
//   * DIIS for every molecule: error F D S - S D F by batched DGEMMs, then one
//     kernel with a CTA per molecule that updates that molecule's B matrix,
//     solves the bordered system and extrapolates F.
// The SCF semantics per molecule are those of the single-molecule loop (core,
// GWH, density or SAD guess, cyclic DIIS from the second stored pair, |dE|
// convergence); a converged molecule drops out of the Fock build, the DIIS
// update and the eigensolves, and its result is the one at its convergence.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#include "diis_solve.cuh"
#include "engine.hpp"

namespace gb {

int core_hamiltonian(Engine& e, double* d_S, double* d_H, cudaStream_t s);

namespace {

constexpr int kBatchDiis = 16;

struct Group {
    int first, count;  // molecules [first, first + count) of the sorted order
    int n, nocc;
    long long base;    // block offset of the first molecule
};

struct BatchState {
    int m = 8;
    double *S = nullptr, *H = nullptr, *X = nullptr, *F = nullptr, *D = nullptr, *C = nullptr, *Fp = nullptr,
           *T1 = nullptr, *T2 = nullptr, *eps = nullptr, *Es = nullptr, *Fs = nullptr, *B = nullptr,
           *energy = nullptr, *work = nullptr;
    int* info = nullptr;
    size_t work_bytes = 0;
    std::vector<void*> owned;
    ~BatchState()
    {
        for (void* p : owned) cudaFree(p);
    }
    template <class T>
    int alloc(T*& p, size_t n)
    {
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            set_error(std::string("cudaMalloc (batch): ") + cudaGetErrorString(e));
            return HF_ERR_OUT_OF_MEMORY;
        }
        owned.push_back(p);
        return HF_OK;
    }
};

int grid_of(long long n) { return static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192))); }

// X = U s^{-1/2} per block (eigenvalues below 1e-6 -> 0), from column-major eigenvectors W
__global__ void batch_transform_kernel(const double* __restrict__ W, const double* __restrict__ evals,
                                       const long long* __restrict__ ebase, const BlockMap M, double* __restrict__ X)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        const int n = M.n[m];
        const long long base = M.base[m], r = k - base;
        const int i = static_cast<int>(r / n), c = static_cast<int>(r % n);
        const double v = evals[ebase[m] + c];
        const double d = (v < 1e-6) ? 0.0 : 1.0 / sqrt(v);
        X[k] = W[base + static_cast<long long>(c) * n + i] * d;
    }
}

// GWH guess 1.75 S_pq (H_pp + H_qq) / 2 per block (src/gpu_kernels.cu:535-545)
__global__ void batch_gwh_kernel(const double* __restrict__ H, const double* __restrict__ S, const BlockMap M,
                                 double* __restrict__ F)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        const int n = M.n[m];
        const long long base = M.base[m], r = k - base;
        const long long p = r / n, q = r % n;
        F[k] = 1.75 * S[k] * (H[base + p * n + p] + H[base + q * n + q]) * 0.5;
    }
}

// D = a (+ b) over the block layout
__global__ void batch_sum_kernel(const double* __restrict__ a, const double* __restrict__ b, long long ne,
                                 double* __restrict__ D)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < ne;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        D[k] = a[k] + (b ? b[k] : 0.0);
}

// G = 2 (J' + J'^T) s s - (K' + K'^T) s s / 2, F = H + G, per block
__global__ void batch_fock_kernel(const double* __restrict__ Jp, const double* __restrict__ Kp,
                                  const double* __restrict__ s, const double* __restrict__ H, const BlockMap M,
                                  const unsigned char* __restrict__ active, double* __restrict__ F)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        if (active && !active[m]) continue;  // converged: F stays
        const int n = M.n[m], g0 = M.bf0[m];
        const long long base = M.base[m], r = k - base;
        const int i = static_cast<int>(r / n), j = static_cast<int>(r % n);
        const long long kt = base + static_cast<long long>(j) * n + i;
        const double ss = s[g0 + i] * s[g0 + j];
        F[k] = H[k] + (2.0 * (Jp[k] + Jp[kt]) - 0.5 * (Kp[k] + Kp[kt])) * ss;
    }
}

// ---- mixed tier of the batch: the single-molecule anchored rule per molecule
// out = D - Dprev over the block layout
__global__ void batch_diff_kernel(const double* __restrict__ D, const double* __restrict__ Dp, long long ne,
                                  double* __restrict__ out)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < ne;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        out[k] = D[k] - Dp[k];
}

// Per molecule, from max|D - Dprev|: FP32 full builds while unanchored and the change
// is >= anchor (or on the first build), then one FP64 full build (the anchor), then
// builds under the FP32 cut tau (incremental dD builds when incremental).  Molecules
// no longer active are not built (tau = skip = inf).
__global__ void batch_phase_kernel(const double* __restrict__ ddiff, const unsigned char* __restrict__ active,
                                   int nmol, int first, double anchor, double tau, double full_tau, double schwarz,
                                   int incremental,
                                   unsigned char* __restrict__ anchored, unsigned char* __restrict__ incr,
                                   double* __restrict__ mol_tau, double* __restrict__ mol_skip)
{
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nmol; m += gridDim.x * blockDim.x) {
        if (!active[m]) { mol_tau[m] = inf; mol_skip[m] = inf; incr[m] = 0; continue; }
        if (!anchored[m]) {
            incr[m] = 0;
            if (first || ddiff[m] >= anchor) {
                mol_tau[m] = inf;  // every quartet FP32, the small ones left out (kPreAnchorDrop)
                mol_skip[m] = fmax(schwarz, kPreAnchorDrop);
            } else {
                mol_tau[m] = 0.0;  // every quartet FP64: the anchor
                mol_skip[m] = schwarz;
                anchored[m] = 1;
            }
        } else {
            // anchored: incremental builds under the cut, or full builds at full_tau
            incr[m] = (incremental && !first) ? 1 : 0;
            mol_tau[m] = incr[m] ? tau : full_tau;
            mol_skip[m] = fmin(schwarz, mol_tau[m]);
        }
    }
}

// input density of the build: dD for incremental molecules, D otherwise
__global__ void batch_input_kernel(const double* __restrict__ D, const double* __restrict__ diff,
                                   const unsigned char* __restrict__ incr, const BlockMap M, double* __restrict__ out)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        out[k] = incr[m] ? diff[k] : D[k];
    }
}

// G (+)= both tiers' J', K' finished per block, F = H + G, Dprev = D (active molecules)
__global__ void batch_fock_mixed_kernel(const double* __restrict__ Jp, const double* __restrict__ Kp,
                                        const float* __restrict__ Jp32, const float* __restrict__ Kp32,
                                        const double* __restrict__ s, const double* __restrict__ H,
                                        const double* __restrict__ D, const BlockMap M,
                                        const unsigned char* __restrict__ active, const unsigned char* __restrict__ incr,
                                        double* __restrict__ G, double* __restrict__ F, double* __restrict__ Dprev)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        if (!active[m]) continue;
        const int n = M.n[m], g0 = M.bf0[m];
        const long long base = M.base[m], r = k - base;
        const int i = static_cast<int>(r / n), j = static_cast<int>(r % n);
        const long long kt = base + static_cast<long long>(j) * n + i;
        const double ss = s[g0 + i] * s[g0 + j];
        const double js = Jp[k] + Jp[kt] + static_cast<double>(Jp32[k]) + static_cast<double>(Jp32[kt]);
        const double ks = Kp[k] + Kp[kt] + static_cast<double>(Kp32[k]) + static_cast<double>(Kp32[kt]);
        const double g = (2.0 * js - 0.5 * ks) * ss;
        const double gn = incr[m] ? G[k] + g : g;
        G[k] = gn;
        F[k] = H[k] + gn;
        Dprev[k] = D[k];
    }
}

// E_m = 1/2 sum D (H + F) over block m: one CTA per molecule
__global__ void batch_energy_kernel(const double* __restrict__ D, const double* __restrict__ H,
                                    const double* __restrict__ F, const BlockMap M, double* __restrict__ out)
{
    __shared__ double red[32];
    const int m = blockIdx.x;
    const long long base = M.base[m], nn = static_cast<long long>(M.n[m]) * M.n[m];
    double s = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) s += D[base + k] * (H[base + k] + F[base + k]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) out[m] = 0.5 * s;
    }
}

// E = T - T^T per block
__global__ void batch_antisym_kernel(const double* __restrict__ T, const BlockMap M, double* __restrict__ E)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        const int n = M.n[m];
        const long long base = M.base[m], r = k - base;
        const int i = static_cast<int>(r / n), j = static_cast<int>(r % n);
        E[k] = T[k] - T[base + static_cast<long long>(j) * n + i];
    }
}

// One CTA per molecule: new row/column `slot` of its DIIS B matrix from the stored
// errors, then (nprev > 1) the bordered solve and F = sum c_i F_i.
__global__ void batch_diis_kernel(const double* __restrict__ Es, const double* __restrict__ Fs, long long nelem,
                                  const BlockMap M, int slot, int nprev, const unsigned char* __restrict__ active,
                                  double* __restrict__ Bm, double* __restrict__ F)
{
    __shared__ double red[32];
    __shared__ double coef[kBatchDiis];
    const int m = blockIdx.x;
    if (active && !active[m]) return;
    const long long base = M.base[m], nn = static_cast<long long>(M.n[m]) * M.n[m];
    double* B = Bm + static_cast<long long>(m) * kBatchDiis * kBatchDiis;
    const double* en = Es + static_cast<long long>(slot) * nelem + base;
    for (int j = 0; j < nprev; ++j) {
        const double* ej = Es + static_cast<long long>(j) * nelem + base;
        double s = 0.0;
        for (long long k = threadIdx.x; k < nn; k += blockDim.x) s += en[k] * ej[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += red[w];
            B[slot * kBatchDiis + j] = t;
            B[j * kBatchDiis + slot] = t;
        }
        __syncthreads();
    }
    if (nprev < 2) return;
    // weights of the independent error vectors (diis_solve.cuh)
    if (threadIdx.x == 0) diis_coefficients<kBatchDiis>(B, kBatchDiis, nprev, coef);
    __syncthreads();
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < nprev; ++i) s += coef[i] * Fs[static_cast<long long>(i) * nelem + base + k];
        F[base + k] = s;
    }
}

// ---- purification over all molecules (eigensolver 2)
// per-molecule Gershgorin interval of F' (one CTA per molecule)
__global__ void batch_gershgorin_kernel(const double* __restrict__ A, const BlockMap M, double* __restrict__ bounds)
{
    __shared__ double rlo[32], rhi[32];
    const int m = blockIdx.x, n = M.n[m];
    const double* a = A + M.base[m];
    double lo = 1e300, hi = -1e300;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r = 0.0;
        for (int j = 0; j < n; ++j)
            if (j != i) r += fabs(a[static_cast<long long>(i) * n + j]);
        const double d = a[static_cast<long long>(i) * n + i];
        lo = fmin(lo, d - r);
        hi = fmax(hi, d + r);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) { rlo[threadIdx.x >> 5] = lo; rhi[threadIdx.x >> 5] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) { lo = fmin(lo, rlo[w]); hi = fmax(hi, rhi[w]); }
        bounds[2 * m] = fmin(lo, rlo[0]);
        bounds[2 * m + 1] = fmax(hi, rhi[0]);
    }
}

__global__ void batch_sp2_init_kernel(const double* __restrict__ Fp, const double* __restrict__ bounds,
                                      const BlockMap M, float* __restrict__ P)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        const int n = M.n[m];
        const long long r = k - M.base[m];
        const double lo = bounds[2 * m], hi = bounds[2 * m + 1];
        const bool diag = (r / n) == (r % n);
        P[k] = static_cast<float>(((diag ? hi : 0.0) - Fp[k]) / (hi - lo));
    }
}

// per molecule: take P^2 if its trace is nearer nocc than 2P - P^2's (one CTA per molecule)
__global__ void batch_sp2_decide_kernel(const float* __restrict__ P, const float* __restrict__ P2, const BlockMap M,
                                        const int* __restrict__ nocc, unsigned char* __restrict__ square)
{
    __shared__ float r1[32], r2[32];
    const int m = blockIdx.x, n = M.n[m];
    const long long base = M.base[m];
    float t1 = 0.f, t2 = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        t1 += P[base + static_cast<long long>(i) * n + i];
        t2 += P2[base + static_cast<long long>(i) * n + i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        t1 += __shfl_xor_sync(0xffffffffu, t1, o);
        t2 += __shfl_xor_sync(0xffffffffu, t2, o);
    }
    if ((threadIdx.x & 31) == 0) { r1[threadIdx.x >> 5] = t1; r2[threadIdx.x >> 5] = t2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) { a += r1[w]; b += r2[w]; }
        const float no = static_cast<float>(nocc[m]);
        square[m] = fabsf(b - no) < fabsf(2.f * a - b - no) ? 1 : 0;
    }
}

__global__ void batch_sp2_update_kernel(const float* __restrict__ P, const float* __restrict__ P2, const BlockMap M,
                                        const unsigned char* __restrict__ square, float* __restrict__ Pn)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        Pn[k] = square[m] ? P2[k] : 2.f * P[k] - P2[k];
    }
}

__global__ void batch_widen_kernel(const float* __restrict__ a, long long nn, double* __restrict__ b)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        b[k] = static_cast<double>(a[k]);
}

__global__ void batch_mcweeny_kernel(const double* __restrict__ P2, const double* __restrict__ P3, long long nn,
                                     double* __restrict__ P)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        P[k] = 3.0 * P2[k] - 2.0 * P3[k];
}

// row-major strided-batched C = alpha op(A) op(B) + beta C over n x n blocks (k inner)
cublasStatus_t gemm_batched(cublasHandle_t h, bool ta, bool tb, int n, int k, double alpha, const double* A, int lda,
                            const double* B, int ldb, double beta, double* C, int count)
{
    const long long st = static_cast<long long>(n) * n;
    return cublasDgemmStridedBatched(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, n, n, k, &alpha,
                                     B, ldb, st, A, lda, st, &beta, C, n, st, count);
}

constexpr int kSyevStreams = 8;

struct Batch {
    Engine* e;
    BatchState w;
    std::vector<Group> groups;
    std::vector<long long> ebase;  // eigenvalue offsets per molecule
    long long* d_ebase = nullptr;
    cusolverDnParams_t params = nullptr;
    // per-molecule divide-and-conquer solves spread over several streams
    cudaStream_t streams[kSyevStreams] = {};
    cusolverDnHandle_t handles[kSyevStreams] = {};
    double* swork[kSyevStreams] = {};
    int* sinfo[kSyevStreams] = {};
    int swork_len = 0;
    cudaEvent_t fork = nullptr, join[kSyevStreams] = {};
    std::vector<unsigned char> active;  // molecules still iterating (host copy)
    bool purify = false;                // eigensolver 2: SP2 + McWeeny instead of batched syev
    // mixed tier (precision HF_PRECISION_MIXED): per-molecule anchored rule
    bool mixed = false;
    double anchor = 0.0, tau = 0.1, full_tau = 0.0;
    int incremental = 1;
    bool first_build = true;
    double *G = nullptr, *Dprev = nullptr, *Din = nullptr, *mol_tau = nullptr, *mol_skip = nullptr,
           *mol_dmax = nullptr, *mol_ddiff = nullptr;
    unsigned char *d_anchored = nullptr, *d_incr = nullptr;
    float *P32a = nullptr, *P32b = nullptr, *P32c = nullptr;
    double* bounds = nullptr;
    unsigned char* square = nullptr;
    int* d_nocc = nullptr;
    // graphs of the iteration's density and Fock steps (replayed when the schedule asks)
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        int uses = 0;
        bool failed = false;
        long long launches = 0;
    } density_graph, fock_graph;
    ~Batch()
    {
        for (StepGraph* g : {&density_graph, &fock_graph})
            if (g->exec) cudaGraphExecDestroy(g->exec);
        if (d_ebase) cudaFree(d_ebase);
        if (params) cusolverDnDestroyParams(params);
        for (void* p : {static_cast<void*>(P32a), static_cast<void*>(P32b), static_cast<void*>(P32c),
                        static_cast<void*>(bounds), static_cast<void*>(square), static_cast<void*>(d_nocc),
                        static_cast<void*>(G), static_cast<void*>(Dprev), static_cast<void*>(Din),
                        static_cast<void*>(mol_tau), static_cast<void*>(mol_skip), static_cast<void*>(mol_dmax),
                        static_cast<void*>(mol_ddiff), static_cast<void*>(d_anchored), static_cast<void*>(d_incr)})
            if (p) cudaFree(p);
        for (int i = 0; i < kSyevStreams; ++i) {
            if (handles[i]) cusolverDnDestroy(handles[i]);
            if (streams[i]) cudaStreamDestroy(streams[i]);
            if (swork[i]) cudaFree(swork[i]);
            if (sinfo[i]) cudaFree(sinfo[i]);
            if (join[i]) cudaEventDestroy(join[i]);
        }
        if (fork) cudaEventDestroy(fork);
    }
};

// eigenvectors (in place, column-major) and eigenvalues of every block of A, group by group
int batch_syev(Batch& b, double* A, double* evals, cudaStream_t s)
{
    Engine& e = *b.e;
    cusolverDnSetStream(e.cusolver, s);
    for (const Group& g : b.groups) {
        double* Ag = A + g.base;
        double* Wg = evals + b.ebase[g.first];
        size_t dbytes = 0, hbytes = 0;
        cusolverStatus_t q = cusolverDnXsyevBatched_bufferSize(e.cusolver, b.params, CUSOLVER_EIG_MODE_VECTOR,
                                                               CUBLAS_FILL_MODE_LOWER, g.n, CUDA_R_64F, Ag, g.n,
                                                               CUDA_R_64F, Wg, CUDA_R_64F, &dbytes, &hbytes, g.count);
        bool batched = (q == CUSOLVER_STATUS_SUCCESS) && hbytes <= (1u << 20);
        if (batched) {
            if (dbytes > b.w.work_bytes) {
                double* nw = nullptr;
                if (b.w.alloc(nw, dbytes / sizeof(double) + 1)) return HF_ERR_OUT_OF_MEMORY;
                b.w.work = nw;
                b.w.work_bytes = dbytes;
            }
            std::vector<char> hwork(std::max<size_t>(hbytes, 1));
            q = cusolverDnXsyevBatched(e.cusolver, b.params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, g.n,
                                       CUDA_R_64F, Ag, g.n, CUDA_R_64F, Wg, CUDA_R_64F, b.w.work, dbytes,
                                       hwork.data(), hbytes, b.w.info, g.count);
            batched = (q == CUSOLVER_STATUS_SUCCESS);
        }
        if (batched) continue;
        // one divide-and-conquer solve per molecule, spread over kSyevStreams streams
        if (!b.streams[0]) {
            for (int k = 0; k < kSyevStreams; ++k) {
                GB_CUDA_TRY(cudaStreamCreateWithFlags(&b.streams[k], cudaStreamNonBlocking));
                if (cusolverDnCreate(&b.handles[k]) != CUSOLVER_STATUS_SUCCESS)
                    return set_error("cusolverDnCreate failed"), HF_ERR_SOLVER;
                cusolverDnSetStream(b.handles[k], b.streams[k]);
                GB_CUDA_TRY(cudaEventCreateWithFlags(&b.join[k], cudaEventDisableTiming));
                GB_CUDA_TRY(cudaMalloc(&b.sinfo[k], sizeof(int)));
            }
            GB_CUDA_TRY(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming));
        }
        int lwork = 0;
        if (cusolverDnDsyevd_bufferSize(b.handles[0], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, g.n, Ag, g.n,
                                        Wg, &lwork) != CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnDsyevd_bufferSize failed"), HF_ERR_SOLVER;
        if (lwork > b.swork_len) {
            for (int k = 0; k < kSyevStreams; ++k) {
                if (b.swork[k]) cudaFree(b.swork[k]);
                GB_CUDA_TRY(cudaMalloc(&b.swork[k], sizeof(double) * static_cast<size_t>(lwork)));
            }
            b.swork_len = lwork;
        }
        GB_CUDA_TRY(cudaEventRecord(b.fork, s));
        const int used = std::min(kSyevStreams, g.count);
        for (int k = 0; k < used; ++k) GB_CUDA_TRY(cudaStreamWaitEvent(b.streams[k], b.fork, 0));
        for (int i = 0; i < g.count; ++i) {
            if (!b.active.empty() && !b.active[g.first + i]) continue;  // converged
            const int k = i % kSyevStreams;
            const long long off = static_cast<long long>(i) * g.n * g.n;
            if (cusolverDnDsyevd(b.handles[k], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, g.n, Ag + off, g.n,
                                 Wg + static_cast<long long>(i) * g.n, b.swork[k], b.swork_len, b.sinfo[k]) !=
                CUSOLVER_STATUS_SUCCESS)
                return set_error("cusolverDnDsyevd (batch) failed"), HF_ERR_SOLVER;
        }
        for (int k = 0; k < used; ++k) {
            GB_CUDA_TRY(cudaEventRecord(b.join[k], b.streams[k]));
            GB_CUDA_TRY(cudaStreamWaitEvent(s, b.join[k], 0));
        }
    }
    return HF_OK;
}

// C and D from F for every molecule: F' = X^T F X, eigenvectors V, C = X V, D = 2 C_occ C_occ^T
int batch_purify(Batch& b, cudaStream_t s);

// cuBLAS on stream s; while a graph is captured on the schedule's capture stream it
// runs on the engine-owned workspace (its own pool may allocate, which a capture forbids)
void bind_cublas(Engine& e, cudaStream_t s)
{
    cublasSetStream(e.cublas, s);
    if (s == e.sched.capture && e.sched.cublas_ws)
        cublasSetWorkspace(e.cublas, e.sched.cublas_ws, kCublasCaptureWorkspace);
}

int batch_density(Batch& b, const double* F, cudaStream_t s)
{
    Engine& e = *b.e;
    BatchState& w = b.w;
    bind_cublas(e, s);
    for (const Group& g : b.groups) {
        const long long o = g.base;
        if (gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, F + o, g.n, w.X + o, g.n, 0.0, w.T1 + o, g.count) ||
            gemm_batched(e.cublas, true, false, g.n, g.n, 1.0, w.X + o, g.n, w.T1 + o, g.n, 0.0, w.Fp + o, g.count))
            return set_error("cublasDgemmStridedBatched (F') failed"), HF_ERR_SOLVER;
    }
    if (b.purify) return batch_purify(b, s);
    int st = batch_syev(b, w.Fp, w.eps, s);
    if (st) return st;
    for (const Group& g : b.groups) {
        const long long o = g.base;
        // V as row-major is V^T (column-major eigenvectors): C = X (V^T)^T
        if (gemm_batched(e.cublas, false, true, g.n, g.n, 1.0, w.X + o, g.n, w.Fp + o, g.n, 0.0, w.C + o, g.count) ||
            gemm_batched(e.cublas, false, true, g.n, g.nocc, 2.0, w.C + o, g.n, w.C + o, g.n, 0.0, w.D + o, g.count))
            return set_error("cublasDgemmStridedBatched (C, D) failed"), HF_ERR_SOLVER;
    }
    return HF_OK;
}

// D = 2 X P X^T with P from FP32 SP2 steps on every molecule's F' (strided-batched SGEMM per
// group, per-molecule trace decisions on the device) and FP64 McWeeny steps
int batch_purify(Batch& b, cudaStream_t s)
{
    Engine& e = *b.e;
    BatchState& w = b.w;
    const long long ne = e.nelem;
    const BlockMap M = e.block_map();
    batch_gershgorin_kernel<<<e.nmol, 256, 0, s>>>(w.Fp, M, b.bounds);
    GB_LAUNCH_CHECK();
    batch_sp2_init_kernel<<<grid_of(ne), 256, 0, s>>>(w.Fp, b.bounds, M, b.P32a);
    GB_LAUNCH_CHECK();
    float* P = b.P32a;
    float* Pn = b.P32b;
    float* P2 = b.P32c;
    const float one = 1.f, zero = 0.f;
    for (int k = 0; k < 50; ++k) {
        for (const Group& g : b.groups) {
            const long long st = static_cast<long long>(g.n) * g.n;
            if (cublasSgemmStridedBatched(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, g.n, g.n, g.n, &one, P + g.base, g.n, st,
                                          P + g.base, g.n, st, &zero, P2 + g.base, g.n, st, g.count) !=
                CUBLAS_STATUS_SUCCESS)
                return set_error("cublasSgemmStridedBatched (purification) failed"), HF_ERR_SOLVER;
        }
        batch_sp2_decide_kernel<<<e.nmol, 256, 0, s>>>(P, P2, M, b.d_nocc, b.square);
        GB_LAUNCH_CHECK();
        batch_sp2_update_kernel<<<grid_of(ne), 256, 0, s>>>(P, P2, M, b.square, Pn);
        GB_LAUNCH_CHECK();
        std::swap(P, Pn);
    }
    batch_widen_kernel<<<grid_of(ne), 256, 0, s>>>(P, ne, w.Fp);
    GB_LAUNCH_CHECK();
    for (int k = 0; k < 3; ++k) {
        for (const Group& g : b.groups) {
            const long long o = g.base;
            if (gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, w.Fp + o, g.n, w.Fp + o, g.n, 0.0, w.T1 + o,
                             g.count) ||
                gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, w.T1 + o, g.n, w.Fp + o, g.n, 0.0, w.T2 + o,
                             g.count))
                return set_error("cublasDgemmStridedBatched (McWeeny) failed"), HF_ERR_SOLVER;
        }
        batch_mcweeny_kernel<<<grid_of(ne), 256, 0, s>>>(w.T1, w.T2, ne, w.Fp);
        GB_LAUNCH_CHECK();
    }
    for (const Group& g : b.groups) {
        const long long o = g.base;
        if (gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, w.X + o, g.n, w.Fp + o, g.n, 0.0, w.T1 + o, g.count) ||
            gemm_batched(e.cublas, false, true, g.n, g.n, 2.0, w.T1 + o, g.n, w.X + o, g.n, 0.0, w.D + o, g.count))
            return set_error("cublasDgemmStridedBatched (X P X^T) failed"), HF_ERR_SOLVER;
    }
    return HF_OK;
}

int batch_fock(Batch& b, cudaStream_t s)
{
    Engine& e = *b.e;
    if (b.mixed) {
        const long long ne = e.nelem;
        batch_diff_kernel<<<grid_of(ne), 256, 0, s>>>(b.w.D, b.Dprev, ne, b.Din);
        GB_LAUNCH_CHECK();
        int st = mol_absmax(e, b.Din, b.mol_ddiff, s);
        if (st) return st;
        batch_phase_kernel<<<(e.nmol + 255) / 256, 256, 0, s>>>(b.mol_ddiff, e.d_mol_active, e.nmol,
                                                                b.first_build ? 1 : 0, b.anchor, b.tau, b.full_tau,
                                                                e.schwarz_threshold, b.incremental, b.d_anchored,
                                                                b.d_incr, b.mol_tau, b.mol_skip);
        GB_LAUNCH_CHECK();
        batch_input_kernel<<<grid_of(ne), 256, 0, s>>>(b.w.D, b.Din, b.d_incr, e.block_map(), b.Din);
        GB_LAUNCH_CHECK();
        if ((st = build_jk_batch(e, b.Din, b.mol_tau, b.mol_skip, b.mol_dmax, s))) return st;
        batch_fock_mixed_kernel<<<grid_of(ne), 256, 0, s>>>(e.d_Jp, e.d_Kp, e.d_Jp32, e.d_Kp32, e.d_scale, b.w.H,
                                                            b.w.D, e.block_map(), e.d_mol_active, b.d_incr, b.G,
                                                            b.w.F, b.Dprev);
        GB_LAUNCH_CHECK();
        b.first_build = false;
        return HF_OK;
    }
    int st = build_jk(e, b.w.D, nullptr, nullptr, HF_PRECISION_FP64, 0.0, s);
    if (st) return st;
    batch_fock_kernel<<<grid_of(e.nelem), 256, 0, s>>>(e.d_Jp, e.d_Kp, e.d_scale, b.w.H, e.block_map(),
                                                       e.d_mol_active, b.w.F);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// One step of the batch iteration (body(stream) issues its launches) under the engine's
// graph schedule: ordinary launches on the first call, captured on the schedule's
// capture stream on the second, replayed from then on.  The step reads the batch's
// buffers (F, D, the active flags, the per-molecule phase) at replay, so it may be
// captured once the iteration's launch sequence no longer changes.  A failed capture
// leaves the step on ordinary launches.
template <class Body>
int run_step(Batch& b, Batch::StepGraph& g, cudaStream_t s, Body body)
{
    Engine& e = *b.e;
    FockSchedule& S = e.sched;
    if (!S.use_graph || g.failed || (!g.exec && g.uses++ == 0)) return body(s);
    if (!g.exec) {
        int st = schedule_streams(e);
        if (st) return st;
        if (!S.cublas_ws) GB_CUDA_TRY(cudaMalloc(&S.cublas_ws, kCublasCaptureWorkspace));
        const long long l0 = launch_count();
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamBeginCapture(S.capture, cudaStreamCaptureModeThreadLocal);
        if (ce == cudaSuccess) {
            st = body(S.capture);
            ce = cudaStreamEndCapture(S.capture, &graph);
        }
        bind_cublas(e, s);
        const long long recorded = launch_count() - l0;
        count_launches(-recorded);  // recorded, not launched
        cudaGraphExec_t exec = nullptr;
        if (!st && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
            g.exec = exec;
            g.launches = recorded;
        }
        if (graph) cudaGraphDestroy(graph);
        if (!g.exec) {
            cudaGetLastError();  // capture errors are not sticky; clear the last-error slot
            g.failed = true;
            clear_error();
            return body(s);
        }
    }
    GB_CUDA_TRY(cudaGraphLaunch(g.exec, s));
    count_launches(g.launches);
    ++S.graph_replays;
    return HF_OK;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int hf_engine_create_batch(int num_molecules, const hf_primitive_shell* const* prims, const int* num_primitives,
                           const double* const* cgto_norm, const int* num_basis, const hf_atom* const* atoms,
                           const int* num_atoms, double schwarz_threshold, hf_engine** out)
{
    clear_error();
    if (num_molecules <= 0 || !prims || !num_primitives || !cgto_norm || !num_basis || !atoms || !num_atoms || !out)
        return set_error("hf_engine_create_batch: null argument"), HF_ERR_INVALID_ARGUMENT;
    std::vector<MolInput> mols(num_molecules);
    for (int m = 0; m < num_molecules; ++m)
        mols[m] = MolInput{prims[m], num_primitives[m], cgto_norm[m], num_basis[m], atoms[m], num_atoms[m]};
    return build_engine(mols.data(), num_molecules, schwarz_threshold, out);
}

int hf_batch_rhf_scf(hf_engine* eng, const int* num_electrons, const hf_scf_options* opt_in, hf_scf_result* results,
                     double* batch_scf_ms, int* batch_iterations)
{
    clear_error();
    if (!eng || !num_electrons || !results) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    hf_scf_options opt;
    if (opt_in) opt = *opt_in; else hf_scf_options_default(&opt);
    if (opt.diis_size < 1 || opt.diis_size > kBatchDiis)
        return set_error("diis_size must be in [1, 16]"), HF_ERR_INVALID_ARGUMENT;
    if (opt.initial_guess < HF_GUESS_CORE || opt.initial_guess > HF_GUESS_SAD)
        return set_error("initial_guess: core, GWH, density or SAD"), HF_ERR_INVALID_ARGUMENT;
    const bool density_guess = opt.initial_guess == HF_GUESS_DENSITY || opt.initial_guess == HF_GUESS_SAD;
    if (density_guess && !opt.guess_density_a)
        return set_error("initial_guess density/SAD needs guess_density_a (block layout)"), HF_ERR_INVALID_ARGUMENT;
    if (opt.orthogonalizer)
        return set_error("hf_batch_rhf_scf: the orthogonalizer option is single-molecule only"),
               HF_ERR_INVALID_ARGUMENT;
    const int nmol = e.nmol;
    Batch b;
    b.e = &e;
    // groups of consecutive molecules with equal (N, nocc)
    for (int m = 0; m < nmol; ++m) {
        const int ne = num_electrons[m];
        if (ne <= 0 || (ne & 1) || ne / 2 > e.mol_n[m])
            return set_error("molecule " + std::to_string(m) + ": RHF needs an even electron count <= 2N"),
                   HF_ERR_INVALID_ARGUMENT;
        if (!b.groups.empty() && b.groups.back().n == e.mol_n[m] && b.groups.back().nocc == ne / 2 &&
            b.groups.back().first + b.groups.back().count == m)
            b.groups.back().count++;
        else
            b.groups.push_back(Group{m, 1, e.mol_n[m], ne / 2, e.mol_base[m]});
    }
    b.ebase.assign(nmol + 1, 0);
    for (int m = 0; m < nmol; ++m) b.ebase[m + 1] = b.ebase[m] + e.mol_n[m];
    cudaStream_t s = nullptr;
    const long long ne = e.nelem;
    BatchState& w = b.w;
    int st;
    if ((st = w.alloc(w.S, ne)) || (st = w.alloc(w.H, ne)) || (st = w.alloc(w.X, ne)) || (st = w.alloc(w.F, ne)) ||
        (st = w.alloc(w.D, ne)) || (st = w.alloc(w.C, ne)) || (st = w.alloc(w.Fp, ne)) || (st = w.alloc(w.T1, ne)) ||
        (st = w.alloc(w.T2, ne)) || (st = w.alloc(w.eps, b.ebase[nmol])) ||
        (st = w.alloc(w.Es, static_cast<size_t>(opt.diis_size) * ne)) ||
        (st = w.alloc(w.Fs, static_cast<size_t>(opt.diis_size) * ne)) ||
        (st = w.alloc(w.B, static_cast<size_t>(nmol) * kBatchDiis * kBatchDiis)) || (st = w.alloc(w.energy, nmol)) ||
        (st = w.alloc(w.info, std::max(nmol, 1))))
        return st;
    if (cudaMalloc(&b.d_ebase, sizeof(long long) * (nmol + 1)) != cudaSuccess)
        return set_error("cudaMalloc failed"), HF_ERR_OUT_OF_MEMORY;
    GB_CUDA_TRY(cudaMemcpy(b.d_ebase, b.ebase.data(), sizeof(long long) * (nmol + 1), cudaMemcpyHostToDevice));
    if (cusolverDnCreateParams(&b.params) != CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnCreateParams failed"), HF_ERR_SOLVER;
    if (opt.eigensolver == HF_EIGEN_PURIFICATION) {
        b.purify = true;
        std::vector<int> nocc(nmol);
        for (int m2 = 0; m2 < nmol; ++m2) nocc[m2] = num_electrons[m2] / 2;
        if (cudaMalloc(&b.P32a, sizeof(float) * ne) != cudaSuccess ||
            cudaMalloc(&b.P32b, sizeof(float) * ne) != cudaSuccess ||
            cudaMalloc(&b.P32c, sizeof(float) * ne) != cudaSuccess ||
            cudaMalloc(&b.bounds, sizeof(double) * 2 * nmol) != cudaSuccess ||
            cudaMalloc(&b.square, nmol) != cudaSuccess || cudaMalloc(&b.d_nocc, sizeof(int) * nmol) != cudaSuccess)
            return set_error("cudaMalloc (batch purification) failed"), HF_ERR_OUT_OF_MEMORY;
        GB_CUDA_TRY(cudaMemcpy(b.d_nocc, nocc.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice));
    }
    if (opt.precision != HF_PRECISION_FP64 && opt.precision != HF_PRECISION_MIXED)
        return set_error("unknown precision"), HF_ERR_INVALID_ARGUMENT;
    if (opt.precision == HF_PRECISION_MIXED) {
        // the anchored mixed tier of hf_rhf_scf, decided per molecule on the device
        b.mixed = true;
        b.anchor = opt.anchor_threshold;
        b.tau = opt.mixed_threshold;
        b.incremental = opt.incremental;
        b.full_tau = (opt.full_build_precision == HF_PRECISION_MIXED) ? opt.mixed_threshold : 0.0;
        const size_t nb = sizeof(double) * ne;
        if (cudaMalloc(&b.G, nb) != cudaSuccess || cudaMalloc(&b.Dprev, nb) != cudaSuccess ||
            cudaMalloc(&b.Din, nb) != cudaSuccess || cudaMalloc(&b.mol_tau, sizeof(double) * nmol) != cudaSuccess ||
            cudaMalloc(&b.mol_skip, sizeof(double) * nmol) != cudaSuccess ||
            cudaMalloc(&b.mol_dmax, sizeof(double) * nmol) != cudaSuccess ||
            cudaMalloc(&b.mol_ddiff, sizeof(double) * nmol) != cudaSuccess ||
            cudaMalloc(&b.d_anchored, nmol) != cudaSuccess || cudaMalloc(&b.d_incr, nmol) != cudaSuccess)
            return set_error("cudaMalloc (batch mixed tier) failed"), HF_ERR_OUT_OF_MEMORY;
        GB_CUDA_TRY(cudaMemsetAsync(b.Dprev, 0, nb, s));
        GB_CUDA_TRY(cudaMemsetAsync(b.G, 0, nb, s));
        // anchor_threshold <= 0: anchored from the start (the first build is a full one), as in hf_rhf_scf
        GB_CUDA_TRY(cudaMemsetAsync(b.d_anchored, opt.anchor_threshold > 0.0 ? 0 : 1, nmol, s));
    }
    GB_CUDA_TRY(cudaMemsetAsync(w.B, 0, sizeof(double) * nmol * kBatchDiis * kBatchDiis, s));
    // molecules still iterating: the Fock kernels, the F update, DIIS and the eigensolves skip the others
    unsigned char* d_active = nullptr;
    if (w.alloc(d_active, nmol)) return HF_ERR_OUT_OF_MEMORY;
    b.active.assign(nmol, 1);
    GB_CUDA_TRY(cudaMemcpyAsync(d_active, b.active.data(), nmol, cudaMemcpyHostToDevice, s));
    struct ActiveGuard {
        Engine& e;
        ~ActiveGuard() { e.d_mol_active = nullptr; }
    } active_guard{e};
    e.d_mol_active = d_active;
    std::vector<double> enuc(nmol, 0.0);
    for (int m = 0; m < nmol; ++m)
        for (int i = 0; i < e.mol_natom[m]; ++i)
            for (int j = i + 1; j < e.mol_natom[m]; ++j) {
                const hf_atom& A = e.atoms[e.mol_atom0[m] + i];
                const hf_atom& B = e.atoms[e.mol_atom0[m] + j];
                const double dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
                enuc[m] += static_cast<double>(A.atomic_number) * B.atomic_number / std::sqrt(dx * dx + dy * dy + dz * dz);
            }

    ScopedEvents<5> evs;
    cudaEvent_t l0 = evs.ev[0], l1 = evs.ev[1];
    // setup: S, H, X = U s^-1/2, guess (core, GWH, density, SAD as in hf_rhf_scf)
    if ((st = core_hamiltonian(e, w.S, w.H, s))) return st;
    GB_CUDA_TRY(cudaMemcpyAsync(w.Fp, w.S, sizeof(double) * ne, cudaMemcpyDeviceToDevice, s));
    if ((st = batch_syev(b, w.Fp, w.eps, s))) return st;
    batch_transform_kernel<<<grid_of(ne), 256, 0, s>>>(w.Fp, w.eps, b.d_ebase, e.block_map(), w.X);
    GB_LAUNCH_CHECK();
    if (density_guess) {
        batch_sum_kernel<<<grid_of(ne), 256, 0, s>>>(opt.guess_density_a, opt.guess_density_b, ne, w.D);
        GB_LAUNCH_CHECK();
        if ((st = batch_fock(b, s))) return st;
        if (opt.initial_guess == HF_GUESS_SAD && ((st = batch_density(b, w.F, s)) || (st = batch_fock(b, s))))
            return st;
    } else {
        if (opt.initial_guess == HF_GUESS_GWH) {
            batch_gwh_kernel<<<grid_of(ne), 256, 0, s>>>(w.H, w.S, e.block_map(), w.F);
            GB_LAUNCH_CHECK();
            if ((st = batch_density(b, w.F, s))) return st;
        } else if ((st = batch_density(b, w.H, s))) {
            return st;
        }
        if ((st = batch_fock(b, s))) return st;
    }

    std::vector<double> E(nmol), prev(nmol, std::numeric_limits<double>::max());
    std::vector<unsigned char> anchored(nmol, 1);
    std::vector<int> done_iter(nmol, -1);
    std::vector<double> done_energy(nmol, 0.0);
    const int m = opt.diis_size;
    int iter = 0, diis_iter = 0, ndone = 0;
    cudaEventRecord(l0, s);
    cudaEvent_t p0 = evs.ev[2], p1 = evs.ev[3], p2 = evs.ev[4];
    double diag_ms = 0.0, fock_ms = 0.0;
    while (iter < opt.max_iter) {
        cudaEventRecord(p0, s);
        // the purified density step and the Fock build have the same launches every
        // iteration (after the first build, whose phase rule differs): graph-replayed
        // under the schedule's use_graph; batched syev stays on ordinary launches
        if (b.purify) {
            if ((st = run_step(b, b.density_graph, s, [&](cudaStream_t cs) { return batch_density(b, w.F, cs); })))
                return st;
        } else if ((st = batch_density(b, w.F, s))) {
            return st;
        }
        cudaEventRecord(p1, s);
        if (b.mixed && b.first_build) {
            if ((st = batch_fock(b, s))) return st;
        } else if ((st = run_step(b, b.fock_graph, s, [&](cudaStream_t cs) { return batch_fock(b, cs); }))) {
            return st;
        }
        cudaEventRecord(p2, s);
        batch_energy_kernel<<<nmol, 256, 0, s>>>(w.D, w.H, w.F, e.block_map(), w.energy);
        GB_LAUNCH_CHECK();
        GB_CUDA_TRY(cudaMemcpyAsync(E.data(), w.energy, sizeof(double) * nmol, cudaMemcpyDeviceToHost, s));
        if (b.mixed)
            GB_CUDA_TRY(cudaMemcpyAsync(anchored.data(), b.d_anchored, nmol, cudaMemcpyDeviceToHost, s));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        {
            float a = 0.f, c = 0.f;
            cudaEventElapsedTime(&a, p0, p1);
            cudaEventElapsedTime(&c, p1, p2);
            diag_ms += a;
            fock_ms += c;
        }
        for (int k = 0; k < nmol; ++k) {
            if (!std::isfinite(E[k])) return set_error("batch SCF energy is not finite"), HF_ERR_NOT_CONVERGED;
            // the mixed tier may not converge before the molecule's FP64 anchor build
            if (done_iter[k] < 0 && std::fabs(E[k] - prev[k]) < opt.convergence_threshold &&
                (!b.mixed || anchored[k])) {
                done_iter[k] = iter;
                done_energy[k] = E[k];
                ++ndone;
                b.active[k] = 0;
            }
        }
        if (ndone == nmol) break;
        GB_CUDA_TRY(cudaMemcpyAsync(d_active, b.active.data(), nmol, cudaMemcpyHostToDevice, s));
        ++iter;
        prev = E;
        // DIIS: e = F D S - S D F per molecule, stored with F in the ring
        const int slot = diis_iter % m;
        double* Es = w.Es + static_cast<long long>(slot) * ne;
        for (const Group& g : b.groups) {
            const long long o = g.base;
            if (gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, w.F + o, g.n, w.D + o, g.n, 0.0, w.T1 + o, g.count) ||
                gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, w.T1 + o, g.n, w.S + o, g.n, 0.0, w.T2 + o, g.count))
                return set_error("cublasDgemmStridedBatched (DIIS) failed"), HF_ERR_SOLVER;
        }
        batch_antisym_kernel<<<grid_of(ne), 256, 0, s>>>(w.T2, e.block_map(), Es);
        GB_LAUNCH_CHECK();
        if (opt.diis_include_transform) {
            for (const Group& g : b.groups) {
                const long long o = g.base;
                if (gemm_batched(e.cublas, true, false, g.n, g.n, 1.0, w.X + o, g.n, Es + o, g.n, 0.0, w.T1 + o, g.count) ||
                    gemm_batched(e.cublas, false, false, g.n, g.n, 1.0, w.T1 + o, g.n, w.X + o, g.n, 0.0, Es + o, g.count))
                    return set_error("cublasDgemmStridedBatched (DIIS transform) failed"), HF_ERR_SOLVER;
            }
        }
        GB_CUDA_TRY(cudaMemcpyAsync(w.Fs + static_cast<long long>(slot) * ne, w.F, sizeof(double) * ne,
                                    cudaMemcpyDeviceToDevice, s));
        const int nprev = std::min(diis_iter + 1, m);
        batch_diis_kernel<<<nmol, 256, 0, s>>>(w.Es, w.Fs, ne, e.block_map(), slot, nprev, e.d_mol_active, w.B,
                                               w.F);
        GB_LAUNCH_CHECK();
        ++diis_iter;
    }
    cudaEventRecord(l1, s);
    GB_CUDA_TRY(cudaEventSynchronize(l1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, l0, l1);
    if (batch_scf_ms) *batch_scf_ms = ms;
    if (batch_iterations) *batch_iterations = iter;
    for (int k = 0; k < nmol; ++k) {
        hf_scf_result& r = results[k];
        r = hf_scf_result{};
        r.nuclear_repulsion = enuc[k];
        r.converged = done_iter[k] >= 0 ? 1 : 0;
        r.electronic_energy = r.converged ? done_energy[k] : E[k];
        r.total_energy = r.electronic_energy + enuc[k];
        r.iterations = r.converged ? done_iter[k] : iter;
        r.scf_ms_total = ms;
        r.diag_ms_total = diag_ms;
        r.fock_ms_total = fock_ms;
    }
    return ndone == nmol ? HF_OK : (set_error("batch SCF: not every molecule converged"), HF_ERR_NOT_CONVERGED);
}

}  // extern "C"
