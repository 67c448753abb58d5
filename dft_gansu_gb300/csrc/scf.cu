// Restricted Hartree-Fock SCF on the device, following the reference loop
// (HF::single_point_energy, src/hf.cu:245-314):
//   X = U s^{-1/2}, eigenvalues below 1e-6 zeroed      src/hf.cu:171-243, src/gpu_kernels.cu:28-43
//   core guess: C from H, D, F = F(D)                   include/rhf.hpp:378-396
//   loop: C from F (F' = X^T F X, syevd, C = X C')     src/gpu_manager.cu:529-599
//         D = 2 C_occ C_occ^T                           src/gpu_kernels.cu:54-69
//         F = F(D); E = 1/2 (<D,H> + <D,F>)             src/gpu_manager.cu:827-836
//         stop when |E - E_prev| < threshold            src/hf.cu:297-300
//         DIIS: e = FDS - SDF, cyclic store of (e, F), extrapolate once two
//         pairs are stored                              include/rhf.hpp:298-327
// The DIIS B matrix, its bordered FP64 solve (partial-pivot Gaussian
// elimination, the algorithm of the reference's getrf/getrs) and the
// extrapolation all run on the device: no host round trip per DIIS step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <limits>
#include <string>
#include <vector>

#include "diis_solve.cuh"
#include "engine.hpp"
#include "purify.hpp"
#include "ri.hpp"

namespace gb {

namespace {

constexpr int kMaxDiis = 16;

// CUDA events and the pinned read-back slots of one SCF call (energy at 0, the
// purification status words at 8), released on every return path (early error
// returns included)
struct LoopResources {
    cudaEvent_t ev[8] = {};
    double* h_energy = nullptr;
    LoopResources()
    {
        for (auto& x : ev) cudaEventCreate(&x);
        cudaMallocHost(&h_energy, (8 + kPurifyStatusWords) * sizeof(double));
    }
    ~LoopResources()
    {
        for (auto x : ev)
            if (x) cudaEventDestroy(x);
        if (h_energy) cudaFreeHost(h_energy);
    }
    LoopResources(const LoopResources&) = delete;
    LoopResources& operator=(const LoopResources&) = delete;
};

int gemm_rm(cublasHandle_t h, bool ta, bool tb, int n, const double* A, const double* B, double* C,
            double alpha = 1.0, double beta = 0.0)
{
    // row-major C = op(A) op(B)  <=>  column-major C^T = op(B)^T op(A)^T
    const cublasStatus_t st = cublasDgemm(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, n, n, n,
                                          &alpha, B, n, A, n, &beta, C, n);
    if (st != CUBLAS_STATUS_SUCCESS) return set_error("cublasDgemm failed"), HF_ERR_CUDA;
    return HF_OK;
}

// eigenvalues of S below this are dropped from X = U s^{-1/2} (src/hf.cu:171-243)
constexpr double kOrthoCut = 1e-6;

__global__ void transform_kernel(const double* __restrict__ W, const double* __restrict__ s, int n,
                                 double* __restrict__ X)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(k / n), c = static_cast<int>(k % n);
        const double v = s[c];
        const double d = (v < kOrthoCut) ? 0.0 : 1.0 / sqrt(v);
        X[k] = W[static_cast<long long>(c) * n + i] * d;  // U[i][c] * s_c^{-1/2}
    }
}

__global__ void density_kernel(const double* __restrict__ C, int n, int nocc, double* __restrict__ D)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = k / n, j = k % n;
        double s = 0.0;
        for (int o = 0; o < nocc; ++o) s += C[i * n + o] * C[j * n + o];
        D[k] = 2.0 * s;
    }
}

__global__ void energy_kernel(const double* __restrict__ D, const double* __restrict__ H,
                              const double* __restrict__ F, long long nn, double* __restrict__ out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) s += D[k] * (H[k] + F[k]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) *out = 0.5 * s;
    }
}

// s = sum Fp (D - Dp), c = sum (F - Fp)(D - Dp) (traces of products of symmetric
// matrices), one block
__global__ void damping_traces_kernel(const double* __restrict__ F, const double* __restrict__ Fp,
                                      const double* __restrict__ D, const double* __restrict__ Dp, long long nn,
                                      double* __restrict__ out)
{
    __shared__ double r1[32], r2[32];
    double s1 = 0.0, s2 = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) {
        const double dd = D[k] - Dp[k];
        s1 += Fp[k] * dd;
        s2 += (F[k] - Fp[k]) * dd;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) { r1[threadIdx.x >> 5] = s1; r2[threadIdx.x >> 5] = s2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) { a += r1[w]; b += r2[w]; }
        out[0] = a;
        out[1] = b;
    }
}

// damping (src/gpu_manager.cu:989-1007): M = (1 - a) M_prev + a M, stored in both
__global__ void damp_kernel(double* __restrict__ Mp, double* __restrict__ M, double a, long long nn)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double v = (1.0 - a) * Mp[k] + a * M[k];
        Mp[k] = v;
        M[k] = v;
    }
}

// E = T - T^T
__global__ void antisym_kernel(const double* __restrict__ T, int n, double* __restrict__ E)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = k / n, j = k % n;
        E[k] = T[k] - T[j * n + i];
    }
}

__global__ void sub_kernel(const double* __restrict__ A, const double* __restrict__ B, long long nn,
                           double* __restrict__ C)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        C[k] = A[k] - B[k];
}

// G (+)= s (2 (J' + J'^T) - 1/2 (K' + K'^T)) s ; F = H + G
__global__ void fock_from_jk_kernel(const double* __restrict__ Jp, const double* __restrict__ Kp,
                                    const float* __restrict__ Jp32, const float* __restrict__ Kp32,
                                    const double* __restrict__ s, const double* __restrict__ H, int n, int accumulate,
                                    double* __restrict__ G, double* __restrict__ F)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(k / n), j = static_cast<int>(k % n);
        const long long kt = static_cast<long long>(j) * n + i;
        double jsum = Jp[k] + Jp[kt], ksum = Kp[k] + Kp[kt];
        if (Jp32) {
            jsum += static_cast<double>(Jp32[k]) + static_cast<double>(Jp32[kt]);
            ksum += static_cast<double>(Kp32[k]) + static_cast<double>(Kp32[kt]);
        }
        const double g = (2.0 * jsum - 0.5 * ksum) * s[i] * s[j];
        const double gn = accumulate ? G[k] + g : g;
        G[k] = gn;
        F[k] = H[k] + gn;
    }
}

// B_ij = <e_i, e_j> for i <= j < m; one block per (i, j).
__global__ void diis_dots_kernel(const double* __restrict__ Es, int m, long long nn, double* __restrict__ B)
{
    __shared__ double red[32];
    int p = blockIdx.x, i = 0;
    while (p >= m - i) { p -= m - i; ++i; }
    const int j = i + p;
    const double* a = Es + i * nn;
    const double* b = Es + j * nn;
    double s = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) s += a[k] * b[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) { B[i * kMaxDiis + j] = s; B[j * kMaxDiis + i] = s; }
    }
}

// DIIS weights (diis_solve.cuh: the constrained minimiser on the independent error
// vectors); *status = how many vectors were left out as dependent on others.
__global__ void diis_solve_kernel(const double* __restrict__ B, int m, double* __restrict__ coef, int* status)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int dropped = diis_coefficients<kMaxDiis>(B, kMaxDiis, m, coef);
    if (dropped) atomicAdd(status, dropped);
}

__global__ void diis_combine_kernel(const double* __restrict__ Fs, const double* __restrict__ coef, int m, long long nn,
                                    double* __restrict__ F)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < m; ++i) s += coef[i] * Fs[i * nn + k];
        F[k] = s;
    }
}

// D = factor sum_{o < nocc} C_o C_o^T (UHF spin densities use factor 1)
__global__ void density_factor_kernel(const double* __restrict__ C, int n, int nocc, double factor,
                                      double* __restrict__ D)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = k / n, j = k % n;
        double s = 0.0;
        for (int o = 0; o < nocc; ++o) s += C[i * n + o] * C[j * n + o];
        D[k] = factor * s;
    }
}

// UHF energy 1/2 sum [(Da + Db) H + Da Fa + Db Fb]
__global__ void uhf_energy_kernel(const double* __restrict__ Da, const double* __restrict__ Db,
                                  const double* __restrict__ H, const double* __restrict__ Fa,
                                  const double* __restrict__ Fb, long long nn, double* __restrict__ out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x)
        s += (Da[k] + Db[k]) * H[k] + Da[k] * Fa[k] + Db[k] * Fb[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) *out = 0.5 * s;
    }
}

// Fa = H + Ja + Jb - Ka, Fb = H + Ja + Jb - Kb
__global__ void uhf_fock_kernel(const double* __restrict__ H, const double* __restrict__ Ja,
                                const double* __restrict__ Jb, const double* __restrict__ Ka,
                                const double* __restrict__ Kb, long long nn, double* __restrict__ Fa,
                                double* __restrict__ Fb)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double h = H[k] + Ja[k] + Jb[k];
        Fa[k] = h - Ka[k];
        Fb[k] = h - Kb[k];
    }
}

// generalised Wolfsberg-Helmholz guess F_pq = c S_pq (H_pp + H_qq) / 2 for every p, q, c = 1.75
// (the reference's computeInitialFockMatrix_GWH_kernel, src/gpu_kernels.cu:535-545, includes the diagonal)
__global__ void gwh_kernel(const double* __restrict__ H, const double* __restrict__ S, int n, double* __restrict__ F)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long p = k / n, q = k % n;
        F[k] = 1.75 * S[k] * (H[p * n + p] + H[q * n + q]) * 0.5;
    }
}

// out = fa a + fb b (b may be NULL)
__global__ void combine_kernel(const double* __restrict__ a, double fa, const double* __restrict__ b, double fb,
                               long long nn, double* __restrict__ out)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        out[k] = fa * a[k] + (b ? fb * b[k] : 0.0);
}

// F_a = H + Ja + Jb - Ka, F_b = H + Ja + Jb - Kb
__global__ void uhf_combine_kernel(const double* __restrict__ H, const double* __restrict__ Ja,
                                   const double* __restrict__ Jb, const double* __restrict__ Ka,
                                   const double* __restrict__ Kb, long long nn, double* __restrict__ Fa,
                                   double* __restrict__ Fb)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double c = H[k] + Ja[k] + Jb[k];
        Fa[k] = c - Ka[k];
        Fb[k] = c - Kb[k];
    }
}

// InitialGuess_UHF::break_symmetry (include/uhf.hpp:429-436): the last basis function's
// row and the last orbital's column of the beta coefficients set to zero
__global__ void break_symmetry_kernel(double* __restrict__ C, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        C[static_cast<long long>(n - 1) * n + i] = 0.0;
        C[static_cast<long long>(i) * n + (n - 1)] = 0.0;
    }
}

// ---- ROHF (src/rohf.cu, src/gpu_kernels.cu:98-139, :351-498)
// D_c = 2 sum_{o < nc} C_o C_o^T, D_o = sum_{nc <= o < nc + no} C_o C_o^T, D = D_c + D_o
__global__ void rohf_density_kernel(const double* __restrict__ C, int n, int nc, int no, double* __restrict__ Dc,
                                    double* __restrict__ Do, double* __restrict__ D)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = k / n, j = k % n;
        double c = 0.0, o = 0.0;
        for (int q = 0; q < nc; ++q) c += C[i * n + q] * C[j * n + q];
        for (int q = nc; q < nc + no; ++q) o += C[i * n + q] * C[j * n + q];
        Dc[k] = 2.0 * c;
        Do[k] = o;
        D[k] = 2.0 * c + o;
    }
}

// F_c = H + J - K_c/2 - K_o/2, F_o = (H + J - K_c/2 - K_o)/2 with J = J(D_c) + J(D_o)
__global__ void rohf_fock_kernel(const double* __restrict__ H, const double* __restrict__ Jc,
                                 const double* __restrict__ Jo, const double* __restrict__ Kc,
                                 const double* __restrict__ Ko, long long nn, double* __restrict__ Fc,
                                 double* __restrict__ Fo)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double h = H[k] + Jc[k] + Jo[k] - 0.5 * Kc[k];
        Fc[k] = h - 0.5 * Ko[k];
        Fo[k] = 0.5 * (h - Ko[k]);
    }
}

struct RohfCoupling {
    double acc, bcc, aoo, boo, avv, bvv;
};

// unified Fock matrix in the MO basis from F_c^MO and F_o^MO, by the classes
// (closed, open, virtual) of the two orbitals; element (i, j) is read at
// (min, max) and mirrored (computeUnifiedFockMatrix_ROHF_kernel)
__global__ void rohf_unified_kernel(const double* __restrict__ Fc, const double* __restrict__ Fo, RohfCoupling p,
                                    int nc, int no, int n, double* __restrict__ R)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int r = static_cast<int>(k / n), c = static_cast<int>(k % n);
        const int i = min(r, c), j = max(r, c);
        const long long ij = static_cast<long long>(i) * n + j;
        const double fc = Fc[ij], fo = Fo[ij];
        const int ci = (i < nc) ? 0 : (i < nc + no ? 1 : 2);
        const int cj = (j < nc) ? 0 : (j < nc + no ? 1 : 2);
        double d;
        if (ci == 0 && cj == 0) d = 2.0 * (p.acc * fo + p.bcc * (fc - fo));
        else if (ci == 0 && cj == 1) d = 2.0 * (fc - fo);
        else if (ci == 0) d = fc;
        else if (ci == 1 && cj == 1) d = 2.0 * (p.aoo * fo + p.boo * (fc - fo));
        else if (ci == 1) d = 2.0 * fo;
        else d = 2.0 * (p.avv * fo + p.bvv * (fc - fo));
        R[k] = d;
    }
}

// ROHF energy 1/2 [<D_c, H + F_c> + <D_o, H> + 2 <D_o, F_o>]
__global__ void rohf_energy_kernel(const double* __restrict__ Dc, const double* __restrict__ Do,
                                   const double* __restrict__ H, const double* __restrict__ Fc,
                                   const double* __restrict__ Fo, long long nn, double* __restrict__ out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x)
        s += Dc[k] * (H[k] + Fc[k]) + Do[k] * (H[k] + 2.0 * Fo[k]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) *out = 0.5 * s;
    }
}

// ---- density by purification (eigensolver 2): no eigenvectors inside the SCF loop
// Gershgorin interval [lo, hi] of the symmetric F' (one block)
__global__ void gershgorin_kernel(const double* __restrict__ A, int n, double* __restrict__ out)
{
    __shared__ double rlo[32], rhi[32];
    double lo = 1e300, hi = -1e300;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r = 0.0;
        for (int j = 0; j < n; ++j)
            if (j != i) r += fabs(A[static_cast<long long>(i) * n + j]);
        const double d = A[static_cast<long long>(i) * n + i];
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
        out[0] = fmin(lo, rlo[0]);
        out[1] = fmax(hi, rhi[0]);
    }
}

// P0 = (hi I - F') / (hi - lo): eigenvalues in [0, 1], the lowest orbitals near 1
__global__ void sp2_init_kernel(const double* __restrict__ Fp, int n, const double* __restrict__ bounds,
                                float* __restrict__ P)
{
    const long long nn = static_cast<long long>(n) * n;
    const double lo = bounds[0], hi = bounds[1];
    const double inv = 1.0 / (hi - lo);
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const bool diag = (k / n) == (k % n);
        P[k] = static_cast<float>(((diag ? hi : 0.0) - Fp[k]) * inv);
    }
}

// One SP2 step (Niklasson): Pn = P^2 or 2P - P^2, whichever trace is closer to nocc.
// Every block reads both traces from the diagonals, so P, P2 and Pn are distinct buffers.
__global__ void sp2_step_kernel(const float* __restrict__ P, const float* __restrict__ P2, int n, int nocc,
                                float* __restrict__ Pn)
{
    __shared__ float r1[32], r2[32];
    __shared__ int take_square;
    float t1 = 0.f, t2 = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        t1 += P[static_cast<long long>(i) * n + i];
        t2 += P2[static_cast<long long>(i) * n + i];
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
        take_square = fabsf(b - nocc) < fabsf(2.f * a - b - nocc) ? 1 : 0;
    }
    __syncthreads();
    const long long nn = static_cast<long long>(n) * n;
    const bool sq = take_square != 0;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        Pn[k] = sq ? P2[k] : 2.f * P[k] - P2[k];
}

__global__ void scale_copy_kernel(const double* __restrict__ a, double f, long long nn, double* __restrict__ b)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        b[k] = f * a[k];
}

__global__ void widen_kernel(const float* __restrict__ a, long long nn, double* __restrict__ b)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        b[k] = static_cast<double>(a[k]);
}

// McWeeny step P = 3 P^2 - 2 P^3
__global__ void mcweeny_kernel(const double* __restrict__ P2, const double* __restrict__ P3, long long nn,
                               double* __restrict__ P)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        P[k] = 3.0 * P2[k] - 2.0 * P3[k];
}

int grid_nn(long long nn) { return static_cast<int>(std::min<long long>((nn + 255) / 256, 8192)); }

template <class T>
int alloc(T*& p, size_t n)
{
    if (p) return HF_OK;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return (e == cudaErrorMemoryAllocation) ? HF_ERR_OUT_OF_MEMORY : HF_ERR_CUDA;
    }
    return HF_OK;
}

int ensure_scf(Engine& e, int m)
{
    auto& w = e.scf;
    const int n = e.num_basis;
    const size_t nn = static_cast<size_t>(n) * n;
    if (w.n == n && w.m >= m) return HF_OK;
    if (w.m < m && w.Es) { cudaFree(w.Es); cudaFree(w.Fs); w.Es = w.Fs = nullptr; }
    int st;
    if ((st = alloc(w.S, nn)) || (st = alloc(w.H, nn)) || (st = alloc(w.X, nn)) || (st = alloc(w.F, nn)) ||
        (st = alloc(w.D, nn)) || (st = alloc(w.Dprev, nn)) || (st = alloc(w.G, nn)) || (st = alloc(w.dD, nn)) ||
        (st = alloc(w.C, nn)) || (st = alloc(w.W, nn)) || (st = alloc(w.eps, n)) || (st = alloc(w.T1, nn)) ||
        (st = alloc(w.T2, nn)) || (st = alloc(w.E, nn)) || (st = alloc(w.Es, nn * m)) || (st = alloc(w.Fs, nn * m)) ||
        (st = alloc(w.diis, kMaxDiis * kMaxDiis + kMaxDiis + 8)) || (st = alloc(w.info, 4)))
        return st;
    if (!w.work) {
        if (cusolverDnDsyevd_bufferSize(e.cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, w.W, n, w.eps,
                                        &w.lwork) != CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnDsyevd_bufferSize failed"), HF_ERR_SOLVER;
        if ((st = alloc(w.work, static_cast<size_t>(w.lwork)))) return st;
    }
    if (!w.syevj_params) {
        if (cusolverDnCreateSyevjInfo(&w.syevj_params) != CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnCreateSyevjInfo failed"), HF_ERR_SOLVER;
        cusolverDnXsyevjSetTolerance(w.syevj_params, 1e-15);
        cusolverDnXsyevjSetMaxSweeps(w.syevj_params, 100);
        if (cusolverDnDsyevj_bufferSize(e.cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, w.W, n, w.eps,
                                        &w.lwork_j, w.syevj_params) != CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnDsyevj_bufferSize failed"), HF_ERR_SOLVER;
        if ((st = alloc(w.work_j, static_cast<size_t>(w.lwork_j)))) return st;
    }
    w.n = n;
    w.m = m;
    return HF_OK;
}

// eigen-decomposition of the symmetric A (row-major) into W (column-major
// eigenvectors) and ascending eigenvalues; solver 0 = syevd, 1 = syevj
int syevd(Engine& e, const double* A, cudaStream_t s, int solver = 0)
{
    auto& w = e.scf;
    const size_t nn = static_cast<size_t>(w.n) * w.n;
    GB_CUDA_TRY(cudaMemcpyAsync(w.W, A, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (solver == 1) {
        if (cusolverDnDsyevj(e.cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, w.n, w.W, w.n, w.eps,
                             w.work_j, w.lwork_j, w.info, w.syevj_params) != CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnDsyevj failed"), HF_ERR_SOLVER;
        return HF_OK;
    }
    if (cusolverDnDsyevd(e.cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, w.n, w.W, w.n, w.eps, w.work,
                         w.lwork, w.info) != CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDsyevd failed"), HF_ERR_SOLVER;
    return HF_OK;
}

__global__ void identity_kernel(int n, double* __restrict__ X)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        X[k] = (k / n == k % n) ? 1.0 : 0.0;
}

// B = A - c I (n x n)
__global__ void shift_diagonal_kernel(const double* __restrict__ A, int n, double c, double* __restrict__ B)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        B[k] = A[k] - ((k / n == k % n) ? c : 0.0);
}

// The reference's X = U s^{-1/2} drops the eigenvectors of S with s < 1e-6.  When S - 1e-6 I
// is positive definite no eigenvalue is dropped, and then any X with X^T S X = I spanning the
// whole space gives the same densities, orbitals (up to sign) and orbital energies; the
// purified loop never needs the eigenvectors of S, so X = L^{-T} from S = L L^T (two potrf and
// one trsm instead of an eigendecomposition).  *used = false: S fails the test (or the
// workspace is too small) and the caller builds the canonical X.
int cholesky_orthogonalizer(Engine& e, const double* S, cudaStream_t s, bool* used)
{
    auto& w = e.scf;
    *used = false;
    const int n = w.n;
    const long long nn = static_cast<long long>(n) * n;
    int lwork = 0;
    if (cusolverDnDpotrf_bufferSize(e.cusolver, CUBLAS_FILL_MODE_LOWER, n, w.T1, n, &lwork) !=
            CUSOLVER_STATUS_SUCCESS ||
        lwork > w.lwork)
        return HF_OK;
    shift_diagonal_kernel<<<grid_nn(nn), 256, 0, s>>>(S, n, kOrthoCut, w.T1);
    GB_LAUNCH_CHECK();
    if (cusolverDnDpotrf(e.cusolver, CUBLAS_FILL_MODE_LOWER, n, w.T1, n, w.work, w.lwork, w.info) !=
        CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDpotrf failed"), HF_ERR_SOLVER;
    int info = -1;
    GB_CUDA_TRY(cudaMemcpyAsync(&info, w.info, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (info != 0) return HF_OK;  // an eigenvalue at or below the cut: canonical orthogonalization
    // S is symmetric, so its row-major array is also its column-major one; the column-major
    // factor L gives the column-major L^{-1}, i.e. the row-major L^{-T} = X
    GB_CUDA_TRY(cudaMemcpyAsync(w.T1, S, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (cusolverDnDpotrf(e.cusolver, CUBLAS_FILL_MODE_LOWER, n, w.T1, n, w.work, w.lwork, w.info) !=
        CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDpotrf failed"), HF_ERR_SOLVER;
    identity_kernel<<<grid_nn(nn), 256, 0, s>>>(n, w.X);
    GB_LAUNCH_CHECK();
    const double one = 1.0;
    if (cublasDtrsm(e.cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one,
                    w.T1, n, w.X, n) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDtrsm failed"), HF_ERR_SOLVER;
    *used = true;
    return HF_OK;
}

int coefficients(Engine& e, const double* F, cudaStream_t s, int solver = 0)
{
    auto& w = e.scf;
    int st;
    if ((st = gemm_rm(e.cublas, true, false, w.n, w.X, F, w.T1))) return st;   // X^T F
    if ((st = gemm_rm(e.cublas, false, false, w.n, w.T1, w.X, w.T2))) return st;  // X^T F X
    if ((st = syevd(e, w.T2, s, solver))) return st;
    return gemm_rm(e.cublas, false, true, w.n, w.X, w.W, w.C);  // C = X C'
}

// D = 2 X P X^T with P the projector on the nocc lowest states of F' = X^T F X, by
// purification: FP32 SP2 steps (cuBLAS SGEMM) from the Gershgorin-scaled F', then FP64
// McWeeny steps to FP64 idempotency.  Equals the aufbau density of a diagonalisation
// whenever the HOMO-LUMO gap is open.
constexpr int kSp2Steps = 50;
constexpr int kMcWeenySteps = 3;

// status words of the library-call purification: tr(P) - nocc and |tr(P) - |P|_F^2|
// of the FP64 projector (one block)
__global__ void purify_check_kernel(const double* __restrict__ P, int n, int nocc, int sp2_steps,
                                    double* __restrict__ status)
{
    __shared__ double rt[32], rf[32];
    double t = 0.0, f = 0.0;
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) {
        const double v = P[k];
        f += v * v;
        if (k / n == k % n) t += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        t += __shfl_xor_sync(0xffffffffu, t, o);
        f += __shfl_xor_sync(0xffffffffu, f, o);
    }
    if ((threadIdx.x & 31) == 0) { rt[threadIdx.x >> 5] = t; rf[threadIdx.x >> 5] = f; }
    __syncthreads();
    if (threadIdx.x == 0) {
        t = 0.0;
        f = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) { t += rt[w]; f += rf[w]; }
        status[kPurifyStatusSteps] = sp2_steps;
        status[kPurifyStatusTraceError] = t - nocc;
        status[kPurifyStatusIdempotency] = fabs(t - f);
        status[kPurifyStatusSp2Error] = 0.0;
        status[kPurifyStatusSp2Converged] = 1.0;
        status[kPurifyStatusMcWeeny] = kMcWeenySteps;
        status[kPurifyStatusFlags] = 0.0;
    }
}

// N <= 512: the fused single-launch purification (purify.cu); larger N: SP2 steps
// as cuBLAS SGEMMs, then McWeeny as DGEMMs.  Both leave their status words.
int purify_density(Engine& e, const double* F, int nocc, double* D, cudaStream_t s, int max_steps)
{
    if (purify_fused_supported(e)) return purify_fused(e, F, nocc, D, s, max_steps);
    const int sp2_steps = max_steps > 0 ? max_steps : kSp2Steps;
    auto& w = e.scf;
    const int n = w.n;
    const long long nn = static_cast<long long>(n) * n;
    int st;
    double* status = nullptr;
    if ((st = purify_status(e, &status))) return st;
    if (!w.P32a) {
        if ((st = alloc(w.P32a, nn)) || (st = alloc(w.P32b, nn)) || (st = alloc(w.P32c, nn))) return st;
    }
    if ((st = gemm_rm(e.cublas, true, false, n, w.X, F, w.T1))) return st;    // X^T F
    if ((st = gemm_rm(e.cublas, false, false, n, w.T1, w.X, w.T2))) return st; // F'
    gershgorin_kernel<<<1, 1024, 0, s>>>(w.T2, n, e.d_scalar + 8);
    GB_LAUNCH_CHECK();
    sp2_init_kernel<<<grid_nn(nn), 256, 0, s>>>(w.T2, n, e.d_scalar + 8, w.P32a);
    GB_LAUNCH_CHECK();
    float* P = w.P32a;
    float* Pn = w.P32b;
    float* P2 = w.P32c;
    const float one = 1.f, zero = 0.f;
    for (int k = 0; k < sp2_steps; ++k) {
        // P symmetric: the column-major product is P^2 as well
        if (cublasSgemm(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, P, n, P, n, &zero, P2, n) !=
            CUBLAS_STATUS_SUCCESS)
            return set_error("cublasSgemm (purification) failed"), HF_ERR_SOLVER;
        sp2_step_kernel<<<grid_nn(nn), 256, 0, s>>>(P, P2, n, nocc, Pn);
        GB_LAUNCH_CHECK();
        std::swap(P, Pn);
    }
    widen_kernel<<<grid_nn(nn), 256, 0, s>>>(P, nn, w.W);
    GB_LAUNCH_CHECK();
    for (int k = 0; k < kMcWeenySteps; ++k) {
        if ((st = gemm_rm(e.cublas, false, false, n, w.W, w.W, w.T1))) return st;  // P^2
        if ((st = gemm_rm(e.cublas, false, false, n, w.T1, w.W, w.T2))) return st; // P^3
        mcweeny_kernel<<<grid_nn(nn), 256, 0, s>>>(w.T1, w.T2, nn, w.W);
        GB_LAUNCH_CHECK();
    }
    purify_check_kernel<<<1, 1024, 0, s>>>(w.W, n, nocc, sp2_steps, status);
    GB_LAUNCH_CHECK();
    if ((st = gemm_rm(e.cublas, false, false, n, w.X, w.W, w.T1))) return st;  // X P
    if ((st = gemm_rm(e.cublas, false, true, n, w.T1, w.X, w.T2))) return st;  // X P X^T
    scale_copy_kernel<<<grid_nn(nn), 256, 0, s>>>(w.T2, 2.0, nn, D);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// purify_density under the engine's graph schedule (single-molecule engines): the
// first call with a given (F, D, nocc) runs as ordinary launches (it also makes the
// lazy allocations), the second is captured on the schedule's capture stream and
// every call from then on replays the graph on s.  cuBLAS runs on the capture
// stream with an engine-owned workspace during the capture (cublasSetStream resets
// cuBLAS to its own workspace pool, which may allocate, and a capture must not).
// If the capture fails, that purification keeps running as ordinary launches.
int purify_density_scheduled(Engine& e, const double* F, int nocc, double* D, cudaStream_t s, int max_steps)
{
    FockSchedule& S = e.sched;
    // the fused path is one launch already: nothing to replay
    if (!S.use_graph || e.nmol != 1 || purify_fused_supported(e)) return purify_density(e, F, nocc, D, s, max_steps);
    FockSchedule::PurifyGraph* g = nullptr;
    for (auto& x : S.purify)
        if (x.F == F && x.D == D && x.nocc == nocc && x.max_steps == max_steps) {
            g = &x;
            break;
        }
    if (!g) {
        if (static_cast<int>(S.purify.size()) >= kMaxFockGraphs) {
            if (S.purify.front().exec) cudaGraphExecDestroy(S.purify.front().exec);
            S.purify.erase(S.purify.begin());
        }
        S.purify.push_back(FockSchedule::PurifyGraph{F, D, nocc, max_steps, 0, false, nullptr, 0});
        g = &S.purify.back();
    }
    if (g->failed || (!g->exec && g->uses++ == 0)) return purify_density(e, F, nocc, D, s, max_steps);
    if (!g->exec) {
        int st = schedule_streams(e);
        if (st) return st;
        if (!S.cublas_ws) GB_CUDA_TRY(cudaMalloc(&S.cublas_ws, kCublasCaptureWorkspace));
        if (cublasSetStream(e.cublas, S.capture) != CUBLAS_STATUS_SUCCESS ||
            cublasSetWorkspace(e.cublas, S.cublas_ws, kCublasCaptureWorkspace) != CUBLAS_STATUS_SUCCESS) {
            cublasSetStream(e.cublas, s);
            g->failed = true;
            return purify_density(e, F, nocc, D, s, max_steps);
        }
        const long long l0 = launch_count();
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamBeginCapture(S.capture, cudaStreamCaptureModeThreadLocal);
        if (ce == cudaSuccess) {
            st = purify_density(e, F, nocc, D, S.capture, max_steps);
            ce = cudaStreamEndCapture(S.capture, &graph);
        }
        cublasSetStream(e.cublas, s);
        const long long recorded = launch_count() - l0;
        count_launches(-recorded);  // recorded, not launched
        cudaGraphExec_t exec = nullptr;
        if (!st && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
            g->exec = exec;
            g->launches = recorded;
        }
        if (graph) cudaGraphDestroy(graph);
        if (!g->exec) {
            cudaGetLastError();  // capture errors are not sticky; clear the last-error slot
            g->failed = true;
            clear_error();
            return purify_density(e, F, nocc, D, s, max_steps);
        }
    }
    GB_CUDA_TRY(cudaGraphLaunch(g->exec, s));
    count_launches(g->launches);
    ++S.graph_replays;
    return HF_OK;
}

// Occupied orbitals without an eigensolver, for the RI K build under purification:
// after purify_density, w.W holds the projector P on the occupied space in the
// orthonormal basis.  Q = orth(P Q_prev) by CholeskyQR2 (M = Y^T Y = U^T U, Y U^{-1},
// twice) spans the same space as P whenever P Q_prev has full rank (the previous
// iteration's occupied basis is close to the new one); C_occ = X Q.  K depends on
// the occupied space only, so any orthonormal basis of it gives the same K.
// first = true (or a failed Cholesky): the orbitals of one diagonalisation seed Q.
int occupied_from_projector(Engine& e, const double* F, int nocc, bool first, cudaStream_t s)
{
    auto& w = e.scf;
    const int n = w.n;
    int st;
    if (!w.Qocc) {
        if ((st = alloc(w.Qocc, static_cast<size_t>(n) * n)) || (st = alloc(w.Mocc, static_cast<size_t>(n) * n)) ||
            (st = alloc(w.qinfo, 1)))
            return st;
        if (cusolverDnDpotrf_bufferSize(e.cusolver, CUBLAS_FILL_MODE_UPPER, n, w.Mocc, n, &w.qlwork) !=
            CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnDpotrf_bufferSize failed"), HF_ERR_SOLVER;
        if ((st = alloc(w.qwork, static_cast<size_t>(std::max(w.qlwork, 1))))) return st;
    }
    const double one = 1.0, zero = 0.0;
    // seed: the eigenvectors of F' (C' = the column-major W^T), Q = first nocc columns
    auto seed = [&]() -> int {
        int r;
        if ((r = coefficients(e, F, s, 0))) return r;
        // row-major Q (n x nocc) = C'[:, :nocc]; column-major W holds eigenvector k in column k
        if (cublasDgeam(e.cublas, CUBLAS_OP_T, CUBLAS_OP_N, nocc, n, &one, w.W, n, &zero, w.Qocc, nocc, w.Qocc,
                        nocc) != CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDgeam (occupied seed) failed"), HF_ERR_SOLVER;
        return HF_OK;
    };
    if (first) return seed();
    // Y = P Q_prev (row-major n x nocc) into T2, then two Cholesky-QR passes in place
    if (cublasDgemm(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, nocc, n, n, &one, w.Qocc, nocc, w.W, n, &zero, w.T2, nocc) !=
        CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDgemm (P Q) failed"), HF_ERR_SOLVER;
    for (int pass = 0; pass < 2; ++pass) {
        // M = Y^T Y (nocc x nocc); column-major view of Y is Y^T (nocc x n, ld nocc)
        if (cublasDgemm(e.cublas, CUBLAS_OP_N, CUBLAS_OP_T, nocc, nocc, n, &one, w.T2, nocc, w.T2, nocc, &zero, w.Mocc,
                        nocc) != CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDgemm (Y^T Y) failed"), HF_ERR_SOLVER;
        if (cusolverDnDpotrf(e.cusolver, CUBLAS_FILL_MODE_UPPER, nocc, w.Mocc, nocc, w.qwork, w.qlwork, w.qinfo) !=
            CUSOLVER_STATUS_SUCCESS)
            return set_error("cusolverDnDpotrf (occupied basis) failed"), HF_ERR_SOLVER;
        // Y^T <- U^{-T} Y^T, i.e. Y <- Y U^{-1}
        if (cublasDtrsm(e.cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, nocc, n,
                        &one, w.Mocc, nocc, w.T2, nocc) != CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDtrsm (occupied basis) failed"), HF_ERR_SOLVER;
    }
    int info = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&info, w.qinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (info != 0) return seed();  // P Q_prev lost rank: reseed from a diagonalisation
    GB_CUDA_TRY(cudaMemcpyAsync(w.Qocc, w.T2, sizeof(double) * n * nocc, cudaMemcpyDeviceToDevice, s));
    // C[:, :nocc] = X Q (row-major, ld n)
    if (cublasDgemm(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, nocc, n, n, &one, w.Qocc, nocc, w.X, n, &zero, w.C, n) !=
        CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDgemm (X Q) failed"), HF_ERR_SOLVER;
    return HF_OK;
}

// e = FDS - SDF; transform 1: X e X^T (diis_include_transform, computeDIISErrorMatrix,
// src/gpu_manager.cu:1020-1068); transform 2: X^T e X, the error in the orthonormal
// basis of a caller's orthogonaliser (its span is a subspace: the AO-basis error
// has a component outside it that does not vanish at convergence)
int diis_error(Engine& e, const double* S, const double* X, const double* F, const double* D, double* E,
               int transform, cudaStream_t s, bool symmetric = true)
{
    auto& w = e.scf;
    const long long nn = static_cast<long long>(w.n) * w.n;
    int st;
    if ((st = gemm_rm(e.cublas, false, false, w.n, F, D, w.T1))) return st;
    if ((st = gemm_rm(e.cublas, false, false, w.n, w.T1, S, w.T2))) return st;  // FDS
    if (symmetric) {
        // the SCF's F, D, S are symmetric: SDF = (FDS)^T, so e = FDS - (FDS)^T
        antisym_kernel<<<grid_nn(nn), 256, 0, s>>>(w.T2, w.n, E);
        GB_LAUNCH_CHECK();
    } else {
        if ((st = gemm_rm(e.cublas, false, false, w.n, S, D, w.T1))) return st;
        if ((st = gemm_rm(e.cublas, false, false, w.n, w.T1, F, E))) return st;  // SDF
        sub_kernel<<<grid_nn(nn), 256, 0, s>>>(w.T2, E, nn, E);
        GB_LAUNCH_CHECK();
    }
    if (transform == 1) {
        if ((st = gemm_rm(e.cublas, false, false, w.n, X, E, w.T1))) return st;
        if ((st = gemm_rm(e.cublas, false, true, w.n, w.T1, X, E))) return st;
    } else if (transform == 2) {
        if ((st = gemm_rm(e.cublas, true, false, w.n, X, E, w.T1))) return st;
        if ((st = gemm_rm(e.cublas, false, false, w.n, w.T1, X, E))) return st;
    }
    return HF_OK;
}

int diis_extrapolate(Engine& e, const double* Es, const double* Fs, int m, double* Fout, cudaStream_t s)
{
    auto& w = e.scf;
    const long long nn = static_cast<long long>(w.n) * w.n;
    double* B = w.diis;
    double* coef = w.diis + kMaxDiis * kMaxDiis;
    diis_dots_kernel<<<m * (m + 1) / 2, 512, 0, s>>>(Es, m, nn, B);
    GB_LAUNCH_CHECK();
    diis_solve_kernel<<<1, 32, 0, s>>>(B, m, coef, w.info + 1);
    GB_LAUNCH_CHECK();
    diis_combine_kernel<<<grid_nn(nn), 256, 0, s>>>(Fs, coef, m, nn, Fout);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

double nuclear_repulsion(const Engine& e)
{
    double v = 0.0;
    for (size_t i = 0; i + 1 < e.atoms.size(); ++i)
        for (size_t j = i + 1; j < e.atoms.size(); ++j) {
            const double dx = e.atoms[i].x - e.atoms[j].x, dy = e.atoms[i].y - e.atoms[j].y,
                         dz = e.atoms[i].z - e.atoms[j].z;
            v += e.atoms[i].atomic_number * e.atoms[j].atomic_number / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    return v;
}

// J(D) and K(D) of one density (standard definitions, N x N each) through the
// direct kernels or, with use_ri, the RI tensor (J from B, K from the density)
int jk_of(Engine& e, bool use_ri, const double* D, double* J, double* K, int precision, double mixed_thr,
          cudaStream_t s)
{
    if (!use_ri) return build_jk(e, D, J, K, precision, mixed_thr, s);
    int r;
    if ((r = ri_j(e, D, J, s))) return r;
    return ri_k_density(e, D, K, s);
}

bool valid_guess(int g) { return g == HF_GUESS_CORE || g == HF_GUESS_GWH || g == HF_GUESS_DENSITY || g == HF_GUESS_SAD; }

// X = U s^{-1/2} from the eigen-decomposition of S already in w.W / w.eps
// (HF::compute_transform_matrix, src/hf.cu:171-243), or the caller's
// orthogonaliser (options.orthogonalizer: a subspace of the AO space, e.g. the
// spherical-harmonic functions; its DIIS error is taken in the orthogonal basis)
// Convergence_*_Damping (include/rhf.hpp:182-262): the first call keeps F and D, later
// calls damp F (and D, with the optimal factor) against the kept ones
struct Damper {
    double* Fp = nullptr;
    double* Dp = nullptr;
    bool first = true;
    ~Damper()
    {
        if (Fp) cudaFree(Fp);
        if (Dp) cudaFree(Dp);
    }
    int step(Engine& e, const hf_scf_options& opt, double* F, double* D, long long nn, cudaStream_t s)
    {
        if (!Fp && (cudaMalloc(&Fp, nn * sizeof(double)) != cudaSuccess ||
                    cudaMalloc(&Dp, nn * sizeof(double)) != cudaSuccess))
            return set_error("cudaMalloc (damping) failed"), HF_ERR_OUT_OF_MEMORY;
        if (first) {
            first = false;
            GB_CUDA_TRY(cudaMemcpyAsync(Fp, F, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(Dp, D, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
            return HF_OK;
        }
        double a = opt.damping_factor;
        const bool optimal = opt.convergence_method == HF_CONV_OPTIMAL_DAMPING;
        if (optimal) {
            damping_traces_kernel<<<1, 1024, 0, s>>>(F, Fp, D, Dp, nn, e.d_scalar + 10);
            GB_LAUNCH_CHECK();
            double sc[2];
            GB_CUDA_TRY(cudaMemcpyAsync(sc, e.d_scalar + 10, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
            GB_CUDA_TRY(cudaStreamSynchronize(s));
            a = (sc[1] <= -sc[0] / 2.0) ? 1.0 : -0.5 * sc[0] / sc[1];
        }
        damp_kernel<<<grid_nn(nn), 256, 0, s>>>(Fp, F, a, nn);
        GB_LAUNCH_CHECK();
        if (optimal) {
            damp_kernel<<<grid_nn(nn), 256, 0, s>>>(Dp, D, a, nn);
            GB_LAUNCH_CHECK();
        }
        return HF_OK;
    }
};

bool valid_convergence(const hf_scf_options& opt)
{
    return opt.convergence_method == HF_CONV_DIIS || opt.convergence_method == HF_CONV_DAMPING ||
           opt.convergence_method == HF_CONV_OPTIMAL_DAMPING;
}

int diis_x(const hf_scf_options& opt) { return opt.orthogonalizer ? 2 : (opt.diis_include_transform != 0 ? 1 : 0); }

int orthogonalizer(Engine& e, const hf_scf_options& opt, cudaStream_t s)
{
    auto& w = e.scf;
    const long long nn = static_cast<long long>(w.n) * w.n;
    if (opt.orthogonalizer) {
        GB_CUDA_TRY(cudaMemcpyAsync(w.X, opt.orthogonalizer, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        return HF_OK;
    }
    transform_kernel<<<grid_nn(nn), 256, 0, s>>>(w.W, w.eps, w.n, w.X);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

}  // namespace

}  // namespace gb

using namespace gb;

extern "C" {

void hf_scf_options_default(hf_scf_options* o)
{
    if (!o) return;
    o->max_iter = 100;
    o->convergence_threshold = 1e-6;
    o->diis_size = 8;
    o->diis_include_transform = 0;
    o->precision = HF_PRECISION_FP64;
    o->mixed_threshold = 1e-7;
    o->incremental = 0;
    o->rebuild_every = 0;
    o->full_build_precision = HF_PRECISION_FP64;
    o->eri_method = HF_ERI_DIRECT;
    o->anchor_threshold = 0.0;
    o->initial_guess = HF_GUESS_CORE;
    o->guess_density_a = nullptr;
    o->guess_density_b = nullptr;
    o->orthogonalizer = nullptr;
    o->convergence_method = HF_CONV_DIIS;
    o->damping_factor = 0.9;
    o->purification_max_steps = 0;
    o->anchor_mixed_threshold = 0.0;
    o->incremental_drop = 0.0;
    o->pre_anchor_drop = 0.0;
    o->eigensolver = 0;
    o->verbose = 0;
}

int hf_compute_diis_error(hf_engine* eng, const double* d_overlap, const double* d_transform, const double* d_fock,
                          const double* d_density, double* d_error, int include_transform, void* stream)
{
    clear_error();
    if (!eng || !d_overlap || !d_fock || !d_density || !d_error || (include_transform && !d_transform))
        return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    int st = ensure_scf(e, std::max(e.scf.m, 2));
    if (st) return st;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    cublasSetStream(e.cublas, s);
    return diis_error(e, d_overlap, d_transform, d_fock, d_density, d_error, include_transform != 0 ? 1 : 0, s, false);
}

int hf_compute_fock_diis(hf_engine* eng, const double* d_errors, const double* d_focks, double* d_new_fock,
                         int num_prev, void* stream)
{
    clear_error();
    if (!eng || !d_errors || !d_focks || !d_new_fock) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    if (num_prev < 2 || num_prev > kMaxDiis)
        return set_error("DIIS requires between 2 and 16 previous Fock matrices"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    int st = ensure_scf(e, std::max(e.scf.m, 2));
    if (st) return st;
    return diis_extrapolate(e, d_errors, d_focks, num_prev, d_new_fock, static_cast<cudaStream_t>(stream));
}

int hf_engine_purification_status(hf_engine* eng, double* h_out, int max_words)
{
    clear_error();
    if (!eng || !h_out || max_words <= 0) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    for (int i = 0; i < max_words; ++i) h_out[i] = 0.0;
    if (!e.scf.pur) return HF_OK;
    GB_CUDA_TRY(cudaMemcpy(h_out, e.scf.pur, sizeof(double) * std::min(max_words, kPurifyStatusWords),
                           cudaMemcpyDeviceToHost));
    return HF_OK;
}

int hf_combine_uhf_fock(const double* d_core_hamiltonian, const double* d_j_a, const double* d_j_b,
                        const double* d_k_a, const double* d_k_b, double* d_fock_a, double* d_fock_b, int num_basis,
                        void* stream)
{
    clear_error();
    if (!d_core_hamiltonian || !d_j_a || !d_j_b || !d_k_a || !d_k_b || !d_fock_a || !d_fock_b || num_basis <= 0)
        return set_error("hf_combine_uhf_fock: null pointer or non-positive num_basis"), HF_ERR_INVALID_ARGUMENT;
    const long long nn = static_cast<long long>(num_basis) * num_basis;
    uhf_combine_kernel<<<grid_nn(nn), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        d_core_hamiltonian, d_j_a, d_j_b, d_k_a, d_k_b, nn, d_fock_a, d_fock_b);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// internal status of rhf_scf_run: a purified density failed its checks (the SCF
// is rerun with a diagonalisation)
constexpr int kPurificationRejected = -100;

static int rhf_scf_run(hf_engine* eng, int num_electrons, const hf_scf_options* opt_in, hf_scf_result* res,
                       double* d_density_out, double* d_fock_out, double* d_orbital_energies_out,
                       double* d_coefficients_out)
{
    clear_error();
    if (!eng || !res) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (e.nmol != 1) return set_error("hf_rhf_scf: a batch engine runs hf_batch_rhf_scf"), HF_ERR_INVALID_ARGUMENT;
    hf_scf_options opt;
    if (opt_in) opt = *opt_in; else hf_scf_options_default(&opt);
    if (num_electrons <= 0 || (num_electrons & 1))
        return set_error("RHF needs an even, positive number of electrons"), HF_ERR_INVALID_ARGUMENT;
    const int nocc = num_electrons / 2;
    const int n = e.num_basis;
    if (nocc > n) return set_error("more occupied orbitals than basis functions"), HF_ERR_INVALID_ARGUMENT;
    if (opt.diis_size < 1 || opt.diis_size > kMaxDiis)
        return set_error("diis_size must be in [1, 16]"), HF_ERR_INVALID_ARGUMENT;
    if (opt.precision != HF_PRECISION_FP64 && opt.precision != HF_PRECISION_MIXED)
        return set_error("unknown precision"), HF_ERR_INVALID_ARGUMENT;
    if (opt.eri_method != HF_ERI_DIRECT && opt.eri_method != HF_ERI_RI && opt.eri_method != HF_ERI_STORED)
        return set_error("unknown eri_method"), HF_ERR_INVALID_ARGUMENT;
    if (opt.eri_method == HF_ERI_STORED && opt.precision != HF_PRECISION_FP64)
        return set_error("eri_method stored is FP64 (the mixed tier belongs to the direct and RI builds)"),
               HF_ERR_INVALID_ARGUMENT;
    if (!valid_guess(opt.initial_guess))
        return set_error("initial_guess: core, GWH, density or SAD"), HF_ERR_INVALID_ARGUMENT;
    const bool density_guess = opt.initial_guess == HF_GUESS_DENSITY || opt.initial_guess == HF_GUESS_SAD;
    if (density_guess && !opt.guess_density_a)
        return set_error("initial_guess density/SAD needs guess_density_a"), HF_ERR_INVALID_ARGUMENT;
    if (!valid_convergence(opt)) return set_error("convergence_method: DIIS, damping or optimal damping"),
                                 HF_ERR_INVALID_ARGUMENT;
    Damper damper;
    const bool use_ri = opt.eri_method == HF_ERI_RI;
    const bool use_stored = opt.eri_method == HF_ERI_STORED;
    if (use_ri && !e.ri)
        return set_error("eri_method RI needs an auxiliary basis (hf_engine_set_auxiliary_basis)"),
               HF_ERR_INVALID_ARGUMENT;
    const int m = opt.diis_size;
    int st = ensure_scf(e, m);
    if (st) return st;
    auto& w = e.scf;
    const long long nn = static_cast<long long>(n) * n;
    cudaStream_t s = nullptr;
    cublasSetStream(e.cublas, s);
    cusolverDnSetStream(e.cusolver, s);
    *res = hf_scf_result{};
    res->nuclear_repulsion = nuclear_repulsion(e);
    GB_CUDA_TRY(cudaMemsetAsync(e.d_counters, 0, kCounterSlots * sizeof(unsigned long long), s));
    GB_CUDA_TRY(cudaMemsetAsync(w.info, 0, 4 * sizeof(int), s));

    LoopResources lr;
    cudaEvent_t f0 = lr.ev[0], f1 = lr.ev[1], c0 = lr.ev[2], c1 = lr.ev[3], q0 = lr.ev[4], q1 = lr.ev[5];
    double fock_ms = 0.0, diag_ms = 0.0, diis_ms = 0.0;
    bool diis_timed = false;
    int fock_builds = 0;
    double* h_energy = lr.h_energy;

    // Mixed tier with anchor_threshold > 0: full low-precision builds (direct: every
    // quartet FP32; RI: split-BF16 K) while max|dD| >= anchor_threshold, then one FP64
    // build (the anchor), then incremental builds.  With anchor_threshold <= 0 the
    // first build is the anchor.  The SCF may not converge before the anchor.
    const bool mixed_tier = opt.precision == HF_PRECISION_MIXED;
    bool anchored = !(mixed_tier && opt.anchor_threshold > 0.0);
    bool ri_anchored = false;  // mixed RI: an FP64 K build has been taken
    // one Fock build: F = H + G(D), full or incremental
    auto fock_build = [&](bool first) -> int {
        cudaEventRecord(f0, s);
        if (use_stored) {
            // ERI_Stored_RHF::compute_fock_matrix (src/eri.cu): F from the stored tensor
            int r = stored_fock(w.D, w.H, e.d_eri, w.F, n, s);
            if (r) return r;
            cudaEventRecord(f1, s);
            ++fock_builds;
            return HF_OK;
        }
        if (use_ri) {
            // J (FP64) from the packed B and D.  K: FP64 from the occupied orbitals
            // (D = 2 C_occ C_occ^T); under the mixed tier, split-BF16 tensor-core builds
            // until max|dD| < anchor_threshold, then one FP64 anchor build, then
            // incremental K(dD) from rotation-aligned orbital differences.
            double *J, *K;
            int r;
            if ((r = ri_work_buffers(e, &J, &K))) return r;
            if ((r = ri_j(e, w.D, J, s))) return r;
            if (opt.precision == HF_PRECISION_FP64) {
                if ((r = ri_k_occupied(e, w.C, nocc, K, s))) return r;
                if ((r = ri_fock_from_jk(e, w.H, J, K, nullptr, false, w.F, s))) return r;
            } else {
                double dmax = 1.0;
                if (!first && (r = ri_absmax_diff(e, w.D, w.Dprev, &dmax, s))) return r;
                double* Kacc = nullptr;
                if ((r = ri_prepare_planes(e, nocc, s))) return r;
                Kacc = e.ri->d_Kacc;
                bool done = false;
                if (ri_anchored) {
                    bool aligned = false;
                    if ((r = ri_k_tc_delta(e, w.C, n, nocc, w.S, K, &aligned, s))) return r;
                    if (aligned) {
                        if ((r = ri_add_inplace(e, Kacc, K, s))) return r;
                        done = true;
                    }
                } else if (!anchored && (first || dmax >= opt.anchor_threshold)) {
                    if ((r = ri_k_tc_full(e, w.C, n, nocc, Kacc, s))) return r;
                    done = true;
                }
                if (!done) {  // FP64 anchor build
                    if ((r = ri_k_occupied(e, w.C, nocc, Kacc, s))) return r;
                    ri_anchored = true;
                    anchored = true;
                }
                if ((r = ri_save_occupied(e, w.C, n, nocc, s))) return r;
                if ((r = ri_fock_from_jk(e, w.H, J, Kacc, nullptr, false, w.F, s))) return r;
                GB_CUDA_TRY(cudaMemcpyAsync(w.Dprev, w.D, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
            }
            cudaEventRecord(f1, s);
            ++fock_builds;
            return HF_OK;
        }
        int r;
        if (!anchored) {
            // before the anchor: full builds with every quartet in the FP32 tier, or the
            // FP64 anchor build once max|dD| falls below anchor_threshold
            double dmax = 1.0;
            if (!first && (r = ri_absmax_diff(e, w.D, w.Dprev, &dmax, s))) return r;
            const bool low = first || dmax >= opt.anchor_threshold;
            // the pre-anchor builds only steer the density towards the anchor: quartets whose
            // bound is below pre_anchor_drop (kPreAnchorDrop by default) are left out of them
            // (the anchor builds every quartet the Schwarz screen keeps: in FP64, or with
            // anchor_mixed_threshold > 0 the quartets with Q_ab Q_cd max|D| below it in FP32)
            const bool mixed_anchor = opt.anchor_mixed_threshold > 0.0;
            const double pre_drop = opt.pre_anchor_drop > 0.0 ? opt.pre_anchor_drop : kPreAnchorDrop;
            if ((r = build_jk(e, w.D, nullptr, nullptr,
                              (low || mixed_anchor) ? HF_PRECISION_MIXED : HF_PRECISION_FP64,
                              low ? std::numeric_limits<double>::infinity() : opt.anchor_mixed_threshold, s,
                              low ? pre_drop : -1.0)))
                return r;
            if (!low) anchored = true;
            fock_from_jk_kernel<<<grid_nn(nn), 256, 0, s>>>(e.d_Jp, e.d_Kp, e.last_mixed ? e.d_Jp32 : nullptr,
                                                             e.last_mixed ? e.d_Kp32 : nullptr, e.d_scale, w.H, n, 0,
                                                             w.G, w.F);
            GB_LAUNCH_CHECK();
            GB_CUDA_TRY(cudaMemcpyAsync(w.Dprev, w.D, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
            cudaEventRecord(f1, s);
            ++fock_builds;
            return HF_OK;
        }
        const bool incremental = opt.incremental && !first &&
                                 !(opt.rebuild_every > 0 && fock_builds % opt.rebuild_every == 0);
        if (incremental) {
            sub_kernel<<<grid_nn(nn), 256, 0, s>>>(w.D, w.Dprev, nn, w.dD);
            GB_LAUNCH_CHECK();
            // the contributions left out change from one build to the next, so the drop is
            // capped by the convergence threshold (each left-out term stays 30x below it)
            const double drop = opt.incremental_drop > 0.0
                                    ? std::min(opt.incremental_drop, 0.03 * opt.convergence_threshold)
                                    : -1.0;
            if ((r = build_jk(e, w.dD, nullptr, nullptr, opt.precision, opt.mixed_threshold, s, drop))) return r;
        } else {
            const int prec = (opt.precision == HF_PRECISION_MIXED) ? opt.full_build_precision : opt.precision;
            if ((r = build_jk(e, w.D, nullptr, nullptr, prec, opt.mixed_threshold, s))) return r;
        }
        fock_from_jk_kernel<<<grid_nn(nn), 256, 0, s>>>(e.d_Jp, e.d_Kp, e.last_mixed ? e.d_Jp32 : nullptr,
                                                         e.last_mixed ? e.d_Kp32 : nullptr, e.d_scale, w.H, n,
                                                         incremental ? 1 : 0, w.G, w.F);
        GB_LAUNCH_CHECK();
        GB_CUDA_TRY(cudaMemcpyAsync(w.Dprev, w.D, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        cudaEventRecord(f1, s);
        ++fock_builds;
        return HF_OK;
    };
    auto elapsed = [&](cudaEvent_t a, cudaEvent_t b) {
        float ms = 0.f;
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        return static_cast<double>(ms);
    };

    const auto t_setup = std::chrono::steady_clock::now();
    // core Hamiltonian, X, core guess (and the RI B tensor)
    if (use_ri && (st = ri_require_b(e, s))) return st;
    if (use_stored && !e.d_eri) {
        // the tensor stays with the engine (ERI_Stored_RHF::precomputation, src/eri.cu)
        const size_t bytes = static_cast<size_t>(nn) * static_cast<size_t>(nn) * sizeof(double);
        if (cudaMalloc(&e.d_eri, bytes) != cudaSuccess) {
            cudaGetLastError();
            e.d_eri = nullptr;
            return set_error("eri_method stored: the N^4 ERI tensor (" + std::to_string(bytes >> 20) +
                             " MiB) does not fit in device memory; use eri_method direct"),
                   HF_ERR_OUT_OF_MEMORY;
        }
        if ((st = compute_eri_tensor(e, e.d_eri, s))) return st;
    }
    if ((st = core_hamiltonian(e, w.S, w.H, s))) return st;
    // purification needs no orbitals; the RI K build takes an orthonormal basis of the
    // occupied space from the projector (occupied_from_projector)
    const bool purify = opt.eigensolver == HF_EIGEN_PURIFICATION;
    bool chol = false;  // the DIIS error must not depend on X, nor X be the caller's
    if (purify && !use_ri && !opt.orthogonalizer && diis_x(opt) == 0 &&
        (st = cholesky_orthogonalizer(e, w.S, s, &chol)))
        return st;
    if (!chol) {
        if ((st = syevd(e, w.S, s, opt.eigensolver))) return st;
        if ((st = orthogonalizer(e, opt, s))) return st;
    }
    GB_LAUNCH_CHECK();
    bool occ_seeded = false;
    auto density_from = [&](const double* Fm) -> int {
        int r;
        if (purify) {
            if ((r = purify_density_scheduled(e, Fm, nocc, w.D, s, opt.purification_max_steps))) return r;
            if (!use_ri) return HF_OK;
            r = occupied_from_projector(e, Fm, nocc, !occ_seeded, s);
            occ_seeded = true;
            return r;
        }
        if ((r = coefficients(e, Fm, s, opt.eigensolver))) return r;
        density_kernel<<<grid_nn(nn), 256, 0, s>>>(w.C, n, nocc, w.D);
        GB_LAUNCH_CHECK();
        return HF_OK;
    };
    if (density_guess) {
        // InitialGuess_RHF_Density: F = F(D_a + D_b); InitialGuess_RHF_SAD then C, D, F
        // (include/rhf.hpp:440-456, :551-584).  The RI K of a density that is no
        // aufbau projector comes from the density itself (not the occupied orbitals).
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(opt.guess_density_a, 1.0, opt.guess_density_b, 1.0, nn, w.D);
        GB_LAUNCH_CHECK();
        if (use_ri) {
            double *J, *K;
            if ((st = ri_require_b(e, s)) || (st = ri_work_buffers(e, &J, &K)) ||
                (st = jk_of(e, true, w.D, J, K, HF_PRECISION_FP64, 0.0, s)) ||
                (st = ri_fock_from_jk(e, w.H, J, K, nullptr, false, w.F, s)))
                return st;
            GB_CUDA_TRY(cudaMemcpyAsync(w.Dprev, w.D, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        } else if ((st = fock_build(true))) {
            return st;
        }
        if (opt.initial_guess == HF_GUESS_SAD) {
            if ((st = density_from(w.F))) return st;
            if ((st = fock_build(true))) return st;
        }
    } else {
        if (opt.initial_guess == HF_GUESS_GWH) {
            gwh_kernel<<<grid_nn(nn), 256, 0, s>>>(w.H, w.S, n, w.E);
            GB_LAUNCH_CHECK();
            if ((st = density_from(w.E))) return st;
        } else if ((st = density_from(w.H))) {
            return st;
        }
        if ((st = fock_build(true))) return st;
    }
    if (!(density_guess && use_ri && opt.initial_guess == HF_GUESS_DENSITY)) fock_ms += elapsed(f0, f1);
    res->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_setup).count();

    cudaEvent_t l0 = lr.ev[6], l1 = lr.ev[7];
    cudaEventRecord(l0, s);
    double prev = std::numeric_limits<double>::max(), energy = 0.0;
    int iter = 0, diis_iter = 0;
    bool converged = false;
    double* d_purify_status = nullptr;
    if (purify && (st = purify_status(e, &d_purify_status))) return st;
    while (iter < opt.max_iter) {
        cudaEventRecord(c0, s);
        if ((st = density_from(w.F))) return st;
        cudaEventRecord(c1, s);
        if ((st = fock_build(false))) return st;
        energy_kernel<<<1, 1024, 0, s>>>(w.D, w.H, w.F, nn, e.d_scalar + 4);
        GB_LAUNCH_CHECK();
        GB_CUDA_TRY(cudaMemcpyAsync(h_energy, e.d_scalar + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
        if (purify)
            GB_CUDA_TRY(cudaMemcpyAsync(h_energy + 8, d_purify_status, kPurifyStatusWords * sizeof(double),
                                        cudaMemcpyDeviceToHost, s));
        fock_ms += elapsed(f0, f1);
        diag_ms += elapsed(c0, c1);
        if (diis_timed) diis_ms += elapsed(q0, q1);
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        energy = *h_energy;
        if (purify) {
            // the purified projector must hold nocc states and be idempotent (a small or
            // closed HOMO-LUMO gap leaves eigenvalues between 0 and 1)
            const double* ps = h_energy + 8;
            if (ps[kPurifyStatusFlags] != 0.0)
                return set_error("purification: a grid-barrier wait ran out"), HF_ERR_CUDA;
            if (!(std::fabs(ps[kPurifyStatusTraceError]) <= kPurifyTraceTol) ||
                !(ps[kPurifyStatusIdempotency] <= kPurifyIdempotencyTol)) {
                if (opt.verbose)
                    std::printf("purification rejected at iteration %d (trace error %.3g, idempotency error %.3g, "
                                "%d SP2 steps): rerunning the SCF with syevd\n",
                                iter, ps[kPurifyStatusTraceError], ps[kPurifyStatusIdempotency],
                                static_cast<int>(ps[kPurifyStatusSteps]));
                return kPurificationRejected;
            }
        }
        const double diff = std::fabs(energy - prev);
        if (opt.verbose)
            std::printf("---- Iteration: %d ----  Energy: %.17g Total energy: %.17g Difference: %.17g\n", iter, energy,
                        energy + res->nuclear_repulsion, diff);
        if (!std::isfinite(energy)) return set_error("SCF energy is not finite"), HF_ERR_NOT_CONVERGED;
        if (diff < opt.convergence_threshold) {
            // mixed RI: energies before the FP64 anchor carry the BF16x3 error of whole K builds
            if (anchored) { converged = true; break; }
        }
        ++iter;
        prev = energy;
        // Fock update: DIIS (Convergence_RHF_DIIS::get_new_fock_matrix) or damping
        cudaEventRecord(q0, s);
        diis_timed = true;
        if (opt.convergence_method != HF_CONV_DIIS) {
            if ((st = damper.step(e, opt, w.F, w.D, nn, s))) return st;
        } else {
            const int slot = diis_iter % m;
            if ((st = diis_error(e, w.S, w.X, w.F, w.D, w.Es + slot * nn, diis_x(opt), s))) return st;
            GB_CUDA_TRY(cudaMemcpyAsync(w.Fs + slot * nn, w.F, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
            const int nprev = std::min(diis_iter + 1, m);
            if (nprev > 1 && (st = diis_extrapolate(e, w.Es, w.Fs, nprev, w.F, s))) return st;
        }
        cudaEventRecord(q1, s);
        ++diis_iter;
    }
    cudaEventRecord(l1, s);
    GB_CUDA_TRY(cudaEventSynchronize(l1));
    if (use_ri && (st = ri_check_flag(e))) return st;
    {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, l0, l1);
        res->scf_ms_total = ms;  // device timeline of the SCF loop (CUDA events on the launching stream)
    }
    int info[4] = {0, 0, 0, 0};
    GB_CUDA_TRY(cudaMemcpy(info, w.info, sizeof(info), cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> cnt(kCounterSlots, 0);
    GB_CUDA_TRY(cudaMemcpy(cnt.data(), e.d_counters, kCounterSlots * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    unsigned long long prim64 = 0, prim32 = 0;
    for (int c = 0; c < kNumClassPairs; ++c) {
        prim64 += cnt[4 * c + 0];
        prim32 += cnt[4 * c + 2];
    }
    if (opt.verbose && info[1])
        std::printf("DIIS: %d error vectors left out of extrapolations as dependent on others\n", info[1]);
    res->diag_ms_total = diag_ms;
    res->diis_ms_total = diis_ms;
    res->electronic_energy = energy;
    res->total_energy = energy + res->nuclear_repulsion;
    res->iterations = iter;
    res->converged = converged ? 1 : 0;
    res->fock_ms_total = fock_ms;
    res->fp64_quartets = static_cast<long long>(prim64);
    res->fp32_quartets = static_cast<long long>(prim32);
    if (info[0] != 0) return set_error("syevd reported info " + std::to_string(info[0])), HF_ERR_SOLVER;
    if (purify && (d_orbital_energies_out || d_coefficients_out)) {
        // purification kept no orbitals: one diagonalisation of the final Fock matrix
        if ((st = coefficients(e, w.F, s, 0))) return st;
    }
    if (d_density_out) GB_CUDA_TRY(cudaMemcpy(d_density_out, w.D, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    if (d_fock_out) GB_CUDA_TRY(cudaMemcpy(d_fock_out, w.F, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    if (d_orbital_energies_out) {
        // orbital energies of the last diagonalised Fock matrix
        GB_CUDA_TRY(cudaMemcpy(d_orbital_energies_out, w.eps, n * sizeof(double), cudaMemcpyDeviceToDevice));
    }
    if (d_coefficients_out) GB_CUDA_TRY(cudaMemcpy(d_coefficients_out, w.C, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    res->eigensolver_used = opt.eigensolver;
    return converged ? HF_OK : (set_error("SCF did not converge"), HF_ERR_NOT_CONVERGED);
}

int hf_rhf_scf(hf_engine* eng, int num_electrons, const hf_scf_options* opt_in, hf_scf_result* res,
               double* d_density_out, double* d_fock_out, double* d_orbital_energies_out, double* d_coefficients_out)
{
    int st = rhf_scf_run(eng, num_electrons, opt_in, res, d_density_out, d_fock_out, d_orbital_energies_out,
                         d_coefficients_out);
    if (st != kPurificationRejected) return st;
    // a purified density failed its checks: the same SCF with a diagonalisation
    hf_scf_options opt;
    if (opt_in) opt = *opt_in; else hf_scf_options_default(&opt);
    opt.eigensolver = HF_EIGEN_SYEVD;
    return rhf_scf_run(eng, num_electrons, &opt, res, d_density_out, d_fock_out, d_orbital_energies_out,
                       d_coefficients_out);
}

}  // extern "C"

extern "C" {

int hf_uhf_scf(hf_engine* eng, int num_alpha, int num_beta, const hf_scf_options* opt_in, hf_scf_result* res,
               double* d_density_a_out, double* d_density_b_out, double* d_orbital_energies_a_out,
               double* d_orbital_energies_b_out, double* d_coefficients_a_out, double* d_coefficients_b_out)
{
    clear_error();
    if (!eng || !res) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (e.nmol != 1) return set_error("hf_uhf_scf: single-molecule engines only"), HF_ERR_INVALID_ARGUMENT;
    hf_scf_options opt;
    if (opt_in) opt = *opt_in; else hf_scf_options_default(&opt);
    const int n = e.num_basis;
    if (num_alpha < 0 || num_beta < 0 || num_alpha + num_beta == 0 || num_alpha > n || num_beta > n)
        return set_error("hf_uhf_scf: bad alpha/beta electron counts"), HF_ERR_INVALID_ARGUMENT;
    if (opt.diis_size < 1 || opt.diis_size > kMaxDiis)
        return set_error("diis_size must be in [1, 16]"), HF_ERR_INVALID_ARGUMENT;
    if (opt.precision != HF_PRECISION_FP64 && opt.precision != HF_PRECISION_MIXED)
        return set_error("unknown precision"), HF_ERR_INVALID_ARGUMENT;
    if (!valid_guess(opt.initial_guess))
        return set_error("initial_guess: core, GWH, density or SAD"), HF_ERR_INVALID_ARGUMENT;
    const bool density_guess = opt.initial_guess == HF_GUESS_DENSITY || opt.initial_guess == HF_GUESS_SAD;
    if (density_guess && !opt.guess_density_a)
        return set_error("initial_guess density/SAD needs guess_density_a"), HF_ERR_INVALID_ARGUMENT;
    if (opt.eri_method != HF_ERI_DIRECT && opt.eri_method != HF_ERI_RI)
        return set_error("unknown eri_method"), HF_ERR_INVALID_ARGUMENT;
    if (!valid_convergence(opt)) return set_error("convergence_method: DIIS, damping or optimal damping"),
                                 HF_ERR_INVALID_ARGUMENT;
    hf_scf_options damp_opt = opt;
    damp_opt.convergence_method = HF_CONV_DAMPING;
    Damper damp_a, damp_b;
    const bool use_ri = opt.eri_method == HF_ERI_RI;
    if (use_ri && !e.ri)
        return set_error("eri_method RI needs an auxiliary basis (hf_engine_set_auxiliary_basis)"),
               HF_ERR_INVALID_ARGUMENT;
    const int m = opt.diis_size;
    int st = ensure_scf(e, m);
    if (st) return st;
    auto& w = e.scf;
    const long long nn = static_cast<long long>(n) * n;
    cudaStream_t s = nullptr;
    cublasSetStream(e.cublas, s);
    cusolverDnSetStream(e.cusolver, s);
    if (use_ri && (st = ri_require_b(e, s))) return st;
    // beta-spin buffers and the two J/K pairs (owned by this call)
    std::vector<void*> owned;
    auto buf = [&](double*& p, size_t count) -> int {
        if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess)
            return set_error("cudaMalloc (UHF) failed"), HF_ERR_OUT_OF_MEMORY;
        owned.push_back(p);
        return HF_OK;
    };
    double *Fb = nullptr, *Db = nullptr, *Ja = nullptr, *Ka = nullptr, *Jb = nullptr, *Kb = nullptr, *epsb = nullptr,
           *Esb = nullptr, *Fsb = nullptr, *Ca = nullptr, *Cb = nullptr, *epsa = nullptr;
    struct Free {
        std::vector<void*>& v;
        ~Free() { for (void* p : v) cudaFree(p); }
    } guard{owned};
    if ((st = buf(Fb, nn)) || (st = buf(Db, nn)) || (st = buf(Ja, nn)) || (st = buf(Ka, nn)) || (st = buf(Jb, nn)) ||
        (st = buf(Kb, nn)) || (st = buf(epsb, n)) || (st = buf(Esb, nn * m)) || (st = buf(Fsb, nn * m)) ||
        (st = buf(Ca, nn)) || (st = buf(Cb, nn)) || (st = buf(epsa, n)))
        return st;
    double* Fa = w.F;
    double* Da = w.D;
    *res = hf_scf_result{};
    res->nuclear_repulsion = nuclear_repulsion(e);
    GB_CUDA_TRY(cudaMemsetAsync(w.info, 0, 4 * sizeof(int), s));
    LoopResources lr;
    double* h_energy = lr.h_energy;

    // spin densities from FA and FB; break = the guess's beta symmetry break
    auto densities = [&](const double* FA, const double* FB, bool brk) -> int {
        int r;
        // the orbitals and orbital energies behind the densities are kept for the export
        if ((r = coefficients(e, FA, s, opt.eigensolver))) return r;
        density_factor_kernel<<<grid_nn(nn), 256, 0, s>>>(w.C, n, num_alpha, 1.0, Da);
        GB_LAUNCH_CHECK();
        GB_CUDA_TRY(cudaMemcpyAsync(Ca, w.C, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        GB_CUDA_TRY(cudaMemcpyAsync(epsa, w.eps, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if ((r = coefficients(e, FB, s, opt.eigensolver))) return r;
        if (brk) {
            break_symmetry_kernel<<<(n + 255) / 256, 256, 0, s>>>(w.C, n);
            GB_LAUNCH_CHECK();
        }
        density_factor_kernel<<<grid_nn(nn), 256, 0, s>>>(w.C, n, num_beta, 1.0, Db);
        GB_LAUNCH_CHECK();
        GB_CUDA_TRY(cudaMemcpyAsync(Cb, w.C, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        GB_CUDA_TRY(cudaMemcpyAsync(epsb, w.eps, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        return HF_OK;
    };
    auto fock = [&]() -> int {
        int r;
        if ((r = jk_of(e, use_ri, Da, Ja, Ka, opt.precision, opt.mixed_threshold, s))) return r;
        if ((r = jk_of(e, use_ri, Db, Jb, Kb, opt.precision, opt.mixed_threshold, s))) return r;
        uhf_fock_kernel<<<grid_nn(nn), 256, 0, s>>>(w.H, Ja, Jb, Ka, Kb, nn, Fa, Fb);
        GB_LAUNCH_CHECK();
        return HF_OK;
    };
    cudaEvent_t l0 = lr.ev[0], l1 = lr.ev[1];
    // core Hamiltonian, X, guess (InitialGuess_UHF_Core / _GWH / _Density / _SAD,
    // include/uhf.hpp:484-620): orbitals for both spins with the beta symmetry break
    if ((st = core_hamiltonian(e, w.S, w.H, s))) return st;
    if ((st = syevd(e, w.S, s, opt.eigensolver))) return st;
    if ((st = orthogonalizer(e, opt, s))) return st;
    GB_LAUNCH_CHECK();
    if (density_guess) {
        // D_a, D_b given (D_b NULL: both halves of D_a); F, C, break, D, F
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(opt.guess_density_a, opt.guess_density_b ? 1.0 : 0.5, nullptr,
                                                    0.0, nn, Da);
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(opt.guess_density_b ? opt.guess_density_b : opt.guess_density_a,
                                                    opt.guess_density_b ? 1.0 : 0.5, nullptr, 0.0, nn, Db);
        GB_LAUNCH_CHECK();
        if ((st = fock())) return st;
        if ((st = densities(Fa, Fb, true))) return st;
    } else if (opt.initial_guess == HF_GUESS_GWH) {
        gwh_kernel<<<grid_nn(nn), 256, 0, s>>>(w.H, w.S, n, w.E);
        GB_LAUNCH_CHECK();
        if ((st = densities(w.E, w.E, true))) return st;
    } else if ((st = densities(w.H, w.H, true))) {
        return st;
    }
    if ((st = fock())) return st;
    cudaEventRecord(l0, s);
    double prev = std::numeric_limits<double>::max(), energy = 0.0;
    int iter = 0, diis_iter = 0;
    bool converged = false;
    while (iter < opt.max_iter) {
        if ((st = densities(Fa, Fb, false))) return st;
        if ((st = fock())) return st;
        uhf_energy_kernel<<<1, 1024, 0, s>>>(Da, Db, w.H, Fa, Fb, nn, e.d_scalar + 4);
        GB_LAUNCH_CHECK();
        GB_CUDA_TRY(cudaMemcpyAsync(h_energy, e.d_scalar + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        energy = *h_energy;
        if (!std::isfinite(energy)) return set_error("UHF energy is not finite"), HF_ERR_NOT_CONVERGED;
        if (std::fabs(energy - prev) < opt.convergence_threshold) { converged = true; break; }
        ++iter;
        prev = energy;
        if (opt.convergence_method != HF_CONV_DIIS) {
            // Convergence_UHF_Damping (include/uhf.hpp:196-250): a constant factor for both spins
            // (the reference has no optimal factor for UHF)
            if ((st = damp_a.step(e, damp_opt, Fa, Da, nn, s)) || (st = damp_b.step(e, damp_opt, Fb, Db, nn, s)))
                return st;
            ++diis_iter;
            continue;
        }
        // DIIS per spin on the same cyclic ring index (Convergence_UHF_DIIS, include/uhf.hpp:291-380)
        const int slot = diis_iter % m;
        const int nprev = std::min(diis_iter + 1, m);
        if ((st = diis_error(e, w.S, w.X, Fa, Da, w.Es + slot * nn, diis_x(opt), s))) return st;
        GB_CUDA_TRY(cudaMemcpyAsync(w.Fs + slot * nn, Fa, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (nprev > 1 && (st = diis_extrapolate(e, w.Es, w.Fs, nprev, Fa, s))) return st;
        if ((st = diis_error(e, w.S, w.X, Fb, Db, Esb + slot * nn, diis_x(opt), s))) return st;
        GB_CUDA_TRY(cudaMemcpyAsync(Fsb + slot * nn, Fb, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (nprev > 1 && (st = diis_extrapolate(e, Esb, Fsb, nprev, Fb, s))) return st;
        ++diis_iter;
    }
    cudaEventRecord(l1, s);
    GB_CUDA_TRY(cudaEventSynchronize(l1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, l0, l1);
    res->scf_ms_total = ms;
    res->electronic_energy = energy;
    res->total_energy = energy + res->nuclear_repulsion;
    res->iterations = iter;
    res->converged = converged ? 1 : 0;
    if (d_density_a_out) GB_CUDA_TRY(cudaMemcpy(d_density_a_out, Da, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    if (d_density_b_out) GB_CUDA_TRY(cudaMemcpy(d_density_b_out, Db, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    // orbital energies and coefficients of the last diagonalisations (the ones behind the
    // returned densities, as the reference's export reads them)
    if (d_orbital_energies_a_out)
        GB_CUDA_TRY(cudaMemcpy(d_orbital_energies_a_out, epsa, n * sizeof(double), cudaMemcpyDeviceToDevice));
    if (d_coefficients_a_out) GB_CUDA_TRY(cudaMemcpy(d_coefficients_a_out, Ca, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    if (d_orbital_energies_b_out)
        GB_CUDA_TRY(cudaMemcpy(d_orbital_energies_b_out, epsb, n * sizeof(double), cudaMemcpyDeviceToDevice));
    if (d_coefficients_b_out) GB_CUDA_TRY(cudaMemcpy(d_coefficients_b_out, Cb, nn * sizeof(double), cudaMemcpyDeviceToDevice));
    return converged ? HF_OK : (set_error("UHF did not converge"), HF_ERR_NOT_CONVERGED);
}


int hf_rohf_scf(hf_engine* eng, int num_alpha, int num_beta, const double* coupling, const hf_scf_options* opt_in,
                hf_scf_result* res, double* d_density_a_out, double* d_density_b_out, double* d_orbital_energies_out,
                double* d_coefficients_out)
{
    clear_error();
    if (!eng || !res) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (e.nmol != 1) return set_error("hf_rohf_scf: single-molecule engines only"), HF_ERR_INVALID_ARGUMENT;
    hf_scf_options opt;
    if (opt_in) opt = *opt_in; else hf_scf_options_default(&opt);
    const int n = e.num_basis;
    if (num_beta < 0 || num_alpha < num_beta || num_alpha == 0 || num_alpha > n)
        return set_error("hf_rohf_scf: needs 0 <= num_beta <= num_alpha <= N, num_alpha > 0"),
               HF_ERR_INVALID_ARGUMENT;
    if (opt.diis_size < 1 || opt.diis_size > kMaxDiis)
        return set_error("diis_size must be in [1, 16]"), HF_ERR_INVALID_ARGUMENT;
    if (opt.precision != HF_PRECISION_FP64 && opt.precision != HF_PRECISION_MIXED)
        return set_error("unknown precision"), HF_ERR_INVALID_ARGUMENT;
    if (!valid_guess(opt.initial_guess))
        return set_error("initial_guess: core, GWH, density or SAD"), HF_ERR_INVALID_ARGUMENT;
    const bool density_guess = opt.initial_guess == HF_GUESS_DENSITY || opt.initial_guess == HF_GUESS_SAD;
    if (density_guess && (!opt.guess_density_a || !opt.guess_density_b))
        return set_error("ROHF initial_guess density/SAD needs guess_density_a and _b"), HF_ERR_INVALID_ARGUMENT;
    if (!valid_convergence(opt)) return set_error("convergence_method: DIIS, damping or optimal damping"),
                                 HF_ERR_INVALID_ARGUMENT;
    Damper damper;
    if (opt.eri_method != HF_ERI_DIRECT && opt.eri_method != HF_ERI_RI)
        return set_error("unknown eri_method"), HF_ERR_INVALID_ARGUMENT;
    const bool use_ri = opt.eri_method == HF_ERI_RI;
    if (use_ri && !e.ri)
        return set_error("eri_method RI needs an auxiliary basis (hf_engine_set_auxiliary_basis)"),
               HF_ERR_INVALID_ARGUMENT;
    // Roothaan's constants by default (rohf_parameter_name = roothaan, src/rohf.cu:31)
    RohfCoupling cp{-0.5, 1.5, 0.5, 0.5, 1.5, -0.5};
    if (coupling) cp = RohfCoupling{coupling[0], coupling[1], coupling[2], coupling[3], coupling[4], coupling[5]};
    const int nc = num_beta, no = num_alpha - num_beta;
    const int m = opt.diis_size;
    int st = ensure_scf(e, m);
    if (st) return st;
    auto& w = e.scf;
    const long long nn = static_cast<long long>(n) * n;
    cudaStream_t s = nullptr;
    cublasSetStream(e.cublas, s);
    cusolverDnSetStream(e.cusolver, s);
    if (use_ri && (st = ri_require_b(e, s))) return st;
    std::vector<void*> owned;
    struct Free {
        std::vector<void*>& v;
        ~Free() { for (void* p : v) cudaFree(p); }
    } guard{owned};
    auto buf = [&](double*& p, size_t count) -> int {
        if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess)
            return set_error("cudaMalloc (ROHF) failed"), HF_ERR_OUT_OF_MEMORY;
        owned.push_back(p);
        return HF_OK;
    };
    double *Dc = nullptr, *Do = nullptr, *Fc = nullptr, *Fo = nullptr, *Jc = nullptr, *Kc = nullptr, *Jo = nullptr,
           *Ko = nullptr, *R = nullptr;
    if ((st = buf(Dc, nn)) || (st = buf(Do, nn)) || (st = buf(Fc, nn)) || (st = buf(Fo, nn)) || (st = buf(Jc, nn)) ||
        (st = buf(Kc, nn)) || (st = buf(Jo, nn)) || (st = buf(Ko, nn)) || (st = buf(R, nn)))
        return st;
    *res = hf_scf_result{};
    res->nuclear_repulsion = nuclear_repulsion(e);
    GB_CUDA_TRY(cudaMemsetAsync(w.info, 0, 4 * sizeof(int), s));
    LoopResources lr;
    double* h_energy = lr.h_energy;

    auto density = [&]() -> int {
        rohf_density_kernel<<<grid_nn(nn), 256, 0, s>>>(w.C, n, nc, no, Dc, Do, w.D);
        GB_LAUNCH_CHECK();
        return HF_OK;
    };
    // F_c, F_o from D_c, D_o; the unified F = S C R C^T S from the current orbitals C
    auto fock = [&]() -> int {
        int r;
        if ((r = jk_of(e, use_ri, Dc, Jc, Kc, opt.precision, opt.mixed_threshold, s))) return r;
        if (no > 0) {
            if ((r = jk_of(e, use_ri, Do, Jo, Ko, opt.precision, opt.mixed_threshold, s))) return r;
        } else {
            GB_CUDA_TRY(cudaMemsetAsync(Jo, 0, nn * sizeof(double), s));
            GB_CUDA_TRY(cudaMemsetAsync(Ko, 0, nn * sizeof(double), s));
        }
        rohf_fock_kernel<<<grid_nn(nn), 256, 0, s>>>(w.H, Jc, Jo, Kc, Ko, nn, Fc, Fo);
        GB_LAUNCH_CHECK();
        // C^T F_c C and C^T F_o C (Jc, Jo reused as the MO-basis matrices)
        if ((r = gemm_rm(e.cublas, true, false, n, w.C, Fc, w.T1)) ||
            (r = gemm_rm(e.cublas, false, false, n, w.T1, w.C, Jc)) ||
            (r = gemm_rm(e.cublas, true, false, n, w.C, Fo, w.T1)) ||
            (r = gemm_rm(e.cublas, false, false, n, w.T1, w.C, Jo)))
            return r;
        rohf_unified_kernel<<<grid_nn(nn), 256, 0, s>>>(Jc, Jo, cp, nc, no, n, R);
        GB_LAUNCH_CHECK();
        // T1 = S C, T2 = T1 R, F = T2 T1^T
        if ((r = gemm_rm(e.cublas, false, false, n, w.S, w.C, w.T1)) ||
            (r = gemm_rm(e.cublas, false, false, n, w.T1, R, w.T2)) ||
            (r = gemm_rm(e.cublas, false, true, n, w.T2, w.T1, w.F)))
            return r;
        return HF_OK;
    };
    // core Hamiltonian, X, guess (InitialGuess_ROHF_Core / _GWH / _Density / _SAD,
    // include/rohf.hpp:416-600).  For the density guesses the first unified Fock
    // matrix is formed with the core-guess orbitals.
    if ((st = core_hamiltonian(e, w.S, w.H, s))) return st;
    if ((st = syevd(e, w.S, s, opt.eigensolver))) return st;
    if ((st = orthogonalizer(e, opt, s))) return st;
    GB_LAUNCH_CHECK();
    if (density_guess) {
        if ((st = coefficients(e, w.H, s, opt.eigensolver))) return st;
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(opt.guess_density_b, 2.0, nullptr, 0.0, nn, Dc);
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(opt.guess_density_a, 1.0, opt.guess_density_b, -1.0, nn, Do);
        GB_LAUNCH_CHECK();
        if ((st = fock())) return st;
        if ((st = coefficients(e, w.F, s, opt.eigensolver))) return st;
    } else if (opt.initial_guess == HF_GUESS_GWH) {
        gwh_kernel<<<grid_nn(nn), 256, 0, s>>>(w.H, w.S, n, w.E);
        GB_LAUNCH_CHECK();
        if ((st = coefficients(e, w.E, s, opt.eigensolver))) return st;
    } else if ((st = coefficients(e, w.H, s, opt.eigensolver))) {
        return st;
    }
    if ((st = density()) || (st = fock())) return st;

    cudaEvent_t l0 = lr.ev[0], l1 = lr.ev[1];
    cudaEventRecord(l0, s);
    double prev = std::numeric_limits<double>::max(), energy = 0.0;
    int iter = 0, diis_iter = 0;
    bool converged = false;
    while (iter < opt.max_iter) {
        if ((st = coefficients(e, w.F, s, opt.eigensolver)) || (st = density()) || (st = fock())) break;
        rohf_energy_kernel<<<1, 1024, 0, s>>>(Dc, Do, w.H, Fc, Fo, nn, e.d_scalar + 4);
        if (cudaGetLastError() != cudaSuccess) { st = (set_error("rohf_energy_kernel launch failed"), HF_ERR_CUDA); break; }
        if (cudaMemcpyAsync(h_energy, e.d_scalar + 4, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            st = (set_error("ROHF energy read failed"), HF_ERR_CUDA);
            break;
        }
        energy = *h_energy;
        if (opt.verbose)
            std::printf("---- Iteration: %d ----  Energy: %.17g Total energy: %.17g\n", iter, energy,
                        energy + res->nuclear_repulsion);
        if (!std::isfinite(energy)) { st = (set_error("ROHF energy is not finite"), HF_ERR_NOT_CONVERGED); break; }
        if (std::fabs(energy - prev) < opt.convergence_threshold) { converged = true; break; }
        ++iter;
        prev = energy;
        if (opt.convergence_method != HF_CONV_DIIS) {
            // Convergence_ROHF_Damping (include/rohf.hpp:216-290) on the unified F with D
            if ((st = damper.step(e, opt, w.F, w.D, nn, s))) break;
            ++diis_iter;
            continue;
        }
        // Convergence_ROHF_DIIS (include/rohf.hpp:307-360): unified F with D = D_c + D_o
        const int slot = diis_iter % m;
        if ((st = diis_error(e, w.S, w.X, w.F, w.D, w.Es + slot * nn, diis_x(opt), s))) break;
        if (cudaMemcpyAsync(w.Fs + slot * nn, w.F, nn * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            st = (set_error("cudaMemcpyAsync failed"), HF_ERR_CUDA);
            break;
        }
        const int nprev = std::min(diis_iter + 1, m);
        if (nprev > 1 && (st = diis_extrapolate(e, w.Es, w.Fs, nprev, w.F, s))) break;
        ++diis_iter;
    }
    cudaEventRecord(l1, s);
    cudaEventSynchronize(l1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, l0, l1);
    if (st) return st;
    res->scf_ms_total = ms;
    res->electronic_energy = energy;
    res->total_energy = energy + res->nuclear_repulsion;
    res->iterations = iter;
    res->converged = converged ? 1 : 0;
    int info[4] = {0, 0, 0, 0};
    GB_CUDA_TRY(cudaMemcpy(info, w.info, sizeof(info), cudaMemcpyDeviceToHost));
    if (info[0] != 0) return set_error("syevd reported info " + std::to_string(info[0])), HF_ERR_SOLVER;
    // export_density_matrix (src/rohf.cu:288-315): alpha = D_c/2 + D_o, beta = D_c/2
    if (d_density_a_out) {
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(Dc, 0.5, Do, 1.0, nn, d_density_a_out);
        GB_LAUNCH_CHECK();
    }
    if (d_density_b_out) {
        combine_kernel<<<grid_nn(nn), 256, 0, s>>>(Dc, 0.5, nullptr, 0.0, nn, d_density_b_out);
        GB_LAUNCH_CHECK();
    }
    if (d_orbital_energies_out)
        GB_CUDA_TRY(cudaMemcpyAsync(d_orbital_energies_out, w.eps, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (d_coefficients_out)
        GB_CUDA_TRY(cudaMemcpyAsync(d_coefficients_out, w.C, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return converged ? HF_OK : (set_error("ROHF did not converge"), HF_ERR_NOT_CONVERGED);
}

}  // extern "C"
