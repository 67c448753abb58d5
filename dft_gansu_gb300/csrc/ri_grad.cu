// Analytic nuclear gradient of the RI (density-fitted) RHF two-electron energy.
//
// The forward path is the reference's RI Fock build (src/gpu_manager.cu:1448-1632):
// V = (P|Q) = L L^T, B = L^-1 T with T_P,mu nu = (mu nu|P), J = sum_P B_P (B_P . D),
// K = sum_P B_P D B_P.  With c = V^-1 d, d_P = T_P . D and C_P = sum_Q (V^-1)_PQ T_Q,
// the two-electron energy E2 = 1/2 d^T V^-1 d - 1/4 sum_PQ (V^-1)_PQ tr(T_P D T_Q D)
// has, at fixed D,
//     dE2/dx = sum_P,mu nu dT_P,mu nu/dx Gamma_P,mu nu - 1/2 sum_PQ dV_PQ/dx gamma_PQ,
//     Gamma_P = c_P D - 1/2 D C_P D,   gamma_PQ = c_P c_Q - 1/2 tr(C_P D C_Q D).
// With D = 2 C_o C_o^T (C_o the occupied orbitals) and X_P = C_o^T C_P C_o:
//     D C_P D = 4 C_o X_P C_o^T,   tr(C_P D C_Q D) = 4 tr(X_P X_Q),
// and X = L^-T Z with Z_P = C_o^T B_P C_o, c = L^-T (B . D): no V^-1 T tensor is
// formed.  The weights are built here with cuBLAS (batched DGEMMs, triangular
// solves with L); the derivative integrals are ri_grad_kernel.cuh.
#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.hpp"
#include "ri.hpp"
#include "ri_grad_kernel.cuh"

namespace gb {
namespace {

// Gamma_P,tri(mu,nu) = c_P D_mu nu - 2 H_P,mu nu for the rows p0 .. p0 + rows of a chunk
__global__ void gamma_pack_kernel(const double* __restrict__ H, const double* __restrict__ D,
                                  const double* __restrict__ c, int n, int p0, int rows, double* __restrict__ G)
{
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    const long long total = npk * rows;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int r = static_cast<int>(k / npk);
        const long long q = k - static_cast<long long>(r) * npk;
        int i = static_cast<int>((sqrt(8.0 * static_cast<double>(q) + 1.0) - 1.0) * 0.5);
        while (static_cast<long long>(i) * (i + 1) / 2 > q) --i;
        while (static_cast<long long>(i + 1) * (i + 2) / 2 <= q) ++i;
        const int j = static_cast<int>(q - static_cast<long long>(i) * (i + 1) / 2);
        const int P = p0 + r;
        G[static_cast<long long>(P) * npk + q] =
            c[P] * D[static_cast<long long>(i) * n + j] - 2.0 * H[(static_cast<long long>(r) * n + i) * n + j];
    }
}

int grid_of(long long work, int num_sms)
{
    return static_cast<int>(std::max<long long>(1, std::min<long long>((work + 255) / 256, num_sms * 16LL)));
}

// device workspace released at scope end
struct DevMem {
    double* p = nullptr;
    ~DevMem() { cudaFree(p); }
    int alloc(size_t n)
    {
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            set_error("cudaMalloc (RI gradient workspace) failed");
            return HF_ERR_OUT_OF_MEMORY;
        }
        return HF_OK;
    }
};

RiDerivLaunch deriv_launcher(int la, int lb, int lp)
{
    switch (lp) {
    case 0: return ri_deriv_launcher<0>(la, lb);
    case 1: return ri_deriv_launcher<1>(la, lb);
    case 2: return ri_deriv_launcher<2>(la, lb);
    case 3: return ri_deriv_launcher<3>(la, lb);
    default: return nullptr;
    }
}

}  // namespace

int ri_gradient_two_electron(Engine& e, const double* d_D, const double* d_C, int ldc, int nocc, cudaStream_t s)
{
    if (!e.ri) return set_error("RI gradient: no auxiliary basis"), HF_ERR_INVALID_ARGUMENT;
    int st;
    if ((st = ri_require_b(e, s))) return st;
    RiState& r = *e.ri;
    const int n = e.num_basis, M = r.naux;
    const long long nn = static_cast<long long>(n) * n, npk = static_cast<long long>(n) * (n + 1) / 2;
    const long long o2 = static_cast<long long>(nocc) * nocc;
    cublasSetStream(e.cublas, s);
    const double one = 1.0, zero = 0.0;
    DevMem Dt, c, Z, G, gam, Y, H;
    if ((st = Dt.alloc(npk)) || (st = c.alloc(M)) || (st = Z.alloc(static_cast<size_t>(M) * o2)) ||
        (st = G.alloc(static_cast<size_t>(M) * npk)) || (st = gam.alloc(static_cast<size_t>(M) * M)))
        return st;
    // c = L^-T (B . D): w_P over the packed triangle (off-diagonal doubled), then a triangular solve
    if ((st = ri_w_of(e, d_D, Dt.p, c.p, s))) return st;
    if (cublasDtrsv(e.cublas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, M, r.d_V, M, c.p, 1) !=
        CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDtrsv (RI gradient) failed"), HF_ERR_SOLVER;
    // Z_P = C_o^T B_P C_o in chunks of auxiliary functions (Y_P = B_P C_o as an intermediate)
    if ((st = ri_full_b(e, s))) return st;
    const int chunk =
        static_cast<int>(std::max<long long>(1, std::min<long long>(M, (1LL << 28) / std::max(nn, 1LL))));
    if ((st = Y.alloc(static_cast<size_t>(chunk) * n * nocc)) || (st = H.alloc(static_cast<size_t>(chunk) * nn)))
        return st;
    for (int p0 = 0; p0 < M; p0 += chunk) {
        const int rows = std::min(chunk, M - p0);
        // column-major: Y_P^T (nocc x n) = C_o^T (nocc x n, ld ldc) B_P;  Z_P = Y_P^T C_o
        if (cublasDgemmStridedBatched(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, nocc, n, n, &one, d_C, ldc, 0,
                                      r.d_B + static_cast<long long>(p0) * nn, n, nn, &zero, Y.p, nocc,
                                      static_cast<long long>(n) * nocc, rows) != CUBLAS_STATUS_SUCCESS ||
            cublasDgemmStridedBatched(e.cublas, CUBLAS_OP_N, CUBLAS_OP_T, nocc, nocc, n, &one, Y.p, nocc,
                                      static_cast<long long>(n) * nocc, d_C, ldc, 0, &zero,
                                      Z.p + static_cast<long long>(p0) * o2, nocc, o2, rows) != CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDgemmStridedBatched (RI gradient Z) failed"), HF_ERR_SOLVER;
    }
    // X = L^-T Z: with Z stored [P][k] (column-major nocc^2 x M), solve X^T L = Z^T in place
    if (cublasDtrsm(e.cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                    static_cast<int>(o2), M, &one, r.d_V, M, Z.p, static_cast<int>(o2)) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDtrsm (RI gradient X) failed"), HF_ERR_SOLVER;
    // gamma = c c^T - 2 X X^T
    const double m2 = -2.0;
    if (cublasDgemm(e.cublas, CUBLAS_OP_T, CUBLAS_OP_N, M, M, static_cast<int>(o2), &m2, Z.p, static_cast<int>(o2),
                    Z.p, static_cast<int>(o2), &zero, gam.p, M) != CUBLAS_STATUS_SUCCESS ||
        cublasDger(e.cublas, M, M, &one, c.p, 1, c.p, 1, gam.p, M) != CUBLAS_STATUS_SUCCESS)
        return set_error("cuBLAS (RI gradient gamma) failed"), HF_ERR_SOLVER;
    // Gamma_P = c_P D - 2 C_o X_P C_o^T, packed
    for (int p0 = 0; p0 < M; p0 += chunk) {
        const int rows = std::min(chunk, M - p0);
        // G_P^T (nocc x n) = X_P C_o^T ; H_P (n x n) = C_o G_P^T
        if (cublasDgemmStridedBatched(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, nocc, n, nocc, &one,
                                      Z.p + static_cast<long long>(p0) * o2, nocc, o2, d_C, ldc, 0, &zero, Y.p, nocc,
                                      static_cast<long long>(n) * nocc, rows) != CUBLAS_STATUS_SUCCESS ||
            cublasDgemmStridedBatched(e.cublas, CUBLAS_OP_T, CUBLAS_OP_N, n, n, nocc, &one, d_C, ldc, 0, Y.p, nocc,
                                      static_cast<long long>(n) * nocc, &zero, H.p, n, nn, rows) !=
                CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDgemmStridedBatched (RI gradient Gamma) failed"), HF_ERR_SOLVER;
        gamma_pack_kernel<<<grid_of(npk * rows, e.num_sms), 256, 0, s>>>(H.p, d_D, c.p, n, p0, rows, G.p);
        GB_LAUNCH_CHECK();
    }
    // metric weights: -1/2 gamma (the metric term's prefactor)
    const double mh = -0.5;
    if (cublasDscal(e.cublas, M * M, &mh, gam.p, 1) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDscal (RI gradient) failed"), HF_ERR_SOLVER;

    // derivative integrals contracted with the weights, into e.d_grad
    const size_t sgrad = sizeof(double) * 3 * e.num_atoms;
    const bool shared = sgrad <= 32 * 1024;
    auto run = [&](const ShellPairDev* bra, int nbra, const PrimPair64* bra_pp, const double* bra_scale, int la,
                   int lb, int lq, const double* weight, long long ld, int mode) -> int {
        RiDerivArgs a;
        a.bra = bra;
        a.nbra = nbra;
        a.bra_pp = bra_pp;
        a.ket = r.d_aux + r.class_begin[lq];
        a.nket = r.class_count[lq];
        a.aux_all = r.d_aux;
        a.aux_pp = r.d_aux_pp;
        a.boys = e.d_boys64;
        a.bra_scale = bra_scale;
        a.aux_scale = r.d_aux_scale;
        a.thr = e.schwarz_threshold;
        a.weight = weight;
        a.ld = ld;
        a.mode = mode;
        a.shell_atom = e.d_shell_atom;
        a.natom = e.num_atoms;
        a.shared_grad = shared ? 1 : 0;
        a.grad = e.d_grad;
        RiDerivLaunch f = deriv_launcher(la, lb, lq);
        if (!f) return set_error("RI gradient: unsupported shell class"), HF_ERR_INVALID_ARGUMENT;
        const long long work = static_cast<long long>(nbra) * a.nket * ncart(lq);
        const int grid = static_cast<int>(std::max<long long>(
            1, std::min<long long>((work + kRiGradThreads - 1) / kRiGradThreads, e.num_sms * 8LL)));
        f(a, grid, shared ? sgrad : 0, s);
        GB_LAUNCH_CHECK();
        return HF_OK;
    };
    for (const PairClass& pc : e.pair_classes) {
        if (!pc.count) continue;
        for (int lq = 0; lq <= kMaxAuxL; ++lq) {
            if (!r.class_count[lq]) continue;
            if ((st = run(e.d_pairs + pc.begin, pc.count, e.d_pp64, e.d_scale, pc.la, pc.lb, lq, G.p, npk, 0)))
                return st;
        }
    }
    for (int lp = 0; lp <= kMaxAuxL; ++lp)
        for (int lq = 0; lq <= kMaxAuxL; ++lq) {
            if (!r.class_count[lp] || !r.class_count[lq]) continue;
            if ((st = run(r.d_aux_pairs + r.class_begin[lp], r.class_count[lp], r.d_aux_pp, r.d_aux_scale, lp, 0, lq,
                          gam.p, M, 1)))
                return st;
        }
    // the workspaces are freed on return: finish the work that reads them first
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return HF_OK;
}

}  // namespace gb
