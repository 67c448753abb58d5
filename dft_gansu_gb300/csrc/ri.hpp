// RI (density fitting) state attached to an Engine.
#pragma once
#include <cuda_bf16.h>

#include "engine.hpp"

namespace gb {

constexpr int kMaxAuxL = 3;  // auxiliary shells up to f (cc-pVDZ-RIFIT for H..Ar)

// One contracted auxiliary shell; its primitives are PrimPair64 records of
// (gamma, unit s) pairs: p = gamma, K = scaled coefficient * sqrt(2 pi^{5/2}),
// P = centre, PA = 0, Q = reference auxiliary bound.
struct AuxShellDev {
    double x, y, z;
    int l, bf, p_off, np;
    int atom;  // atom of the shell (the RI gradient's third centre)
};

struct RiState {
    int naux = 0;
    int class_begin[kMaxAuxL + 1] = {0, 0, 0, 0};  // auxiliary shells sorted by l
    int class_count[kMaxAuxL + 1] = {0, 0, 0, 0};
    std::vector<AuxShellDev> shells;
    AuxShellDev* d_aux = nullptr;
    PrimPair64* d_aux_pp = nullptr;
    ShellPairDev* d_aux_pairs = nullptr;  // (P, unit) bra pairs for the metric
    double* d_aux_scale = nullptr;        // s_P = auxiliary CGTO factor * component factor

    bool have_b = false, have_full = false;
    double* d_V = nullptr;   // metric, then its Cholesky factor (column-major lower)
    double* d_Bp = nullptr;  // B packed: naux x N(N+1)/2, row-major
    double* d_B = nullptr;   // B full: [P][mu][nu] (the reference layout), expanded on first use by K
    double* d_Dt = nullptr;  // packed density with doubled off-diagonal
    double* d_W = nullptr;   // naux
    double* d_X = nullptr;   // K intermediate: N x (naux r), row-major
    size_t x_len = 0;
    double* d_J = nullptr;
    double* d_K = nullptr;
    double* d_Y = nullptr;     // density factor
    double* d_evec = nullptr;  // density eigenvectors (arbitrary-D K)
    double* d_eval = nullptr;
    double* d_work = nullptr;  // cuSOLVER workspace
    size_t work_len = 0;
    int* d_info = nullptr;

    // mixed tier: B as BF16 hi/lo planes [(P, mu)][nu] (row pitch kpad_n), tensor-core K
    __nv_bfloat16 *d_Bh = nullptr, *d_Bl = nullptr;
    long long kpad_n = 0;
    __nv_bfloat16 *d_Yh = nullptr, *d_Yl = nullptr, *d_Y2h = nullptr, *d_Y2l = nullptr;  // factor planes (r x kpad_n)
    __nv_bfloat16 *d_Xh = nullptr, *d_Xl = nullptr, *d_X2h = nullptr, *d_X2l = nullptr;  // N x (naux r_blk)
    int r_blk = 0;            // columns per auxiliary function in the X planes (multiple of 64)
    int r_cap = 0;            // factor rows the plane buffers hold
    double* d_Kacc = nullptr; // accumulated K of the incremental builds
    double* d_Cprev = nullptr;  // occupied orbitals of the last build (N x r, row-major)
    double *d_T1 = nullptr, *d_M = nullptr, *d_U = nullptr, *d_U2 = nullptr, *d_Ca = nullptr;  // alignment work
    int* d_flag = nullptr;    // tensor-core pipeline error flag
};

int ri_set_auxiliary(Engine& e, const hf_primitive_shell* prims, int nprim, const double* cgto, int naux);
int ri_metric(Engine& e, double* d_V, cudaStream_t s);
int ri_three_center_packed(Engine& e, double* d_T, cudaStream_t s);
int ri_expand(Engine& e, const double* d_packed, long long rows, double* d_full, cudaStream_t s);
int ri_build_b(Engine& e, cudaStream_t s);
int ri_require_b(Engine& e, cudaStream_t s);
int ri_j(Engine& e, const double* d_D, double* d_J, cudaStream_t s);
int ri_k_occupied(Engine& e, const double* d_C, int nocc, double* d_K, cudaStream_t s);
int ri_k_density(Engine& e, const double* d_D, double* d_K, cudaStream_t s);
int ri_fock_from_jk(Engine& e, const double* d_H, const double* d_J, const double* d_K, double* d_G, bool accumulate,
                    double* d_F, cudaStream_t s);
int ri_work_buffers(Engine& e, double** J, double** K);
// B in the full [P][mu][nu] layout (expanded once from the packed B)
int ri_full_b(Engine& e, cudaStream_t s);
// w_P = sum_mu nu B_P,mu nu D_mu nu (packed density into d_Dt, N(N+1)/2 doubles)
int ri_w_of(Engine& e, const double* d_D, double* d_Dt, double* d_w, cudaStream_t s);
// RI two-electron part of the RHF gradient, accumulated into e.d_grad (ri_grad.cu)
int ri_gradient_two_electron(Engine& e, const double* d_D, const double* d_C, int ldc, int nocc, cudaStream_t s);

// mixed tier (tensor cores)
int ri_prepare_planes(Engine& e, int nocc, cudaStream_t s);
int ri_k_tc_full(Engine& e, const double* d_C, int ldc, int nocc, double* d_K, cudaStream_t s);
int ri_k_tc_delta(Engine& e, const double* d_C, int ldc, int nocc, const double* d_S, double* d_K, bool* aligned,
                  cudaStream_t s);
int ri_save_occupied(Engine& e, const double* d_C, int ldc, int nocc, cudaStream_t s);
int ri_check_flag(Engine& e);
int ri_absmax_diff(Engine& e, const double* d_A, const double* d_B, double* h_out, cudaStream_t s);
int ri_add_inplace(Engine& e, double* d_A, const double* d_B, cudaStream_t s);

}  // namespace gb
