// DIIS coefficients from the error-overlap matrix B_ij = <e_i, e_j>, one thread.
//
// The extrapolation weights minimise |sum_i c_i e_i|^2 subject to sum_i c_i = 1
// (the reference solves the bordered system [B -1; -1 0] c = [0 .. 0 -1] by LU,
// src/gpu_manager.cu:1078-1194).  Here the same minimiser is computed so that a
// rank-deficient B gives a defined answer:
//   * B is equilibrated to unit diagonal, A_ij = B_ij / (d_i d_j), d_i = |e_i|;
//     in y = d c the problem is min y^T A y subject to w^T y = 1, w_i = 1 / d_i;
//   * a pivoted Cholesky factorisation of A picks, largest remaining Schur
//     diagonal first (ties: lowest index), the vectors that are independent to
//     within an angle of ~1e-6 rad (Schur diagonal >= kDiisRankTol); the others
//     get weight 0, so two equal error vectors count once;
//   * on the kept set, y = A^{-1} w / (w^T A^{-1} w), c_i = y_i / d_i.
// On a B of full rank this is the reference's solution (the minimiser is
// unique).  An exactly zero error vector means its Fock matrix is already
// self-consistent: it gets weight 1 (the lowest such index).
// Returns the number of vectors given weight 0 because they depend on others.
#pragma once

namespace gb {

constexpr double kDiisRankTol = 1e-12;

template <int MAXM>
__device__ inline int diis_coefficients(const double* __restrict__ B, int ldb, int m, double* __restrict__ coef)
{
    double d[MAXM];
    for (int i = 0; i < m; ++i) {
        const double b = B[i * ldb + i];
        d[i] = b > 0.0 ? sqrt(b) : 0.0;
    }
    for (int i = 0; i < m; ++i)
        if (d[i] == 0.0) {
            for (int k = 0; k < m; ++k) coef[k] = (k == i) ? 1.0 : 0.0;
            return 0;
        }
    // L (row p = p-th pivot) over the equilibrated matrix, pivoted Cholesky
    double L[MAXM][MAXM];
    double schur[MAXM];
    int perm[MAXM];
    for (int i = 0; i < m; ++i) { schur[i] = 1.0; perm[i] = i; }
    int r = 0;
    for (; r < m; ++r) {
        int best = r;
        for (int q = r + 1; q < m; ++q)
            if (schur[perm[q]] > schur[perm[best]]) best = q;
        if (!(schur[perm[best]] >= kDiisRankTol)) break;
        const int t = perm[r]; perm[r] = perm[best]; perm[best] = t;
        for (int k = 0; k < r; ++k) { const double u = L[r][k]; L[r][k] = L[best][k]; L[best][k] = u; }
        const int p = perm[r];
        const double lrr = sqrt(schur[p]);
        L[r][r] = lrr;
        for (int q = r + 1; q < m; ++q) {
            const int j = perm[q];
            double a = B[p * ldb + j] / (d[p] * d[j]);
            for (int k = 0; k < r; ++k) a -= L[r][k] * L[q][k];
            L[q][r] = a / lrr;
            schur[j] -= L[q][r] * L[q][r];
        }
    }
    // z = A_kept^{-1} w_kept by two triangular solves (kept = perm[0..r))
    double z[MAXM];
    for (int i = 0; i < r; ++i) {
        double s = 1.0 / d[perm[i]];
        for (int k = 0; k < i; ++k) s -= L[i][k] * z[k];
        z[i] = s / L[i][i];
    }
    for (int i = r - 1; i >= 0; --i) {
        double s = z[i];
        for (int k = i + 1; k < r; ++k) s -= L[k][i] * z[k];
        z[i] = s / L[i][i];
    }
    double wz = 0.0;
    for (int i = 0; i < r; ++i) wz += z[i] / d[perm[i]];
    for (int k = 0; k < m; ++k) coef[k] = 0.0;
    for (int i = 0; i < r; ++i) coef[perm[i]] = z[i] / (wz * d[perm[i]]);
    return m - r;
}

}  // namespace gb
