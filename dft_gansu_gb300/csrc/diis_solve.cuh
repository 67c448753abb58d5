// DIIS coefficients from the error-overlap matrix B_ij = <e_i, e_j>, one thread.
//
// The extrapolation weights minimise |sum_i c_i e_i|^2 subject to sum_i c_i = 1
// (the reference solves the bordered system [B -1; -1 0] c = [0 .. 0 -1] by LU,
// src/gpu_manager.cu:1078-1194).  The bordered matrix is singular exactly when
// some c != 0 with sum_i c_i = 0 has B c = 0, i.e. when error vectors repeat
// (e_i = e_j): LU then has no answer.  Here the same minimiser is computed in a
// form that stays defined:
//   * anchor r = the error vector of smallest norm (ties: lowest index); with
//     c = e_r + sum_{i != r} z_i (u_i - u_r) (u = unit vectors) the constraint
//     holds for any z, and |E c|^2 is a least-squares problem in z with normal
//     equations G z = -g, G_ij = <e_i - e_r, e_j - e_r>, g_i = <e_i - e_r, e_r>;
//   * G is factorised by Cholesky with diagonal pivoting (largest remaining
//     Schur diagonal relative to max(|e_i|^2, |e_r|^2) first, ties: lowest
//     index); directions whose relative Schur diagonal falls below
//     kDiisRankTol (an error vector within ~1e-7 of a combination of the
//     others) get z_i = 0, so a repeated error vector counts once;
//   * c_i = z_i, c_r = 1 - sum_i z_i.
// On a nonsingular bordered system this is the reference's solution (the
// minimiser is unique).  Parallel error vectors of different length are not
// dependent in this sense: their combination that cancels the error is kept,
// as LU keeps it.  An exactly zero error vector means its Fock matrix is
// already self-consistent: it gets weight 1.
// Returns the number of vectors left out as dependent on the others.
#pragma once

namespace gb {

constexpr double kDiisRankTol = 1e-14;

template <int MAXM>
__device__ inline int diis_coefficients(const double* __restrict__ B, int ldb, int m, double* __restrict__ coef)
{
    int r = 0;
    for (int i = 1; i < m; ++i)
        if (B[i * ldb + i] < B[r * ldb + r]) r = i;
    for (int k = 0; k < m; ++k) coef[k] = 0.0;
    const double brr = B[r * ldb + r];
    if (!(brr > 0.0)) {
        coef[r] = 1.0;
        return 0;
    }
    // unknowns: the directions u_i - u_r, i != r, in index order
    int idx[MAXM];
    int q = 0;
    for (int i = 0; i < m; ++i)
        if (i != r) idx[q++] = i;
    double G[MAXM][MAXM], g[MAXM], scale[MAXM], schur[MAXM];
    for (int a = 0; a < q; ++a) {
        const int i = idx[a];
        g[a] = B[i * ldb + r] - brr;
        scale[a] = fmax(B[i * ldb + i], brr);
        for (int b = 0; b < q; ++b) {
            const int j = idx[b];
            G[a][b] = B[i * ldb + j] - B[i * ldb + r] - B[r * ldb + j] + brr;
        }
        schur[a] = G[a][a];
    }
    // pivoted Cholesky G[perm, perm] = L L^T over the kept directions
    double L[MAXM][MAXM];
    int perm[MAXM];
    for (int a = 0; a < q; ++a) perm[a] = a;
    int kept = 0;
    for (; kept < q; ++kept) {
        int best = kept;
        for (int p = kept + 1; p < q; ++p)
            if (schur[perm[p]] / scale[perm[p]] > schur[perm[best]] / scale[perm[best]]) best = p;
        if (!(schur[perm[best]] / scale[perm[best]] >= kDiisRankTol)) break;
        const int t = perm[kept]; perm[kept] = perm[best]; perm[best] = t;
        for (int k = 0; k < kept; ++k) { const double u = L[kept][k]; L[kept][k] = L[best][k]; L[best][k] = u; }
        const int p = perm[kept];
        const double lkk = sqrt(schur[p]);
        L[kept][kept] = lkk;
        for (int s = kept + 1; s < q; ++s) {
            const int j = perm[s];
            double a = G[p][j];
            for (int k = 0; k < kept; ++k) a -= L[kept][k] * L[s][k];
            L[s][kept] = a / lkk;
            schur[j] -= L[s][kept] * L[s][kept];
        }
    }
    // L L^T z = -g on the kept directions
    double z[MAXM];
    for (int i = 0; i < kept; ++i) {
        double s = -g[perm[i]];
        for (int k = 0; k < i; ++k) s -= L[i][k] * z[k];
        z[i] = s / L[i][i];
    }
    for (int i = kept - 1; i >= 0; --i) {
        double s = z[i];
        for (int k = i + 1; k < kept; ++k) s -= L[k][i] * z[k];
        z[i] = s / L[i][i];
    }
    double zsum = 0.0;
    for (int i = 0; i < kept; ++i) {
        coef[idx[perm[i]]] = z[i];
        zsum += z[i];
    }
    coef[r] = 1.0 - zsum;
    return q - kept;
}

}  // namespace gb
