/*
 * CPU FP64 oracle: a plain-C restatement of the reference's McMurchie-Davidson
 * integral arithmetic, used ONLY as test infrastructure (the parity checker in
 * tests/, the CPU leg of bench.py and the reference arm).  The product never
 * links or calls this file.
 *
 * Parity is pinned two ways:
 *   - against the reference's own integral kernels compiled for the CPU from
 *     their sources (oracle/refcpu/, built into oracle/_ref/), element by
 *     element for S, H, the primitive Schwarz bounds and the full ERI tensor;
 *   - against the reference's own linear-algebra known answers
 *     (test/test_gpu_manager.cu) for the SCF pieces in oracle/oracle.py.
 *
 * What it restates (reference file:line):
 *   Boys function F_n(x) = int_0^1 t^{2n} exp(-x t^2) dt      include/boys.hpp:32-182
 *     (here: series + downward recursion / erf + upward recursion, long double)
 *   Hermite expansion E^{ij}_t with E^{00}_0 = exp(-ab/p X_AB^2)
 *                                                              include/Et_functions.hpp:3000
 *   Hermite Coulomb R^{n}_{tuv} recursion, R^n_000=(-2xi)^n F_n  src/int2e.cu:1842-1893
 *   ERI prefactor 2 pi^{5/2}/(pq sqrt(p+q)), ket sign (-1)^{tau+nu+phi}
 *                                                              src/int2e.cu:1920-1922
 *   primitive norm calcNorm(a,l,m,n)                           include/int2e.hpp:127-130
 *   CGTO factor (with the integer-division quirk for odd L)    include/basis_set.hpp:106-137
 *   primitive-pair Schwarz bound sqrt(max_comp (ab|ab))        src/schwarz.txt:239-470
 *   screening of a primitive quartet by Q_ab*Q_cd < thr        src/int2e.cu:1677-1680
 *   Fock F_ij = H_ij + sum_kl D_kl[(ij|kl) - 1/2 (ik|jl)]      src/gpu_kernels.cu:230-287
 *   S, T (kinetic) and V (nuclear attraction) matrices         src/gpu_manager.cu:333-404
 *   RI: auxiliary functions are contracted shells of their own basis file,
 *     normalised like orbital shells; (mu nu|P) and (P|Q) are four-centre
 *     integrals with an exponent-0 unit s function as partner
 *                                                              src/int3c2e.cu:1102-1330,
 *                                                              src/int2c2e.cu:468-690
 *     auxiliary Cartesian order loop_to_ang_RI (f differs)     include/int2c2e.hpp:39-47
 *     auxiliary primitive bound sqrt(max_comp g_P^2 N^2 c^2 (P|P)), with the
 *     auxiliary CGTO factor                                    src/schwarz.txt:480-682
 *     screening Q_ab*Q_P < thr (3c) and Q_P*Q_Q < thr (2c)     src/int3c2e.cu, src/int2c2e.cu
 *     (P|mu nu) written to both (mu,nu) and (nu,mu)            include/int3c2e.hpp:150-154
 *
 * Cartesian component order within a shell follows include/types.hpp:197-228.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_LMAX 4              /* up to g shells */
#define OR_NMAX (4 * OR_LMAX + 2)
#define OR_PI 3.14159265358979323846264338327950288

/* Cartesian exponents in the reference order (include/types.hpp:197-228). */
static const int or_cart[OR_LMAX + 1][15][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
    {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {1, 2, 0}, {2, 1, 0}, {2, 0, 1}, {1, 0, 2}, {0, 1, 2}, {0, 2, 1}, {1, 1, 1}},
    {{4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1}, {1, 0, 3}, {0, 1, 3},
     {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}}};

static int or_ncart(int l) { return (l + 1) * (l + 2) / 2; }

static double or_dfact(int n) /* (n)!! with (-1)!! = 1 */
{
    double r = 1.0;
    for (int k = n; k > 1; k -= 2) r *= k;
    return r;
}

/* ------------------------------------------------------------------ Boys */
int oracle_boys(int nmax, double x, double* out)
{
    if (nmax < 0 || nmax > 64) return -1;
    if (x < 1e-300) {
        for (int n = 0; n <= nmax; ++n) out[n] = 1.0 / (2 * n + 1);
        return 0;
    }
    if (x < 40.0) {
        /* F_N(x) = exp(-x) sum_k (2x)^k / ((2N+1)(2N+3)...(2N+2k+1)) */
        long double X = x, ex = expl(-X);
        long double term = 1.0L / (2 * nmax + 1), sum = term;
        for (int k = 1; k < 2000; ++k) {
            term *= 2.0L * X / (2 * nmax + 2 * k + 1);
            sum += term;
            if (term < 1e-22L * sum) break;
        }
        long double f = ex * sum;
        out[nmax] = (double)f;
        for (int n = nmax; n > 0; --n) { /* stable downward recursion */
            f = (2.0L * X * f + ex) / (2 * n - 1);
            out[n - 1] = (double)f;
        }
        return 0;
    }
    long double X = x, ex = expl(-X);
    long double f = 0.5L * sqrtl(OR_PI / X) * erfl(sqrtl(X));
    out[0] = (double)f;
    for (int n = 0; n < nmax; ++n) { /* upward recursion, stable for large x */
        f = ((2 * n + 1) * f - ex) / (2.0L * X);
        out[n + 1] = (double)f;
    }
    return 0;
}

/* ------------------------------------------------ Hermite E coefficients */
/* E[i][j][t] for one axis, i<=la, j<=lb (+extra), t<=i+j, scaled so that
 * E[0][0][0] = exp(-a b / p * XAB^2).  Standard MD recursion. */
#define OR_EDIM (OR_LMAX + 3)
typedef double or_etab[OR_EDIM][OR_EDIM][2 * OR_EDIM];

static void or_hermite_e(int la, int lb, double a, double b, double xab, or_etab E)
{
    const double p = a + b, mu = a * b / p;
    const double xpa = -b / p * xab, xpb = a / p * xab, oo2p = 0.5 / p;
    memset(E, 0, sizeof(or_etab));
    E[0][0][0] = exp(-mu * xab * xab);
    for (int i = 0; i <= la; ++i) {
        for (int j = 0; j <= lb; ++j) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; ++t) {
                double v;
                if (i > 0) {
                    v = xpa * E[i - 1][j][t];
                    if (t > 0) v += oo2p * E[i - 1][j][t - 1];
                    if (t + 1 <= i - 1 + j) v += (t + 1) * E[i - 1][j][t + 1];
                } else {
                    v = xpb * E[i][j - 1][t];
                    if (t > 0) v += oo2p * E[i][j - 1][t - 1];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[i][j - 1][t + 1];
                }
                E[i][j][t] = v;
            }
        }
    }
}

/* -------------------------------------------------- Hermite Coulomb R */
#define OR_RDIM (OR_NMAX + 1)
/* R[t][u][v] = R^{0}_{tuv}(alpha, PQ) for t+u+v <= L */
static void or_hermite_r(int L, double alpha, double px, double py, double pz, double* R /* RDIM^3 */)
{
    static const int D = OR_RDIM;
    double F[OR_NMAX + 2];
    double r2 = px * px + py * py + pz * pz;
    oracle_boys(L, alpha * r2, F);
    /* Rn[n][t][u][v] */
    double* Rn = (double*)calloc((size_t)(L + 1) * D * D * D, sizeof(double));
#define RN(n, t, u, v) Rn[(((size_t)(n) * D + (t)) * D + (u)) * D + (v)]
    double fac = 1.0;
    for (int n = 0; n <= L; ++n) { RN(n, 0, 0, 0) = fac * F[n]; fac *= -2.0 * alpha; }
    for (int n = L - 1; n >= 0; --n) {
        int top = L - n;
        for (int t = 0; t <= top; ++t)
            for (int u = 0; u + t <= top; ++u)
                for (int v = 0; v + u + t <= top; ++v) {
                    if (t + u + v == 0) continue;
                    double val;
                    if (t > 0) {
                        val = px * RN(n + 1, t - 1, u, v);
                        if (t > 1) val += (t - 1) * RN(n + 1, t - 2, u, v);
                    } else if (u > 0) {
                        val = py * RN(n + 1, t, u - 1, v);
                        if (u > 1) val += (u - 1) * RN(n + 1, t, u - 2, v);
                    } else {
                        val = pz * RN(n + 1, t, u, v - 1);
                        if (v > 1) val += (v - 1) * RN(n + 1, t, u, v - 2);
                    }
                    RN(n, t, u, v) = val;
                }
    }
    for (int t = 0; t <= L; ++t)
        for (int u = 0; u + t <= L; ++u)
            for (int v = 0; v + u + t <= L; ++v) R[(t * D + u) * D + v] = RN(0, t, u, v);
#undef RN
    free(Rn);
}

/* ----------------------------------------------------------- basis data */
typedef struct {
    int nshell;
    const int* l;          /* angular momentum per shell */
    const int* nprim;      /* primitives per shell */
    const int* prim_off;   /* offset into alpha/coef */
    const int* bf_off;     /* first basis function */
    const double* xyz;     /* 3*nshell centre */
    const double* alpha;   /* exponents */
    const double* coef;    /* raw contraction coefficients */
    const double* cgto;    /* per basis function CGTO factor */
    int nbf;
} or_basis;

/* reference calcNorm: 2^L / sqrt((2l-1)!!(2m-1)!!(2n-1)!!) (2/pi)^{3/4} a^{(2L+3)/4} */
/* Cartesian order of auxiliary shells (include/int2c2e.hpp:39-47): the same
 * as or_cart except for f. */
static const int or_cart_ri[OR_LMAX + 1][15][3] = {
    {{0, 0, 0}},
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
    {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
    {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {0, 2, 1}, {1, 2, 0}, {0, 1, 2}, {1, 0, 2}, {1, 1, 1}},
    {{4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {0, 3, 1}, {1, 3, 0}, {0, 1, 3}, {1, 0, 3},
     {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}}};

/* Normalisation of a primitive Cartesian; an exponent of exactly 0 marks the
 * unit s function that turns a four-centre integral into a 3c/2c one. */
static double or_prim_norm(double a, int l, int m, int n)
{
    if (a == 0.0) return 1.0;
    int L = l + m + n;
    return pow(2.0, L) / sqrt(or_dfact(2 * l - 1) * or_dfact(2 * m - 1) * or_dfact(2 * n - 1)) *
           pow(2.0 / OR_PI, 0.75) * pow(a, (2.0 * L + 3.0) / 4.0);
}

/* CGTO factor of one contracted shell, reference convention including the
 * integer division L/2 in the second primitive's exponent (basis_set.hpp:123). */
double oracle_cgto_factor(int L, int nprim, const double* alpha, const double* coef)
{
    double s = 0.0;
    for (int i = 0; i < nprim; ++i) {
        double na = pow(2.0 * OR_PI, -0.75) * pow(4.0 * alpha[i], L / 2.0 + 0.75);
        for (int j = 0; j < nprim; ++j) {
            double nb = pow(2.0 * OR_PI, -0.75) * pow(4.0 * alpha[j], (double)(L / 2) + 0.75);
            s += coef[i] * na * coef[j] * nb / pow(2.0 * (alpha[i] + alpha[j]), L + 1.5);
        }
    }
    s *= pow(2.0 * OR_PI, 1.5);
    return pow(s, -0.5);
}

/* Primitive quartet integrals over normalised primitive Cartesians (prim
 * norms included, coefficients and CGTO factors not), out[a][b][c][d]. */
typedef const int (*or_order)[15][3];

static void or_prim_quartet_o(int la, int lb, int lc, int ld,
                              double a, double b, double c, double d,
                              const double* A, const double* B, const double* C, const double* D,
                              or_order oa, or_order ob, or_order oc, or_order od, double* out)
{
    const int RD = OR_RDIM;
    const double p = a + b, q = c + d, alpha = p * q / (p + q);
    double P[3], Q[3];
    for (int k = 0; k < 3; ++k) { P[k] = (a * A[k] + b * B[k]) / p; Q[k] = (c * C[k] + d * D[k]) / q; }
    static or_etab Eab[3], Ecd[3];
#pragma omp threadprivate(Eab, Ecd)
    for (int k = 0; k < 3; ++k) {
        or_hermite_e(la, lb, a, b, A[k] - B[k], Eab[k]);
        or_hermite_e(lc, ld, c, d, C[k] - D[k], Ecd[k]);
    }
    int L = la + lb + lc + ld;
    double* R = (double*)malloc(sizeof(double) * RD * RD * RD);
    or_hermite_r(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], R);
    const double pref = 2.0 * pow(OR_PI, 2.5) / (p * q * sqrt(p + q));
    int na = or_ncart(la), nb = or_ncart(lb), nc = or_ncart(lc), nd = or_ncart(ld);
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib)
            for (int ic = 0; ic < nc; ++ic)
                for (int id = 0; id < nd; ++id) {
                    const int* ea = oa[la][ia]; const int* eb = ob[lb][ib];
                    const int* ec = oc[lc][ic]; const int* ed = od[ld][id];
                    double s = 0.0;
                    for (int t = 0; t <= ea[0] + eb[0]; ++t)
                        for (int u = 0; u <= ea[1] + eb[1]; ++u)
                            for (int v = 0; v <= ea[2] + eb[2]; ++v) {
                                double eab = Eab[0][ea[0]][eb[0]][t] * Eab[1][ea[1]][eb[1]][u] * Eab[2][ea[2]][eb[2]][v];
                                if (eab == 0.0) continue;
                                for (int tau = 0; tau <= ec[0] + ed[0]; ++tau)
                                    for (int nu = 0; nu <= ec[1] + ed[1]; ++nu)
                                        for (int phi = 0; phi <= ec[2] + ed[2]; ++phi) {
                                            double ecd = Ecd[0][ec[0]][ed[0]][tau] * Ecd[1][ec[1]][ed[1]][nu] *
                                                         Ecd[2][ec[2]][ed[2]][phi];
                                            double sg = ((tau + nu + phi) & 1) ? -1.0 : 1.0;
                                            s += eab * sg * ecd * R[((t + tau) * RD + (u + nu)) * RD + (v + phi)];
                                        }
                            }
                    double nrm = or_prim_norm(a, ea[0], ea[1], ea[2]) * or_prim_norm(b, eb[0], eb[1], eb[2]) *
                                 or_prim_norm(c, ec[0], ec[1], ec[2]) * or_prim_norm(d, ed[0], ed[1], ed[2]);
                    out[((ia * nb + ib) * nc + ic) * nd + id] = pref * s * nrm;
                }
    free(R);
}

static void or_prim_quartet(int la, int lb, int lc, int ld,
                            double a, double b, double c, double d,
                            const double* A, const double* B, const double* C, const double* D,
                            double* out)
{
    or_prim_quartet_o(la, lb, lc, ld, a, b, c, d, A, B, C, D, or_cart, or_cart, or_cart, or_cart, out);
}

/* Primitive-pair Schwarz bound, reference definition: sqrt(max over Cartesian
 * component pairs of c_a^2 c_b^2 (ab|ab)), no CGTO factors. */
static double or_prim_pair_bound(int la, int lb, double a, double b, double ca, double cb,
                                 const double* A, const double* B)
{
    int na = or_ncart(la), nb = or_ncart(lb);
    double* buf = (double*)malloc(sizeof(double) * na * nb * na * nb);
    or_prim_quartet(la, lb, la, lb, a, b, a, b, A, B, A, B, buf);
    double mx = 0.0;
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib) {
            double v = fabs(buf[((ia * nb + ib) * na + ia) * nb + ib]) * ca * ca * cb * cb;
            if (v > mx) mx = v;
        }
    free(buf);
    return sqrt(mx);
}

static void or_make_basis(or_basis* bs, int nshell, const int* l, const int* nprim, const int* prim_off,
                          const int* bf_off, const double* xyz, const double* alpha, const double* coef,
                          const double* cgto, int nbf)
{
    bs->nshell = nshell; bs->l = l; bs->nprim = nprim; bs->prim_off = prim_off; bs->bf_off = bf_off;
    bs->xyz = xyz; bs->alpha = alpha; bs->coef = coef; bs->cgto = cgto; bs->nbf = nbf;
}

/* Contracted shell quartet block (with coefficients and CGTO factors) under
 * the reference's primitive screening; returns number of primitive quartets kept. */
static long or_shell_quartet(const or_basis* bs, const double* Qp, const int* qp_off,
                             int A, int B, int C, int D, double thr, double* blk)
{
    int la = bs->l[A], lb = bs->l[B], lc = bs->l[C], ld = bs->l[D];
    int na = or_ncart(la), nb = or_ncart(lb), nc = or_ncart(lc), nd = or_ncart(ld);
    int n = na * nb * nc * nd;
    double* tmp = (double*)malloc(sizeof(double) * n);
    memset(blk, 0, sizeof(double) * n);
    long kept = 0;
    for (int i = 0; i < bs->nprim[A]; ++i)
        for (int j = 0; j < bs->nprim[B]; ++j) {
            double qab = Qp ? Qp[qp_off[A * bs->nshell + B] + i * bs->nprim[B] + j] : 1.0;
            for (int k = 0; k < bs->nprim[C]; ++k)
                for (int m = 0; m < bs->nprim[D]; ++m) {
                    double qcd = Qp ? Qp[qp_off[C * bs->nshell + D] + k * bs->nprim[D] + m] : 1.0;
                    if (Qp && qab * qcd < thr) continue;
                    ++kept;
                    int pa = bs->prim_off[A] + i, pb = bs->prim_off[B] + j;
                    int pc = bs->prim_off[C] + k, pd = bs->prim_off[D] + m;
                    or_prim_quartet(la, lb, lc, ld, bs->alpha[pa], bs->alpha[pb], bs->alpha[pc], bs->alpha[pd],
                                    &bs->xyz[3 * A], &bs->xyz[3 * B], &bs->xyz[3 * C], &bs->xyz[3 * D], tmp);
                    double cf = bs->coef[pa] * bs->coef[pb] * bs->coef[pc] * bs->coef[pd];
                    for (int e = 0; e < n; ++e) blk[e] += cf * tmp[e];
                }
        }
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib)
            for (int ic = 0; ic < nc; ++ic)
                for (int id = 0; id < nd; ++id)
                    blk[((ia * nb + ib) * nc + ic) * nd + id] *=
                        bs->cgto[bs->bf_off[A] + ia] * bs->cgto[bs->bf_off[B] + ib] *
                        bs->cgto[bs->bf_off[C] + ic] * bs->cgto[bs->bf_off[D] + id];
    free(tmp);
    return kept;
}

/* All primitive-pair bounds, laid out per ordered shell pair (A,B):
 * Qp[qp_off[A*nshell+B] + i*nprim[B] + j]. */
static double* or_all_bounds(const or_basis* bs, int** qp_off_out)
{
    int ns = bs->nshell;
    int* off = (int*)malloc(sizeof(int) * ns * ns);
    long tot = 0;
    for (int A = 0; A < ns; ++A)
        for (int B = 0; B < ns; ++B) { off[A * ns + B] = (int)tot; tot += bs->nprim[A] * bs->nprim[B]; }
    double* Q = (double*)malloc(sizeof(double) * (tot > 0 ? tot : 1));
#pragma omp parallel for schedule(dynamic)
    for (int AB = 0; AB < ns * ns; ++AB) {
        int A = AB / ns, B = AB % ns;
        for (int i = 0; i < bs->nprim[A]; ++i)
            for (int j = 0; j < bs->nprim[B]; ++j) {
                int pa = bs->prim_off[A] + i, pb = bs->prim_off[B] + j;
                Q[off[AB] + i * bs->nprim[B] + j] =
                    or_prim_pair_bound(bs->l[A], bs->l[B], bs->alpha[pa], bs->alpha[pb], bs->coef[pa],
                                       bs->coef[pb], &bs->xyz[3 * A], &bs->xyz[3 * B]);
            }
    }
    *qp_off_out = off;
    return Q;
}

/* Primitive-pair Schwarz bounds for each ordered primitive pair (pa, pb) of the
 * global primitive list, out[pa*nprim_total + pb]. */
int oracle_prim_pair_bounds(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                            const double* xyz, const double* alpha, const double* coef, const double* cgto,
                            int nbf, int nprim_total, double* out)
{
    or_basis bs;
    or_make_basis(&bs, nshell, l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, nbf);
    int* off;
    double* Q = or_all_bounds(&bs, &off);
    for (int A = 0; A < nshell; ++A)
        for (int B = 0; B < nshell; ++B)
            for (int i = 0; i < nprim[A]; ++i)
                for (int j = 0; j < nprim[B]; ++j)
                    out[(size_t)(prim_off[A] + i) * nprim_total + prim_off[B] + j] =
                        Q[off[A * nshell + B] + i * nprim[B] + j];
    free(Q); free(off);
    return 0;
}

/* Full N^4 ERI tensor (row-major ((i*N+j)*N+k)*N+l), primitive-screened. */
int oracle_eri_tensor(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                      const double* xyz, const double* alpha, const double* coef, const double* cgto, int nbf,
                      double thr, double* eri)
{
    or_basis bs;
    or_make_basis(&bs, nshell, l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, nbf);
    int* off = NULL;
    double* Q = thr > 0 ? or_all_bounds(&bs, &off) : NULL;
    const size_t N = (size_t)nbf;
    memset(eri, 0, sizeof(double) * N * N * N * N);
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int A = 0; A < nshell; ++A)
        for (int B = 0; B < nshell; ++B) {
            double blk[15 * 15 * 15 * 15];
            for (int C = 0; C < nshell; ++C)
                for (int D = 0; D < nshell; ++D) {
                    or_shell_quartet(&bs, Q, off, A, B, C, D, thr, blk);
                    int na = or_ncart(l[A]), nb = or_ncart(l[B]), nc = or_ncart(l[C]), nd = or_ncart(l[D]);
                    for (int ia = 0; ia < na; ++ia)
                        for (int ib = 0; ib < nb; ++ib)
                            for (int ic = 0; ic < nc; ++ic)
                                for (int id = 0; id < nd; ++id) {
                                    size_t i = bf_off[A] + ia, j = bf_off[B] + ib, k = bf_off[C] + ic, m = bf_off[D] + id;
                                    eri[((i * N + j) * N + k) * N + m] = blk[((ia * nb + ib) * nc + ic) * nd + id];
                                }
                }
        }
    free(Q); free(off);
    return 0;
}

/* Direct J and K: J_ij = sum_kl D_kl (ij|kl), K_ij = sum_kl D_kl (ik|jl), over
 * unique shell quartets with 8-fold symmetry, primitive screening at thr.
 * Returns the number of primitive quartets evaluated (unique quartets). */
long oracle_direct_jk_sample(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                             const double* xyz, const double* alpha, const double* coef, const double* cgto, int nbf,
                             double thr, const double* Dm, double* J, double* K, int nthreads, int bra_stride);

long oracle_direct_jk(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                      const double* xyz, const double* alpha, const double* coef, const double* cgto, int nbf,
                      double thr, const double* Dm, double* J, double* K, int nthreads)
{
    return oracle_direct_jk_sample(nshell, l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, nbf, thr, Dm, J, K,
                                   nthreads, 1);
}

/* Same as oracle_direct_jk over the bra pairs ij with ij % bra_stride == 0
 * only: a bounded sample of the work for CPU timing (J, K then incomplete). */
long oracle_direct_jk_sample(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                             const double* xyz, const double* alpha, const double* coef, const double* cgto, int nbf,
                             double thr, const double* Dm, double* J, double* K, int nthreads, int bra_stride)
{
    or_basis bs;
    or_make_basis(&bs, nshell, l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, nbf);
    int* off = NULL;
    double* Q = or_all_bounds(&bs, &off);
    const int N = nbf;
    long total_kept = 0;
    int npair = nshell * (nshell + 1) / 2;
    int* pa = (int*)malloc(sizeof(int) * npair);
    int* pb = (int*)malloc(sizeof(int) * npair);
    for (int A = 0, k = 0; A < nshell; ++A)
        for (int B = 0; B <= A; ++B, ++k) { pa[k] = A; pb[k] = B; }
    /* contracted-pair max primitive bound for a cheap exact pre-skip */
    double* qmax = (double*)calloc(npair, sizeof(double));
    for (int k = 0; k < npair; ++k) {
        int A = pa[k], B = pb[k];
        for (int i = 0; i < nprim[A] * nprim[B]; ++i)
            if (Q[off[A * nshell + B] + i] > qmax[k]) qmax[k] = Q[off[A * nshell + B] + i];
    }
    memset(J, 0, sizeof(double) * N * N);
    memset(K, 0, sizeof(double) * N * N);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : total_kept)
    {
        double* Jt = (double*)calloc((size_t)N * N, sizeof(double));
        double* Kt = (double*)calloc((size_t)N * N, sizeof(double));
        double* blk = (double*)malloc(sizeof(double) * 15 * 15 * 15 * 15);
#pragma omp for schedule(dynamic, 4)
        for (int ij = 0; ij < npair; ++ij) {
            if (bra_stride > 1 && ij % bra_stride) continue;
            for (int kl = 0; kl <= ij; ++kl) {
                if (qmax[ij] * qmax[kl] < thr) continue;
                int A = pa[ij], B = pb[ij], C = pa[kl], D = pb[kl];
                total_kept += or_shell_quartet(&bs, Q, off, A, B, C, D, thr, blk);
                double f = 1.0;
                if (A == B) f *= 0.5;
                if (C == D) f *= 0.5;
                if (ij == kl) f *= 0.5;
                int na = or_ncart(l[A]), nb = or_ncart(l[B]), nc = or_ncart(l[C]), nd = or_ncart(l[D]);
                for (int ia = 0; ia < na; ++ia)
                    for (int ib = 0; ib < nb; ++ib)
                        for (int ic = 0; ic < nc; ++ic)
                            for (int id = 0; id < nd; ++id) {
                                double v = f * blk[((ia * nb + ib) * nc + ic) * nd + id];
                                int a = bf_off[A] + ia, b = bf_off[B] + ib, c = bf_off[C] + ic, d = bf_off[D] + id;
                                Jt[a * N + b] += Dm[c * N + d] * v;
                                Jt[c * N + d] += Dm[a * N + b] * v;
                                Kt[a * N + c] += Dm[b * N + d] * v;
                                Kt[b * N + d] += Dm[a * N + c] * v;
                                Kt[a * N + d] += Dm[b * N + c] * v;
                                Kt[b * N + c] += Dm[a * N + d] * v;
                            }
            }
        }
#pragma omp critical
        {
            for (int i = 0; i < N; ++i)
                for (int j = 0; j < N; ++j) {
                    J[i * N + j] += 2.0 * (Jt[i * N + j] + Jt[j * N + i]);
                    K[i * N + j] += Kt[i * N + j] + Kt[j * N + i];
                }
        }
        free(Jt); free(Kt); free(blk);
    }
    free(Q); free(off); free(pa); free(pb); free(qmax);
    return total_kept;
}

/* ------------------------------------------------ one-electron integrals */
/* S, T and V (nuclear attraction, point charges Z) with CGTO factors. */
int oracle_one_electron(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                        const double* xyz, const double* alpha, const double* coef, const double* cgto, int nbf,
                        int natom, const double* atom_z, const double* atom_xyz, double* S, double* T, double* V)
{
    const int N = nbf, RD = OR_RDIM;
    memset(S, 0, sizeof(double) * N * N);
    memset(T, 0, sizeof(double) * N * N);
    memset(V, 0, sizeof(double) * N * N);
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int A = 0; A < nshell; ++A)
        for (int B = 0; B < nshell; ++B) {
            int la = l[A], lb = l[B], na = or_ncart(la), nb = or_ncart(lb);
            const double *PA = &xyz[3 * A], *PB = &xyz[3 * B];
            double* R = (double*)malloc(sizeof(double) * RD * RD * RD);
            or_etab E[3];
            for (int i = 0; i < nprim[A]; ++i)
                for (int j = 0; j < nprim[B]; ++j) {
                    int pa = prim_off[A] + i, pb = prim_off[B] + j;
                    double a = alpha[pa], b = alpha[pb], p = a + b;
                    double P[3];
                    for (int k = 0; k < 3; ++k) {
                        or_hermite_e(la, lb + 2, a, b, PA[k] - PB[k], E[k]);
                        P[k] = (a * PA[k] + b * PB[k]) / p;
                    }
                    double cf = coef[pa] * coef[pb];
                    double sp = sqrt(OR_PI / p);
                    for (int ia = 0; ia < na; ++ia)
                        for (int ib = 0; ib < nb; ++ib) {
                            const int* ea = or_cart[la][ia]; const int* eb = or_cart[lb][ib];
                            double s1[3], t1[3];
                            for (int k = 0; k < 3; ++k) {
                                int x = ea[k], y = eb[k];
                                s1[k] = E[k][x][y][0] * sp;
                                double tt = 4.0 * b * b * E[k][x][y + 2][0] - 2.0 * b * (2 * y + 1) * E[k][x][y][0];
                                if (y >= 2) tt += y * (y - 1) * E[k][x][y - 2][0];
                                t1[k] = -0.5 * tt * sp;
                            }
                            double nrm = or_prim_norm(a, ea[0], ea[1], ea[2]) * or_prim_norm(b, eb[0], eb[1], eb[2]) * cf *
                                         cgto[bf_off[A] + ia] * cgto[bf_off[B] + ib];
                            size_t idx = (size_t)(bf_off[A] + ia) * N + bf_off[B] + ib;
                            S[idx] += nrm * s1[0] * s1[1] * s1[2];
                            T[idx] += nrm * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
                        }
                    for (int c = 0; c < natom; ++c) {
                        const double* Cc = &atom_xyz[3 * c];
                        or_hermite_r(la + lb, p, P[0] - Cc[0], P[1] - Cc[1], P[2] - Cc[2], R);
                        for (int ia = 0; ia < na; ++ia)
                            for (int ib = 0; ib < nb; ++ib) {
                                const int* ea = or_cart[la][ia]; const int* eb = or_cart[lb][ib];
                                double s = 0.0;
                                for (int t = 0; t <= ea[0] + eb[0]; ++t)
                                    for (int u = 0; u <= ea[1] + eb[1]; ++u)
                                        for (int v = 0; v <= ea[2] + eb[2]; ++v)
                                            s += E[0][ea[0]][eb[0]][t] * E[1][ea[1]][eb[1]][u] * E[2][ea[2]][eb[2]][v] *
                                                 R[(t * RD + u) * RD + v];
                                double nrm = or_prim_norm(a, ea[0], ea[1], ea[2]) * or_prim_norm(b, eb[0], eb[1], eb[2]) *
                                             cf * cgto[bf_off[A] + ia] * cgto[bf_off[B] + ib];
                                V[(size_t)(bf_off[A] + ia) * N + bf_off[B] + ib] += -atom_z[c] * 2.0 * OR_PI / p * s * nrm;
                            }
                    }
                }
            free(R);
        }
    return 0;
}

/* ------------------------------------------------------------------ RI */

/* Auxiliary primitive bounds (src/schwarz.txt:480-682), one per auxiliary
 * primitive in the order of the auxiliary primitive list. */
static void or_aux_bounds(const or_basis* ax, double* out)
{
    for (int P = 0; P < ax->nshell; ++P) {
        const int lp = ax->l[P], np = or_ncart(lp);
        double buf[15 * 15];
        for (int i = 0; i < ax->nprim[P]; ++i) {
            const int pi = ax->prim_off[P] + i;
            const double g = ax->alpha[pi], c = ax->coef[pi];
            or_prim_quartet_o(lp, 0, lp, 0, g, 0.0, g, 0.0, &ax->xyz[3 * P], &ax->xyz[3 * P], &ax->xyz[3 * P],
                              &ax->xyz[3 * P], or_cart_ri, or_cart, or_cart_ri, or_cart, buf);
            double mx = 0.0;
            for (int k = 0; k < np; ++k) {
                const double f = ax->cgto[ax->bf_off[P] + k];
                const double v = f * f * c * c * buf[k * np + k];
                if (fabs(v) > fabs(mx)) mx = v;
            }
            out[pi] = sqrt(mx);
        }
    }
}

/* RI metric V[P*naux+Q] = (P|Q) and three-centre T[(P*nbf+mu)*nbf+nu] = (mu nu|P)
 * with the reference's primitive screening; aux_bounds (may be NULL) receives
 * the auxiliary primitive bounds. */
int oracle_ri_integrals(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                        const double* xyz, const double* alpha, const double* coef, const double* cgto, int nbf,
                        int ashell, const int* al, const int* anprim, const int* aprim_off, const int* abf_off,
                        const double* axyz, const double* aalpha, const double* acoef, const double* acgto,
                        int naux, double thr, double* V, double* T, double* aux_bounds)
{
    or_basis bs, ax;
    or_make_basis(&bs, nshell, l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, nbf);
    or_make_basis(&ax, ashell, al, anprim, aprim_off, abf_off, axyz, aalpha, acoef, acgto, naux);
    int naprim = 0;
    for (int P = 0; P < ashell; ++P) naprim += anprim[P];
    double* QP = (double*)malloc(sizeof(double) * (naprim > 0 ? naprim : 1));
    or_aux_bounds(&ax, QP);
    if (aux_bounds) memcpy(aux_bounds, QP, sizeof(double) * naprim);
    int* off;
    double* Q = or_all_bounds(&bs, &off);
    const size_t N = (size_t)nbf, M = (size_t)naux;
    if (V) {
        memset(V, 0, sizeof(double) * M * M);
#pragma omp parallel for collapse(2) schedule(dynamic)
        for (int P = 0; P < ashell; ++P)
            for (int R = 0; R < ashell; ++R) {
                const int lp = al[P], lr = al[R], np = or_ncart(lp), nr = or_ncart(lr);
                double blk[15 * 15], tmp[15 * 15];
                memset(blk, 0, sizeof(blk));
                for (int i = 0; i < anprim[P]; ++i)
                    for (int k = 0; k < anprim[R]; ++k) {
                        const int pi = aprim_off[P] + i, pk = aprim_off[R] + k;
                        if (QP[pi] * QP[pk] < thr) continue;
                        or_prim_quartet_o(lp, 0, lr, 0, aalpha[pi], 0.0, aalpha[pk], 0.0, &axyz[3 * P], &axyz[3 * P],
                                          &axyz[3 * R], &axyz[3 * R], or_cart_ri, or_cart, or_cart_ri, or_cart, tmp);
                        for (int e = 0; e < np * nr; ++e) blk[e] += acoef[pi] * acoef[pk] * tmp[e];
                    }
                for (int ip = 0; ip < np; ++ip)
                    for (int ir = 0; ir < nr; ++ir)
                        V[(size_t)(abf_off[P] + ip) * M + abf_off[R] + ir] =
                            blk[ip * nr + ir] * acgto[abf_off[P] + ip] * acgto[abf_off[R] + ir];
            }
    }
    if (T) {
        memset(T, 0, sizeof(double) * M * N * N);
#pragma omp parallel for collapse(2) schedule(dynamic)
        for (int A = 0; A < nshell; ++A)
            for (int B = 0; B < nshell; ++B) {
                const int la = l[A], lb = l[B], na = or_ncart(la), nb = or_ncart(lb);
                double blk[15 * 15 * 15], tmp[15 * 15 * 15];
                for (int P = 0; P < ashell; ++P) {
                    const int lp = al[P], np = or_ncart(lp);
                    memset(blk, 0, sizeof(double) * na * nb * np);
                    for (int i = 0; i < nprim[A]; ++i)
                        for (int j = 0; j < nprim[B]; ++j) {
                            const int pa = prim_off[A] + i, pb = prim_off[B] + j;
                            const double qab = Q[off[A * nshell + B] + i * nprim[B] + j];
                            for (int k = 0; k < anprim[P]; ++k) {
                                const int pk = aprim_off[P] + k;
                                if (qab * QP[pk] < thr) continue;
                                or_prim_quartet_o(la, lb, lp, 0, alpha[pa], alpha[pb], aalpha[pk], 0.0, &xyz[3 * A],
                                                  &xyz[3 * B], &axyz[3 * P], &axyz[3 * P], or_cart, or_cart, or_cart_ri,
                                                  or_cart, tmp);
                                const double cf = coef[pa] * coef[pb] * acoef[pk];
                                for (int e = 0; e < na * nb * np; ++e) blk[e] += cf * tmp[e];
                            }
                        }
                    for (int ia = 0; ia < na; ++ia)
                        for (int ib = 0; ib < nb; ++ib)
                            for (int ip = 0; ip < np; ++ip) {
                                const size_t mu = bf_off[A] + ia, nu = bf_off[B] + ib, r = abf_off[P] + ip;
                                T[(r * N + mu) * N + nu] =
                                    blk[(ia * nb + ib) * np + ip] * cgto[mu] * cgto[nu] * acgto[r];
                            }
                }
            }
    }
    free(QP); free(Q); free(off);
    return 0;
}

/* Three-centre integrals (mu nu|P) of selected AO shell pairs only (checks of the
 * B tensor at sizes where the full naux x N^2 tensor is too large for the CPU):
 * T[((k * ncart_max^2) + ia * nb + ib) * naux + r] for the k-th pair (pairA[k],
 * pairB[k]), ncart_max = 15; same screening and factors as oracle_ri_integrals. */
int oracle_ri_three_center_pairs(int nshell, const int* l, const int* nprim, const int* prim_off, const int* bf_off,
                                 const double* xyz, const double* alpha, const double* coef, const double* cgto,
                                 int nbf, int ashell, const int* al, const int* anprim, const int* aprim_off,
                                 const int* abf_off, const double* axyz, const double* aalpha, const double* acoef,
                                 const double* acgto, int naux, double thr, int npairs, const int* pairA,
                                 const int* pairB, double* T)
{
    or_basis bs, ax;
    or_make_basis(&bs, nshell, l, nprim, prim_off, bf_off, xyz, alpha, coef, cgto, nbf);
    or_make_basis(&ax, ashell, al, anprim, aprim_off, abf_off, axyz, aalpha, acoef, acgto, naux);
    int naprim = 0;
    for (int P = 0; P < ashell; ++P) naprim += anprim[P];
    double* QP = (double*)malloc(sizeof(double) * (naprim > 0 ? naprim : 1));
    or_aux_bounds(&ax, QP);
    int* off;
    double* Q = or_all_bounds(&bs, &off);
    const size_t M = (size_t)naux;
    memset(T, 0, sizeof(double) * (size_t)npairs * 225 * M);
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int k = 0; k < npairs; ++k)
        for (int P = 0; P < ashell; ++P) {
            const int A = pairA[k], B = pairB[k];
            const int la = l[A], lb = l[B], na = or_ncart(la), nb = or_ncart(lb);
            const int lp = al[P], np = or_ncart(lp);
            double blk[15 * 15 * 15], tmp[15 * 15 * 15];
            memset(blk, 0, sizeof(double) * na * nb * np);
            for (int i = 0; i < nprim[A]; ++i)
                for (int j = 0; j < nprim[B]; ++j) {
                    const int pa = prim_off[A] + i, pb = prim_off[B] + j;
                    const double qab = Q[off[A * nshell + B] + i * nprim[B] + j];
                    for (int q = 0; q < anprim[P]; ++q) {
                        const int pk = aprim_off[P] + q;
                        if (qab * QP[pk] < thr) continue;
                        or_prim_quartet_o(la, lb, lp, 0, alpha[pa], alpha[pb], aalpha[pk], 0.0, &xyz[3 * A],
                                          &xyz[3 * B], &axyz[3 * P], &axyz[3 * P], or_cart, or_cart, or_cart_ri,
                                          or_cart, tmp);
                        const double cf = coef[pa] * coef[pb] * acoef[pk];
                        for (int e = 0; e < na * nb * np; ++e) blk[e] += cf * tmp[e];
                    }
                }
            for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib)
                    for (int ip = 0; ip < np; ++ip) {
                        const size_t mu = bf_off[A] + ia, nu = bf_off[B] + ib, r = abf_off[P] + ip;
                        T[((size_t)k * 225 + ia * nb + ib) * M + r] =
                            blk[(ia * nb + ib) * np + ip] * cgto[mu] * cgto[nu] * acgto[r];
                    }
        }
    free(QP); free(Q); free(off);
    return 0;
}
