// Analytic RHF nuclear gradient (no counterpart in the reference, whose
// "geometry optimisation" is an energy-only coordinate search,
// include/builder.hpp:108-275).
//
//   dE/dR = sum D dH/dR - sum W dS/dR + sum_{unique quartets} f G_abcd d(ab|cd)/dR + dV_nn/dR
//   G_abcd = 4 D_ab D_cd - D_ac D_bd - D_ad D_bc            (8 permutations folded)
//   W      = 2 sum_occ eps_i C_i C_i^T                     (energy-weighted density)
//
// Derivatives of a Cartesian Gaussian with respect to its centre,
//   d/dA_x phi_a = 2 alpha phi_{a+1x} - a_x phi_{a-1x},
// turn every derivative integral into integrals of shifted angular momentum,
// evaluated with the same McMurchie-Davidson Hermite expansions as the Fock
// build (md_math.cuh); nothing is stored: Hermite intermediates are rebuilt
// for every primitive quartet.  The two-electron term differentiates the bra
// centres A, B and the ket centre C; D follows from translational invariance
// (dA + dB + dC + dD = 0).  One thread handles one ket component pair (c,d)
// of one contracted quartet (the quartet lists of the Fock build), so the
// density weights of a column fit in registers.
#include <algorithm>
#include <cmath>
#include <vector>

#include "grad_kernel.cuh"
#include "ri.hpp"

namespace gb {
namespace {


template <class T>
__device__ __forceinline__ void grad_e_table(int l1, int l2, T xpa, T xpb, T oo2p, T* e)
{
    e[0] = T(1);
    for (int i = 0; i <= l1; ++i)
        for (int j = 0; j <= l2; ++j) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; ++t) {
                T v;
                if (i > 0) {
                    v = (t <= i - 1 + j) ? xpa * e[((i - 1) * kGI + j) * kGT + t] : T(0);
                    if (t > 0) v += oo2p * e[((i - 1) * kGI + j) * kGT + t - 1];
                    if (t + 1 <= i - 1 + j) v += (t + 1) * e[((i - 1) * kGI + j) * kGT + t + 1];
                } else {
                    v = (t <= j - 1) ? xpb * e[(j - 1) * kGT + t] : T(0);
                    if (t > 0) v += oo2p * e[(j - 1) * kGT + t - 1];
                    if (t + 1 <= j - 1) v += (t + 1) * e[(j - 1) * kGT + t + 1];
                }
                e[(i * kGI + j) * kGT + t] = v;
            }
        }
}

template <class T>
__device__ __forceinline__ void grad_boys(int n, T x, const T* table, T* F)
{
#define GB_B(N)                              \
    case N: {                                \
        T f[N + 1];                          \
        BoysEval<T>::template run<N>(x, table, f); \
        for (int i = 0; i <= N; ++i) F[i] = f[i]; \
        break;                               \
    }
    switch (n) {
        GB_B(0) GB_B(1) GB_B(2) GB_B(3) GB_B(4) GB_B(5) GB_B(6) GB_B(7) GB_B(8) GB_B(9)
    default: break;
    }
#undef GB_B
}

template <class T>
__device__ __forceinline__ void grad_r_table(int L, const T* Fs, T X, T Y, T Z, T* r)
{
    r[0] = Fs[L];
    for (int n = L - 1; n >= 0; --n) {
        for (int k = L - n; k >= 1; --k)
            for (int t = k; t >= 0; --t)
                for (int u = k - t; u >= 0; --u) {
                    const int v = k - t - u;
                    T val;
                    if (t > 0) {
                        val = X * r[gidx(t - 1, u, v)];
                        if (t > 1) val += (t - 1) * r[gidx(t - 2, u, v)];
                    } else if (u > 0) {
                        val = Y * r[gidx(0, u - 1, v)];
                        if (u > 1) val += (u - 1) * r[gidx(0, u - 2, v)];
                    } else {
                        val = Z * r[gidx(0, 0, v - 1)];
                        if (v > 1) val += (v - 1) * r[gidx(0, 0, v - 2)];
                    }
                    r[gidx(t, u, v)] = val;
                }
        r[0] = Fs[n];
    }
}


// Item offsets of a class pair's list: entry e owns cnt_e kets, each split into the
// entry's bra primitive pairs, so one work item is one (ket, bra primitive pair).
// One block per class pair (the layout of the quartet plan's offsets).
__global__ void __launch_bounds__(256) grad_items_kernel(const long long* __restrict__ off,
                                                         const int* __restrict__ entry_bra,
                                                         const int* __restrict__ entry_prim,
                                                         const ShellPairDev* __restrict__ pairs,
                                                         const int* __restrict__ cp_meta, int ncp,
                                                         long long* __restrict__ goff)
{
    __shared__ long long part[256];
    const int cp = blockIdx.x;
    const int eb = cp_meta[cp], ne = cp_meta[ncp + cp], ob = cp_meta[3 * ncp + cp];
    long long base = 0;
    if (threadIdx.x == 0) goff[ob] = 0;
    for (int start = 0; start < ne; start += blockDim.x) {
        const int i = start + threadIdx.x;
        long long v = 0;
        if (i < ne) {
            const int pr = entry_prim[eb + i];
            v = (off[ob + i + 1] - off[ob + i]) * static_cast<long long>((pr >> 16) - (pr & 0xffff));
        }
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < blockDim.x; o <<= 1) {  // inclusive Hillis-Steele scan
            const long long add = (threadIdx.x >= o) ? part[threadIdx.x - o] : 0;
            __syncthreads();
            part[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < ne) goff[ob + i + 1] = base + part[threadIdx.x];
        base += part[blockDim.x - 1];
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(kGradThreads) grad_eri_kernel(const GradLaunch G, int ncd)
{
    extern __shared__ double sgrad[];
    const FockClassLaunch& L = G.L;
    if (G.shared_grad) {
        for (int i = threadIdx.x; i < 3 * G.natom; i += blockDim.x) sgrad[i] = 0.0;
        __syncthreads();
    }
    double* const gacc = G.shared_grad ? sgrad : G.grad;
    const long long total = G.goff[L.nentry];
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((total + 31) >> 5) * ncd;
    const long long warp_stride = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
    using PP = typename FockTypes<T>::PP;
    const T* __restrict__ Dp = static_cast<const T*>(L.density);
    const PP* __restrict__ pp = static_cast<const PP*>(L.prim_pairs);
    const T* __restrict__ boys = static_cast<const T*>(L.boys_table);
    const int N = L.num_basis;
    const T thr = static_cast<T>(L.schwarz_threshold);
    // one set of E tables: the bra's (used only to build H0/HA) and then each ket primitive pair's
    T ex[kGE], ey[kGE], ez[kGE];
    T* const fx = ex;
    T* const fy = ey;
    T* const fz = ez;
    T Fs[kGL + 1], r[kGR];
    T z0[kGR], zD[kGR];  // separable ket-contraction intermediates (R's buffer holds the y stages)
    T wcol[kGNAB];

    for (long long wid = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; wid < nwarps;
         wid += warp_stride) {
        const int cdi = static_cast<int>(wid % ncd);
        const long long w = (wid / ncd) * 32 + lane;
        const int e = find_entry_warp(G.goff, L.nentry, (wid / ncd) * 32, w, total);
        if (w >= total) continue;
        const int bra = __ldg(L.entry_bra + e);
        const ShellPairDev bp = L.pairs[bra];
        const long long item = w - __ldg(G.goff + e);
        const int pr = __ldg(L.entry_prim + e), nip = (pr >> 16) - (pr & 0xffff);
        const int ip = (pr & 0xffff) + static_cast<int>(item % nip);
        const int ket = L.ket_base + __ldg(L.entry_lo + e) + static_cast<int>(item / nip);
        const ShellPairDev kp = L.pairs[ket];
        const int la = bp.la, lb = bp.lb, lc = kp.la, ld = kp.lb;
        const int na = ncart(la), nb = ncart(lb), nd = ncart(ld);
        const int lab = la + lb, lt = lab + lc + ld + 1;
        const int ic = cdi / nd, id = cdi % nd;
        const int c[3] = {cart_exp(lc, ic, 0), cart_exp(lc, ic, 1), cart_exp(lc, ic, 2)};
        const int d[3] = {cart_exp(ld, id, 0), cart_exp(ld, id, 1), cart_exp(ld, id, 2)};
        const int cf = kp.bfA + ic, df = kp.bfB + id;
        T fsym = T(1);
        if (bp.A == bp.B) fsym *= T(0.5);
        if (kp.A == kp.B) fsym *= T(0.5);
        if (bra == ket) fsym *= T(0.5);
        // bra/ket geometry in the tier's type
        const T bABx = sizeof(T) == 4 ? static_cast<T>(bp.fABx) : static_cast<T>(bp.ABx);
        const T bABy = sizeof(T) == 4 ? static_cast<T>(bp.fABy) : static_cast<T>(bp.ABy);
        const T bABz = sizeof(T) == 4 ? static_cast<T>(bp.fABz) : static_cast<T>(bp.ABz);
        const T kABx = sizeof(T) == 4 ? static_cast<T>(kp.fABx) : static_cast<T>(kp.ABx);
        const T kABy = sizeof(T) == 4 ? static_cast<T>(kp.fABy) : static_cast<T>(kp.ABy);
        const T kABz = sizeof(T) == 4 ? static_cast<T>(kp.fABz) : static_cast<T>(kp.ABz);
        const T kQmax = sizeof(T) == 4 ? static_cast<T>(kp.fQmax) : static_cast<T>(kp.Qmax);
        // density weights of this (c,d) column: f (4 D_ab D_cd - D_ac D_bd - D_ad D_bc)
        const T dcd = Dp[cf * N + df];
        bool any = false;
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                const int a = bp.bfA + ia, b = bp.bfB + ib;
                const T v = fsym * (T(4) * Dp[a * N + b] * dcd - Dp[a * N + cf] * Dp[b * N + df] -
                                    Dp[a * N + df] * Dp[b * N + cf]);
                wcol[ia * nb + ib] = v;
                any |= (v != T(0));
            }
        if (!any) continue;
        // Bra side in Hermite space: per bra primitive pair, the weighted Hermite densities
        //   H0[tuv]   = sum_ab w_ab E^{ab}_tuv
        //   HA_k[tuv] = sum_ab w_ab (2 alpha E^{a+1_k, b}_tuv - a_k E^{a-1_k, b}_tuv)
        // are built once and reused for every ket primitive pair, so the inner loop does
        // not grow with the number of bra components.  Then
        //   dA_k = sum HA_k x0,  dP_k = sum H0 x0[tuv + 1_k] (= dA_k + dB_k),
        //   dC_k = sum H0 (2 gamma x[c + 1_k] - c_k x[c - 1_k]).
        T gA[3] = {0, 0, 0}, gP[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
        T H0[kGX], HA[3][kGX];
        {  // this item's bra primitive pair
            const PP pb = pp[bp.pp_off + ip];
            if (pb.Q * kQmax < thr) continue;
            const T alpha2 = T(2) * (pb.p - pb.b);
            const T oo2p = T(0.5) * pb.invp;
            grad_e_table<T>(la + 1, lb, pb.PAx, pb.PAx + bABx, oo2p, ex);
            grad_e_table<T>(la + 1, lb, pb.PAy, pb.PAy + bABy, oo2p, ey);
            grad_e_table<T>(la + 1, lb, pb.PAz, pb.PAz + bABz, oo2p, ez);
            const int nh = nherm(lab + 1);
            for (int h = 0; h < nh; ++h) { H0[h] = T(0); HA[0][h] = T(0); HA[1][h] = T(0); HA[2][h] = T(0); }
            for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib) {
                    const T wv = wcol[ia * nb + ib];
                    if (wv == T(0)) continue;
                    const int a[3] = {cart_exp(la, ia, 0), cart_exp(la, ia, 1), cart_exp(la, ia, 2)};
                    const int b[3] = {cart_exp(lb, ib, 0), cart_exp(lb, ib, 1), cart_exp(lb, ib, 2)};
                    // per-axis factors: e0 = E^{a b}, e1 = 2 alpha E^{a+1, b} - a E^{a-1, b}
                    T e0[3][kGT], e1[3][kGT];
                    const T* tab[3] = {ex, ey, ez};
                    for (int k = 0; k < 3; ++k) {
                        const T* row0 = tab[k] + (a[k] * kGI + b[k]) * kGT;
                        const T* rowp = tab[k] + ((a[k] + 1) * kGI + b[k]) * kGT;
                        const T* rowm = tab[k] + ((a[k] > 0 ? a[k] - 1 : 0) * kGI + b[k]) * kGT;
                        for (int t = 0; t <= a[k] + b[k] + 1; ++t) {
                            e0[k][t] = (t <= a[k] + b[k]) ? row0[t] : T(0);
                            T v = alpha2 * rowp[t];
                            if (a[k] > 0 && t <= a[k] + b[k] - 1) v -= T(a[k]) * rowm[t];
                            e1[k][t] = v;
                        }
                    }
                    for (int t = 0; t <= a[0] + b[0] + 1; ++t)
                        for (int u = 0; u <= a[1] + b[1] + 1; ++u)
                            for (int v = 0; v <= a[2] + b[2] + 1; ++v) {
                                if (t + u + v > lab + 1) continue;
                                const int h = gidx(t, u, v);
                                HA[0][h] += wv * e1[0][t] * e0[1][u] * e0[2][v];
                                HA[1][h] += wv * e0[0][t] * e1[1][u] * e0[2][v];
                                HA[2][h] += wv * e0[0][t] * e0[1][u] * e1[2][v];
                                H0[h] += wv * e0[0][t] * e0[1][u] * e0[2][v];
                            }
                }
            for (int jq = 0; jq < kp.pp_n; ++jq) {
                const PP pk = pp[kp.pp_off + jq];
                if (pb.Q * pk.Q < thr) break;  // primitive pairs sorted by Q (descending)
                const T gamma2 = T(2) * (pk.p - pk.b);
                const T oo2q = T(0.5) * pk.invp;
                grad_e_table<T>(lc + 1, ld, pk.PAx, pk.PAx + kABx, oo2q, fx);
                grad_e_table<T>(lc + 1, ld, pk.PAy, pk.PAy + kABy, oo2q, fy);
                grad_e_table<T>(lc + 1, ld, pk.PAz, pk.PAz + kABz, oo2q, fz);
                const T rr = rsqrt(pb.p + pk.p);
                const T rho = pb.p * pk.p * rr * rr;
                const T X = pb.Px - pk.Px, Y = pb.Py - pk.Py, Z = pb.Pz - pk.Pz;
                grad_boys<T>(lt, rho * (X * X + Y * Y + Z * Z), boys, Fs);
                T scale = pb.KoP * pk.KoP * rr;
                for (int n = 0; n <= lt; ++n) { Fs[n] *= scale; scale *= T(-2) * rho; }
                grad_r_table<T>(lt, Fs, X, Y, Z, r);
                // Separable ket contraction, one axis at a time, with (-1)^tau folded into
                // the per-axis vectors:  e0_k = E^{c_k d_k},  eD_k = 2 gamma E^{c_k+1, d_k} - c_k E^{c_k-1, d_k}.
                //   x0[tuv]  = sum e0_x e0_y e0_z R[t+tau, u+nu, v+phi]   (tuv <= lab + 1)
                //   xD_k[tuv] = the same with eD along axis k              (tuv <= lab)
                // built as z-, then y-, then x-contractions; the intermediates are only
                // needed for v (and u + v) <= lab + 1.
                T e0[3][kGT], eD[3][kGT];
                int n0[3], nD[3];
                for (int k = 0; k < 3; ++k) {
                    const T* tab = k == 0 ? fx : (k == 1 ? fy : fz);
                    const T* row0 = tab + (c[k] * kGI + d[k]) * kGT;
                    const T* rowp = tab + ((c[k] + 1) * kGI + d[k]) * kGT;
                    const T* rowm = tab + ((c[k] > 0 ? c[k] - 1 : 0) * kGI + d[k]) * kGT;
                    n0[k] = c[k] + d[k];
                    nD[k] = c[k] + d[k] + 1;
                    for (int t = 0; t <= nD[k]; ++t) {
                        const T sg = (t & 1) ? T(-1) : T(1);
                        e0[k][t] = (t <= n0[k]) ? sg * row0[t] : T(0);
                        T v = gamma2 * rowp[t];
                        if (c[k] > 0 && t <= c[k] - 1 + d[k]) v -= T(c[k]) * rowm[t];
                        eD[k][t] = sg * v;
                    }
                }
                const int lv = lab + 1;
                // z stage: out[t,u,v] = sum_phi ez[phi] R[t, u, v + phi]
                auto zstage = [&](const T* ez, int nz, T* out) {
                    for (int v = 0; v <= lv; ++v)
                        for (int t = 0; t + v <= lt; ++t)
                            for (int u = 0; t + u + v <= lt; ++u) {
                                T acc = T(0);
                                for (int f = 0; f <= nz && t + u + v + f <= lt; ++f) acc += ez[f] * r[gidx(t, u, v + f)];
                                out[gidx(t, u, v)] = acc;
                            }
                };
                // y stage: out[t,u,v] = sum_nu ey[nu] zin[t, u + nu, v]  (u + v <= lv)
                auto ystage = [&](const T* ey, int ny, const T* zin, T* out) {
                    for (int u = 0; u <= lv; ++u)
                        for (int v = 0; u + v <= lv; ++v)
                            for (int t = 0; t + u + v <= lt; ++t) {
                                T acc = T(0);
                                for (int g = 0; g <= ny && t + u + g + v <= lt; ++g) acc += ey[g] * zin[gidx(t, u + g, v)];
                                out[gidx(t, u, v)] = acc;
                            }
                };
                // both z stages first (R is then dead and its buffer holds each y stage)
                zstage(e0[2], n0[2], z0);
                zstage(eD[2], nD[2], zD);
                // base: x stage fused with the bra contractions
                //   gA += HA x0,  gP += H0[tuv - 1_k] x0[tuv],  gC_x += H0 xD_x
                ystage(e0[1], n0[1], z0, r);
                for (int t = 0; t <= lv; ++t)
                    for (int u = 0; u + t <= lv; ++u)
                        for (int v = 0; v + u + t <= lv; ++v) {
                            T x = T(0);
                            for (int a = 0; a <= n0[0] && t + a + u + v <= lt; ++a) x += e0[0][a] * r[gidx(t + a, u, v)];
                            const int h = gidx(t, u, v);
                            gA[0] += HA[0][h] * x;
                            gA[1] += HA[1][h] * x;
                            gA[2] += HA[2][h] * x;
                            if (t > 0) gP[0] += H0[gidx(t - 1, u, v)] * x;
                            if (u > 0) gP[1] += H0[gidx(t, u - 1, v)] * x;
                            if (v > 0) gP[2] += H0[gidx(t, u, v - 1)] * x;
                            if (t + u + v > lab) continue;
                            T xx = T(0);
                            for (int a = 0; a <= nD[0] && t + a + u + v <= lt; ++a) xx += eD[0][a] * r[gidx(t + a, u, v)];
                            gC[0] += H0[h] * xx;
                        }
                // y and z derivatives of the ket centre: gC_k += H0 xD_k (tuv <= lab)
                for (int k = 1; k < 3; ++k) {
                    if (k == 1) ystage(eD[1], nD[1], z0, r); else ystage(e0[1], n0[1], zD, r);
                    T acc = T(0);
                    for (int t = 0; t <= lab; ++t)
                        for (int u = 0; u + t <= lab; ++u)
                            for (int v = 0; v + u + t <= lab; ++v) {
                                const T h0 = H0[gidx(t, u, v)];
                                if (h0 == T(0)) continue;
                                T x = T(0);
                                for (int a = 0; a <= n0[0] && t + a + u + v <= lt; ++a) x += e0[0][a] * r[gidx(t + a, u, v)];
                                acc += h0 * x;
                            }
                    gC[k] += acc;
                }
            }
        }
        T gB[3];
        for (int k = 0; k < 3; ++k) gB[k] = gP[k] - gA[k];
        const int atA = G.shell_atom[bp.A], atB = G.shell_atom[bp.B], atC = G.shell_atom[kp.A],
                  atD = G.shell_atom[kp.B];
        for (int k = 0; k < 3; ++k) {
            atomicAdd(&gacc[3 * atA + k], static_cast<double>(gA[k]));
            atomicAdd(&gacc[3 * atB + k], static_cast<double>(gB[k]));
            atomicAdd(&gacc[3 * atC + k], static_cast<double>(gC[k]));
            atomicAdd(&gacc[3 * atD + k], -static_cast<double>(gA[k] + gB[k] + gC[k]));
        }
    }
    if (G.shared_grad) {  // one flush per block
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * G.natom; i += blockDim.x)
            if (sgrad[i] != 0.0) atomicAdd(&G.grad[i], sgrad[i]);
    }
}

// One-electron part per shell pair: sum over the (a,b) block and its mirror of
// D_ab d(T+V)_ab/dR - W_ab dS_ab/dR, including the Hellmann-Feynman term of
// each nucleus C (dV/dC_x = Z (2 pi / p) K sum_tuv E_tuv R_{t+1,u,v}).
template <int LA, int LB>
__global__ void __launch_bounds__(128)
grad_one_electron_kernel(const ShellPairDev* __restrict__ pairs, int begin, int count,
                         const PrimPair64* __restrict__ pp, const double* __restrict__ boys,
                         const double* __restrict__ atoms, int natom, const int* __restrict__ shell_atom,
                         const double* __restrict__ scale, const double* __restrict__ D,
                         const double* __restrict__ W, int n, double kfold, double* __restrict__ grad)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), L = LA + LB + 1;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    const ShellPairDev sp = pairs[begin + idx];
    // density weights in the unnormalised space: factor 2 for the mirror block
    const double mirror = (sp.A == sp.B) ? 1.0 : 2.0;
    double dw[NA][NB], ww[NA][NB];
    for (int ia = 0; ia < NA; ++ia)
        for (int ib = 0; ib < NB; ++ib) {
            const int a = sp.bfA + ia, b = sp.bfB + ib;
            const double ss = scale[a] * scale[b] * mirror;
            dw[ia][ib] = D[a * n + b] * ss;
            ww[ia][ib] = W[a * n + b] * ss;
        }
    double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
    const int atA = shell_atom[sp.A], atB = shell_atom[sp.B];
    for (int ip = 0; ip < sp.pp_n; ++ip) {
        const PrimPair64 q = pp[sp.pp_off + ip];
        const double p = q.p, bexp = q.b, aexp = p - bexp, oo2p = 0.5 * q.invp;
        const double k1 = q.K / kfold;
        HermiteE<double, LA + 1, LB + 2> Ex, Ey, Ez;
        Ex.build(q.PAx, q.PAx + sp.ABx, oo2p);
        Ey.build(q.PAy, q.PAy + sp.ABy, oo2p);
        Ez.build(q.PAz, q.PAz + sp.ABz, oo2p);
        const double sq = sqrt(kPi / p);
        // overlap and kinetic 1D factors for i <= LA+1, j <= LB
        auto s1 = [&](const HermiteE<double, LA + 1, LB + 2>& E, int i, int j) { return E.e[i][j][0] * sq; };
        auto t1 = [&](const HermiteE<double, LA + 1, LB + 2>& E, int i, int j) {
            double tt = 4.0 * bexp * bexp * E.e[i][j + 2][0] - 2.0 * bexp * (2 * j + 1) * E.e[i][j][0];
            if (j >= 2) tt += j * (j - 1) * E.e[i][j - 2][0];
            return -0.5 * tt * sq;
        };
        for (int ia = 0; ia < NA && blockIdx.y == 0; ++ia)  // S and T: the blocks of the first nucleus
            for (int ib = 0; ib < NB; ++ib) {
                int a[3] = {cart_exp(LA, ia, 0), cart_exp(LA, ia, 1), cart_exp(LA, ia, 2)};
                const int b[3] = {cart_exp(LB, ib, 0), cart_exp(LB, ib, 1), cart_exp(LB, ib, 2)};
                const HermiteE<double, LA + 1, LB + 2>* E3[3] = {&Ex, &Ey, &Ez};
                for (int k = 0; k < 3; ++k) {
                    // d/dA_k of S and T: shift a along k
                    double dS = 0.0, dT = 0.0;
                    for (int sgn = 0; sgn < 2; ++sgn) {
                        int ak = a[k] + (sgn == 0 ? 1 : -1);
                        if (ak < 0) continue;
                        const double c = (sgn == 0) ? 2.0 * aexp : -static_cast<double>(a[k]);
                        int aa[3] = {a[0], a[1], a[2]};
                        aa[k] = ak;
                        const double sx = s1(*E3[0], aa[0], b[0]), sy = s1(*E3[1], aa[1], b[1]), sz = s1(*E3[2], aa[2], b[2]);
                        const double tx = t1(*E3[0], aa[0], b[0]), ty = t1(*E3[1], aa[1], b[1]), tz = t1(*E3[2], aa[2], b[2]);
                        dS += c * sx * sy * sz;
                        dT += c * (tx * sy * sz + sx * ty * sz + sx * sy * tz);
                    }
                    const double g = k1 * (dw[ia][ib] * dT - ww[ia][ib] * dS);
                    gA[k] += g;
                    gB[k] -= g;  // S and T depend on A - B only
                }
            }
        // nuclear attraction: basis centres (shift of a) and the operator centre, one
        // nucleus per grid row (blockIdx.y)
        {
            const int cidx = blockIdx.y;
            const double X = q.Px - atoms[4 * cidx], Y = q.Py - atoms[4 * cidx + 1], Z = q.Pz - atoms[4 * cidx + 2];
            double Fs[L + 1];
            boys_fp64<L>(p * (X * X + Y * Y + Z * Z), boys, Fs);
            double sc = -atoms[4 * cidx + 3] * 2.0 * kPi / p * k1;
            for (int m = 0; m <= L; ++m) { Fs[m] *= sc; sc *= -2.0 * p; }
            HermiteR<double, L> R;
            R.build(Fs, X, Y, Z);
            double gCn[3] = {0, 0, 0};
            for (int ia = 0; ia < NA; ++ia)
                for (int ib = 0; ib < NB; ++ib) {
                    const int a[3] = {cart_exp(LA, ia, 0), cart_exp(LA, ia, 1), cart_exp(LA, ia, 2)};
                    const int b[3] = {cart_exp(LB, ib, 0), cart_exp(LB, ib, 1), cart_exp(LB, ib, 2)};
                    const double dwv = dw[ia][ib];
                    if (dwv == 0.0) continue;
                    for (int k = 0; k < 3; ++k) {
                        double dA = 0.0;
                        for (int sgn = 0; sgn < 2; ++sgn) {
                            int aa[3] = {a[0], a[1], a[2]};
                            aa[k] += (sgn == 0 ? 1 : -1);
                            if (aa[k] < 0) continue;
                            const double c = (sgn == 0) ? 2.0 * aexp : -static_cast<double>(a[k]);
                            double acc = 0.0;
                            for (int t = 0; t <= aa[0] + b[0]; ++t)
                                for (int u = 0; u <= aa[1] + b[1]; ++u)
                                    for (int v = 0; v <= aa[2] + b[2]; ++v)
                                        acc += Ex.e[aa[0]][b[0]][t] * Ey.e[aa[1]][b[1]][u] * Ez.e[aa[2]][b[2]][v] *
                                               R(t, u, v);
                            dA += c * acc;
                        }
                        // operator centre: d/dC_k R_tuv(P - C) = -R_{tuv + 1_k}
                        double dC = 0.0;
                        for (int t = 0; t <= a[0] + b[0]; ++t)
                            for (int u = 0; u <= a[1] + b[1]; ++u)
                                for (int v = 0; v <= a[2] + b[2]; ++v) {
                                    const double ev = Ex.e[a[0]][b[0]][t] * Ey.e[a[1]][b[1]][u] * Ez.e[a[2]][b[2]][v];
                                    const double rv = (k == 0) ? R(t + 1, u, v) : (k == 1) ? R(t, u + 1, v) : R(t, u, v + 1);
                                    dC -= ev * rv;
                                }
                        gA[k] += dwv * dA;
                        gB[k] -= dwv * (dA + dC);
                        gCn[k] += dwv * dC;
                    }
                }
            for (int k = 0; k < 3; ++k)
                if (gCn[k] != 0.0) atomicAdd(&grad[3 * cidx + k], gCn[k]);
        }
    }
    for (int k = 0; k < 3; ++k) {
        atomicAdd(&grad[3 * atA + k], gA[k]);
        atomicAdd(&grad[3 * atB + k], gB[k]);
    }
}

// W = 2 sum_{i < nocc} eps_i C_i C_i^T (C row-major, columns = orbitals)
__global__ void energy_weighted_density_kernel(const double* __restrict__ C, const double* __restrict__ eps, int n,
                                               int nocc, double* __restrict__ W)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long i = k / n, j = k % n;
        double s = 0.0;
        for (int o = 0; o < nocc; ++o) s += eps[o] * C[i * n + o] * C[j * n + o];
        W[k] = 2.0 * s;
    }
}

}  // namespace

int energy_weighted_density(Engine& e, const double* d_C, const double* d_eps, int nocc, double* d_W, cudaStream_t s)
{
    const long long nn = static_cast<long long>(e.num_basis) * e.num_basis;
    energy_weighted_density_kernel<<<static_cast<int>(std::min<long long>((nn + 255) / 256, 4096)), 256, 0, s>>>(
        d_C, d_eps, e.num_basis, nocc, d_W);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

int rhf_gradient(Engine& e, const double* d_D, const double* d_W, double* h_grad, cudaStream_t s, float* ms_out,
                 int precision, double mixed_threshold, const double* d_C, int ldc, int nocc)
{
    const int natom = e.num_atoms;
    if (!e.d_grad) {
        if (cudaMalloc(&e.d_grad, sizeof(double) * 3 * natom) != cudaSuccess ||
            cudaMalloc(&e.d_shell_atom, sizeof(int) * e.num_shells) != cudaSuccess)
            return set_error("cudaMalloc of gradient buffers failed"), HF_ERR_OUT_OF_MEMORY;
        std::vector<int> sa(e.num_shells);
        for (int i = 0; i < e.num_shells; ++i) sa[i] = e.shells[i].atom;
        GB_CUDA_TRY(cudaMemcpy(e.d_shell_atom, sa.data(), sizeof(int) * e.num_shells, cudaMemcpyHostToDevice));
    }
    const bool mixed = precision == HF_PRECISION_MIXED;
    ScopedEvents<2> evs;
    cudaEvent_t t0 = evs.ev[0], t1 = evs.ev[1];
    cudaEventRecord(t0, s);
    GB_CUDA_TRY(cudaMemsetAsync(e.d_grad, 0, sizeof(double) * 3 * natom, s));
    int st = HF_OK;
    if (d_C) {
        // density fitting: derivative three-centre and metric integrals (ri_grad.cu)
        if ((st = ri_gradient_two_electron(e, d_D, d_C, ldc, nocc, s))) return st;
    } else {
    st = scale_density(e, d_D, mixed, s);
    if (st) return st;
    if (mixed) {
        // FP64 for the quartets with Qs_ab Qs_cd c_max^4 max|D|^2 >= mixed_threshold, FP32 for the rest
        const double c2 = e.cgto_max * e.cgto_max;
        if ((st = mixed_plan(e, d_D, c2 * c2, true, mixed_threshold, 0.0, s))) return st;
    }
    // work items (ket, bra primitive pair) of every list in use
    const int ncp = static_cast<int>(e.class_pairs.size());
    const size_t noff = e.off_static.size();
    if (!e.d_goff64 && (cudaMalloc(&e.d_goff64, sizeof(long long) * noff) != cudaSuccess ||
                        cudaMalloc(&e.d_goff32, sizeof(long long) * noff) != cudaSuccess))
        return set_error("cudaMalloc of gradient item offsets failed"), HF_ERR_OUT_OF_MEMORY;
    grad_items_kernel<<<ncp, 256, 0, s>>>(mixed ? e.plan.off64 : e.d_off_static, e.d_entry_bra, e.d_entry_prim,
                                          e.d_pairs, e.d_cp_meta, ncp, e.d_goff64);
    GB_LAUNCH_CHECK();
    if (mixed) {
        grad_items_kernel<<<ncp, 256, 0, s>>>(e.plan.off32, e.d_entry_bra, e.d_entry_prim, e.d_pairs, e.d_cp_meta, ncp,
                                              e.d_goff32);
        GB_LAUNCH_CHECK();
    }
    const size_t sgrad_bytes = sizeof(double) * 3 * natom;
    const bool shared_grad = sgrad_bytes <= 32 * 1024;
    // two-electron part over the quartet lists of every class, on the branches of
    // the engine's Fock schedule (class pairs accumulate into d_grad with atomics)
    st = launch_class_pairs(e, s, [&](int c, cudaStream_t cs) -> int {
        const ClassPair& cp = e.class_pairs[c];
        const PairClass& Y = e.pair_classes[cp.Y];
        const PairClass& X = e.pair_classes[cp.X];
        int max_pp = 1;
        for (int i = X.begin; i < X.begin + X.count; ++i) max_pp = std::max(max_pp, e.pairs[i].pp_n);
        for (int tier = 0; tier < (mixed ? 2 : 1); ++tier) {
            const bool f32 = tier == 1;
            GradLaunch G;
            G.L.pairs = e.d_pairs;
            G.L.prim_pairs = f32 ? static_cast<const void*>(e.d_pp32) : static_cast<const void*>(e.d_pp64);
            G.L.boys_table = f32 ? static_cast<const void*>(e.d_boys32) : static_cast<const void*>(e.d_boys64);
            G.L.density = f32 ? static_cast<const void*>(e.d_Dp32) : static_cast<const void*>(e.d_Dp64);
            G.L.J = nullptr;
            G.L.K = nullptr;
            G.L.J32 = nullptr;
            G.L.K32 = nullptr;
            const long long* off = !mixed ? e.d_off_static : (f32 ? e.plan.off32 : e.plan.off64);
            const int* lo = f32 ? e.plan.lo32 : e.d_entry_lo0;
            G.L.off = off + cp.entry_begin + c;
            G.L.entry_bra = e.d_entry_bra + cp.entry_begin;
            G.L.entry_lo = lo + cp.entry_begin;
            G.L.entry_prim = e.d_entry_prim + cp.entry_begin;
            G.L.nentry = cp.nentry;
            G.L.ket_base = Y.begin;
            G.L.num_basis = e.num_basis;
            G.L.schwarz_threshold = e.schwarz_threshold;
            G.L.counters = e.d_counters;
            G.L.block_dmax = nullptr;
            G.L.nshell = e.num_shells;
            G.L.skip_cut = 0.0;
            G.L.mol_active = nullptr;
            G.L.shell_mol = e.d_shell_mol;
            G.goff = (f32 ? e.d_goff32 : e.d_goff64) + cp.entry_begin + c;
            G.shell_atom = e.d_shell_atom;
            G.grad = e.d_grad;
            G.natom = natom;
            G.shared_grad = shared_grad ? 1 : 0;
            const int ncd = ncart(Y.la) * ncart(Y.lb);
            // items <= survivors x the class's largest bra primitive-pair count (grid-stride loop)
            const long long warps = ((cp.n_survivors * max_pp + 31) / 32) * ncd;
            const int grid = static_cast<int>(std::max<long long>(
                1, std::min<long long>((warps * 32 + kGradThreads - 1) / kGradThreads,
                                       static_cast<long long>(e.num_sms) * 32)));
            const size_t smem = shared_grad ? sgrad_bytes : 0;
            const bool done = f32 ? launch_grad_class_f32(X.la, X.lb, Y.la, Y.lb, G, grid, smem, cs)
                                  : launch_grad_class_f64(X.la, X.lb, Y.la, Y.lb, G, grid, smem, cs);
            if (!done) {
                if (f32)
                    grad_eri_kernel<float><<<grid, kGradThreads, smem, cs>>>(G, ncd);
                else
                    grad_eri_kernel<double><<<grid, kGradThreads, smem, cs>>>(G, ncd);
            }
            GB_LAUNCH_CHECK();
        }
        return HF_OK;
    });
    if (st) return st;
    }  // four-centre part
    // one-electron part
    const double kfold = std::sqrt(2.0 * std::pow(kPi, 2.5));
    for (const PairClass& pc : e.pair_classes) {
        if (pc.count == 0) continue;
        const dim3 grid((pc.count + 127) / 128, natom);  // one row of blocks per nucleus C
#define GB_G1(a, b)                                                                                                 \
    if (pc.la == a && pc.lb == b)                                                                                   \
        grad_one_electron_kernel<a, b><<<grid, 128, 0, s>>>(e.d_pairs, pc.begin, pc.count, e.d_pp64, e.d_boys64,    \
                                                            e.d_atoms, e.num_atoms, e.d_shell_atom, e.d_scale, d_D, \
                                                            d_W, e.num_basis, kfold, e.d_grad);
        GB_G1(0, 0) GB_G1(1, 0) GB_G1(1, 1) GB_G1(2, 0) GB_G1(2, 1) GB_G1(2, 2)
#undef GB_G1
        GB_LAUNCH_CHECK();
    }
    cudaEventRecord(t1, s);
    GB_CUDA_TRY(cudaMemcpyAsync(h_grad, e.d_grad, sizeof(double) * 3 * natom, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    if (ms_out) *ms_out = ms;
    // nuclear repulsion: d/dR_A sum_{A<B} Z_A Z_B / |R_A - R_B|
    for (int A = 0; A < natom; ++A)
        for (int B = 0; B < natom; ++B) {
            if (A == B) continue;
            const double dx = e.atoms[A].x - e.atoms[B].x, dy = e.atoms[A].y - e.atoms[B].y,
                         dz = e.atoms[A].z - e.atoms[B].z;
            const double r2 = dx * dx + dy * dy + dz * dz, r = std::sqrt(r2);
            const double f = -static_cast<double>(e.atoms[A].atomic_number) * e.atoms[B].atomic_number / (r2 * r);
            h_grad[3 * A] += f * dx;
            h_grad[3 * A + 1] += f * dy;
            h_grad[3 * A + 2] += f * dz;
        }
    return HF_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int hf_energy_weighted_density(hf_engine* eng, const double* d_coefficients, const double* d_orbital_energies,
                               int num_occupied, double* d_out, void* stream)
{
    clear_error();
    if (!eng || !d_coefficients || !d_orbital_energies || !d_out || num_occupied <= 0)
        return set_error("null argument or non-positive num_occupied"), HF_ERR_INVALID_ARGUMENT;
    return energy_weighted_density(*reinterpret_cast<Engine*>(eng), d_coefficients, d_orbital_energies, num_occupied,
                                   d_out, static_cast<cudaStream_t>(stream));
}

int hf_rhf_gradient(hf_engine* eng, const double* d_density, const double* d_energy_weighted_density,
                    double* h_gradient, double* gradient_ms, void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_energy_weighted_density || !h_gradient)
        return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<Engine*>(eng)->nmol != 1)
        return set_error("hf_rhf_gradient: single-molecule engines only"), HF_ERR_INVALID_ARGUMENT;
    float ms = 0.f;
    const int st = rhf_gradient(*reinterpret_cast<Engine*>(eng), d_density, d_energy_weighted_density, h_gradient,
                                static_cast<cudaStream_t>(stream), &ms);
    if (gradient_ms) *gradient_ms = ms;
    return st;
}

int hf_rhf_gradient_ri(hf_engine* eng, const double* d_density, const double* d_energy_weighted_density,
                       const double* d_coefficients, int num_occupied, double* h_gradient, double* gradient_ms,
                       void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_energy_weighted_density || !d_coefficients || !h_gradient || num_occupied <= 0)
        return set_error("null argument or non-positive num_occupied"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (e.nmol != 1) return set_error("hf_rhf_gradient_ri: single-molecule engines only"), HF_ERR_INVALID_ARGUMENT;
    if (!e.ri) return set_error("hf_rhf_gradient_ri needs an auxiliary basis"), HF_ERR_INVALID_ARGUMENT;
    if (num_occupied > e.num_basis)
        return set_error("more occupied orbitals than basis functions"), HF_ERR_INVALID_ARGUMENT;
    float ms = 0.f;
    const int st = rhf_gradient(e, d_density, d_energy_weighted_density, h_gradient, static_cast<cudaStream_t>(stream),
                                &ms, HF_PRECISION_FP64, 0.0, d_coefficients, e.num_basis, num_occupied);
    if (gradient_ms) *gradient_ms = ms;
    return st;
}

int hf_rhf_gradient_mixed(hf_engine* eng, const double* d_density, const double* d_energy_weighted_density,
                          double mixed_threshold, double* h_gradient, double* gradient_ms, void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_energy_weighted_density || !h_gradient || !(mixed_threshold >= 0.0))
        return set_error("null argument or negative threshold"), HF_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<Engine*>(eng)->nmol != 1)
        return set_error("hf_rhf_gradient_mixed: single-molecule engines only"), HF_ERR_INVALID_ARGUMENT;
    float ms = 0.f;
    const int st = rhf_gradient(*reinterpret_cast<Engine*>(eng), d_density, d_energy_weighted_density, h_gradient,
                                static_cast<cudaStream_t>(stream), &ms, HF_PRECISION_MIXED, mixed_threshold);
    if (gradient_ms) *gradient_ms = ms;
    return st;
}

}  // extern "C"
