// The one-(c,d)-column-per-thread form of the direct Fock build, shared by the
// generic kernel (runtime angular momenta, fock_generic.cu) and the class
// kernels of the large classes (compile-time angular momenta, fock_inst.cu).
//
// One thread evaluates one ket Cartesian component pair (c,d) of one
// contracted quartet, so a quartet of ncart^4 integrals spreads over
// ncart(LC)*ncart(LD) threads.  The split is warp-uniform (a warp takes 32
// quartets and one (c,d)); digestion follows the 8-fold rules of the unrolled
// kernels with the partial sums of one (c,d) column.  Runtime tables use
// packed storage:
//   E^{ij}_t    e[(i * 3 + j) * 5 + t]           (i, j <= 2, t <= 4)
//   R^{0}_{tuv} r[P(t,u,v)], P = k(k+1)(k+2)/6 + (k-t)(k-t+1)/2 + v, k = t+u+v
#pragma once
#include "fock_kernel.cuh"

namespace gb {
namespace fock_column {


constexpr int kEI = kMaxL + 1, kET = 2 * kMaxL + 1;
constexpr int kLT = 4 * kMaxL;            // highest total angular momentum
constexpr int kHR = nherm(kLT);           // packed R entries
constexpr int kHAB = nherm(2 * kMaxL);    // packed bra Hermite entries
constexpr int kNAB = ncart(kMaxL) * ncart(kMaxL);

__host__ __device__ constexpr int hx(int t, int u, int v)
{
    return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

__device__ __forceinline__ int hidx(int t, int u, int v)
{
    const int k = t + u + v, m = k - t;
    return k * (k + 1) * (k + 2) / 6 + m * (m + 1) / 2 + v;
}

template <class T>
__device__ __forceinline__ void hermite_e_rt(int l1, int l2, T xpa, T xpb, T oo2p, T* e)
{
    e[0] = T(1);
    for (int i = 0; i <= l1; ++i)
        for (int j = 0; j <= l2; ++j) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; ++t) {
                T v;
                if (i > 0) {
                    v = (t <= i - 1 + j) ? xpa * e[((i - 1) * kEI + j) * kET + t] : T(0);
                    if (t > 0) v += oo2p * e[((i - 1) * kEI + j) * kET + t - 1];
                    if (t + 1 <= i - 1 + j) v += T(t + 1) * e[((i - 1) * kEI + j) * kET + t + 1];
                } else {
                    v = (t <= j - 1) ? xpb * e[(j - 1) * kET + t] : T(0);
                    if (t > 0) v += oo2p * e[(j - 1) * kET + t - 1];
                    if (t + 1 <= j - 1) v += T(t + 1) * e[(j - 1) * kET + t + 1];
                }
                e[(i * kEI + j) * kET + t] = v;
            }
        }
}

template <class T>
__device__ __forceinline__ void boys_rt(int n, T x, const T* table, T* F)
{
#define GB_B(N)                                  \
    case N: {                                    \
        T f[N + 1];                              \
        BoysEval<T>::template run<N>(x, table, f); \
        for (int i = 0; i <= N; ++i) F[i] = f[i]; \
        break;                                   \
    }
    switch (n) {
        GB_B(0) GB_B(1) GB_B(2) GB_B(3) GB_B(4) GB_B(5) GB_B(6) GB_B(7) GB_B(8)
    default: break;
    }
#undef GB_B
}

// R^{0}_{tuv} for t+u+v <= L into packed r[], from Fs[n] = R^{n}_{000}
template <class T>
__device__ __forceinline__ void hermite_r_rt(int L, const T* Fs, T X, T Y, T Z, T* r)
{
    r[0] = Fs[L];
    for (int n = L - 1; n >= 0; --n) {
        for (int k = L - n; k >= 1; --k)
            for (int t = k; t >= 0; --t)
                for (int u = k - t; u >= 0; --u) {
                    const int v = k - t - u;
                    T val;
                    if (t > 0) {
                        val = X * r[hidx(t - 1, u, v)];
                        if (t > 1) val += T(t - 1) * r[hidx(t - 2, u, v)];
                    } else if (u > 0) {
                        val = Y * r[hidx(0, u - 1, v)];
                        if (u > 1) val += T(u - 1) * r[hidx(0, u - 2, v)];
                    } else {
                        val = Z * r[hidx(0, 0, v - 1)];
                        if (v > 1) val += T(v - 1) * r[hidx(0, 0, v - 2)];
                    }
                    r[hidx(t, u, v)] = val;
                }
        r[0] = Fs[n];
    }
}

// (ab|cd)' for all (a,b) and one ket component pair cd into I[ab], over the
// bra's primitive pairs [ip0, ip1); returns the primitive quartets evaluated
template <class T>
__device__ int quartet_column(const ShellPairDev& bp, const ShellPairDev& kp, int cd, int ip0, int ip1,
                              const typename FockTypes<T>::PP* __restrict__ pp, const T* __restrict__ boys_table, T thr,
                              T* I)
{
    using PP = typename FockTypes<T>::PP;
    const int la = bp.la, lb = bp.lb, lc = kp.la, ld = kp.lb;
    const int na = ncart(la), nb = ncart(lb), nd = ncart(ld);
    const int lab = la + lb, lt = lab + lc + ld;
    const int ic = cd / nd, id = cd % nd;
    const int cx = cart_exp(lc, ic, 0), cy = cart_exp(lc, ic, 1), cz = cart_exp(lc, ic, 2);
    const int dx = cart_exp(ld, id, 0), dy = cart_exp(ld, id, 1), dz = cart_exp(ld, id, 2);
    for (int ab = 0; ab < na * nb; ++ab) I[ab] = T(0);
    T ex[kEI * kEI * kET], ey[kEI * kEI * kET], ez[kEI * kEI * kET];
    T fx[kEI * kEI * kET], fy[kEI * kEI * kET], fz[kEI * kEI * kET];
    T Fs[kLT + 1], r[kHR], xh[kHAB];
    int count = 0;
    const typename TierTypes<T>::Geom gb_(bp), gk_(kp);
    const T qket_max = gk_.qmax;
    for (int ip = ip0; ip < ip1; ++ip) {
        const PP pb = pp[bp.pp_off + ip];
        if (pb.Q * qket_max < thr) break;  // primitive pairs sorted by Q (descending)
        const T oo2p = T(0.5) * pb.invp;
        hermite_e_rt<T>(la, lb, pb.PAx, pb.PAx + gb_.x, oo2p, ex);
        hermite_e_rt<T>(la, lb, pb.PAy, pb.PAy + gb_.y, oo2p, ey);
        hermite_e_rt<T>(la, lb, pb.PAz, pb.PAz + gb_.z, oo2p, ez);
        for (int jq = 0; jq < kp.pp_n; ++jq) {
            const PP pk = pp[kp.pp_off + jq];
            if (pb.Q * pk.Q < thr) break;
            ++count;
            const T oo2q = T(0.5) * pk.invp;
            hermite_e_rt<T>(lc, ld, pk.PAx, pk.PAx + gk_.x, oo2q, fx);
            hermite_e_rt<T>(lc, ld, pk.PAy, pk.PAy + gk_.y, oo2q, fy);
            hermite_e_rt<T>(lc, ld, pk.PAz, pk.PAz + gk_.z, oo2q, fz);
            const T rr = fast_rsqrt(pb.p + pk.p);
            const T rho = pb.p * pk.p * (rr * rr);
            const T X = pb.Px - pk.Px, Y = pb.Py - pk.Py, Z = pb.Pz - pk.Pz;
            boys_rt<T>(lt, rho * (X * X + Y * Y + Z * Z), boys_table, Fs);
            T scale = pb.KoP * pk.KoP * rr;
            const T m2rho = T(-2) * rho;
            for (int n = 0; n <= lt; ++n) { Fs[n] *= scale; scale *= m2rho; }
            hermite_r_rt<T>(lt, Fs, X, Y, Z, r);
            // ket contraction for this (c,d) into the bra Hermite index
            const T* fxc = fx + (cx * kEI + dx) * kET;
            const T* fyc = fy + (cy * kEI + dy) * kET;
            const T* fzc = fz + (cz * kEI + dz) * kET;
            for (int t = 0; t <= lab; ++t)
                for (int u = 0; u + t <= lab; ++u)
                    for (int v = 0; v + u + t <= lab; ++v) {
                        T s = T(0);
                        for (int tau = 0; tau <= cx + dx; ++tau)
                            for (int nu = 0; nu <= cy + dy; ++nu) {
                                const T exy = fxc[tau] * fyc[nu];
                                for (int phi = 0; phi <= cz + dz; ++phi) {
                                    const T c = exy * fzc[phi] * r[hidx(t + tau, u + nu, v + phi)];
                                    s += ((tau + nu + phi) & 1) ? -c : c;
                                }
                            }
                        xh[hidx(t, u, v)] = s;
                    }
            // bra contraction
            for (int ia = 0; ia < na; ++ia)
                for (int ib = 0; ib < nb; ++ib) {
                    const int ax = cart_exp(la, ia, 0), ay = cart_exp(la, ia, 1), az = cart_exp(la, ia, 2);
                    const int bx = cart_exp(lb, ib, 0), by = cart_exp(lb, ib, 1), bz = cart_exp(lb, ib, 2);
                    const T* exa = ex + (ax * kEI + bx) * kET;
                    const T* eya = ey + (ay * kEI + by) * kET;
                    const T* eza = ez + (az * kEI + bz) * kET;
                    T s = T(0);
                    for (int t = 0; t <= ax + bx; ++t)
                        for (int u = 0; u <= ay + by; ++u) {
                            const T exy = exa[t] * eya[u];
                            for (int v = 0; v <= az + bz; ++v) s += exy * eza[v] * xh[hidx(t, u, v)];
                        }
                    I[ia * nb + ib] += s;
                }
        }
    }
    return count;
}

// column evaluator with runtime angular momenta
template <class T>
struct RuntimeColumn {
    static constexpr int kNAB = fock_column::kNAB;
    static constexpr int kNA = 0, kNB = 0, kND = 0;  // runtime angular momenta
    __device__ static int eval(const ShellPairDev& bp, const ShellPairDev& kp, int cd, int ip0, int ip1,
                               const typename FockTypes<T>::PP* __restrict__ pp, const T* __restrict__ boys, T thr,
                               T* I)
    {
        return quartet_column<T>(bp, kp, cd, ip0, ip1, pp, boys, thr, I);
    }
};

// (ab|cd)' for all (a,b) and one ket component pair cd of class (LA LB|LC LD), every
// loop bound and table index a compile-time constant: the runtime (c, d) selects
// zero-padded ket coefficient vectors ((-1)^tau folded in), and the ket contraction
// is separable (z, y, then x stages of R).
template <class T, int LA, int LB, int LC, int LD>
__device__ __forceinline__ int quartet_column_ct(const ShellPairDev& bp, const ShellPairDev& kp, int cd, int ip0, int ip1,
                                                 const typename FockTypes<T>::PP* __restrict__ pp,
                                                 const T* __restrict__ boys_table, T thr, T* I)
{
    using PP = typename FockTypes<T>::PP;
    constexpr int NA = ncart(LA), NB = ncart(LB), ND = ncart(LD);
    constexpr int LAB = LA + LB, LCD = LC + LD, LT = LAB + LCD;
    constexpr int NT = nherm(LT), NX = nherm(LAB), PC = LCD + 1;
    const int ic = cd / ND, id = cd % ND;
    int c[3], d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { c[k] = cart_exp(LC, ic, k); d[k] = cart_exp(LD, id, k); }
#pragma unroll
    for (int ab = 0; ab < NA * NB; ++ab) I[ab] = T(0);
    int count = 0;
    const typename TierTypes<T>::Geom gb_(bp), gk_(kp);
    const T qket_max = gk_.qmax;
    constexpr bool kPrefetch = sizeof(T) == 4;  // next ket record one iteration ahead (FP32 tier)
    const PP* __restrict__ kpp = pp + kp.pp_off;
    PP pk_next;
    if constexpr (kPrefetch) pk_next = kpp[0];
    for (int ip = ip0; ip < ip1; ++ip) {
        const PP pb = pp[bp.pp_off + ip];
        if (pb.Q * qket_max < thr) break;  // primitive pairs sorted by Q (descending)
        const T oo2p = T(0.5) * pb.invp;
        HermiteE<T, LA, LB> Ex, Ey, Ez;
        Ex.build(pb.PAx, pb.PAx + gb_.x, oo2p);
        Ey.build(pb.PAy, pb.PAy + gb_.y, oo2p);
        Ez.build(pb.PAz, pb.PAz + gb_.z, oo2p);
        for (int jq = 0; jq < kp.pp_n; ++jq) {
            PP pk;
            if constexpr (kPrefetch) {
                pk = pk_next;
                pk_next = kpp[jq + 1 < kp.pp_n ? jq + 1 : 0];
            } else {
                pk = kpp[jq];
            }
            if (pb.Q * pk.Q < thr) {
                if constexpr (kPrefetch) pk_next = kpp[0];
                break;
            }
            ++count;
            T e[3][PC];
            {
                const T oo2q = T(0.5) * pk.invp;
                HermiteE<T, LC, LD> Fx, Fy, Fz;
                Fx.build(pk.PAx, pk.PAx + gk_.x, oo2q);
                Fy.build(pk.PAy, pk.PAy + gk_.y, oo2q);
                Fz.build(pk.PAz, pk.PAz + gk_.z, oo2q);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const HermiteE<T, LC, LD>& F = (k == 0) ? Fx : ((k == 1) ? Fy : Fz);
#pragma unroll
                    for (int t = 0; t < PC; ++t) e[k][t] = T(0);
#pragma unroll
                    for (int i = 0; i <= LC; ++i)
#pragma unroll
                        for (int j = 0; j <= LD; ++j) {
                            if (i != c[k] || j != d[k]) continue;
#pragma unroll
                            for (int t = 0; t <= i + j; ++t) e[k][t] = (t & 1) ? -F.e[i][j][t] : F.e[i][j][t];
                        }
                }
            }
            const T rr = fast_rsqrt(pb.p + pk.p);
            const T rho = pb.p * pk.p * (rr * rr);
            const T X = pb.Px - pk.Px, Y = pb.Py - pk.Py, Z = pb.Pz - pk.Pz;
            T Fs[LT + 1];
            BoysEval<T>::template run<LT>(rho * (X * X + Y * Y + Z * Z), boys_table, Fs);
            T scale = pb.KoP * pk.KoP * rr;
            const T m2rho = T(-2) * rho;
#pragma unroll
            for (int n = 0; n <= LT; ++n) { Fs[n] *= scale; scale *= m2rho; }
            // z stage (v <= LAB), then y stage (u + v <= LAB), into the same buffer layout
            T zb[NT], yb[NT];
            {
                HermiteR<T, LT> R;
                R.build(Fs, X, Y, Z);
#pragma unroll
                for (int v = 0; v <= LAB; ++v)
#pragma unroll
                    for (int t = 0; t + v <= LT; ++t)
#pragma unroll
                        for (int u = 0; t + u + v <= LT; ++u) {
                            T acc = T(0);
#pragma unroll
                            for (int f = 0; f < PC; ++f)
                                if (t + u + v + f <= LT) acc += e[2][f] * R(t, u, v + f);
                            zb[hx(t, u, v)] = acc;
                        }
            }
#pragma unroll
            for (int u = 0; u <= LAB; ++u)
#pragma unroll
                for (int v = 0; u + v <= LAB; ++v)
#pragma unroll
                    for (int t = 0; t + u + v <= LT; ++t) {
                        T acc = T(0);
#pragma unroll
                        for (int g = 0; g < PC; ++g)
                            if (t + u + g + v <= LT) acc += e[1][g] * zb[hx(t, u + g, v)];
                        yb[hx(t, u, v)] = acc;
                    }
            T xh[NX];
#pragma unroll
            for (int t = 0; t <= LAB; ++t)
#pragma unroll
                for (int u = 0; u + t <= LAB; ++u)
#pragma unroll
                    for (int v = 0; v + u + t <= LAB; ++v) {
                        T acc = T(0);
#pragma unroll
                        for (int a = 0; a < PC; ++a)
                            if (t + a + u + v <= LT) acc += e[0][a] * yb[hx(t + a, u, v)];
                        xh[hx(t, u, v)] = acc;
                    }
            // bra contraction
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int ib = 0; ib < NB; ++ib) {
                    const int ax = cart_exp(LA, ia, 0), ay = cart_exp(LA, ia, 1), az = cart_exp(LA, ia, 2);
                    const int bx = cart_exp(LB, ib, 0), by = cart_exp(LB, ib, 1), bz = cart_exp(LB, ib, 2);
                    T acc = T(0);
#pragma unroll
                    for (int t = 0; t <= ax + bx; ++t)
#pragma unroll
                        for (int u = 0; u <= ay + by; ++u)
#pragma unroll
                            for (int v = 0; v <= az + bz; ++v)
                                acc += Ex.e[ax][bx][t] * Ey.e[ay][by][u] * Ez.e[az][bz][v] * xh[hx(t, u, v)];
                    I[ia * NB + ib] += acc;
                }
        }
    }
    return count;
}

template <class T, int LA, int LB, int LC, int LD>
struct ClassColumn {
    static constexpr int kNAB = ncart(LA) * ncart(LB);
    static constexpr int kNA = ncart(LA), kNB = ncart(LB), kND = ncart(LD);  // compile-time digestion bounds
    __device__ static int eval(const ShellPairDev& bp, const ShellPairDev& kp, int cd, int ip0, int ip1,
                               const typename FockTypes<T>::PP* __restrict__ pp, const T* __restrict__ boys, T thr,
                               T* I)
    {
        return quartet_column_ct<T, LA, LB, LC, LD>(bp, kp, cd, ip0, ip1, pp, boys, thr, I);
    }
};

// FP32: compiled for 4 resident blocks per SM (128 registers; the latency-bound FP32 tier
// gains more from warps than it loses to the extra spills: mixed SCF 3.04-3.29 -> 2.93
// ms/iter in an A/B on one box); FP64 (pipe-bound) keeps the compiler's choice
template <class T, class Column>
__global__ void __launch_bounds__(kFockThreads, (sizeof(T) == 4 ? 4 : 1)) column_kernel(const FockClassLaunch L, int ncd)
{
    using PP = typename FockTypes<T>::PP;
    const long long total = L.off[L.nentry];
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((total + 31) >> 5) * ncd;
    const long long warp_stride = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
    long long prim_quartets = 0, contracted = 0;
    T I[Column::kNAB];

    for (long long wid = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; wid < nwarps;
         wid += warp_stride) {
        const int cd = static_cast<int>(wid % ncd);
        const long long w = (wid / ncd) * 32 + lane;
        bool active = w < total;
        int bra = -1, ket = -1, prim = -1;
        ShellPairDev bp{}, kp{};
        T fsym = T(0);
        const int e = find_entry_warp(L.off, L.nentry, (wid / ncd) * 32, w, total);
        if (active) {
            bra = __ldg(L.entry_bra + e);
            prim = entry_prim_range(L, e);
            ket = L.ket_base + __ldg(L.entry_lo + e) + static_cast<int>(w - __ldg(L.off + e));
            if (negligible_quartet(L, bra, ket)) {
                active = false;
                bra = ket = -1;
            }
        }
        if (active) {
            bp = L.pairs[bra];
            kp = L.pairs[ket];
            fsym = T(1);
            if (bp.A == bp.B) fsym *= T(0.5);
            if (kp.A == kp.B) fsym *= T(0.5);
            if (bra == ket) fsym *= T(0.5);
            const int ip0 = prim < 0 ? 0 : (prim & 0xffff), ip1 = prim < 0 ? bp.pp_n : (prim >> 16);
            const int pq = Column::eval(bp, kp, cd, ip0, ip1, static_cast<const PP*>(L.prim_pairs),
                                        static_cast<const T*>(L.boys_table), static_cast<T>(L.schwarz_threshold), I);
            if (cd == 0) {
                prim_quartets += pq;
                if (ip0 == 0) ++contracted;  // a quartet split over entries counts once
            }
        } else {
            for (int ab = 0; ab < Column::kNAB; ++ab) I[ab] = T(0);
        }
        // molecule block of this quartet (bra and ket pairs share it)
        const int N = active ? bp.mn : L.num_basis;
        const T* __restrict__ Dp = static_cast<const T*>(L.density) + (active ? bp.mbase : 0);
        T* __restrict__ Jp = TierTypes<T>::J(L) + (active ? bp.mbase : 0);
        T* __restrict__ Kp = TierTypes<T>::K(L) + (active ? bp.mbase : 0);
        // with a compile-time class every digestion bound is a constant, so the
        // loops unroll and I stays in registers
        constexpr bool kCT = Column::kNA > 0;
        const int na = kCT ? Column::kNA : ncart(bp.la), nb = kCT ? Column::kNB : ncart(bp.lb);
        const int nd = kCT ? Column::kND : ncart(kp.lb);
        const int ic = cd / (nd > 0 ? nd : 1), id = cd % (nd > 0 ? nd : 1);
        const int c = kp.bfA + ic, d = kp.bfB + id;
        // J'_ab (partial over cd): warp-reduced when the bra is warp-uniform
        const int bra0 = __shfl_sync(0xffffffffu, bra, 0);
        const bool uniform_bra = __all_sync(0xffffffffu, (!active) || bra == bra0) && bra0 >= 0;
        const int na0 = kCT ? Column::kNA : __shfl_sync(0xffffffffu, na, 0);
        const int nb0 = kCT ? Column::kNB : __shfl_sync(0xffffffffu, nb, 0);
        const int bfA0 = __shfl_sync(0xffffffffu, bp.bfA, 0), bfB0 = __shfl_sync(0xffffffffu, bp.bfB, 0);
        const int N0 = __shfl_sync(0xffffffffu, N, 0), mbase0 = __shfl_sync(0xffffffffu, active ? bp.mbase : 0, 0);
        T* __restrict__ Jp0 = TierTypes<T>::J(L) + mbase0;
        const T dcd = active ? Dp[c * N + d] : T(0);
        if (uniform_bra) {
#pragma unroll
            for (int ab = 0; ab < na0 * nb0; ++ab) {
                const T s = warp_sum(dcd * I[ab] * fsym);
                if (lane == 0) atomicAdd(&Jp0[(bfA0 + ab / nb0) * N0 + bfB0 + ab % nb0], s);
            }
        } else if (active) {
#pragma unroll
            for (int ab = 0; ab < na * nb; ++ab)
                atomicAdd(&Jp[(bp.bfA + ab / nb) * N + bp.bfB + ab % nb], dcd * I[ab] * fsym);
        }
        if (!active) continue;
        T jcd = T(0);
#pragma unroll
        for (int ia = 0; ia < na; ++ia)
#pragma unroll
            for (int ib = 0; ib < nb; ++ib) jcd += Dp[(bp.bfA + ia) * N + bp.bfB + ib] * I[ia * nb + ib];
        atomicAdd(&Jp[c * N + d], jcd * fsym);
#pragma unroll
        for (int ia = 0; ia < na; ++ia) {
            const int a = bp.bfA + ia;
            T kac = T(0), kad = T(0);
#pragma unroll
            for (int ib = 0; ib < nb; ++ib) {
                const int b = bp.bfB + ib;
                kac += Dp[b * N + d] * I[ia * nb + ib];
                kad += Dp[b * N + c] * I[ia * nb + ib];
            }
            atomicAdd(&Kp[a * N + c], kac * fsym);
            atomicAdd(&Kp[a * N + d], kad * fsym);
        }
#pragma unroll
        for (int ib = 0; ib < nb; ++ib) {
            const int b = bp.bfB + ib;
            T kbd = T(0), kbc = T(0);
#pragma unroll
            for (int ia = 0; ia < na; ++ia) {
                const int a = bp.bfA + ia;
                kbd += Dp[a * N + c] * I[ia * nb + ib];
                kbc += Dp[a * N + d] * I[ia * nb + ib];
            }
            atomicAdd(&Kp[b * N + d], kbd * fsym);
            atomicAdd(&Kp[b * N + c], kbc * fsym);
        }
    }
    unsigned long long pq = static_cast<unsigned long long>(prim_quartets);
    unsigned long long cq = static_cast<unsigned long long>(contracted);
    for (int o = 16; o > 0; o >>= 1) {
        pq += __shfl_xor_sync(0xffffffffu, pq, o);
        cq += __shfl_xor_sync(0xffffffffu, cq, o);
    }
    if (lane == 0 && (pq || cq)) {
        atomicAdd(L.counters, pq);
        atomicAdd(L.counters + 1, cq);
    }
}


}  // namespace fock_column
}  // namespace gb
