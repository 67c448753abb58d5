// Direct (integral-direct) Fock build: Schwarz-screened McMurchie-Davidson
// ERIs fused with the J/K contraction.  No ERI tensor is stored.
//
// Work decomposition: for one quartet class (bra shell-pair class (LA,LB),
// ket class (LC,LD)) a thread evaluates one contracted shell quartet (AB|CD)
// with every loop unrolled at compile time; classes whose block of ncart^4
// integrals exceeds the register budget (FockSplit) run in the generic kernel
// of fock_generic.cu instead, one ket component pair per thread.  The thread
// loops over the primitive
// quartets that pass the reference's primitive Schwarz test
// (src/int2e.cu:1677-1680), accumulates its integrals in registers and
// digests them into J' and K' with the 8-fold permutational symmetry:
//     J'_ab += D'_cd v   J'_cd += D'_ab v
//     K'_ac += D'_bd v   K'_bd += D'_ac v   K'_ad += D'_bc v   K'_bc += D'_ad v
// where v = f (ab|cd)', f = (A==B ? 1/2 : 1)(C==D ? 1/2 : 1)(AB==CD ? 1/2 : 1).
// The finishing kernel forms J = 2(J' + J'^T), K = K' + K'^T.
//
// (ab|cd)' omits the per-basis-function factors s_i = cgto_i * component_i;
// the caller passes D' = s D s and scales the result back, which also
// reproduces the reference's CGTO convention (include/basis_set.hpp:106-137).
//
// Items of a class are laid out as a flat list: entry e (a bra pair) owns kets
// [lo[e], lo[e] + off[e+1] - off[e]).  A warp whose lanes all share one bra
// reduces its J'_ab sums with shuffles before a single atomic.
#pragma once
#include "md_math.cuh"
#include "engine_types.hpp"

namespace gb {

constexpr int kFockThreads = 128;

template <class T>
struct FockTypes;
template <>
struct FockTypes<double> {
    using PP = PrimPair64;
};
template <>
struct FockTypes<float> {
    using PP = PrimPair32;
};

// Threads per contracted quartet: 1 (fully unrolled kernel), or one per ket
// component pair (generic kernel) for the classes whose unrolled form would
// spill heavily: measured with -Xptxas -v, FP64 blocks above 162 integrals or a
// (dd| bra with ket components (10 KB of spills), FP32 blocks above 162
// ((dp|dp) and (dd|pp) spill about 3 KB and ran slower than the generic path).
template <class T, int LA, int LB, int LC, int LD>
struct FockSplit {
    static constexpr int NAB = ncart(LA) * ncart(LB), NCD = ncart(LC) * ncart(LD);
    static constexpr bool kDDBra = (LA == 2 && LB == 2);
    static constexpr bool kLarge =
        sizeof(T) == 8 ? ((NAB * NCD > 162) || (kDDBra && NCD > 1)) : (NAB * NCD > 162);
    static constexpr int value = kLarge ? NCD : 1;
};

__device__ __forceinline__ int find_entry(const long long* __restrict__ off, int n, long long w)
{
    // largest e in [0, n) with off[e] <= w
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= w) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// find_entry for the 32 consecutive items wbase .. wbase + 31 of a warp (all lanes
// call it): lanes 0 and 1 bisect the whole list for the warp's first and last
// items, then each lane bisects between those two entries (empty entries of a
// split list included), which replaces a dozen dependent global loads per lane
// by a few L1-resident ones.
__device__ __forceinline__ int find_entry_warp(const long long* __restrict__ off, int n, long long wbase,
                                               long long w, long long total)
{
    const int lane = threadIdx.x & 31;
    int eb = 0;
    if (lane < 2) eb = find_entry(off, n, lane == 0 ? wbase : min(wbase + 31, total - 1));
    const int e0 = __shfl_sync(0xffffffffu, eb, 0);
    const int e1 = __shfl_sync(0xffffffffu, eb, 1);
    if (w >= total) return e0;
    int lo = e0, hi = e1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= w) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double fast_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float fast_rsqrt(float x) { return rsqrtf(x); }

// Pair geometry in the arithmetic type of the tier (A-B and the largest
// primitive bound), read without conversions.
struct PairGeom64 {
    double x, y, z, qmax;
    __device__ __forceinline__ explicit PairGeom64(const ShellPairDev& p) : x(p.ABx), y(p.ABy), z(p.ABz), qmax(p.Qmax) {}
};
struct PairGeom32 {
    float x, y, z, qmax;
    __device__ __forceinline__ explicit PairGeom32(const ShellPairDev& p)
        : x(p.fABx), y(p.fABy), z(p.fABz), qmax(p.fQmax) {}
};
template <class T>
struct TierTypes;
template <>
struct TierTypes<double> {
    using Geom = PairGeom64;
    __device__ __forceinline__ static double* J(const FockClassLaunch& L) { return L.J; }
    __device__ __forceinline__ static double* K(const FockClassLaunch& L) { return L.K; }
};
template <>
struct TierTypes<float> {
    using Geom = PairGeom32;
    // the FP32 tier accumulates in FP32 (merged into FP64 by the finishing kernel)
    __device__ __forceinline__ static float* J(const FockClassLaunch& L) { return L.J32; }
    __device__ __forceinline__ static float* K(const FockClassLaunch& L) { return L.K32; }
};

// Accumulates the ket component pairs [CD0, CD1) of the contracted quartet
// (AB|CD)' into I[ab][cd - CD0], over the primitive quartets of the bra's
// primitive pairs [ip0, ip1) that pass the primitive Schwarz test.  Returns the
// number of primitive quartets.
template <class T, int LA, int LB, int LC, int LD, int CD0, int CD1>
__device__ __forceinline__ int quartet_block(const ShellPairDev& bp, const ShellPairDev& kp, int ip0, int ip1,
                                             const typename FockTypes<T>::PP* __restrict__ pp,
                                             const T* __restrict__ boys_table, T thr,
                                             T (&I)[ncart(LA) * ncart(LB)][CD1 - CD0])
{
    using PP = typename FockTypes<T>::PP;
    constexpr int NB = ncart(LB), ND = ncart(LD);
    constexpr int LAB = LA + LB, LCD = LC + LD, LT = LAB + LCD;
    int count = 0;
    const typename TierTypes<T>::Geom gb_(bp), gk_(kp);
    const T qket_max = gk_.qmax;
    const T abx = gb_.x, aby = gb_.y, abz = gb_.z;
    const T cdx = gk_.x, cdy = gk_.y, cdz = gk_.z;
    // FP32 tier (latency-bound): the next ket primitive-pair record is loaded one
    // iteration ahead (wrapping to the first for the next bra primitive)
    constexpr bool kPrefetch = sizeof(T) == 4;
    const PP* __restrict__ kpp = pp + kp.pp_off;
    PP pk_next;
    if constexpr (kPrefetch) pk_next = kpp[0];
    for (int ip = ip0; ip < ip1; ++ip) {
        const PP pb = pp[bp.pp_off + ip];
        // the primitive pairs of a shell pair are sorted by Q (descending), so the
        // first primitive quartet that fails the Schwarz test ends its loop
        if (pb.Q * qket_max < thr) break;
        const T p = pb.p;
        HermiteE<T, LA, LB> Ex, Ey, Ez;
        const T oo2p = T(0.5) * pb.invp;
        Ex.build(pb.PAx, pb.PAx + abx, oo2p);
        Ey.build(pb.PAy, pb.PAy + aby, oo2p);
        Ez.build(pb.PAz, pb.PAz + abz, oo2p);
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
            const T q = pk.p;
            HermiteE<T, LC, LD> Fx, Fy, Fz;
            const T oo2q = T(0.5) * pk.invp;
            Fx.build(pk.PAx, pk.PAx + cdx, oo2q);
            Fy.build(pk.PAy, pk.PAy + cdy, oo2q);
            Fz.build(pk.PAz, pk.PAz + cdz, oo2q);
            // rho = pq/(p+q); prefactor K_ab K_cd / (p q sqrt(p+q)) with K/p stored
            const T r = fast_rsqrt(p + q);
            const T rho = p * q * (r * r);
            const T X = pb.Px - pk.Px, Y = pb.Py - pk.Py, Z = pb.Pz - pk.Pz;
            T Fs[LT + 1];
            BoysEval<T>::template run<LT>(rho * (X * X + Y * Y + Z * Z), boys_table, Fs);
            T scale = pb.KoP * pk.KoP * r;
            const T m2rho = T(-2) * rho;
#pragma unroll
            for (int n = 0; n <= LT; ++n) { Fs[n] *= scale; scale *= m2rho; }
            HermiteR<T, LT> R;
            R.build(Fs, X, Y, Z);
#pragma unroll
            for (int cd = CD0; cd < CD1; ++cd) {
                const int ic = cd / ND, id = cd % ND;
                const int cx = cart_exp(LC, ic, 0), cy = cart_exp(LC, ic, 1), cz = cart_exp(LC, ic, 2);
                const int dx = cart_exp(LD, id, 0), dy = cart_exp(LD, id, 1), dz = cart_exp(LD, id, 2);
                // ket contraction into the bra Hermite index
                T Xh[nherm(LAB)];
#pragma unroll
                for (int t = 0; t <= LAB; ++t)
#pragma unroll
                    for (int u = 0; u + t <= LAB; ++u)
#pragma unroll
                        for (int v = 0; v + u + t <= LAB; ++v) {
                            T s = T(0);
#pragma unroll
                            for (int tau = 0; tau <= LCD; ++tau) {
                                if (tau > cx + dx) continue;
#pragma unroll
                                for (int nu = 0; nu <= LCD; ++nu) {
                                    if (nu > cy + dy) continue;
                                    const T exy = Fx.e[cx][dx][tau] * Fy.e[cy][dy][nu];
#pragma unroll
                                    for (int phi = 0; phi <= LCD; ++phi) {
                                        if (phi > cz + dz) continue;
                                        const T c = exy * Fz.e[cz][dz][phi];
                                        const T rv = R(t + tau, u + nu, v + phi);
                                        if ((tau + nu + phi) & 1) s -= c * rv; else s += c * rv;
                                    }
                                }
                            }
                            Xh[hermite_index(t, u, v)] = s;
                        }
                // bra contraction
#pragma unroll
                for (int ia = 0; ia < ncart(LA); ++ia) {
#pragma unroll
                    for (int ib = 0; ib < NB; ++ib) {
                        const int ax = cart_exp(LA, ia, 0), ay = cart_exp(LA, ia, 1), az = cart_exp(LA, ia, 2);
                        const int bx = cart_exp(LB, ib, 0), by = cart_exp(LB, ib, 1), bz = cart_exp(LB, ib, 2);
                        T s = T(0);
#pragma unroll
                        for (int t = 0; t <= LAB; ++t) {
                            if (t > ax + bx) continue;
#pragma unroll
                            for (int u = 0; u <= LAB; ++u) {
                                if (u > ay + by) continue;
                                const T exy = Ex.e[ax][bx][t] * Ey.e[ay][by][u];
#pragma unroll
                                for (int v = 0; v <= LAB; ++v) {
                                    if (v > az + bz) continue;
                                    s += exy * Ez.e[az][bz][v] * Xh[hermite_index(t, u, v)];
                                }
                            }
                        }
                        I[ia * NB + ib][cd - CD0] += s;
                    }
                }
            }
        }
    }
    return count;
}

struct QuartetRef {
    int bra, ket;
    bool active;
    int prim;  // bra primitive-pair range first | (end << 16), or -1 for all
};

// bra primitive-pair range [ip0, ip1) of an entry (all of the bra's when the list has none)
__device__ __forceinline__ int entry_prim_range(const FockClassLaunch& L, int e)
{
    return L.entry_prim ? __ldg(L.entry_prim + e) : -1;
}

// Density-weighted screening of one contracted quartet (incremental builds):
// true when Qs_ab Qs_cd times the largest |dD| over the six shell blocks the
// quartet reads (AB, CD, AC, AD, BC, BD) is below the cut.
__device__ __forceinline__ bool negligible_quartet(const FockClassLaunch& L, int bra, int ket)
{
    const ShellPairDev* __restrict__ P = L.pairs;
    // batches: quartets of molecules that have converged are not built again
    if (L.mol_active && !L.mol_active[L.shell_mol[P[bra].A]]) return true;
    if (!L.block_dmax) return false;
    const int A = P[bra].A, B = P[bra].B, C = P[ket].A, D = P[ket].B;
    const int ns = L.nshell;
    const float* __restrict__ bd = L.block_dmax;
    const float dm = fmaxf(fmaxf(__ldg(bd + A * ns + B), __ldg(bd + C * ns + D)),
                           fmaxf(fmaxf(__ldg(bd + A * ns + C), __ldg(bd + A * ns + D)),
                                 fmaxf(__ldg(bd + B * ns + C), __ldg(bd + B * ns + D))));
    return P[bra].Qs * P[ket].Qs * static_cast<double>(dm) < L.skip_cut;
}

// Evaluates and digests ket components [CD0, CD1) of one quartet per lane.
template <class T, int LA, int LB, int LC, int LD, int CD0, int CD1>
__device__ __forceinline__ void process_quartet(const FockClassLaunch& L, const QuartetRef q, int lane,
                                                long long& prim_quartets)
{
    using PP = typename FockTypes<T>::PP;
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NCH = CD1 - CD0;
    int N = L.num_basis;
    int mbase = 0;

    T I[NA * NB][NCH];
#pragma unroll
    for (int i = 0; i < NA * NB; ++i)
#pragma unroll
        for (int j = 0; j < NCH; ++j) I[i][j] = T(0);

    int bfA = 0, bfB = 0, bfC = 0, bfD = 0;
    T fsym = T(0);
    if (q.active) {
        const ShellPairDev bp = L.pairs[q.bra];
        const ShellPairDev kp = L.pairs[q.ket];
        bfA = bp.bfA; bfB = bp.bfB; bfC = kp.bfA; bfD = kp.bfB;
        mbase = bp.mbase;  // bra and ket pairs belong to the same molecule
        N = bp.mn;
        fsym = T(1);
        if (bp.A == bp.B) fsym *= T(0.5);
        if (kp.A == kp.B) fsym *= T(0.5);
        if (q.bra == q.ket) fsym *= T(0.5);
        const int ip0 = q.prim < 0 ? 0 : (q.prim & 0xffff), ip1 = q.prim < 0 ? bp.pp_n : (q.prim >> 16);
        prim_quartets += quartet_block<T, LA, LB, LC, LD, CD0, CD1>(
            bp, kp, ip0, ip1, static_cast<const PP*>(L.prim_pairs), static_cast<const T*>(L.boys_table),
            static_cast<T>(L.schwarz_threshold), I);
    }

    const T* __restrict__ Dp = static_cast<const T*>(L.density) + mbase;
    T* __restrict__ Jp = TierTypes<T>::J(L) + mbase;
    T* __restrict__ Kp = TierTypes<T>::K(L) + mbase;
    const int bra0 = __shfl_sync(0xffffffffu, q.bra, 0);
    const bool uniform_bra = __all_sync(0xffffffffu, (!q.active) || q.bra == bra0) && bra0 >= 0;
    // J'_ab += sum_cd D'_cd v  (a partial sum when the thread holds a component chunk)
    {
        T dcd[NCH];
#pragma unroll
        for (int cd = CD0; cd < CD1; ++cd)
            dcd[cd - CD0] = q.active ? Dp[(bfC + cd / ND) * N + bfD + cd % ND] : T(0);
        const int bfA0 = __shfl_sync(0xffffffffu, bfA, 0), bfB0 = __shfl_sync(0xffffffffu, bfB, 0);
        const int N0 = __shfl_sync(0xffffffffu, N, 0), mbase0 = __shfl_sync(0xffffffffu, mbase, 0);
        T* __restrict__ Jp0 = TierTypes<T>::J(L) + mbase0;
#pragma unroll
        for (int ab = 0; ab < NA * NB; ++ab) {
            T s = T(0);
#pragma unroll
            for (int j = 0; j < NCH; ++j) s += dcd[j] * I[ab][j];
            s *= fsym;
            if (uniform_bra) {
                s = warp_sum(s);
                if (lane == 0) atomicAdd(&Jp0[(bfA0 + ab / NB) * N0 + bfB0 + ab % NB], s);
            } else if (q.active) {
                atomicAdd(&Jp[(bfA + ab / NB) * N + bfB + ab % NB], s);
            }
        }
    }
    if (!q.active) return;
    T dab[NA * NB];
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
        for (int ib = 0; ib < NB; ++ib) dab[ia * NB + ib] = Dp[(bfA + ia) * N + bfB + ib];
    // J'_cd += sum_ab D'_ab v
#pragma unroll
    for (int cd = CD0; cd < CD1; ++cd) {
        T s = T(0);
#pragma unroll
        for (int ab = 0; ab < NA * NB; ++ab) s += dab[ab] * I[ab][cd - CD0];
        atomicAdd(&Jp[(bfC + cd / ND) * N + bfD + cd % ND], s * fsym);
    }
    // K'_ac += sum_bd D'_bd v ; K'_ad += sum_bc D'_bc v
#pragma unroll
    for (int ia = 0; ia < NA; ++ia) {
#pragma unroll
        for (int ic = 0; ic < NC; ++ic) {
            if (ic * ND + ND <= CD0 || ic * ND >= CD1) continue;  // c not held by this thread
            T s = T(0);
#pragma unroll
            for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                for (int id = 0; id < ND; ++id) {
                    const int cd = ic * ND + id;
                    if (cd < CD0 || cd >= CD1) continue;
                    s += Dp[(bfB + ib) * N + bfD + id] * I[ia * NB + ib][cd - CD0];
                }
            atomicAdd(&Kp[(bfA + ia) * N + bfC + ic], s * fsym);
        }
#pragma unroll
        for (int id = 0; id < ND; ++id) {
            bool held = false;
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) held |= (ic * ND + id >= CD0 && ic * ND + id < CD1);
            if (!held) continue;
            T s = T(0);
#pragma unroll
            for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                for (int ic = 0; ic < NC; ++ic) {
                    const int cd = ic * ND + id;
                    if (cd < CD0 || cd >= CD1) continue;
                    s += Dp[(bfB + ib) * N + bfC + ic] * I[ia * NB + ib][cd - CD0];
                }
            atomicAdd(&Kp[(bfA + ia) * N + bfD + id], s * fsym);
        }
    }
    // K'_bd += sum_ac D'_ac v ; K'_bc += sum_ad D'_ad v
#pragma unroll
    for (int ib = 0; ib < NB; ++ib) {
#pragma unroll
        for (int id = 0; id < ND; ++id) {
            bool held = false;
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) held |= (ic * ND + id >= CD0 && ic * ND + id < CD1);
            if (!held) continue;
            T s = T(0);
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int ic = 0; ic < NC; ++ic) {
                    const int cd = ic * ND + id;
                    if (cd < CD0 || cd >= CD1) continue;
                    s += Dp[(bfA + ia) * N + bfC + ic] * I[ia * NB + ib][cd - CD0];
                }
            atomicAdd(&Kp[(bfB + ib) * N + bfD + id], s * fsym);
        }
#pragma unroll
        for (int ic = 0; ic < NC; ++ic) {
            if (ic * ND + ND <= CD0 || ic * ND >= CD1) continue;
            T s = T(0);
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int id = 0; id < ND; ++id) {
                    const int cd = ic * ND + id;
                    if (cd < CD0 || cd >= CD1) continue;
                    s += Dp[(bfA + ia) * N + bfD + id] * I[ia * NB + ib][cd - CD0];
                }
            atomicAdd(&Kp[(bfB + ib) * N + bfC + ic], s * fsym);
        }
    }
}

// Resident blocks per SM the FP32 class kernels are compiled for (their loads are the
// latency they wait on, so occupancy buys more than registers): 8 (64 registers) for the
// classes of at most 9 integrals, 5 (96) up to 27, 3 (168) up to 54; the larger FP32
// classes and the FP64 kernels (bound by the FP64 pipe) keep the compiler's choice.
template <class T, int LA, int LB, int LC, int LD>
struct FockMinBlocks {
    static constexpr int NI = ncart(LA) * ncart(LB) * ncart(LC) * ncart(LD);
    static constexpr int value = sizeof(T) == 8 ? 1 : (NI <= 9 ? 8 : (NI <= 27 ? 5 : (NI <= 54 ? 3 : 1)));
};

template <class T, int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(kFockThreads, (FockMinBlocks<T, LA, LB, LC, LD>::value))
fock_direct_kernel(const FockClassLaunch launch)
{
    static_assert(FockSplit<T, LA, LB, LC, LD>::value == 1, "large classes use the generic kernel");
    constexpr int NCD = ncart(LC) * ncart(LD);
    const long long total = launch.off[launch.nentry];
    const int lane = threadIdx.x & 31;
    const long long nwarps = (total + 31) >> 5;
    const long long warp_stride = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
    long long prim_quartets = 0, contracted = 0;

    for (long long wid = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; wid < nwarps;
         wid += warp_stride) {
        const long long w = wid * 32 + lane;
        QuartetRef q{-1, -1, w < total, -1};
        const int e = find_entry_warp(launch.off, launch.nentry, wid * 32, w, total);
        if (q.active) {
            q.bra = __ldg(launch.entry_bra + e);
            q.prim = entry_prim_range(launch, e);
            q.ket = launch.ket_base + __ldg(launch.entry_lo + e) + static_cast<int>(w - __ldg(launch.off + e));
            if (negligible_quartet(launch, q.bra, q.ket)) {
                q.active = false;  // screened lanes look like lanes past the end (bra = -1)
                q.bra = q.ket = -1;
            } else if (q.prim < 0 || (q.prim & 0xffff) == 0) {
                ++contracted;  // a quartet split over entries counts once
            }
        }
        process_quartet<T, LA, LB, LC, LD, 0, NCD>(launch, q, lane, prim_quartets);
    }
    // statistics (one atomic per warp): [0] primitive quartets, [1] contracted quartets
    unsigned long long pq = static_cast<unsigned long long>(prim_quartets);
    unsigned long long cq = static_cast<unsigned long long>(contracted);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pq += __shfl_xor_sync(0xffffffffu, pq, o);
        cq += __shfl_xor_sync(0xffffffffu, cq, o);
    }
    if (lane == 0 && (pq || cq)) {
        atomicAdd(launch.counters, pq);
        atomicAdd(launch.counters + 1, cq);
    }
}

// Classes above the register budget and the stored-ERI tensor: fock_generic.cu
void launch_fock_generic(bool fp32, const FockClassLaunch& launch, int ncd, int grid, cudaStream_t stream);
void launch_eri_generic(const FockClassLaunch& launch, int ncd, const double* scale, double* eri, int grid,
                        cudaStream_t stream);

}  // namespace gb
