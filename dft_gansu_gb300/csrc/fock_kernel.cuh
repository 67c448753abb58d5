// Direct (integral-direct) Fock build: Schwarz-screened McMurchie-Davidson
// ERIs fused with the J/K contraction.  No ERI tensor is stored.
//
// Work decomposition: for one quartet class (bra shell-pair class (LA,LB),
// ket class (LC,LD)) each thread evaluates ONE contracted shell quartet
// (AB|CD): it loops over the primitive quartets that pass the reference's
// primitive Schwarz test (src/int2e.cu:1677-1680), accumulates all
// ncart(LA)*ncart(LB)*ncart(LC)*ncart(LD) integrals in registers and then
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
// [lo[e], lo[e] + off[e+1] - off[e]).  Threads stride over the flat list; a
// warp whose lanes all share one bra reduces its J'_ab sums with shuffles
// before a single atomic.
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

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Accumulates the contracted quartet (AB|CD)' into I[ab][cd] over the
// primitive quartets that pass the reference's primitive Schwarz test.
// Returns the number of primitive quartets evaluated.
template <class T, int LA, int LB, int LC, int LD>
__device__ __forceinline__ int quartet_block(const ShellPairDev& bp, const ShellPairDev& kp,
                                             const typename FockTypes<T>::PP* __restrict__ pp,
                                             const T* __restrict__ boys_table, T thr,
                                             T (&I)[ncart(LA) * ncart(LB)][ncart(LC) * ncart(LD)])
{
    using PP = typename FockTypes<T>::PP;
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int LAB = LA + LB, LCD = LC + LD, LT = LAB + LCD;
    (void)NA;
    int count = 0;
    const T qket_max = static_cast<T>(kp.Qmax);
    const T abx = static_cast<T>(bp.ABx), aby = static_cast<T>(bp.ABy), abz = static_cast<T>(bp.ABz);
    const T cdx = static_cast<T>(kp.ABx), cdy = static_cast<T>(kp.ABy), cdz = static_cast<T>(kp.ABz);
    for (int ip = 0; ip < bp.pp_n; ++ip) {
        const PP pb = pp[bp.pp_off + ip];
        if (pb.Q * qket_max < thr) continue;
        const T p = pb.p;
        HermiteE<T, LA, LB> Ex, Ey, Ez;
        const T oo2p = T(0.5) / p;
        Ex.build(pb.PAx, pb.PAx + abx, oo2p);
        Ey.build(pb.PAy, pb.PAy + aby, oo2p);
        Ez.build(pb.PAz, pb.PAz + abz, oo2p);
        for (int jq = 0; jq < kp.pp_n; ++jq) {
            const PP pk = pp[kp.pp_off + jq];
            if (pb.Q * pk.Q < thr) continue;
            ++count;
            const T q = pk.p;
            HermiteE<T, LC, LD> Fx, Fy, Fz;
            const T oo2q = T(0.5) / q;
            Fx.build(pk.PAx, pk.PAx + cdx, oo2q);
            Fy.build(pk.PAy, pk.PAy + cdy, oo2q);
            Fz.build(pk.PAz, pk.PAz + cdz, oo2q);
            const T pq = p + q;
            const T rho = p * q / pq;
            const T X = pb.Px - pk.Px, Y = pb.Py - pk.Py, Z = pb.Pz - pk.Pz;
            T Fs[LT + 1];
            BoysEval<T>::template run<LT>(rho * (X * X + Y * Y + Z * Z), boys_table, Fs);
            T scale = pb.K * pk.K / (p * q * sqrt(pq));
            const T m2rho = T(-2) * rho;
#pragma unroll
            for (int n = 0; n <= LT; ++n) { Fs[n] *= scale; scale *= m2rho; }
            HermiteR<T, LT> R;
            R.build(Fs, X, Y, Z);
#pragma unroll
            for (int ic = 0; ic < NC; ++ic) {
#pragma unroll
                for (int id = 0; id < ND; ++id) {
                    const int cx = cart_exp(LC, ic, 0), cy = cart_exp(LC, ic, 1), cz = cart_exp(LC, ic, 2);
                    const int dx = cart_exp(LD, id, 0), dy = cart_exp(LD, id, 1), dz = cart_exp(LD, id, 2);
                    // ket contraction into the bra Hermite index
                    T Xh[LAB + 1][LAB + 1][LAB + 1];
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
                                            const T r = R.r[t + tau][u + nu][v + phi];
                                            if ((tau + nu + phi) & 1) s -= c * r; else s += c * r;
                                        }
                                    }
                                }
                                Xh[t][u][v] = s;
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
                                        s += exy * Ez.e[az][bz][v] * Xh[t][u][v];
                                    }
                                }
                            }
                            I[ia * NB + ib][ic * ND + id] += s;
                        }
                    }
                }
            }
        }
    }
    return count;
}

template <class T, int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(kFockThreads)
fock_direct_kernel(const FockClassLaunch launch)
{
    using PP = typename FockTypes<T>::PP;
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);

    const long long total = launch.off[launch.nentry];
    const int lane = threadIdx.x & 31;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    const T* __restrict__ Dp = static_cast<const T*>(launch.density);
    const PP* __restrict__ pp = static_cast<const PP*>(launch.prim_pairs);
    const T* __restrict__ boys_table = static_cast<const T*>(launch.boys_table);
    const T thr = static_cast<T>(launch.schwarz_threshold);
    const int N = launch.num_basis;
    long long prim_quartets = 0, contracted = 0;

    for (long long base = static_cast<long long>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); base < total;
         base += stride) {
        const long long w = base + lane;
        const bool active = w < total;
        int bra = -1, ket = -1;
        if (active) {
            const int e = find_entry(launch.off, launch.nentry, w);
            bra = __ldg(launch.entry_bra + e);
            ket = launch.ket_base + __ldg(launch.entry_lo + e) + static_cast<int>(w - __ldg(launch.off + e));
        }

        T I[NA * NB][NC * ND];
#pragma unroll
        for (int i = 0; i < NA * NB; ++i)
#pragma unroll
            for (int j = 0; j < NC * ND; ++j) I[i][j] = T(0);

        int bfA = 0, bfB = 0, bfC = 0, bfD = 0;
        T fsym = T(0);
        if (active) {
            const ShellPairDev bp = launch.pairs[bra];
            const ShellPairDev kp = launch.pairs[ket];
            bfA = bp.bfA; bfB = bp.bfB; bfC = kp.bfA; bfD = kp.bfB;
            fsym = T(1);
            if (bp.A == bp.B) fsym *= T(0.5);
            if (kp.A == kp.B) fsym *= T(0.5);
            if (bra == ket) fsym *= T(0.5);
            prim_quartets += quartet_block<T, LA, LB, LC, LD>(bp, kp, pp, boys_table, thr, I);
            ++contracted;
        }

        // ------------------------------------------------------- digestion
        double* __restrict__ Jp = launch.J;
        double* __restrict__ Kp = launch.K;
        const int bra0 = __shfl_sync(0xffffffffu, bra, 0);
        const bool uniform_bra = __all_sync(0xffffffffu, (!active) || bra == bra0) && bra0 >= 0;
        // J'_ab += sum_cd D'_cd v
        {
            T dcd[NC * ND];
#pragma unroll
            for (int ic = 0; ic < NC; ++ic)
#pragma unroll
                for (int id = 0; id < ND; ++id)
                    dcd[ic * ND + id] = active ? Dp[(bfC + ic) * N + bfD + id] : T(0);
            const int bfA0 = __shfl_sync(0xffffffffu, bfA, 0), bfB0 = __shfl_sync(0xffffffffu, bfB, 0);
#pragma unroll
            for (int ab = 0; ab < NA * NB; ++ab) {
                T s = T(0);
#pragma unroll
                for (int cd = 0; cd < NC * ND; ++cd) s += dcd[cd] * I[ab][cd];
                s *= fsym;
                if (uniform_bra) {
                    s = warp_sum(s);
                    if (lane == 0) atomicAdd(&Jp[(bfA0 + ab / NB) * N + bfB0 + ab % NB], static_cast<double>(s));
                } else if (active) {
                    atomicAdd(&Jp[(bfA + ab / NB) * N + bfB + ab % NB], static_cast<double>(s));
                }
            }
        }
        if (active) {
            // J'_cd += sum_ab D'_ab v
            T dab[NA * NB];
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int ib = 0; ib < NB; ++ib) dab[ia * NB + ib] = Dp[(bfA + ia) * N + bfB + ib];
#pragma unroll
            for (int cd = 0; cd < NC * ND; ++cd) {
                T s = T(0);
#pragma unroll
                for (int ab = 0; ab < NA * NB; ++ab) s += dab[ab] * I[ab][cd];
                atomicAdd(&Jp[(bfC + cd / ND) * N + bfD + cd % ND], static_cast<double>(s * fsym));
            }
            // K'_ac += sum_bd D'_bd v ; K'_bd += sum_ac D'_ac v
            {
                T dbd[NB * ND], dac[NA * NC];
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int id = 0; id < ND; ++id) dbd[ib * ND + id] = Dp[(bfB + ib) * N + bfD + id];
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic) dac[ia * NC + ic] = Dp[(bfA + ia) * N + bfC + ic];
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic) {
                        T s = T(0);
#pragma unroll
                        for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                            for (int id = 0; id < ND; ++id) s += dbd[ib * ND + id] * I[ia * NB + ib][ic * ND + id];
                        atomicAdd(&Kp[(bfA + ia) * N + bfC + ic], static_cast<double>(s * fsym));
                    }
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int id = 0; id < ND; ++id) {
                        T s = T(0);
#pragma unroll
                        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                            for (int ic = 0; ic < NC; ++ic) s += dac[ia * NC + ic] * I[ia * NB + ib][ic * ND + id];
                        atomicAdd(&Kp[(bfB + ib) * N + bfD + id], static_cast<double>(s * fsym));
                    }
            }
            // K'_ad += sum_bc D'_bc v ; K'_bc += sum_ad D'_ad v
            {
                T dbc[NB * NC], dad[NA * ND];
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic) dbc[ib * NC + ic] = Dp[(bfB + ib) * N + bfC + ic];
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int id = 0; id < ND; ++id) dad[ia * ND + id] = Dp[(bfA + ia) * N + bfD + id];
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int id = 0; id < ND; ++id) {
                        T s = T(0);
#pragma unroll
                        for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                            for (int ic = 0; ic < NC; ++ic) s += dbc[ib * NC + ic] * I[ia * NB + ib][ic * ND + id];
                        atomicAdd(&Kp[(bfA + ia) * N + bfD + id], static_cast<double>(s * fsym));
                    }
#pragma unroll
                for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                    for (int ic = 0; ic < NC; ++ic) {
                        T s = T(0);
#pragma unroll
                        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                            for (int id = 0; id < ND; ++id) s += dad[ia * ND + id] * I[ia * NB + ib][ic * ND + id];
                        atomicAdd(&Kp[(bfB + ib) * N + bfC + ic], static_cast<double>(s * fsym));
                    }
            }
        }
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

// Stored-ERI path (the reference's computeERIMatrix, src/gpu_manager.cu:434-517):
// the same contracted quartets, scaled by s_a s_b s_c s_d and written to all
// eight permutations of a dense N^4 tensor ((i*N+j)*N+k)*N+l.  Every element
// is written by exactly one quartet (coincident permutations carry equal
// values), so plain stores suffice.
template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(kFockThreads)
eri_tensor_kernel(const FockClassLaunch launch, const double* __restrict__ scale, double* __restrict__ eri)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    const long long total = launch.off[launch.nentry];
    const long long N = launch.num_basis;
    for (long long w = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; w < total;
         w += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int e = find_entry(launch.off, launch.nentry, w);
        const int bra = __ldg(launch.entry_bra + e);
        const int ket = launch.ket_base + __ldg(launch.entry_lo + e) + static_cast<int>(w - __ldg(launch.off + e));
        const ShellPairDev bp = launch.pairs[bra];
        const ShellPairDev kp = launch.pairs[ket];
        double I[NA * NB][NC * ND];
#pragma unroll
        for (int i = 0; i < NA * NB; ++i)
#pragma unroll
            for (int j = 0; j < NC * ND; ++j) I[i][j] = 0.0;
        quartet_block<double, LA, LB, LC, LD>(bp, kp, static_cast<const PrimPair64*>(launch.prim_pairs),
                                              static_cast<const double*>(launch.boys_table),
                                              launch.schwarz_threshold, I);
        for (int ia = 0; ia < NA; ++ia)
            for (int ib = 0; ib < NB; ++ib)
                for (int ic = 0; ic < NC; ++ic)
                    for (int id = 0; id < ND; ++id) {
                        const long long a = bp.bfA + ia, b = bp.bfB + ib, c = kp.bfA + ic, d = kp.bfB + id;
                        const double v = I[ia * NB + ib][ic * ND + id] * scale[a] * scale[b] * scale[c] * scale[d];
                        eri[((a * N + b) * N + c) * N + d] = v;
                        eri[((b * N + a) * N + c) * N + d] = v;
                        eri[((a * N + b) * N + d) * N + c] = v;
                        eri[((b * N + a) * N + d) * N + c] = v;
                        eri[((c * N + d) * N + a) * N + b] = v;
                        eri[((d * N + c) * N + a) * N + b] = v;
                        eri[((c * N + d) * N + b) * N + a] = v;
                        eri[((d * N + c) * N + b) * N + a] = v;
                    }
    }
}

}  // namespace gb
