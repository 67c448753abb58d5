// Gradient kernels shared by the translation units of the analytic gradient:
// the launch record and the class kernels with compile-time loops (one
// translation unit per arithmetic type instantiates them, so they compile in
// parallel).
#pragma once
#include "engine.hpp"
#include "fock_kernel.cuh"

namespace gb {

constexpr int kGI = kMaxL + 2;             // E table dimension (l + 1 shift)
constexpr int kGT = 2 * (kMaxL + 1) + 1;   // t range
constexpr int kGE = kGI * kGI * kGT;
constexpr int kGL = 4 * kMaxL + 1;         // highest R order
constexpr int kGR = nherm(kGL);
constexpr int kGX = nherm(2 * kMaxL + 1);  // bra Hermite entries with one extra order
constexpr int kGNAB = ncart(kMaxL) * ncart(kMaxL);
constexpr int kGradThreads = 64;

__host__ __device__ constexpr int gidx(int t, int u, int v)
{
    return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

struct GradLaunch {
    FockClassLaunch L;       // work list, pairs, primitive pairs, Boys table, D' of the tier
    const long long* goff;   // nentry+1 prefix offsets of items: (ket, bra primitive pair) per entry
    const int* shell_atom;   // contracted shell -> atom
    double* grad;            // 3 * natom accumulators
    int natom;
    int shared_grad;         // accumulate per block in shared memory (3 * natom doubles)
};

// The same derivative integrals for one quartet class with every loop bound and
// table index a compile-time constant (classes with la + lb + lc + ld <= 4, which
// carry most of the primitive quartets of contracted basis sets): the item's
// ket components (c, d) only select coefficient vectors, zero-padded to the
// class's longest, so the Hermite tables and the separable contraction need
// no index arithmetic.  Work items and accumulation as grad_eri_kernel.
template <class T, int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(kGradThreads) grad_class_kernel(const GradLaunch G)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), ND = ncart(LD), NCD = ncart(LC) * ND;
    constexpr int LAB = LA + LB, LCD = LC + LD, LT = LAB + LCD + 1, LV = LAB + 1;
    constexpr int NH1 = nherm(LV), NT = nherm(LT);
    constexpr int PD = LCD + 2;  // padded length of the ket coefficient vectors
    extern __shared__ double sgrad[];
    const FockClassLaunch& L = G.L;
    if (G.shared_grad) {
        for (int i = threadIdx.x; i < 3 * G.natom; i += blockDim.x) sgrad[i] = 0.0;
        __syncthreads();
    }
    double* const gacc = G.shared_grad ? sgrad : G.grad;
    const long long total = G.goff[L.nentry];
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((total + 31) >> 5) * NCD;
    const long long warp_stride = (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
    using PP = typename FockTypes<T>::PP;
    const T* __restrict__ Dp = static_cast<const T*>(L.density);
    const PP* __restrict__ pp = static_cast<const PP*>(L.prim_pairs);
    const T* __restrict__ boys = static_cast<const T*>(L.boys_table);
    const int N = L.num_basis;
    const T thr = static_cast<T>(L.schwarz_threshold);

    for (long long wid = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; wid < nwarps;
         wid += warp_stride) {
        const int cdi = static_cast<int>(wid % NCD);
        const long long w = (wid / NCD) * 32 + lane;
        const int e = find_entry_warp(G.goff, L.nentry, (wid / NCD) * 32, w, total);
        if (w >= total) continue;
        const int bra = __ldg(L.entry_bra + e);
        const ShellPairDev bp = L.pairs[bra];
        const long long item = w - __ldg(G.goff + e);
        const int pr = __ldg(L.entry_prim + e), nip = (pr >> 16) - (pr & 0xffff);
        const int ip = (pr & 0xffff) + static_cast<int>(item % nip);
        const int ket = L.ket_base + __ldg(L.entry_lo + e) + static_cast<int>(item / nip);
        const ShellPairDev kp = L.pairs[ket];
        const int ic = cdi / ND, id = cdi % ND;
        int c[3], d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) { c[k] = cart_exp(LC, ic, k); d[k] = cart_exp(LD, id, k); }
        const int cf = kp.bfA + ic, df = kp.bfB + id;
        T fsym = T(1);
        if (bp.A == bp.B) fsym *= T(0.5);
        if (kp.A == kp.B) fsym *= T(0.5);
        if (bra == ket) fsym *= T(0.5);
        const T bABx = sizeof(T) == 4 ? static_cast<T>(bp.fABx) : static_cast<T>(bp.ABx);
        const T bABy = sizeof(T) == 4 ? static_cast<T>(bp.fABy) : static_cast<T>(bp.ABy);
        const T bABz = sizeof(T) == 4 ? static_cast<T>(bp.fABz) : static_cast<T>(bp.ABz);
        const T kABx = sizeof(T) == 4 ? static_cast<T>(kp.fABx) : static_cast<T>(kp.ABx);
        const T kABy = sizeof(T) == 4 ? static_cast<T>(kp.fABy) : static_cast<T>(kp.ABy);
        const T kABz = sizeof(T) == 4 ? static_cast<T>(kp.fABz) : static_cast<T>(kp.ABz);
        const T kQmax = sizeof(T) == 4 ? static_cast<T>(kp.fQmax) : static_cast<T>(kp.Qmax);
        // density weights f (4 D_ab D_cd - D_ac D_bd - D_ad D_bc) of this (c, d) column
        const T dcd = Dp[cf * N + df];
        T wcol[NA][NB];
        bool any = false;
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ib = 0; ib < NB; ++ib) {
                const int a = bp.bfA + ia, b = bp.bfB + ib;
                const T v = fsym * (T(4) * Dp[a * N + b] * dcd - Dp[a * N + cf] * Dp[b * N + df] -
                                    Dp[a * N + df] * Dp[b * N + cf]);
                wcol[ia][ib] = v;
                any |= (v != T(0));
            }
        if (!any) continue;
        const PP pb = pp[bp.pp_off + ip];
        if (pb.Q * kQmax < thr) continue;
        const T alpha2 = T(2) * (pb.p - pb.b);
        // bra Hermite densities H0 = sum w E^{ab}, HA_k = sum w (2 alpha E^{a+1_k, b} - a_k E^{a-1_k, b})
        T H0[NH1], HA[3][NH1];
        {
            const T oo2p = T(0.5) * pb.invp;
            HermiteE<T, LA + 1, LB> Ex, Ey, Ez;
            Ex.build(pb.PAx, pb.PAx + bABx, oo2p);
            Ey.build(pb.PAy, pb.PAy + bABy, oo2p);
            Ez.build(pb.PAz, pb.PAz + bABz, oo2p);
#pragma unroll
            for (int h = 0; h < NH1; ++h) { H0[h] = T(0); HA[0][h] = T(0); HA[1][h] = T(0); HA[2][h] = T(0); }
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int ib = 0; ib < NB; ++ib) {
                    const int a[3] = {cart_exp(LA, ia, 0), cart_exp(LA, ia, 1), cart_exp(LA, ia, 2)};
                    const int b[3] = {cart_exp(LB, ib, 0), cart_exp(LB, ib, 1), cart_exp(LB, ib, 2)};
                    const T wv = wcol[ia][ib];
                    T e0[3][LV + 1], e1[3][LV + 1];
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const HermiteE<T, LA + 1, LB>& E = (k == 0) ? Ex : ((k == 1) ? Ey : Ez);
#pragma unroll
                        for (int t = 0; t <= LV; ++t) {
                            e0[k][t] = (t <= a[k] + b[k]) ? E.e[a[k]][b[k]][t] : T(0);
                            T v = (t <= a[k] + b[k] + 1) ? alpha2 * E.e[a[k] + 1][b[k]][t] : T(0);
                            if (a[k] > 0 && t <= a[k] - 1 + b[k]) v -= T(a[k]) * E.e[a[k] > 0 ? a[k] - 1 : 0][b[k]][t];
                            e1[k][t] = v;
                        }
                    }
#pragma unroll
                    for (int t = 0; t <= LV; ++t)
#pragma unroll
                        for (int u = 0; u + t <= LV; ++u)
#pragma unroll
                            for (int v = 0; v + u + t <= LV; ++v) {
                                if (t > a[0] + b[0] + 1 || u > a[1] + b[1] + 1 || v > a[2] + b[2] + 1) continue;
                                const int h = gidx(t, u, v);
                                const T x0 = e0[0][t], y0 = e0[1][u], z0 = e0[2][v];
                                H0[h] += wv * x0 * y0 * z0;
                                HA[0][h] += wv * e1[0][t] * y0 * z0;
                                HA[1][h] += wv * x0 * e1[1][u] * z0;
                                HA[2][h] += wv * x0 * y0 * e1[2][v];
                            }
                }
        }
        T gA[3] = {0, 0, 0}, gP[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
        for (int jq = 0; jq < kp.pp_n; ++jq) {
            const PP pk = pp[kp.pp_off + jq];
            if (pb.Q * pk.Q < thr) break;
            const T gamma2 = T(2) * (pk.p - pk.b);
            const T oo2q = T(0.5) * pk.invp;
            // coefficient vectors of the item's (c, d), (-1)^tau folded in:
            //   e0_k = E^{c_k d_k},  eD_k = 2 gamma E^{c_k+1, d_k} - c_k E^{c_k-1, d_k}
            T e0[3][PD], eD[3][PD];
            {
                HermiteE<T, LC + 1, LD> Fx, Fy, Fz;
                Fx.build(pk.PAx, pk.PAx + kABx, oo2q);
                Fy.build(pk.PAy, pk.PAy + kABy, oo2q);
                Fz.build(pk.PAz, pk.PAz + kABz, oo2q);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const HermiteE<T, LC + 1, LD>& F = (k == 0) ? Fx : ((k == 1) ? Fy : Fz);
#pragma unroll
                    for (int t = 0; t < PD; ++t) { e0[k][t] = T(0); eD[k][t] = T(0); }
#pragma unroll
                    for (int i = 0; i <= LC; ++i)
#pragma unroll
                        for (int j = 0; j <= LD; ++j) {
                            if (i != c[k] || j != d[k]) continue;
#pragma unroll
                            for (int t = 0; t < PD; ++t) {
                                const T sg = (t & 1) ? T(-1) : T(1);
                                if (t <= i + j) e0[k][t] = sg * F.e[i][j][t];
                                T v = (t <= i + 1 + j) ? gamma2 * F.e[i + 1][j][t] : T(0);
                                if (i > 0 && t <= i - 1 + j) v -= T(i) * F.e[i > 0 ? i - 1 : 0][j][t];
                                eD[k][t] = sg * v;
                            }
                        }
                }
            }
            const T rr = fast_rsqrt(pb.p + pk.p);
            const T rho = pb.p * pk.p * rr * rr;
            const T X = pb.Px - pk.Px, Y = pb.Py - pk.Py, Z = pb.Pz - pk.Pz;
            T Fs[LT + 1];
            BoysEval<T>::template run<LT>(rho * (X * X + Y * Y + Z * Z), boys, Fs);
            T scale = pb.KoP * pk.KoP * rr;
#pragma unroll
            for (int n = 0; n <= LT; ++n) { Fs[n] *= scale; scale *= T(-2) * rho; }
            // z stages (R is dead afterwards): z0 with e0_z, zD with eD_z, for v <= LV
            T z0[NT], zD[NT];
            {
                HermiteR<T, LT> R;
                R.build(Fs, X, Y, Z);
#pragma unroll
                for (int v = 0; v <= LV; ++v)
#pragma unroll
                    for (int t = 0; t + v <= LT; ++t)
#pragma unroll
                        for (int u = 0; t + u + v <= LT; ++u) {
                            T a0 = T(0), aD = T(0);
#pragma unroll
                            for (int f = 0; f < PD; ++f)
                                if (t + u + v + f <= LT) {
                                    a0 += e0[2][f] * R(t, u, v + f);
                                    aD += eD[2][f] * R(t, u, v + f);
                                }
                            z0[gidx(t, u, v)] = a0;
                            zD[gidx(t, u, v)] = aD;
                        }
            }
            // y stages for u + v <= LV: y0 (e0_y on z0), yy (eD_y on z0), yz (e0_y on zD)
            T y0[NT], yy[NT], yz[NT];
#pragma unroll
            for (int u = 0; u <= LV; ++u)
#pragma unroll
                for (int v = 0; u + v <= LV; ++v)
#pragma unroll
                    for (int t = 0; t + u + v <= LT; ++t) {
                        T a0 = T(0), ay = T(0), az = T(0);
#pragma unroll
                        for (int g = 0; g < PD; ++g)
                            if (t + u + g + v <= LT) {
                                a0 += e0[1][g] * z0[gidx(t, u + g, v)];
                                ay += eD[1][g] * z0[gidx(t, u + g, v)];
                                az += e0[1][g] * zD[gidx(t, u + g, v)];
                            }
                        y0[gidx(t, u, v)] = a0;
                        yy[gidx(t, u, v)] = ay;
                        yz[gidx(t, u, v)] = az;
                    }
            // x stage with the bra contractions
#pragma unroll
            for (int t = 0; t <= LV; ++t)
#pragma unroll
                for (int u = 0; u + t <= LV; ++u)
#pragma unroll
                    for (int v = 0; v + u + t <= LV; ++v) {
                        T x = T(0);
#pragma unroll
                        for (int a = 0; a < PD; ++a)
                            if (t + a + u + v <= LT) x += e0[0][a] * y0[gidx(t + a, u, v)];
                        const int h = gidx(t, u, v);
                        gA[0] += HA[0][h] * x;
                        gA[1] += HA[1][h] * x;
                        gA[2] += HA[2][h] * x;
                        if (t > 0) gP[0] += H0[gidx(t > 0 ? t - 1 : 0, u, v)] * x;
                        if (u > 0) gP[1] += H0[gidx(t, u > 0 ? u - 1 : 0, v)] * x;
                        if (v > 0) gP[2] += H0[gidx(t, u, v > 0 ? v - 1 : 0)] * x;
                        if (t + u + v <= LAB) {
                            T xx = T(0), xy = T(0), xz = T(0);
#pragma unroll
                            for (int a = 0; a < PD; ++a)
                                if (t + a + u + v <= LT) {
                                    xx += eD[0][a] * y0[gidx(t + a, u, v)];
                                    xy += e0[0][a] * yy[gidx(t + a, u, v)];
                                    xz += e0[0][a] * yz[gidx(t + a, u, v)];
                                }
                            gC[0] += H0[h] * xx;
                            gC[1] += H0[h] * xy;
                            gC[2] += H0[h] * xz;
                        }
                    }
        }
        T gB[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) gB[k] = gP[k] - gA[k];
        const int atA = G.shell_atom[bp.A], atB = G.shell_atom[bp.B], atC = G.shell_atom[kp.A],
                  atD = G.shell_atom[kp.B];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicAdd(&gacc[3 * atA + k], static_cast<double>(gA[k]));
            atomicAdd(&gacc[3 * atB + k], static_cast<double>(gB[k]));
            atomicAdd(&gacc[3 * atC + k], static_cast<double>(gC[k]));
            atomicAdd(&gacc[3 * atD + k], -static_cast<double>(gA[k] + gB[k] + gC[k]));
        }
    }
    if (G.shared_grad) {
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * G.natom; i += blockDim.x)
            if (sgrad[i] != 0.0) atomicAdd(&G.grad[i], sgrad[i]);
    }
}


// launchers of the class kernels (grad_class_f64*.cu, grad_class_f32*.cu): false
// when the class has no compile-time kernel in that type
bool launch_grad_class_f64(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem, cudaStream_t s);
bool launch_grad_class_f32(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem, cudaStream_t s);
bool launch_grad_class_f64_l5(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem,
                              cudaStream_t s);
bool launch_grad_class_f64_l6(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem,
                              cudaStream_t s);
bool launch_grad_class_f32_l56(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem,
                               cudaStream_t s);

}  // namespace gb
