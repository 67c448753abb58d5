// One-electron integrals: overlap S, kinetic T and nuclear attraction V over
// contracted shell pairs, with McMurchie-Davidson Hermite expansions:
//   S_ab = K1 (pi/p)^{3/2} E^x_0 E^y_0 E^z_0
//   T_ab = sum over axes of T1_x S_y S_z with
//          T1_x = -1/2 [ 4b^2 E^{i,j+2}_0 - 2b(2j+1) E^{ij}_0 + j(j-1) E^{i,j-2}_0 ] sqrt(pi/p)
//   V_ab = -sum_C Z_C (2 pi / p) K1 sum_tuv E_t E_u E_v R_tuv(p, P - C)
// (K1 = contraction coefficients x primitive norms x exp(-ab/p |AB|^2)).
// One warp per shell pair: the lanes share its primitive pairs (S, T) and its
// (primitive pair, nucleus) combinations (V), the sums are warp-reduced, and lane
// 0 writes both the (a,b) and (b,a) blocks, scaled by the per-function factors
// s_a s_b.  Replaces the reference's
// computeCoreHamiltonianMatrix (src/gpu_manager.cu:333-404), which evaluates
// the same matrices with Obara-Saika kernels (src/OS_kernel.txt).
#include "engine.hpp"
#include "md_math.cuh"

namespace gb {

namespace {

constexpr int kOneThreads = 128;

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int LA, int LB>
__global__ void __launch_bounds__(kOneThreads)
one_electron_kernel(const ShellPairDev* __restrict__ pairs, int begin, int count, const PrimPair64* __restrict__ pp,
                    const double* __restrict__ boys, const double* __restrict__ atoms,
                    const int* __restrict__ shell_mol, const int2* __restrict__ mol_atoms,
                    const int* __restrict__ mol_bf0, const double* __restrict__ scale, double kfold,
                    double* __restrict__ S, double* __restrict__ H)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), L = LA + LB;
    const int lane = threadIdx.x & 31;
    const int idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // warp-uniform
    if (idx >= count) return;
    const ShellPairDev sp = pairs[begin + idx];
    // the pair's molecule: its atoms (nuclear attraction), first global function, matrix block
    const int mol = shell_mol[sp.A];
    const int2 arange = mol_atoms[mol];
    const int g0 = mol_bf0[mol], n = sp.mn;
    S += sp.mbase;
    H += sp.mbase;
    double s_[NA][NB], t_[NA][NB], v_[NA][NB];
#pragma unroll
    for (int i = 0; i < NA; ++i)
#pragma unroll
        for (int j = 0; j < NB; ++j) s_[i][j] = t_[i][j] = v_[i][j] = 0.0;
    // overlap and kinetic energy: the primitive pairs over the lanes
    for (int ip = lane; ip < sp.pp_n; ip += 32) {
        const PrimPair64 q = pp[sp.pp_off + ip];
        const double p = q.p, b = q.b, oo2p = 0.5 * q.invp;
        const double k1 = q.K / kfold;
        HermiteE<double, LA, LB + 2> Ex, Ey, Ez;
        Ex.build(q.PAx, q.PAx + sp.ABx, oo2p);
        Ey.build(q.PAy, q.PAy + sp.ABy, oo2p);
        Ez.build(q.PAz, q.PAz + sp.ABz, oo2p);
        const double sq = sqrt(kPi / p);
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ib = 0; ib < NB; ++ib) {
                const int ax = cart_exp(LA, ia, 0), ay = cart_exp(LA, ia, 1), az = cart_exp(LA, ia, 2);
                const int bx = cart_exp(LB, ib, 0), by = cart_exp(LB, ib, 1), bz = cart_exp(LB, ib, 2);
                const double sx = Ex.e[ax][bx][0] * sq, sy = Ey.e[ay][by][0] * sq, sz = Ez.e[az][bz][0] * sq;
                auto kin = [&](const HermiteE<double, LA, LB + 2>& E, int i, int j) {
                    double tt = 4.0 * b * b * E.e[i][j + 2][0] - 2.0 * b * (2 * j + 1) * E.e[i][j][0];
                    if (j >= 2) tt += j * (j - 1) * E.e[i][j - 2][0];
                    return -0.5 * tt * sq;
                };
                s_[ia][ib] += k1 * sx * sy * sz;
                t_[ia][ib] += k1 * (kin(Ex, ax, bx) * sy * sz + sx * kin(Ey, ay, by) * sz + sx * sy * kin(Ez, az, bz));
            }
    }
    // nuclear attraction: the (primitive pair, nucleus) combinations over the lanes
    const int nat = arange.y;
    for (int w = lane; w < sp.pp_n * nat; w += 32) {
        const int ip = w / nat, c = arange.x + w % nat;
        const PrimPair64 q = pp[sp.pp_off + ip];
        const double p = q.p, oo2p = 0.5 * q.invp;
        const double k1 = q.K / kfold;
        HermiteE<double, LA, LB> Ex, Ey, Ez;
        Ex.build(q.PAx, q.PAx + sp.ABx, oo2p);
        Ey.build(q.PAy, q.PAy + sp.ABy, oo2p);
        Ez.build(q.PAz, q.PAz + sp.ABz, oo2p);
        const double X = q.Px - atoms[4 * c], Y = q.Py - atoms[4 * c + 1], Z = q.Pz - atoms[4 * c + 2];
        double Fs[L + 1];
        boys_fp64<L>(p * (X * X + Y * Y + Z * Z), boys, Fs);
        double sc = -atoms[4 * c + 3] * 2.0 * kPi / p * k1;
#pragma unroll
        for (int m = 0; m <= L; ++m) { Fs[m] *= sc; sc *= -2.0 * p; }
        HermiteR<double, L> R;
        R.build(Fs, X, Y, Z);
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int ib = 0; ib < NB; ++ib) {
                const int ax = cart_exp(LA, ia, 0), ay = cart_exp(LA, ia, 1), az = cart_exp(LA, ia, 2);
                const int bx = cart_exp(LB, ib, 0), by = cart_exp(LB, ib, 1), bz = cart_exp(LB, ib, 2);
                double acc = 0.0;
#pragma unroll
                for (int t = 0; t <= L; ++t) {
                    if (t > ax + bx) continue;
#pragma unroll
                    for (int u = 0; u <= L; ++u) {
                        if (u > ay + by) continue;
#pragma unroll
                        for (int v = 0; v <= L; ++v) {
                            if (v > az + bz) continue;
                            acc += Ex.e[ax][bx][t] * Ey.e[ay][by][u] * Ez.e[az][bz][v] * R(t, u, v);
                        }
                    }
                }
                v_[ia][ib] += acc;
            }
    }
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
        for (int ib = 0; ib < NB; ++ib) {
            const double sv0 = warp_sum_d(s_[ia][ib]), tv0 = warp_sum_d(t_[ia][ib]), vv0 = warp_sum_d(v_[ia][ib]);
            if (lane != 0) continue;
            const int a = sp.bfA + ia, bb = sp.bfB + ib;
            const double ss = scale[g0 + a] * scale[g0 + bb];
            const double sv = sv0 * ss, hv = (tv0 + vv0) * ss;
            S[static_cast<long long>(a) * n + bb] = sv;
            S[static_cast<long long>(bb) * n + a] = sv;
            H[static_cast<long long>(a) * n + bb] = hv;
            H[static_cast<long long>(bb) * n + a] = hv;
        }
}

}  // namespace

int core_hamiltonian(Engine& e, double* d_S, double* d_H, cudaStream_t s)
{
    const double kfold = std::sqrt(2.0 * std::pow(kPi, 2.5));
    for (const PairClass& pc : e.pair_classes) {
        if (pc.count == 0) continue;
        const int grid = static_cast<int>((static_cast<long long>(pc.count) * 32 + kOneThreads - 1) / kOneThreads);
#define GB_ONE(a, b)                                                                                           \
    if (pc.la == a && pc.lb == b)                                                                              \
        one_electron_kernel<a, b><<<grid, kOneThreads, 0, s>>>(e.d_pairs, pc.begin, pc.count, e.d_pp64,        \
                                                               e.d_boys64, e.d_atoms, e.d_shell_mol,           \
                                                               e.d_mol_atoms, e.d_mol_bf0, e.d_scale, kfold,   \
                                                               d_S, d_H);
        GB_ONE(0, 0) GB_ONE(1, 0) GB_ONE(1, 1) GB_ONE(2, 0) GB_ONE(2, 1) GB_ONE(2, 2)
#undef GB_ONE
        GB_LAUNCH_CHECK();
    }
    return HF_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int hf_compute_core_hamiltonian(hf_engine* eng, double* d_overlap, double* d_core_hamiltonian, void* stream)
{
    clear_error();
    if (!eng || !d_overlap || !d_core_hamiltonian) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    return core_hamiltonian(*reinterpret_cast<Engine*>(eng), d_overlap, d_core_hamiltonian,
                            static_cast<cudaStream_t>(stream));
}
