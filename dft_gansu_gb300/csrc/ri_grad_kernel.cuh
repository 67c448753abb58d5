// Derivative three-centre and metric integrals of the RI gradient, contracted
// with their weights (ri_grad.cu builds the weights; ri_grad_inst.cu
// instantiates this kernel once per auxiliary angular momentum).
//
// A Cartesian Gaussian's derivative in its centre is 2 alpha phi(a + 1) -
// a phi(a - 1); McMurchie-Davidson with the bra's Hermite tables one order
// higher and R one order higher gives d/dA and d/dB of (ab|P) for every
// component of a (bra pair, auxiliary component) in one thread, and
// d/dP = -(d/dA + d/dB) (translational invariance of the three-centre
// integral).  The metric uses the same kernel with (P, unit s) bras:
// d(P|Q)/dP, and d/dQ = -d/dP.  FP64; per-block shared-memory accumulation of
// the gradient when 3 * natom doubles fit.
#pragma once
#include "engine.hpp"
#include "ri.hpp"

namespace gb {

constexpr int kRiGradThreads = 128;

struct RiDerivArgs {
    const ShellPairDev* bra;     // bra pairs of one class (AO pairs, or (P, unit) pairs for the metric)
    int nbra;
    const PrimPair64* bra_pp;
    const AuxShellDev* ket;      // auxiliary shells of one angular momentum
    int nket;
    const AuxShellDev* aux_all;  // every auxiliary shell (atoms of the metric's bra shells)
    const PrimPair64* aux_pp;
    const double* boys;
    const double* bra_scale;
    const double* aux_scale;
    double thr;
    const double* weight;        // mode 0: Gamma packed [P][tri(mu,nu)]; mode 1: metric weights [Q][P]
    long long ld;
    int mode;                    // 0: three-centre, 1: metric
    const int* shell_atom;       // AO shell -> atom
    int natom;
    int shared_grad;             // 1: accumulate per block in shared memory
    double* grad;                // 3 * natom
};

using RiDerivLaunch = void (*)(const RiDerivArgs&, int grid, size_t smem, cudaStream_t);
// launcher of the kernel for bra class (la, lb) and auxiliary angular momentum LP (nullptr if none)
template <int LP>
RiDerivLaunch ri_deriv_launcher(int la, int lb);

#ifdef GB_RI_GRAD_KERNELS

__host__ __device__ constexpr int cart_exp_aux_g(int l, int i, int ax)
{
    // auxiliary Cartesian order (include/int2c2e.hpp:39-47): the AO order for l <= 2, its own for f
    if (l != 3) return cart_exp(l, i, ax);
    constexpr int t[10] = {300, 30, 3, 210, 201, 21, 120, 12, 102, 111};
    const int pk = t[i];
    return ax == 0 ? pk / 100 : (ax == 1 ? (pk / 10) % 10 : pk % 10);
}

__host__ __device__ __forceinline__ long long tri_g(int i, int j)
{
    return i >= j ? static_cast<long long>(i) * (i + 1) / 2 + j : static_cast<long long>(j) * (j + 1) / 2 + i;
}

// sum_{t,u,v} ex[t] ey[u] ez[v] x[t][u][v] over t <= nx, u <= ny, v <= nz
template <int M>
__device__ __forceinline__ double hsum(const double* ex, int nx, const double* ey, int ny, const double* ez, int nz,
                                       const double (&x)[M + 1][M + 1][M + 1])
{
    double s = 0.0;
#pragma unroll
    for (int t = 0; t <= M; ++t) {
        if (t > nx) break;
#pragma unroll
        for (int u = 0; u + t <= M; ++u) {
            if (u > ny) break;
            const double exy = ex[t] * ey[u];
#pragma unroll
            for (int v = 0; v + u + t <= M; ++v) {
                if (v > nz) break;
                s += exy * ez[v] * x[t][u][v];
            }
        }
    }
    return s;
}

__device__ __forceinline__ void ri_add_grad(const RiDerivArgs& a, double* sg, int atom, int k, double v)
{
    if (v == 0.0) return;
    if (a.shared_grad) atomicAdd(&sg[3 * atom + k], v);
    else atomicAdd(&a.grad[3 * atom + k], v);
}

template <int LA, int LB, int LP>
__global__ void __launch_bounds__(kRiGradThreads) ri_deriv_kernel(const RiDerivArgs a)
{
    extern __shared__ double sg[];
    constexpr int NA = ncart(LA), NB = ncart(LB), NP = ncart(LP), LAB = LA + LB, M = LAB + 1, L = LAB + LP + 1;
    if (a.shared_grad) {
        for (int i = threadIdx.x; i < 3 * a.natom; i += blockDim.x) sg[i] = 0.0;
        __syncthreads();
    }
    const long long total = static_cast<long long>(a.nbra) * a.nket * NP;
    for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int ip = static_cast<int>(idx % NP);
        const long long rest = idx / NP;
        const int is = static_cast<int>(rest % a.nket);
        const int ib = static_cast<int>(rest / a.nket);
        const ShellPairDev bp = a.bra[ib];
        const AuxShellDev ks = a.ket[is];
        const int px = cart_exp_aux_g(LP, ip, 0), py = cart_exp_aux_g(LP, ip, 1), pz = cart_exp_aux_g(LP, ip, 2);
        const int pf = ks.bf + ip;
        const double sp = a.aux_scale[pf];
        // weights of the block's components (scale factors folded in)
        double w[NA][NB];
        bool any = false;
#pragma unroll
        for (int ia = 0; ia < NA; ++ia)
#pragma unroll
            for (int jb = 0; jb < NB; ++jb) {
                double v;
                if (a.mode == 0) {
                    const int mu = bp.bfA + ia, nu = bp.bfB + jb;
                    // both triangles: the (B, A) block of a pair of distinct shells is this block's transpose
                    const double pair = (bp.A != bp.B) ? 2.0 : 1.0;
                    v = pair * a.weight[static_cast<long long>(pf) * a.ld + tri_g(mu, nu)] * sp * a.bra_scale[mu] *
                        a.bra_scale[nu];
                } else {
                    const int P = bp.bfA + ia;
                    v = a.weight[static_cast<long long>(pf) * a.ld + P] * sp * a.bra_scale[P];
                }
                w[ia][jb] = v;
                any |= (v != 0.0);
            }
        if (!any) continue;
        double gA[3] = {0.0, 0.0, 0.0}, gB[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < ks.np; ++k) {
            const PrimPair64 q = a.aux_pp[ks.p_off + k];
            HermiteE<double, LP, 0> Ep;
            Ep.build(0.0, 0.0, 0.5 * q.invp);
            for (int i = 0; i < bp.pp_n; ++i) {
                const PrimPair64 pb = a.bra_pp[bp.pp_off + i];
                if (pb.Q * q.Q < a.thr) continue;
                const double beta = pb.b, alpha = pb.p - pb.b;
                HermiteE<double, LA + 1, LB + 1> Ex, Ey, Ez;
                Ex.build(pb.PAx, pb.PAx + bp.ABx, 0.5 * pb.invp);
                Ey.build(pb.PAy, pb.PAy + bp.ABy, 0.5 * pb.invp);
                Ez.build(pb.PAz, pb.PAz + bp.ABz, 0.5 * pb.invp);
                const double rr = rsqrt(pb.p + q.p);
                const double rho = pb.p * q.p * rr * rr;
                const double X = pb.Px - q.Px, Y = pb.Py - q.Py, Z = pb.Pz - q.Pz;
                double Fs[L + 1];
                boys_fp64<L>(rho * (X * X + Y * Y + Z * Z), a.boys, Fs);
                double sc = pb.KoP * q.KoP * rr;
#pragma unroll
                for (int n = 0; n <= L; ++n) { Fs[n] *= sc; sc *= -2.0 * rho; }
                HermiteR<double, L> R;
                R.build(Fs, X, Y, Z);
                // ket contraction for this auxiliary component, bra Hermite indices up to LAB + 1
                double x[M + 1][M + 1][M + 1];
#pragma unroll
                for (int t = 0; t <= M; ++t)
#pragma unroll
                    for (int u = 0; u + t <= M; ++u)
#pragma unroll
                        for (int v = 0; v + u + t <= M; ++v) {
                            double s = 0.0;
#pragma unroll
                            for (int tau = 0; tau <= LP; ++tau) {
                                if (tau > px) break;
#pragma unroll
                                for (int nu = 0; nu <= LP; ++nu) {
                                    if (nu > py) break;
#pragma unroll
                                    for (int phi = 0; phi <= LP; ++phi) {
                                        if (phi > pz) break;
                                        const double c = Ep.e[px][0][tau] * Ep.e[py][0][nu] * Ep.e[pz][0][phi] *
                                                         R(t + tau, u + nu, v + phi);
                                        s += ((tau + nu + phi) & 1) ? -c : c;
                                    }
                                }
                            }
                            x[t][u][v] = s;
                        }
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int jb = 0; jb < NB; ++jb) {
                        const double wv = w[ia][jb];
                        if (wv == 0.0) continue;
                        const int ae[3] = {cart_exp_aux_g(LA, ia, 0), cart_exp_aux_g(LA, ia, 1),
                                           cart_exp_aux_g(LA, ia, 2)};
                        const int be[3] = {cart_exp(LB, jb, 0), cart_exp(LB, jb, 1), cart_exp(LB, jb, 2)};
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            // the differentiated axis d; the other two keep their exponents
                            const auto& Ed = d == 0 ? Ex : (d == 1 ? Ey : Ez);
                            const auto& E1 = d == 0 ? Ey : Ex;
                            const auto& E2 = d == 2 ? Ey : Ez;
                            const int o1 = d == 0 ? 1 : 0, o2 = d == 2 ? 1 : 2;
                            const int a1 = ae[o1], b1 = be[o1], a2 = ae[o2], b2 = be[o2];
                            const int ad = ae[d], bd = be[d];
                            // hsum over the axes in x, y, z order
                            auto h = [&](const double* ed, int nd) {
                                const double* e1 = E1.e[a1][b1];
                                const double* e2 = E2.e[a2][b2];
                                if (d == 0) return hsum<M>(ed, nd, e1, a1 + b1, e2, a2 + b2, x);
                                if (d == 1) return hsum<M>(e1, a1 + b1, ed, nd, e2, a2 + b2, x);
                                return hsum<M>(e1, a1 + b1, e2, a2 + b2, ed, nd, x);
                            };
                            double dA = 2.0 * alpha * h(Ed.e[ad + 1][bd], ad + 1 + bd);
                            if (ad > 0) dA -= ad * h(Ed.e[ad - 1][bd], ad - 1 + bd);
                            double dB = 2.0 * beta * h(Ed.e[ad][bd + 1], ad + bd + 1);
                            if (bd > 0) dB -= bd * h(Ed.e[ad][bd - 1], ad + bd - 1);
                            gA[d] += wv * dA;
                            gB[d] += wv * dB;
                        }
                    }
            }
        }
        if (a.mode == 0) {
            const int atA = a.shell_atom[bp.A], atB = a.shell_atom[bp.B], atP = ks.atom;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                ri_add_grad(a, sg, atA, d, gA[d]);
                ri_add_grad(a, sg, atB, d, gB[d]);
                ri_add_grad(a, sg, atP, d, -(gA[d] + gB[d]));
            }
        } else {
            const int atP = a.aux_all[bp.A].atom, atQ = ks.atom;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                ri_add_grad(a, sg, atP, d, gA[d]);
                ri_add_grad(a, sg, atQ, d, -gA[d]);
            }
        }
    }
    if (a.shared_grad) {
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * a.natom; i += blockDim.x)
            if (sg[i] != 0.0) atomicAdd(&a.grad[i], sg[i]);
    }
}

template <int LA, int LB, int LP>
void ri_deriv_launch(const RiDerivArgs& a, int grid, size_t smem, cudaStream_t s)
{
    ri_deriv_kernel<LA, LB, LP><<<grid, kRiGradThreads, smem, s>>>(a);
}

#endif  // GB_RI_GRAD_KERNELS

}  // namespace gb
