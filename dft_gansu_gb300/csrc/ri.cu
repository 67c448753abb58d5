// Resolution of the identity (density fitting) on the device.
//
// What the reference does (src/eri.cu:119-236, src/gpu_manager.cu:1448-1632):
//   (P|Q)   metric over auxiliary functions               computeTwoCenterERIs   :1963-2041
//   V = L L^T (Cholesky)                                    choleskyDecomposition  :1311-1349
//   (mu nu|P) three-centre integrals, [P][mu][nu]           computeThreeCenterERIs :2048-2141
//   B = L^-1 (mu nu|P)                                      solve_lower_triangular :1359-1416
//   J = sum_P B_P (B_P . D), K = sum_P B_P D B_P^T, F = H + J - K/2
//                                                           computeFockMatrix_RI_RHF :1543-1632
//
// How it is laid out here:
//   * auxiliary shells are contracted shells of their own basis file (the
//     reference builds them with the same Molecular code), normalised like AO
//     shells, with the auxiliary Cartesian order of include/int2c2e.hpp:39-47;
//   * a three-centre integral (ab|P) is the four-centre MD integral with an
//     exponent-0 unit s function as the partner of P, so the metric reuses the
//     same kernel with (P, unit) "pairs" as bra;
//   * (mu nu|P) is produced as a packed lower triangle T[P][mu(mu+1)/2 + nu]
//     (mu >= nu): the triangular solve then runs on N(N+1)/2 columns instead of
//     N^2, and RI-J streams half the bytes;
//   * B is kept packed (FP64) and, for K, expanded once into the reference's
//     full [P][mu][nu] layout;
//   * K is formed from a factor of the density, D = Y+ Y+^T - Y- Y-^T (from the
//     occupied orbitals inside the SCF, D = 2 C_occ C_occ^T, or from an
//     eigendecomposition for an arbitrary symmetric D): X_P = B_P Y, then
//     K = sum_P X_P X_P^T, which is 3 naux N^2 r flops instead of the
//     reference's 4 naux N^3 (r = number of occupied orbitals).
#include <algorithm>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "engine.hpp"
#include "ri.hpp"
#include "tc_gemm.hpp"

namespace gb {

namespace {

constexpr int kRiThreads = 128;

// Cartesian exponent of component i of an auxiliary shell (include/int2c2e.hpp:39-47):
// the AO order for l <= 2, its own order for f.
__host__ __device__ constexpr int cart_exp_aux(int l, int i, int ax)
{
    if (l != 3) return cart_exp(l, i, ax);
    constexpr int t[10] = {300, 30, 3, 210, 201, 21, 120, 12, 102, 111};
    const int pk = t[i];
    return ax == 0 ? pk / 100 : (ax == 1 ? (pk / 10) % 10 : pk % 10);
}

__host__ __device__ inline double component_factor_aux(int l, int i)
{
    return 1.0 / sqrt(dfact(2 * cart_exp_aux(l, i, 0) - 1) * dfact(2 * cart_exp_aux(l, i, 1) - 1) *
                      dfact(2 * cart_exp_aux(l, i, 2) - 1));
}

__host__ __device__ __forceinline__ long long tri(int i, int j)
{
    return i >= j ? static_cast<long long>(i) * (i + 1) / 2 + j : static_cast<long long>(j) * (j + 1) / 2 + i;
}

struct ThreeCenterArgs {
    const ShellPairDev* bra;    // bra pairs of one class
    int nbra;
    const PrimPair64* bra_pp;
    const AuxShellDev* aux;     // auxiliary shells of one angular momentum
    int naux;
    const PrimPair64* aux_pp;   // auxiliary primitives as (gamma, unit) pairs
    const double* boys;
    const double* bra_scale;    // s per bra function (AO or auxiliary)
    const double* aux_scale;
    double thr;
    double* out;
    int mode;                   // 0: packed AO triangle T[P][tri(mu,nu)]; 1: metric V[Q][P]
    long long ld;               // row length of out (N(N+1)/2 or naux)
};

// One thread = one (bra pair, auxiliary shell, auxiliary component); it sums
// the primitive triples passing Q_ab * Q_P >= thr and writes the NA x NB
// block of that component.  Consecutive threads share the bra pair.
template <int LA, int LB, int LP>
__global__ void __launch_bounds__(kRiThreads) three_center_kernel(const ThreeCenterArgs a)
{
    constexpr int NA = ncart(LA), NB = ncart(LB), NP = ncart(LP), L = LA + LB + LP, LAB = LA + LB;
    const long long total = static_cast<long long>(a.nbra) * a.naux * NP;
    for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int ip = static_cast<int>(idx % NP);
        const long long rest = idx / NP;
        const int is = static_cast<int>(rest % a.naux);
        const int ib = static_cast<int>(rest / a.naux);
        const ShellPairDev bp = a.bra[ib];
        const AuxShellDev as = a.aux[is];
        const int px = cart_exp_aux(LP, ip, 0), py = cart_exp_aux(LP, ip, 1), pz = cart_exp_aux(LP, ip, 2);
        double acc[NA][NB];
#pragma unroll
        for (int i = 0; i < NA; ++i)
#pragma unroll
            for (int j = 0; j < NB; ++j) acc[i][j] = 0.0;
        for (int k = 0; k < as.np; ++k) {
            const PrimPair64 q = a.aux_pp[as.p_off + k];
            // Hermite expansion of the auxiliary primitive (centre = its own, PA = 0): same table on every axis
            HermiteE<double, LP, 0> Ep;
            Ep.build(0.0, 0.0, 0.5 * q.invp);
            for (int i = 0; i < bp.pp_n; ++i) {
                const PrimPair64 pb = a.bra_pp[bp.pp_off + i];
                if (pb.Q * q.Q < a.thr) continue;
                HermiteE<double, LA, LB> Ex, Ey, Ez;
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
                // ket contraction for this auxiliary component
                double x[LAB + 1][LAB + 1][LAB + 1];
#pragma unroll
                for (int t = 0; t <= LAB; ++t)
#pragma unroll
                    for (int u = 0; u + t <= LAB; ++u)
#pragma unroll
                        for (int v = 0; v + u + t <= LAB; ++v) {
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
                                        if (t + tau + u + nu + v + phi > L) continue;
                                        const double w = Ep.e[px][0][tau] * Ep.e[py][0][nu] * Ep.e[pz][0][phi] *
                                                         R(t + tau, u + nu, v + phi);
                                        s += ((tau + nu + phi) & 1) ? -w : w;
                                    }
                                }
                            }
                            x[t][u][v] = s;
                        }
#pragma unroll
                for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                    for (int jb = 0; jb < NB; ++jb) {
                        // the bra's first shell is auxiliary (l = 3 possible) only in the metric; for
                        // l <= 2 the auxiliary and AO orders coincide
                        const int ax = cart_exp_aux(LA, ia, 0), ay = cart_exp_aux(LA, ia, 1),
                                  az = cart_exp_aux(LA, ia, 2);
                        const int bx = cart_exp(LB, jb, 0), by = cart_exp(LB, jb, 1), bz = cart_exp(LB, jb, 2);
                        double s = 0.0;
#pragma unroll
                        for (int t = 0; t <= ax + bx; ++t)
#pragma unroll
                            for (int u = 0; u <= ay + by; ++u)
#pragma unroll
                                for (int v = 0; v <= az + bz; ++v)
                                    s += Ex.e[ax][bx][t] * Ey.e[ay][by][u] * Ez.e[az][bz][v] * x[t][u][v];
                        acc[ia][jb] += s;
                    }
            }
        }
        const int pf = as.bf + ip;
        const double sp = a.aux_scale[pf];
        if (a.mode == 0) {
            double* row = a.out + static_cast<long long>(pf) * a.ld;
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int jb = 0; jb < NB; ++jb) {
                    const int mu = bp.bfA + ia, nu = bp.bfB + jb;
                    row[tri(mu, nu)] = acc[ia][jb] * sp * a.bra_scale[mu] * a.bra_scale[nu];
                }
        } else {
#pragma unroll
            for (int ia = 0; ia < NA; ++ia) {
                const int P = bp.bfA + ia;
                a.out[static_cast<long long>(pf) * a.ld + P] = acc[ia][0] * sp * a.bra_scale[P];
            }
        }
    }
}

using TcLaunch = void (*)(const ThreeCenterArgs&, int grid, cudaStream_t);
template <int LA, int LB, int LP>
void tc_launch(const ThreeCenterArgs& a, int grid, cudaStream_t s)
{
    three_center_kernel<LA, LB, LP><<<grid, kRiThreads, 0, s>>>(a);
}

TcLaunch tc_table(int la, int lb, int lp)
{
#define GB_TC(A, B)                                                                                \
    if (la == A && lb == B) {                                                                      \
        switch (lp) {                                                                              \
        case 0: return tc_launch<A, B, 0>;                                                         \
        case 1: return tc_launch<A, B, 1>;                                                         \
        case 2: return tc_launch<A, B, 2>;                                                         \
        case 3: return tc_launch<A, B, 3>;                                                         \
        default: return nullptr;                                                                   \
        }                                                                                          \
    }
    GB_TC(0, 0) GB_TC(1, 0) GB_TC(1, 1) GB_TC(2, 0) GB_TC(2, 1) GB_TC(2, 2) GB_TC(3, 0)
#undef GB_TC
    return nullptr;
}

// ---------------------------------------------------------------- small kernels
__global__ void expand_packed_kernel(const double* __restrict__ Bp, long long npk, int n, long long rows,
                                     double* __restrict__ B)
{
    const long long nn = static_cast<long long>(n) * n, total = rows * nn;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long P = k / nn, r = k % nn;
        const int i = static_cast<int>(r / n), j = static_cast<int>(r % n);
        B[k] = Bp[P * npk + tri(i, j)];
    }
}

// Dt[tri(i,j)] = D_ij + D_ji (i > j), D_ii
__global__ void pack_density_kernel(const double* __restrict__ D, int n, double* __restrict__ Dt)
{
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < npk;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>((sqrt(8.0 * static_cast<double>(k) + 1.0) - 1.0) * 0.5);
        int ii = i;
        while (static_cast<long long>(ii) * (ii + 1) / 2 > k) --ii;
        while (static_cast<long long>(ii + 1) * (ii + 2) / 2 <= k) ++ii;
        const int j = static_cast<int>(k - static_cast<long long>(ii) * (ii + 1) / 2);
        Dt[k] = (ii == j) ? D[static_cast<long long>(ii) * n + ii]
                          : D[static_cast<long long>(ii) * n + j] + D[static_cast<long long>(j) * n + ii];
    }
}

// W_P = sum_k Bp[P][k] Dt[k]: one block per auxiliary function
__global__ void __launch_bounds__(256) ri_w_kernel(const double* __restrict__ Bp, const double* __restrict__ Dt,
                                                  long long npk, double* __restrict__ W)
{
    __shared__ double red[8];
    const double* row = Bp + static_cast<long long>(blockIdx.x) * npk;
    double s = 0.0;
    for (long long k = threadIdx.x; k < npk; k += blockDim.x) s += row[k] * Dt[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) W[blockIdx.x] = s;
    }
}

// J[i][j] = sum_P W_P Bp[P][tri(i,j)] for the packed column k; written to both triangles
__global__ void ri_j_kernel(const double* __restrict__ Bp, const double* __restrict__ W, int naux, int n,
                            double* __restrict__ J)
{
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < npk;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (int P = 0; P < naux; ++P) s += W[P] * Bp[static_cast<long long>(P) * npk + k];
        int i = static_cast<int>((sqrt(8.0 * static_cast<double>(k) + 1.0) - 1.0) * 0.5);
        while (static_cast<long long>(i) * (i + 1) / 2 > k) --i;
        while (static_cast<long long>(i + 1) * (i + 2) / 2 <= k) ++i;
        const int j = static_cast<int>(k - static_cast<long long>(i) * (i + 1) / 2);
        J[static_cast<long long>(i) * n + j] = s;
        J[static_cast<long long>(j) * n + i] = s;
    }
}

// K from the lower triangle of a column-major SYRK result: K = K^T
__global__ void mirror_lower_colmajor_kernel(double* __restrict__ K, int n)
{
    const long long nn = static_cast<long long>(n) * n;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int c = static_cast<int>(k / n), r = static_cast<int>(k % n);  // column-major (r, c)
        if (r < c) K[k] = K[static_cast<long long>(r) * n + c];             // upper <- lower (c, r)
    }
}

// Y[v][j] = V[v + idx_j * n] * sqrt(|lambda_idx_j|), Y row-major n x r
__global__ void scaled_columns_kernel(const double* __restrict__ V, const double* __restrict__ lam, int n,
                                      int first, int r, double* __restrict__ Y)
{
    const long long total = static_cast<long long>(n) * r;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int v = static_cast<int>(k / r), j = static_cast<int>(k % r);
        const int c = first + j;
        Y[k] = V[static_cast<long long>(c) * n + v] * sqrt(fabs(lam[c]));
    }
}

// F = H + J - K/2 (or G = J - K/2 accumulated into G, F = H + G)
__global__ void ri_fock_kernel(const double* __restrict__ H, const double* __restrict__ J,
                               const double* __restrict__ K, long long nn, int accumulate, double* __restrict__ G,
                               double* __restrict__ F)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double g = J[k] - 0.5 * K[k];
        if (G) {
            const double gn = accumulate ? G[k] + g : g;
            G[k] = gn;
            F[k] = H[k] + gn;
        } else {
            F[k] = H[k] + g;
        }
    }
}

int grid_for(long long work, int threads, int num_sms)
{
    return static_cast<int>(std::max<long long>(1, std::min<long long>((work + threads - 1) / threads,
                                                                          static_cast<long long>(num_sms) * 32)));
}

template <class T>
int ri_alloc(T*& p, size_t n)
{
    if (p) return HF_OK;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) {
        p = nullptr;
        set_error(std::string("cudaMalloc (RI): ") + cudaGetErrorString(e));
        return (e == cudaErrorMemoryAllocation) ? HF_ERR_OUT_OF_MEMORY : HF_ERR_CUDA;
    }
    return HF_OK;
}

}  // namespace

void ri_destroy(RiState* r)
{
    if (!r) return;
    void* ptrs[] = {r->d_aux, r->d_aux_pp, r->d_aux_pairs, r->d_aux_scale, r->d_V, r->d_Bp, r->d_B,
                    r->d_Dt, r->d_W, r->d_X, r->d_J, r->d_K, r->d_Y, r->d_evec, r->d_eval, r->d_work,
                    r->d_info, r->d_Bh, r->d_Bl, r->d_Yh, r->d_Yl, r->d_Y2h, r->d_Y2l, r->d_Xh, r->d_Xl,
                    r->d_X2h, r->d_X2l, r->d_Kacc, r->d_Cprev, r->d_T1, r->d_M, r->d_U, r->d_U2, r->d_Ca,
                    r->d_flag};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete r;
}

int ri_set_auxiliary(Engine& e, const hf_primitive_shell* prims, int nprim, const double* cgto, int naux)
{
    for (int i = 0; i < nprim; ++i)
        if (prims[i].shell_type < 0 || prims[i].shell_type > kMaxAuxL)
            return set_error("auxiliary shell type " + std::to_string(prims[i].shell_type) +
                             " not supported (s..f)"), HF_ERR_INVALID_ARGUMENT;
    ri_destroy(e.ri);
    e.ri = new RiState;
    RiState& r = *e.ri;
    r.naux = naux;
    // contracted auxiliary shells: group by (shell_type, basis_index) as for AO shells
    std::map<std::pair<int, size_t>, std::vector<int>> groups;
    for (int i = 0; i < nprim; ++i) groups[{prims[i].shell_type, prims[i].basis_index}].push_back(i);
    std::vector<double> boys;
    host_boys_table(boys);
    std::vector<AuxShellDev> shells;
    std::vector<PrimPair64> pp;
    std::vector<double> scale(naux, 0.0);
    for (int l = 0; l <= kMaxAuxL; ++l) {
        r.class_begin[l] = static_cast<int>(shells.size());
        for (auto& kv : groups) {
            if (kv.first.first != l) continue;
            AuxShellDev s{};
            const auto& p0 = prims[kv.second[0]];
            s.x = p0.x; s.y = p0.y; s.z = p0.z;
            s.l = l;
            s.bf = static_cast<int>(kv.first.second);
            s.p_off = static_cast<int>(pp.size());
            s.np = static_cast<int>(kv.second.size());
            s.atom = p0.atom_index;
            if (s.bf < 0 || s.bf + ncart(l) > naux)
                return set_error("auxiliary basis index out of range"), HF_ERR_INVALID_ARGUMENT;
            const double C[3] = {s.x, s.y, s.z};
            for (int idx : kv.second) {
                PrimPair64 q = make_prim_pair(prims[idx].exponent,
                                              scaled_coef(prims[idx].coefficient, prims[idx].exponent, l), C, 0.0,
                                              1.0, C);
                // reference auxiliary bound (src/schwarz.txt:480-682): includes the auxiliary CGTO factor
                q.Q = cgto[s.bf] * aux_prim_bound(l, q, boys.data());
                pp.push_back(q);
            }
            for (int i = 0; i < ncart(l); ++i) scale[s.bf + i] = cgto[s.bf + i] * component_factor_aux(l, i);
            shells.push_back(s);
        }
        r.class_count[l] = static_cast<int>(shells.size()) - r.class_begin[l];
    }
    // (P, unit) bra pairs for the metric
    std::vector<ShellPairDev> apairs;
    for (int i = 0; i < static_cast<int>(shells.size()); ++i) {
        ShellPairDev sp{};
        sp.A = i; sp.B = -1; sp.bfA = shells[i].bf; sp.bfB = 0;
        sp.la = shells[i].l; sp.lb = 0;
        sp.mbase = 0;
        sp.mn = naux;
        sp.pp_off = shells[i].p_off; sp.pp_n = shells[i].np;
        double qm = 0.0, qs = 0.0;
        for (int k = 0; k < shells[i].np; ++k) { qm = std::max(qm, pp[shells[i].p_off + k].Q); qs += pp[shells[i].p_off + k].Q; }
        sp.Qmax = qm; sp.Qs = qs;
        apairs.push_back(sp);
    }
    r.shells = shells;
    int st = HF_OK;
    if ((st = ri_alloc(r.d_aux, shells.size())) || (st = ri_alloc(r.d_aux_pp, pp.size())) ||
        (st = ri_alloc(r.d_aux_pairs, apairs.size())) || (st = ri_alloc(r.d_aux_scale, scale.size())))
        return st;
    GB_CUDA_TRY(cudaMemcpy(r.d_aux, shells.data(), shells.size() * sizeof(AuxShellDev), cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaMemcpy(r.d_aux_pp, pp.data(), pp.size() * sizeof(PrimPair64), cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaMemcpy(r.d_aux_pairs, apairs.data(), apairs.size() * sizeof(ShellPairDev), cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaMemcpy(r.d_aux_scale, scale.data(), scale.size() * sizeof(double), cudaMemcpyHostToDevice));
    e.bytes_h2d += static_cast<long long>(shells.size() * sizeof(AuxShellDev) + pp.size() * sizeof(PrimPair64) +
                                          apairs.size() * sizeof(ShellPairDev) + scale.size() * sizeof(double));
    return HF_OK;
}

int ri_metric(Engine& e, double* d_V, cudaStream_t s)
{
    RiState& r = *e.ri;
    GB_CUDA_TRY(cudaMemsetAsync(d_V, 0, sizeof(double) * r.naux * r.naux, s));
    for (int lp = 0; lp <= kMaxAuxL; ++lp)
        for (int lq = 0; lq <= kMaxAuxL; ++lq) {
            if (!r.class_count[lp] || !r.class_count[lq]) continue;
            ThreeCenterArgs a;
            a.bra = r.d_aux_pairs + r.class_begin[lp];
            a.nbra = r.class_count[lp];
            a.bra_pp = r.d_aux_pp;
            a.aux = r.d_aux + r.class_begin[lq];
            a.naux = r.class_count[lq];
            a.aux_pp = r.d_aux_pp;
            a.boys = e.d_boys64;
            a.bra_scale = r.d_aux_scale;
            a.aux_scale = r.d_aux_scale;
            a.thr = e.schwarz_threshold;
            a.out = d_V;
            a.mode = 1;
            a.ld = r.naux;
            const long long work = static_cast<long long>(a.nbra) * a.naux * ncart(lq);
            tc_table(lp, 0, lq)(a, grid_for(work, kRiThreads, e.num_sms), s);
            GB_LAUNCH_CHECK();
        }
    return HF_OK;
}

int ri_three_center_packed(Engine& e, double* d_T, cudaStream_t s)
{
    RiState& r = *e.ri;
    const long long npk = static_cast<long long>(e.num_basis) * (e.num_basis + 1) / 2;
    GB_CUDA_TRY(cudaMemsetAsync(d_T, 0, sizeof(double) * npk * r.naux, s));
    for (const PairClass& pc : e.pair_classes) {
        if (!pc.count) continue;
        for (int lp = 0; lp <= kMaxAuxL; ++lp) {
            if (!r.class_count[lp]) continue;
            ThreeCenterArgs a;
            a.bra = e.d_pairs + pc.begin;
            a.nbra = pc.count;
            a.bra_pp = e.d_pp64;
            a.aux = r.d_aux + r.class_begin[lp];
            a.naux = r.class_count[lp];
            a.aux_pp = r.d_aux_pp;
            a.boys = e.d_boys64;
            a.bra_scale = e.d_scale;
            a.aux_scale = r.d_aux_scale;
            a.thr = e.schwarz_threshold;
            a.out = d_T;
            a.mode = 0;
            a.ld = npk;
            const long long work = static_cast<long long>(a.nbra) * a.naux * ncart(lp);
            tc_table(pc.la, pc.lb, lp)(a, grid_for(work, kRiThreads, e.num_sms), s);
            GB_LAUNCH_CHECK();
        }
    }
    return HF_OK;
}

int ri_expand(Engine& e, const double* d_packed, long long rows, double* d_full, cudaStream_t s)
{
    const int n = e.num_basis;
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    const long long total = rows * n * n;
    expand_packed_kernel<<<grid_for(total, 256, e.num_sms), 256, 0, s>>>(d_packed, npk, n, rows, d_full);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

int ri_build_b(Engine& e, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis, M = r.naux;
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    int st;
    if ((st = ri_alloc(r.d_V, static_cast<size_t>(M) * M)) || (st = ri_alloc(r.d_Bp, static_cast<size_t>(M) * npk)) ||
        (st = ri_alloc(r.d_info, 1)))
        return st;
    if ((st = ri_metric(e, r.d_V, s))) return st;
    // V = L L^T (column-major lower; V is symmetric so its row-major copy is the same matrix)
    cusolverDnSetStream(e.cusolver, s);
    int lwork = 0;
    if (cusolverDnDpotrf_bufferSize(e.cusolver, CUBLAS_FILL_MODE_LOWER, M, r.d_V, M, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDpotrf_bufferSize failed"), HF_ERR_SOLVER;
    if (static_cast<size_t>(lwork) > r.work_len) {
        if (r.d_work) cudaFree(r.d_work);
        r.d_work = nullptr;
        if ((st = ri_alloc(r.d_work, static_cast<size_t>(lwork)))) return st;
        r.work_len = static_cast<size_t>(lwork);
    }
    if (cusolverDnDpotrf(e.cusolver, CUBLAS_FILL_MODE_LOWER, M, r.d_V, M, r.d_work, lwork, r.d_info) !=
        CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDpotrf failed"), HF_ERR_SOLVER;
    int info = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&info, r.d_info, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (info != 0)
        return set_error("RI metric is not positive definite (potrf info " + std::to_string(info) + ")"),
               HF_ERR_NOT_SPD;
    if ((st = ri_three_center_packed(e, r.d_Bp, s))) return st;
    // B^T L^T = T^T: in column-major the packed T is (npk x M), solve X L^T = T from the right
    cublasSetStream(e.cublas, s);
    const double one = 1.0;
    if (cublasDtrsm(e.cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT,
                    static_cast<int>(npk), M, &one, r.d_V, M, r.d_Bp, static_cast<int>(npk)) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDtrsm failed"), HF_ERR_SOLVER;
    r.have_b = true;
    r.have_full = false;
    return HF_OK;
}

static int ensure_full_b(Engine& e, cudaStream_t s)
{
    RiState& r = *e.ri;
    if (r.have_full) return HF_OK;
    const size_t nn = static_cast<size_t>(e.num_basis) * e.num_basis;
    int st;
    if ((st = ri_alloc(r.d_B, nn * r.naux))) return st;
    if ((st = ri_expand(e, r.d_Bp, r.naux, r.d_B, s))) return st;
    r.have_full = true;
    return HF_OK;
}

int ri_full_b(Engine& e, cudaStream_t s) { return ensure_full_b(e, s); }

int ri_w_of(Engine& e, const double* d_D, double* d_Dt, double* d_w, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis;
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    pack_density_kernel<<<grid_for(npk, 256, e.num_sms), 256, 0, s>>>(d_D, n, d_Dt);
    GB_LAUNCH_CHECK();
    ri_w_kernel<<<r.naux, 256, 0, s>>>(r.d_Bp, d_Dt, npk, d_w);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

int ri_j(Engine& e, const double* d_D, double* d_J, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis;
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    int st;
    if ((st = ri_alloc(r.d_Dt, npk)) || (st = ri_alloc(r.d_W, r.naux))) return st;
    pack_density_kernel<<<grid_for(npk, 256, e.num_sms), 256, 0, s>>>(d_D, n, r.d_Dt);
    GB_LAUNCH_CHECK();
    ri_w_kernel<<<r.naux, 256, 0, s>>>(r.d_Bp, r.d_Dt, npk, r.d_W);
    GB_LAUNCH_CHECK();
    ri_j_kernel<<<grid_for(npk, 256, e.num_sms), 256, 0, s>>>(r.d_Bp, r.d_W, r.naux, n, d_J);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// K = alpha * sum_P (B_P Y)(B_P Y)^T + beta * K, Y row-major n x r with row stride ldy
static int ri_k_factor(Engine& e, const double* d_Y, int r_cols, int ldy, double alpha, double beta, double* d_K,
                       cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis, M = r.naux;
    if (r_cols <= 0) return HF_OK;
    int st;
    if ((st = ensure_full_b(e, s))) return st;
    const size_t need = static_cast<size_t>(n) * M * r_cols;
    if (need > r.x_len) {
        if (r.d_X) cudaFree(r.d_X);
        r.d_X = nullptr;
        if ((st = ri_alloc(r.d_X, need))) return st;
        r.x_len = need;
    }
    cublasSetStream(e.cublas, s);
    const double one = 1.0, zero = 0.0;
    const long long ldx = static_cast<long long>(M) * r_cols;
    if (ldx > 0x7fffffffLL) return set_error("RI-K: naux * r exceeds the BLAS index range"), HF_ERR_INVALID_ARGUMENT;
    // column-major: X_P^T (r x n, ld M*r, at X + P*r) = Y^T (r x n, ld ldy) * B_P (n x n)
    if (cublasDgemmStridedBatched(e.cublas, CUBLAS_OP_N, CUBLAS_OP_N, r_cols, n, n, &one, d_Y, ldy, 0, r.d_B, n,
                                  static_cast<long long>(n) * n, &zero, r.d_X, static_cast<int>(ldx), r_cols,
                                  M) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDgemmStridedBatched (RI-K) failed"), HF_ERR_SOLVER;
    // K (col-major lower) = alpha Xc^T Xc + beta K, Xc = X as column-major (M r) x n
    if (cublasDsyrk(e.cublas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, n, static_cast<int>(ldx), &alpha, r.d_X,
                    static_cast<int>(ldx), &beta, d_K, n) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDsyrk (RI-K) failed"), HF_ERR_SOLVER;
    return HF_OK;
}

int ri_k_occupied(Engine& e, const double* d_C, int nocc, double* d_K, cudaStream_t s)
{
    // D = 2 C_occ C_occ^T: Y = C[:, :nocc] (row stride n), alpha = 2
    int st = ri_k_factor(e, d_C, nocc, e.num_basis, 2.0, 0.0, d_K, s);
    if (st) return st;
    const long long nn = static_cast<long long>(e.num_basis) * e.num_basis;
    mirror_lower_colmajor_kernel<<<grid_for(nn, 256, e.num_sms), 256, 0, s>>>(d_K, e.num_basis);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

int ri_k_density(Engine& e, const double* d_D, double* d_K, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis;
    const long long nn = static_cast<long long>(n) * n;
    int st;
    if ((st = ri_alloc(r.d_evec, nn)) || (st = ri_alloc(r.d_eval, n)) || (st = ri_alloc(r.d_Y, nn)) ||
        (st = ri_alloc(r.d_info, 1)))
        return st;
    GB_CUDA_TRY(cudaMemcpyAsync(r.d_evec, d_D, nn * sizeof(double), cudaMemcpyDeviceToDevice, s));
    cusolverDnSetStream(e.cusolver, s);
    int lwork = 0;
    if (cusolverDnDsyevd_bufferSize(e.cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, r.d_evec, n,
                                    r.d_eval, &lwork) != CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDsyevd_bufferSize failed"), HF_ERR_SOLVER;
    if (static_cast<size_t>(lwork) > r.work_len) {
        if (r.d_work) cudaFree(r.d_work);
        r.d_work = nullptr;
        if ((st = ri_alloc(r.d_work, static_cast<size_t>(lwork)))) return st;
        r.work_len = static_cast<size_t>(lwork);
    }
    if (cusolverDnDsyevd(e.cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, r.d_evec, n, r.d_eval,
                         r.d_work, lwork, r.d_info) != CUSOLVER_STATUS_SUCCESS)
        return set_error("cusolverDnDsyevd failed"), HF_ERR_SOLVER;
    std::vector<double> lam(n);
    int info = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(lam.data(), r.d_eval, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaMemcpyAsync(&info, r.d_info, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (info != 0) return set_error("syevd of the density reported info " + std::to_string(info)), HF_ERR_SOLVER;
    double mx = 0.0;
    for (double v : lam) mx = std::max(mx, std::fabs(v));
    const double cut = 1e-14 * std::max(mx, 1e-300);
    int nneg = 0, npos = 0;
    for (double v : lam) {
        if (v < -cut) ++nneg;
        if (v > cut) ++npos;
    }
    // eigenvalues ascending: negatives first, positives last
    bool first = true;
    if (npos) {
        scaled_columns_kernel<<<grid_for(static_cast<long long>(n) * npos, 256, e.num_sms), 256, 0, s>>>(
            r.d_evec, r.d_eval, n, n - npos, npos, r.d_Y);
        GB_LAUNCH_CHECK();
        if ((st = ri_k_factor(e, r.d_Y, npos, npos, 1.0, 0.0, d_K, s))) return st;
        first = false;
    }
    if (nneg) {
        scaled_columns_kernel<<<grid_for(static_cast<long long>(n) * nneg, 256, e.num_sms), 256, 0, s>>>(
            r.d_evec, r.d_eval, n, 0, nneg, r.d_Y);
        GB_LAUNCH_CHECK();
        if ((st = ri_k_factor(e, r.d_Y, nneg, nneg, -1.0, first ? 0.0 : 1.0, d_K, s))) return st;
        first = false;
    }
    if (first) {
        GB_CUDA_TRY(cudaMemsetAsync(d_K, 0, nn * sizeof(double), s));
        return HF_OK;
    }
    mirror_lower_colmajor_kernel<<<grid_for(nn, 256, e.num_sms), 256, 0, s>>>(d_K, n);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

int ri_fock_from_jk(Engine& e, const double* d_H, const double* d_J, const double* d_K, double* d_G, bool accumulate,
                    double* d_F, cudaStream_t s)
{
    const long long nn = static_cast<long long>(e.num_basis) * e.num_basis;
    ri_fock_kernel<<<grid_for(nn, 256, e.num_sms), 256, 0, s>>>(d_H, d_J, d_K, nn, accumulate ? 1 : 0, d_G, d_F);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

int ri_require_b(Engine& e, cudaStream_t s)
{
    if (!e.ri) return set_error("no auxiliary basis attached (hf_engine_set_auxiliary_basis)"), HF_ERR_INVALID_ARGUMENT;
    if (!e.ri->have_b) return ri_build_b(e, s);
    return HF_OK;
}

int ri_work_buffers(Engine& e, double** J, double** K)
{
    RiState& r = *e.ri;
    const size_t nn = static_cast<size_t>(e.num_basis) * e.num_basis;
    int st;
    if ((st = ri_alloc(r.d_J, nn)) || (st = ri_alloc(r.d_K, nn))) return st;
    *J = r.d_J;
    *K = r.d_K;
    return HF_OK;
}


// ------------------------------------------------------------------ mixed tier
namespace {

// B planes: row (P, mu) of the full B, columns nu (zero padded to kpad), split into BF16 hi/lo
__global__ void b_planes_kernel(const double* __restrict__ Bp, int naux, int n, long long kpad,
                                __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo)
{
    const long long npk = static_cast<long long>(n) * (n + 1) / 2;
    const long long total = static_cast<long long>(naux) * n * kpad;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long row = k / kpad, c = k % kpad;
        const long long P = row / n;
        const int mu = static_cast<int>(row % n);
        double v = 0.0;
        if (c < n) v = Bp[P * npk + tri(mu, static_cast<int>(c))];
        const float x = static_cast<float>(v);
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        hi[k] = h;
        lo[k] = __float2bfloat16_rn(static_cast<float>(v - static_cast<double>(__bfloat162float(h))));
    }
}

// factor planes Y^T[i][nu] = C[nu * ldc + i] + sgn * C2[nu * ld2 + i] for i < r, nu < n (pitch kpad)
__global__ void factor_planes_kernel(const double* __restrict__ C, int ldc, const double* __restrict__ C2, int ld2,
                                     double sgn, int r, int n, long long kpad, __nv_bfloat16* __restrict__ hi,
                                     __nv_bfloat16* __restrict__ lo)
{
    const long long total = static_cast<long long>(r) * kpad;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(k / kpad);
        const long long nu = k % kpad;
        double v = 0.0;
        if (nu < n) {
            v = C[nu * ldc + i];
            if (C2) v += sgn * C2[nu * ld2 + i];
        }
        const float x = static_cast<float>(v);
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        hi[k] = h;
        lo[k] = __float2bfloat16_rn(static_cast<float>(v - static_cast<double>(__bfloat162float(h))));
    }
}

__global__ void copy_cols_kernel(const double* __restrict__ C, int ldc, int n, int r, double* __restrict__ out)
{
    const long long total = static_cast<long long>(n) * r;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        out[k] = C[(k / r) * ldc + (k % r)];
}

// U2 = (3 I - U^T U) / 2 stored in place of the product buffer P (r x r)
__global__ void ns_step_kernel(double* __restrict__ P, int r)
{
    const long long rr = static_cast<long long>(r) * r;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < rr;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const bool diag = (k / r) == (k % r);
        P[k] = 0.5 * ((diag ? 3.0 : 0.0) - P[k]);
    }
}

// max |U^T U - I| (P = U^T U) into out (single block)
__global__ void orth_residual_kernel(const double* __restrict__ P, int r, double* __restrict__ out)
{
    __shared__ double red[32];
    double m = 0.0;
    const long long rr = static_cast<long long>(r) * r;
    for (long long k = threadIdx.x; k < rr; k += blockDim.x) {
        const double v = P[k] - (((k / r) == (k % r)) ? 1.0 : 0.0);
        m = fmax(m, fabs(v));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) *out = m;
    }
}

// row-major C (m x n) = alpha op(A) op(B) + beta C
cublasStatus_t gemm_rm(cublasHandle_t h, bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
                       const double* B, int ldb, double beta, double* C, int ldc)
{
    return cublasDgemm(h, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, n, m, k, &alpha, B, ldb, A,
                       lda, &beta, C, ldc);
}

template <class T>
int ri_alloc_zero(T*& p, size_t n, cudaStream_t s)
{
    if (p) return HF_OK;
    int st = ri_alloc(p, n);
    if (st) return st;
    GB_CUDA_TRY(cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(T), s));
    return HF_OK;
}

}  // namespace

int ri_prepare_planes(Engine& e, int nocc, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis, M = r.naux;
    const long long kpad = (n + 63) / 64 * 64;
    int st;
    if (!r.d_Bh) {
        r.kpad_n = kpad;
        const size_t plane = static_cast<size_t>(M) * n * kpad;
        if ((st = ri_alloc(r.d_Bh, plane)) || (st = ri_alloc(r.d_Bl, plane))) return st;
        b_planes_kernel<<<grid_for(static_cast<long long>(plane), 256, e.num_sms), 256, 0, s>>>(r.d_Bp, M, n, kpad,
                                                                                              r.d_Bh, r.d_Bl);
        GB_LAUNCH_CHECK();
    }
    if (nocc > r.r_cap) {
        // factor planes and X planes sized for nocc rows
        for (void* p : {static_cast<void*>(r.d_Yh), static_cast<void*>(r.d_Yl), static_cast<void*>(r.d_Y2h),
                        static_cast<void*>(r.d_Y2l), static_cast<void*>(r.d_Xh), static_cast<void*>(r.d_Xl),
                        static_cast<void*>(r.d_X2h), static_cast<void*>(r.d_X2l), static_cast<void*>(r.d_Cprev),
                        static_cast<void*>(r.d_T1), static_cast<void*>(r.d_M), static_cast<void*>(r.d_U),
                        static_cast<void*>(r.d_U2), static_cast<void*>(r.d_Ca)})
            if (p) cudaFree(p);
        r.d_Yh = r.d_Yl = r.d_Y2h = r.d_Y2l = r.d_Xh = r.d_Xl = r.d_X2h = r.d_X2l = nullptr;
        r.d_Cprev = r.d_T1 = r.d_M = r.d_U = r.d_U2 = r.d_Ca = nullptr;
        r.r_cap = nocc;
        r.r_blk = (nocc + 63) / 64 * 64;
        const size_t yplane = static_cast<size_t>(nocc) * kpad;
        const size_t xplane = static_cast<size_t>(n) * M * r.r_blk;
        if ((st = ri_alloc(r.d_Yh, yplane)) || (st = ri_alloc(r.d_Yl, yplane)) || (st = ri_alloc(r.d_Y2h, yplane)) ||
            (st = ri_alloc(r.d_Y2l, yplane)))
            return st;
        // padding columns of the X planes (i >= nocc) stay zero: the GEMM writes only i < nocc
        if ((st = ri_alloc_zero(r.d_Xh, xplane, s)) || (st = ri_alloc_zero(r.d_Xl, xplane, s)) ||
            (st = ri_alloc_zero(r.d_X2h, xplane, s)) || (st = ri_alloc_zero(r.d_X2l, xplane, s)))
            return st;
        const size_t nr = static_cast<size_t>(n) * nocc, rr = static_cast<size_t>(nocc) * nocc;
        if ((st = ri_alloc(r.d_Cprev, nr)) || (st = ri_alloc(r.d_T1, nr)) || (st = ri_alloc(r.d_Ca, nr)) ||
            (st = ri_alloc(r.d_M, rr)) || (st = ri_alloc(r.d_U, rr)) || (st = ri_alloc(r.d_U2, rr)))
            return st;
    }
    if ((st = ri_alloc_zero(r.d_flag, 1, s)) || (st = ri_alloc(r.d_Kacc, static_cast<size_t>(n) * n))) return st;
    return HF_OK;
}

// X planes (N x naux r_blk) from the factor planes: X[mu][(P, i)] = sum_nu B_P[mu][nu] Y[nu][i]
static int ri_x_planes(Engine& e, const __nv_bfloat16* yh, const __nv_bfloat16* yl, int nocc, __nv_bfloat16* xh,
                       __nv_bfloat16* xl, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis;
    SplitGemmArgs a{};
    a.a_hi = r.d_Bh; a.a_lo = r.d_Bl;
    a.b_hi = yh; a.b_lo = yl;
    a.a_rows = static_cast<long long>(r.naux) * n;
    a.b_rows = nocc;
    a.kpad = r.kpad_n;
    a.mode = kSplitStore;
    a.out_hi = xh; a.out_lo = xl;
    a.rows_per_block = n;
    a.ld_out = static_cast<long long>(r.naux) * r.r_blk;
    a.block_cols = r.r_blk;
    a.col_off = 0;
    a.scale = 1.0f;
    a.error_flag = r.d_flag;
    return split_bf16_gemm(a, e.num_sms, s);
}

static int ri_k_from_x(Engine& e, const __nv_bfloat16* xh, const __nv_bfloat16* xl, const __nv_bfloat16* x2h,
                       const __nv_bfloat16* x2l, int mode, double alpha, double* d_K, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis;
    SplitGemmArgs a{};
    a.a_hi = xh; a.a_lo = xl;
    a.b_hi = x2h; a.b_lo = x2l;
    a.a_rows = n;
    a.b_rows = n;
    a.kpad = static_cast<long long>(r.naux) * r.r_blk;
    a.mode = mode;
    const long long tiles = (n + 127) / 128;
    const long long ntile = (mode == kSymmetricAdd) ? tiles * (tiles + 1) / 2 : tiles * tiles;
    const long long nkb = a.kpad / 64;
    a.split_k = static_cast<int>(std::max<long long>(1, std::min<long long>(nkb, (2LL * e.num_sms + ntile - 1) / ntile)));
    a.K = d_K;
    a.ldk = n;
    a.alpha = alpha;
    a.error_flag = r.d_flag;
    return split_bf16_gemm(a, e.num_sms, s);
}

int ri_k_tc_full(Engine& e, const double* d_C, int ldc, int nocc, double* d_K, cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis;
    int st;
    if ((st = ri_prepare_planes(e, nocc, s))) return st;
    factor_planes_kernel<<<grid_for(static_cast<long long>(nocc) * r.kpad_n, 256, e.num_sms), 256, 0, s>>>(
        d_C, ldc, nullptr, 0, 0.0, nocc, n, r.kpad_n, r.d_Yh, r.d_Yl);
    GB_LAUNCH_CHECK();
    if ((st = ri_x_planes(e, r.d_Yh, r.d_Yl, nocc, r.d_Xh, r.d_Xl, s))) return st;
    GB_CUDA_TRY(cudaMemsetAsync(d_K, 0, sizeof(double) * n * n, s));
    // D = 2 C_occ C_occ^T
    return ri_k_from_x(e, r.d_Xh, r.d_Xl, r.d_Xh, r.d_Xl, kSymmetricAdd, 2.0, d_K, s);
}

int ri_save_occupied(Engine& e, const double* d_C, int ldc, int nocc, cudaStream_t s)
{
    RiState& r = *e.ri;
    int st = ri_prepare_planes(e, nocc, s);
    if (st) return st;
    copy_cols_kernel<<<grid_for(static_cast<long long>(e.num_basis) * nocc, 256, e.num_sms), 256, 0, s>>>(
        d_C, ldc, e.num_basis, nocc, r.d_Cprev);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// K(D_new) - K(D_old) with D = 2 C_occ C_occ^T: the old orbitals are rotated onto the new ones
// (U = polar factor of C_old^T S C_new, Newton-Schulz), then with A = C_new - C_old U and
// S = C_new + C_old U, D_new - D_old = A S^T + S A^T exactly and
// K(dD) = sum_P (B_P A)(B_P S)^T + transpose, whose low-precision error scales with |A|.
int ri_k_tc_delta(Engine& e, const double* d_C, int ldc, int nocc, const double* d_S, double* d_K, bool* aligned,
                  cudaStream_t s)
{
    RiState& r = *e.ri;
    const int n = e.num_basis, k = nocc;
    int st;
    if ((st = ri_prepare_planes(e, nocc, s))) return st;
    cublasSetStream(e.cublas, s);
    // new occupied block (N x k, pitch k) into Ca
    copy_cols_kernel<<<grid_for(static_cast<long long>(n) * k, 256, e.num_sms), 256, 0, s>>>(d_C, ldc, n, k, r.d_Ca);
    GB_LAUNCH_CHECK();
    // M = C_old^T S C_new
    if (gemm_rm(e.cublas, false, false, n, k, n, 1.0, d_S, n, r.d_Ca, k, 0.0, r.d_T1, k) != CUBLAS_STATUS_SUCCESS ||
        gemm_rm(e.cublas, true, false, k, k, n, 1.0, r.d_Cprev, k, r.d_T1, k, 0.0, r.d_M, k) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDgemm (RI alignment) failed"), HF_ERR_SOLVER;
    // Newton-Schulz: U <- U (3 I - U^T U) / 2, from U = M (singular values in (0, 1])
    GB_CUDA_TRY(cudaMemcpyAsync(r.d_U, r.d_M, sizeof(double) * k * k, cudaMemcpyDeviceToDevice, s));
    double res = 1.0;
    *aligned = false;
    for (int it = 0; it < 60; ++it) {
        if (gemm_rm(e.cublas, true, false, k, k, k, 1.0, r.d_U, k, r.d_U, k, 0.0, r.d_U2, k) != CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDgemm (Newton-Schulz) failed"), HF_ERR_SOLVER;
        if (it % 4 == 3) {
            orth_residual_kernel<<<1, 256, 0, s>>>(r.d_U2, k, e.d_scalar + 6);
            GB_LAUNCH_CHECK();
            GB_CUDA_TRY(cudaMemcpyAsync(&res, e.d_scalar + 6, sizeof(double), cudaMemcpyDeviceToHost, s));
            GB_CUDA_TRY(cudaStreamSynchronize(s));
            if (res < 1e-13) { *aligned = true; break; }
        }
        ns_step_kernel<<<grid_for(static_cast<long long>(k) * k, 256, e.num_sms), 256, 0, s>>>(r.d_U2, k);
        GB_LAUNCH_CHECK();
        if (gemm_rm(e.cublas, false, false, k, k, k, 1.0, r.d_U, k, r.d_U2, k, 0.0, r.d_M, k) != CUBLAS_STATUS_SUCCESS)
            return set_error("cublasDgemm (Newton-Schulz) failed"), HF_ERR_SOLVER;
        std::swap(r.d_U, r.d_M);
    }
    if (!*aligned) return HF_OK;  // caller falls back to a full build
    // C_old U into T1
    if (gemm_rm(e.cublas, false, false, n, k, k, 1.0, r.d_Cprev, k, r.d_U, k, 0.0, r.d_T1, k) != CUBLAS_STATUS_SUCCESS)
        return set_error("cublasDgemm (RI alignment) failed"), HF_ERR_SOLVER;
    // A = C_new - C_old U, S = C_new + C_old U as factor planes
    const long long work = static_cast<long long>(k) * r.kpad_n;
    factor_planes_kernel<<<grid_for(work, 256, e.num_sms), 256, 0, s>>>(r.d_Ca, k, r.d_T1, k, -1.0, k, n, r.kpad_n,
                                                                       r.d_Yh, r.d_Yl);
    GB_LAUNCH_CHECK();
    factor_planes_kernel<<<grid_for(work, 256, e.num_sms), 256, 0, s>>>(r.d_Ca, k, r.d_T1, k, 1.0, k, n, r.kpad_n,
                                                                       r.d_Y2h, r.d_Y2l);
    GB_LAUNCH_CHECK();
    if ((st = ri_x_planes(e, r.d_Yh, r.d_Yl, k, r.d_Xh, r.d_Xl, s))) return st;
    if ((st = ri_x_planes(e, r.d_Y2h, r.d_Y2l, k, r.d_X2h, r.d_X2l, s))) return st;
    GB_CUDA_TRY(cudaMemsetAsync(d_K, 0, sizeof(double) * n * n, s));
    return ri_k_from_x(e, r.d_Xh, r.d_Xl, r.d_X2h, r.d_X2l, kSymmetrizedAdd, 1.0, d_K, s);
}

int ri_check_flag(Engine& e)
{
    if (!e.ri || !e.ri->d_flag) return HF_OK;
    int f = 0;
    GB_CUDA_TRY(cudaMemcpy(&f, e.ri->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (f) return set_error("tensor-core GEMM pipeline wait timed out"), HF_ERR_CUDA;
    return HF_OK;
}


namespace {
__global__ void absmax_diff_kernel(const double* __restrict__ A, const double* __restrict__ B, long long nn,
                                   double* __restrict__ out)
{
    __shared__ double red[32];
    double m = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) m = fmax(m, fabs(A[k] - B[k]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) *out = m;
    }
}

__global__ void add_inplace_kernel(double* __restrict__ A, const double* __restrict__ B, long long nn)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x)
        A[k] += B[k];
}
}  // namespace

int ri_absmax_diff(Engine& e, const double* d_A, const double* d_B, double* h_out, cudaStream_t s)
{
    const long long nn = static_cast<long long>(e.num_basis) * e.num_basis;
    absmax_diff_kernel<<<1, 1024, 0, s>>>(d_A, d_B, nn, e.d_scalar + 7);
    GB_LAUNCH_CHECK();
    GB_CUDA_TRY(cudaMemcpyAsync(h_out, e.d_scalar + 7, sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return HF_OK;
}

int ri_add_inplace(Engine& e, double* d_A, const double* d_B, cudaStream_t s)
{
    const long long nn = static_cast<long long>(e.num_basis) * e.num_basis;
    add_inplace_kernel<<<grid_for(nn, 256, e.num_sms), 256, 0, s>>>(d_A, d_B, nn);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int hf_engine_set_auxiliary_basis(hf_engine* eng, const hf_primitive_shell* aux_prims, int num_aux_primitives,
                                  const double* aux_cgto_norm, int num_aux_basis)
{
    clear_error();
    if (!eng || !aux_prims || !aux_cgto_norm || num_aux_primitives <= 0 || num_aux_basis <= 0)
        return set_error("null argument or empty auxiliary basis"), HF_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<Engine*>(eng)->nmol != 1)
        return set_error("RI: single-molecule engines only"), HF_ERR_INVALID_ARGUMENT;
    return ri_set_auxiliary(*reinterpret_cast<Engine*>(eng), aux_prims, num_aux_primitives, aux_cgto_norm,
                            num_aux_basis);
}

int hf_compute_two_center_eris(hf_engine* eng, double* d_metric, void* stream)
{
    clear_error();
    if (!eng || !d_metric) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (!e.ri) return set_error("no auxiliary basis attached"), HF_ERR_INVALID_ARGUMENT;
    return ri_metric(e, d_metric, static_cast<cudaStream_t>(stream));
}

int hf_compute_three_center_eris(hf_engine* eng, double* d_three_center, void* stream)
{
    clear_error();
    if (!eng || !d_three_center) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (!e.ri) return set_error("no auxiliary basis attached"), HF_ERR_INVALID_ARGUMENT;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long npk = static_cast<long long>(e.num_basis) * (e.num_basis + 1) / 2;
    double* tmp = nullptr;
    GB_CUDA_TRY(cudaMalloc(&tmp, sizeof(double) * npk * e.ri->naux));
    int st = ri_three_center_packed(e, tmp, s);
    if (!st) st = ri_expand(e, tmp, e.ri->naux, d_three_center, s);
    cudaStreamSynchronize(s);
    cudaFree(tmp);
    return st;
}

int hf_compute_ri_intermediate_b(hf_engine* eng, double* d_b_out, void* stream)
{
    clear_error();
    if (!eng) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    if (!e.ri) return set_error("no auxiliary basis attached"), HF_ERR_INVALID_ARGUMENT;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = ri_build_b(e, s);
    if (st) return st;
    if (d_b_out) return ri_expand(e, e.ri->d_Bp, e.ri->naux, d_b_out, s);
    return HF_OK;
}

int hf_compute_jk_ri(hf_engine* eng, const double* d_density, double* d_J, double* d_K, void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_J || !d_K) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = ri_require_b(e, s);
    if (st) return st;
    if ((st = ri_j(e, d_density, d_J, s))) return st;
    return ri_k_density(e, d_density, d_K, s);
}

int hf_compute_fock_ri_rhf(hf_engine* eng, const double* d_density, const double* d_core_hamiltonian,
                           double* d_fock, void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_core_hamiltonian || !d_fock) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = ri_require_b(e, s);
    if (st) return st;
    double *J, *K;
    if ((st = ri_work_buffers(e, &J, &K))) return st;
    if ((st = ri_j(e, d_density, J, s))) return st;
    if ((st = ri_k_density(e, d_density, K, s))) return st;
    return ri_fock_from_jk(e, d_core_hamiltonian, J, K, nullptr, false, d_fock, s);
}

}  // extern "C"
