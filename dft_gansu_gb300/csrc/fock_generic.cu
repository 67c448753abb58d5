// Direct Fock build for the quartet classes whose integral block exceeds the
// register budget of the fully unrolled kernels, with runtime angular momenta
// (the column kernel of fock_column.cuh), and the stored-ERI tensor for every
// class.
#include "engine.hpp"
#include "fock_column.cuh"

namespace gb {

namespace {

using namespace fock_column;

// Stored-ERI path (src/gpu_manager.cu:434-517): one (quartet, c, d) per thread,
// scaled by s_a s_b s_c s_d and written to the eight permutations.
__global__ void __launch_bounds__(kFockThreads)
eri_generic_kernel(const FockClassLaunch L, int ncd, const double* __restrict__ scale, double* __restrict__ eri)
{
    const long long total = L.off[L.nentry] * ncd;
    const long long N = L.num_basis;
    double I[kNAB];
    for (long long w = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; w < total;
         w += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long qi = w / ncd;
        const int cd = static_cast<int>(w % ncd);
        const int e = find_entry(L.off, L.nentry, qi);
        // a bra split over entries by primitive range: its first entry writes the whole quartet
        const int prim = entry_prim_range(L, e);
        if (prim > 0 && (prim & 0xffff) != 0) continue;
        const int bra = __ldg(L.entry_bra + e);
        const int ket = L.ket_base + __ldg(L.entry_lo + e) + static_cast<int>(qi - __ldg(L.off + e));
        const ShellPairDev bp = L.pairs[bra];
        const ShellPairDev kp = L.pairs[ket];
        quartet_column<double>(bp, kp, cd, 0, bp.pp_n, static_cast<const PrimPair64*>(L.prim_pairs),
                               static_cast<const double*>(L.boys_table), L.schwarz_threshold, I);
        const int na = ncart(bp.la), nb = ncart(bp.lb), nd = ncart(kp.lb);
        const long long c = kp.bfA + cd / nd, d = kp.bfB + cd % nd;
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                const long long a = bp.bfA + ia, b = bp.bfB + ib;
                const double v = I[ia * nb + ib] * scale[a] * scale[b] * scale[c] * scale[d];
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

}  // namespace

void launch_fock_generic(bool fp32, const FockClassLaunch& launch, int ncd, int grid, cudaStream_t stream)
{
    if (fp32) column_kernel<float, RuntimeColumn<float>><<<grid, kFockThreads, 0, stream>>>(launch, ncd);
    else column_kernel<double, RuntimeColumn<double>><<<grid, kFockThreads, 0, stream>>>(launch, ncd);
}

void launch_eri_generic(const FockClassLaunch& launch, int ncd, const double* scale, double* eri, int grid,
                        cudaStream_t stream)
{
    eri_generic_kernel<<<grid, kFockThreads, 0, stream>>>(launch, ncd, scale, eri);
}

}  // namespace gb
