/*
 * CPU driver for the reference's own integral kernels (TEST INFRASTRUCTURE).
 *
 * The reference's src/int2e.cu and src/int1e.cu are compiled unchanged from
 * their own sources with g++ (see oracle/refcpu/Makefile and
 * cuda_cpu_shim.h).  This file replays the host launch loops of the reference
 * and runs each __global__ function once per "thread id" on the CPU:
 *   - computeSchwarzUpperBounds   src/gpu_manager.cu:2154-2179
 *   - computeERIMatrix            src/gpu_manager.cu:434-517
 *   - computeCoreHamiltonianMatrix src/gpu_manager.cu:333-404 (+ the upper->lower
 *     copy that Matrix_Symmetrization does, src/int1e.cu:67-84)
 *   - makeShellPairTypeInfo       src/gpu_manager.cu:413-432
 *   - computeAuxiliarySchwarzUpperBounds, computeTwoCenterERIs,
 *     computeThreeCenterERIs      src/gpu_manager.cu:1963-2210 (pair indices in
 *     the order of the Schwarz kernels; the reference sorts them by bound,
 *     src/eri.cu:119-236, which changes only the summation order)
 * The Boys table is the reference's own (src/boys/boys_30720.h, loaded the
 * same way as src/hf.cu:74-77).
 *
 * Its outputs are the reference's S, H, primitive Schwarz bounds and full ERI
 * tensor for small molecules, used to pin the oracle (oracle/md_oracle.c).
 */
#include <vector>
#include <tuple>
#include <algorithm>
#include <cstring>

#include "types.hpp"
#include "int2e.hpp"
#include "int1e.hpp"
#include "int2c2e.hpp"
#include "int3c2e.hpp"
#include "boys/boys_30720.h"

thread_local RefcpuDim3 threadIdx{0, 0, 0};
thread_local RefcpuDim3 blockIdx{0, 0, 0};
thread_local RefcpuDim3 blockDim{1, 1, 1};
thread_local RefcpuDim3 gridDim{1, 1, 1};

namespace {

using namespace gansu;

template <class F>
void run_threads(size_t n, F&& f)
{
#pragma omp parallel for schedule(dynamic, 64)
    for (long long id = 0; id < static_cast<long long>(n); ++id) {
        blockDim = {1, 1, 1};
        threadIdx = {0, 0, 0};
        blockIdx = {static_cast<unsigned int>(id), 0, 0};
        f();
    }
}

int index_2to1_horizontal(int i, int j, const int n)
{
    if (i > j) std::swap(i, j);
    return j - static_cast<int>(i * (i - 2 * n + 1) / 2);
}

std::vector<PrimitiveShell> make_prims(int n, const double* exps, const double* coefs, const double* xyz,
                                       const int* shell_type, const long long* basis_index, const int* atom_index)
{
    std::vector<PrimitiveShell> prims(n);
    for (int i = 0; i < n; ++i) {
        prims[i].exponent = exps[i];
        prims[i].coefficient = coefs[i];
        prims[i].coordinate = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        prims[i].shell_type = shell_type[i];
        prims[i].basis_index = static_cast<size_t>(basis_index[i]);
        prims[i].atom_index = atom_index[i];
    }
    return prims;
}

std::vector<ShellTypeInfo> type_infos(const std::vector<PrimitiveShell>& prims)
{
    std::vector<ShellTypeInfo> sti(prims.back().shell_type + 1, {0, 0});
    for (auto& p : prims) sti[p.shell_type].count++;
    for (size_t i = 1; i < sti.size(); ++i) sti[i].start_index = sti[i - 1].start_index + sti[i - 1].count;
    return sti;
}

}  // namespace

extern "C" {

/* Primitive list must already be ordered by shell type (as Molecular sorts it). */
int refcpu_integrals(int nprim, const double* exps, const double* coefs, const double* xyz, const int* shell_type,
                     const long long* basis_index, const int* atom_index, const double* cgto_norm, int nbf,
                     int natom, const int* atomic_number, const double* atom_xyz, double thr,
                     double* S, double* H, double* eri, double* schwarz, long long* n_schwarz)
{
    std::vector<PrimitiveShell> prims(nprim);
    for (int i = 0; i < nprim; ++i) {
        prims[i].exponent = exps[i];
        prims[i].coefficient = coefs[i];
        prims[i].coordinate = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        prims[i].shell_type = shell_type[i];
        prims[i].basis_index = static_cast<size_t>(basis_index[i]);
        prims[i].atom_index = atom_index[i];
    }
    const int max_type = prims.back().shell_type;
    std::vector<ShellTypeInfo> sti(max_type + 1, {0, 0});
    for (auto& p : prims) sti[p.shell_type].count++;
    for (int i = 1; i <= max_type; ++i) sti[i].start_index = sti[i - 1].start_index + sti[i - 1].count;
    const int ntype = static_cast<int>(sti.size());

    std::vector<ShellPairTypeInfo> spti(ntype * (ntype + 1) / 2);
    size_t npairs = 0;
    for (int s0 = 0; s0 < ntype; ++s0)
        for (int s1 = s0; s1 < ntype; ++s1) {
            size_t nb = (s0 == s1) ? static_cast<size_t>(sti[s0].count) * (sti[s0].count + 1) / 2
                                   : static_cast<size_t>(sti[s0].count) * sti[s1].count;
            spti[index_2to1_horizontal(s0, s1, ntype)] = {nb, npairs};
            npairs += nb;
        }

    std::vector<Atom> atoms(natom);
    for (int i = 0; i < natom; ++i)
        atoms[i] = {atomic_number[i], {atom_xyz[3 * i], atom_xyz[3 * i + 1], atom_xyz[3 * i + 2]}};

    const double* boys = gansu::h_boys_grid;

    /* Schwarz bounds */
    std::vector<double> bounds(npairs, 0.0);
    for (int s0 = 0; s0 < ntype; ++s0)
        for (int s1 = s0; s1 < ntype; ++s1) {
            const size_t head = spti[index_2to1_horizontal(s0, s1, ntype)].start_index;
            const size_t nb = spti[index_2to1_horizontal(s0, s1, ntype)].count;
            auto k = gpu::get_schwarz_kernel(s0, s1);
            run_threads(nb, [&] { k(prims.data(), cgto_norm, sti[s0], sti[s1], head, nb, boys, bounds.data()); });
        }
    if (schwarz) std::memcpy(schwarz, bounds.data(), sizeof(double) * npairs);
    if (n_schwarz) *n_schwarz = static_cast<long long>(npairs);

    /* ERI tensor */
    if (eri) {
        const size_t N = nbf;
        std::memset(eri, 0, sizeof(double) * N * N * N * N);
        std::vector<std::tuple<int, int, int, int>> quads;
        for (int a = 0; a < ntype; ++a)
            for (int b = a; b < ntype; ++b)
                for (int c = 0; c < ntype; ++c)
                    for (int d = c; d < ntype; ++d)
                        if (a < c || (a == c && b <= d)) quads.emplace_back(a, b, c, d);
        std::reverse(quads.begin(), quads.end());
        for (auto& q : quads) {
            int s0, s1, s2, s3;
            std::tie(s0, s1, s2, s3) = q;
            const size_t num_bra = (s0 == s1) ? static_cast<size_t>(sti[s0].count) * (sti[s0].count + 1) / 2
                                              : static_cast<size_t>(sti[s0].count) * sti[s1].count;
            const size_t num_ket = (s2 == s3) ? static_cast<size_t>(sti[s2].count) * (sti[s2].count + 1) / 2
                                              : static_cast<size_t>(sti[s2].count) * sti[s3].count;
            const size_t num_braket = ((s0 == s2) && (s1 == s3)) ? num_bra * (num_bra + 1) / 2 : num_bra * num_ket;
            const size_t head_bra = spti[index_2to1_horizontal(s0, s1, ntype)].start_index;
            const size_t head_ket = spti[index_2to1_horizontal(s2, s3, ntype)].start_index;
            auto k = gpu::get_eri_kernel(s0, s1, s2, s3);
            run_threads(num_braket, [&] {
                k(eri, prims.data(), cgto_norm, sti[s0], sti[s1], sti[s2], sti[s3], num_braket, thr, bounds.data(), nbf,
                  boys, head_bra, head_ket);
            });
        }
    }

    /* one-electron: S and H = T + V, upper triangle then mirrored */
    if (S && H) {
        const size_t N = nbf;
        std::memset(S, 0, sizeof(double) * N * N);
        std::memset(H, 0, sizeof(double) * N * N);
        for (int s0 = ntype - 1; s0 >= 0; s0--)
            for (int s1 = ntype - 1; s1 >= s0; s1--) {
                const int np = (s0 == s1) ? (sti[s0].count * (sti[s0].count + 1) / 2) : (sti[s0].count * sti[s1].count);
                auto ok = gpu::get_overlap_kinetic_kernel(s0, s1);
                auto nk = gpu::get_nuclear_attraction_kernel(s0, s1);
                run_threads(np, [&] { ok(S, H, prims.data(), cgto_norm, sti[s0], sti[s1], np, nbf); });
                run_threads(np, [&] {
                    nk(H, prims.data(), cgto_norm, atoms.data(), natom, sti[s0], sti[s1], np, nbf, boys);
                });
            }
        for (size_t i = 0; i < N; ++i)
            for (size_t j = 0; j < i; ++j) {
                S[i * N + j] = S[j * N + i];
                H[i * N + j] = H[j * N + i];
            }
    }
    return 0;
}

/* The reference's RI integrals: metric V[P*naux+Q] = (P|Q), three-centre
 * T[(P*nbf + mu)*nbf + nu] = (mu nu|P), and the auxiliary Schwarz bounds. */
int refcpu_ri_integrals(int nprim, const double* exps, const double* coefs, const double* xyz, const int* shell_type,
                        const long long* basis_index, const int* atom_index, const double* cgto, int nbf,
                        int naprim, const double* aexps, const double* acoefs, const double* axyz,
                        const int* ashell_type, const long long* abasis_index, const int* aatom_index,
                        const double* acgto, int naux, double thr, double* V, double* T, double* aux_bounds)
{
    std::vector<PrimitiveShell> prims = make_prims(nprim, exps, coefs, xyz, shell_type, basis_index, atom_index);
    std::vector<PrimitiveShell> aprims = make_prims(naprim, aexps, acoefs, axyz, ashell_type, abasis_index, aatom_index);
    std::vector<ShellTypeInfo> sti = type_infos(prims), asti = type_infos(aprims);
    const int ntype = static_cast<int>(sti.size()), natype = static_cast<int>(asti.size());
    const double* boys = gansu::h_boys_grid;

    // AO primitive-pair Schwarz bounds and the pair index lists in the same order
    std::vector<ShellPairTypeInfo> spti(ntype * (ntype + 1) / 2);
    size_t npairs = 0;
    for (int s0 = 0; s0 < ntype; ++s0)
        for (int s1 = s0; s1 < ntype; ++s1) {
            size_t nb = (s0 == s1) ? static_cast<size_t>(sti[s0].count) * (sti[s0].count + 1) / 2
                                   : static_cast<size_t>(sti[s0].count) * sti[s1].count;
            spti[index_2to1_horizontal(s0, s1, ntype)] = {nb, npairs};
            npairs += nb;
        }
    std::vector<double> bounds(npairs, 0.0);
    std::vector<size_t2> pair_idx(npairs);
    for (int s0 = 0; s0 < ntype; ++s0)
        for (int s1 = s0; s1 < ntype; ++s1) {
            const size_t head = spti[index_2to1_horizontal(s0, s1, ntype)].start_index;
            const size_t nb = spti[index_2to1_horizontal(s0, s1, ntype)].count;
            auto k = gpu::get_schwarz_kernel(s0, s1);
            run_threads(nb, [&] { k(prims.data(), cgto, sti[s0], sti[s1], head, nb, boys, bounds.data()); });
            for (size_t id = 0; id < nb; ++id) {
                if (s0 == s1) {
                    const size_t r2 = static_cast<size_t>(std::floor((std::sqrt(8.0 * id + 1) - 1) / 2));
                    pair_idx[head + id] = {id - r2 * (r2 + 1) / 2, r2};
                } else {
                    pair_idx[head + id] = {id / sti[s1].count, id % sti[s1].count};
                }
            }
        }
    // auxiliary bounds
    std::vector<double> abounds(naprim, 0.0);
    for (int s0 = 0; s0 < natype; ++s0) {
        auto k = gpu::get_schwarz_aux_kernel(s0);
        const size_t head = asti[s0].start_index, nb = asti[s0].count;
        run_threads(nb, [&] { k(aprims.data(), acgto, asti[s0], head, nb, boys, abounds.data()); });
    }
    if (aux_bounds) std::memcpy(aux_bounds, abounds.data(), sizeof(double) * naprim);
    // two-centre metric
    std::memset(V, 0, sizeof(double) * naux * naux);
    for (int a = 0; a < natype; ++a)
        for (int b = a; b < natype; ++b) {
            const int np = (a == b) ? asti[a].count * (asti[a].count + 1) / 2 : asti[a].count * asti[b].count;
            auto k = gpu::get_2center_kernel(a, b);
            run_threads(np, [&] { k(V, aprims.data(), acgto, asti[a], asti[b], np, abounds.data(), thr, naux, boys); });
        }
    // three-centre tensor
    std::memset(T, 0, sizeof(double) * static_cast<size_t>(naux) * nbf * nbf);
    for (int a = 0; a < ntype; ++a)
        for (int b = a; b < ntype; ++b)
            for (int c = 0; c < natype; ++c) {
                const size_t head = spti[index_2to1_horizontal(a, b, ntype)].start_index;
                const int64_t ntask = static_cast<int64_t>(spti[index_2to1_horizontal(a, b, ntype)].count) * asti[c].count;
                auto k = gpu::get_3center_kernel(a, b, c);
                run_threads(ntask, [&] {
                    k(T, prims.data(), aprims.data(), cgto, acgto, sti[a], sti[b], asti[c], ntask, nbf,
                      &pair_idx[head], &bounds[head], abounds.data(), thr, naux, boys);
                });
            }
    return 0;
}

}  // extern "C"
