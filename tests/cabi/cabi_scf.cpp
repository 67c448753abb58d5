// A caller of the C ABI written in C++, with no Python in the process: water
// STO-3G from files through hf_molecule_from_files -> hf_engine_create ->
// hf_compute_core_hamiltonian -> hf_rhf_scf, then the allocation-free DIIS on
// device buffers it owns.  Prints `key value` lines that the test reads.
// Usage: cabi_scf <water.xyz> <sto-3g.gbs>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "gansu_gb300.h"

#define CHECK(call)                                                                  \
    do {                                                                             \
        const int st_ = (call);                                                      \
        if (st_ != HF_OK) {                                                          \
            std::fprintf(stderr, "%s failed (%d): %s\n", #call, st_, hf_last_error()); \
            return 1;                                                                \
        }                                                                            \
    } while (0)

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    std::printf("version %s\n", hf_version());
    hf_molecule* mol = nullptr;
    CHECK(hf_molecule_from_files(argv[1], argv[2], 0, 0, &mol));
    int nbf = 0, nprim = 0, natom = 0, nel = 0, na = 0, nb = 0;
    CHECK(hf_molecule_sizes(mol, &nbf, &nprim, &natom, &nel, &na, &nb));
    std::vector<hf_primitive_shell> prims(nprim);
    std::vector<double> cgto(nbf);
    std::vector<hf_atom> atoms(natom);
    CHECK(hf_molecule_get(mol, prims.data(), cgto.data(), atoms.data()));
    std::printf("num_basis %d\nnum_primitives %d\nnum_electrons %d\n", nbf, nprim, nel);

    hf_engine* eng = nullptr;
    CHECK(hf_engine_create(prims.data(), nprim, cgto.data(), nbf, atoms.data(), natom, 1e-12, &eng));
    const size_t nn = static_cast<size_t>(nbf) * nbf;
    double *S = nullptr, *H = nullptr, *D = nullptr, *E = nullptr, *F = nullptr, *out = nullptr;
    if (cudaMalloc(&S, nn * sizeof(double)) || cudaMalloc(&H, nn * sizeof(double)) ||
        cudaMalloc(&D, nn * sizeof(double)) || cudaMalloc(&E, 2 * nn * sizeof(double)) ||
        cudaMalloc(&F, 2 * nn * sizeof(double)) || cudaMalloc(&out, nn * sizeof(double)))
        return 3;
    CHECK(hf_compute_core_hamiltonian(eng, S, H, nullptr));
    std::vector<double> hS(nn);
    cudaMemcpy(hS.data(), S, nn * sizeof(double), cudaMemcpyDeviceToHost);
    std::printf("overlap_00 %.17g\n", hS[0]);

    hf_scf_options opt;
    hf_scf_options_default(&opt);
    opt.convergence_threshold = 1e-10;
    hf_scf_result res;
    CHECK(hf_rhf_scf(eng, nel, &opt, &res, D, nullptr, nullptr, nullptr));
    std::printf("total_energy %.15f\niterations %d\nconverged %d\n", res.total_energy, res.iterations, res.converged);

    // allocation-free DIIS: two pairs, the second error half the first -> weights (-1, 2)
    std::vector<double> he(2 * nn), hf(2 * nn);
    for (size_t k = 0; k < nn; ++k) {
        he[k] = std::sin(0.1 * k + 0.3);
        he[nn + k] = 0.5 * he[k];
        hf[k] = 1.0;
        hf[nn + k] = 3.0;
    }
    cudaMemcpy(E, he.data(), 2 * nn * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(F, hf.data(), 2 * nn * sizeof(double), cudaMemcpyHostToDevice);
    CHECK(hf_compute_fock_diis_noalloc(E, F, out, 2, nbf, nullptr));
    double o0 = 0.0;
    cudaMemcpy(&o0, out, sizeof(double), cudaMemcpyDeviceToHost);
    std::printf("diis_noalloc_00 %.15f\n", o0);

    cudaFree(S); cudaFree(H); cudaFree(D); cudaFree(E); cudaFree(F); cudaFree(out);
    hf_engine_destroy(eng);
    hf_molecule_destroy(mol);
    return 0;
}
