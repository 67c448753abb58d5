// gansu::gpu free functions (include/gpu_manager.hpp:34-109) implemented on
// libgansu_gb300, for callers that use the kernel-host seam directly.  Linking
// this file into the reference in place of the same functions of
// src/gpu_manager.cu keeps every caller unchanged: same signatures, device
// pointers in, exceptions (THROW_EXCEPTION, include/utils.hpp:91) on failure.
// The DIIS shims use the workspaces of the engine the ERI plugin created
// (gb300_shared_engine, gansu_gb300_eri.hpp).
#include "gansu_gb300_eri.hpp"
#include "gpu_manager.hpp"

namespace gansu::gpu {

void computeDIISErrorMatrix(const real_t* d_overlap_matrix, const real_t* d_transform_matrix,
                            const real_t* d_fock_matrix, const real_t* d_density_matrix, real_t* d_diis_error_matrix,
                            const int num_basis, const bool is_include_transform)
{
    (void)num_basis;  // the engine knows N
    gb300_check(hf_compute_diis_error(gb300_shared_engine(), d_overlap_matrix, d_transform_matrix, d_fock_matrix,
                                      d_density_matrix, d_diis_error_matrix, is_include_transform ? 1 : 0, nullptr));
}

void computeFockMatrixDIIS(real_t* d_error_matrices, real_t* d_fock_matrices, real_t* d_new_fock_matrix,
                           const int num_prev, const int num_basis)
{
    // no engine needed: the allocation-free entry (at most 16 stored pairs)
    gb300_check(hf_compute_fock_diis_noalloc(d_error_matrices, d_fock_matrices, d_new_fock_matrix, num_prev,
                                             num_basis, nullptr));
}

void computeFockMatrix_RHF(const real_t* d_density_matrix, const real_t* d_core_hamiltonian_matrix,
                           const real_t* d_eri, real_t* d_fock_matrix, const int num_basis)
{
    gb300_check(hf_compute_fock_stored_rhf(d_density_matrix, d_core_hamiltonian_matrix, d_eri, d_fock_matrix,
                                           num_basis, nullptr));
}

void computeERIMatrix(const std::vector<ShellTypeInfo>& shell_type_infos,
                      const std::vector<ShellPairTypeInfo>& shell_pair_type_infos,
                      const PrimitiveShell* d_primitive_shells, const real_t* d_boys_grid,
                      const real_t* d_cgto_normalization_factors, real_t* d_eri_matrix,
                      const real_t* d_schwarz_upper_bound_factors, const real_t schwarz_screening_threshold,
                      const int num_basis, const bool verbose)
{
    // the engine holds the molecule and its own Boys table and bounds; the reference's
    // device arrays describe the same molecule
    (void)shell_type_infos; (void)shell_pair_type_infos; (void)d_primitive_shells; (void)d_boys_grid;
    (void)d_cgto_normalization_factors; (void)d_schwarz_upper_bound_factors; (void)schwarz_screening_threshold;
    (void)num_basis; (void)verbose;
    gb300_check(hf_compute_eri_matrix(gb300_shared_engine(), d_eri_matrix, nullptr));
}

}  // namespace gansu::gpu
