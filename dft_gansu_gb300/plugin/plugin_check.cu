// Compile check of the reference-side plugin and shims against the reference's
// own headers (include/eri.hpp, include/rhf.hpp, include/uhf.hpp,
// include/gpu_manager.hpp): a translation unit that instantiates every plugin
// class and takes the address of every shim.  Compiled (not linked) by the
// host tests when the reference tree is available.
#include "gansu_gb300_gpu_shims.cu"

namespace {
[[maybe_unused]] void instantiate(gansu::RHF& rhf, gansu::UHF& uhf)
{
    std::unique_ptr<gansu::ERI> a = std::make_unique<gansu::ERI_GB300_Direct_RHF>(rhf);
    std::unique_ptr<gansu::ERI> b = std::make_unique<gansu::ERI_GB300_Direct_RHF>(rhf, HF_PRECISION_MIXED, 0.1, true);
    std::unique_ptr<gansu::ERI> c = std::make_unique<gansu::ERI_GB300_Direct_UHF>(uhf);
    a->precomputation();
    a->compute_fock_matrix();
    (void)b->get_algorithm_name();
    (void)c->get_algorithm_name();
}
[[maybe_unused]] auto* p1 = &gansu::gpu::computeDIISErrorMatrix;
[[maybe_unused]] auto* p2 = &gansu::gpu::computeFockMatrixDIIS;
[[maybe_unused]] auto* p3 = &gansu::gpu::computeFockMatrix_RHF;
[[maybe_unused]] auto* p4 = &gansu::gpu::computeERIMatrix;
}  // namespace
