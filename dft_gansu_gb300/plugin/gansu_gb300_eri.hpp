// ERI plugins that put libgansu_gb300 behind the reference's own plugin boundary.
//
// gansu::ERI (include/eri.hpp:36-63) is the reference's two-electron backend:
// RHF::RHF picks one by eri_method (src/rhf.cu:72-88), calls precomputation()
// once (RHF::precompute_eri_matrix, src/rhf.cu:110-114) and
// compute_fock_matrix() every iteration (src/rhf.cu:275-279).  The classes
// here create one engine in precomputation() from the getters the reference
// already has (include/hf.hpp:144-208, include/rhf.hpp:78-92,
// include/uhf.hpp:86-115) and run the fused direct build on the reference's
// own device matrices.  PrimitiveShell and Atom have the binary layouts of
// hf_primitive_shell and hf_atom (checked below), so the host copies pass as
// they are.
//
// Include this header in the reference's build (it needs the reference's
// include/ directory and this repository's include/) and register the plugins
// next to the existing methods in RHF::RHF / UHF::UHF:
//     else if (eri_method == "direct")
//         set_eri_method(std::make_unique<gansu::ERI_GB300_Direct_RHF>(*this));
//     else if (eri_method == "direct_mixed")
//         set_eri_method(std::make_unique<gansu::ERI_GB300_Direct_RHF>(*this, HF_PRECISION_MIXED, 0.1));
#pragma once

#include <string>
#include <type_traits>

#include "eri.hpp"
#include "gansu_gb300.h"
#include "rhf.hpp"
#include "uhf.hpp"

namespace gansu {

static_assert(sizeof(PrimitiveShell) == sizeof(hf_primitive_shell), "PrimitiveShell layout");
static_assert(sizeof(Atom) == sizeof(hf_atom), "Atom layout");
static_assert(std::is_same<real_t, double>::value, "the engine works on double matrices");

// the engine of the most recent plugin, for the gansu::gpu shims (gansu_gb300_gpu_shims.cu)
inline hf_engine*& gb300_shared_engine()
{
    static hf_engine* e = nullptr;
    return e;
}

inline void gb300_check(int st)
{
    if (st != HF_OK) THROW_EXCEPTION(std::string("libgansu_gb300: ") + hf_last_error());
}

// one engine over the molecule of an HF object (the plugin's precomputation)
inline hf_engine* gb300_create_engine(const HF& hf, bool autotune, const double* d_any_density)
{
    const auto& prims = hf.get_primitive_shells();
    const auto& cgto = hf.get_cgto_nomalization_factors();
    const auto& atoms = hf.get_atoms();
    hf_engine* e = nullptr;
    gb300_check(hf_engine_create(reinterpret_cast<const hf_primitive_shell*>(prims.host_ptr()),
                                 static_cast<int>(prims.size()), cgto.host_ptr(), hf.get_num_basis(),
                                 reinterpret_cast<const hf_atom*>(atoms.host_ptr()), static_cast<int>(atoms.size()),
                                 hf.get_schwarz_screening_threshold(), &e));
    if (autotune) {
        // grid caps and branch count chosen by timing (~1 s); every later build replays a CUDA graph
        hf_autotune_report rep;
        gb300_check(hf_engine_autotune(e, d_any_density, &rep, nullptr));
        gb300_check(hf_engine_set_fock_schedule(e, rep.num_branches, 1));
    }
    gb300_shared_engine() = e;
    return e;
}

// eri_method = direct (the reference's ERI_Direct_RHF throws, src/gpu_manager.cu:2212-2227):
// F = H + J(D) - K(D)/2 by the fused McMurchie-Davidson build, FP64 or the mixed tier
class ERI_GB300_Direct_RHF : public ERI {
public:
    explicit ERI_GB300_Direct_RHF(RHF& rhf, int precision = HF_PRECISION_FP64, double mixed_threshold = 0.1,
                                  bool autotune = false)
        : rhf_(rhf), precision_(precision), tau_(mixed_threshold), autotune_(autotune)
    {
    }
    ~ERI_GB300_Direct_RHF() override
    {
        if (gb300_shared_engine() == engine_) gb300_shared_engine() = nullptr;
        hf_engine_destroy(engine_);
    }
    void precomputation() override
    {
        engine_ = gb300_create_engine(rhf_, autotune_, rhf_.get_density_matrix().device_ptr());
    }
    void compute_fock_matrix() override
    {
        gb300_check(hf_compute_fock_direct_rhf(engine_, rhf_.get_density_matrix().device_ptr(),
                                               rhf_.get_core_hamiltonian_matrix().device_ptr(),
                                               rhf_.get_fock_matrix().device_ptr(), precision_, tau_, nullptr));
    }
    std::string get_algorithm_name() override
    {
        return precision_ == HF_PRECISION_MIXED ? "GB300 direct, FP32/FP64 mixed" : "GB300 direct";
    }
    hf_engine* engine() const { return engine_; }

private:
    RHF& rhf_;
    hf_engine* engine_ = nullptr;
    int precision_;
    double tau_;
    bool autotune_;
};

// UHF: J and K of both spin densities on one engine, combined as computeFockMatrix_UHF
// does (F_s = H + J(D_a + D_b) - K(D_s)); J(D_a + D_b) = J(D_a) + J(D_b)
class ERI_GB300_Direct_UHF : public ERI {
public:
    explicit ERI_GB300_Direct_UHF(UHF& uhf, int precision = HF_PRECISION_FP64, double mixed_threshold = 0.1)
        : uhf_(uhf), precision_(precision), tau_(mixed_threshold)
    {
    }
    ~ERI_GB300_Direct_UHF() override
    {
        if (gb300_shared_engine() == engine_) gb300_shared_engine() = nullptr;
        hf_engine_destroy(engine_);
        for (double* p : {Ja_, Ka_, Jb_, Kb_}) cudaFree(p);
    }
    void precomputation() override
    {
        engine_ = gb300_create_engine(uhf_, false, nullptr);
        const size_t bytes = sizeof(double) * uhf_.get_num_basis() * uhf_.get_num_basis();
        for (double** p : {&Ja_, &Ka_, &Jb_, &Kb_})
            if (cudaMalloc(p, bytes) != cudaSuccess) THROW_EXCEPTION("cudaMalloc failed");
    }
    void compute_fock_matrix() override
    {
        gb300_check(hf_compute_jk_direct(engine_, uhf_.get_density_matrix_a().device_ptr(), Ja_, Ka_, precision_,
                                         tau_, nullptr));
        gb300_check(hf_compute_jk_direct(engine_, uhf_.get_density_matrix_b().device_ptr(), Jb_, Kb_, precision_,
                                         tau_, nullptr));
        gb300_check(hf_combine_uhf_fock(uhf_.get_core_hamiltonian_matrix().device_ptr(), Ja_, Jb_, Ka_, Kb_,
                                        uhf_.get_fock_matrix_a().device_ptr(), uhf_.get_fock_matrix_b().device_ptr(),
                                        uhf_.get_num_basis(), nullptr));
    }
    std::string get_algorithm_name() override { return "GB300 direct (UHF)"; }

private:
    UHF& uhf_;
    hf_engine* engine_ = nullptr;
    int precision_;
    double tau_;
    double *Ja_ = nullptr, *Ka_ = nullptr, *Jb_ = nullptr, *Kb_ = nullptr;
};

}  // namespace gansu
