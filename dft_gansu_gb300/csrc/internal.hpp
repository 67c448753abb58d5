// Internal host-side types of libgansu_gb300 (never exposed through the C ABI).
#pragma once
#include <string>
#include <vector>

#include "gansu_gb300.h"

namespace gb {

// ------------------------------------------------------------ errors
void set_error(const std::string& msg);
void clear_error();
// process-wide count of kernel launches issued by this library
void count_launch();
// adds n (may be negative) to the count: launches replayed from a CUDA graph,
// or recorded into one during a capture (which run later, not then)
void count_launches(long long n);
long long launch_count();

struct Molecule {
    std::vector<hf_atom> atoms;
    std::vector<hf_primitive_shell> prims;  // sorted by shell type
    std::vector<double> cgto;               // per basis function
    int num_basis = 0;
    int num_electrons = 0, num_alpha = 0, num_beta = 0;
};

int element_to_z(const std::string& sym);
const char* z_to_element(int z);
double cgto_factor(int L, const std::vector<double>& a, const std::vector<double>& c);

}  // namespace gb

#ifdef __CUDACC__
#include <cuda_runtime.h>
#define GB_CUDA_TRY(expr)                                                                                 \
    do {                                                                                                  \
        cudaError_t _e = (expr);                                                                          \
        if (_e != cudaSuccess) {                                                                          \
            gb::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));                            \
            cudaGetLastError(); /* a non-sticky error must not surface again at the next launch check */  \
            return (_e == cudaErrorMemoryAllocation) ? HF_ERR_OUT_OF_MEMORY : HF_ERR_CUDA;                \
        }                                                                                                 \
    } while (0)
namespace gb {
// CUDA events released when the scope ends (early error returns included)
template <int N>
struct ScopedEvents {
    cudaEvent_t ev[N] = {};
    ScopedEvents()
    {
        for (auto& x : ev) cudaEventCreate(&x);
    }
    ~ScopedEvents()
    {
        for (auto x : ev)
            if (x) cudaEventDestroy(x);
    }
    ScopedEvents(const ScopedEvents&) = delete;
    ScopedEvents& operator=(const ScopedEvents&) = delete;
};
}  // namespace gb
#define GB_LAUNCH_CHECK()                                                                                 \
    do {                                                                                                  \
        gb::count_launch();                                                                               \
        cudaError_t _e = cudaGetLastError();                                                              \
        if (_e != cudaSuccess) {                                                                          \
            gb::set_error(std::string("kernel launch: ") + cudaGetErrorString(_e));                       \
            return HF_ERR_CUDA;                                                                           \
        }                                                                                                 \
    } while (0)
#endif
