// Instantiates the RI derivative kernel (ri_grad_kernel.cuh) for one auxiliary
// angular momentum GB_RI_LP and every bra class: the AO pair classes (s, p, d)
// of the three-centre term and the (P, unit) classes (s .. f) of the metric
// term.  Compiled once per GB_RI_LP so the four units build in parallel.
#define GB_RI_GRAD_KERNELS
#include "ri_grad_kernel.cuh"

#ifndef GB_RI_LP
#error "GB_RI_LP (auxiliary angular momentum 0..3) must be defined"
#endif

namespace gb {

template <>
RiDerivLaunch ri_deriv_launcher<GB_RI_LP>(int la, int lb)
{
#define GB_RD(A, B) \
    if (la == A && lb == B) return ri_deriv_launch<A, B, GB_RI_LP>;
    GB_RD(0, 0) GB_RD(1, 0) GB_RD(1, 1) GB_RD(2, 0) GB_RD(2, 1) GB_RD(2, 2) GB_RD(3, 0)
#undef GB_RD
    return nullptr;
}

}  // namespace gb
