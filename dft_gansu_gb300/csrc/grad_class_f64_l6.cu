// FP64 class kernels of the analytic gradient for la + lb + lc + ld = 6:
// (dp|dp), (dd|pp), (dd|ds).  They spill several KB, like the L = 5 classes that
// beat the generic kernel; a translation unit of their own so that they compile
// in parallel with the rest.
#include "grad_kernel.cuh"

namespace gb {

bool launch_grad_class_f64_l6(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem,
                              cudaStream_t s)
{
#define GB_GC(a, b, c, d)                                                                       \
    if (la == a && lb == b && lc == c && ld == d) {                                             \
        grad_class_kernel<double, a, b, c, d><<<grid, kGradThreads, smem, s>>>(G);              \
        return true;                                                                            \
    }
    GB_GC(2, 1, 2, 1) GB_GC(2, 2, 1, 1) GB_GC(2, 2, 2, 0)
#undef GB_GC
    return false;
}

}  // namespace gb
