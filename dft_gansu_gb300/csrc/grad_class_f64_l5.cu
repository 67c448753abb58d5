// FP64 class kernels of the analytic gradient for la + lb + lc + ld = 5:
// (dp|pp), (dp|ds), (dd|ps).  They spill but still beat the generic kernel
// (measured: FP64 decane cc-pVDZ gradient 634 -> 598 ms); a translation unit of
// their own so that they compile in parallel with the rest.
#include "grad_kernel.cuh"

namespace gb {

bool launch_grad_class_f64_l5(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem,
                              cudaStream_t s)
{
#define GB_GC(a, b, c, d)                                                                       \
    if (la == a && lb == b && lc == c && ld == d) {                                             \
        grad_class_kernel<double, a, b, c, d><<<grid, kGradThreads, smem, s>>>(G);              \
        return true;                                                                            \
    }
    GB_GC(2, 1, 1, 1) GB_GC(2, 1, 2, 0) GB_GC(2, 2, 1, 0)
#undef GB_GC
    return launch_grad_class_f64_l6(la, lb, lc, ld, G, grid, smem, s);
}

}  // namespace gb
