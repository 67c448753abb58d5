// FP32 class kernels of the analytic gradient for la + lb + lc + ld = 5, 6: FP32
// tables take half the registers of FP64, so these classes stay within 1-2 KB of
// spills and run well ahead of the generic kernel.
#include "grad_kernel.cuh"

namespace gb {

bool launch_grad_class_f32_l56(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem,
                               cudaStream_t s)
{
#define GB_GC(a, b, c, d)                                                                       \
    if (la == a && lb == b && lc == c && ld == d) {                                             \
        grad_class_kernel<float, a, b, c, d><<<grid, kGradThreads, smem, s>>>(G);               \
        return true;                                                                            \
    }
    GB_GC(2, 1, 1, 1) GB_GC(2, 1, 2, 0) GB_GC(2, 2, 1, 0) GB_GC(2, 1, 2, 1) GB_GC(2, 2, 1, 1) GB_GC(2, 2, 2, 0)
#undef GB_GC
    return false;
}

}  // namespace gb
