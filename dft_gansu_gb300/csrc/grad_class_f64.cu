// FP64 class kernels of the analytic gradient with compile-time loops:
// la + lb + lc + ld <= 4 (the L = 5 classes in grad_class_f64_l5.cu; the larger
// FP64 classes run the generic kernel of grad.cu).
#include "grad_kernel.cuh"

namespace gb {

bool launch_grad_class_f64(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem, cudaStream_t s)
{
#define GB_GC(a, b, c, d)                                                                       \
    if (la == a && lb == b && lc == c && ld == d) {                                             \
        grad_class_kernel<double, a, b, c, d><<<grid, kGradThreads, smem, s>>>(G);              \
        return true;                                                                            \
    }
    GB_GC(0, 0, 0, 0) GB_GC(1, 0, 0, 0) GB_GC(1, 0, 1, 0) GB_GC(1, 1, 0, 0) GB_GC(1, 1, 1, 0) GB_GC(1, 1, 1, 1)
    GB_GC(2, 0, 0, 0) GB_GC(2, 0, 1, 0) GB_GC(2, 0, 1, 1) GB_GC(2, 0, 2, 0) GB_GC(2, 1, 0, 0) GB_GC(2, 1, 1, 0)
    GB_GC(2, 2, 0, 0) GB_GC(2, 1, 1, 1) GB_GC(2, 1, 2, 0) GB_GC(2, 2, 1, 0)
#undef GB_GC
    return false;
}

}  // namespace gb
