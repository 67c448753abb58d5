// FP32 class kernels of the analytic gradient with compile-time loops:
// la + lb + lc + ld <= 4 (L = 5, 6 in grad_class_f32_l56.cu).
#include "grad_kernel.cuh"

namespace gb {

bool launch_grad_class_f32(int la, int lb, int lc, int ld, const GradLaunch& G, int grid, size_t smem, cudaStream_t s)
{
#define GB_GC(a, b, c, d)                                                                       \
    if (la == a && lb == b && lc == c && ld == d) {                                             \
        grad_class_kernel<float, a, b, c, d><<<grid, kGradThreads, smem, s>>>(G);               \
        return true;                                                                            \
    }
    GB_GC(0, 0, 0, 0) GB_GC(1, 0, 0, 0) GB_GC(1, 0, 1, 0) GB_GC(1, 1, 0, 0) GB_GC(1, 1, 1, 0) GB_GC(1, 1, 1, 1)
    GB_GC(2, 0, 0, 0) GB_GC(2, 0, 1, 0) GB_GC(2, 0, 1, 1) GB_GC(2, 0, 2, 0) GB_GC(2, 1, 0, 0) GB_GC(2, 1, 1, 0)
    GB_GC(2, 2, 0, 0)
#undef GB_GC
    return launch_grad_class_f32_l56(la, lb, lc, ld, G, grid, smem, s);
}

}  // namespace gb
