// One quartet class of the direct Fock build, selected at compile time.
// The build compiles this file once per class (GB_LA, GB_LB, GB_LC, GB_LD)
// so that the classes compile in parallel; each object exports
// launch_fock_<la>_<lb>_<lc>_<ld> and launch_eri_<la>_<lb>_<lc>_<ld>.
#include "fock_column.cuh"

#if !defined(GB_LA) || !defined(GB_LB) || !defined(GB_LC) || !defined(GB_LD)
#error "fock_inst.cu needs GB_LA, GB_LB, GB_LC and GB_LD"
#endif

#define GB_CAT2(a, b) a##b
#define GB_CAT(a, b) GB_CAT2(a, b)
#define GB_SUFFIX GB_CAT(GB_CAT(GB_CAT(GB_CAT(_, GB_LA), GB_CAT(_, GB_LB)), GB_CAT(_, GB_LC)), GB_CAT(_, GB_LD))

namespace gb {

constexpr int kNCD = ncart(GB_LC) * ncart(GB_LD);

// grid: blocks for one thread per quartet; the generic path needs kNCD times more
void GB_CAT(launch_fock, GB_SUFFIX)(bool fp32, const FockClassLaunch& launch, int grid, cudaStream_t stream)
{
    // classes above the register budget: one thread per ket component pair, compile-time tables
    using fock_column::ClassColumn;
    using fock_column::column_kernel;
    if (fp32) {
        if constexpr (FockSplit<float, GB_LA, GB_LB, GB_LC, GB_LD>::value == 1)
            fock_direct_kernel<float, GB_LA, GB_LB, GB_LC, GB_LD><<<grid, kFockThreads, 0, stream>>>(launch);
        else
            column_kernel<float, ClassColumn<float, GB_LA, GB_LB, GB_LC, GB_LD>>
                <<<grid * kNCD, kFockThreads, 0, stream>>>(launch, kNCD);
    } else {
        if constexpr (FockSplit<double, GB_LA, GB_LB, GB_LC, GB_LD>::value == 1)
            fock_direct_kernel<double, GB_LA, GB_LB, GB_LC, GB_LD><<<grid, kFockThreads, 0, stream>>>(launch);
        else
            column_kernel<double, ClassColumn<double, GB_LA, GB_LB, GB_LC, GB_LD>>
                <<<grid * kNCD, kFockThreads, 0, stream>>>(launch, kNCD);
    }
}

void GB_CAT(launch_eri, GB_SUFFIX)(const FockClassLaunch& launch, const double* scale, double* eri, int grid,
                                  cudaStream_t stream)
{
    launch_eri_generic(launch, kNCD, scale, eri, grid * kNCD, stream);
}

}  // namespace gb
