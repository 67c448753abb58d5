// DIIS extrapolation that allocates nothing.
//
// Who needs this: callers that must not (or cannot) allocate device memory
// while they run an SCF step -- code recording a CUDA graph of the iteration,
// an application that hands all device memory to its own pool allocator, or a
// host thread that is not allowed to synchronise the device (cudaMalloc and
// cudaFree can synchronise).  hf_compute_fock_diis needs an engine, and
// creating one allocates; this variant needs only the caller's matrices.
//
// Its small scratch (the DIIS B matrix, the coefficients and a status word)
// lives in g_noalloc_scratch below: a file-scope __device__ array that every
// GPU loading this library holds until the process exits.  Host code cannot
// use the array's name as a device address, so the first call on each device
// looks the address up once with cudaGetSymbolAddress while that device is
// current (make that first call before any stream capture), and later calls
// reuse the cached pointer.  The cache is keyed on the device's current CUDA
// context as well: after cudaDeviceReset (a new primary context) the next
// call looks the address up again, and that call too belongs before any
// stream capture.
//
// Repeated error vectors: the weights come from diis_coefficients
// (diis_solve.cuh), which gives weight 0 to an error vector that repeats
// others (two equal vectors count once: the case in which the bordered
// system is singular) and returns the constrained minimiser over the rest;
// the number left out is written to the status word of the scratch.  The
// output is therefore always a finite extrapolation, never the zero matrix.
//
// Limits and sharing: at most kNoAllocMaxPrev (16) stored error/Fock pairs.
// All calls share the one scratch array and every call rewrites the parts it
// reads, so nothing carries over between calls; calls that overlap on the GPU
// (different streams or threads without ordering) race on the scratch and
// must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "diis_solve.cuh"
#include "internal.hpp"

namespace gb {
namespace {

constexpr int kNoAllocMaxPrev = 16;
constexpr int kNoAllocB = kNoAllocMaxPrev * kNoAllocMaxPrev;   // B matrix
constexpr int kNoAllocDoubles = kNoAllocB + kNoAllocMaxPrev + 8;  // + coefficients + status
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};
CUcontext g_noalloc_ctx[kNoAllocMaxDevices] = {};

// B_ij = <e_i, e_j> for i <= j < m, one block per pair; writes every B entry
// the solve reads, so the scratch needs no clearing between calls.
__global__ void noalloc_dots_kernel(const double* __restrict__ Es, int m, long long nn, double* __restrict__ scratch)
{
    __shared__ double red[32];
    int p = blockIdx.x, i = 0;
    while (p >= m - i) { p -= m - i; ++i; }
    const int j = i + p;
    const double* a = Es + i * nn;
    const double* b = Es + j * nn;
    double s = 0.0;
    for (long long k = threadIdx.x; k < nn; k += blockDim.x) s += a[k] * b[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) {
            scratch[i * kNoAllocMaxPrev + j] = s;
            scratch[j * kNoAllocMaxPrev + i] = s;
        }
    }
}

// weights of the independent error vectors (diis_solve.cuh) to scratch[kNoAllocB ..];
// the count of vectors left out as dependent goes to the status word
__global__ void noalloc_solve_kernel(int m, double* __restrict__ scratch)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int dropped = diis_coefficients<kNoAllocMaxPrev>(scratch, kNoAllocMaxPrev, m, scratch + kNoAllocB);
    scratch[kNoAllocB + kNoAllocMaxPrev] = static_cast<double>(dropped);
}

__global__ void noalloc_combine_kernel(const double* __restrict__ Fs, int m, long long nn,
                                       const double* __restrict__ scratch, double* __restrict__ F)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < nn;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < m; ++i) s += scratch[kNoAllocB + i] * Fs[i * nn + k];
        F[k] = s;
    }
}

// the current CUDA context (cuCtxGetCurrent through the runtime's driver entry point)
CUcontext current_context()
{
    using Fn = CUresult (*)(CUcontext*);
    static Fn fn = nullptr;
    static bool looked = false;
    if (!looked) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<Fn>(p);
        looked = true;
    }
    CUcontext c = nullptr;
    if (fn) fn(&c);
    return c;
}

// device address of the scratch array for the current device and context
// (looked up once per device, again after the device's context changed)
int noalloc_scratch(double** out)
{
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error("device ordinal out of range"), HF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    const CUcontext ctx = current_context();  // null before the runtime made a context current
    if (!ctx || !g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != ctx) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_error(std::string("cudaGetSymbolAddress of the DIIS scratch: ") + cudaGetErrorString(e));
            return HF_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<double*>(p);
        g_noalloc_ctx[dev] = current_context();
    }
    *out = g_noalloc_ptr[dev];
    return HF_OK;
}

}  // namespace
}  // namespace gb

extern "C" int hf_compute_fock_diis_noalloc(const double* d_errors, const double* d_focks, double* d_new_fock,
                                            int num_prev, int num_basis, void* stream)
{
    gb::clear_error();
    if (!d_errors || !d_focks || !d_new_fock || num_basis <= 0)
        return gb::set_error("hf_compute_fock_diis_noalloc: null pointer or non-positive num_basis"),
               HF_ERR_INVALID_ARGUMENT;
    if (num_prev < 2 || num_prev > gb::kNoAllocMaxPrev)
        return gb::set_error("hf_compute_fock_diis_noalloc: num_prev must be between 2 and 16 (the size of its "
                             "static scratch)"),
               HF_ERR_INVALID_ARGUMENT;
    double* scratch = nullptr;
    int st = gb::noalloc_scratch(&scratch);
    if (st) return st;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long nn = static_cast<long long>(num_basis) * num_basis;
    gb::noalloc_dots_kernel<<<num_prev * (num_prev + 1) / 2, 512, 0, s>>>(d_errors, num_prev, nn, scratch);
    GB_LAUNCH_CHECK();
    gb::noalloc_solve_kernel<<<1, 32, 0, s>>>(num_prev, scratch);
    GB_LAUNCH_CHECK();
    const int grid = static_cast<int>(std::min<long long>((nn + 255) / 256, 8192));
    gb::noalloc_combine_kernel<<<grid, 256, 0, s>>>(d_focks, num_prev, nn, scratch, d_new_fock);
    GB_LAUNCH_CHECK();
    return HF_OK;
}
