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
// reuse the cached pointer.
//
// Limits and sharing: at most kNoAllocMaxPrev (16) stored error/Fock pairs.
// All calls share the one scratch array and every call rewrites the parts it
// reads, so nothing carries over between calls; calls that overlap on the GPU
// (different streams or threads without ordering) race on the scratch and
// must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

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

// bordered system [B -1; -1 0] c = [0 .. 0 -1] by Gaussian elimination with
// partial pivoting in FP64 (one thread); coefficients to scratch[kNoAllocB ..]
__global__ void noalloc_solve_kernel(int m, double* __restrict__ scratch)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n = m + 1;
    double A[kNoAllocMaxPrev + 1][kNoAllocMaxPrev + 2];
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            if (i < m && j < m) A[i][j] = scratch[i * kNoAllocMaxPrev + j];
            else if (i == m && j == m) A[i][j] = 0.0;
            else A[i][j] = -1.0;
        }
        A[i][n] = (i == m) ? -1.0 : 0.0;
    }
    int singular = 0;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        if (A[piv][c] == 0.0) { singular = 1; continue; }
        if (piv != c)
            for (int k = 0; k <= n; ++k) { const double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
        for (int r = c + 1; r < n; ++r) {
            const double f = A[r][c] / A[c][c];
            for (int k = c; k <= n; ++k) A[r][k] -= f * A[c][k];
        }
    }
    double x[kNoAllocMaxPrev + 1];
    for (int r = n - 1; r >= 0; --r) {
        double s = A[r][n];
        for (int k = r + 1; k < n; ++k) s -= A[r][k] * x[k];
        x[r] = (A[r][r] != 0.0) ? s / A[r][r] : 0.0;
    }
    for (int i = 0; i < m; ++i) scratch[kNoAllocB + i] = x[i];
    scratch[kNoAllocB + kNoAllocMaxPrev] = singular;
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

// device address of the scratch array for the current device (looked up once)
int noalloc_scratch(double** out)
{
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error("device ordinal out of range"), HF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_error(std::string("cudaGetSymbolAddress of the DIIS scratch: ") + cudaGetErrorString(e));
            return HF_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<double*>(p);
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
