/*
 * CPU shim for compiling the reference's own CUDA integral kernels with g++.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is force-included (-include) when the
 * recipe in oracle/refcpu/Makefile compiles the reference's src/int2e.cu and
 * src/int1e.cu as plain C++ so that their __global__ functions can be called
 * one "thread" at a time on the CPU.  The resulting library (oracle/_ref/) is a
 * checker for the oracle; the product never loads it.
 *
 * Everything here is this project's own code: CUDA qualifiers become no-ops
 * (__constant__ becomes `static` so header-defined tables get one copy per
 * translation unit), the thread coordinates become thread_local variables that
 * the driver sets before each call, and the device intrinsics the reference
 * uses are mapped to their IEEE double meaning.
 */
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <algorithm>

#define __global__
#define __device__
#define __host__
#define __constant__ static
#define __forceinline__ inline
#define __restrict__
#define __shared__ static

struct RefcpuDim3 { unsigned int x, y, z; };
extern thread_local RefcpuDim3 threadIdx;
extern thread_local RefcpuDim3 blockIdx;
extern thread_local RefcpuDim3 blockDim;
extern thread_local RefcpuDim3 gridDim;

inline double __drcp_rn(double x) { return 1.0 / x; }
inline double __dsqrt_rn(double x) { return std::sqrt(x); }
inline unsigned int __double2uint_rd(double x) { return static_cast<unsigned int>(std::floor(x)); }
inline int __double2int_rd(double x) { return static_cast<int>(std::floor(x)); }
inline int __double2int_ru(double x) { return static_cast<int>(std::ceil(x)); }
inline long long __double2ll_rd(double x) { return static_cast<long long>(std::floor(x)); }
inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }

/* The driver runs "threads" in parallel with OpenMP, so accumulation is atomic. */
inline double atomicAdd(double* address, double value)
{
    double old;
#pragma omp atomic capture
    { old = *address; *address += value; }
    return old;
}

inline void __syncthreads() {}

struct double3 { double x, y, z; };
inline double3 make_double3(double x, double y, double z) { return double3{x, y, z}; }
