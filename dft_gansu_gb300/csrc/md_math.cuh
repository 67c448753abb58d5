// McMurchie-Davidson building blocks shared by every integral kernel.
//
// All routines are __host__ __device__ templates over the arithmetic type
// (double for the FP64 tier, float for the FP32 tier) and over the angular
// momenta, so that loops unroll at compile time and the Hermite tables live in
// registers.  Semantics follow the reference:
//   Boys F_n(x) = int_0^1 t^{2n} exp(-x t^2) dt            include/boys.hpp:148-182
//   Hermite E^{ij}_t, E^{00}_0 = exp(-ab/p X_AB^2)          include/Et_functions.hpp:3000
//   Hermite R^{n}_{tuv}, R^{n}_{000} = (-2 xi)^n F_n(T)     src/int2e.cu:1842-1893
//   Cartesian component order of a shell                    include/types.hpp:197-228
#pragma once
#include <cstdint>
#include <cmath>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace gb {

constexpr int kMaxL = 2;            // AO shells up to d (every configured basis)
constexpr int kMaxLTotal = 4 * kMaxL + 1;  // +1 order for derivative integrals
constexpr int kBoysOrders = 32;     // tabulated orders 0..31
constexpr int kBoysRows = kBoysOrders + 1;  // values per grid-point record: exp(-x_k), F_0 .. F_31
constexpr int kBoysTaylor = 6;      // Taylor terms around a grid point (FP64)
constexpr int kBoysTaylorF = 4;     // Taylor terms (FP32)
constexpr double kBoysStep = 1.0 / 32.0;
constexpr int kBoysPoints = 2049;   // grid x = 0 .. 64
constexpr double kBoysXMax = 64.0;  // asymptotic branch beyond this (FP64)
constexpr float kBoysXMaxF = 30.0f; // asymptotic branch beyond this (FP32)
// FP32 table: per order n < kBoysOrdersF and grid point k < kBoysGridF (x_k = k/32 <= 30)
// the four values F_n .. F_{n+3}(x_k) of one Taylor evaluation as one 16-byte
// vector, orders in separate slabs: an evaluation is one aligned load, and one
// kernel's order touches a 15 KB slab (cache-resident)
constexpr int kBoysGridF = 961;
constexpr int kBoysOrdersF = kBoysOrders - kBoysTaylorF + 1;
__host__ __device__ constexpr long long boys32_at(int n, int k)
{
    return (static_cast<long long>(n) * kBoysGridF + k) * kBoysTaylorF;
}
constexpr double kPi = 3.14159265358979323846;

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int nherm(int l) { return (l + 1) * (l + 2) * (l + 3) / 6; }

// Cartesian exponent of component i of a shell of angular momentum l along
// axis ax (0=x,1=y,2=z), in the reference order.
__host__ __device__ constexpr int cart_exp(int l, int i, int ax)
{
    // packed as x*100 + y*10 + z
    int pk = 0;
    switch (l) {
    case 0: pk = 0; break;
    case 1: pk = (i == 0) ? 100 : (i == 1) ? 10 : 1; break;
    case 2: {
        constexpr int t[6] = {200, 20, 2, 110, 101, 11};
        pk = t[i];
        break;
    }
    case 3: {
        constexpr int t[10] = {300, 30, 3, 120, 210, 201, 102, 12, 21, 111};
        pk = t[i];
        break;
    }
    default: {
        constexpr int t[15] = {400, 40, 4, 310, 301, 130, 31, 103, 13, 220, 202, 22, 211, 121, 112};
        pk = t[i];
        break;
    }
    }
    return ax == 0 ? pk / 100 : (ax == 1 ? (pk / 10) % 10 : pk % 10);
}

// (2n-1)!! with (-1)!! = 1
__host__ __device__ constexpr double dfact(int n) { return n <= 1 ? 1.0 : n * dfact(n - 2); }

// Component-dependent part of the reference primitive norm (calcNorm,
// include/int2e.hpp:127-130): 1/sqrt((2l-1)!!(2m-1)!!(2n-1)!!).
__host__ __device__ inline double component_factor(int l, int i)
{
    return 1.0 / sqrt(dfact(2 * cart_exp(l, i, 0) - 1) * dfact(2 * cart_exp(l, i, 1) - 1) *
                      dfact(2 * cart_exp(l, i, 2) - 1));
}

// ------------------------------------------------------------------ Boys
// Tabulated F_n(x_k), x_k = k/32, n < kBoysOrders, and exp(-x_k), one record of
// kBoysRows values per grid point (boys_at): the Taylor terms of one evaluation
// are consecutive in memory (one or two cache lines instead of one per term).  F_{nmax}(x) from a Taylor expansion
// about the nearest grid point (dF_n/dx = -F_{n+1}), then the stable downward
// recursion F_{n-1} = (2x F_n + e^{-x}) / (2n - 1), with
// e^{-x} = e^{-x_k} e^{x_k - x} and the second factor from its degree-6
// Taylor polynomial (|x_k - x| <= 1/64: error below 1e-16).  Beyond the grid:
// F_0 = sqrt(pi/x)/2 (erf(sqrt x) = 1 to the precision of the type) and the
// upward recursion F_{n+1} = ((2n+1) F_n - e^{-x}) / (2x), stable for large
// x; for x >= 64, e^{-x} is below 1e-27 and is dropped.
// record of grid point k: [0] = exp(-x_k), [n + 1] = F_n(x_k)
__host__ __device__ constexpr long long boys_at(int n, int k) { return static_cast<long long>(k) * kBoysRows + n + 1; }
__host__ __device__ constexpr long long boys_exp_at(int k) { return static_cast<long long>(k) * kBoysRows; }

template <int NMAX>
__host__ __device__ __forceinline__ void boys_fp64(double x, const double* __restrict__ table, double (&F)[NMAX + 1])
{
    if (x < kBoysXMax) {
        const int k = static_cast<int>(x * 32.0 + 0.5);
        const double dx = k * kBoysStep - x;  // expand at x_k: F(x) = sum F_{n+j}(x_k) dx^j / j!
        const double* t = table + boys_at(NMAX, k);
        double f = t[kBoysTaylor - 1];
#pragma unroll
        for (int j = kBoysTaylor - 1; j >= 1; --j) f = t[j - 1] + f * dx * (1.0 / j);
        F[NMAX] = f;
        if (NMAX > 0) {
            double e = 1.0 / 720.0;
            e = e * dx + 1.0 / 120.0;
            e = e * dx + 1.0 / 24.0;
            e = e * dx + 1.0 / 6.0;
            e = e * dx + 0.5;
            e = e * dx + 1.0;
            e = e * dx + 1.0;
            const double ex = table[boys_exp_at(k)] * e;
#pragma unroll
            for (int n = NMAX; n >= 1; --n) F[n - 1] = (2.0 * x * F[n] + ex) * (1.0 / (2 * n - 1));
        }
    } else {
#ifdef __CUDA_ARCH__
        const double r = rsqrt(x);
#else
        const double r = 1.0 / sqrt(x);
#endif
        const double rx = r * r;
        F[0] = 0.88622692545275801365 * r;  // sqrt(pi)/2
#pragma unroll
        for (int n = 0; n < NMAX; ++n) F[n + 1] = (n + 0.5) * F[n] * rx;
    }
}

template <int NMAX>
__host__ __device__ __forceinline__ void boys_fp32(float x, const float* __restrict__ table, float (&F)[NMAX + 1])
{
    if (x < kBoysXMaxF) {
        const int k = static_cast<int>(x * 32.0f + 0.5f);
        const float dx = k * static_cast<float>(kBoysStep) - x;
        static_assert(kBoysTaylorF == 4, "one float4 per FP32 Boys evaluation");
#ifdef __CUDA_ARCH__
        const float4 q = __ldg(reinterpret_cast<const float4*>(table + boys32_at(NMAX, k)));
        const float t[4] = {q.x, q.y, q.z, q.w};
#else
        const float* t = table + boys32_at(NMAX, k);
#endif
        float f = t[kBoysTaylorF - 1];
#pragma unroll
        for (int j = kBoysTaylorF - 1; j >= 1; --j) f = t[j - 1] + f * dx * (1.0f / j);
        F[NMAX] = f;
        if (NMAX > 0) {
#ifdef __CUDA_ARCH__
            const float ex = __expf(-x);
#else
            const float ex = expf(-x);
#endif
#pragma unroll
            for (int n = NMAX; n >= 1; --n) F[n - 1] = (2.0f * x * F[n] + ex) * (1.0f / (2 * n - 1));
        }
    } else {
        const float rx = 1.0f / x;
#ifdef __CUDA_ARCH__
        const float ex = (NMAX > 0) ? __expf(-x) : 0.0f;
#else
        const float ex = (NMAX > 0) ? expf(-x) : 0.0f;
#endif
        F[0] = 0.5f * sqrtf(static_cast<float>(kPi) * rx);
#pragma unroll
        for (int n = 0; n < NMAX; ++n) F[n + 1] = ((n + 0.5f) * F[n] - 0.5f * ex) * rx;
    }
}

template <class T>
struct BoysEval;
template <>
struct BoysEval<double> {
    template <int N>
    __host__ __device__ __forceinline__ static void run(double x, const double* t, double (&F)[N + 1]) { boys_fp64<N>(x, t, F); }
};
template <>
struct BoysEval<float> {
    template <int N>
    __host__ __device__ __forceinline__ static void run(float x, const float* t, float (&F)[N + 1]) { boys_fp32<N>(x, t, F); }
};

// ------------------------------------------------------- Hermite E (1D)
// E[i][j][t] for i<=LA, j<=LB, t<=i+j, with E^{00}_0 = 1 (the Gaussian
// product exponential is carried by the primitive-pair prefactor).
template <class T, int LA, int LB>
struct HermiteE {
    T e[LA + 1][LB + 1][LA + LB + 1];
    __host__ __device__ __forceinline__ void build(T xpa, T xpb, T oo2p)
    {
        e[0][0][0] = T(1);
#pragma unroll
        for (int i = 0; i <= LA; ++i) {
#pragma unroll
            for (int j = 0; j <= LB; ++j) {
                if (i == 0 && j == 0) continue;
#pragma unroll
                for (int t = 0; t <= i + j; ++t) {
                    T v;
                    if (i > 0) {
                        v = (t <= i - 1 + j) ? xpa * e[i - 1][j][t] : T(0);
                        if (t > 0) v += oo2p * e[i - 1][j][t - 1];
                        if (t + 1 <= i - 1 + j) v += T(t + 1) * e[i - 1][j][t + 1];
                    } else {
                        v = (t <= j - 1) ? xpb * e[0][j - 1][t] : T(0);
                        if (t > 0) v += oo2p * e[0][j - 1][t - 1];
                        if (t + 1 <= j - 1) v += T(t + 1) * e[0][j - 1][t + 1];
                    }
                    e[i][j][t] = v;
                }
            }
        }
    }
};

// ------------------------------------------------------- Hermite R (3D)
// Packed position of the Hermite index (t, u, v): levels k = t + u + v in
// ascending order, within a level by descending t, then descending u.
__host__ __device__ constexpr int hermite_index(int t, int u, int v)
{
    return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

// R(t, u, v) = R^{0}_{tuv} for t+u+v <= L, given Fs[n] = R^{n}_{000}, in packed
// storage (nherm(L) values, so that fully unrolled kernels keep the table in
// registers).  In-place evaluation: pass n overwrites levels k = L-n .. 1 in
// descending order, which only reads R^{n+1} values of lower levels not yet
// overwritten in the pass.
template <class T, int L>
struct HermiteR {
    T r[nherm(L)];
    __host__ __device__ __forceinline__ T& operator()(int t, int u, int v) { return r[hermite_index(t, u, v)]; }
    __host__ __device__ __forceinline__ const T& operator()(int t, int u, int v) const
    {
        return r[hermite_index(t, u, v)];
    }
    __host__ __device__ __forceinline__ void build(const T (&Fs)[L + 1], T X, T Y, T Z)
    {
        HermiteR& R = *this;
        R(0, 0, 0) = Fs[L];
#pragma unroll
        for (int n = L - 1; n >= 0; --n) {
#pragma unroll
            for (int k = L - n; k >= 1; --k) {
#pragma unroll
                for (int t = k; t >= 0; --t) {
#pragma unroll
                    for (int u = k - t; u >= 0; --u) {
                        const int v = k - t - u;
                        T val;
                        if (t > 0) {
                            val = X * R(t - 1, u, v);
                            if (t > 1) val += T(t - 1) * R(t - 2, u, v);
                        } else if (u > 0) {
                            val = Y * R(0, u - 1, v);
                            if (u > 1) val += T(u - 1) * R(0, u - 2, v);
                        } else {
                            val = Z * R(0, 0, v - 1);
                            if (v > 1) val += T(v - 1) * R(0, 0, v - 2);
                        }
                        R(t, u, v) = val;
                    }
                }
            }
            R(0, 0, 0) = Fs[n];
        }
    }
};

}  // namespace gb
