// RHF density by purification in one cooperative launch (N <= 512).
//
// The reference gets the density from a diagonalisation of F' = X^T F X every
// iteration (computeCoefficientMatrix, src/gpu_manager.cu:529-599, then
// computeDensityMatrix_RHF_kernel, src/gpu_kernels.cu:54-69).  Purification
// gives the same aufbau density whenever the HOMO-LUMO gap is open:
//   F' = X^T F X                              FP64
//   P0 = (hi I - F') / (hi - lo)              Gershgorin interval [lo, hi]
//   SP2 steps P <- P^2 or 2P - P^2            FP32 (trace nearest nocc)
//   McWeeny P <- 3P^2 - 2P^3                  FP64, once or twice
//   D = 2 X P X^T                             FP64
// At N = 194 every one of these products is a few MFLOP: as library calls each
// one runs on a handful of SMs, and GB300 executes FP64 at 2 FMA per clock per
// SM, so a 194^3 DGEMM needs the whole chip to finish in ~12 us.  Here one
// persistent grid (one CTA per SM, co-resident by cooperative launch) runs the
// whole sequence; every product is spread over all CTAs in 16 x 16 output
// tiles (symmetric products: upper tiles only, mirrored), and the phases are
// separated by a grid barrier of this file (bounded wait: a CTA that waits
// longer than 2 s records the failure and returns).
//
// SP2 needs tr(P) and tr(P^2) to choose its step before P^2 exists: with P
// symmetric, tr(P^2) = |P|_F^2, so every CTA writes tr and |.|_F^2 partial sums
// of the tiles it produced, and after the barrier every CTA adds them up in the
// same fixed order (the same decision everywhere, reproducible).  Stop:
// e_k = |tr(P) - |P|_F^2| = sum lambda (1 - lambda) stops shrinking over two
// steps once below 1e-2 (the FP32 rounding floor), or falls below 1e-9 N;
// at most kPurifyMaxSteps steps (or the caller's smaller limit).
//
// The result is checked: after McWeeny |tr(P) - nocc| and |tr(P) - |P|_F^2|
// go to the status words that the SCF reads back with the energy.  A small or
// closed gap leaves eigenvalues of P between 0 and 1 (McWeeny keeps 1/2 at
// 1/2), which these checks catch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "engine.hpp"
#include "purify.hpp"

namespace gb {
namespace {

constexpr int kPT = 16;  // output tile edge
constexpr int kPurifyThreads = kPT * kPT;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;

struct PurifyArgs {
    int n, nocc, nt, nup, kpad, ldp, max_steps;  // ldp: row stride of the FP32 projectors
    const double* X;
    const double* F;
    double* T1;
    double* T2;
    double* W;
    double* D;
    float* Pa;
    float* Pb;
    double* part;     // [2][nup][2]: tr and |.|_F^2 partial sums per upper tile (double-buffered)
    double* rowpart;  // [n][nt]: Gershgorin row sums of |F'_ij|, j != i, per tile column
    double* status;   // kPurifyStatusWords
    unsigned* bar;    // grid barrier: arrivals, generation
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier over all CTAs of the launch (co-resident by cooperative launch).
// The arrival counter only grows: barrier number `epoch` is complete when
// gridDim.x * epoch CTAs have arrived.  Returns false when the wait ran out.
__device__ bool grid_barrier(const PurifyArgs& a, unsigned& epoch)
{
    __shared__ int ok;
    __syncthreads();
    ++epoch;
    if (threadIdx.x == 0) {
        ok = 1;
        __threadfence();
        const unsigned target = gridDim.x * epoch;
        if (atomicAdd(&a.bar[0], 1u) + 1u == target) {
            st_release(&a.bar[1], epoch);
        } else {
            const unsigned long long t0 = global_ns();
            while (ld_acquire(&a.bar[1]) < epoch) {
                if (global_ns() - t0 > kBarrierTimeoutNs) {
                    a.status[kPurifyStatusFlags] = 1.0;  // barrier wait ran out
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// CTA 0 records when it finished phase `slot` (microseconds from t0)
__device__ __forceinline__ void mark_phase(const PurifyArgs& a, unsigned long long t0, int slot)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) a.status[kPurifyStatusPhase + slot] = (global_ns() - t0) * 1e-3;
}

__device__ __forceinline__ void upper_tile(int u, int nt, int& I, int& J)
{
    I = 0;
    while (u >= nt - I) {
        u -= nt - I;
        ++I;
    }
    J = I + u;
}

template <int V, bool CG, class TI>
__device__ __forceinline__ void load_vec(const TI* __restrict__ p, TI (&v)[V])
{
    if constexpr (V == 1) {
        v[0] = CG ? __ldcg(p) : __ldg(p);
    } else if constexpr (sizeof(TI) == 4) {
        const float4* q = reinterpret_cast<const float4*>(p);
        const float4 x = CG ? __ldcg(q) : __ldg(q);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else {
        const double2* q = reinterpret_cast<const double2*>(p);
        const double2 x = CG ? __ldcg(q) : __ldg(q);
        v[0] = x.x; v[1] = x.y;
    }
}

// rows base .. base + 15 of M (row stride ld, vectors of V elements: 16-byte aligned
// rows and ld >= n rounded up to V) into sm[r][k]; kU loads in flight per thread
template <int V, bool CG, class TI, class TO>
__device__ __forceinline__ void load_rows(const TI* __restrict__ M, int n, int ld, int base, TO* __restrict__ sm,
                                          int kpad)
{
    constexpr int kU = 4;
    const int nv = (n + V - 1) / V;
    const int total = kPT * nv;
    for (int i0 = threadIdx.x; i0 < total; i0 += kU * kPurifyThreads) {
        TI v[kU][V];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int idx = i0 + u * kPurifyThreads;
            const int r = idx / nv, c = idx - r * nv;
            if (idx < total && base + r < n) {
                load_vec<V, CG>(M + static_cast<long long>(base + r) * ld + c * V, v[u]);
            } else {
#pragma unroll
                for (int e = 0; e < V; ++e) v[u][e] = TI(0);
            }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int idx = i0 + u * kPurifyThreads;
            if (idx < total) {
                const int r = idx / nv, c = idx - r * nv;
#pragma unroll
                for (int e = 0; e < V; ++e) sm[r * kpad + c * V + e] = static_cast<TO>(v[u][e]);
            }
        }
    }
}

// panel[r][k] (r < 16, k < n) of rows (COLS = false: M[(base + r) ld + k]) or
// columns (COLS = true: M[k ld + base + r]); out-of-range rows are zero.  CG: the
// matrix was written inside this launch, read past L1.  Rows move as 16-byte
// vectors where the row stride allows it; several loads are in flight per thread.
template <bool COLS, bool CG, class TI, class TO>
__device__ void load_panel(const TI* __restrict__ M, int n, int ld, int base, TO* __restrict__ sm, int kpad)
{
    if (COLS) {
        constexpr int kU = 4;
        const int total = kPT * n;
        for (int i0 = threadIdx.x; i0 < total; i0 += kU * kPurifyThreads) {
            TI v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int idx = i0 + u * kPurifyThreads;
                const int k = idx / kPT, r = idx - k * kPT;
                v[u] = (idx < total && base + r < n)
                           ? (CG ? __ldcg(M + static_cast<long long>(k) * ld + base + r)
                                 : __ldg(M + static_cast<long long>(k) * ld + base + r))
                           : TI(0);
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int idx = i0 + u * kPurifyThreads;
                if (idx < total) sm[(idx % kPT) * kpad + idx / kPT] = static_cast<TO>(v[u]);
            }
        }
    } else if constexpr (sizeof(TI) == 4) {
        if (ld % 4 == 0) load_rows<4, CG>(M, n, ld, base, sm, kpad);
        else load_rows<1, CG>(M, n, ld, base, sm, kpad);
    } else {
        if (ld % 2 == 0) load_rows<2, CG>(M, n, ld, base, sm, kpad);
        else load_rows<1, CG>(M, n, ld, base, sm, kpad);
    }
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }

template <class T>
__device__ __forceinline__ T tile_dot(const T* __restrict__ sa, const T* __restrict__ sb, int n)
{
    T c0 = T(0), c1 = T(0), c2 = T(0), c3 = T(0);
    int k = 0;
    for (; k + 3 < n; k += 4) {
        c0 = fma_t(sa[k], sb[k], c0);
        c1 = fma_t(sa[k + 1], sb[k + 1], c1);
        c2 = fma_t(sa[k + 2], sb[k + 2], c2);
        c3 = fma_t(sa[k + 3], sb[k + 3], c3);
    }
    for (; k < n; ++k) c0 = fma_t(sa[k], sb[k], c0);
    return (c0 + c1) + (c2 + c3);
}

// block sum of two values to thread 0 (fixed order)
__device__ void block_sum2(double& x, double& y)
{
    __shared__ double rx[kPurifyThreads / 32], ry[kPurifyThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if ((threadIdx.x & 31) == 0) { rx[threadIdx.x >> 5] = x; ry[threadIdx.x >> 5] = y; }
    __syncthreads();
    if (threadIdx.x == 0) {
        x = 0.0;
        y = 0.0;
        for (int w = 0; w < kPurifyThreads / 32; ++w) { x += rx[w]; y += ry[w]; }
    }
    __syncthreads();
}

// sums of the per-tile partials (tr, |.|_F^2) of buffer `slot`, same order in every CTA
__device__ void tile_totals(const PurifyArgs& a, int slot, double& tr, double& fro)
{
    __shared__ double st[2];
    if (threadIdx.x < 32) {
        double x = 0.0, y = 0.0;
        const double* p = a.part + static_cast<long long>(slot) * a.nup * 2;
        for (int u = threadIdx.x; u < a.nup; u += 32) {
            x += __ldcg(p + 2 * u);
            y += __ldcg(p + 2 * u + 1);
        }
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_xor_sync(0xffffffffu, x, o);
            y += __shfl_xor_sync(0xffffffffu, y, o);
        }
        if (threadIdx.x == 0) { st[0] = x; st[1] = y; }
    }
    __syncthreads();
    tr = st[0];
    fro = st[1];
    __syncthreads();
}

// tr and |.|_F^2 partials of the tile value v at (i, j) of upper tile (I, J), to part[slot][u]
__device__ void tile_partials(const PurifyArgs& a, int slot, int u, bool diag_tile, int i, int j, double v)
{
    double t = 0.0, f = 0.0;
    if (i < a.n && j < a.n) {
        if (diag_tile && i == j) t = v;
        f = (diag_tile ? 1.0 : 2.0) * v * v;
    }
    block_sum2(t, f);
    if (threadIdx.x == 0) {
        double* p = a.part + (static_cast<long long>(slot) * a.nup + u) * 2;
        p[0] = t;
        p[1] = f;
    }
}

template <class T>
__device__ __forceinline__ void store_sym(T* __restrict__ M, int n, int ld, int i, int j, T v)
{
    if (i < n && j < n) {
        M[static_cast<long long>(i) * ld + j] = v;
        M[static_cast<long long>(j) * ld + i] = v;
    }
}

__global__ void __launch_bounds__(kPurifyThreads, 1) purify_kernel(PurifyArgs a)
{
    extern __shared__ double smem[];
    double* sa = smem;
    double* sb = smem + kPT * a.kpad;
    float* fa = reinterpret_cast<float*>(smem);
    float* fb = fa + kPT * a.kpad;
    const int ty = threadIdx.x / kPT, tx = threadIdx.x % kPT;
    const int n = a.n, nt = a.nt;
    unsigned epoch = 0;
    const unsigned long long t_start = global_ns();

    // 1. T1 = X^T F (all tiles)
    for (int t = blockIdx.x; t < nt * nt; t += gridDim.x) {
        const int I = t / nt, J = t % nt;
        __syncthreads();
        load_panel<true, false>(a.X, n, n, I * kPT, sa, a.kpad);   // rows of X^T = columns of X
        load_panel<false, false>(a.F, n, n, J * kPT, sb, a.kpad);  // F symmetric: columns = rows
        __syncthreads();
        const int i = I * kPT + ty, j = J * kPT + tx;
        const double v = tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n);
        if (i < n && j < n) a.T1[static_cast<long long>(i) * n + j] = v;
    }
    if (!grid_barrier(a, epoch)) return;

    // 2. F' = T1 X (upper tiles, mirrored) into T2, Gershgorin partial row sums
    for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
        int I, J;
        upper_tile(u, nt, I, J);
        __syncthreads();
        load_panel<false, true>(a.T1, n, n, I * kPT, sa, a.kpad);
        load_panel<true, false>(a.X, n, n, J * kPT, sb, a.kpad);
        __syncthreads();
        const int i = I * kPT + ty, j = J * kPT + tx;
        const double v = tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n);
        store_sym(a.T2, n, n, i, j, v);
        // |F'_ij| off the diagonal: row i of tile column J and (mirror) row j of tile column I
        __shared__ double tabs[kPT][kPT + 1];
        tabs[ty][tx] = (i < n && j < n && i != j) ? fabs(v) : 0.0;
        __syncthreads();
        if (threadIdx.x < kPT) {
            const int r = threadIdx.x;
            double rs = 0.0, cs = 0.0;
            for (int c = 0; c < kPT; ++c) { rs += tabs[r][c]; cs += tabs[c][r]; }
            if (I * kPT + r < n) a.rowpart[static_cast<long long>(I * kPT + r) * nt + J] = rs;
            if (I != J && J * kPT + r < n) a.rowpart[static_cast<long long>(J * kPT + r) * nt + I] = cs;
        }
    }
    if (!grid_barrier(a, epoch)) return;
    mark_phase(a, t_start, 0);

    // 3. Gershgorin interval (every CTA, same order) and P0 in Pa with its partial sums
    __shared__ double bounds[2];
    {
        double lo = 1e300, hi = -1e300;
        for (int i = threadIdx.x; i < n; i += kPurifyThreads) {
            double r = 0.0;
            for (int c = 0; c < nt; ++c) r += __ldcg(a.rowpart + static_cast<long long>(i) * nt + c);
            const double d = __ldcg(a.T2 + static_cast<long long>(i) * n + i);
            lo = fmin(lo, d - r);
            hi = fmax(hi, d + r);
        }
        __shared__ double rlo[kPurifyThreads / 32], rhi[kPurifyThreads / 32];
        for (int o = 16; o > 0; o >>= 1) {
            lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if ((threadIdx.x & 31) == 0) { rlo[threadIdx.x >> 5] = lo; rhi[threadIdx.x >> 5] = hi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 0; w < kPurifyThreads / 32; ++w) { lo = fmin(lo, rlo[w]); hi = fmax(hi, rhi[w]); }
            if (!(hi > lo)) hi = lo + 1.0;  // F' a multiple of I: any positive width
            bounds[0] = lo;
            bounds[1] = hi;
        }
        __syncthreads();
    }
    {
        const double lo = bounds[0], hi = bounds[1], inv = 1.0 / (hi - lo);
        for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
            int I, J;
            upper_tile(u, nt, I, J);
            const int i = I * kPT + ty, j = J * kPT + tx;
            float v = 0.f;
            if (i < n && j < n) {
                const double f = __ldcg(a.T2 + static_cast<long long>(i) * n + j);
                v = static_cast<float>(((i == j ? hi : 0.0) - f) * inv);
            }
            store_sym(a.Pa, n, a.ldp, i, j, v);
            tile_partials(a, 0, u, I == J, i, j, static_cast<double>(v));
        }
    }
    if (!grid_barrier(a, epoch)) return;
    mark_phase(a, t_start, 1);

    // 4. SP2 steps in FP32
    float* P = a.Pa;
    float* Pn = a.Pb;
    double e1 = -1.0, e2 = -1.0;  // e_{k-1}, e_{k-2}
    double e = 0.0;
    int k = 0;
    bool converged = false;
    __shared__ double totals[2];
    const int lane = threadIdx.x & 31;
    for (; k < a.max_steps; ++k) {
        // warp 0 issues the loads of the tile partials of P (for tr P and |P|_F^2) first,
        // then every thread loads the panels of this CTA's first tile, so the two L2
        // round trips overlap; the totals are summed in the same order in every CTA
        const double2* pp = reinterpret_cast<const double2*>(a.part + static_cast<long long>(k & 1) * a.nup * 2);
        double2 pre[4];
        if (threadIdx.x < 32) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int u = lane + 32 * j;
                pre[j] = u < a.nup ? __ldcg(pp + u) : make_double2(0.0, 0.0);
            }
        }
        const int u0 = blockIdx.x;
        int I0 = 0, J0 = 0;
        if (u0 < a.nup) {
            upper_tile(u0, nt, I0, J0);
            load_panel<false, true>(P, n, a.ldp, I0 * kPT, fa, a.kpad);
            load_panel<false, true>(P, n, a.ldp, J0 * kPT, fb, a.kpad);  // P symmetric: columns = rows
        }
        if (threadIdx.x < 32) {
            double x = 0.0, y = 0.0;
#pragma unroll
            for (int j = 0; j < 4; ++j) { x += pre[j].x; y += pre[j].y; }
            for (int u = lane + 128; u < a.nup; u += 32) {
                const double2 q = __ldcg(pp + u);
                x += q.x;
                y += q.y;
            }
            for (int o = 16; o > 0; o >>= 1) {
                x += __shfl_xor_sync(0xffffffffu, x, o);
                y += __shfl_xor_sync(0xffffffffu, y, o);
            }
            if (lane == 0) { totals[0] = x; totals[1] = y; }
        }
        __syncthreads();
        const double tr = totals[0], fro = totals[1];
        e = fabs(tr - fro);
        if (e < 1e-9 * n || (k >= 2 && e < 1e-2 && e >= e2)) {
            converged = true;
            break;
        }
        e2 = e1;
        e1 = e;
        const bool square = fabs(fro - a.nocc) < fabs(2.0 * tr - fro - a.nocc);
        for (int u = u0; u < a.nup; u += gridDim.x) {
            int I = I0, J = J0;
            if (u != u0) {
                upper_tile(u, nt, I, J);
                __syncthreads();
                load_panel<false, true>(P, n, a.ldp, I * kPT, fa, a.kpad);
                load_panel<false, true>(P, n, a.ldp, J * kPT, fb, a.kpad);
                __syncthreads();
            }
            const int i = I * kPT + ty, j = J * kPT + tx;
            const float p2 = tile_dot(fa + ty * a.kpad, fb + tx * a.kpad, n);
            float v = p2;
            if (!square) {
                // P_ij is in the panels: row i of the I panel, column j = the J panel's row j
                const float p = (J * kPT + tx < n) ? fa[ty * a.kpad + J * kPT + tx] : 0.f;
                v = 2.f * p - p2;
            }
            store_sym(Pn, n, a.ldp, i, j, v);
            tile_partials(a, (k + 1) & 1, u, I == J, i, j, static_cast<double>(v));
        }
        if (!grid_barrier(a, epoch)) return;
        float* t = P;
        P = Pn;
        Pn = t;
    }

    mark_phase(a, t_start, 2);
    // 5. McWeeny in FP64: T2 = P^2, W = 3 T2 - 2 T2 P (step 1 from the FP32 P); a second
    //    step (T2 = W^2, T1 = 3 T2 - 2 T2 W) only if step 1 left |tr - |.|_F^2| above 1e-13 N
    for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
        int I, J;
        upper_tile(u, nt, I, J);
        __syncthreads();
        load_panel<false, true>(P, n, a.ldp, I * kPT, sa, a.kpad);
        load_panel<false, true>(P, n, a.ldp, J * kPT, sb, a.kpad);
        __syncthreads();
        store_sym(a.T2, n, n, I * kPT + ty, J * kPT + tx, tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n));
    }
    if (!grid_barrier(a, epoch)) return;
    for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
        int I, J;
        upper_tile(u, nt, I, J);
        __syncthreads();
        load_panel<false, true>(a.T2, n, n, I * kPT, sa, a.kpad);
        load_panel<false, true>(P, n, a.ldp, J * kPT, sb, a.kpad);
        __syncthreads();
        const int i = I * kPT + ty, j = J * kPT + tx;
        const double p3 = tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n);
        const double p2 = (j < n) ? sa[ty * a.kpad + j] : 0.0;
        const double v = 3.0 * p2 - 2.0 * p3;
        store_sym(a.W, n, n, i, j, v);
        tile_partials(a, 0, u, I == J, i, j, v);
    }
    if (!grid_barrier(a, epoch)) return;
    double tr, fro;
    tile_totals(a, 0, tr, fro);
    const bool second = fabs(tr - fro) > 1e-13 * n;
    if (second) {
        for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
            int I, J;
            upper_tile(u, nt, I, J);
            __syncthreads();
            load_panel<false, true>(a.W, n, n, I * kPT, sa, a.kpad);
            load_panel<false, true>(a.W, n, n, J * kPT, sb, a.kpad);
            __syncthreads();
            store_sym(a.T2, n, n, I * kPT + ty, J * kPT + tx, tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n));
        }
        if (!grid_barrier(a, epoch)) return;
        for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
            int I, J;
            upper_tile(u, nt, I, J);
            __syncthreads();
            load_panel<false, true>(a.T2, n, n, I * kPT, sa, a.kpad);
            load_panel<false, true>(a.W, n, n, J * kPT, sb, a.kpad);
            __syncthreads();
            const int i = I * kPT + ty, j = J * kPT + tx;
            const double p3 = tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n);
            const double p2 = (j < n) ? sa[ty * a.kpad + j] : 0.0;
            const double v = 3.0 * p2 - 2.0 * p3;
            store_sym(a.T1, n, n, i, j, v);
            tile_partials(a, 1, u, I == J, i, j, v);
        }
        if (!grid_barrier(a, epoch)) return;
        tile_totals(a, 1, tr, fro);
    }
    mark_phase(a, t_start, 3);
    const double* Pf = second ? a.T1 : a.W;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.status[kPurifyStatusSteps] = k;
        a.status[kPurifyStatusTraceError] = tr - a.nocc;
        a.status[kPurifyStatusIdempotency] = fabs(tr - fro);
        a.status[kPurifyStatusSp2Error] = e;
        a.status[kPurifyStatusSp2Converged] = converged ? 1.0 : 0.0;
        a.status[kPurifyStatusMcWeeny] = second ? 2.0 : 1.0;
    }

    // 6. T2 = X P (all tiles); the projector to W when it ended in T1
    for (int t = blockIdx.x; t < nt * nt; t += gridDim.x) {
        const int I = t / nt, J = t % nt;
        __syncthreads();
        load_panel<false, false>(a.X, n, n, I * kPT, sa, a.kpad);
        load_panel<false, true>(Pf, n, n, J * kPT, sb, a.kpad);  // P symmetric
        __syncthreads();
        const int i = I * kPT + ty, j = J * kPT + tx;
        const double v = tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n);
        if (i < n && j < n) {
            a.T2[static_cast<long long>(i) * n + j] = v;
            if (second) a.W[static_cast<long long>(i) * n + j] = __ldcg(a.T1 + static_cast<long long>(i) * n + j);
        }
    }
    if (!grid_barrier(a, epoch)) return;
    mark_phase(a, t_start, 4);

    // 7. D = 2 T2 X^T (upper tiles, mirrored)
    for (int u = blockIdx.x; u < a.nup; u += gridDim.x) {
        int I, J;
        upper_tile(u, nt, I, J);
        __syncthreads();
        load_panel<false, true>(a.T2, n, n, I * kPT, sa, a.kpad);
        load_panel<false, false>(a.X, n, n, J * kPT, sb, a.kpad);  // rows of X = columns of X^T
        __syncthreads();
        store_sym(a.D, n, n, I * kPT + ty, J * kPT + tx, 2.0 * tile_dot(sa + ty * a.kpad, sb + tx * a.kpad, n));
    }
    mark_phase(a, t_start, 5);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.status[kPurifyStatusBarriers] = epoch;
}

}  // namespace

bool purify_fused_supported(const Engine& e) { return e.scf.n >= 1 && e.scf.n <= kPurifyMaxN; }

// scratch layout (doubles): status words, 2 words of barrier, then (fused path)
// the per-tile partial sums [2][nup][2] and the Gershgorin partials [n][nt]
int purify_status(Engine& e, double** status)
{
    auto& w = e.scf;
    const int n = w.n;
    const int nt = (n + kPT - 1) / kPT;
    const int nup = nt * (nt + 1) / 2;
    const size_t need = kPurifyStatusWords + 2 + 4 * static_cast<size_t>(nup) + static_cast<size_t>(n) * nt;
    if (!w.pur || w.pur_doubles < need) {
        if (w.pur) cudaFree(w.pur);
        w.pur = nullptr;
        w.pur_doubles = 0;
        GB_CUDA_TRY(cudaMalloc(&w.pur, need * sizeof(double)));
        w.pur_doubles = need;
    }
    *status = w.pur;
    return HF_OK;
}

int purify_fused(Engine& e, const double* F, int nocc, double* D, cudaStream_t s, int max_steps)
{
    auto& w = e.scf;
    const int n = w.n;
    if (n < 1 || n > kPurifyMaxN) return set_error("fused purification: N out of range"), HF_ERR_INVALID_ARGUMENT;
    const int nt = (n + kPT - 1) / kPT;
    const int nup = nt * (nt + 1) / 2;
    const size_t nld = static_cast<size_t>(n) * ((n + 3) & ~3);  // projector rows padded to 4 floats
    if (!w.P32a) {
        GB_CUDA_TRY(cudaMalloc(&w.P32a, nld * sizeof(float)));
        GB_CUDA_TRY(cudaMalloc(&w.P32b, nld * sizeof(float)));
    }
    double* status = nullptr;
    int st = purify_status(e, &status);
    if (st) return st;
    PurifyArgs a;
    a.n = n;
    a.nocc = nocc;
    a.nt = nt;
    a.nup = nup;
    a.ldp = (n + 3) & ~3;             // FP32 projector rows of 16-byte multiples (float4 loads)
    a.kpad = ((n + 3) & ~3) + 1;      // odd shared-memory row stride: conflict-free columns
    a.max_steps = max_steps > 0 ? std::min(max_steps, kPurifyMaxSteps) : kPurifyMaxSteps;
    a.X = w.X;
    a.F = F;
    a.T1 = w.T1;
    a.T2 = w.T2;
    a.W = w.W;
    a.D = D;
    a.Pa = w.P32a;
    a.Pb = w.P32b;
    a.status = status;
    a.bar = reinterpret_cast<unsigned*>(status + kPurifyStatusWords);
    a.part = status + kPurifyStatusWords + 2;
    a.rowpart = a.part + 4 * nup;
    const size_t smem = 2 * kPT * static_cast<size_t>(a.kpad) * sizeof(double);
    GB_CUDA_TRY(cudaFuncSetAttribute(purify_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(2 * kPT * (((kPurifyMaxN + 3) & ~3) + 1) * sizeof(double))));
    int per_sm = 0;
    GB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, purify_kernel, kPurifyThreads, smem));
    if (per_sm < 1) return set_error("fused purification: the kernel does not fit on an SM"), HF_ERR_CUDA;
    const int grid = e.num_sms;  // one CTA per SM, all co-resident
    // status words and the barrier start at zero
    GB_CUDA_TRY(cudaMemsetAsync(status, 0, (kPurifyStatusWords + 2) * sizeof(double), s));
    void* args[] = {&a};
    GB_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(purify_kernel), dim3(grid), dim3(kPurifyThreads),
                                            args, smem, s));
    count_launch();
    return HF_OK;
}

}  // namespace gb
