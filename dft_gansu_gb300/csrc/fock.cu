// Fock-build orchestration: density scaling, the mixed-precision plan, the
// per-class launches and the symmetrising finish.
//
//   D' = s D s                      (s_i = cgto_i * component factor)
//   J', K' accumulated by the class kernels (fock_kernel.cuh)
//   J = s (2 (J' + J'^T)) s,  K = s (K' + K'^T) s,  F = H + J - K/2
//                                   (src/gpu_kernels.cu:230-287 semantics)
//
// Mixed precision: a quartet goes to the FP32 queue when
// Qs_bra * Qs_ket * c_max^4 * max|D| < mixed_threshold, i.e. when the bound on
// its Fock contribution is below the threshold (c_max = largest CGTO factor,
// Qs = sum of primitive-pair Schwarz bounds).  Kets of a bra are sorted by Qs,
// so each bra's FP64 kets are a prefix of its surviving kets; the plan kernel
// finds that prefix by bisection and prefix-sums both queues on the device,
// so no host round trip is needed between the density and the launches.
#include <algorithm>
#include <limits>
#include <string>

#include "engine.hpp"
#include "fock_kernel.cuh"

namespace gb {

// ------------------------------------------------------------------ tables
#define GB_DECL(a, b, c, d)                                                                                   \
    void launch_fock_##a##_##b##_##c##_##d(bool, const FockClassLaunch&, int, cudaStream_t);                 \
    void launch_eri_##a##_##b##_##c##_##d(const FockClassLaunch&, const double*, double*, int, cudaStream_t);
#define GB_CLASSES(X)                                                                                         \
    X(0, 0, 0, 0) X(1, 0, 0, 0) X(1, 0, 1, 0) X(1, 1, 0, 0) X(1, 1, 1, 0) X(1, 1, 1, 1) X(2, 0, 0, 0)         \
    X(2, 0, 1, 0) X(2, 0, 1, 1) X(2, 0, 2, 0) X(2, 1, 0, 0) X(2, 1, 1, 0) X(2, 1, 1, 1) X(2, 1, 2, 0)         \
    X(2, 1, 2, 1) X(2, 2, 0, 0) X(2, 2, 1, 0) X(2, 2, 1, 1) X(2, 2, 2, 0) X(2, 2, 2, 1) X(2, 2, 2, 2)
GB_CLASSES(GB_DECL)
#undef GB_DECL

FockLauncher fock_launcher(int la, int lb, int lc, int ld)
{
#define GB_CASE(a, b, c, d)                                                 \
    if (la == a && lb == b && lc == c && ld == d) return &launch_fock_##a##_##b##_##c##_##d;
    GB_CLASSES(GB_CASE)
#undef GB_CASE
    return nullptr;
}

EriLauncher eri_launcher(int la, int lb, int lc, int ld)
{
#define GB_CASE(a, b, c, d)                                                 \
    if (la == a && lb == b && lc == c && ld == d) return &launch_eri_##a##_##b##_##c##_##d;
    GB_CLASSES(GB_CASE)
#undef GB_CASE
    return nullptr;
}

namespace {

constexpr int kPlanThreads = 256;

// D' = s D s per molecule block (global function g = bf0 + local index)
__global__ void scale_density_kernel(const double* __restrict__ D, const double* __restrict__ s, const BlockMap M,
                                     double* __restrict__ Dp64, float* __restrict__ Dp32)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        const int n = M.n[m], g0 = M.bf0[m];
        const long long r = k - M.base[m];
        const int i = static_cast<int>(r / n), j = static_cast<int>(r % n);
        const double v = s[g0 + i] * D[k] * s[g0 + j];
        Dp64[k] = v;
        if (Dp32) Dp32[k] = static_cast<float>(v);
    }
}

// max |D| over each shell block, both orders: out[A * ns + B] (shell first function and size in info)
__global__ void block_absmax_kernel(const double* __restrict__ D, const int2* __restrict__ info, int ns, int n,
                                    float* __restrict__ out)
{
    const long long total = static_cast<long long>(ns) * ns;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int A = static_cast<int>(k / ns), B = static_cast<int>(k % ns);
        const int2 a = info[A], b = info[B];
        double m = 0.0;
        for (int i = 0; i < a.y; ++i)
            for (int j = 0; j < b.y; ++j) m = fmax(m, fabs(D[static_cast<long long>(a.x + i) * n + b.x + j]));
        out[k] = static_cast<float>(m);
    }
}

__global__ void absmax_kernel(const double* __restrict__ A, long long n, double* __restrict__ out)
{
    __shared__ double red[32];
    double m = 0.0;
    for (long long k = threadIdx.x; k < n; k += blockDim.x) m = fmax(m, fabs(A[k]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) *out = m;
    }
}

// max |D| of every molecule's block: one CTA per molecule
__global__ void mol_absmax_kernel(const double* __restrict__ A, const BlockMap M, double* __restrict__ out)
{
    __shared__ double red[32];
    const int m = blockIdx.x;
    const long long b0 = M.base[m], b1 = M.base[m + 1];
    double v = 0.0;
    for (long long k = b0 + threadIdx.x; k < b1; k += blockDim.x) v = fmax(v, fabs(A[k]));
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) out[m] = v;
    }
}

// Exclusive-scan helper over one block (values of this pass), returns the
// pass total; the running base is kept by the caller.
__device__ long long block_scan_exclusive(long long v, long long* smem, long long& total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[wid] = x;
    __syncthreads();
    if (wid == 0) {
        long long w = (lane < (blockDim.x >> 5)) ? smem[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        smem[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const long long warp_base = (wid > 0) ? smem[wid - 1] : 0;
    total = smem[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_base + x - v;
}

struct PlanArgs {
    const int* entry_bra;
    const int* entry_cnt;
    const int* entry_lo0;       // class-relative first ket of the entry's group
    const double* pair_qs;
    const int* cp_entry_begin;  // per class pair
    const int* cp_nentry;
    const int* cp_ket_base;
    const int* cp_off_base;     // start of the class pair's offsets
    const double* dmax;
    double factor;              // c_max^4
    double mixed_threshold;
    double skip_threshold;      // quartets with Qs_ab*Qs_cd*c_max^4*max|D| below this are dropped
    int square;                 // weight by max|D|^2 (gradient) instead of max|D| (Fock)
    long long* off64;
    long long* off32;
    int* lo32;
    // batches: per-molecule max|D|, FP32 cut and drop threshold (the bra pair's
    // molecule through pairs[bra].A -> shell_mol); null for one molecule
    const ShellPairDev* pairs = nullptr;
    const int* shell_mol = nullptr;
    const double* mol_dmax = nullptr;
    const double* mol_tau = nullptr;
    const double* mol_skip = nullptr;
};

// The plan in two launches: plan_count_kernel, one thread per entry of every class pair
// (the two bisections of an entry are independent of the others), writes the entry's FP64
// and FP32 ket counts into its slot of the offset arrays; plan_scan_kernel, one block per
// class pair, turns each class pair's counts into the prefix offsets in place.
__global__ void __launch_bounds__(kPlanThreads) plan_count_kernel(PlanArgs a, int ncp, int nentries)
{
    __shared__ int sbeg[kNumClassPairs + 1];
    for (int c = threadIdx.x; c <= ncp; c += blockDim.x)
        sbeg[c] = (c < ncp) ? a.cp_entry_begin[c] : nentries;
    __syncthreads();
    const double dmv = *a.dmax;
    const double dm = (a.square ? dmv * dmv : dmv) * a.factor;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nentries; e += gridDim.x * blockDim.x) {
        int cp = 0;  // class pair of entry e: the last with sbeg[cp] <= e
        for (int lo = 0, hi = ncp - 1; lo <= hi;) {
            const int mid = (lo + hi) >> 1;
            if (sbeg[mid] <= e) { cp = mid; lo = mid + 1; } else { hi = mid - 1; }
        }
        const int i = e - sbeg[cp], ob = a.cp_off_base[cp];
        const int cnt = a.entry_cnt[e];
        const int k0 = a.cp_ket_base[cp] + a.entry_lo0[e];
        const int bra = a.entry_bra[e];
        double qb = a.pair_qs[bra] * dm, tau = a.mixed_threshold, skip = a.skip_threshold;
        if (a.mol_dmax) {
            const int m = a.shell_mol[a.pairs[bra].A];
            const double d = a.mol_dmax[m];
            qb = a.pair_qs[bra] * (a.square ? d * d : d) * a.factor;
            tau = a.mol_tau[m];
            skip = a.mol_skip[m];
        }
        int lo = 0, hi = cnt;  // first ket of the group with qb*Qs_ket < tau
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (qb * a.pair_qs[k0 + mid] >= tau) lo = mid + 1; else hi = mid;
        }
        // density-weighted screening: the tail whose bound times max|D| is below the
        // Schwarz threshold contributes nothing measurable (it matters for dD builds)
        int hi2 = cnt, lo2 = lo;
        while (lo2 < hi2) {
            const int mid = (lo2 + hi2) >> 1;
            if (qb * a.pair_qs[k0 + mid] >= skip) lo2 = mid + 1; else hi2 = mid;
        }
        a.lo32[e] = a.entry_lo0[e] + lo;
        a.off64[ob + i + 1] = lo;
        a.off32[ob + i + 1] = lo2 - lo;
    }
}

// One block per class pair: in-place inclusive scan of the counts at off[ob + 1 .. ob + ne].
__global__ void __launch_bounds__(kPlanThreads) plan_scan_kernel(PlanArgs a)
{
    __shared__ long long smem[32];
    const int cp = blockIdx.x;
    const int ne = a.cp_nentry[cp], ob = a.cp_off_base[cp];
    if (threadIdx.x == 0) { a.off64[ob] = 0; a.off32[ob] = 0; }
    long long base64 = 0, base32 = 0;
    for (int start = 0; start < ne; start += blockDim.x) {
        const int i = start + threadIdx.x;
        const long long c64 = (i < ne) ? a.off64[ob + i + 1] : 0, c32 = (i < ne) ? a.off32[ob + i + 1] : 0;
        long long t64, t32;
        const long long x64 = block_scan_exclusive(c64, smem, t64);
        const long long x32 = block_scan_exclusive(c32, smem, t32);
        if (i < ne) {
            a.off64[ob + i + 1] = base64 + x64 + c64;
            a.off32[ob + i + 1] = base32 + x32 + c32;
        }
        base64 += t64;
        base32 += t32;
    }
}

void launch_plan(const PlanArgs& a, int ncp, int nentries, int num_sms, cudaStream_t s)
{
    const int grid = std::max(1, std::min((nentries + kPlanThreads - 1) / kPlanThreads, 4 * num_sms));
    plan_count_kernel<<<grid, kPlanThreads, 0, s>>>(a, ncp, nentries);
    plan_scan_kernel<<<ncp, kPlanThreads, 0, s>>>(a);
}

__global__ void finish_kernel(const double* __restrict__ Jp, const double* __restrict__ Kp,
                              const float* __restrict__ Jp32, const float* __restrict__ Kp32,
                              const double* __restrict__ s, const double* __restrict__ H, const BlockMap M,
                              double* __restrict__ J, double* __restrict__ K, double* __restrict__ F)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < M.nelem;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int m = block_of(M, k);
        const int n = M.n[m], g0 = M.bf0[m];
        const long long base = M.base[m], r = k - base;
        const int i = static_cast<int>(r / n), j = static_cast<int>(r % n);
        const long long kt = base + static_cast<long long>(j) * n + i;
        const double ss = s[g0 + i] * s[g0 + j];
        double jsum = Jp[k] + Jp[kt], ksum = Kp[k] + Kp[kt];
        if (Jp32) {
            jsum += static_cast<double>(Jp32[k]) + static_cast<double>(Jp32[kt]);
            ksum += static_cast<double>(Kp32[k]) + static_cast<double>(Kp32[kt]);
        }
        const double jv = 2.0 * jsum * ss;
        const double kv = ksum * ss;
        if (J) J[k] = jv;
        if (K) K[k] = kv;
        if (F) F[k] = H[k] + jv - 0.5 * kv;
    }
}

// blocks for one thread per work item, at most num_sms * blocks_per_sm (the kernels loop over the rest)
int grid_for_cap(long long work, int num_sms, int blocks_per_sm)
{
    const long long blocks = (work + kFockThreads - 1) / kFockThreads;
    return static_cast<int>(
        std::max<long long>(1, std::min<long long>(blocks, static_cast<long long>(num_sms) * blocks_per_sm)));
}

int grid_for(long long work, int num_sms) { return grid_for_cap(work, num_sms, kFockBlocksPerSm); }

// grid of class pair c's FP64 or FP32 launch under the engine's schedule
int class_grid(const Engine& e, int c, bool fp32)
{
    const std::vector<int>& v = fp32 ? e.sched.cap32 : e.sched.cap64;
    const int cap = (c < static_cast<int>(v.size()) && v[c] > 0) ? v[c] : kFockBlocksPerSm;
    return grid_for_cap(e.class_pairs[c].n_survivors, e.num_sms, cap);
}

FockClassLaunch make_launch(Engine& e, int cpi, bool fp32, const long long* off, const int* lo)
{
    const ClassPair& cp = e.class_pairs[cpi];
    FockClassLaunch L;
    L.pairs = e.d_pairs;
    L.prim_pairs = fp32 ? static_cast<const void*>(e.d_pp32) : static_cast<const void*>(e.d_pp64);
    L.boys_table = fp32 ? static_cast<const void*>(e.d_boys32) : static_cast<const void*>(e.d_boys64);
    L.density = fp32 ? static_cast<const void*>(e.d_Dp32) : static_cast<const void*>(e.d_Dp64);
    L.J = e.d_Jp;
    L.K = e.d_Kp;
    L.J32 = e.d_Jp32;
    L.K32 = e.d_Kp32;
    L.off = off + cp.entry_begin + cpi;
    L.entry_bra = e.d_entry_bra + cp.entry_begin;
    L.entry_lo = lo + cp.entry_begin;
    L.entry_prim = e.d_entry_prim + cp.entry_begin;
    L.nentry = cp.nentry;
    L.ket_base = e.pair_classes[cp.Y].begin;
    L.num_basis = e.num_basis;
    L.schwarz_threshold = e.schwarz_threshold;
    L.counters = e.d_counters + 2 * (2 * cpi + (fp32 ? 1 : 0));
    L.block_dmax = nullptr;
    L.nshell = e.num_shells;
    L.skip_cut = 0.0;
    L.mol_active = e.d_mol_active;
    L.shell_mol = e.d_shell_mol;
    return L;
}

}  // namespace

// branch streams and events of the schedule, created on first use
int schedule_streams(Engine& e)
{
    FockSchedule& S = e.sched;
    if (!S.fork) GB_CUDA_TRY(cudaEventCreateWithFlags(&S.fork, cudaEventDisableTiming));
    for (int b = 0; b < S.nbranch && b < kMaxBranches; ++b) {
        if (!S.branch[b]) GB_CUDA_TRY(cudaStreamCreateWithFlags(&S.branch[b], cudaStreamNonBlocking));
        if (!S.join[b]) GB_CUDA_TRY(cudaEventCreateWithFlags(&S.join[b], cudaEventDisableTiming));
    }
    if (S.use_graph && !S.capture) GB_CUDA_TRY(cudaStreamCreateWithFlags(&S.capture, cudaStreamNonBlocking));
    return HF_OK;
}

int scale_density(Engine& e, const double* d_D, bool want_fp32, cudaStream_t s)
{
    const long long nn = e.nelem;
    const int grid = static_cast<int>(std::min<long long>((nn + 255) / 256, 4096));
    scale_density_kernel<<<grid, 256, 0, s>>>(d_D, e.d_scale, e.block_map(), e.d_Dp64, want_fp32 ? e.d_Dp32 : nullptr);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// Splits every class pair's static quartet list into an FP64 prefix and an FP32
// remainder on the device: FP64 where Qs_bra*Qs_ket*factor*max|D| >= tau
// (max|D|^2 with square), dropped below skip.  max|D| from an absmax of d_D.
static int mixed_plan_args(Engine& e, const double* d_D, double factor, bool square, double tau, double skip,
                           cudaStream_t s, PlanArgs* out)
{
    const int ncp = static_cast<int>(e.class_pairs.size());
    absmax_kernel<<<1, 1024, 0, s>>>(d_D, e.nelem, e.d_scalar);
    GB_LAUNCH_CHECK();
    PlanArgs a;
    a.entry_bra = e.d_entry_bra;
    a.entry_cnt = e.d_entry_cnt;
    a.entry_lo0 = e.d_entry_lo0;
    a.pair_qs = e.d_pair_qs;
    a.cp_entry_begin = e.d_cp_meta;
    a.cp_nentry = e.d_cp_meta + ncp;
    a.cp_ket_base = e.d_cp_meta + 2 * ncp;
    a.cp_off_base = e.d_cp_meta + 3 * ncp;
    a.dmax = e.d_scalar;
    a.factor = factor;
    a.mixed_threshold = tau;
    a.skip_threshold = skip;
    a.square = square ? 1 : 0;
    a.off64 = e.plan.off64;
    a.off32 = e.plan.off32;
    a.lo32 = e.plan.lo32;
    launch_plan(a, ncp, static_cast<int>(e.entry_bra.size()), e.num_sms, s);
    GB_LAUNCH_CHECK();
    if (out) *out = a;
    return HF_OK;
}

int mixed_plan(Engine& e, const double* d_D, double factor, bool square, double tau, double skip, cudaStream_t s)
{
    return mixed_plan_args(e, d_D, factor, square, tau, skip, s, nullptr);
}

int mol_absmax(Engine& e, const double* d_A, double* d_out, cudaStream_t s)
{
    mol_absmax_kernel<<<e.nmol, 256, 0, s>>>(d_A, e.block_map(), d_out);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

// Batch build with a precision rule per molecule: quartets of molecule m go to
// FP64 where Qs_ab Qs_cd c_max^4 max|D_m| >= mol_tau[m], to FP32 below that, and
// are dropped below mol_skip[m] (tau = skip = inf: the molecule is not built).
// d_D holds each molecule's density or density difference; mol_dmax receives
// max|D_m|.  J', K' (FP64 and FP32 tiers) are left for the caller's finish.
int build_jk_batch(Engine& e, const double* d_D, const double* d_mol_tau, const double* d_mol_skip,
                   double* d_mol_dmax, cudaStream_t s)
{
    const size_t nn = static_cast<size_t>(e.nelem);
    int st = scale_density(e, d_D, true, s);
    if (st) return st;
    GB_CUDA_TRY(cudaMemsetAsync(e.d_Jp, 0, nn * sizeof(double), s));
    GB_CUDA_TRY(cudaMemsetAsync(e.d_Kp, 0, nn * sizeof(double), s));
    GB_CUDA_TRY(cudaMemsetAsync(e.d_Jp32, 0, nn * sizeof(float), s));
    GB_CUDA_TRY(cudaMemsetAsync(e.d_Kp32, 0, nn * sizeof(float), s));
    e.last_mixed = true;
    mol_absmax_kernel<<<e.nmol, 256, 0, s>>>(d_D, e.block_map(), d_mol_dmax);
    GB_LAUNCH_CHECK();
    const int ncp = static_cast<int>(e.class_pairs.size());
    const double c2 = e.cgto_max * e.cgto_max;
    PlanArgs a;
    a.entry_bra = e.d_entry_bra;
    a.entry_cnt = e.d_entry_cnt;
    a.entry_lo0 = e.d_entry_lo0;
    a.pair_qs = e.d_pair_qs;
    a.cp_entry_begin = e.d_cp_meta;
    a.cp_nentry = e.d_cp_meta + ncp;
    a.cp_ket_base = e.d_cp_meta + 2 * ncp;
    a.cp_off_base = e.d_cp_meta + 3 * ncp;
    a.dmax = d_mol_dmax;
    a.factor = c2 * c2;
    a.mixed_threshold = 0.0;
    a.skip_threshold = 0.0;
    a.square = 0;
    a.off64 = e.plan.off64;
    a.off32 = e.plan.off32;
    a.lo32 = e.plan.lo32;
    a.pairs = e.d_pairs;
    a.shell_mol = e.d_shell_mol;
    a.mol_dmax = d_mol_dmax;
    a.mol_tau = d_mol_tau;
    a.mol_skip = d_mol_skip;
    launch_plan(a, ncp, static_cast<int>(e.entry_bra.size()), e.num_sms, s);
    GB_LAUNCH_CHECK();
    return launch_class_pairs(e, s, [&](int c, cudaStream_t cs) -> int {
        const ClassPair& cp = e.class_pairs[c];
        const PairClass& X = e.pair_classes[cp.X];
        const PairClass& Y = e.pair_classes[cp.Y];
        FockLauncher f = fock_launcher(X.la, X.lb, Y.la, Y.lb);
        if (!f) return set_error("no kernel for quartet class"), HF_ERR_INVALID_ARGUMENT;
        f(false, make_launch(e, c, false, e.plan.off64, e.d_entry_lo0), class_grid(e, c, false), cs);
        GB_LAUNCH_CHECK();
        f(true, make_launch(e, c, true, e.plan.off32, e.plan.lo32), class_grid(e, c, true), cs);
        GB_LAUNCH_CHECK();
        return HF_OK;
    });
}

namespace {

// One direct J/K build as ordinary launches (build_jk below adds the graph replay).
int build_jk_body(Engine& e, const double* d_D, double* d_J, double* d_K, int precision, double mixed_thr,
                  cudaStream_t s, double drop)
{
    const size_t nn = static_cast<size_t>(e.nelem);
    const bool mixed = (precision == HF_PRECISION_MIXED);
    int st = scale_density(e, d_D, mixed, s);
    if (st) return st;
    GB_CUDA_TRY(cudaMemsetAsync(e.d_Jp, 0, nn * sizeof(double), s));
    GB_CUDA_TRY(cudaMemsetAsync(e.d_Kp, 0, nn * sizeof(double), s));
    e.last_mixed = mixed;
    if (mixed) {
        GB_CUDA_TRY(cudaMemsetAsync(e.d_Jp32, 0, nn * sizeof(float), s));
        GB_CUDA_TRY(cudaMemsetAsync(e.d_Kp32, 0, nn * sizeof(float), s));
    }
    if (!mixed) {
        st = launch_class_pairs(e, s, [&](int c, cudaStream_t cs) -> int {
            const ClassPair& cp = e.class_pairs[c];
            const PairClass& X = e.pair_classes[cp.X];
            const PairClass& Y = e.pair_classes[cp.Y];
            FockLauncher f = fock_launcher(X.la, X.lb, Y.la, Y.lb);
            if (!f) return set_error("no kernel for quartet class"), HF_ERR_INVALID_ARGUMENT;
            f(false, make_launch(e, c, false, e.d_off_static, e.d_entry_lo0), class_grid(e, c, false), cs);
            GB_LAUNCH_CHECK();
            return HF_OK;
        });
        if (st) return st;
    } else {
        const double c2 = e.cgto_max * e.cgto_max;
        PlanArgs a;
        const double skip = drop > 0.0 ? drop : std::min(e.schwarz_threshold, mixed_thr);
        int pst = mixed_plan_args(e, d_D, c2 * c2, false, mixed_thr, skip, s, &a);
        if (pst) return pst;
        // per-shell-block maxima of the (difference) density for the per-quartet screen
        // (single-molecule engines: the table is num_shells^2)
        if (e.nmol == 1 && !e.d_block_dmax) {
            std::vector<int2> info(e.num_shells);
            for (int i = 0; i < e.num_shells; ++i) info[i] = make_int2(e.shells[i].bf, ncart(e.shells[i].l));
            GB_CUDA_TRY(cudaMalloc(&e.d_shell_info, sizeof(int2) * e.num_shells));
            GB_CUDA_TRY(cudaMalloc(&e.d_block_dmax, sizeof(float) * e.num_shells * e.num_shells));
            GB_CUDA_TRY(cudaMemcpy(e.d_shell_info, info.data(), sizeof(int2) * e.num_shells, cudaMemcpyHostToDevice));
        }
        if (e.nmol == 1) {
            const long long nsq = static_cast<long long>(e.num_shells) * e.num_shells;
            const int g = static_cast<int>(std::min<long long>((nsq + 255) / 256, 4096));
            block_absmax_kernel<<<g, 256, 0, s>>>(d_D, e.d_shell_info, e.num_shells, e.num_basis, e.d_block_dmax);
            GB_LAUNCH_CHECK();
        }
        st = launch_class_pairs(e, s, [&](int c, cudaStream_t cs) -> int {
            const ClassPair& cp = e.class_pairs[c];
            const PairClass& X = e.pair_classes[cp.X];
            const PairClass& Y = e.pair_classes[cp.Y];
            FockLauncher f = fock_launcher(X.la, X.lb, Y.la, Y.lb);
            if (!f) return set_error("no kernel for quartet class"), HF_ERR_INVALID_ARGUMENT;
            FockClassLaunch l64 = make_launch(e, c, false, e.plan.off64, e.d_entry_lo0);
            FockClassLaunch l32 = make_launch(e, c, true, e.plan.off32, e.plan.lo32);
            l64.block_dmax = l32.block_dmax = e.d_block_dmax;
            l64.skip_cut = l32.skip_cut = a.skip_threshold / a.factor;  // Qs Qs c_max^4 max|dD| < thr
            f(false, l64, class_grid(e, c, false), cs);
            GB_LAUNCH_CHECK();
            f(true, l32, class_grid(e, c, true), cs);
            GB_LAUNCH_CHECK();
            return HF_OK;
        });
        if (st) return st;
    }
    if (d_J || d_K) {
        const int grid = static_cast<int>(std::min<long long>((static_cast<long long>(nn) + 255) / 256, 4096));
        finish_kernel<<<grid, 256, 0, s>>>(e.d_Jp, e.d_Kp, mixed ? e.d_Jp32 : nullptr, mixed ? e.d_Kp32 : nullptr,
                                           e.d_scale, nullptr, e.block_map(), d_J, d_K, nullptr);
        GB_LAUNCH_CHECK();
    }
    return HF_OK;
}

void destroy_graph(FockSchedule::Graph& g)
{
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
}

// graphs hold the grid caps and branch assignment of the schedule they were captured under
void clear_graphs(FockSchedule& S)
{
    for (auto& g : S.graphs) destroy_graph(g);
    S.graphs.clear();
    for (auto& g : S.purify)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    S.purify.clear();
}

}  // namespace

void schedule_release(FockSchedule& S)
{
    clear_graphs(S);
    for (int b = 0; b < kMaxBranches; ++b) {
        if (S.branch[b]) cudaStreamDestroy(S.branch[b]);
        if (S.join[b]) cudaEventDestroy(S.join[b]);
        S.branch[b] = nullptr;
        S.join[b] = nullptr;
    }
    if (S.fork) cudaEventDestroy(S.fork);
    if (S.capture) cudaStreamDestroy(S.capture);
    if (S.cublas_ws) cudaFree(S.cublas_ws);
    S.fork = nullptr;
    S.capture = nullptr;
    S.cublas_ws = nullptr;
}

// One direct J/K build.  With the schedule's use_graph (single-molecule engines),
// the first build with a given (density, J, K, precision, cuts) runs as ordinary
// launches (it also makes the lazy allocations), the second is captured into a
// CUDA graph on the schedule's capture stream, and that and every later one
// replay the graph on s.  The graph reads the density and writes J'/K' (and J, K)
// at replay, so the buffers' contents may change between builds, not their addresses.
int build_jk(Engine& e, const double* d_D, double* d_J, double* d_K, int precision, double mixed_thr,
             cudaStream_t s, double drop)
{
    FockSchedule& S = e.sched;
    if (!S.use_graph || e.nmol != 1) return build_jk_body(e, d_D, d_J, d_K, precision, mixed_thr, s, drop);
    FockSchedule::Graph* g = nullptr;
    for (auto& x : S.graphs)
        if (x.D == d_D && x.J == d_J && x.K == d_K && x.precision == precision && x.mixed_thr == mixed_thr &&
            x.drop == drop) {
            g = &x;
            break;
        }
    if (!g) {
        if (static_cast<int>(S.graphs.size()) >= kMaxFockGraphs) {
            destroy_graph(S.graphs.front());
            S.graphs.erase(S.graphs.begin());
        }
        S.graphs.push_back(FockSchedule::Graph{d_D, d_J, d_K, precision, mixed_thr, drop, 0, nullptr, false, 0});
        g = &S.graphs.back();
    }
    if (!g->exec && g->uses++ == 0) return build_jk_body(e, d_D, d_J, d_K, precision, mixed_thr, s, drop);
    if (!g->exec) {
        int st = schedule_streams(e);
        if (st) return st;
        const long long l0 = launch_count();
        GB_CUDA_TRY(cudaStreamBeginCapture(S.capture, cudaStreamCaptureModeThreadLocal));
        st = build_jk_body(e, d_D, d_J, d_K, precision, mixed_thr, S.capture, drop);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(S.capture, &graph);
        const long long recorded = launch_count() - l0;
        count_launches(-recorded);  // recorded, not launched
        if (st || ce != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            if (!st) set_error(std::string("Fock build capture: ") + cudaGetErrorString(ce));
            return st ? st : HF_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&g->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            g->exec = nullptr;
            return set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie)), HF_ERR_CUDA;
        }
        g->mixed = e.last_mixed;
        g->launches = recorded;
    }
    GB_CUDA_TRY(cudaGraphLaunch(g->exec, s));
    count_launches(g->launches);
    ++S.graph_replays;
    e.last_mixed = g->mixed;
    return HF_OK;
}

// Autotuner of the direct Fock build's launch schedule (hf_engine_autotune).
// Times, on the caller's density, every class pair's FP64 and FP32 launch over
// its whole quartet list at grid caps of 2, 4, 8, 16 and 32 blocks per SM and
// keeps the fastest (the default unless another is 3% faster), then assigns
// the class pairs to 1, 2, 4 or 8 branches (longest measured time first, to the
// least loaded branch) and keeps the branch count whose FP64 build is fastest.
int autotune_schedule(Engine& e, const double* d_D, hf_autotune_report* rep, cudaStream_t s)
{
    FockSchedule& S = e.sched;
    clear_graphs(S);
    const bool use_graph = S.use_graph;
    S.use_graph = false;
    S.nbranch = 1;
    S.branch_of.clear();
    S.cap64.clear();
    S.cap32.clear();
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events()
        {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    GB_CUDA_TRY(cudaEventCreate(&ev.a));
    GB_CUDA_TRY(cudaEventCreate(&ev.b));
    // best of `reps` timings of issue() on s, in ms
    auto timed = [&](int reps, auto&& issue, double* ms) -> int {
        double best = std::numeric_limits<double>::infinity();
        for (int r = 0; r < reps; ++r) {
            GB_CUDA_TRY(cudaEventRecord(ev.a, s));
            int st = issue();
            if (st) return st;
            GB_CUDA_TRY(cudaEventRecord(ev.b, s));
            GB_CUDA_TRY(cudaEventSynchronize(ev.b));
            float f = 0.f;
            GB_CUDA_TRY(cudaEventElapsedTime(&f, ev.a, ev.b));
            best = std::min(best, static_cast<double>(f));
        }
        *ms = best;
        return HF_OK;
    };
    auto fp64_build = [&]() { return build_jk_body(e, d_D, nullptr, nullptr, HF_PRECISION_FP64, 0.0, s, -1.0); };
    int st;
    double ms_default = 0.0;
    if ((st = fp64_build())) return st;  // warm-up
    if ((st = timed(2, fp64_build, &ms_default))) return st;

    // per class pair and precision tier: grid cap
    if ((st = scale_density(e, d_D, true, s))) return st;  // the FP32 tier reads D' in FP32
    const int ncp = static_cast<int>(e.class_pairs.size());
    const int caps[] = {kFockBlocksPerSm, 2, 4, 8, 32};
    S.cap64.assign(ncp, 0);
    S.cap32.assign(ncp, 0);
    std::vector<double> cost(ncp, 0.0);
    int active = 0, changed = 0;
    for (int c = 0; c < ncp; ++c) {
        const ClassPair& cp = e.class_pairs[c];
        if (cp.n_survivors == 0) continue;
        ++active;
        FockLauncher f = fock_launcher(e.pair_classes[cp.X].la, e.pair_classes[cp.X].lb, e.pair_classes[cp.Y].la,
                                       e.pair_classes[cp.Y].lb);
        if (!f) return set_error("no kernel for quartet class"), HF_ERR_INVALID_ARGUMENT;
        for (int tier = 0; tier < 2; ++tier) {
            const bool fp32 = tier == 1;
            const FockClassLaunch L = make_launch(e, c, fp32, e.d_off_static, e.d_entry_lo0);
            f(fp32, L, grid_for_cap(cp.n_survivors, e.num_sms, kFockBlocksPerSm), s);  // warm-up
            GB_LAUNCH_CHECK();
            int best = kFockBlocksPerSm;
            double best_ms = std::numeric_limits<double>::infinity();
            for (int cap : caps) {
                const int grid = grid_for_cap(cp.n_survivors, e.num_sms, cap);
                double ms = 0.0;
                if ((st = timed(2, [&]() -> int {
                         f(fp32, L, grid, s);
                         GB_LAUNCH_CHECK();
                         return HF_OK;
                     }, &ms)))
                    return st;
                if (cap == kFockBlocksPerSm || ms < 0.97 * best_ms) {
                    best_ms = ms;
                    best = cap;
                }
            }
            (fp32 ? S.cap32 : S.cap64)[c] = best;
            if (best != kFockBlocksPerSm) ++changed;
            cost[c] += best_ms;
        }
    }

    // branches: longest processing time first onto the least loaded branch
    std::vector<int> order(ncp);
    for (int c = 0; c < ncp; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    int best_nb = 1;
    std::vector<int> best_map(ncp, 0);
    double best_ms = std::numeric_limits<double>::infinity();
    for (int nb : {1, 2, 4, 8}) {
        std::vector<int> map(ncp, 0);
        std::vector<double> load(nb, 0.0);
        for (int c : order) {
            const int b = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
            map[c] = b;
            load[b] += cost[c];
        }
        S.nbranch = nb;
        S.branch_of = map;
        double ms = 0.0;
        if ((st = fp64_build())) return st;  // warm-up (creates the branch streams)
        if ((st = timed(2, fp64_build, &ms))) return st;
        if (nb == 1 || ms < 0.97 * best_ms) {
            best_ms = ms;
            best_nb = nb;
            best_map = map;
        }
    }
    S.nbranch = best_nb;
    S.branch_of = best_map;
    S.use_graph = use_graph;
    // the timings ran the class kernels outside any build: J'/K' and the class counters start afresh
    GB_CUDA_TRY(cudaMemsetAsync(e.d_counters, 0, kCounterSlots * sizeof(unsigned long long), s));
    if ((st = fp64_build())) return st;
    GB_CUDA_TRY(cudaMemsetAsync(e.d_counters, 0, kCounterSlots * sizeof(unsigned long long), s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (rep) {
        rep->build_ms_default = ms_default;
        rep->build_ms_tuned = best_ms;
        rep->num_branches = best_nb;
        rep->num_class_pairs = active;
        rep->num_caps_changed = changed;
    }
    return HF_OK;
}

int finish_fock(Engine& e, const double* d_H, const double* d_J, const double* d_K, double* d_F, cudaStream_t s)
{
    (void)d_J; (void)d_K;
    const long long nn = e.nelem;
    const int grid = static_cast<int>(std::min<long long>((nn + 255) / 256, 4096));
    finish_kernel<<<grid, 256, 0, s>>>(e.d_Jp, e.d_Kp, e.last_mixed ? e.d_Jp32 : nullptr,
                                       e.last_mixed ? e.d_Kp32 : nullptr, e.d_scale, d_H, e.block_map(), nullptr, nullptr,
                                       d_F);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

}  // namespace gb

// ------------------------------------------------------------ stored path
namespace gb {
namespace {

// F_ij = H_ij + sum_kl D_kl [(ij|kl) - 1/2 (ik|jl)]  (src/gpu_kernels.cu:230-287);
// one warp per (i, j), lanes stride over l.
__global__ void stored_fock_kernel(const double* __restrict__ D, const double* __restrict__ H,
                                   const double* __restrict__ eri, double* __restrict__ F, int n)
{
    const long long warp = (blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long nn = static_cast<long long>(n) * n;
    if (warp >= nn) return;
    const long long i = warp / n, j = warp % n;
    double acc = 0.0;
    for (long long k = 0; k < n; ++k)
        for (long long l = lane; l < n; l += 32) {
            const double d = D[k * n + l];
            acc += d * (eri[((i * n + j) * n + k) * n + l] - 0.5 * eri[((i * n + k) * n + j) * n + l]);
        }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) F[warp] = H[warp] + acc;
}

}  // namespace

int compute_eri_tensor(Engine& e, double* d_eri, cudaStream_t s)
{
    if (e.nmol != 1) return set_error("the stored ERI tensor is for single-molecule engines"), HF_ERR_INVALID_ARGUMENT;
    const size_t n = e.num_basis;
    GB_CUDA_TRY(cudaMemsetAsync(d_eri, 0, n * n * n * n * sizeof(double), s));
    for (int c = 0; c < static_cast<int>(e.class_pairs.size()); ++c) {
        const ClassPair& cp = e.class_pairs[c];
        if (cp.n_survivors == 0) continue;
        const PairClass& X = e.pair_classes[cp.X];
        const PairClass& Y = e.pair_classes[cp.Y];
        EriLauncher f = eri_launcher(X.la, X.lb, Y.la, Y.lb);
        if (!f) return set_error("no kernel for quartet class"), HF_ERR_INVALID_ARGUMENT;
        f(make_launch(e, c, false, e.d_off_static, e.d_entry_lo0), e.d_scale, d_eri, grid_for(cp.n_survivors, e.num_sms),
          s);
        GB_LAUNCH_CHECK();
    }
    return HF_OK;
}

int stored_fock(const double* d_D, const double* d_H, const double* d_eri, double* d_F, int n, cudaStream_t s)
{
    const long long warps = static_cast<long long>(n) * n;
    const long long blocks = (warps * 32 + 255) / 256;
    stored_fock_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(d_D, d_H, d_eri, d_F, n);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int hf_compute_jk_direct(hf_engine* eng, const double* d_density, double* d_J, double* d_K, int precision,
                         double mixed_threshold, void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_J || !d_K) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    if (precision != HF_PRECISION_FP64 && precision != HF_PRECISION_MIXED)
        return set_error("unknown precision"), HF_ERR_INVALID_ARGUMENT;
    return build_jk(*reinterpret_cast<Engine*>(eng), d_density, d_J, d_K, precision, mixed_threshold,
                    static_cast<cudaStream_t>(stream));
}

int hf_compute_fock_direct_rhf(hf_engine* eng, const double* d_density, const double* d_core_hamiltonian,
                               double* d_fock, int precision, double mixed_threshold, void* stream)
{
    clear_error();
    if (!eng || !d_density || !d_core_hamiltonian || !d_fock) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    if (precision != HF_PRECISION_FP64 && precision != HF_PRECISION_MIXED)
        return set_error("unknown precision"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = build_jk(e, d_density, nullptr, nullptr, precision, mixed_threshold, s);
    if (st) return st;
    return finish_fock(e, d_core_hamiltonian, nullptr, nullptr, d_fock, s);
}

int hf_engine_set_fock_schedule(hf_engine* eng, int num_branches, int use_graph)
{
    clear_error();
    if (!eng || num_branches < 1 || num_branches > kMaxBranches)
        return set_error("hf_engine_set_fock_schedule: num_branches must be 1..8"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    clear_graphs(e.sched);
    e.sched.nbranch = num_branches;
    e.sched.use_graph = use_graph != 0;
    return HF_OK;
}

int hf_engine_set_fock_grid_caps(hf_engine* eng, int num_class_pairs, const int* cap_fp64, const int* cap_fp32,
                                 const int* branch)
{
    clear_error();
    if (!eng) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    Engine& e = *reinterpret_cast<Engine*>(eng);
    FockSchedule& S = e.sched;
    const int ncp = static_cast<int>(e.class_pairs.size());
    if (num_class_pairs != ncp)
        return set_error("hf_engine_set_fock_grid_caps: the engine has " + std::to_string(ncp) + " class pairs, not " +
                         std::to_string(num_class_pairs)),
               HF_ERR_INVALID_ARGUMENT;
    for (int c = 0; c < ncp; ++c)
        if ((cap_fp64 && (cap_fp64[c] < 1 || cap_fp64[c] > 64)) || (cap_fp32 && (cap_fp32[c] < 1 || cap_fp32[c] > 64)) ||
            (branch && (branch[c] < 0 || branch[c] >= kMaxBranches)))
            return set_error("hf_engine_set_fock_grid_caps: caps must be 1..64 blocks per SM, branches 0..7"),
                   HF_ERR_INVALID_ARGUMENT;
    clear_graphs(S);
    S.cap64.assign(cap_fp64 ? cap_fp64 : nullptr, cap_fp64 ? cap_fp64 + ncp : nullptr);
    S.cap32.assign(cap_fp32 ? cap_fp32 : nullptr, cap_fp32 ? cap_fp32 + ncp : nullptr);
    S.branch_of.assign(branch ? branch : nullptr, branch ? branch + ncp : nullptr);
    return HF_OK;
}

int hf_engine_autotune(hf_engine* eng, const double* d_density, hf_autotune_report* report, void* stream)
{
    clear_error();
    if (!eng || !d_density) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    return autotune_schedule(*reinterpret_cast<Engine*>(eng), d_density, report, static_cast<cudaStream_t>(stream));
}

int hf_engine_graph_stats(const hf_engine* eng, int* fock_graphs, int* purification_graphs, long long* replays)
{
    clear_error();
    if (!eng) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    const FockSchedule& S = reinterpret_cast<const Engine*>(eng)->sched;
    int nf = 0, np = 0;
    for (const auto& g : S.graphs) nf += g.exec ? 1 : 0;
    for (const auto& g : S.purify) np += g.exec ? 1 : 0;
    if (fock_graphs) *fock_graphs = nf;
    if (purification_graphs) *purification_graphs = np;
    if (replays) *replays = S.graph_replays;
    return HF_OK;
}

int hf_engine_fock_schedule(const hf_engine* eng, int max_class_pairs, int* num_class_pairs, int* cap_fp64,
                            int* cap_fp32, int* branch)
{
    clear_error();
    if (!eng || !num_class_pairs) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    const Engine& e = *reinterpret_cast<const Engine*>(eng);
    const FockSchedule& S = e.sched;
    const int ncp = static_cast<int>(e.class_pairs.size());
    *num_class_pairs = ncp;
    const int nb = std::max(1, std::min(S.nbranch, kMaxBranches));
    for (int c = 0; c < ncp && c < max_class_pairs; ++c) {
        if (cap_fp64) cap_fp64[c] = (c < static_cast<int>(S.cap64.size()) && S.cap64[c] > 0) ? S.cap64[c] : kFockBlocksPerSm;
        if (cap_fp32) cap_fp32[c] = (c < static_cast<int>(S.cap32.size()) && S.cap32[c] > 0) ? S.cap32[c] : kFockBlocksPerSm;
        if (branch) branch[c] = nb == 1 ? 0 : (c < static_cast<int>(S.branch_of.size()) ? S.branch_of[c] : c) % nb;
    }
    return HF_OK;
}

int hf_compute_eri_matrix(hf_engine* eng, double* d_eri, void* stream)
{
    clear_error();
    if (!eng || !d_eri) return set_error("null argument"), HF_ERR_INVALID_ARGUMENT;
    return compute_eri_tensor(*reinterpret_cast<Engine*>(eng), d_eri, static_cast<cudaStream_t>(stream));
}

int hf_compute_fock_stored_rhf(const double* d_density, const double* d_core_hamiltonian, const double* d_eri,
                               double* d_fock, int num_basis, void* stream)
{
    clear_error();
    if (!d_density || !d_core_hamiltonian || !d_eri || !d_fock || num_basis <= 0)
        return set_error("null argument or bad size"), HF_ERR_INVALID_ARGUMENT;
    return stored_fock(d_density, d_core_hamiltonian, d_eri, d_fock, num_basis, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
