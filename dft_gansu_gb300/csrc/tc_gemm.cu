// Split-BF16 GEMM on the tcgen05 tensor cores.  See tc_gemm.hpp for the
// arithmetic; this file holds the kernel and its launcher.
//
// CTA = 128 threads (4 warps), one 128 x BN output tile:
//   warp 0, lane 0  TMA producer: per K block of 64, four boxes (A_hi, A_lo,
//                   B_hi, B_lo) into a STAGES-deep ring, completion counted on
//                   the stage's "full" mbarrier (expect_tx)
//   warp 1, lane 0  MMA issuer: per K block, 4 K-steps x 3 products of
//                   tcgen05.mma.cta_group::1.kind::f16 (M=128, N=BN, K=16,
//                   BF16 in, FP32 accumulate in TMEM); tcgen05.commit frees
//                   the stage ("empty" mbarrier) and finally signals "done"
//   all 4 warps     epilogue: tcgen05.ld of the accumulator (warp w reads TMEM
//                   lanes 32w..32w+31 = tile rows), then the mode's store
//   warp 0          TMEM alloc / dealloc (power of two >= BN columns)
// Shared-memory tiles use the 128-byte swizzle that TMA writes and the UMMA
// descriptors read (8-row atoms of 1024 bytes, SBO = 1024).  Every wait is
// bounded by the global timer (2 s); a CTA that times out sets the error flag,
// skips its epilogue, frees its TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "internal.hpp"
#include "tc_gemm.hpp"
#include "../../include/gansu_gb300.h"

namespace gb {
namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;                    // BF16 elements per K block = 128 bytes = swizzle span
constexpr unsigned long long kWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait on the phase with the given parity; false after kWaitNs
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row atoms 1024 bytes apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);  // start address (bits 0-13)
    d |= static_cast<uint64_t>(1024u >> 4) << 32;         // stride byte offset (bits 32-45)
    d |= static_cast<uint64_t>(1u) << 46;                 // descriptor version (bits 46-47)
    d |= static_cast<uint64_t>(2u) << 61;                 // layout: 128-byte swizzle (bits 61-63)
    return d;
}

// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 accumulator, M = 128, N = BN
template <int BN>
__host__ __device__ constexpr uint32_t idesc_bf16()
{
    return (1u << 4)                                  // D format F32
           | (1u << 7)                                // A format BF16
           | (1u << 10)                               // B format BF16
           | (static_cast<uint32_t>(BN >> 3) << 17)   // N >> 3
           | (static_cast<uint32_t>(kBM >> 4) << 24); // M >> 4
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct TmaMaps {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
};

template <int BN, int STAGES>
struct GemmSmem {
    static constexpr int kATile = kBM * kBK * 2;  // bytes of one A plane tile
    static constexpr int kBTile = BN * kBK * 2;
    static constexpr int kStage = 2 * kATile + 2 * kBTile;
    static constexpr int kBytes = STAGES * kStage + 1024 /* alignment */ + 256 /* barriers, TMEM slot */;
    static constexpr int kTmemCols = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(128, 1)
split_gemm_kernel(const __grid_constant__ TmaMaps maps, const SplitGemmArgs a)
{
    using S = GemmSmem<BN, STAGES>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * S::kStage);
    uint64_t* empty = full + STAGES;
    uint64_t* done = empty + STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    __shared__ int s_fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- tile and K range
    long long tm, tn;
    int z = blockIdx.z;
    if (a.mode == kSymmetricAdd) {
        long long p = blockIdx.x, t = 0, T = (a.a_rows + kBM - 1) / kBM;
        while (p >= T - t) { p -= T - t; ++t; }
        tm = t;
        tn = t + p;
    } else {
        tm = blockIdx.x;
        tn = blockIdx.y;
    }
    const long long m0 = tm * kBM, n0 = tn * BN;
    const int nkb_total = static_cast<int>(a.kpad / kBK);
    const int splits = (a.mode == kSplitStore) ? 1 : a.split_k;
    const int kb0 = static_cast<int>(static_cast<long long>(nkb_total) * z / splits);
    const int kb1 = static_cast<int>(static_cast<long long>(nkb_total) * (z + 1) / splits);
    const int nk = kb1 - kb0;

    if (threadIdx.x == 0) {
        s_fail = 0;
        for (int i = 0; i < STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(static_cast<uint32_t>(S::kTmemCols)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (nk > 0) {
        if (warp == 0 && lane == 0) {
            // ---- TMA producer
            for (int i = 0; i < nk; ++i) {
                const int st = i % STAGES;
                const uint32_t round = static_cast<uint32_t>(i / STAGES);
                if (!mbar_wait(&empty[st], (round & 1u) ^ 1u)) { atomicExch(&s_fail, 1); break; }
                uint8_t* base = smem + st * S::kStage;
                mbar_expect_tx(&full[st], S::kStage);
                const int kx = (kb0 + i) * kBK;  // multiple of 64 elements = 128 bytes
                tma_load_2d(base, &maps.a_hi, &full[st], kx, static_cast<int>(m0));
                tma_load_2d(base + S::kATile, &maps.a_lo, &full[st], kx, static_cast<int>(m0));
                tma_load_2d(base + 2 * S::kATile, &maps.b_hi, &full[st], kx, static_cast<int>(n0));
                tma_load_2d(base + 2 * S::kATile + S::kBTile, &maps.b_lo, &full[st], kx, static_cast<int>(n0));
            }
        } else if (warp == 1 && lane == 0) {
            // ---- MMA issuer
            constexpr uint32_t idesc = idesc_bf16<BN>();
            for (int i = 0; i < nk; ++i) {
                const int st = i % STAGES;
                const uint32_t round = static_cast<uint32_t>(i / STAGES);
                if (!mbar_wait(&full[st], round & 1u)) { atomicExch(&s_fail, 1); break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t base = smem_u32(smem + st * S::kStage);
                const uint64_t ah = sw128_desc(base), al = sw128_desc(base + S::kATile);
                const uint64_t bh = sw128_desc(base + 2 * S::kATile), bl = sw128_desc(base + 2 * S::kATile + S::kBTile);
#pragma unroll
                for (int k = 0; k < kBK / 16; ++k) {
                    const uint64_t dk = static_cast<uint64_t>(k * 32 >> 4);  // 16 BF16 = 32 bytes per K step
                    umma_bf16(tmem, ah + dk, bh + dk, idesc, (i > 0 || k > 0) ? 1u : 0u);
                    umma_bf16(tmem, ah + dk, bl + dk, idesc, 1u);
                    umma_bf16(tmem, al + dk, bh + dk, idesc, 1u);
                }
                umma_commit(&empty[st]);
            }
            umma_commit(done);
        }
        // ---- epilogue (all warps)
        __syncwarp();
        const bool ok = mbar_wait(done, 0u);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!ok) atomicExch(&s_fail, 1);
        __syncthreads();
        if (!s_fail) {
            const int row = warp * 32 + lane;
            const long long m = m0 + row;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                float v[32];
                tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0), v);
                if (m >= a.a_rows) continue;
                if (a.mode == kSplitStore) {
                    const long long blk = m / a.rows_per_block, r = m % a.rows_per_block;
                    __nv_bfloat16* oh = a.out_hi + r * a.ld_out + blk * a.block_cols + a.col_off + n0 + c0;
                    __nv_bfloat16* ol = a.out_lo + r * a.ld_out + blk * a.block_cols + a.col_off + n0 + c0;
                    const long long valid = a.b_rows - (n0 + c0);
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        __align__(16) __nv_bfloat16 h8[8], l8[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const float x = v[8 * g + j] * a.scale;
                            const __nv_bfloat16 h = __float2bfloat16_rn(x);
                            h8[j] = h;
                            l8[j] = __float2bfloat16_rn(x - __bfloat162float(h));
                        }
                        if (valid >= 8 * g + 8) {
                            *reinterpret_cast<uint4*>(oh + 8 * g) = *reinterpret_cast<const uint4*>(h8);
                            *reinterpret_cast<uint4*>(ol + 8 * g) = *reinterpret_cast<const uint4*>(l8);
                        } else {
                            for (int j = 0; j < 8 && 8 * g + j < valid; ++j) {
                                oh[8 * g + j] = h8[j];
                                ol[8 * g + j] = l8[j];
                            }
                        }
                    }
                } else {
#pragma unroll 4
                    for (int j = 0; j < 32; ++j) {
                        const long long n = n0 + c0 + j;
                        if (n >= a.b_rows) break;
                        const double x = a.alpha * static_cast<double>(v[j]);
                        if (a.mode == kSymmetrizedAdd) {
                            atomicAdd(&a.K[m * a.ldk + n], x);
                            atomicAdd(&a.K[n * a.ldk + m], x);
                        } else if (tm != tn) {
                            atomicAdd(&a.K[m * a.ldk + n], x);
                            atomicAdd(&a.K[n * a.ldk + m], x);
                        } else if (n >= m) {  // diagonal tile: upper half, mirrored, so K is exactly symmetric
                            atomicAdd(&a.K[m * a.ldk + n], x);
                            if (n != m) atomicAdd(&a.K[n * a.ldk + m], x);
                        }
                    }
                }
            }
        } else if (threadIdx.x == 0 && a.error_flag) {
            atomicExch(a.error_flag, 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(static_cast<uint32_t>(S::kTmemCols)));
    }
}

__global__ void split_planes_kernel(const double* __restrict__ src, long long rows, long long cols, long long ld_src,
                                    double scale, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                    long long dst_rows, long long ld_dst)
{
    const long long total = dst_rows * ld_dst;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long r = k / ld_dst, c = k % ld_dst;
        float x = 0.f;
        double xd = 0.0;
        if (r < rows && c < cols) xd = src[r * ld_src + c] * scale;
        x = static_cast<float>(xd);
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        hi[k] = h;
        lo[k] = __float2bfloat16_rn(static_cast<float>(xd - static_cast<double>(__bfloat162float(h))));
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

int make_map(CUtensorMap* m, const __nv_bfloat16* base, long long rows, long long kpad, int box_rows)
{
    auto fn = encode_fn();
    if (!fn) return set_error("cuTensorMapEncodeTiled is not available"), HF_ERR_CUDA;
    if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (kpad % kBK) != 0)
        return set_error("split GEMM operand not 16-byte aligned or pitch not a multiple of 64"), HF_ERR_INVALID_ARGUMENT;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(kpad), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(kpad) * 2};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(kBK), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error("cuTensorMapEncodeTiled failed: " + std::to_string(static_cast<int>(r))), HF_ERR_CUDA;
    return HF_OK;
}

template <int BN, int STAGES>
int launch(const SplitGemmArgs& a, cudaStream_t s)
{
    using S = GemmSmem<BN, STAGES>;
    TmaMaps maps;
    int st;
    if ((st = make_map(&maps.a_hi, a.a_hi, a.a_rows, a.kpad, kBM)) || (st = make_map(&maps.a_lo, a.a_lo, a.a_rows, a.kpad, kBM)) ||
        (st = make_map(&maps.b_hi, a.b_hi, a.b_rows, a.kpad, BN)) || (st = make_map(&maps.b_lo, a.b_lo, a.b_rows, a.kpad, BN)))
        return st;
    static bool attr_set = false;
    if (!attr_set) {
        GB_CUDA_TRY(cudaFuncSetAttribute(split_gemm_kernel<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         S::kBytes));
        attr_set = true;
    }
    const long long tiles_m = (a.a_rows + kBM - 1) / kBM, tiles_n = (a.b_rows + BN - 1) / BN;
    dim3 grid;
    if (a.mode == kSplitStore) {
        grid = dim3(static_cast<unsigned>(tiles_m), static_cast<unsigned>(tiles_n), 1);
    } else if (a.mode == kSymmetricAdd) {
        grid = dim3(static_cast<unsigned>(tiles_m * (tiles_m + 1) / 2), 1, static_cast<unsigned>(a.split_k));
    } else {
        grid = dim3(static_cast<unsigned>(tiles_m), static_cast<unsigned>(tiles_n), static_cast<unsigned>(a.split_k));
    }
    split_gemm_kernel<BN, STAGES><<<grid, 128, S::kBytes, s>>>(maps, a);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

}  // namespace

int split_bf16_gemm(const SplitGemmArgs& a, int num_sms, cudaStream_t s)
{
    (void)num_sms;
    if (a.a_rows <= 0 || a.b_rows <= 0 || a.kpad <= 0) return HF_OK;
    if (a.a_rows > 0x7fffffffLL || a.b_rows > 0x7fffffffLL)
        return set_error("split GEMM: more rows than a TMA coordinate holds"), HF_ERR_INVALID_ARGUMENT;
    if (a.mode == kSplitStore) {
        if ((a.ld_out % 8) || (a.block_cols % 8) || (a.col_off % 8))
            return set_error("split GEMM store: output pitch/offsets must be multiples of 8"), HF_ERR_INVALID_ARGUMENT;
        const long long nblk = (a.a_rows + a.rows_per_block - 1) / a.rows_per_block;
        if (a.rows_per_block <= 0 || a.col_off + a.b_rows > a.block_cols || nblk * a.block_cols > a.ld_out)
            return set_error("split GEMM store: output block layout does not hold the product"), HF_ERR_INVALID_ARGUMENT;
        return launch<192, 2>(a, s);
    }
    if (a.a_rows != a.b_rows || a.ldk < a.a_rows)
        return set_error("split GEMM add: needs a square output with ldk >= rows"), HF_ERR_INVALID_ARGUMENT;
    if (a.split_k < 1 || a.split_k > static_cast<int>(a.kpad / kBK))
        return set_error("split GEMM: split_k out of range"), HF_ERR_INVALID_ARGUMENT;
    return launch<128, 3>(a, s);
}

int split_planes(const double* src, long long rows, long long cols, long long ld_src, double scale,
                 __nv_bfloat16* hi, __nv_bfloat16* lo, long long dst_rows, long long ld_dst, int num_sms,
                 cudaStream_t s)
{
    const long long total = dst_rows * ld_dst;
    const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>((total + 255) / 256, num_sms * 32LL)));
    split_planes_kernel<<<grid, 256, 0, s>>>(src, rows, cols, ld_src, scale, hi, lo, dst_rows, ld_dst);
    GB_LAUNCH_CHECK();
    return HF_OK;
}

}  // namespace gb

namespace gb {
namespace {
__global__ void recombine_kernel(const __nv_bfloat16* __restrict__ hi, const __nv_bfloat16* __restrict__ lo,
                                 long long rows, long long cols, long long ld, double* __restrict__ C)
{
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < rows * cols;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long r = k / cols, c = k % cols;
        C[k] = static_cast<double>(__bfloat162float(hi[r * ld + c])) + static_cast<double>(__bfloat162float(lo[r * ld + c]));
    }
}
}  // namespace
}  // namespace gb

extern "C" int hf_split_bf16_matmul(const double* d_a, const double* d_b, double* d_c, int m, int n, int k, int mode,
                                    void* stream)
{
    using namespace gb;
    clear_error();
    if (!d_a || !d_c || m <= 0 || n <= 0 || k <= 0 || mode < 0 || mode > 2 || (mode != 1 && !d_b))
        return set_error("hf_split_bf16_matmul: bad argument"), HF_ERR_INVALID_ARGUMENT;
    if (mode != 0 && m != n) return set_error("hf_split_bf16_matmul: modes 1 and 2 need m == n"), HF_ERR_INVALID_ARGUMENT;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long kpad = (k + 63) / 64 * 64, npad = (n + 7) / 8 * 8;
    __nv_bfloat16 *ah = nullptr, *al = nullptr, *bh = nullptr, *bl = nullptr, *oh = nullptr, *ol = nullptr;
    int* flag = nullptr;
    int st = HF_OK;
    auto alloc = [&](void** p, size_t bytes) {
        if (st == HF_OK && cudaMalloc(p, bytes) != cudaSuccess) st = (set_error("cudaMalloc failed"), HF_ERR_OUT_OF_MEMORY);
    };
    alloc(reinterpret_cast<void**>(&ah), sizeof(__nv_bfloat16) * m * kpad);
    alloc(reinterpret_cast<void**>(&al), sizeof(__nv_bfloat16) * m * kpad);
    alloc(reinterpret_cast<void**>(&bh), sizeof(__nv_bfloat16) * n * kpad);
    alloc(reinterpret_cast<void**>(&bl), sizeof(__nv_bfloat16) * n * kpad);
    alloc(reinterpret_cast<void**>(&flag), sizeof(int));
    if (mode == 0) {
        alloc(reinterpret_cast<void**>(&oh), sizeof(__nv_bfloat16) * m * npad);
        alloc(reinterpret_cast<void**>(&ol), sizeof(__nv_bfloat16) * m * npad);
    }
    if (st == HF_OK) st = split_planes(d_a, m, k, k, 1.0, ah, al, m, kpad, sms, s);
    if (st == HF_OK) st = split_planes(mode == 1 ? d_a : d_b, n, k, k, 1.0, bh, bl, n, kpad, sms, s);
    if (st == HF_OK && cudaMemsetAsync(flag, 0, sizeof(int), s) != cudaSuccess) st = HF_ERR_CUDA;
    if (st == HF_OK) {
        SplitGemmArgs a{};
        a.a_hi = ah; a.a_lo = al; a.b_hi = bh; a.b_lo = bl;
        a.a_rows = m; a.b_rows = n; a.kpad = kpad;
        a.mode = mode;
        a.error_flag = flag;
        if (mode == 0) {
            a.out_hi = oh; a.out_lo = ol;
            a.rows_per_block = m; a.ld_out = npad; a.block_cols = npad; a.col_off = 0; a.scale = 1.0f;
        } else {
            if (cudaMemsetAsync(d_c, 0, sizeof(double) * m * n, s) != cudaSuccess) st = HF_ERR_CUDA;
            a.K = d_c; a.ldk = n; a.alpha = 1.0;
            a.split_k = static_cast<int>(std::min<long long>(4, kpad / 64));
        }
        if (st == HF_OK) st = split_bf16_gemm(a, sms, s);
        if (st == HF_OK && mode == 0) {
            recombine_kernel<<<256, 256, 0, s>>>(oh, ol, m, n, npad, d_c);
            if (cudaGetLastError() != cudaSuccess) st = (set_error("recombine launch failed"), HF_ERR_CUDA);
        }
    }
    int h_flag = 0;
    if (cudaStreamSynchronize(s) != cudaSuccess && st == HF_OK) st = (set_error("split GEMM execution failed"), HF_ERR_CUDA);
    if (flag) cudaMemcpy(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost);
    for (void* p : {static_cast<void*>(ah), static_cast<void*>(al), static_cast<void*>(bh), static_cast<void*>(bl),
                    static_cast<void*>(oh), static_cast<void*>(ol), static_cast<void*>(flag)})
        if (p) cudaFree(p);
    if (st == HF_OK && h_flag) st = (set_error("split GEMM pipeline wait timed out"), HF_ERR_CUDA);
    return st;
}
