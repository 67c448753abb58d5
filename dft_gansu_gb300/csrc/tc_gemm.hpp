// Split-BF16 GEMM on the 5th-generation tensor cores (tcgen05.mma with TMEM
// accumulators, TMA tile loads, an mbarrier pipeline).
//
//   C[m][n] = sum_k A[m][k] B[n][k],  A = A_hi + A_lo,  B = B_hi + B_lo (BF16 planes)
//
// evaluated as A_hi B_hi + A_hi B_lo + A_lo B_hi with FP32 accumulation: about
// 17 significant bits per product, the dropped A_lo B_lo term is 2^-16 of it.
// Operands are row-major with K contiguous (K-major for the MMA), each plane
// with a row pitch that is a multiple of 64 elements (128 bytes), so that every
// TMA box starts on a 128-byte boundary.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace gb {

enum SplitGemmMode {
    kSplitStore = 0,      // out_hi/out_lo[(r % rows_per_block) * ld_out + (r / rows_per_block) * block_cols + col_off + c]
    kSymmetricAdd = 1,    // K[m][n] += alpha C (tiles m <= n only; mirrored into K[n][m])
    kSymmetrizedAdd = 2,  // K[m][n] += alpha C and K[n][m] += alpha C (all tiles): K += alpha (C + C^T)
};

struct SplitGemmArgs {
    // operands: planes of rows x kpad BF16 each (kpad = row pitch, multiple of 64)
    const __nv_bfloat16 *a_hi, *a_lo, *b_hi, *b_lo;
    long long a_rows, b_rows;  // valid rows (m extent, n extent)
    long long kpad;            // row pitch in elements (multiple of 64); columns beyond k_valid are zero
    int mode;
    int split_k;               // K split across CTAs (modes 1 and 2)
    // kSplitStore
    __nv_bfloat16 *out_hi, *out_lo;
    long long rows_per_block;  // r -> (r / rows_per_block, r % rows_per_block)
    long long ld_out;          // row pitch of the output planes
    long long block_cols;      // columns per block in the output
    long long col_off;
    float scale;
    // kSymmetricAdd / kSymmetrizedAdd
    double* K;
    int ldk;
    double alpha;
    int* error_flag;           // set to 1 by a CTA whose pipeline wait timed out
};

// Launches the GEMM on stream s; returns HF_OK or an error status (with hf_last_error set).
int split_bf16_gemm(const SplitGemmArgs& args, int num_sms, cudaStream_t s);

// FP64 rows x cols (row pitch ld_src) -> BF16 hi/lo planes with row pitch ld_dst (zero padded to
// dst_rows x ld_dst); the value is multiplied by scale first.
int split_planes(const double* src, long long rows, long long cols, long long ld_src, double scale,
                 __nv_bfloat16* hi, __nv_bfloat16* lo, long long dst_rows, long long ld_dst, int num_sms,
                 cudaStream_t s);

}  // namespace gb
