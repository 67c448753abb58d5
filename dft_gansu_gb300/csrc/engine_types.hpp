// Device-side data layout of the engine (HBM-resident for the engine's life).
//
//   contracted shell pairs   ShellPairDev[npairs]    grouped by pair class, each
//                            class sorted by the contracted bound Qs descending
//   primitive pairs          PrimPair64[] + PrimPair32[] (same order), per shell
//                            pair a contiguous run [pp_off, pp_off + pp_n)
//   quartet work entries     per class pair: entry_bra[], entry_lo[], off[]
//                            (exclusive prefix over the per-bra ket counts)
//   Boys table               double[32][1281] and float copy, x = k/32
//   J', K' accumulators      double N x N each; D' = s D s in double and float
#pragma once
#include <cstdint>

namespace gb {

// One contracted shell pair (A,B), l_A >= l_B (A >= B when l_A == l_B).  The
// records are 16-byte aligned so that a whole-record copy in a kernel moves as
// 16-byte vector loads (the gathers of pair and primitive-pair records are the
// latency the integral kernels wait on).
struct alignas(16) ShellPairDev {
    int A, B;          // contracted shell indices
    int bfA, bfB;      // first basis function of each shell
    int pp_off, pp_n;  // primitive-pair run
    int la, lb;
    double ABx, ABy, ABz;  // A - B
    double Qmax;           // max primitive-pair Schwarz bound (reference definition)
    double Qs;             // sum of primitive-pair bounds (bounds the contracted integral)
    int mbase;             // molecule block: D/J/K element (a, b) of this pair's molecule is at
    int mn;                //   mbase + a * mn + b (a single molecule: mbase = 0, mn = N)
    float fABx, fABy, fABz, fQmax;  // FP32-tier copies (no conversions in FP32 kernels)
};
static_assert(sizeof(ShellPairDev) == 96, "ShellPairDev layout");

// One primitive pair of a shell pair.  K carries the contraction coefficients,
// the component-independent part of the primitive norms, exp(-ab/p |AB|^2)
// and sqrt(2 pi^{5/2}); KoP = K/p, so that a primitive quartet prefactor is
// KoP_ab KoP_cd / sqrt(p+q).  b is the exponent of the second primitive
// (kinetic-energy integrals).
struct alignas(16) PrimPair64 {
    double p, invp, K, KoP, Q;
    double Px, Py, Pz;
    double PAx, PAy, PAz;
    double b;
};
struct alignas(16) PrimPair32 {
    float p, invp, K, KoP, Q;
    float Px, Py, Pz;
    float PAx, PAy, PAz;
    float b;
};
static_assert(sizeof(PrimPair32) == 48 && sizeof(PrimPair64) == 96, "primitive-pair layouts");

struct FockClassLaunch {
    const ShellPairDev* pairs;     // all shell pairs (global indices)
    const void* prim_pairs;        // PrimPair64* or PrimPair32*
    const void* boys_table;        // double* or float*
    const void* density;           // D' (double* or float*), N x N
    double* J;                     // J' accumulator
    double* K;                     // K' accumulator
    float* J32;                    // FP32-tier accumulators
    float* K32;
    const long long* off;          // nentry+1 prefix offsets
    const int* entry_bra;          // global bra pair index per entry
    const int* entry_lo;           // first ket (class-relative) per entry
    const int* entry_prim = nullptr;  // bra primitive pairs [first, end) per entry as first | (end << 16);
                                      // null: all of the bra's primitive pairs
    int nentry;
    int ket_base;                  // global index of the ket class's first pair
    int num_basis;
    double schwarz_threshold;
    unsigned long long* counters;  // [0] primitive quartets, [1] contracted quartets
    const float* block_dmax;       // incremental builds: max |dD| per shell block [A * nshell + B], or null
    int nshell;
    double skip_cut;               // skip when Qs_ab * Qs_cd * block max < skip_cut
    const unsigned char* mol_active;  // batches: molecules still iterating (null = all)
    const int* shell_mol;             // contracted shell -> molecule
};

}  // namespace gb
