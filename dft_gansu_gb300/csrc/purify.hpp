// RHF density by purification (purify.cu): the fused single-launch path and the
// status words both purification paths leave for the SCF to check.
#pragma once
#include <cuda_runtime.h>

namespace gb {

struct Engine;

constexpr int kPurifyMaxN = 512;        // fused path: panels of 16 rows x N in shared memory
constexpr int kPurifyMaxSteps = 100;    // SP2 steps at most
// status words (doubles) at the start of the engine's purification scratch
constexpr int kPurifyStatusSteps = 0;        // SP2 steps taken
constexpr int kPurifyStatusTraceError = 1;   // tr(P) - nocc after McWeeny
constexpr int kPurifyStatusIdempotency = 2;  // |tr(P) - |P|_F^2| after McWeeny
constexpr int kPurifyStatusSp2Error = 3;     // |tr(P) - |P|_F^2| when SP2 stopped
constexpr int kPurifyStatusSp2Converged = 4; // 1: SP2 met its stopping rule
constexpr int kPurifyStatusMcWeeny = 5;      // McWeeny steps taken
constexpr int kPurifyStatusFlags = 6;        // nonzero: a grid-barrier wait ran out
constexpr int kPurifyStatusBarriers = 7;     // grid barriers passed (fused path)
constexpr int kPurifyStatusPhase = 8;        // fused path, CTA 0: microseconds from the start to the end of
                                             // F' (+0), P0 (+1), SP2 (+2), McWeeny (+3), X P (+4), D (+5)
constexpr int kPurifyStatusWords = 16;
// acceptance of a purified projector (else the SCF reruns with a diagonalisation)
constexpr double kPurifyTraceTol = 1e-6;
constexpr double kPurifyIdempotencyTol = 1e-8;

bool purify_fused_supported(const Engine& e);
// D = 2 X P X^T from F (the engine's SCF workspace: X, T1, T2, W = the projector)
// max_steps: SP2 steps at most (<= 0: kPurifyMaxSteps)
int purify_fused(Engine& e, const double* F, int nocc, double* D, cudaStream_t s, int max_steps);
// device address of the status words (allocates the scratch on first use)
int purify_status(Engine& e, double** status);

}  // namespace gb
