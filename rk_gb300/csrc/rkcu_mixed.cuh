// Mixed-precision step loop (FP32 stage vectors, FP64 state and norm), BRUSS2D-MIX.
#pragma once

#include <cuda.h>  // CUtensorMap

#include "rkcu_device.cuh"

namespace rkcu {

// TMA staging of the FP32 stages (even N, at most kMixTmaStages stages): one
// tensor map per vector, slot 0 = f0, 1 = y32, 1 + j = dF_j.
constexpr int kMixTmaStages = 8;

struct MixedParams {
  int npairs, n, s, ord, step_limit, budget, nblocks, extra_arrivals;
  double te, tol;
  unsigned long long timeout_ns;
  double A[kMaxStages * kMaxStages];
  double b[kMaxStages], bh[kMaxStages], csum[kMaxStages];  // csum_i = sum_j a_ij
  double bsum, bhsum;                                       // sum b, sum (b - b^)
  unsigned char nzA[kMaxStages * kMaxStages];
  double2 *y[2];
  float2 *f0, *y32;
  float2 *f0lo;            // F0 = f0 + f0lo, a double-float pair per component
  float2 *dF[kMaxStages];  // dF[1 .. s-2]: the stages' right-hand-side increments
  DevState *st;
  Bruss bruss;
  int path;                // FP32 stages: kMixTilesTma (tm valid) or kMixTiles
  CUtensorMap tm[kMixTmaStages];
};

// How the FP32 stages run: all stages of a step per 32 x 32 tile in shared
// memory (kMixFused: F0 and y32 with a halo of s-1 points through TMA, even N
// and s <= 8), or one stage at a time over 8 x 32 tiles with a one-point halo,
// their inputs staged by TMA boxes (kMixTilesTma) or plain loads (kMixTiles).
constexpr int kMixTilesTma = 1, kMixTiles = 2, kMixFused = 3;

// Launches the persistent mixed kernel with the given kMix* path (kMixFused
// and kMixTilesTma fall back to kMixTiles where TMA boxes do not fit: odd N or
// more than kMixTmaStages stages).
cudaError_t launch_mixed(const MixedParams &p, int path, int num_sms, cudaStream_t stream,
                         int *grid_out);
// Whether kMixFused runs for an N x N grid and s stages (even N, 2 <= s <= 8,
// TMA available); it needs only the f0 and y32 vectors, not dF_1 .. dF_{s-2}.
bool mixed_fused_available(int N, int s);

}  // namespace rkcu
