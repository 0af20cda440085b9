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
  float2 *dF[kMaxStages];  // dF[1 .. s-2]: the stages' right-hand-side increments
  DevState *st;
  Bruss bruss;
  int path;                // FP32 stages: kMixTilesTma (tm valid) or kMixTiles
  CUtensorMap tm[kMixTmaStages];
};

// How the FP32 stages load their 8 x 32 tiles (with a one-point halo in
// shared memory): TMA boxes, double-buffered, or plain loads.
constexpr int kMixTilesTma = 1, kMixTiles = 2;

// Launches the persistent mixed kernel with the given kMix* path (kMixTilesTma
// falls back to kMixTiles where TMA boxes do not fit: odd N or more than
// kMixTmaStages stages).
cudaError_t launch_mixed(const MixedParams &p, int path, int num_sms, cudaStream_t stream,
                         int *grid_out);

}  // namespace rkcu
