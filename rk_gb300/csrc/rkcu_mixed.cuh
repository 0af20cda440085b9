// Mixed-precision step loop (FP32 stage vectors, FP64 state and norm), BRUSS2D-MIX.
#pragma once

#include "rkcu_device.cuh"

namespace rkcu {

struct MixedParams {
  int npairs, n, s, ord, step_limit, budget, nblocks, extra_arrivals;
  double te, tol;
  unsigned long long timeout_ns;
  double A[kMaxStages * kMaxStages];
  double b[kMaxStages], bh[kMaxStages], csum[kMaxStages];  // csum_i = sum_j a_ij
  double bsum, bhsum;                                       // sum b, sum (b - b^)
  unsigned char nzA[kMaxStages * kMaxStages];
  double2 *y[2];
  float2 *f0, *y32, *S[kMaxStages], *dys, *dyc, *err;
  DevState *st;
  Bruss bruss;
};

cudaError_t launch_mixed(const MixedParams &p, int num_sms, cudaStream_t stream, int *grid_out);

}  // namespace rkcu
