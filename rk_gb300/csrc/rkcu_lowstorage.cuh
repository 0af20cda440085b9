// Low-storage (pipelined wavefront) step loop for BRUSS2D-MIX.
#pragma once

#include "rkcu_device.cuh"

namespace rkcu {

struct LsParams {
  int N, R, nb;                  // grid size, rows per block, blocks
  unsigned long long inv_n;      // floor(2^40 / N) + 1: q / N = (q * inv_n) >> 40 for q < R N
  int s, ord, step_limit, budget, nblocks, extra_arrivals;
  double te, tol;
  unsigned long long timeout_ns;
  double A[kMaxStages * kMaxStages];
  double b[kMaxStages], bh[kMaxStages];
  unsigned char nzA[kMaxStages * kMaxStages];
  unsigned char nzb[kMaxStages], nzbh[kMaxStages];
  double2 *y[2];
  double2 *ring[kMaxStages];     // ring[l], l = 1..s-1: 2l+2 block slots of R N pairs
  double2 *dyring, *errring;     // 2s-1 block slots each
  DevState *st;
  Bruss bruss;
  unsigned int *flags;           // per-CTA progress (zeroed by each launch), gridDim.x words
  int sync;                      // 0: neighbour flags between wavefront steps, 1: grid barrier
};

cudaError_t launch_lowstorage(const LsParams &p, bool exact, int num_sms, cudaStream_t stream,
                              int *grid_out);
// pairs of ring storage for s stages, R rows per block, grid size N
size_t lowstorage_ring_pairs(int s, int R, int N);

}  // namespace rkcu
