// Plain FP64 form: one persistent cooperative kernel runs whole steps of the
// embedded RK method (stage combine, right-hand side, embedded error, error
// norm, accept/reject) with the step control on the device.
#pragma once

#include "rkcu_device.cuh"

namespace rkcu {

struct PlainParams {
  int npairs;        // number of component pairs (ceil(n/2))
  int n;
  int s, ord;
  int problem;       // RKCU_PROBLEM_*
  int step_limit;    // 0 = none
  int budget;        // attempted steps this launch at most
  int nblocks;
  int extra_arrivals;  // test hook: phantom CTAs the barrier waits for
  double te, tol;
  unsigned long long timeout_ns;
  double A[kMaxStages * kMaxStages];  // row-major, strictly lower
  double b[kMaxStages];
  double bh[kMaxStages];              // b - b_hat (src/impl/seq/D.c:40-41)
  unsigned char nzA[kMaxStages * kMaxStages];
  unsigned char nzb[kMaxStages], nzbh[kMaxStages];
  double2 *y[2];                      // current / candidate state (ping-pong)
  double2 *w[kMaxStages];             // w[1..s-1]
  double2 *dy, *err;
  DevState *st;
  unsigned int *flags;                // progress words (reset by each launch): kMaxPlainGrid
                                      // CTA words, or the flow schedule's 2 tickets + tiles
  int schedule;                       // kScheduleGrid, kScheduleNeighbour, kScheduleFlow or
                                      // kScheduleRowRing
  int flow_tile;                      // flow schedule: pairs per tile
  int flow_ntiles;                    //   tiles per stage
  int flow_dep;                       //   tiles either side a stage's stencil reads
  int flow_skew;                      //   K: stage i runs K tiles behind stage i-1
  // per-step trace (include/tools.h:239-256, -DDUMP): for attempted step k <
  // trace_cap, trace_meta[3k..3k+2] = t, h, error max and, if trace_y is set,
  // trace_y[k * npairs ..] = the step's candidate state
  int trace_cap;
  double *trace_meta;
  double2 *trace_y;
  // Mailbox for step-size updates left to the host (device view of mapped host
  // memory), set only while the host polls it; null: such an update ends the
  // launch and the host finishes it before the next one.
  PowBox *pow_box;
  Bruss bruss;
  LvPairs lvp;
  LvBanded lvb;
};

// Largest grid the plain kernel uses (the progress words are sized for it).
constexpr int kMaxPlainGrid = 2048;
// Stage synchronisation of the plain kernel: a grid barrier after every stage
// (grid-stride work), per-CTA ranges with neighbour progress flags, or a
// dataflow over (stage, tile) tickets in wavefront order (one grid barrier per
// step; the window of live rows stays in L2).
constexpr int kScheduleGrid = 1;
constexpr int kScheduleNeighbour = 2;
constexpr int kScheduleFlow = 3;
// Neighbour progress flags between stages, with each stage input's grid rows
// staged in shared memory by bulk copies (BRUSS2D-MIX; one CTA per SM).
constexpr int kScheduleRowRing = 4;
// Largest grid the row ring holds (kRingSlots rows of N pairs in 227 KB).
constexpr int kRowRingMaxN = 3600;
// Progress words the flow schedule needs for ntiles tiles.
inline size_t flow_words(int ntiles) { return 2 + static_cast<size_t>(ntiles); }

// Launches one persistent kernel (cooperative) for up to p.budget steps.
// mode: kArithFused, kArithExact or kArithExactSoftMul
cudaError_t launch_plain(const PlainParams &p, int mode, int blocks_per_sm, int num_sms,
                         cudaStream_t stream, int *grid_out);

// Device RHS over all pairs of y (exact arithmetic), for ode_eval_rng.
cudaError_t launch_eval_rhs(int problem, const Bruss &bruss, const LvBanded &lvb, int npairs,
                            const double2 *y, double2 *f, cudaStream_t stream);

// Host side: record the text rkcu_last_cuda_error() returns for a failed CUDA
// call (returns RKCU_ERR_NOMEM or RKCU_ERR_CUDA) or for a device wait that ran
// out at `site` (returns RKCU_ERR_TIMEOUT).
int record_cuda_error(cudaError_t e, const char *what);
int record_wait_timeout(int site);

// Step-size updates on the device (count values), for tests of the controller.
cudaError_t launch_step_sizes(const double *h, const double *err, int count, double tol, int ord,
                              double *out, cudaStream_t stream);

}  // namespace rkcu
