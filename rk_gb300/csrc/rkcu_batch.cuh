// Batched / served step loop: many independent instances, each with its own
// size, parameters, step size and tolerance, advanced together in sweeps.
#pragma once

#include "rkcu_device.cuh"

namespace rkcu {

// One instance slot (device memory).  The host fills it when it admits an
// instance; the kernel's step-control phase updates it.
struct InstDesc {
  int kind;          // RKCU_PROBLEM_*
  int n, npairs;
  int grid_n;        // BRUSS2D-MIX
  double coef;       // BRUSS2D-MIX (alpha (N-1)) (N-1)
  const double *lv_r, *lv_a;  // banded LV parameters (arena)
  double2 *vec;      // y[0], y[1], w[1..s-1], dy, err: s+3 vectors of npairs double2 (arena)
  double t, h, te, tol;
  int steps_acc, steps_rej, cur, done, active, step_limit;
  long long host_id;            // caller's id, returned with the result
  unsigned long long errbits;   // error max of the running step (bit pattern, >= 0)
  // A step whose size update waits for the C library's pow on the host (the
  // accept/reject decision, t and the counters are applied): the instance sits
  // out the sweeps until the host's answer with sequence number pend_seq is in
  // its PowBox.
  int pending;
  unsigned int pend_seq;
};


// h*A, h*b, h*(b - b^) of the running step, one per slot (device memory)
struct InstCoef {
  double hA[kMaxStages * kMaxStages];
  double hb[kMaxStages], hbh[kMaxStages];
};

struct BatchParams {
  int s, ord;
  double A[kMaxStages * kMaxStages];
  double b[kMaxStages], bh[kMaxStages];
  unsigned char nzA[kMaxStages * kMaxStages];
  unsigned char nzb[kMaxStages], nzbh[kMaxStages];
  InstDesc *desc;
  InstCoef *coef;
  int *nslots;         // slots [0, *nslots) may be active (device, so a captured graph stays valid)
  int2 *chunks;        // (slot, first pair) of every chunk of every active instance
  int *nchunks;
  int chunk_pairs;     // pairs per chunk (the tuned length)
  int *chunk_len;      // pairs per chunk of the current list (device; at most chunk_pairs)
  int *rebuild;        // set when an instance finished during a sweep
  int *done_list;      // slots that finished, in order
  int *done_count;
  int *budget;         // sweeps per launch (device, so that one captured graph serves every
                       // count; a sweep = one attempted step of every active instance)
  int nblocks;
  unsigned long long timeout_ns;
  DevState *st;        // barrier words and error flag
  PowBox *pow_box;     // one mailbox per slot (device view of mapped host memory)
};

cudaError_t launch_batch_rebuild(const BatchParams &p, cudaStream_t stream);
cudaError_t launch_batch(const BatchParams &p, bool exact, int threads, int blocks_per_sm,
                         int num_sms, cudaStream_t stream, int *grid_out);
// grid size launch_batch would use (for graph capture and tuning)
int batch_grid(bool exact, int threads, int blocks_per_sm, int num_sms);

}  // namespace rkcu
