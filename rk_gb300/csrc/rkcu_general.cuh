// General right-hand sides: the step loop around a device function the caller
// supplies (problems without a limited access distance, which the fused
// kernels cannot stencil).  Gather order of the reference's A variant
// (src/impl/seq/A.c:57-85, include/block-inline.h:76-134): per stage a combine
// kernel forms w_l = y + sum_j h a_lj F_j, the caller evaluates F_l = f(t +
// h c_l, w_l), and after the last stage an output kernel forms dy, err, the
// new y and the error max; a one-thread kernel takes the step decision.
#pragma once

#include "rkcu_device.cuh"

namespace rkcu {

struct GenCoef {
  double hA[kMaxStages * kMaxStages];  // h a_lj, row-major
  double hb[kMaxStages], hbh[kMaxStages];
  unsigned char nzA[kMaxStages * kMaxStages];
  unsigned char nzb[kMaxStages], nzbh[kMaxStages];
  int s;
};

// w = y + sum_{j<l} h a_lj F_j  (F_j at F + j * ld), n components
cudaError_t launch_gen_combine(const GenCoef &c, int l, const double *y, const double *F, size_t ld,
                               double *w, long long n, int mode, int num_sms, cudaStream_t stream);
// dy = sum h b_j F_j, err = sum h (b_j - b^_j) F_j, ynew = y + dy, error max into st->err_slot
cudaError_t launch_gen_output(const GenCoef &c, const double *y, const double *F, size_t ld,
                              double *ynew, long long n, DevState *st, int mode, int num_sms,
                              cudaStream_t stream);
// the step decision of include/tools.h:235-278 on the device (one thread)
cudaError_t launch_gen_control(DevState *st, double tol, int ord, double te, int step_limit,
                               cudaStream_t stream);

}  // namespace rkcu
