// Kernels of the general right-hand-side step loop (see rkcu_general.cuh).
// Every component sees the operations of the reference's A variant in the
// same order; with the exact arithmetic modes the results are bit-identical to
// the fused kernels' (the D variant's scatter accumulates the same sums in the
// same order).
#include "rkcu_general.cuh"

namespace rkcu {

constexpr int kGenThreads = 256;

// include/block-inline.h:76-94
template <int kMode>
__global__ void __launch_bounds__(kGenThreads)
    gen_combine_kernel(const __grid_constant__ GenCoef c, int l, const double *__restrict__ y,
                       const double *__restrict__ F, size_t ld, double *__restrict__ w, long long n) {
  using M = Arith<kMode>;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double acc = y[i];
    if (c.nzA[l * kMaxStages]) acc = M::mac(acc, c.hA[l * kMaxStages], F[i]);
    for (int j = 1; j < l; ++j)
      if (c.nzA[l * kMaxStages + j]) acc = M::mac(acc, c.hA[l * kMaxStages + j], F[j * ld + i]);
    w[i] = acc;
  }
}

// include/block-inline.h:98-134, the update and error max of src/impl/seq/A.c:73-80
template <int kMode>
__global__ void __launch_bounds__(kGenThreads)
    gen_output_kernel(const __grid_constant__ GenCoef c, const double *__restrict__ y,
                      const double *__restrict__ F, size_t ld, double *__restrict__ ynew, long long n,
                      DevState *st) {
  using M = Arith<kMode>;
  __shared__ double s_wmax[kGenThreads / 32];
  ErrMax em;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double err = M::mul(c.hbh[0], F[i]);
    double dy = M::mul(c.hb[0], F[i]);
    for (int j = 1; j < c.s; ++j) {
      if (c.nzbh[j]) err = M::mac(err, c.hbh[j], F[j * ld + i]);
      if (c.nzb[j]) dy = M::mac(dy, c.hb[j], F[j * ld + i]);
    }
    const double yo = y[i];
    const double yn = M::add(yo, dy);
    ynew[i] = yn;
    em.add(err, yn, yo);
  }
  double m = em.value();
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = s_wmax[0];
    for (int k = 1; k < kGenThreads / 32; ++k) b = fmax(b, s_wmax[k]);
    atomicMax(&st->err_slot[st->step & 1], (unsigned long long)__double_as_longlong(b));
  }
}

// include/tools.h:191-198, 235-278, as the fused kernels take it
__global__ void gen_control_kernel(DevState *st, double tol, int ord, double te, int step_limit) {
  const unsigned long long step = st->step;
  const double errmax = __longlong_as_double((long long)st->err_slot[step & 1]);
  st->err_slot[(step + 1) & 1] = 0ull;  // the next step's slot
  double t = st->t, hh = st->h;
  int acc = st->steps_acc, rej = st->steps_rej, cur = st->cur;
  bool host_pow = false;
  if (tol <= 0.0) {
    t += hh;
    ++acc;
    cur ^= 1;
  } else {
    const double hn = h_new(hh, errmax, tol, ord, &host_pow);
    if (errmax <= tol) {
      t += hh;
      ++acc;
      cur ^= 1;
    } else {
      ++rej;
    }
    if (host_pow) {
      st->pend_err = errmax;
      st->pend_h = hh;
    } else {
      hh = hn;
    }
  }
  st->pending = host_pow;
  if (!host_pow) {
    hh = fmin(hh, te - t);
    st->done = !(t < te) || (step_limit > 0 && acc + rej >= step_limit);
  }
  st->t = t;
  st->h = hh;
  st->steps_acc = acc;
  st->steps_rej = rej;
  st->cur = cur;
  st->step = step + 1;
}

static int grid_for(long long n, int num_sms) {
  long long g = (n + kGenThreads - 1) / kGenThreads;
  const long long cap = 8LL * num_sms;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

cudaError_t launch_gen_combine(const GenCoef &c, int l, const double *y, const double *F, size_t ld,
                               double *w, long long n, int mode, int num_sms, cudaStream_t stream) {
  const int g = grid_for(n, num_sms);
  switch (mode) {
    case kArithExact:
      gen_combine_kernel<kArithExact><<<g, kGenThreads, 0, stream>>>(c, l, y, F, ld, w, n);
      break;
    case kArithExactSoftMul:
      gen_combine_kernel<kArithExactSoftMul><<<g, kGenThreads, 0, stream>>>(c, l, y, F, ld, w, n);
      break;
    default:
      gen_combine_kernel<kArithFused><<<g, kGenThreads, 0, stream>>>(c, l, y, F, ld, w, n);
  }
  return cudaGetLastError();
}

cudaError_t launch_gen_output(const GenCoef &c, const double *y, const double *F, size_t ld,
                              double *ynew, long long n, DevState *st, int mode, int num_sms,
                              cudaStream_t stream) {
  const int g = grid_for(n, num_sms);
  switch (mode) {
    case kArithExact:
      gen_output_kernel<kArithExact><<<g, kGenThreads, 0, stream>>>(c, y, F, ld, ynew, n, st);
      break;
    case kArithExactSoftMul:
      gen_output_kernel<kArithExactSoftMul><<<g, kGenThreads, 0, stream>>>(c, y, F, ld, ynew, n, st);
      break;
    default:
      gen_output_kernel<kArithFused><<<g, kGenThreads, 0, stream>>>(c, y, F, ld, ynew, n, st);
  }
  return cudaGetLastError();
}

cudaError_t launch_gen_control(DevState *st, double tol, int ord, double te, int step_limit,
                               cudaStream_t stream) {
  gen_control_kernel<<<1, 1, 0, stream>>>(st, tol, ord, te, step_limit);
  return cudaGetLastError();
}

}  // namespace rkcu
