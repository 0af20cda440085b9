// Mixed-precision form of the step loop (BRUSS2D-MIX): FP32 stage vectors and
// right-hand-side increments, FP64 state, FP64 update and error-norm reduction.
//
// On GB300 the FP64 pipe (and every FP64<->FP32 conversion) runs at 1/72 of
// the FP32 rate, so the FP32 stages must avoid both.  Per step and component:
//   F0 = f(y)                          FP64 (fused), once per step
//   y1 = y + (h * sum b) * F0           FP64, the large part of the update
//   stage i >= 1:  delta_i = h c_i F0 + S_i,  S_i = sum_{1<=j<i} h a_ij dF_j   (FP32)
//                  dF_i = f(y + delta_i) - F0 = alpha (N-1)^2 lap(delta_i)
//                         + [u^2 v](y + delta) - [u^2 v](y) -/+ 4.4 du / 3.4 du  (FP32)
//     (the Laplacian is linear, and the cubic term is expanded exactly, so the
//      large diffusion coefficient never multiplies FP32 rounding of y itself)
//   dY = sum_{j>=1} h b_j dF_j          FP32, Kahan-compensated across stages
//   e  = sum_{j>=1} h (b_j - b^_j) dF_j FP32 (the F0 terms cancel: sum(b - b^) = 0)
//   y_new = y1 + dY                     FP64
//   err max = max |e| / max(|y_new|, |y_old|): per thread in FP32, reduced in FP64
// c_i is taken as the row sum of A (sum_j a_ij), so sum_j h a_ij F0 = h c_i F0.
// FP64 instructions per component-step: about 12 (RHS 7.5, update 2, two
// conversions) instead of 85-128 for the FP64 forms.
#include "rkcu.h"
#include "rkcu_mixed.cuh"

namespace rkcu {

constexpr int kMixThreads = 256;

// float with the sign, exponent and leading 23 mantissa bits of x (truncation),
// built with integer instructions: a double->float conversion runs on the FP64
// pipe on this part.  Values outside the float range use the conversion.
__device__ __forceinline__ float trunc_to_float(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = static_cast<unsigned>(__double2loint(x));
  const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0 || e >= 255) return __double2float_rn(x);
  const unsigned bits = (static_cast<unsigned>(hi) & 0x80000000u) | (static_cast<unsigned>(e) << 23) |
                        ((static_cast<unsigned>(hi) & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float(bits);
}

// delta_i at pair q: h c_i F0(q) + S_i(q)
struct DeltaView {
  const float2 *__restrict__ f0;
  const float2 *__restrict__ S;  // null for stage 1
  float hc;
  __device__ __forceinline__ float2 at(int q) const {
    const float2 f = f0[q];
    float2 d = make_float2(hc * f.x, hc * f.y);
    if (S) {
      const float2 s = S[q];
      d.x += s.x;
      d.y += s.y;
    }
    return d;
  }
};

// dF_i at grid point p (both components)
__device__ __forceinline__ float2 delta_rhs(const DeltaView &dv, const float2 y32, int p, int N,
                                            float coef) {
  const int k = p / N;
  const int j = p - k * N;
  const float2 c = dv.at(p);
  const float2 up = dv.at(k == 0 ? p + N : p - N);
  const float2 dn = dv.at(k == N - 1 ? p - N : p + N);
  float lu = up.x + dn.x, lv = up.y + dn.y;
  if (j == 0) {
    const float2 e = dv.at(p + 1);
    lu = fmaf(2.0f, e.x, lu);
    lv = fmaf(2.0f, e.y, lv);
  } else if (j == N - 1) {
    const float2 w = dv.at(p - 1);
    lu = fmaf(2.0f, w.x, lu);
    lv = fmaf(2.0f, w.y, lv);
  } else {
    const float2 w = dv.at(p - 1);
    const float2 e = dv.at(p + 1);
    lu = (lu + w.x) + e.x;
    lv = (lv + w.y) + e.y;
  }
  lu = fmaf(-4.0f, c.x, lu);
  lv = fmaf(-4.0f, c.y, lv);
  const float u = y32.x, v = y32.y, du = c.x, dvv = c.y;
  // (u+du)^2 (v+dv) - u^2 v = du (2u + du)(v + dv) + u^2 dv
  const float dX = fmaf(du * fmaf(2.0f, u, du), v + dvv, u * u * dvv);
  return make_float2(fmaf(coef, lu, fmaf(-4.4f, du, dX)), fmaf(coef, lv, fmaf(3.4f, du, -dX)));
}

__global__ void __launch_bounds__(kMixThreads) mixed_kernel(const __grid_constant__ MixedParams P) {
  __shared__ double s_t, s_h;
  __shared__ int s_acc, s_rej, s_cur, s_done;
  __shared__ unsigned long long s_step;
  __shared__ double s_wmax[kMixThreads / 32];
  __shared__ float hA[kMaxStages * kMaxStages], hb[kMaxStages], hbh[kMaxStages], hc[kMaxStages];
  __shared__ double s_hbsum;
  __shared__ float s_hbhsum;

  DevState *st = P.st;
  const int s = P.s;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gstride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Bruss &br = P.bruss;
  const float coef = static_cast<float>(br.coef);

  if (threadIdx.x == 0) {
    s_t = st->t;
    s_h = st->h;
    s_acc = st->steps_acc;
    s_rej = st->steps_rej;
    s_cur = st->cur;
    s_done = st->done;
    s_step = st->step;
  }
  __syncthreads();

  bool ok = true;
  for (int it = 0; it < P.budget; ++it) {
    if (s_done) break;
    const double h = s_h;
    for (int idx = threadIdx.x; idx < kMaxStages * kMaxStages; idx += blockDim.x)
      hA[idx] = static_cast<float>(h * P.A[idx]);
    if (threadIdx.x < kMaxStages) {
      hb[threadIdx.x] = static_cast<float>(h * P.b[threadIdx.x]);
      hbh[threadIdx.x] = static_cast<float>(h * P.bh[threadIdx.x]);
      hc[threadIdx.x] = static_cast<float>(h * P.csum[threadIdx.x]);
    }
    if (threadIdx.x == 0) {
      s_hbsum = h * P.bsum;
      s_hbhsum = static_cast<float>(h * P.bhsum);
    }
    __syncthreads();
    const double2 *__restrict__ ycur = P.y[s_cur];
    double2 *__restrict__ ynew = P.y[s_cur ^ 1];

    // stage 0: F0 = f(y) in FP64, y1 = y + h sum(b) F0, F0 and y rounded to FP32
    {
      const double hbs = s_hbsum;
      for (int p = gtid; p < P.npairs; p += gstride) {
        const double2 F = br.eval<kArithFused>(ycur, p);
        const double2 Y = ycur[p];
        ynew[p] = make_double2(fma(hbs, F.x, Y.x), fma(hbs, F.y, Y.y));
        P.f0[p] = make_float2(__double2float_rn(F.x), __double2float_rn(F.y));
        P.y32[p] = make_float2(trunc_to_float(Y.x), trunc_to_float(Y.y));
      }
    }
    if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 11))) break;

    float emax = 0.0f;
    for (int i = 1; i < s; ++i) {
      DeltaView dv{P.f0, i >= 2 ? P.S[i] : nullptr, hc[i]};
      const bool last = (i == s - 1);
      const float bi = hb[i], bhi = hbh[i];
      for (int p = gtid; p < P.npairs; p += gstride) {
        const float2 y32 = P.y32[p];
        const float2 dF = delta_rhs(dv, y32, p, br.N, coef);
        for (int l = i + 1; l < s; ++l) {
          if (!P.nzA[l * kMaxStages + i] && i > 1) continue;
          const float a = hA[l * kMaxStages + i];
          float2 acc = (i == 1) ? make_float2(0.f, 0.f) : P.S[l][p];
          acc.x = fmaf(a, dF.x, acc.x);
          acc.y = fmaf(a, dF.y, acc.y);
          P.S[l][p] = acc;
        }
        // Kahan-compensated dY and the error estimate
        float2 sum, cmp, e;
        if (i == 1) {
          // the F0 terms of the error estimate: h sum(b - b^) F0 (zero for embedded pairs)
          const float2 f = P.f0[p];
          sum = make_float2(0.f, 0.f);
          cmp = make_float2(0.f, 0.f);
          e = make_float2(s_hbhsum * f.x, s_hbhsum * f.y);
        } else {
          sum = P.dys[p];
          cmp = P.dyc[p];
          e = P.err[p];
        }
        {
          const float ax = fmaf(bi, dF.x, -cmp.x), ay = fmaf(bi, dF.y, -cmp.y);
          const float tx = sum.x + ax, ty = sum.y + ay;
          cmp.x = (tx - sum.x) - ax;
          cmp.y = (ty - sum.y) - ay;
          sum.x = tx;
          sum.y = ty;
        }
        e.x = fmaf(bhi, dF.x, e.x);
        e.y = fmaf(bhi, dF.y, e.y);
        if (!last) {
          P.dys[p] = sum;
          P.dyc[p] = cmp;
          P.err[p] = e;
        } else {
          const double2 y1 = ynew[p];
          const double2 yn = make_double2(y1.x + static_cast<double>(sum.x - cmp.x),
                                          y1.y + static_cast<double>(sum.y - cmp.y));
          ynew[p] = yn;
          const float dnx = fmaxf(fabsf(trunc_to_float(yn.x)), fabsf(y32.x));
          const float dny = fmaxf(fabsf(trunc_to_float(yn.y)), fabsf(y32.y));
          emax = fmaxf(emax, dnx == 0.0f ? 3.0e38f : fabsf(e.x) / dnx);
          if (2 * p + 1 < P.n) emax = fmaxf(emax, dny == 0.0f ? 3.0e38f : fabsf(e.y) / dny);
        }
      }
      if (!last) {
        if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 12))) break;
      }
    }
    if (!ok) break;

    double dmax = static_cast<double>(emax);  // the norm is reduced in FP64
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
    if (lane == 0) s_wmax[warp] = dmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = s_wmax[0];
      for (int k = 1; k < kMixThreads / 32; ++k) m = fmax(m, s_wmax[k]);
      atomicMax(&st->err_slot[s_step & 1], (unsigned long long)__double_as_longlong(m));
    }
    if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 13))) break;

    if (threadIdx.x == 0) {
      if (blockIdx.x == 0) st->err_slot[(s_step + 1) & 1] = 0ull;
      const double errmax =
          __longlong_as_double((long long)*(volatile unsigned long long *)&st->err_slot[s_step & 1]);
      double t = s_t, hh = s_h;
      int acc = s_acc, rej = s_rej, cur = s_cur;
      bool host_pow;  // the mixed form does not defer to the host: its h need not be bit-exact
      const double hn = h_new(hh, errmax, P.tol, P.ord, &host_pow);
      if (P.tol <= 0.0 || errmax <= P.tol) {
        t += hh;
        ++acc;
        cur ^= 1;
      } else {
        ++rej;
      }
      if (P.tol > 0.0) hh = hn;
      hh = fmin(hh, P.te - t);
      s_t = t;
      s_h = hh;
      s_acc = acc;
      s_rej = rej;
      s_cur = cur;
      s_step = s_step + 1;
      s_done = !(t < P.te) || (P.step_limit > 0 && acc + rej >= P.step_limit);
    }
    __syncthreads();
  }

  if (ok && blockIdx.x == 0 && threadIdx.x == 0) {
    st->t = s_t;
    st->h = s_h;
    st->steps_acc = s_acc;
    st->steps_rej = s_rej;
    st->cur = s_cur;
    st->done = s_done;
    st->step = s_step;
    st->pending = 0;
  }
}

cudaError_t launch_mixed(const MixedParams &p, int num_sms, cudaStream_t stream, int *grid_out) {
  int occ = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mixed_kernel, kMixThreads, 0);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  int grid = occ * num_sms;
  const int useful = (p.npairs + kMixThreads - 1) / kMixThreads;
  if (grid > useful) grid = useful > 0 ? useful : 1;
  MixedParams q = p;
  q.nblocks = grid + (p.extra_arrivals > 0 ? p.extra_arrivals : 0);
  void *args[] = {&q};
  *grid_out = grid;
  return cudaLaunchCooperativeKernel((const void *)mixed_kernel, dim3(grid), dim3(kMixThreads), args,
                                     0, stream);
}

}  // namespace rkcu
