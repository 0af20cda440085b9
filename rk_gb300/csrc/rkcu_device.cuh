// Device building blocks shared by the rkcu kernels: arithmetic policies, the
// right-hand sides of the problem modules, and a bounded grid barrier.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rkcu_errmax.cuh"
#include "rkcu_pow.cuh"
#include "rkcu_softfp64.cuh"

namespace rkcu {

constexpr int kMaxStages = 13;   // DOPRI87 (src/methods.c:476) is the largest tableau

// ---------------------------------------------------------------------------
// Arithmetic policies (template argument kExact of the evaluators and kernels).
//
// kArithExact (1): every product and sum is rounded once, in the order the
// reference's C expressions imply, with explicit round-to-nearest intrinsics
// so that nvcc cannot contract them into FMAs.  The two FMAs it does use,
// fma(-4,y,s) and fma(2,y,s), are exact rewrites: 4y and 2y are exact in
// binary floating point, so fma(-4,y,s) == s - 4.0*y rounded once, as in the
// reference.
// kArithExactSoftMul (2): the same results bit for bit, with the products
// computed on the integer pipe (rkcu_softfp64.cuh) while the sums stay on the
// FP64 pipe -- on this part the FP64 pipe is the bottleneck and the integer
// issue slots are idle.
// kArithFused (0): contracts a*b+c into one FMA (fewer FP64 instructions).
// ---------------------------------------------------------------------------
constexpr int kArithFused = 0;
constexpr int kArithExact = 1;
constexpr int kArithExactSoftMul = 2;
// kArithFusedSoftMul (3): as kArithFused (a*b+c contracted into FMAs), with the
// products that stay plain products computed in software binary64 on the
// integer pipe -- the same bits as kArithFused, fewer FP64 instructions.
constexpr int kArithFusedSoftMul = 3;

template <int kMode>
struct Arith;

template <>
struct Arith<kArithExact> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  // acc + a*b with the product rounded first (C semantics without contraction)
  static __device__ __forceinline__ double mac(double acc, double a, double b) {
    return __dadd_rn(acc, __dmul_rn(a, b));
  }
  // a*b - c with the product rounded first
  static __device__ __forceinline__ double msub(double a, double b, double c) {
    return __dsub_rn(__dmul_rn(a, b), c);
  }
  // x - a*b with the product rounded first
  static __device__ __forceinline__ double submul(double x, double a, double b) {
    return __dsub_rn(x, __dmul_rn(a, b));
  }
};

template <>
struct Arith<kArithExactSoftMul> {
  static __device__ __forceinline__ double mul(double a, double b) { return softfp::mul(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mac(double acc, double a, double b) {
    return __dadd_rn(acc, softfp::mul(a, b));
  }
  static __device__ __forceinline__ double msub(double a, double b, double c) {
    return __dsub_rn(softfp::mul(a, b), c);
  }
  static __device__ __forceinline__ double submul(double x, double a, double b) {
    return __dsub_rn(x, softfp::mul(a, b));
  }
};

template <>
struct Arith<kArithFusedSoftMul> {
  static __device__ __forceinline__ double mul(double a, double b) { return softfp::mul(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double mac(double acc, double a, double b) { return fma(a, b, acc); }
  static __device__ __forceinline__ double msub(double a, double b, double c) { return fma(a, b, -c); }
  static __device__ __forceinline__ double submul(double x, double a, double b) { return fma(-a, b, x); }
};

template <>
struct Arith<kArithFused> {
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double add(double a, double b) { return a + b; }
  static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
  static __device__ __forceinline__ double mac(double acc, double a, double b) { return fma(a, b, acc); }
  static __device__ __forceinline__ double msub(double a, double b, double c) { return fma(a, b, -c); }
  static __device__ __forceinline__ double submul(double x, double a, double b) { return fma(-a, b, x); }
};

// ---------------------------------------------------------------------------
// Right-hand sides.  The unit of work is a pair of consecutive components
// (2p, 2p+1): one grid point (u, v) of BRUSS2D-MIX, one prey/predator pair of
// LV, two neighbours of the banded chain.  Every vector is padded to an even
// length, so a pair is one 16-byte aligned double2.
// ---------------------------------------------------------------------------

// BRUSS2D-MIX (src/problems/bruss2d-mix.c:66-206), grid point p = k*N + j.
//   U: 1 + u^2 v - 4.4 u + alpha (N-1)^2 (sum of the 4 neighbours - 4u)
//   V: 3.4 u - u^2 v     + alpha (N-1)^2 (sum of the 4 neighbours - 4v)
// A missing neighbour at the boundary is replaced by the opposite one.  The
// reference sums "yN + yS" first (a boundary row doubles the inner neighbour,
// which "y + y" reproduces exactly), then adds W and E left to right in
// interior columns, or "2 * inner" in one rounding in the first/last column.
// The BRUSS2D-MIX Laplacian on the FP64 pipe in the order of
// src/problems/bruss2d-mix.c (see Bruss::eval_rows); out of line, so that the
// integer path's callers do not get it if-converted into every lane.
static __device__ __noinline__ double2 lap2_fp64(double2 n, double2 s, double2 w, double2 e, double2 c,
                                                  int jcase) {
  double2 l = make_double2(__dadd_rn(n.x, s.x), __dadd_rn(n.y, s.y));
  if (jcase == 0) {
    l = make_double2(__dadd_rn(__dadd_rn(l.x, w.x), e.x), __dadd_rn(__dadd_rn(l.y, w.y), e.y));
  } else {
    const double2 t = jcase == 1 ? e : w;
    l = make_double2(__fma_rn(2.0, t.x, l.x), __fma_rn(2.0, t.y, l.y));
  }
  return make_double2(__fma_rn(-4.0, c.x, l.x), __fma_rn(-4.0, c.y, l.y));
}

struct Bruss {
  int N;        // grid size
  double coef;  // (alpha * (N-1)) * (N-1), evaluated on the host in that order
  // pairs on either side a point's stencil reaches: one grid row (ode_acc_dist = 2N components)
  __device__ __forceinline__ int dep_pairs() const { return N; }

  template <int kExact>
  __device__ __forceinline__ double2 eval(const double2 *__restrict__ w, int p) const {
    const int k = p / N;
    return eval_kj<kExact>(w, p, k, p - k * N);
  }
  // Same, with the pair's grid row k and column j given (loops that advance
  // p by a fixed stride track them without a division).
  template <int kExact>
  __device__ __forceinline__ double2 eval_kj(const double2 *__restrict__ w, int p, int k, int j) const {
    const double2 *row = w + (p - j);
    return eval_rows<kExact>(k == 0 ? row + N : row - N, row, k == N - 1 ? row - N : row + N, j);
  }
  // pairs per grid row (the period of the column index)
  __device__ __forceinline__ int row_pairs() const { return N; }

  // Same, given the grid rows above (`up`: row k-1, or row k+1 on the first row),
  // at (`cr`: row k) and below (`dn`: row k+1, or row k-1 on the last row) of the
  // point, each indexed by column; lets stage vectors live in ring buffers.
  template <int kExact>
  __device__ __forceinline__ double2 eval_rows(const double2 *__restrict__ upr,
                                               const double2 *__restrict__ cr,
                                               const double2 *__restrict__ dnr, int j) const {
    using M = Arith<kExact>;
    const double2 c = cr[j];
    const double2 up = upr[j];
    const double2 dn = dnr[j];
    // jcase 1: first column (the east neighbour twice), 2: last column (the
    // west one twice), 0: interior
    const int jcase = j == 0 ? 1 : (j == N - 1 ? 2 : 0);
    const double2 ww = cr[jcase == 1 ? j + 1 : j - 1];
    const double2 e = cr[jcase == 2 ? j - 1 : j + 1];
    // ((up + dn) + w) + e - 4c, or (up + dn) + 2t - 4c at a boundary column,
    // each operation rounded: in integer arithmetic where the five values share
    // a binade (bit-identical), else on the FP64 pipe
    double lu = 0.0, lv = 0.0;
    const bool fast = softfp::lap_same_binade(up.x, dn.x, ww.x, e.x, c.x, jcase, &lu) &
                      softfp::lap_same_binade(up.y, dn.y, ww.y, e.y, c.y, jcase, &lv);
    if (!fast) {
      const double2 l = lap2_fp64(up, dn, ww, e, c, jcase);
      lu = l.x;
      lv = l.y;
    }
    const double u2v = M::mul(M::mul(c.x, c.x), c.y);  // shared by U and V
    const double ru = M::submul(M::add(1.0, u2v), 4.4, c.x);
    const double rv = M::msub(3.4, c.x, u2v);
    return make_double2(M::mac(ru, coef, lu), M::mac(rv, coef, lv));
  }
};

// LV pairs (src/problems/lv.c:66-87):
//   prey  f0 = c0*y0 - d0*y0*y1,  predator f1 = d1*y0*y1 - c1*y1
struct LvPairs {
  __device__ __forceinline__ int dep_pairs() const { return 0; }
  // no grid: the row and column a caller tracks are unused
  __device__ __forceinline__ int row_pairs() const { return 1 << 30; }
  template <int kExact>
  __device__ __forceinline__ double2 eval_kj(const double2 *__restrict__ w, int p, int, int) const {
    return eval<kExact>(w, p);
  }
  template <int kExact>
  __device__ __forceinline__ double2 eval(const double2 *__restrict__ w, int p) const {
    using M = Arith<kExact>;
    const double2 c = w[p];
    const double f0 = M::sub(M::mul(0.1, c.x), M::mul(M::mul(0.2, c.x), c.y));
    const double f1 = M::msub(M::mul(0.4, c.x), c.y, M::mul(0.2, c.y));
    return make_double2(f0, f1);
  }
};

// Banded LV chain (no reference module): f_i = y_i (r_i + sum_{d=-2..2} a_{i,d} y_{i+d}),
// terms added in order of d, band truncated at the ends of [0, n).
struct LvBanded {
  int n;
  const double *__restrict__ r;  // r[n_pad]
  const double *__restrict__ a;  // a[n_pad][5]
  __device__ __forceinline__ int dep_pairs() const { return 1; }
  __device__ __forceinline__ int row_pairs() const { return 1 << 30; }
  template <int kExact>
  __device__ __forceinline__ double2 eval_kj(const double2 *__restrict__ w, int p, int, int) const {
    return eval<kExact>(w, p);
  }

  template <int kExact>
  __device__ __forceinline__ double comp(const double *__restrict__ y, int i) const {
    using M = Arith<kExact>;
    double acc = r[i];
#pragma unroll
    for (int d = -2; d <= 2; ++d) {
      const int jj = i + d;
      if (jj >= 0 && jj < n) acc = M::mac(acc, a[5 * i + d + 2], y[jj]);
    }
    return M::mul(y[i], acc);
  }
  template <int kExact>
  __device__ __forceinline__ double2 eval(const double2 *__restrict__ w, int p) const {
    const double *y = reinterpret_cast<const double *>(w);
    const int i = 2 * p;
    const double f0 = comp<kExact>(y, i);
    const double f1 = (i + 1 < n) ? comp<kExact>(y, i + 1) : 0.0;
    return make_double2(f0, f1);
  }
};

// ---------------------------------------------------------------------------
// Solver state shared by all CTAs of a persistent launch and kept across
// launches.  The step-control scalars are written back by CTA 0 only.
// ---------------------------------------------------------------------------
struct DevState {
  double t, h;
  int steps_acc, steps_rej;
  int cur;            // which of the two y buffers holds the current y
  int done;
  unsigned long long step;          // attempted steps so far (slot parity)
  unsigned long long err_slot[2];   // bit pattern of the step's error max (>= 0)
  unsigned int bar_count;
  unsigned int bar_gen;
  int error;          // nonzero once a device wait ran out of time
  int error_site;
  // A step whose size update is left to the host (the accept/reject decision,
  // t, the counters and y are already applied on the device):
  int pending;        // 1 while the host has not finished the update
  double pend_err;    // the step's error max
  double pend_h;      // the step's h
  long long host_pow_steps;  // how many updates the host finished so far
  // Updates answered through the mailbox while the kernel runs (PowBox): the
  // sequence number of the last one posted, whether its answer came in time,
  // and the answer.
  unsigned int host_seq;
  int host_answered;
  double host_h;
};

// Mailbox in mapped, pinned host memory for a step-size update left to the
// host: the kernel posts the step's error max and step size (req = sequence
// number, written last with release semantics); the host answers with the new
// step size (ans = req, written last).
struct PowBox {
  unsigned int req, ans;
  double err, h, h_new;
};

// System-scope release store / acquire load of a word in mapped host memory.
__device__ __forceinline__ void st_release_sys(unsigned int *p, unsigned int v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int ld_acquire_sys(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier for a cooperative launch (all CTAs co-resident).  The
// wait is bounded by timeout_ns: on expiry the CTA records an error in the
// state and the barrier returns false; callers then leave the kernel.
__device__ __forceinline__ bool grid_barrier(DevState *st, unsigned int nblocks,
                                             unsigned long long timeout_ns, int site) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int *gen = &st->bar_gen;
    const unsigned int g = *gen;
    __threadfence();
    const unsigned int arrived = atomicAdd(&st->bar_count, 1u);
    int ok = 1;
    if (arrived == nblocks - 1) {
      st->bar_count = 0;
      __threadfence();
      atomicAdd(&st->bar_gen, 1u);
    } else {
      const unsigned long long t0 = globaltimer_ns();
      unsigned int ns = 32;
      while (*gen == g) {
        if (*(volatile int *)&st->error) { ok = 0; break; }
        if (globaltimer_ns() - t0 > timeout_ns) {
          if (atomicCAS(&st->error, 0, 1) == 0) st->error_site = site;
          ok = 0;
          break;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
      }
    }
    __threadfence();
    s_ok = ok && (*(volatile int *)&st->error == 0);
  }
  __syncthreads();
  return s_ok != 0;
}

// Neighbour synchronisation for the plain step loop: each CTA publishes how
// many stages it has completed in this launch; a CTA starts a stage once the
// CTAs whose pairs its stencil reads have completed the previous one.
__device__ __forceinline__ void publish_progress(unsigned int *flags, unsigned int value) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicExch(&flags[blockIdx.x], value);
  }
}

__device__ __forceinline__ bool wait_neighbours(const unsigned int *flags, int c_lo, int c_hi,
                                                unsigned int target, DevState *st,
                                                unsigned long long timeout_ns, int site) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned long long t0 = globaltimer_ns();
    for (int c = c_lo; c <= c_hi && ok; ++c) {
      if (c == static_cast<int>(blockIdx.x)) continue;
      unsigned int ns = 32;
      while (*(volatile const unsigned int *)&flags[c] < target) {
        if (*(volatile int *)&st->error) {
          ok = 0;
          break;
        }
        if (globaltimer_ns() - t0 > timeout_ns) {
          if (atomicCAS(&st->error, 0, 1) == 0) st->error_site = site;
          ok = 0;
          break;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Dataflow tiles: after the whole CTA has written tile c, mark it with value.
__device__ __forceinline__ void publish_tile(unsigned int *done, int c, unsigned int value) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(&done[c], value);
  }
}

// Wait until tiles c_lo..c_hi are marked with at least target (bounded by
// timeout_ns, as the grid barrier); the CTA may then read what they wrote.
__device__ __forceinline__ bool wait_tiles(const unsigned int *done, int c_lo, int c_hi,
                                           unsigned int target, DevState *st,
                                           unsigned long long timeout_ns, int site) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned long long t0 = 0;
    for (int c = c_lo; c <= c_hi && ok; ++c) {
      unsigned int ns = 32;
      while (ld_acquire(&done[c]) < target) {
        if (t0 == 0) t0 = globaltimer_ns();
        if (*(volatile int *)&st->error) {
          ok = 0;
          break;
        }
        if (globaltimer_ns() - t0 > timeout_ns) {
          if (atomicCAS(&st->error, 0, 1) == 0) st->error_site = site;
          ok = 0;
          break;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Step-size update of include/tools.h:221-233 (AMAX 2, AMIN 0.5, ASAF 0.9),
// with a correctly rounded pow; *host_pow flags the rare updates the host
// finishes with the C library's pow (see step_factor_h).
__device__ __forceinline__ double h_new(double h, double err, double tol, int ord, bool *host_pow) {
  return step_factor_h(h, err, tol, ord, host_pow);
}

}  // namespace rkcu
