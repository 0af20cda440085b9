// Plain form of the step loop: one persistent cooperative kernel executes
// whole embedded-RK steps with the stage order of the reference's D variant
// (src/impl/seq/D.c:58-78 with the scatter kernels of
// include/block-inline.h:253-320), the error max of include/tools.h:280-288
// and the step control of include/tools.h:191-278 -- all on the device.
//
// Layout in HBM (component pairs as double2, every vector padded to even n):
//   y[2]            current state and the candidate of the running step; an
//                   accepted step flips the index, a rejected one keeps it, so
//                   the reference's y_old restore copy (tools.h:273) is not needed
//   w[1..s-1]       stage arguments, accumulated in scatter order
//   dy, err         the b- and (b - b_hat)-weighted sums
// Every CTA owns one contiguous range of pairs (block distribution as
// src/tools.c:42-56).  Between stages a CTA waits only for the CTAs whose
// pairs its stencil reads (one grid row either side for BRUSS2D-MIX) to
// publish the previous stage; one bounded grid barrier per step closes the
// last stage before the error max is read.  The error max is reduced by warp
// shuffles, shared memory and one 64-bit atomicMax per CTA on the bit pattern
// (the values are >= 0).
//
// Arithmetic per mode (all modes give the hardware's bits): the exact mode
// runs the tableau products in software binary64 and the right-hand side's
// products on the FP64 pipe, the fused mode its remaining plain products in
// software; in every mode the right-hand side's Laplacian sums run in exact
// integer arithmetic where the operands share a binade.  Resident CTAs per SM
// are set per mode (plain_min_blocks).
#include <type_traits>

#include "rkcu_plain.cuh"
#include "rkcu_tma.cuh"
#include "rkcu.h"

namespace rkcu {

constexpr int kThreads = 256;
// Row-ring schedule (kScheduleRowRing): one CTA of kRingThreads per SM, the
// stage input's grid rows staged in a ring of kRingSlots rows of shared memory.
constexpr int kRingThreads = 1024;
constexpr int kRingSlots = 4;
// How long CTA 0 waits for the host's answer to a posted step-size update.
constexpr unsigned long long kHostAnswerNs = 2000000ull;

template <class Prob>
__device__ __forceinline__ const Prob &problem_of(const PlainParams &P);
template <>
__device__ __forceinline__ const Bruss &problem_of<Bruss>(const PlainParams &P) { return P.bruss; }
template <>
__device__ __forceinline__ const LvPairs &problem_of<LvPairs>(const PlainParams &P) { return P.lvp; }
template <>
__device__ __forceinline__ const LvBanded &problem_of<LvBanded>(const PlainParams &P) { return P.lvb; }

// Between stages: either the CTAs whose pairs this CTA's stencil reads have
// published the stage (neighbour flags), or every CTA has (grid barrier).
__device__ __forceinline__ bool stage_sync(const PlainParams &P, int c_lo, int c_hi,
                                           unsigned int progress, int site) {
  if (P.schedule == kScheduleGrid) return grid_barrier(P.st, P.nblocks, P.timeout_ns, site);
  publish_progress(P.flags, progress);
  return wait_neighbours(P.flags, c_lo, c_hi, progress, P.st, P.timeout_ns, site);
}

// Resident CTAs per SM (the register budget) and the arithmetic of the
// right-hand side, per mode, as measured on BRUSS2D-MIX at N=2000 (all bit-identical): with
// the Laplacian on the integer pipe, the exact mode is fastest with the
// right-hand side's products on the FP64 pipe (the tableau products stay in
// software) at 5 CTAs, the fused mode with all plain products in software at 6.
// A pair index with its grid row k and column j (rows of `row` pairs),
// advanced by a fixed stride without a division.
struct GridCursor {
  int p, k, j;
  __device__ __forceinline__ GridCursor(int p0, int row) : p(p0), k(p0 / row), j(p0 - (p0 / row) * row) {}
  __device__ __forceinline__ void advance(int step, int dk, int dj, int row) {
    p += step;
    k += dk;
    j += dj;
    if (j >= row) {
      j -= row;
      ++k;
    }
  }
};

template <class Prob, int kExact>
constexpr int plain_min_blocks() {
  return !std::is_same<Prob, Bruss>::value ? 4 : kExact == kArithFusedSoftMul ? 6 : kExact == kArithExactSoftMul ? 5 : 4;
}
template <int kExact>
constexpr int plain_rhs_mode() {
  return kExact == kArithExactSoftMul ? kArithExact : kExact;
}

template <class Prob, int kExact, bool kRing>
__global__ void __launch_bounds__(kRing ? kRingThreads : kThreads, kRing ? 1 : plain_min_blocks<Prob, kExact>())
    plain_kernel(const __grid_constant__ PlainParams P) {
  using M = Arith<kExact>;
  constexpr int kRhs = plain_rhs_mode<kExact>();
  constexpr int kT = kRing ? kRingThreads : kThreads;
  __shared__ double hA[kMaxStages * kMaxStages];
  __shared__ double hb[kMaxStages], hbh[kMaxStages];
  __shared__ double s_t, s_h;
  __shared__ int s_acc, s_rej, s_cur, s_done, s_pending;
  __shared__ unsigned long long s_step;
  __shared__ double s_pend_err, s_pend_h;
  __shared__ double s_wmax[kT / 32];
  __shared__ unsigned int s_tk[2];

  const Prob &prob = problem_of<Prob>(P);
  DevState *st = P.st;
  const int s = P.s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  if (threadIdx.x == 0) {
    s_t = st->t;
    s_h = st->h;
    s_acc = st->steps_acc;
    s_rej = st->steps_rej;
    s_cur = st->cur;
    s_done = st->done;
    s_step = st->step;
    s_pending = st->pending;
    s_pend_err = st->pend_err;
    s_pend_h = st->pend_h;
  }
  // row ring: kRingSlots rows of pairs in dynamic shared memory, one mbarrier
  // per slot; rpar holds the parity each slot's next completion will have
  extern __shared__ __align__(128) unsigned char s_ring_raw[];
  __shared__ __align__(8) uint64_t s_rbar[kRingSlots];
  unsigned rpar = 0, rpend = 0;  // rpend: slots with a copy issued and not yet waited for
  auto ring_row = [&](int q) {
    return reinterpret_cast<double2 *>(s_ring_raw) + static_cast<size_t>(q) * prob.row_pairs();
  };
  if constexpr (kRing) {
    if (threadIdx.x == 0) {
      for (int q = 0; q < kRingSlots; ++q) mbar_init(&s_rbar[q], 1);
      mbar_fence_init();
    }
  }
  __syncthreads();

  // this CTA's pairs [lo, hi) and the CTAs whose pairs its stencil reads
  const int G = gridDim.x;
  const int q = P.npairs / G, rr = P.npairs % G;
  const int bx = blockIdx.x;
  const int lo = bx < rr ? bx * (q + 1) : rr * (q + 1) + (bx - rr) * q;
  const int hi = lo + (bx < rr ? q + 1 : q);
  // grid schedule: grid-stride over all pairs; neighbour schedule: own range
  const bool grid_sched = P.schedule == kScheduleGrid;
  const int p0 = grid_sched ? bx * blockDim.x + threadIdx.x : lo + threadIdx.x;
  const int pend = grid_sched ? P.npairs : hi;
  const int pstep = grid_sched ? G * blockDim.x : blockDim.x;
  const int dep = prob.dep_pairs();
  // grid row and column steps of the two pair strides the loops use
  const int rowN = prob.row_pairs();
  const int dk_s = pstep / rowN, dj_s = pstep - dk_s * rowN;
  const int dk_b = static_cast<int>(blockDim.x) / rowN, dj_b = static_cast<int>(blockDim.x) - dk_b * rowN;
  auto owner = [&](int p) { return p < rr * (q + 1) ? p / (q + 1) : rr + (p - rr * (q + 1)) / max(q, 1); };
  const int c_lo = owner(max(0, lo - dep));
  const int c_hi = owner(min(P.npairs - 1, max(lo, hi - 1) + dep));
  unsigned int progress = 0;

  bool ok = true;
  for (int it = 0; it < P.budget; ++it) {
    if (s_done || s_pending) break;
    // premult (src/methods.c:43-58): hA = h*A, hb = h*b, hbh = h*(b - b_hat)
    const double h = s_h;
    for (int idx = threadIdx.x; idx < kMaxStages * kMaxStages; idx += blockDim.x)
      hA[idx] = h * P.A[idx];
    if (threadIdx.x < kMaxStages) {
      hb[threadIdx.x] = h * P.b[threadIdx.x];
      hbh[threadIdx.x] = h * P.bh[threadIdx.x];
    }
    __syncthreads();
    const double2 *__restrict__ ycur = P.y[s_cur];
    double2 *__restrict__ ynew = P.y[s_cur ^ 1];
    const int kstep = s_acc + s_rej;  // this step's index (for the trace)
    double2 *__restrict__ ytr =
        (P.trace_y && kstep < P.trace_cap) ? P.trace_y + static_cast<size_t>(kstep) * P.npairs : nullptr;

    // first stage at pair p (block-inline.h:253-272), from F = f(y) and y at p
    auto stage_first_f = [&](int p, const double2 F, const double2 Y) {
      for (int l = 1; l < s; ++l) {
        double2 wv = Y;
        if (P.nzA[l * kMaxStages]) {
          const double a = hA[l * kMaxStages];
          wv.x = M::mac(Y.x, a, F.x);
          wv.y = M::mac(Y.y, a, F.y);
        }
        P.w[l][p] = wv;
      }
      P.dy[p] = make_double2(M::mul(hb[0], F.x), M::mul(hb[0], F.y));
      P.err[p] = make_double2(M::mul(hbh[0], F.x), M::mul(hbh[0], F.y));
    };
    auto stage_first = [&](int p, int k, int j) {
      stage_first_f(p, prob.template eval_kj<kRhs>(ycur, p, k, j), ycur[p]);
    };
    // intermediate stage i at pair p (block-inline.h:276-294), from F = f(w_i) at p
    auto stage_mid_f = [&](int i, int p, const double2 F) {
      for (int l = i + 1; l < s; ++l) {
        if (!P.nzA[l * kMaxStages + i]) continue;
        const double a = hA[l * kMaxStages + i];
        double2 wv = P.w[l][p];
        wv.x = M::mac(wv.x, a, F.x);
        wv.y = M::mac(wv.y, a, F.y);
        P.w[l][p] = wv;
      }
      if (P.nzb[i]) {
        const double bi = hb[i];
        double2 d = P.dy[p];
        d.x = M::mac(d.x, bi, F.x);
        d.y = M::mac(d.y, bi, F.y);
        P.dy[p] = d;
      }
      if (P.nzbh[i]) {
        const double bhi = hbh[i];
        double2 e = P.err[p];
        e.x = M::mac(e.x, bhi, F.x);
        e.y = M::mac(e.y, bhi, F.y);
        P.err[p] = e;
      }
    };
    auto stage_mid = [&](int i, int p, int k, int j) {
      stage_mid_f(i, p, prob.template eval_kj<kRhs>(P.w[i], p, k, j));
    };
    // last stage at pair p (block-inline.h:298-320) and its error terms
    // (tools.h:280-288), from F = f(w_{s-1}) at p
    ErrMax em;
    auto stage_last_f = [&](int p, const double2 F) {
      const int i = s - 1;
      double2 d = P.dy[p];
      double2 e = P.err[p];
      if (P.nzb[i]) {
        d.x = M::mac(d.x, hb[i], F.x);
        d.y = M::mac(d.y, hb[i], F.y);
      }
      if (P.nzbh[i]) {
        e.x = M::mac(e.x, hbh[i], F.x);
        e.y = M::mac(e.y, hbh[i], F.y);
      }
      const double2 Y = ycur[p];
      const double2 yn = make_double2(M::add(Y.x, d.x), M::add(Y.y, d.y));
      ynew[p] = yn;
      if (ytr) ytr[p] = yn;
      em.add(e.x, yn.x, Y.x);
      if (2 * p + 1 < P.n) em.add(e.y, yn.y, Y.y);
    };
    auto stage_last = [&](int p, int k, int j) {
      stage_last_f(p, prob.template eval_kj<kRhs>(P.w[s - 1], p, k, j));
    };

    // Software prefetch (to L1) of the next pair's stage vectors, in the fused
    // mode only: it stalls most on memory latency (measured +2 % there, nothing
    // in the exact mode).  q < pend keeps every address inside the vectors.
    auto pf = [&](const void *a) {
      if constexpr (kExact == kArithFusedSoftMul) asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
    };
    auto pf_first = [&](int q) {
      if (kExact == kArithFusedSoftMul && q < pend) pf(&ycur[q]);
    };
    auto pf_mid = [&](int i, int q) {
      if (kExact == kArithFusedSoftMul && q < pend) {
        pf(&P.w[i][q]);
        for (int l = i + 1; l < s; ++l)
          if (P.nzA[l * kMaxStages + i]) pf(&P.w[l][q]);
        if (P.nzb[i]) pf(&P.dy[q]);
        if (P.nzbh[i]) pf(&P.err[q]);
      }
    };
    auto pf_last = [&](int q) {
      if (kExact == kArithFusedSoftMul && q < pend) {
        pf(&P.w[s - 1][q]);
        pf(&P.dy[q]);
        pf(&P.err[q]);
        pf(&ycur[q]);
      }
    };
    if (P.schedule == kScheduleFlow) {
      // Dataflow over (stage, tile) tickets in skewed wavefront order: tile c
      // of stage i is ticket (c + K i) s + i, and waits only until stage i-1
      // is complete on tiles c-dt .. c+dt (the rows its stencil reads).  With
      // K >= dt every dependency holds a smaller ticket, and the CTA holding
      // the smallest unfinished ticket never waits, so the schedule cannot
      // deadlock among co-resident CTAs.  Tiles completed: done[c] =
      // it s + i + 1 (the counters are zeroed by each launch).
      const int nt = P.flow_ntiles, tp = P.flow_tile, K = P.flow_skew, dt = P.flow_dep;
      unsigned int *ticket = P.flags;
      unsigned int *done = P.flags + 2;
      const unsigned int total = static_cast<unsigned int>(nt + K * (s - 1)) * s;
      const unsigned int base = static_cast<unsigned int>(it) * s;
      // the counter of the next step was last used a step ago: clear it
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&ticket[(it + 1) & 1], 0u);
      if (threadIdx.x == 0) s_tk[0] = atomicAdd(&ticket[it & 1], 1u);
      __syncthreads();
      unsigned int tk = s_tk[0];
      int slot = 0;
      while (tk < total) {
        // fetch the next ticket while this tile runs
        if (threadIdx.x == 0) s_tk[slot ^ 1] = atomicAdd(&ticket[it & 1], 1u);
        const int i = static_cast<int>(tk % s);
        const int c = static_cast<int>(tk / s) - K * i;
        if (c >= 0 && c < nt) {
          if (i > 0) {
            if (!(ok = wait_tiles(done, max(0, c - dt), min(nt - 1, c + dt), base + i, st,
                                  P.timeout_ns, 4)))
              break;
          }
          const int p_hi = min(P.npairs, (c + 1) * tp);
          if (i == 0) {
            for (GridCursor g(c * tp + threadIdx.x, rowN); g.p < p_hi; g.advance(blockDim.x, dk_b, dj_b, rowN))
              stage_first(g.p, g.k, g.j);
          } else if (i < s - 1) {
            for (GridCursor g(c * tp + threadIdx.x, rowN); g.p < p_hi; g.advance(blockDim.x, dk_b, dj_b, rowN))
              stage_mid(i, g.p, g.k, g.j);
          } else {
            for (GridCursor g(c * tp + threadIdx.x, rowN); g.p < p_hi; g.advance(blockDim.x, dk_b, dj_b, rowN))
              stage_last(g.p, g.k, g.j);
          }
          publish_tile(done, c, base + i + 1);
        }
        __syncthreads();
        tk = s_tk[slot ^ 1];
        slot ^= 1;
      }
      if (!ok) break;
    } else if constexpr (kRing) {
      // Row ring (BRUSS2D-MIX): for each stage, the stage input's grid rows that
      // this CTA's pairs and their stencils touch arrive by 1-D bulk copies
      // (TMA) into a ring of kRingSlots rows of shared memory, one row ahead of
      // the row being computed; the stencil reads shared memory, the other
      // vectors are read and written in place.
      auto ring_stage = [&](const double2 *src, auto &&body) {
        const int N = rowN;
        if (lo >= hi) return true;
        const int r0 = lo / N, r1 = (hi - 1) / N;
        const unsigned row_bytes = static_cast<unsigned>(N) * 16u;
        auto issue = [&](int r) {
          if (r < 0 || r >= N || r > r1 + 1 || r < r0 - 1) return;
          const int q = r % kRingSlots;
          mbar_arrive_expect_tx(&s_rbar[q], row_bytes);
          bulk_load(ring_row(q), src + static_cast<size_t>(r) * N, row_bytes, &s_rbar[q]);
          rpend |= 1u << q;
        };
        auto wait_row = [&](int r) {
          if (r < 0 || r >= N || r > r1 + 1) return true;
          const int q = r % kRingSlots;
          const bool got = mbar_wait(&s_rbar[q], (rpar >> q) & 1u, st, P.timeout_ns, 5);
          if (got) {
            rpar ^= 1u << q;
            rpend &= ~(1u << q);
          }
          return got;
        };
        // rows r0 - 1 .. r0 + kRingSlots - 2 first; then, once row r is done (its
        // up row's slot is free), row r + kRingSlots - 1
        if (threadIdx.x == 0)
          for (int r = r0 - 1; r <= r0 + kRingSlots - 2; ++r) issue(r);
        bool good = wait_row(r0 - 1) & wait_row(r0);
        for (int r = r0; r <= r1; ++r) {
          good = wait_row(r + 1) && good;
          if (__syncthreads_or(!good)) return false;
          const double2 *cr = ring_row(r % kRingSlots);
          const double2 *up = ring_row((r == 0 ? 1 : r - 1) % kRingSlots);
          const double2 *dn = ring_row((r == N - 1 ? N - 2 : r + 1) % kRingSlots);
          const int jlo = max(lo, r * N) - r * N, jhi = min(hi, (r + 1) * N) - r * N;
          for (int j = jlo + threadIdx.x; j < jhi; j += kT) body(r * N + j, r, j, up, cr, dn);
          __syncthreads();
          if (threadIdx.x == 0) issue(r + kRingSlots - 1);
        }
        return true;
      };
      auto ring_eval = [&](const double2 *up, const double2 *cr, const double2 *dn, int j) {
        return prob.template eval_rows<kRhs>(up, cr, dn, j);
      };
      // generic-proxy writes of this stage, read by later bulk copies (this CTA's
      // and its neighbours'), are ordered before the progress flag
      ok = ring_stage(ycur, [&](int p, int, int j, const double2 *up, const double2 *cr, const double2 *dn) {
        stage_first_f(p, ring_eval(up, cr, dn, j), cr[j]);
      });
      if (!ok) break;
      fence_proxy_async_global();
      if (!(ok = stage_sync(P, c_lo, c_hi, ++progress, 1))) break;
      for (int i = 1; i < s - 1; ++i) {
        ok = ring_stage(P.w[i], [&](int p, int, int j, const double2 *up, const double2 *cr, const double2 *dn) {
          stage_mid_f(i, p, ring_eval(up, cr, dn, j));
        });
        if (!ok) break;
        fence_proxy_async_global();
        if (!(ok = stage_sync(P, c_lo, c_hi, ++progress, 2))) break;
      }
      if (!ok) break;
      ok = ring_stage(P.w[s - 1], [&](int p, int, int j, const double2 *up, const double2 *cr, const double2 *dn) {
        stage_last_f(p, ring_eval(up, cr, dn, j));
      });
      if (!ok) break;
      fence_proxy_async_global();  // y_new is the next step's bulk-copied input
    } else {
      for (GridCursor g(p0, rowN); g.p < pend; g.advance(pstep, dk_s, dj_s, rowN)) {
        pf_first(g.p + pstep);
        stage_first(g.p, g.k, g.j);
      }
      if (!(ok = stage_sync(P, c_lo, c_hi, ++progress, 1))) break;
      for (int i = 1; i < s - 1; ++i) {
        for (GridCursor g(p0, rowN); g.p < pend; g.advance(pstep, dk_s, dj_s, rowN)) {
          pf_mid(i, g.p + pstep);
          stage_mid(i, g.p, g.k, g.j);
        }
        if (!(ok = stage_sync(P, c_lo, c_hi, ++progress, 2))) break;
      }
      if (!ok) break;
      for (GridCursor g(p0, rowN); g.p < pend; g.advance(pstep, dk_s, dj_s, rowN)) {
        pf_last(g.p + pstep);
        stage_last(g.p, g.k, g.j);
      }
    }
    double emax = em.value();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if (lane == 0) s_wmax[warp] = emax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = s_wmax[0];
      for (int k = 1; k < kT / 32; ++k) m = fmax(m, s_wmax[k]);
      atomicMax(&st->err_slot[s_step & 1], (unsigned long long)__double_as_longlong(m));
    }
    if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 3))) break;

    // step control (tools.h:191-198, 235-278), taken identically by every CTA
    if (threadIdx.x == 0) {
      if (blockIdx.x == 0) st->err_slot[(s_step + 1) & 1] = 0ull;
      const double errmax =
          __longlong_as_double((long long)*(volatile unsigned long long *)&st->err_slot[s_step & 1]);
      double t = s_t, hh = s_h;
      int acc = s_acc, rej = s_rej, cur = s_cur;
      bool host_pow = false;
      if (blockIdx.x == 0 && P.trace_meta && acc + rej < P.trace_cap) {
        double *m = P.trace_meta + 3 * static_cast<size_t>(acc + rej);
        m[0] = t;
        m[1] = hh;
        m[2] = errmax;
      }
      if (P.tol <= 0.0) {
        t += hh;
        ++acc;
        cur ^= 1;
      } else {
        const double hn = h_new(hh, errmax, P.tol, P.ord, &host_pow);
        if (errmax <= P.tol) {
          t += hh;
          ++acc;
          cur ^= 1;
        } else {
          ++rej;
        }
        if (host_pow) {
          s_pend_err = errmax;
          s_pend_h = hh;
        } else {
          hh = hn;
        }
      }
      s_pending = host_pow;
      if (!host_pow) {
        hh = fmin(hh, P.te - t);
        s_done = !(t < P.te) || (P.step_limit > 0 && acc + rej >= P.step_limit);
      }
      s_t = t;
      s_h = hh;
      s_acc = acc;
      s_rej = rej;
      s_cur = cur;
      s_step = s_step + 1;
    }
    __syncthreads();
    if (s_pending && P.pow_box) {
      // The host polls the mailbox while this launch runs: CTA 0 posts the
      // update and waits a short, bounded time for the C library's pow; the
      // grid barrier hands the answer to every CTA.  Without an answer in time
      // the launch ends as below and the host finishes the update after it.
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        PowBox *box = P.pow_box;
        const unsigned int seq = st->host_seq + 1;
        st->host_seq = seq;
        *(volatile double *)&box->err = s_pend_err;
        *(volatile double *)&box->h = s_pend_h;
        st_release_sys(&box->req, seq);
        const unsigned long long t0 = globaltimer_ns();
        bool got = false;
        while (!(got = ld_acquire_sys(&box->ans) == seq) && globaltimer_ns() - t0 < kHostAnswerNs)
          __nanosleep(64);
        st->host_h = got ? *(volatile double *)&box->h_new : 0.0;
        st->host_answered = got ? 1 : 0;
        if (got) ++st->host_pow_steps;
      }
      if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 7))) break;
      if (threadIdx.x == 0 && *(volatile int *)&st->host_answered) {
        // as the host would finish it: the loop increment and test of tools.h:196-197
        s_h = fmin(*(volatile double *)&st->host_h, P.te - s_t);
        s_done = !(s_t < P.te) || (P.step_limit > 0 && s_acc + s_rej >= P.step_limit);
        s_pending = 0;
      }
      __syncthreads();
    }
    if (s_pending) break;  // the host finishes this step's size update
  }

  // after a wait that ran out of time, let the row copies still in flight land
  // before the CTA leaves (bounded as well)
  if constexpr (kRing) {
    if (rpend && threadIdx.x == 0)
      for (int q = 0; q < kRingSlots; ++q)
        if ((rpend >> q) & 1u) mbar_wait(&s_rbar[q], (rpar >> q) & 1u, st, P.timeout_ns, 6);
  }

  if (ok && blockIdx.x == 0 && threadIdx.x == 0) {
    st->t = s_t;
    st->h = s_h;
    st->steps_acc = s_acc;
    st->steps_rej = s_rej;
    st->cur = s_cur;
    st->done = s_done;
    st->step = s_step;
    st->pending = s_pending;
    st->pend_err = s_pend_err;
    st->pend_h = s_pend_h;
  }
}

template <class Prob>
__global__ void __launch_bounds__(kThreads) eval_rhs_kernel(Prob prob, int npairs,
                                                            const double2 *__restrict__ y,
                                                            double2 *__restrict__ f) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += gridDim.x * blockDim.x)
    f[p] = prob.template eval<kArithExact>(y, p);
}

template <class Prob, int kExact>
static cudaError_t launch_one(const PlainParams &p, int blocks_per_sm, int num_sms,
                              cudaStream_t stream, int *grid_out) {
  if constexpr (std::is_same<Prob, Bruss>::value) {
    if (p.schedule == kScheduleRowRing) {
      // one CTA of kRingThreads per SM with the row ring in dynamic shared memory
      auto kern = plain_kernel<Prob, kExact, true>;
      const size_t dyn = static_cast<size_t>(kRingSlots) * p.bruss.N * sizeof(double2);
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
      if (e != cudaSuccess) return e;
      int occ = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kRingThreads, dyn);
      if (e != cudaSuccess) return e;
      if (occ < 1) return cudaErrorInvalidConfiguration;
      int grid = occ * num_sms;
      const int useful = (p.npairs + kRingThreads - 1) / kRingThreads;
      if (grid > useful) grid = useful > 0 ? useful : 1;
      if (grid > kMaxPlainGrid) grid = kMaxPlainGrid;
      PlainParams q = p;
      q.nblocks = grid + (p.extra_arrivals > 0 ? p.extra_arrivals : 0);
      void *args[] = {&q};
      *grid_out = grid;
      e = cudaMemsetAsync(p.flags, 0, sizeof(unsigned int) * grid, stream);
      if (e != cudaSuccess) return e;
      return cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kRingThreads), args, dyn,
                                         stream);
    }
  }
  auto kern = plain_kernel<Prob, kExact, false>;
  int occ = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreads, 0);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  int per_sm = blocks_per_sm > 0 ? (blocks_per_sm < occ ? blocks_per_sm : occ) : occ;
  int grid = per_sm * num_sms;
  const int useful = (p.npairs + kThreads - 1) / kThreads;
  if (grid > useful) grid = useful > 0 ? useful : 1;
  if (grid > kMaxPlainGrid) grid = kMaxPlainGrid;
  PlainParams q = p;
  q.nblocks = grid + (p.extra_arrivals > 0 ? p.extra_arrivals : 0);
  size_t words = grid;
  if (p.schedule == kScheduleFlow) {
    // skew K: by default about one ticket window of the grid, so that a tile's
    // dependencies were handed out a full round of CTAs earlier
    int K = p.flow_skew > 0 ? p.flow_skew : (grid + p.s - 1) / p.s;
    if (K < p.flow_dep) K = p.flow_dep;
    if (K < 1) K = 1;
    q.flow_skew = K;
    words = flow_words(p.flow_ntiles);
  }
  void *args[] = {&q};
  *grid_out = grid;
  e = cudaMemsetAsync(p.flags, 0, sizeof(unsigned int) * words, stream);
  if (e != cudaSuccess) return e;
  return cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kThreads), args, 0,
                                     stream);
}

template <class Prob>
static cudaError_t launch_mode(const PlainParams &p, int mode, int blocks_per_sm, int num_sms,
                               cudaStream_t stream, int *grid_out) {
  switch (mode) {
    case kArithExact: return launch_one<Prob, kArithExact>(p, blocks_per_sm, num_sms, stream, grid_out);
    case kArithExactSoftMul:
      return launch_one<Prob, kArithExactSoftMul>(p, blocks_per_sm, num_sms, stream, grid_out);
    case kArithFusedSoftMul:
      return launch_one<Prob, kArithFusedSoftMul>(p, blocks_per_sm, num_sms, stream, grid_out);
    default: return launch_one<Prob, kArithFused>(p, blocks_per_sm, num_sms, stream, grid_out);
  }
}

cudaError_t launch_plain(const PlainParams &p, int mode, int blocks_per_sm, int num_sms,
                         cudaStream_t stream, int *grid_out) {
  switch (p.problem) {
    case RKCU_PROBLEM_BRUSS2D_MIX:
      return launch_mode<Bruss>(p, mode, blocks_per_sm, num_sms, stream, grid_out);
    case RKCU_PROBLEM_LV_PAIRS:
      return launch_mode<LvPairs>(p, mode, blocks_per_sm, num_sms, stream, grid_out);
    case RKCU_PROBLEM_LV_BANDED:
      return launch_mode<LvBanded>(p, mode, blocks_per_sm, num_sms, stream, grid_out);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_eval_rhs(int problem, const Bruss &bruss, const LvBanded &lvb, int npairs,
                            const double2 *y, double2 *f, cudaStream_t stream) {
  const int grid = (npairs + kThreads - 1) / kThreads;
  switch (problem) {
    case RKCU_PROBLEM_BRUSS2D_MIX:
      eval_rhs_kernel<Bruss><<<grid, kThreads, 0, stream>>>(bruss, npairs, y, f);
      break;
    case RKCU_PROBLEM_LV_PAIRS:
      eval_rhs_kernel<LvPairs><<<grid, kThreads, 0, stream>>>(LvPairs{}, npairs, y, f);
      break;
    case RKCU_PROBLEM_LV_BANDED:
      eval_rhs_kernel<LvBanded><<<grid, kThreads, 0, stream>>>(lvb, npairs, y, f);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rkcu

namespace rkcu {

__global__ void step_sizes_kernel(const double *__restrict__ h, const double *__restrict__ err,
                                  int count, double tol, int ord, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool host_pow;
  if (i < count) {
    out[i] = h_new(h[i], err[i], tol, ord, &host_pow);
    out[count + i] = host_pow ? 1.0 : 0.0;
  }
}

cudaError_t launch_step_sizes(const double *h, const double *err, int count, double tol, int ord,
                              double *out, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  step_sizes_kernel<<<(count + 255) / 256, 256, 0, stream>>>(h, err, count, tol, ord, out);
  return cudaGetLastError();
}

}  // namespace rkcu
