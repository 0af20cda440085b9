// Low-storage form of the step loop for BRUSS2D-MIX (the GPU counterpart of
// the reference's pipelined low-storage variant, src/impl/seq/PipeDls.c:49-131).
//
// The grid's rows are cut into nb blocks of R rows (a block is at least the
// access distance, one row = 2N components).  One RK step is a wavefront of
// nb + 2(s-1) steps tau; at wavefront step tau, stage i works on block
// b = tau - 2i.  With this skew of two, everything stage i reads on blocks
// b-1, b, b+1 was completed at an earlier tau, and no stage reads a block
// another stage writes at the same tau, so all stages of a wavefront step run
// concurrently and one synchronisation per tau suffices: either a grid
// barrier, or (the default) neighbour flags.  With flags every CTA works on
// the same slice of block positions in every active block, and before tau it
// waits only for the CTAs whose slices hold the rows its stencils read (the
// rows next to its slice in the same block, and the edge rows of the blocks
// before and after): each read-after-write and each ring-slot reuse is
// between such neighbours and at least one tau apart.
//
// Storage: y (two full vectors, ping-pong as in the plain form) plus ring
// buffers: w_l keeps the blocks from tau-2l-1 to tau (2l+2 slots), dy and err
// keep 2s-1 blocks -- 2n + (s^2 + 5s - 4) R 2N doubles instead of (s+3) n;
// for N = 2000, R = 64, DOPRI5(4): 128 MB + 164 MB instead of 640 MB, and the
// window stays in L2.  Every component sees the same operations in the same
// order as in the plain form, so results are bit-identical to it.
#include "rkcu.h"
#include "rkcu_lowstorage.cuh"
#include "rkcu_plain.cuh"  // kMaxPlainGrid: the progress words a solver allocates

namespace rkcu {

constexpr int kLsThreads = 256;

// Wait until every CTA in the ranges [lo[r], hi[r]] (other than this one) has
// published at least `target` -- one polling thread per CTA, each bounded by
// the time limit -- then a CTA barrier.  False on a time-out or an error set
// elsewhere.
__device__ bool wait_ranges(const unsigned int *flags, const int *lo, const int *hi, int nr,
                            unsigned int target, DevState *st, unsigned long long timeout_ns,
                            int site) {
  int bad = 0;
  int base = 0;
  for (int r = 0; r < nr; ++r) {
    const int cnt = hi[r] - lo[r] + 1;
    for (int q = static_cast<int>(threadIdx.x) - base; q < cnt && !bad; q += blockDim.x) {
      if (q < 0) continue;
      const int c = lo[r] + q;
      if (c == static_cast<int>(blockIdx.x)) continue;
      const unsigned long long t0 = globaltimer_ns();
      unsigned int ns = 32;
      while (ld_acquire(&flags[c]) < target) {
        if (*(volatile int *)&st->error) {
          bad = 1;
          break;
        }
        if (globaltimer_ns() - t0 > timeout_ns) {
          if (atomicCAS(&st->error, 0, 1) == 0) st->error_site = site;
          bad = 1;
          break;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
      }
    }
    base += cnt > 0 ? cnt : 0;
  }
  return !__syncthreads_or(bad);
}

template <int kExact>
__global__ void __launch_bounds__(kLsThreads, 4) ls_kernel(const __grid_constant__ LsParams P) {
  using M = Arith<kExact>;
  // the right-hand side's products on the FP64 pipe in the exact mode (its
  // Laplacian runs on the integer pipe, the tableau products in software):
  // measured faster, same bits
  constexpr int kRhs = kExact == kArithExactSoftMul ? kArithExact : kExact;
  __shared__ double hA[kMaxStages * kMaxStages];
  __shared__ double hb[kMaxStages], hbh[kMaxStages];
  __shared__ double s_t, s_h, s_pend_err, s_pend_h;
  __shared__ int s_acc, s_rej, s_cur, s_done, s_pending;
  __shared__ unsigned long long s_step;
  __shared__ double s_wmax[kLsThreads / 32];
  __shared__ int s_start[kMaxStages + 1], s_stage[kMaxStages], s_blk[kMaxStages], s_nact;
  // per active stage of a wavefront step: ring-slot bases, so that the item
  // loop needs no division -- the stage's argument ring at blocks b-1, b, b+1,
  // every ring at block b (the stage's writes), and the dy / err slots
  __shared__ const double2 *s_rd[kMaxStages][3];
  __shared__ double2 *s_wr[kMaxStages][kMaxStages];
  __shared__ double2 *s_dyb[kMaxStages], *s_erb[kMaxStages];
  // neighbour flags: this CTA's slice of each active item (first pair in the
  // block, start in the CTA's own list), and the CTAs it depends on
  __shared__ int s_mlo[kMaxStages], s_mstart[kMaxStages + 1];
  __shared__ int s_rlo[3], s_rhi[3], s_nr;

  DevState *st = P.st;
  const int s = P.s, N = P.N, R = P.R, nb = P.nb;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gstride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t blk = static_cast<size_t>(R) * N;  // pairs per block slot

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
  const bool flags = P.sync == 0;
  const int G = gridDim.x;
  if (flags && threadIdx.x == 0) {
    // Slices: CTA c takes the block positions [c R N / G, (c+1) R N / G) of
    // every block (truncated in a shorter last block), so a ring slot's
    // position belongs to the same CTA whichever block it holds.  The stencils
    // of a slice read the rows next to it in its block, the previous block's
    // last row if it starts the block, the next block's first row if it ends
    // it; the CTAs reading the slice are the same ones.
    const int c = blockIdx.x;
    const int npf = R * N;
    auto owner = [&](long long q) { return static_cast<int>(((q + 1) * G - 1) / npf); };
    int nr = 0;
    const long long a = static_cast<long long>(c) * npf / G, e = static_cast<long long>(c + 1) * npf / G;
    if (a < e) {
      const int k0 = static_cast<int>(a / N), k1 = static_cast<int>((e - 1) / N);
      s_rlo[nr] = owner(k0 > 0 ? static_cast<long long>(k0 - 1) * N : 0);
      s_rhi[nr++] = owner(k1 + 2 < R ? static_cast<long long>(k1 + 2) * N - 1 : npf - 1);
      if (k0 == 0 && nb > 1) {
        s_rlo[nr] = owner(static_cast<long long>(R - 1) * N);
        s_rhi[nr++] = G - 1;
      }
      if (k1 == R - 1 && nb > 1) {
        s_rlo[nr] = 0;
        s_rhi[nr++] = owner(N - 1);
      }
    }
    s_nr = nr;
  }
  __syncthreads();
  unsigned int progress = 0;  // wavefront steps this CTA has completed in this launch

  bool ok = true;
  for (int it = 0; it < P.budget; ++it) {
    if (s_done || s_pending) break;
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
    ErrMax em;

    const int ntau = nb + 2 * (s - 1);
    for (int tau = 0; tau < ntau && ok; ++tau) {
      // the stages active at this wavefront step and where their items start
      if (threadIdx.x == 0) {
        int cnt = 0, off = 0;
        for (int i = 0; i < s; ++i) {
          const int b = tau - 2 * i;
          if (b < 0 || b >= nb) continue;
          const int rows = min(R, N - b * R);
          s_stage[cnt] = i;
          s_start[cnt] = off;
          off += rows * N;
          ++cnt;
        }
        s_start[cnt] = off;
        s_nact = cnt;
        int mine = 0;
        const long long npf = static_cast<long long>(R) * N;
        for (int a = 0; a < cnt; ++a) {
          const int np = s_start[a + 1] - s_start[a];
          const int lo = min(np, static_cast<int>(static_cast<long long>(blockIdx.x) * npf / G));
          const int hi = min(np, static_cast<int>(static_cast<long long>(blockIdx.x + 1) * npf / G));
          s_mlo[a] = lo;
          s_mstart[a] = mine;
          mine += hi - lo;
        }
        s_mstart[cnt] = mine;
      }
      __syncthreads();
      if (threadIdx.x < s_nact) {
        const int a = threadIdx.x, i = s_stage[a], b = tau - 2 * i;
        s_blk[a] = b;
        const int md = 2 * s - 1;
        s_dyb[a] = P.dyring + static_cast<size_t>(b % md) * blk;
        s_erb[a] = P.errring + static_cast<size_t>(b % md) * blk;
        for (int l = 1; l < s; ++l)
          s_wr[a][l] = P.ring[l] + static_cast<size_t>(b % (2 * l + 2)) * blk;
        if (i > 0) {
          const int m = 2 * i + 2;
          for (int d = 0; d < 3; ++d) {
            const int bb = b - 1 + d;  // blocks outside [0, nb) are never read
            s_rd[a][d] = (bb >= 0 && bb < nb) ? P.ring[i] + static_cast<size_t>(bb % m) * blk : nullptr;
          }
        }
      }
      __syncthreads();
      const int nact = s_nact;
      // neighbour flags: the CTAs this slice reads have completed tau - 1
      // (tau 0 follows the step's grid barrier)
      if (flags && tau > 0 &&
          !(ok = wait_ranges(P.flags, s_rlo, s_rhi, s_nr, progress, st, P.timeout_ns, 32)))
        break;
      // flags: this CTA's slices (its own list, block stride); grid barrier:
      // all items' pairs over the grid
      const int total = flags ? s_mstart[nact] : s_start[nact];
      for (int u = flags ? static_cast<int>(threadIdx.x) : gtid; u < total;
           u += flags ? static_cast<int>(blockDim.x) : gstride) {
        int a = 0;
        const int *starts = flags ? s_mstart : s_start;
        while (a + 1 < nact && u >= starts[a + 1]) ++a;
        const int i = s_stage[a];
        const int b = s_blk[a];
        const int q = flags ? s_mlo[a] + (u - s_mstart[a]) : u - s_start[a];
        const int r = static_cast<int>((static_cast<unsigned long long>(q) * P.inv_n) >> 40);
        const int j = q - r * N;
        const int k = b * R + r;  // grid row
        // argument vector rows: y for stage 0, the ring of w_i otherwise
        const double2 *upr, *cr, *dnr;
        const int ku = (k == 0) ? k + 1 : k - 1;
        const int kd = (k == N - 1) ? k - 1 : k + 1;
        if (i == 0) {
          cr = ycur + static_cast<size_t>(k) * N;
          upr = ycur + static_cast<size_t>(ku) * N;
          dnr = ycur + static_cast<size_t>(kd) * N;
        } else {
          // the neighbour rows lie in blocks b-1, b or b+1
          const double2 *const *rd = s_rd[a];
          const int k0 = b * R;
          cr = rd[1] + static_cast<size_t>(r) * N;
          upr = ku < k0 ? rd[0] + static_cast<size_t>(ku - (k0 - R)) * N
                : ku >= k0 + R ? rd[2] + static_cast<size_t>(ku - (k0 + R)) * N
                               : rd[1] + static_cast<size_t>(ku - k0) * N;
          dnr = kd < k0 ? rd[0] + static_cast<size_t>(kd - (k0 - R)) * N
                : kd >= k0 + R ? rd[2] + static_cast<size_t>(kd - (k0 + R)) * N
                               : rd[1] + static_cast<size_t>(kd - k0) * N;
        }
        const double2 F = P.bruss.eval_rows<kRhs>(upr, cr, dnr, j);
        const size_t loc = static_cast<size_t>(r) * N + j;  // position inside a block slot
        double2 *dyp = s_dyb[a] + loc;
        double2 *erp = s_erb[a] + loc;
        if (i == 0) {
          const double2 Y = cr[j];
          for (int l = 1; l < s; ++l) {
            double2 wv = Y;
            if (P.nzA[l * kMaxStages]) {
              const double aa = hA[l * kMaxStages];
              wv.x = M::mac(Y.x, aa, F.x);
              wv.y = M::mac(Y.y, aa, F.y);
            }
            s_wr[a][l][loc] = wv;
          }
          *dyp = make_double2(M::mul(hb[0], F.x), M::mul(hb[0], F.y));
          *erp = make_double2(M::mul(hbh[0], F.x), M::mul(hbh[0], F.y));
        } else {
          double2 dd = *dyp, e = *erp;
          if (P.nzb[i]) {
            dd.x = M::mac(dd.x, hb[i], F.x);
            dd.y = M::mac(dd.y, hb[i], F.y);
          }
          if (P.nzbh[i]) {
            e.x = M::mac(e.x, hbh[i], F.x);
            e.y = M::mac(e.y, hbh[i], F.y);
          }
          if (i < s - 1) {
            for (int l = i + 1; l < s; ++l) {
              if (!P.nzA[l * kMaxStages + i]) continue;
              const double aa = hA[l * kMaxStages + i];
              double2 *wl = s_wr[a][l] + loc;
              double2 wv = *wl;
              wv.x = M::mac(wv.x, aa, F.x);
              wv.y = M::mac(wv.y, aa, F.y);
              *wl = wv;
            }
            *dyp = dd;
            *erp = e;
          } else {
            const size_t g = static_cast<size_t>(k) * N + j;
            const double2 Y = ycur[g];
            const double2 yn = make_double2(M::add(Y.x, dd.x), M::add(Y.y, dd.y));
            ynew[g] = yn;
            em.add(e.x, yn.x, Y.x);
            em.add(e.y, yn.y, Y.y);
          }
        }
      }
      if (flags)
        publish_progress(P.flags, ++progress);
      else
        ok = grid_barrier(st, P.nblocks, P.timeout_ns, 30);
    }
    if (!ok) break;

    double emax = em.value();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if (lane == 0) s_wmax[warp] = emax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double mm = s_wmax[0];
      for (int k = 1; k < kLsThreads / 32; ++k) mm = fmax(mm, s_wmax[k]);
      atomicMax(&st->err_slot[s_step & 1], (unsigned long long)__double_as_longlong(mm));
    }
    if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 31))) break;

    // step control: as in the plain form (tools.h:191-198, 235-278)
    if (threadIdx.x == 0) {
      if (blockIdx.x == 0) st->err_slot[(s_step + 1) & 1] = 0ull;
      const double errmax =
          __longlong_as_double((long long)*(volatile unsigned long long *)&st->err_slot[s_step & 1]);
      double t = s_t, hh = s_h;
      int acc = s_acc, rej = s_rej, cur = s_cur;
      bool host_pow = false;
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
    if (s_pending) break;
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

template <int kExact>
static cudaError_t launch_t(const LsParams &p, int num_sms, cudaStream_t stream, int *grid_out) {
  int occ = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ls_kernel<kExact>, kLsThreads, 0);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  int grid = occ * num_sms;
  LsParams q = p;
  q.nblocks = grid + (p.extra_arrivals > 0 ? p.extra_arrivals : 0);
  if (q.sync == 0 && (q.flags == nullptr || grid > kMaxPlainGrid)) q.sync = 1;  // more CTAs than flag words
  if (q.sync == 0) {
    e = cudaMemsetAsync(q.flags, 0, sizeof(unsigned int) * grid, stream);
    if (e != cudaSuccess) return e;
  }
  void *args[] = {&q};
  *grid_out = grid;
  return cudaLaunchCooperativeKernel((const void *)ls_kernel<kExact>, dim3(grid), dim3(kLsThreads),
                                     args, 0, stream);
}

cudaError_t launch_lowstorage(const LsParams &p, bool exact, int num_sms, cudaStream_t stream,
                              int *grid_out) {
  return exact ? launch_t<kArithExactSoftMul>(p, num_sms, stream, grid_out)
               : launch_t<kArithFusedSoftMul>(p, num_sms, stream, grid_out);
}

size_t lowstorage_ring_pairs(int s, int R, int N) {
  size_t slots = 2 * (2 * static_cast<size_t>(s) - 1);
  for (int l = 1; l < s; ++l) slots += 2 * static_cast<size_t>(l) + 2;
  return slots * static_cast<size_t>(R) * N;
}

}  // namespace rkcu
