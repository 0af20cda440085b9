// Batched step loop: one persistent cooperative launch advances every active
// instance by `budget` sweeps.  A sweep is one attempted step of every active
// instance, with the stage order and rounding of the plain kernel (reference
// seq/D.c with block-inline.h:253-320) per instance.
//
//   stages   all chunks of all active instances, grid-stride over chunks (one
//            CTA per chunk at a time, equal-size chunks so the stages stay
//            balanced however uneven the instances are); grid barrier after
//            each stage
//   error    per-chunk block reduction, 64-bit atomicMax into the instance
//   control  one thread per instance: accept/reject, step size (correctly
//            rounded pow), t, counters, next h*A (include/tools.h:191-278);
//            a factor within 0.03 ulp of a rounding boundary is posted to the
//            host, which answers with the C library's pow while the kernel
//            runs (mapped host memory); the instance sits out the sweeps
//            until the answer is there, so every instance takes the
//            reference's step sizes
//   compact  when an instance finished, CTA 0 rebuilds the chunk list; the
//            chunk length is the tuned one, shortened when the active pairs
//            would give fewer than two chunks per CTA (a few large instances)
// Instances are independent, so no problem ever waits for another one's data;
// the only synchronisation is the grid barrier between stages.
#include "rkcu.h"
#include "rkcu_batch.cuh"

namespace rkcu {

template <int kExact>
__device__ __forceinline__ double2 batch_rhs(const InstDesc &d, const double2 *w, int p) {
  switch (d.kind) {
    case RKCU_PROBLEM_BRUSS2D_MIX: {
      const Bruss b{d.grid_n, d.coef};
      return b.eval<kExact>(w, p);
    }
    case RKCU_PROBLEM_LV_PAIRS: {
      const LvPairs l{};
      return l.eval<kExact>(w, p);
    }
    default: {
      const LvBanded l{d.n, d.lv_r, d.lv_a};
      return l.eval<kExact>(w, p);
    }
  }
}

// CTA-wide rebuild of the chunk list from the active slots (called by one CTA)
template <int kT>
__device__ void rebuild_chunks(const BatchParams &P) {
  __shared__ int s_cnt;
  __shared__ unsigned long long s_pairs;
  if (threadIdx.x == 0) {
    s_cnt = 0;
    s_pairs = 0ull;
  }
  __syncthreads();
  const int nslots = *(volatile int *)P.nslots;
  for (int slot = threadIdx.x; slot < nslots; slot += kT) {
    const InstDesc &d = P.desc[slot];
    if (d.active && !d.done) atomicAdd(&s_pairs, static_cast<unsigned long long>(d.npairs));
  }
  __syncthreads();
  // The tuned chunk length, shortened (a multiple of 128 pairs, at least 128)
  // when the active pairs would give fewer than two chunks per CTA, so that a
  // few large instances still occupy the whole grid.
  int len = P.chunk_pairs;
  if (P.nblocks > 0) {
    const unsigned long long want = 2ull * static_cast<unsigned long long>(P.nblocks);
    if (s_pairs < want * static_cast<unsigned long long>(len)) {
      const unsigned long long l = ((s_pairs + want - 1) / want + 127) / 128 * 128;
      len = static_cast<int>(l < 128ull ? 128ull : l);
    }
  }
  for (int slot = threadIdx.x; slot < nslots; slot += kT) {
    const InstDesc &d = P.desc[slot];
    if (!d.active || d.done) continue;
    const int k = (d.npairs + len - 1) / len;
    const int base = atomicAdd(&s_cnt, k);
    for (int j = 0; j < k; ++j) P.chunks[base + j] = make_int2(slot, j * len);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *P.nchunks = s_cnt;
    *P.chunk_len = len;
    __threadfence();
  }
}

template <int kT>
__global__ void __launch_bounds__(kT) batch_rebuild_kernel(const __grid_constant__ BatchParams P) {
  rebuild_chunks<kT>(P);
}

// 1024 resident threads per SM (64 registers) for every block size: fewer
// registers spill, and a single large instance then ran 2.7x slower than the
// plain form at 256 or 128 threads per block (1.3x at 64 registers)
template <int kExact>
constexpr int batch_threads_per_sm() {
  return 1024;
}

template <int kExact, int kT>
__global__ void __launch_bounds__(kT, batch_threads_per_sm<kExact>() / kT) batch_kernel(const __grid_constant__ BatchParams P) {
  using M = Arith<kExact>;
  __shared__ double s_wmax[kT / 32];
  __shared__ int s_nch, s_clen, s_rebuild;
  DevState *st = P.st;
  const int s = P.s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gtid = blockIdx.x * kT + threadIdx.x;
  const int gstride = gridDim.x * kT;
  bool ok = true;

  const int budget = *(volatile int *)P.budget;
  for (int it = 0; it < budget; ++it) {
    if (threadIdx.x == 0) {
      s_nch = *(volatile int *)P.nchunks;
      s_clen = *(volatile int *)P.chunk_len;
    }
    __syncthreads();
    const int nch = s_nch, clen = s_clen;
    if (nch == 0) break;

    for (int i = 0; i < s && ok; ++i) {
      const bool last = (i == s - 1);
      for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const int2 ch = P.chunks[c];
        const InstDesc &d = P.desc[ch.x];
        if (d.pending) continue;  // waits for its step size from the host (same for every CTA)
        const InstCoef &K = P.coef[ch.x];
        const size_t np = static_cast<size_t>(d.npairs);
        double2 *__restrict__ vec = d.vec;
        const double2 *__restrict__ ycur = vec + (d.cur ? np : 0);
        double2 *__restrict__ ynew = vec + (d.cur ? 0 : np);
        double2 *__restrict__ dy = vec + static_cast<size_t>(s + 1) * np;
        double2 *__restrict__ er = vec + static_cast<size_t>(s + 2) * np;
        const int pend = min(ch.y + clen, d.npairs);
        ErrMax em;
        if (i == 0) {
          for (int p = ch.y + threadIdx.x; p < pend; p += kT) {
            const double2 F = batch_rhs<kExact == kArithExactSoftMul ? kArithExact : kExact>(d, ycur, p);
            const double2 Y = ycur[p];
            for (int l = 1; l < s; ++l) {
              double2 wv = Y;
              if (P.nzA[l * kMaxStages]) {
                const double a = K.hA[l * kMaxStages];
                wv.x = M::mac(Y.x, a, F.x);
                wv.y = M::mac(Y.y, a, F.y);
              }
              vec[static_cast<size_t>(1 + l) * np + p] = wv;
            }
            dy[p] = make_double2(M::mul(K.hb[0], F.x), M::mul(K.hb[0], F.y));
            er[p] = make_double2(M::mul(K.hbh[0], F.x), M::mul(K.hbh[0], F.y));
          }
        } else {
          const double2 *__restrict__ wi = vec + static_cast<size_t>(1 + i) * np;
          const double bi = K.hb[i], bhi = K.hbh[i];
          const bool nzb = P.nzb[i], nzbh = P.nzbh[i];
          for (int p = ch.y + threadIdx.x; p < pend; p += kT) {
            const double2 F = batch_rhs<kExact == kArithExactSoftMul ? kArithExact : kExact>(d, wi, p);
            double2 dd = dy[p], e = er[p];
            if (nzb) {
              dd.x = M::mac(dd.x, bi, F.x);
              dd.y = M::mac(dd.y, bi, F.y);
            }
            if (nzbh) {
              e.x = M::mac(e.x, bhi, F.x);
              e.y = M::mac(e.y, bhi, F.y);
            }
            if (!last) {
              for (int l = i + 1; l < s; ++l) {
                if (!P.nzA[l * kMaxStages + i]) continue;
                const double a = K.hA[l * kMaxStages + i];
                double2 *wl = vec + static_cast<size_t>(1 + l) * np;
                double2 wv = wl[p];
                wv.x = M::mac(wv.x, a, F.x);
                wv.y = M::mac(wv.y, a, F.y);
                wl[p] = wv;
              }
              dy[p] = dd;
              er[p] = e;
            } else {
              const double2 Y = ycur[p];
              const double2 yn = make_double2(M::add(Y.x, dd.x), M::add(Y.y, dd.y));
              ynew[p] = yn;
              em.add(e.x, yn.x, Y.x);
              if (2 * p + 1 < d.n) em.add(e.y, yn.y, Y.y);
            }
          }
        }
        if (last) {
          double emax = em.value();
#pragma unroll
          for (int off = 16; off > 0; off >>= 1)
            emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, off));
          if (lane == 0) s_wmax[warp] = emax;
          __syncthreads();
          if (threadIdx.x == 0) {
            double m = s_wmax[0];
            for (int k = 1; k < kT / 32; ++k) m = fmax(m, s_wmax[k]);
            atomicMax(&P.desc[ch.x].errbits, (unsigned long long)__double_as_longlong(m));
          }
          __syncthreads();
        }
      }
      ok = grid_barrier(st, P.nblocks, P.timeout_ns, 20 + i);
    }
    if (!ok) break;

    // step control, one thread per instance (include/tools.h:191-278)
    const int nslots = *(volatile int *)P.nslots;
    for (int slot = gtid; slot < nslots; slot += gstride) {
      InstDesc &d = P.desc[slot];
      if (!d.active || d.done) continue;
      double t = d.t, hh = d.h;
      if (d.pending) {
        // the host's step size (tools.h:221-233 with the C library's pow), once posted
        PowBox *box = P.pow_box + slot;
        if (ld_acquire_sys(&box->ans) != d.pend_seq) continue;
        hh = *(volatile double *)&box->h_new;
        d.pending = 0;
      } else {
        const double errmax = __longlong_as_double((long long)d.errbits);
        if (d.tol <= 0.0) {
          t += hh;
          ++d.steps_acc;
          d.cur ^= 1;
        } else {
          bool host_pow;
          const double hn = h_new(hh, errmax, d.tol, P.ord, &host_pow);
          if (errmax <= d.tol) {
            t += hh;
            ++d.steps_acc;
            d.cur ^= 1;
          } else {
            ++d.steps_rej;
          }
          if (host_pow) {
            // within 0.03 ulp of a rounding boundary the C library's pow, which the
            // reference uses, may round the other way: post the update to the host
            // and sit out the sweeps until its answer arrives
            PowBox *box = P.pow_box + slot;
            d.t = t;
            d.errbits = 0ull;
            d.pending = 1;
            d.pend_seq = d.pend_seq + 1;
            *(volatile double *)&box->err = errmax;
            *(volatile double *)&box->h = hh;
            st_release_sys(&box->req, d.pend_seq);
            continue;
          }
          hh = hn;
        }
      }
      hh = fmin(hh, d.te - t);
      d.t = t;
      d.h = hh;
      d.errbits = 0ull;
      const bool done = !(t < d.te) || (d.step_limit > 0 && d.steps_acc + d.steps_rej >= d.step_limit);
      if (done) {
        d.done = 1;
        const int k = atomicAdd(P.done_count, 1);
        P.done_list[k] = slot;
        atomicExch(P.rebuild, 1);
      } else {
        InstCoef &K = P.coef[slot];
        for (int r = 1; r < s; ++r)
          for (int c = 0; c < r; ++c) K.hA[r * kMaxStages + c] = hh * P.A[r * kMaxStages + c];
        for (int r = 0; r < s; ++r) {
          K.hb[r] = hh * P.b[r];
          K.hbh[r] = hh * P.bh[r];
        }
      }
    }
    if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 40))) break;
    if (threadIdx.x == 0) s_rebuild = *(volatile int *)P.rebuild;
    __syncthreads();
    if (s_rebuild) {
      if (blockIdx.x == 0) rebuild_chunks<kT>(P);
      if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 41))) break;
      if (blockIdx.x == 0 && threadIdx.x == 0) *P.rebuild = 0;
      // every CTA read the flag before the barrier above; the reset is seen
      // by all after the next barrier
    }
  }
}

cudaError_t launch_batch_rebuild(const BatchParams &p, cudaStream_t stream) {
  batch_rebuild_kernel<256><<<1, 256, 0, stream>>>(p);
  return cudaGetLastError();
}

template <int kExact, int kT>
static int grid_of(int blocks_per_sm, int num_sms) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel<kExact, kT>, kT, 0) !=
          cudaSuccess ||
      occ < 1)
    return 0;
  const int per = blocks_per_sm > 0 && blocks_per_sm < occ ? blocks_per_sm : occ;
  return per * num_sms;
}

int batch_grid(bool exact, int threads, int blocks_per_sm, int num_sms) {
  if (threads == 128)
    return exact ? grid_of<kArithExactSoftMul, 128>(blocks_per_sm, num_sms)
                 : grid_of<kArithFusedSoftMul, 128>(blocks_per_sm, num_sms);
  if (threads == 512)
    return exact ? grid_of<kArithExactSoftMul, 512>(blocks_per_sm, num_sms)
                 : grid_of<kArithFusedSoftMul, 512>(blocks_per_sm, num_sms);
  return exact ? grid_of<kArithExactSoftMul, 256>(blocks_per_sm, num_sms)
               : grid_of<kArithFusedSoftMul, 256>(blocks_per_sm, num_sms);
}

template <int kExact, int kT>
static cudaError_t launch_t(const BatchParams &p, int grid, cudaStream_t stream) {
  BatchParams q = p;
  q.nblocks = grid;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, batch_kernel<kExact, kT>, q);
}

cudaError_t launch_batch(const BatchParams &p, bool exact, int threads, int blocks_per_sm,
                         int num_sms, cudaStream_t stream, int *grid_out) {
  const int grid = batch_grid(exact, threads, blocks_per_sm, num_sms);
  if (grid <= 0) return cudaErrorInvalidConfiguration;
  *grid_out = grid;
  if (threads == 128)
    return exact ? launch_t<kArithExactSoftMul, 128>(p, grid, stream) : launch_t<kArithFusedSoftMul, 128>(p, grid, stream);
  if (threads == 512)
    return exact ? launch_t<kArithExactSoftMul, 512>(p, grid, stream) : launch_t<kArithFusedSoftMul, 512>(p, grid, stream);
  return exact ? launch_t<kArithExactSoftMul, 256>(p, grid, stream) : launch_t<kArithFusedSoftMul, 256>(p, grid, stream);
}

}  // namespace rkcu
