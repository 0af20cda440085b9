// Mixed-precision form of the step loop (BRUSS2D-MIX): FP32 stage increments,
// FP64 state, FP64 update and error-norm reduction.
//
// On GB300 the FP64 pipe (and every FP64<->FP32 conversion) runs at 1/72 of
// the FP32 rate, so the FP32 stages must avoid both.  Per step and component:
//   F0 = f(y)                          double-float, once per step: the
//                                       Laplacian exact in 64-bit fixed point
//                                       on the integer pipe, the rest in FP32
//                                       pairs (about 2^-46 relative), FP64 only
//                                       where a value leaves those ranges
//   stage i >= 1:  delta_i = h c_i F0 + sum_{1<=j<i} h a_ij dF_j                (FP32)
//                  dF_i = f(y + delta_i) - F0 = alpha (N-1)^2 lap(delta_i)
//                         + [u^2 v](y + delta) - [u^2 v](y) -/+ 4.4 du / 3.4 du  (FP32)
//     (the Laplacian is linear, and the cubic term is expanded exactly, so the
//      large diffusion coefficient never multiplies FP32 rounding of y itself)
//   dY = sum_{j>=1} h b_j dF_j          FP32, Kahan-compensated, in order of j
//   inc = (h * sum b) * F0 + dY         double-float
//   y_new = (y + inc.hi) + inc.lo       two FP64 sums
//   e  = h sum(b - b^) F0 + sum_{j>=1} h (b_j - b^_j) dF_j
//                                       double-float (the F0 term is nearly
//                                       zero: sum(b - b^) = 0)
//   err max = max |e| / max(|y_new|, |y_old|): per thread in FP32, reduced in FP64
// c_i is taken as the row sum of A (sum_j a_ij), so sum_j h a_ij F0 = h c_i F0.
// FP64 instructions per component-step: 2 (the sums of the update; the
// conversions between float and double are built from bit fields) instead of
// 54-73 on the FP64 pipe for the FP64 forms.
//
// Memory: this form is bound by HBM traffic, not arithmetic, so it stores each
// stage's dF_i once and gathers delta_i from dF_1 .. dF_{i-1} at the five
// stencil points when stage i runs (FP32 multiply-adds are cheap here, and the
// neighbours' reads hit L1/L2), instead of scattering dF_i into running sums
// that every later stage reads and rewrites (the D order of the FP64 forms).
// dY and e are formed in the last stage from the stored dF_j.  DRAM traffic
// per grid point and step: about 336 bytes instead of 656, in s FP32 vectors
// (f0, y32, dF_1 .. dF_{s-2}) instead of s + 3.
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <type_traits>

#include "rkcu.h"
#include "rkcu_dfloat.cuh"
#include "rkcu_mixed.cuh"
#include "rkcu_tma.cuh"

namespace rkcu {

constexpr int kMixThreads = 256;
// FP32 stages work on tiles of kTileR x kTileC grid points (one warp per tile
// row), so delta_i is gathered once per point of the tile and its halo
constexpr int kTileR = 8, kTileC = 32;
static_assert(kTileR * kTileC == kMixThreads, "one grid point per thread");
// TMA box per vector: kTileR + 2 rows of kBoxPairs pairs starting two columns
// left of the tile (the box must start at an even pair: 16-byte rule), i.e.
// the tile, its one-point halo and one spare column either side.
constexpr int kBoxRows = kTileR + 2, kBoxPairs = kTileC + 4;
constexpr unsigned kBoxBytes = kBoxRows * kBoxPairs * 8;
constexpr unsigned kSlotBytes = (kBoxBytes + 127) / 128 * 128;  // 128-byte aligned slots

// float with the sign, exponent and leading 23 mantissa bits of x (truncation),
// built with integer instructions: a double->float conversion runs on the FP64
// pipe on this part.  Values outside the float range use the conversion.
__device__ __forceinline__ float trunc_to_float(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = static_cast<unsigned>(__double2loint(x));
  const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
  if (e <= 0 || e >= 255) return softfp::hw_to_float(x);  // out of line: not if-converted
  const unsigned bits = (static_cast<unsigned>(hi) & 0x80000000u) | (static_cast<unsigned>(e) << 23) |
                        ((static_cast<unsigned>(hi) & 0xfffffu) << 3) | (lo >> 29);
  return __uint_as_float(bits);
}

// dF_i at one grid point from delta_i at the point (c), its vertical
// neighbours (up, dn: the row above/below, or the inner row twice at a
// boundary row) and horizontal ones; jcase 1: first column (only e, doubled),
// 2: last column (only w, doubled), 0: interior.
__device__ __forceinline__ float2 delta_rhs(const float2 c, const float2 up, const float2 dn,
                                            const float2 w, const float2 e, int jcase,
                                            const float2 y32, float coef) {
  float lu = up.x + dn.x, lv = up.y + dn.y;
  if (jcase == 1) {
    lu = fmaf(2.0f, e.x, lu);
    lv = fmaf(2.0f, e.y, lv);
  } else if (jcase == 2) {
    lu = fmaf(2.0f, w.x, lu);
    lv = fmaf(2.0f, w.y, lv);
  } else {
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

// delta_i at pair q: h c_i F0(q) + sum over the stage's nonzero j of h a_ij dF_j(q),
// accumulated in order of j (jp: the dF_j vectors, ja: h a_ij, nj of them, at most
// kMaxJ).  All loads are issued before the multiply-adds that use them.
template <int kMaxJ>
__device__ __forceinline__ float2 delta_at(const float2 *const *jp, const float *ja, int nj,
                                           const float2 *__restrict__ f0, float hc, int q) {
  float2 d[kMaxJ > 0 ? kMaxJ : 1];
#pragma unroll
  for (int k = 0; k < kMaxJ; ++k)
    if (k < nj) d[k] = jp[k][q];
  const float2 f = f0[q];
  float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int k = 0; k < kMaxJ; ++k) {
    if (k < nj) {
      acc.x = fmaf(ja[k], d[k].x, acc.x);
      acc.y = fmaf(ja[k], d[k].y, acc.y);
    }
  }
  return make_float2(fmaf(hc, f.x, acc.x), fmaf(hc, f.y, acc.y));
}

// Coefficients of the update at one grid point, per step (shared memory):
// h b_j and h (b_j - b^_j) as FP32 (hb) and as double-float pairs (hbh_hi/lo).
struct MixCoef {
  float hb[kMaxStages], hbh_hi[kMaxStages], hbh_lo[kMaxStages];
  float hbhs_hi, hbhs_lo;  // h sum_j (b_j - b^_j), the F0 term of the estimate
};

// h c x + lo as a double-float product of the pair (c_hi, c_lo) with the float
// x: the leading product exact (TwoProduct), the low part's product rounded.
__device__ __forceinline__ dfl::df df_term(float c_hi, float c_lo, float x) {
  const dfl::df p = dfl::two_prod(c_hi, x);
  return {p.hi, dfl::f_fma(c_lo, x, p.lo)};
}

// The step's update at one grid point from its stage increments d[1..s-2]
// and dlast (dF_1 .. dF_{s-1}), F0 as a double-float pair (f, flo) and y:
//   dY  = sum_j h b_j dF_j          FP32, Kahan-compensated, in stage order
//   inc = h sum(b) F0 + dY          double-float (about 2^-44 relative)
//   y_new = (y + inc.hi) + inc.lo   two FP64 sums, the form's only FP64 work
//   e = h sum(b - b^) F0 + sum_j h (b_j - b^_j) dF_j
//                                   double-float: every product to about 2^-47,
//                                   the sum to about 2^-44 relative, in stage order
// and the error ratios |e| / max(|y_new|, |y|) of the pair's two components
// (FP32 from the estimate's leading part; a zero divisor gives 3e38, so the
// step is rejected, as the reference's 1.7e308 of include/tools.h:284 would).
template <int kMaxS>
__device__ __forceinline__ double2 mix_update(const float2 (&d)[kMaxS], float2 dlast, int s, float2 f,
                                              float2 flo, float2 y32, double2 y, dfl::df hbd,
                                              const MixCoef &c, float *rx, float *ry) {
  float2 sum = make_float2(0.f, 0.f), cmp = make_float2(0.f, 0.f);
  dfl::df ex = df_term(c.hbhs_hi, c.hbhs_lo, f.x), ey = df_term(c.hbhs_hi, c.hbhs_lo, f.y);
#pragma unroll
  for (int jj = 1; jj < kMaxS; ++jj) {
    if (jj >= s) break;
    const float2 dj = jj == s - 1 ? dlast : d[jj];
    const float ax = fmaf(c.hb[jj], dj.x, -cmp.x), ay = fmaf(c.hb[jj], dj.y, -cmp.y);
    const float tx = sum.x + ax, ty = sum.y + ay;
    cmp.x = (tx - sum.x) - ax;
    cmp.y = (ty - sum.y) - ay;
    sum.x = tx;
    sum.y = ty;
    ex = dfl::df_add(ex, df_term(c.hbh_hi[jj], c.hbh_lo[jj], dj.x));
    ey = dfl::df_add(ey, df_term(c.hbh_hi[jj], c.hbh_lo[jj], dj.y));
  }
  const dfl::df ix = dfl::df_add(dfl::df_mul(hbd, {f.x, flo.x}), dfl::fast_two_sum(sum.x, -cmp.x));
  const dfl::df iy = dfl::df_add(dfl::df_mul(hbd, {f.y, flo.y}), dfl::fast_two_sum(sum.y, -cmp.y));
  const double2 yn = make_double2(__dadd_rn(__dadd_rn(y.x, dfl::dbl_of(ix.hi)), dfl::dbl_of(ix.lo)),
                                  __dadd_rn(__dadd_rn(y.y, dfl::dbl_of(iy.hi)), dfl::dbl_of(iy.lo)));
  const float dnx = fmaxf(fabsf(trunc_to_float(yn.x)), fabsf(y32.x));
  const float dny = fmaxf(fabsf(trunc_to_float(yn.y)), fabsf(y32.y));
  const float erx = ex.hi + ex.lo, ery = ey.hi + ey.lo;
  *rx = dnx == 0.0f ? 3.0e38f : fabsf(erx) / dnx;
  *ry = dny == 0.0f ? 3.0e38f : fabsf(ery) / dny;
  return yn;
}

// Fused FP32 stages: all stages 1 .. s-1 of a step on one tile of kFTR x kFTC
// grid points in shared memory.  Stage i is evaluated on the tile and a halo
// of s-1-i points (its increments are read one point further out by the next
// stage's stencil), so the last stage needs the tile alone; only F0 and y32
// (with a halo of s-1 points) are read from memory, one TMA box each,
// double-buffered, and only y_new is written.
constexpr int kFTR = 16, kFTC = 32;  // tile rows, columns
constexpr int kFusedThreads = 512;   // two CTAs per SM
constexpr int mix_threads(int path) { return path == kMixFused ? kFusedThreads : kMixThreads; }

template <int kS>
struct FusedGeom {
  static constexpr int HY = kS - 1;                       // row halo
  static constexpr int HX = (kS - 1 + 1) / 2 * 2;         // column halo, even: a TMA box
                                                          // must start on 16 bytes
  static constexpr int FR = kFTR + 2 * HY, FC = kFTC + 2 * HX;  // frame rows, columns
  static constexpr int kFrame = FR * FC;                  // points (float2) per frame
  static constexpr unsigned kFrameBytes = (kFrame * 8u + 127u) / 128u * 128u;
  // F0 and y32 twice (double buffer), delta twice (this stage's and the
  // next one's), dF_1 .. dF_{s-2}
  static constexpr int kFrames = 6 + (kS > 2 ? kS - 2 : 0);
  static constexpr int kDelta = 4, kDF = 5;  // frame of delta_i: kDelta + (i & 1); of dF_j: kDF + j
  static constexpr size_t kSmem = static_cast<size_t>(kFrames) * kFrameBytes + 128;
  static_assert(2 * FC <= 256 && FR <= 256, "TMA box dimensions are at most 256 elements");
};

template <int kFirst, int kLast, class F>
__device__ __forceinline__ void static_for(F &&f) {
  if constexpr (kFirst < kLast) {
    f(std::integral_constant<int, kFirst>{});
    static_for<kFirst + 1, kLast>(f);
  }
}

// Stage 0 at one pair in FP64 (fused, products in software binary64): the
// path for points whose values the double-float evaluation does not cover.
// Out of line, so that its FP64 instructions are not if-converted into the
// double-float loop.
static __device__ __noinline__ void stage0_point_fp64(const Bruss &br, const double2 *__restrict__ ycur, int p,
                                                      float2 *__restrict__ f0, float2 *__restrict__ f0lo) {
  const double2 F = br.eval<kArithFusedSoftMul>(ycur, p);
  const float hx = softfp::to_float(F.x), hy = softfp::to_float(F.y);
  f0[p] = make_float2(hx, hy);
  f0lo[p] = make_float2(softfp::to_float(F.x - static_cast<double>(hx)),
                        softfp::to_float(F.y - static_cast<double>(hy)));
}

// kMaxS: an upper bound of the stage count (8 or 13), so that the per-stage
// loops over earlier stages unroll; kPath: how the FP32 stages walk the grid.
template <int kMaxS, int kPath>
__global__ void __launch_bounds__(mix_threads(kPath), kPath == kMixFused ? 1024 / kFusedThreads : (kMaxS <= 8 ? 4 : 2))
    mixed_kernel(const __grid_constant__ MixedParams P) {
  // TMA staging buffers: 2 (double buffer) x s slots of kSlotBytes, from the
  // first 128-byte boundary of the dynamic shared memory (128 bytes spare)
  extern __shared__ __align__(128) unsigned char s_dyn[];
  unsigned char *const s_box = s_dyn + ((128u - (smem_u32(s_dyn) & 127u)) & 127u);
  __shared__ __align__(8) uint64_t s_mbar[2];
  __shared__ double s_t, s_h;
  __shared__ int s_acc, s_rej, s_cur, s_done;
  __shared__ unsigned long long s_step;
  constexpr int kT = mix_threads(kPath);
  __shared__ double s_wmax[kT / 32];
  __shared__ float hb[kMaxStages], hc[kMaxStages];
  __shared__ MixCoef s_coef;
  // per stage i: the j < i with a_ij != 0 (j = 1 always, as the running sums
  // of the scatter order start there) and h a_ij, for the gather
  __shared__ const float2 *s_jp[kMaxStages][kMaxStages];
  __shared__ int s_jl[kMaxStages][kMaxStages];
  __shared__ float s_ja[kMaxStages][kMaxStages];
  __shared__ int s_nj[kMaxStages];
  __shared__ float s_hbs_hi, s_hbs_lo;  // h sum(b) as a double-float pair
  __shared__ float2 s_delta[kTileR + 2][kTileC + 2];  // delta_i on a tile and its halo

  DevState *st = P.st;
  const int s = P.s;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gstride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Bruss &br = P.bruss;
  const float coef = static_cast<float>(br.coef);
  const dfl::df coef_df = {coef, static_cast<float>(br.coef - static_cast<double>(coef))};

  if (threadIdx.x == 0) {
    s_t = st->t;
    s_h = st->h;
    s_acc = st->steps_acc;
    s_rej = st->steps_rej;
    s_cur = st->cur;
    s_done = st->done;
    s_step = st->step;
  }
  if (threadIdx.x == 0 && (kPath == kMixTilesTma || kPath == kMixFused)) {
    mbar_init(&s_mbar[0], 1);
    mbar_init(&s_mbar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  unsigned phase = 0;    // parity of the next completion of each TMA buffer (bits 0, 1)
  unsigned pending = 0;  // buffers with copies issued and not yet waited for (bits 0, 1)

  bool ok = true;
  for (int it = 0; it < P.budget; ++it) {
    if (s_done) break;
    const double h = s_h;
    if (threadIdx.x < kMaxStages) {
      const int i = threadIdx.x;
      int nj = 0;
      for (int j = 1; j < i && i < s; ++j) {
        if (j > 1 && !P.nzA[i * kMaxStages + j]) continue;
        s_jp[i][nj] = P.dF[j];
        s_jl[i][nj] = j;
        s_ja[i][nj] = static_cast<float>(h * P.A[i * kMaxStages + j]);
        ++nj;
      }
      s_nj[i] = nj;
    }
    if (threadIdx.x < kMaxStages) {
      const int j = threadIdx.x;
      hb[j] = static_cast<float>(h * P.b[j]);
      hc[j] = static_cast<float>(h * P.csum[j]);
      const double hbh = h * P.bh[j];
      s_coef.hb[j] = hb[j];
      s_coef.hbh_hi[j] = static_cast<float>(hbh);
      s_coef.hbh_lo[j] = static_cast<float>(hbh - static_cast<double>(s_coef.hbh_hi[j]));
    }
    if (threadIdx.x == 0) {
      const double hbs = h * P.bsum;
      s_hbs_hi = static_cast<float>(hbs);
      s_hbs_lo = static_cast<float>(hbs - static_cast<double>(s_hbs_hi));
      const double hbhs = h * P.bhsum;
      s_coef.hbhs_hi = static_cast<float>(hbhs);
      s_coef.hbhs_lo = static_cast<float>(hbhs - static_cast<double>(s_coef.hbhs_hi));
    }
    __syncthreads();
    const double2 *__restrict__ ycur = P.y[s_cur];
    double2 *__restrict__ ynew = P.y[s_cur ^ 1];

    // stage 0: F0 = f(y) in double-float (fixed-point Laplacian, FP32 pairs),
    // stored as its leading (f0) and trailing (f0lo) floats, and y rounded to
    // FP32; a point whose values fall outside the double-float ranges takes
    // the FP64 evaluation
    {
      const int N = br.N;
      // grid point (k, j) of pair p, advanced by the grid stride without a division
      const int dk = gstride / N, dj = gstride - dk * N;
      int k = gtid / N, j = gtid - (gtid / N) * N;
      // four points in flight per thread: their loads overlap (1.4 % of a step)
#pragma unroll 4
      for (int p = gtid; p < P.npairs; p += gstride, j += dj, k += dk) {
        if (j >= N) {
          j -= N;
          ++k;
        }
        const double2 *row = ycur + (p - j);
        const double2 c = row[j];
        const double2 up = (k == 0 ? row + N : row - N)[j];
        const double2 dn = (k == N - 1 ? row - N : row + N)[j];
        // a boundary column passes its inner neighbour twice
        const double2 w = row[j == 0 ? 1 : j - 1];
        const double2 e = row[j == N - 1 ? j - 1 : j + 1];
        dfl::df fu, fv;
        if (dfl::bruss_rhs_df(c, up, dn, w, e, coef_df, &fu, &fv)) {
          P.f0[p] = make_float2(fu.hi, fv.hi);
          P.f0lo[p] = make_float2(fu.lo, fv.lo);
        } else {
          stage0_point_fp64(br, ycur, p, P.f0, P.f0lo);
        }
        P.y32[p] = make_float2(trunc_to_float(c.x), trunc_to_float(c.y));
      }
    }
    if (kPath == kMixTilesTma || kPath == kMixFused) fence_proxy_async_global();  // f0, y32 are read by TMA next
    if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 11))) break;

    float emax = 0.0f;
    const int N = br.N;
    const dfl::df hbd = {s_hbs_hi, s_hbs_lo};  // h sum(b)
    if constexpr (kPath == kMixFused) {
      // All FP32 stages per tile (FusedGeom): F0 and y32 frames through TMA,
      // double-buffered; delta_i and dF_i in shared-memory frames.
      using G = FusedGeom<kMaxS>;
      auto frame = [&](int f) { return reinterpret_cast<float2 *>(s_box + static_cast<size_t>(f) * G::kFrameBytes); };
      const int tiles_x = (N + kFTC - 1) / kFTC;
      const int ntiles = tiles_x * ((N + kFTR - 1) / kFTR);
      auto issue = [&](int t, int b) {
        const int k0 = (t / tiles_x) * kFTR, j0 = (t % tiles_x) * kFTC;
        mbar_arrive_expect_tx(&s_mbar[b], 2u * G::kFrame * 8u);
        tma_load_2d(frame(2 * b), &P.tm[0], 2 * (j0 - G::HX), k0 - G::HY, &s_mbar[b]);
        tma_load_2d(frame(2 * b + 1), &P.tm[1], 2 * (j0 - G::HX), k0 - G::HY, &s_mbar[b]);
      };
      int b = 0;
      __syncthreads();  // the frames are free (the previous step is done with them)
      if (blockIdx.x < ntiles) {
        if (threadIdx.x == 0) issue(blockIdx.x, 0);
        pending |= 1u;
      }
      // A thread whose wait ran out of time skips the tile's work; the CTA
      // agrees on it at the next tile's first barrier (the solve then ends
      // with the error set).
      bool bad = false;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x, b ^= 1) {
        const int tn = t + gridDim.x;
        if (__syncthreads_or(bad)) break;  // buffer b^1, delta and the dF frames are free
        if (tn < ntiles) {
          if (threadIdx.x == 0) issue(tn, b ^ 1);
          pending |= 2u >> b;  // bit of buffer b^1
        }
        const bool got = mbar_wait(&s_mbar[b], (phase >> b) & 1u, st, P.timeout_ns, 16);
        bad = bad || !got;
        if (got) {
          phase ^= 1u << b;
          pending &= ~(1u << b);
        }
        const int k0 = (t / tiles_x) * kFTR, j0 = (t % tiles_x) * kFTC;
        const float2 *const ff0 = frame(2 * b), *const fy32 = frame(2 * b + 1);
        // A tile whose regions lie inside the grid away from its edges (all but
        // the outermost ring of tiles) needs no bounds checks and no boundary
        // stencils: its loops are compiled without them.
        const bool interior = k0 >= kMaxS - 1 && j0 >= kMaxS - 1 && k0 + kFTR + kMaxS - 1 <= N &&
                              j0 + kFTC + kMaxS - 1 <= N;
        auto stages = [&](auto interior_c) {
          constexpr bool kIn = decltype(interior_c)::value;
          // One pass per stage i over the tile and a halo of s-1-i points:
          // dF_i from delta_i's stencil, and at the same point delta_{i+1} =
          // h c_{i+1} F0 + sum_{j<=i} h a_{i+1,j} dF_j (the region the next
          // stage's stencil reads); delta_1 = h c_1 F0 comes from F0 itself.
          static_for<1, kMaxS>([&](auto ic) {
            constexpr int i = decltype(ic)::value;
            constexpr bool kLast = i == kMaxS - 1;
            constexpr int dq = kMaxS - 1 - i, RQ = kFTC + 2 * dq, RR = kFTR + 2 * dq;  // region cols, rows
            constexpr int eb_q = (G::HY - dq) * G::FC + (G::HX - dq);
            constexpr int kJ = i;  // delta_{i+1} sums over j = 1 .. i
            const float2 *const fdi = i == 1 ? ff0 : frame(G::kDelta + (i & 1));
            const float sdi = i == 1 ? hc[1] : 1.0f;  // delta_1 = h c_1 F0
            float2 *const fdn = frame(G::kDelta + ((i + 1) & 1));
            const int nj = kLast ? 0 : s_nj[i + 1];
            const float hcn = kLast ? 0.0f : hc[i + 1];
            const float2 *jf[kJ];
            float ja[kJ];
            int jl[kJ];
#pragma unroll
            for (int kk = 0; kk < kJ; ++kk) {
              jl[kk] = kk < nj ? s_jl[i + 1][kk] : 0;
              ja[kk] = kk < nj ? s_ja[i + 1][kk] : 0.0f;
              jf[kk] = frame(G::kDF + (jl[kk] >= 1 && jl[kk] < i ? jl[kk] : 1));
            }
            for (int idx = threadIdx.x; got && idx < RR * RQ; idx += kFusedThreads) {
              const int r = idx / RQ, c = idx - r * RQ;
              const int k = k0 - dq + r, j = j0 - dq + c;
              const int e = eb_q + r * G::FC + c;
              int eu = e - G::FC, en = e + G::FC, jcase = 0;
              if constexpr (!kIn) {
                if (static_cast<unsigned>(k) >= static_cast<unsigned>(N) ||
                    static_cast<unsigned>(j) >= static_cast<unsigned>(N))
                  continue;
                // a boundary row or column uses its inner neighbour twice
                if (k == 0) eu = en;
                if (k == N - 1) en = eu;
                jcase = j == 0 ? 1 : (j == N - 1 ? 2 : 0);
              }
              auto dl = [&](int x) {
                const float2 v = fdi[x];
                return i == 1 ? make_float2(fmaf(sdi, v.x, 0.0f), fmaf(sdi, v.y, 0.0f)) : v;
              };
              const float2 dF = delta_rhs(dl(e), dl(eu), dl(en), dl(e - 1), dl(e + 1), jcase, fy32[e], coef);
              if constexpr (!kLast) {
                if constexpr (i <= kMaxS - 2) frame(G::kDF + i)[e] = dF;
                float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int kk = 0; kk < kJ; ++kk) {
                  if (kk < nj) {
                    const float2 d = jl[kk] == i ? dF : jf[kk][e];
                    acc.x = fmaf(ja[kk], d.x, acc.x);
                    acc.y = fmaf(ja[kk], d.y, acc.y);
                  }
                }
                const float2 f = ff0[e];
                fdn[e] = make_float2(fmaf(hcn, f.x, acc.x), fmaf(hcn, f.y, acc.y));
              } else {
                // the last stage: the update and the error ratio at the tile's point
                float2 dall[kMaxS];
                dall[0] = make_float2(0.f, 0.f);
#pragma unroll
                for (int jj = 1; jj < kMaxS - 1; ++jj) dall[jj] = frame(G::kDF + jj)[e];
                const size_t p = static_cast<size_t>(k) * N + j;
                float rx, ry;
                ynew[p] = mix_update<kMaxS>(dall, dF, kMaxS, ff0[e], P.f0lo[p], fy32[e], ycur[p], hbd, s_coef,
                                            &rx, &ry);
                emax = fmaxf(emax, rx);
                if (2 * p + 1 < static_cast<size_t>(P.n)) emax = fmaxf(emax, ry);
              }
            }
            if constexpr (!kLast) __syncthreads();
          });
        };
        if (interior)
          stages(std::true_type{});
        else
          stages(std::false_type{});
      }
      if (__syncthreads_or(bad)) ok = false;
      if (!ok) break;
    } else {
    const int tiles_x = (N + kTileC - 1) / kTileC;
    const int ntiles = tiles_x * ((N + kTileR - 1) / kTileR);
    const int tr = threadIdx.x / kTileC, tc = threadIdx.x % kTileC;
    for (int i = 1; i < s; ++i) {
      const bool last = (i == s - 1);
      const float2 *const *jp = s_jp[i];
      const float *ja = s_ja[i];
      const int nj = s_nj[i];
      const float hci = hc[i];
      // dF_i (and, in the last stage, dY, e and y_new) at grid point p from
      // delta_i on the tile (s_delta), y32, and the point's own dF_j / f0
      auto finish_point_at = [&](int p, int k, int j, float2 c, float2 up, float2 dn, float2 w,
                                 float2 e, float2 y32, auto &&own_dF, auto &&own_f0) {
        const int jcase = j == 0 ? 1 : (j == N - 1 ? 2 : 0);
        const float2 dF = delta_rhs(c, up, dn, w, e, jcase, y32, coef);
        if (!last) {
          P.dF[i][p] = dF;
          return;
        }
        // dY, y_new and the error estimate, in order of the stages
        float2 dall[kMaxS];
        dall[0] = make_float2(0.f, 0.f);
#pragma unroll
        for (int jj = 1; jj < kMaxS; ++jj)
          if (jj < s - 1) dall[jj] = own_dF(jj);
        float rx, ry;
        ynew[p] = mix_update<kMaxS>(dall, dF, s, own_f0(), P.f0lo[p], y32, ycur[p], hbd, s_coef, &rx, &ry);
        emax = fmaxf(emax, rx);
        if (2 * p + 1 < P.n) emax = fmaxf(emax, ry);
      };
      auto finish_point = [&](int tr_, int tc_, int k, int j, float2 y32, auto &&own_dF,
                              auto &&own_f0) {
        finish_point_at(k * N + j, k, j, s_delta[tr_ + 1][tc_ + 1],
                        s_delta[k == 0 ? tr_ + 2 : tr_][tc_ + 1],
                        s_delta[k == N - 1 ? tr_ : tr_ + 2][tc_ + 1], s_delta[tr_ + 1][tc_],
                        s_delta[tr_ + 1][tc_ + 2], y32, own_dF, own_f0);
      };

      if constexpr (kPath == kMixTilesTma) {
        // Tiles through TMA, double-buffered: while tile t is evaluated, the
        // boxes of the CTA's next tile are in flight.  Box slot 0: f0, 1: y32,
        // 1 + j: dF_j for j < i.
        const int nvec = 1 + i;
        const unsigned tile_bytes = nvec * kBoxBytes;
        auto slot = [&](int b, int v) {
          return reinterpret_cast<const float2 *>(s_box + (static_cast<size_t>(b) * s + v) * kSlotBytes);
        };
        auto issue = [&](int t, int b) {
          const int k0 = (t / tiles_x) * kTileR, j0 = (t % tiles_x) * kTileC;
          mbar_arrive_expect_tx(&s_mbar[b], tile_bytes);
          for (int v = 0; v < nvec; ++v)
            tma_load_2d(s_box + (static_cast<size_t>(b) * s + v) * kSlotBytes, &P.tm[v],
                        2 * (j0 - 2), k0 - 1, &s_mbar[b]);
        };
        int b = 0;
        __syncthreads();  // the buffers are free (the previous stage is done with them)
        if (blockIdx.x < ntiles) {
          if (threadIdx.x == 0) issue(blockIdx.x, 0);
          pending |= 1u;
        }
        // A thread whose wait ran out of time skips the tile; the CTA agrees on
        // it at the next barrier (the solve then ends with the error set).
        bool bad = false;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, b ^= 1) {
          const int tn = t + gridDim.x;
          if (__syncthreads_or(bad)) break;  // buffer b^1 and s_delta are free
          if (tn < ntiles) {
            if (threadIdx.x == 0) issue(tn, b ^ 1);
            pending |= 2u >> b;  // bit of buffer b^1
          }
          const int k0 = (t / tiles_x) * kTileR, j0 = (t % tiles_x) * kTileC;
          const bool got = mbar_wait(&s_mbar[b], (phase >> b) & 1u, st, P.timeout_ns, 14);
          bad = bad || !got;
          if (got) {  // (a wait that ran out keeps the parity, for the final wait)
            phase ^= 1u << b;
            pending &= ~(1u << b);
          }
          const float2 *bf0 = slot(b, 0);
          // delta_i on the tile and its halo, with the stage's term count as a
          // compile-time constant (no predicated-off terms in the early stages)
          auto halo = [&](auto nj_c) {
            constexpr int kNj = decltype(nj_c)::value;
            for (int hh = threadIdx.x; got && hh < (kTileR + 2) * (kTileC + 2); hh += blockDim.x) {
              const int hr = hh / (kTileC + 2), hcl = hh % (kTileC + 2);
              const int k = k0 + hr - 1, j = j0 + hcl - 1;
              if (k < 0 || k >= N || j < 0 || j >= N) continue;
              const int e = hr * kBoxPairs + hcl + 1;
              float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
              for (int kk = 0; kk < kNj; ++kk) {
                const float2 d = slot(b, 1 + s_jl[i][kk])[e];
                acc.x = fmaf(ja[kk], d.x, acc.x);
                acc.y = fmaf(ja[kk], d.y, acc.y);
              }
              const float2 f = bf0[e];
              s_delta[hr][hcl] = make_float2(fmaf(hci, f.x, acc.x), fmaf(hci, f.y, acc.y));
            }
          };
          switch (nj) {
            case 0: halo(std::integral_constant<int, 0>{}); break;
            case 1: halo(std::integral_constant<int, 1>{}); break;
            case 2: halo(std::integral_constant<int, 2>{}); break;
            case 3: halo(std::integral_constant<int, 3>{}); break;
            case 4: halo(std::integral_constant<int, 4>{}); break;
            case 5: halo(std::integral_constant<int, 5>{}); break;
            default: halo(std::integral_constant<int, (kMaxS - 2 > 6 ? 6 : kMaxS - 2)>{}); break;
          }
          __syncthreads();
          const int k = k0 + tr, j = j0 + tc;
          if (got && k < N && j < N) {
            const int eo = (tr + 1) * kBoxPairs + tc + 2;  // the point itself in a box
            finish_point(tr, tc, k, j, slot(b, 1)[eo],
                         [&](int jj) { return slot(b, 1 + jj)[eo]; },
                         [&]() { return bf0[eo]; });
          }
        }
        if (__syncthreads_or(bad)) ok = false;
        if (!ok) break;
        fence_proxy_async_global();  // dF_i is read by TMA in later stages
      } else {
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
          // delta_i on the tile and a one-point halo (rows and columns outside
          // the grid are not needed: a boundary uses the inner neighbour twice)
          const int k0 = (t / tiles_x) * kTileR, j0 = (t % tiles_x) * kTileC;
          __syncthreads();  // the previous tile's reads of s_delta are done
          for (int hh = threadIdx.x; hh < (kTileR + 2) * (kTileC + 2); hh += blockDim.x) {
            const int hr = hh / (kTileC + 2), hcl = hh % (kTileC + 2);
            const int k = k0 + hr - 1, j = j0 + hcl - 1;
            if (k >= 0 && k < N && j >= 0 && j < N)
              s_delta[hr][hcl] = delta_at<kMaxS - 2>(jp, ja, nj, P.f0, hci, k * N + j);
          }
          __syncthreads();
          const int k = k0 + tr, j = j0 + tc;
          if (k >= N || j >= N) continue;
          const int p = k * N + j;
          finish_point(tr, tc, k, j, P.y32[p], [&](int jj) { return P.dF[jj][p]; },
                       [&]() { return P.f0[p]; });
        }
      }
      if (!last) {
        if (!(ok = grid_barrier(st, P.nblocks, P.timeout_ns, 12))) break;
      }
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
      for (int k = 1; k < kT / 32; ++k) m = fmax(m, s_wmax[k]);
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

  // after a failed wait, let the copies still in flight land before the CTA
  // leaves (bounded as well)
  if (pending && threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b)
      if ((pending >> b) & 1u) mbar_wait(&s_mbar[b], (phase >> b) & 1u, st, P.timeout_ns, 15);
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

// cuTensorMapEncodeTiled from the driver, found once through the runtime
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    else
      cudaGetLastError();
  }
  return fn;
}

// 2-D map of an N x N grid of float2 pairs (rows of 2N floats) with boxes of
// box_rows rows x box_pairs pairs; false if the layout does not allow TMA.
static bool encode_box_map(CUtensorMap *m, const float2 *base, int N, int box_pairs = kBoxPairs,
                           int box_rows = kBoxRows) {
  auto fn = encode_fn();
  if (!fn || N % 2 || (reinterpret_cast<uintptr_t>(base) & 15)) return false;
  const cuuint64_t dims[2] = {2ull * N, static_cast<cuuint64_t>(N)};
  const cuuint64_t strides[1] = {8ull * N};  // bytes between rows: a multiple of 16 for even N
  const cuuint32_t box[2] = {2u * static_cast<cuuint32_t>(box_pairs), static_cast<cuuint32_t>(box_rows)};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2 *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The fused path's kernel, shared memory and TMA box for s stages (2..8).
struct FusedShape {
  const void *kern;
  size_t smem;
  int box_pairs, box_rows;
};
template <int kS>
static FusedShape fused_shape() {
  return {(const void *)mixed_kernel<kS, kMixFused>, FusedGeom<kS>::kSmem, FusedGeom<kS>::FC,
          FusedGeom<kS>::FR};
}
static bool fused_shape_of(int s, FusedShape *out) {
  switch (s) {
    case 2: *out = fused_shape<2>(); return true;
    case 3: *out = fused_shape<3>(); return true;
    case 4: *out = fused_shape<4>(); return true;
    case 5: *out = fused_shape<5>(); return true;
    case 6: *out = fused_shape<6>(); return true;
    case 7: *out = fused_shape<7>(); return true;
    case 8: *out = fused_shape<8>(); return true;
    default: return false;
  }
}

bool mixed_fused_available(int N, int s) {
  FusedShape f;
  return encode_fn() != nullptr && N % 2 == 0 && fused_shape_of(s, &f);
}

cudaError_t launch_mixed(const MixedParams &p, int path, int num_sms, cudaStream_t stream,
                         int *grid_out) {
  MixedParams q = p;
  const void *kern = nullptr;
  size_t dyn = 0;
  int threads = kMixThreads;
  int useful = (p.npairs + kMixThreads - 1) / kMixThreads;
  if (path == kMixFused) {
    // needs mixed_fused_available(N, s); the dF vectors are not allocated then
    FusedShape f;
    if (!fused_shape_of(p.s, &f) ||
        !encode_box_map(&q.tm[0], p.f0, p.bruss.N, f.box_pairs, f.box_rows) ||
        !encode_box_map(&q.tm[1], p.y32, p.bruss.N, f.box_pairs, f.box_rows))
      return cudaErrorInvalidValue;
    q.path = kMixFused;
    kern = f.kern;
    dyn = f.smem;
    threads = kFusedThreads;
    useful = ((p.bruss.N + kFTC - 1) / kFTC) * ((p.bruss.N + kFTR - 1) / kFTR);
  } else {
    q.path = kMixTiles;
    if (path == kMixTilesTma && p.s <= kMixTmaStages) {
      bool good = encode_box_map(&q.tm[0], p.f0, p.bruss.N) && encode_box_map(&q.tm[1], p.y32, p.bruss.N);
      for (int j = 1; good && j <= p.s - 2; ++j) good = encode_box_map(&q.tm[1 + j], p.dF[j], p.bruss.N);
      if (good) q.path = kMixTilesTma;
    }
    // one instantiation per path, so that each gets its own register allocation
    kern = p.s > 8                  ? (const void *)mixed_kernel<kMaxStages, kMixTiles>
           : q.path == kMixTilesTma ? (const void *)mixed_kernel<8, kMixTilesTma>
                                    : (const void *)mixed_kernel<8, kMixTiles>;
    dyn = q.path == kMixTilesTma ? 2ull * p.s * kSlotBytes + 128 : 0;
  }
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, dyn);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  int grid = occ * num_sms;
  if (grid > useful) grid = useful > 0 ? useful : 1;
  q.nblocks = grid + (p.extra_arrivals > 0 ? p.extra_arrivals : 0);
  void *args[] = {&q};
  *grid_out = grid;
  return cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(threads), args, dyn, stream);
}

}  // namespace rkcu
