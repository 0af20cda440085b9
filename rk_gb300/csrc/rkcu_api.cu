// C ABI of the step loop (include/rkcu.h): solver objects, device buffers,
// launches and the problem-module helpers.  Host code only; the kernels are in
// rkcu_plain.cu.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <new>

#include "rkcu.h"
#include "rkcu_general.cuh"
#include "rkcu_lowstorage.cuh"
#include "rkcu_mixed.cuh"
#include "rkcu_plain.cuh"

using rkcu::DevState;
using rkcu::kMaxStages;

namespace {

// Text behind rkcu_last_cuda_error(), per host thread.
thread_local char g_cuda_err[256] = "";

int cuda_fail(cudaError_t e, const char *what) {
  std::snprintf(g_cuda_err, sizeof(g_cuda_err), "%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? RKCU_ERR_NOMEM : RKCU_ERR_CUDA;
}

}  // namespace

namespace rkcu {

int record_cuda_error(cudaError_t e, const char *what) { return cuda_fail(e, what); }

int record_wait_timeout(int site) {
  std::snprintf(g_cuda_err, sizeof(g_cuda_err), "device wait timed out at site %d", site);
  return RKCU_ERR_TIMEOUT;
}

}  // namespace rkcu

namespace {

#define RKCU_CK(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

size_t pairs_of(int n) { return (static_cast<size_t>(n) + 1) / 2; }

int check_problem(const rkcu_problem *p) {
  if (!p || p->n <= 0) return RKCU_ERR_INVALID;
  switch (p->problem) {
    case RKCU_PROBLEM_BRUSS2D_MIX:
      if (p->grid_n < 2 || static_cast<long long>(p->n) != 2LL * p->grid_n * p->grid_n)
        return RKCU_ERR_INVALID;
      return RKCU_OK;
    case RKCU_PROBLEM_LV_PAIRS:
      return (p->n % 2 == 0) ? RKCU_OK : RKCU_ERR_INVALID;
    case RKCU_PROBLEM_LV_BANDED:
      return (p->lv_r && p->lv_a) ? RKCU_OK : RKCU_ERR_INVALID;
    default:
      return RKCU_ERR_INVALID;
  }
}

// (alpha * (N-1)) * (N-1): the association of "BRUSS_ALPHA * N1 * N1" in
// src/problems/bruss2d-mix.c:84
double bruss_coef(const rkcu_problem *p) {
  const double n1 = static_cast<double>(p->grid_n) - 1.0;
  return p->alpha * n1 * n1;
}

}  // namespace

struct rkcu_solver {
  rkcu_problem prob{};
  rkcu_options opt{};
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // tableau
  bool have_method = false;
  int s = 0, ord = 0;
  double A[kMaxStages * kMaxStages] = {};
  double b[kMaxStages] = {}, bh[kMaxStages] = {}, c[kMaxStages] = {};
  // caller's right-hand side (RKCU_PROBLEM_RHS)
  rkcu_rhs_fn rhs = nullptr;
  void *rhs_user = nullptr;
  // device memory
  size_t npairs = 0;
  double2 *y[2] = {nullptr, nullptr};
  double2 *stage = nullptr;  // w[1..s-1], dy, err
  int stage_vectors = 0;
  float2 *mstage = nullptr;  // mixed form: f0, y32, dF[1..s-2]
  int mstage_vectors = 0;
  double2 *rings = nullptr;  // low-storage form: ring buffers
  size_t ring_pairs = 0;
  int ls_rows = 0;
  double *lv_r = nullptr, *lv_a = nullptr;
  DevState *st = nullptr;
  DevState *st_host = nullptr;  // pinned
  rkcu::PowBox *h_box = nullptr;  // step-size mailbox, mapped pinned host memory
  rkcu::PowBox *d_box = nullptr;  // its device address
  bool polling = false;           // the calling thread answers the mailbox (rkcu_run, rkcu_solve)
  unsigned int *flags = nullptr;  // plain kernel: per-CTA stage progress
  // per-step trace (plain form)
  int trace_cap = 0;
  double *trace_meta = nullptr;  // 3 doubles per step: t, h, error max
  double2 *trace_y = nullptr;    // npairs per step, or none
  // run
  bool begun = false;
  double te = 0.0, tol = 0.0;
  long long launches = 0;
  long long dev_bytes = 0;
  int last_grid = 0;
  int extra_arrivals = 0;
};

// Tiles of the flow schedule: BRUSS2D-MIX tiles are block_rows grid rows (one
// by default), so a stage reads one tile either side; the LV chains use tiles
// of 2048 pairs (pairs: no neighbours; banded: one pair either side).
static void flow_geometry(const rkcu_solver *s, int *tile, int *ntiles, int *dep) {
  const int np = (int)s->npairs;
  int t, d;
  if (s->prob.problem == RKCU_PROBLEM_BRUSS2D_MIX) {
    const int rows = s->opt.block_rows > 0 ? s->opt.block_rows : 1;
    t = rows * s->prob.grid_n;
    d = 1;
  } else {
    t = 2048;
    d = s->prob.problem == RKCU_PROBLEM_LV_BANDED ? 1 : 0;
  }
  if (t > np) t = np > 0 ? np : 1;
  *tile = t;
  *ntiles = (np + t - 1) / t;
  *dep = d;
}

// The step loop of src/impl/seq/A.c:57-85 around the caller's right-hand side:
// stage vectors F_0..F_{s-1} and w in the solver's stage storage, one state
// read-back per step (the host passes t + h c_l to the function).  Stops after
// a step whose size update is left to the host, as the fused kernels do.
static int advance_rhs(rkcu_solver *s, int max_steps) {
  const int mode = s->opt.precision == RKCU_FP64_EXACT        ? rkcu::kArithExactSoftMul
                   : s->opt.precision == RKCU_FP64_EXACT_HWMUL ? rkcu::kArithExact
                                                               : rkcu::kArithFused;
  const size_t ld = 2 * s->npairs;  // doubles per stage vector
  double *F = reinterpret_cast<double *>(s->stage);
  double *w = F + (size_t)s->s * ld;
  const long long n = s->prob.n;
  DevState *h = s->st_host;
  rkcu::GenCoef cf;
  std::memset(&cf, 0, sizeof(cf));
  cf.s = s->s;
  for (int k = 0; k < max_steps; ++k) {
    if (h->done || h->pending || h->error) break;
    // premult (src/methods.c:43-58)
    const double hh = h->h, t = h->t;
    double hc[kMaxStages];
    for (int i = 0; i < s->s; ++i) {
      for (int j = 0; j < i; ++j) {
        cf.hA[i * kMaxStages + j] = hh * s->A[i * kMaxStages + j];
        cf.nzA[i * kMaxStages + j] = s->A[i * kMaxStages + j] != 0.0;
      }
      cf.hb[i] = hh * s->b[i];
      cf.hbh[i] = hh * s->bh[i];
      cf.nzb[i] = s->b[i] != 0.0;
      cf.nzbh[i] = s->bh[i] != 0.0;
      hc[i] = hh * s->c[i];
    }
    const double *ycur = reinterpret_cast<const double *>(s->y[h->cur & 1]);
    double *ynew = reinterpret_cast<double *>(s->y[(h->cur & 1) ^ 1]);
    if (s->rhs(t + hc[0], ycur, F, (int)n, (void *)s->stream, s->rhs_user) != 0) return RKCU_ERR_RHS;
    for (int l = 1; l < s->s; ++l) {
      cudaError_t e = rkcu::launch_gen_combine(cf, l, ycur, F, ld, w, n, mode, s->num_sms, s->stream);
      if (e != cudaSuccess) return cuda_fail(e, "combine kernel");
      if (s->rhs(t + hc[l], w, F + (size_t)l * ld, (int)n, (void *)s->stream, s->rhs_user) != 0)
        return RKCU_ERR_RHS;
    }
    cudaError_t e = rkcu::launch_gen_output(cf, ycur, F, ld, ynew, n, s->st, mode, s->num_sms, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "output kernel");
    e = rkcu::launch_gen_control(s->st, s->tol, s->ord, s->te, s->opt.step_limit, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "step control kernel");
    s->launches += s->s + 1;
    RKCU_CK(cudaMemcpyAsync(h, s->st, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
    RKCU_CK(cudaStreamSynchronize(s->stream));
  }
  return RKCU_OK;
}

extern "C" {

void rkcu_options_default(rkcu_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = RKCU_FP64_EXACT;
  o->variant = RKCU_VARIANT_D;
  o->step_limit = 0;
  o->device = 0;
  o->stream = nullptr;
  o->wait_timeout_s = 10.0;
  o->h_init = 0.0;
}

const char *rkcu_strerror(int status) {
  switch (status) {
    case RKCU_OK: return "ok";
    case RKCU_ERR_INVALID: return "invalid argument";
    case RKCU_ERR_CUDA: return "CUDA error";
    case RKCU_ERR_NOMEM: return "out of memory";
    case RKCU_ERR_TIMEOUT: return "device wait timed out";
    case RKCU_ERR_STATE: return "call out of order";
    case RKCU_ERR_NO_DEVICE: return "no usable CUDA device";
    case RKCU_ERR_TOO_LARGE: return "system larger than the allocation-free limit (65536 components)";
    case RKCU_ERR_RHS: return "the caller's right-hand side failed";
    default: return "unknown status";
  }
}

const char *rkcu_last_cuda_error(void) { return g_cuda_err; }

int rkcu_destroy(rkcu_solver *s) {
  if (!s) return RKCU_ERR_INVALID;
  cudaSetDevice(s->opt.device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  cudaFree(s->y[0]);
  cudaFree(s->y[1]);
  cudaFree(s->stage);
  cudaFree(s->mstage);
  cudaFree(s->rings);
  cudaFree(s->lv_r);
  cudaFree(s->lv_a);
  cudaFree(s->st);
  cudaFree(s->flags);
  cudaFree(s->trace_meta);
  cudaFree(s->trace_y);
  cudaFreeHost(s->st_host);
  if (s->h_box) cudaFreeHost(s->h_box);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return RKCU_OK;
}

int rkcu_create(rkcu_solver **out, const rkcu_problem *prob, const rkcu_options *opt) {
  if (!out) return RKCU_ERR_INVALID;
  *out = nullptr;
  const bool general = prob && prob->problem == RKCU_PROBLEM_RHS;
  int rc = general ? (prob->n > 0 ? RKCU_OK : RKCU_ERR_INVALID) : check_problem(prob);
  if (rc != RKCU_OK) return rc;
  rkcu_options o;
  if (opt)
    o = *opt;
  else
    rkcu_options_default(&o);
  if (o.precision != RKCU_FP64_EXACT && o.precision != RKCU_FP64_FMA && o.precision != RKCU_MIXED &&
      o.precision != RKCU_FP64_EXACT_HWMUL)
    return RKCU_ERR_INVALID;
  if (o.precision == RKCU_MIXED && prob->problem != RKCU_PROBLEM_BRUSS2D_MIX) return RKCU_ERR_INVALID;
  if (general && o.variant != RKCU_VARIANT_D) return RKCU_ERR_INVALID;
  if (o.variant != RKCU_VARIANT_D && o.variant != RKCU_VARIANT_LOWSTORAGE) return RKCU_ERR_INVALID;
  if (o.variant == RKCU_VARIANT_LOWSTORAGE &&
      (prob->problem != RKCU_PROBLEM_BRUSS2D_MIX || o.precision == RKCU_MIXED || o.block_rows < 0))
    return RKCU_ERR_INVALID;
  if (o.step_limit < 0) return RKCU_ERR_INVALID;
  if (!(o.wait_timeout_s > 0.0)) o.wait_timeout_s = 10.0;
  if (!(o.h_init >= 0.0)) return RKCU_ERR_INVALID;
  if (o.schedule < 0 || o.schedule > 4 || o.flow_skew < 0) return RKCU_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= o.device || o.device < 0)
    return RKCU_ERR_NO_DEVICE;

  rkcu_solver *s = new (std::nothrow) rkcu_solver();
  if (!s) return RKCU_ERR_NOMEM;
  s->prob = *prob;
  s->prob.lv_r = s->prob.lv_a = nullptr;
  s->opt = o;
  s->npairs = pairs_of(prob->n);
  auto fail = [&](int code) {
    rkcu_destroy(s);
    return code;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(o.device)) != cudaSuccess) return fail(cuda_fail(e, "cudaSetDevice"));
  if ((e = cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, o.device)) !=
      cudaSuccess)
    return fail(cuda_fail(e, "cudaDeviceGetAttribute"));
  if (o.stream) {
    s->stream = static_cast<cudaStream_t>(o.stream);
  } else {
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess)
      return fail(cuda_fail(e, "cudaStreamCreate"));
    s->own_stream = true;
  }
  const size_t ybytes = s->npairs * sizeof(double2);
  for (int k = 0; k < 2; ++k) {
    if ((e = cudaMalloc(&s->y[k], ybytes)) != cudaSuccess) return fail(cuda_fail(e, "cudaMalloc y"));
    if ((e = cudaMemset(s->y[k], 0, ybytes)) != cudaSuccess) return fail(cuda_fail(e, "cudaMemset"));
    s->dev_bytes += ybytes;
  }
  if ((e = cudaMalloc(&s->st, sizeof(DevState))) != cudaSuccess)
    return fail(cuda_fail(e, "cudaMalloc state"));
  if ((e = cudaMallocHost(&s->st_host, sizeof(DevState))) != cudaSuccess)
    return fail(cuda_fail(e, "cudaMallocHost"));
  if ((e = cudaHostAlloc(&s->h_box, sizeof(rkcu::PowBox), cudaHostAllocMapped | cudaHostAllocPortable)) !=
      cudaSuccess)
    return fail(cuda_fail(e, "step-size mailbox"));
  std::memset(s->h_box, 0, sizeof(rkcu::PowBox));
  if ((e = cudaHostGetDevicePointer(&s->d_box, s->h_box, 0)) != cudaSuccess)
    return fail(cuda_fail(e, "step-size mailbox"));
  {
    int tile = 0, ntiles = 0, dep = 0;
    flow_geometry(s, &tile, &ntiles, &dep);
    size_t words = rkcu::flow_words(ntiles);
    if (words < (size_t)rkcu::kMaxPlainGrid) words = rkcu::kMaxPlainGrid;
    if ((e = cudaMalloc(&s->flags, sizeof(unsigned int) * words)) != cudaSuccess)
      return fail(cuda_fail(e, "cudaMalloc flags"));
  }
  if (prob->problem == RKCU_PROBLEM_LV_BANDED) {
    const size_t np = 2 * s->npairs;
    if ((e = cudaMalloc(&s->lv_r, np * sizeof(double))) != cudaSuccess)
      return fail(cuda_fail(e, "cudaMalloc r"));
    if ((e = cudaMalloc(&s->lv_a, 5 * np * sizeof(double))) != cudaSuccess)
      return fail(cuda_fail(e, "cudaMalloc a"));
    cudaMemset(s->lv_r, 0, np * sizeof(double));
    cudaMemset(s->lv_a, 0, 5 * np * sizeof(double));
    if ((e = cudaMemcpy(s->lv_r, prob->lv_r, prob->n * sizeof(double), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return fail(cuda_fail(e, "cudaMemcpy r"));
    if ((e = cudaMemcpy(s->lv_a, prob->lv_a, 5 * (size_t)prob->n * sizeof(double),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
      return fail(cuda_fail(e, "cudaMemcpy a"));
    s->dev_bytes += 6 * np * sizeof(double);
  }
  *out = s;
  return RKCU_OK;
}

int rkcu_set_method(rkcu_solver *s, double **A, const double *b, const double *b_hat,
                    const double *c, int stages, int ord) {
  // c enters only through t + h c_l, which the autonomous built-in modules
  // ignore; a caller's right-hand side receives it (RKCU_PROBLEM_RHS)
  if (!s || !A || !b || !b_hat || stages < 2 || stages > kMaxStages || ord < 1)
    return RKCU_ERR_INVALID;
  std::memset(s->A, 0, sizeof(s->A));
  std::memset(s->b, 0, sizeof(s->b));
  std::memset(s->bh, 0, sizeof(s->bh));
  std::memset(s->c, 0, sizeof(s->c));
  for (int i = 0; i < stages; ++i) {
    if (!A[i]) return RKCU_ERR_INVALID;
    for (int j = 0; j < i; ++j) s->A[i * kMaxStages + j] = A[i][j];
    s->b[i] = b[i];
    s->bh[i] = b[i] - b_hat[i];  // src/impl/seq/D.c:40-41
    s->c[i] = c ? c[i] : 0.0;
  }
  s->s = stages;
  s->ord = ord;
  s->have_method = true;
  s->begun = false;
  return RKCU_OK;
}

int rkcu_set_method_by_name(rkcu_solver *s, const char *name) {
  if (!s) return RKCU_ERR_INVALID;
  double A[kMaxStages * kMaxStages], b[16], bh[16], c[16];
  int st = 0, ord = 0, emb = 0;
  int rc = rkcu_builtin_method(name, A, b, bh, c, &st, &ord, &emb);
  if (rc != RKCU_OK) return rc;
  double *rows[kMaxStages];
  for (int i = 0; i < st; ++i) rows[i] = A + i * st;
  return rkcu_set_method(s, rows, b, bh, c, st, ord);
}

// How the mixed form runs its FP32 stages: schedule 0 (automatic) and 3 all
// stages per tile in shared memory where that path exists (even N, s <= 8),
// else one stage at a time over TMA-staged tiles; 1 tiles with plain loads;
// 2 TMA-staged tiles.
static int mixed_path(const rkcu_solver *s) {
  if (s->opt.schedule == 1) return rkcu::kMixTiles;
  if (s->opt.schedule == 2) return rkcu::kMixTilesTma;
  return rkcu::mixed_fused_available(s->prob.grid_n, s->s) ? rkcu::kMixFused : rkcu::kMixTilesTma;
}

int rkcu_begin(rkcu_solver *s, double t0, double te, const double *y0, int y0_on_device,
               double tol) {
  if (!s || !y0 || !s->have_method) return s ? RKCU_ERR_STATE : RKCU_ERR_INVALID;
  if (!(te == te) || !(t0 == t0)) return RKCU_ERR_INVALID;
  if (tol <= 0.0 && s->opt.step_limit <= 0) return RKCU_ERR_INVALID;  // fixed step needs a limit
  if (s->prob.problem == RKCU_PROBLEM_RHS && !s->rhs) return RKCU_ERR_STATE;
  RKCU_CK(cudaSetDevice(s->opt.device));
  if (s->opt.precision == RKCU_MIXED) {
    // f0, y32, f0lo and, unless all FP32 stages run per tile in shared memory, dF[1..s-2]
    const int mneed = mixed_path(s) == rkcu::kMixFused ? 3 : s->s + 1;
    if (s->mstage_vectors < mneed) {
      if (s->mstage) {
        RKCU_CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->mstage);
        s->dev_bytes -= (long long)s->mstage_vectors * s->npairs * sizeof(float2);
        s->mstage = nullptr;
        s->mstage_vectors = 0;
      }
      RKCU_CK(cudaMalloc(&s->mstage, (size_t)mneed * s->npairs * sizeof(float2)));
      s->mstage_vectors = mneed;
      s->dev_bytes += (long long)mneed * s->npairs * sizeof(float2);
    }
  }
  if (s->opt.variant == RKCU_VARIANT_LOWSTORAGE) {
    const int N = s->prob.grid_n;
    // blocks of 64 rows (32 for the 13-stage DOPRI87): fewer wavefront steps
    // (grid barriers) per RK step than smaller blocks, still a third of the
    // plain form's storage at N = 2000
    int R = s->opt.block_rows > 0 ? s->opt.block_rows : (s->s <= 8 ? 64 : 32);
    if (R > N) R = N;
    while (R > 1 && (double)R * N * N >= 1099511627776.0) R /= 2;  // row division needs q N < 2^40
    const size_t need_pairs = rkcu::lowstorage_ring_pairs(s->s, R, N);
    if (s->ring_pairs < need_pairs) {
      if (s->rings) {
        RKCU_CK(cudaStreamSynchronize(s->stream));
        cudaFree(s->rings);
        s->dev_bytes -= (long long)s->ring_pairs * sizeof(double2);
        s->rings = nullptr;
        s->ring_pairs = 0;
      }
      RKCU_CK(cudaMalloc(&s->rings, need_pairs * sizeof(double2)));
      s->ring_pairs = need_pairs;
      s->dev_bytes += (long long)need_pairs * sizeof(double2);
    }
    s->ls_rows = R;
  }
  const int need = (s->opt.precision == RKCU_MIXED || s->opt.variant == RKCU_VARIANT_LOWSTORAGE)
                       ? 0
                       : s->s + 1;  // w[1..s-1], dy, err
  if (s->stage_vectors < need) {
    if (s->stage) {
      RKCU_CK(cudaStreamSynchronize(s->stream));
      cudaFree(s->stage);
      s->dev_bytes -= (long long)s->stage_vectors * s->npairs * sizeof(double2);
      s->stage = nullptr;
      s->stage_vectors = 0;
    }
    RKCU_CK(cudaMalloc(&s->stage, (size_t)need * s->npairs * sizeof(double2)));
    s->stage_vectors = need;
    s->dev_bytes += (long long)need * s->npairs * sizeof(double2);
  }
  const size_t nbytes = (size_t)s->prob.n * sizeof(double);
  if (s->prob.n % 2) RKCU_CK(cudaMemsetAsync(s->y[0], 0, s->npairs * sizeof(double2), s->stream));
  RKCU_CK(cudaMemcpyAsync(s->y[0], y0, nbytes,
                          y0_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          s->stream));
  // src/tools.c:25-36 (H_INIT unset): h = min(10 tol, H / STEP_LIMIT); STEP_LIMIT 0 gives H/0
  const double H = te - t0;
  const double lim = H / static_cast<double>(s->opt.step_limit);  // 0 gives +inf as in the reference
  const double h0 = s->opt.h_init > 0.0 ? s->opt.h_init : tol > 0.0 ? std::fmin(10.0 * tol, lim) : lim;
  DevState *h = s->st_host;
  std::memset(h, 0, sizeof(*h));
  s->h_box->req = s->h_box->ans = 0;  // no kernel that uses it runs now (rkcu_run waits for its own)
  h->t = t0;
  h->h = h0;
  h->cur = 0;
  h->done = !(t0 < te) || (s->opt.step_limit > 0 && 0 >= s->opt.step_limit);
  RKCU_CK(cudaMemcpyAsync(s->st, h, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
  RKCU_CK(cudaStreamSynchronize(s->stream));
  s->te = te;
  s->tol = tol;
  s->begun = true;
  return RKCU_OK;
}

int rkcu_advance(rkcu_solver *s, int max_steps) {
  if (!s) return RKCU_ERR_INVALID;
  if (!s->begun) return RKCU_ERR_STATE;
  if (max_steps <= 0) return RKCU_OK;
  RKCU_CK(cudaSetDevice(s->opt.device));
  if (s->prob.problem == RKCU_PROBLEM_RHS) return advance_rhs(s, max_steps);
  if (s->opt.variant == RKCU_VARIANT_LOWSTORAGE) {
    rkcu::LsParams q;
    std::memset(&q, 0, sizeof(q));
    const int N = s->prob.grid_n, R = s->ls_rows;
    q.N = N;
    q.R = R;
    q.nb = (N + R - 1) / R;
    q.inv_n = (1ull << 40) / (unsigned long long)N + 1ull;
    q.s = s->s;
    q.ord = s->ord;
    q.step_limit = s->opt.step_limit;
    q.budget = max_steps;
    q.extra_arrivals = s->extra_arrivals;
    q.te = s->te;
    q.tol = s->tol;
    q.timeout_ns = (unsigned long long)(s->opt.wait_timeout_s * 1e9);
    for (int i = 0; i < kMaxStages * kMaxStages; ++i) {
      q.A[i] = s->A[i];
      q.nzA[i] = s->A[i] != 0.0;
    }
    for (int i = 0; i < kMaxStages; ++i) {
      q.b[i] = s->b[i];
      q.bh[i] = s->bh[i];
      q.nzb[i] = s->b[i] != 0.0;
      q.nzbh[i] = s->bh[i] != 0.0;
    }
    q.y[0] = s->y[0];
    q.y[1] = s->y[1];
    const size_t blk = (size_t)R * N;
    double2 *p = s->rings;
    for (int l = 1; l < s->s; ++l) {
      q.ring[l] = p;
      p += (size_t)(2 * l + 2) * blk;
    }
    q.dyring = p;
    p += (size_t)(2 * s->s - 1) * blk;
    q.errring = p;
    q.st = s->st;
    q.bruss.N = N;
    q.bruss.coef = bruss_coef(&s->prob);
    // automatic (0): neighbour flags between wavefront steps; 1: a grid barrier per step
    q.flags = s->flags;
    q.sync = s->opt.schedule == 1 ? 1 : 0;
    int grid = 0;
    cudaError_t e = rkcu::launch_lowstorage(q, s->opt.precision != RKCU_FP64_FMA, s->num_sms,
                                            s->stream, &grid);
    if (e != cudaSuccess) return cuda_fail(e, "low-storage kernel launch");
    s->last_grid = grid;
    ++s->launches;
    return RKCU_OK;
  }
  if (s->opt.precision == RKCU_MIXED) {
    rkcu::MixedParams m;
    std::memset(&m, 0, sizeof(m));
    m.npairs = (int)s->npairs;
    m.n = s->prob.n;
    m.s = s->s;
    m.ord = s->ord;
    m.step_limit = s->opt.step_limit;
    m.budget = max_steps;
    m.te = s->te;
    m.tol = s->tol;
    m.timeout_ns = (unsigned long long)(s->opt.wait_timeout_s * 1e9);
    m.extra_arrivals = s->extra_arrivals;
    for (int i = 0; i < kMaxStages; ++i) {
      double rs = 0.0;
      for (int j = 0; j < kMaxStages; ++j) {
        m.A[i * kMaxStages + j] = s->A[i * kMaxStages + j];
        m.nzA[i * kMaxStages + j] = s->A[i * kMaxStages + j] != 0.0;
        rs += s->A[i * kMaxStages + j];
      }
      m.csum[i] = rs;
      m.b[i] = s->b[i];
      m.bh[i] = s->bh[i];
      m.bsum += s->b[i];
      m.bhsum += s->bh[i];
    }
    m.y[0] = s->y[0];
    m.y[1] = s->y[1];
    const size_t np = s->npairs;
    m.f0 = s->mstage;
    m.y32 = s->mstage + np;
    m.f0lo = s->mstage + 2 * np;
    // the dF vectors exist unless the FP32 stages run per tile in shared memory
    if (s->mstage_vectors >= s->s + 1)
      for (int j = 1; j <= s->s - 2; ++j) m.dF[j] = s->mstage + (size_t)(2 + j) * np;
    m.st = s->st;
    m.bruss.N = s->prob.grid_n;
    m.bruss.coef = bruss_coef(&s->prob);
    int grid = 0;
    const int path = mixed_path(s);
    cudaError_t e = rkcu::launch_mixed(m, path, s->num_sms, s->stream, &grid);
    if (e != cudaSuccess) return cuda_fail(e, "mixed kernel launch");
    s->last_grid = grid;
    ++s->launches;
    return RKCU_OK;
  }
  rkcu::PlainParams p;
  std::memset(&p, 0, sizeof(p));
  p.npairs = (int)s->npairs;
  p.n = s->prob.n;
  p.s = s->s;
  p.ord = s->ord;
  p.problem = s->prob.problem;
  p.step_limit = s->opt.step_limit;
  p.budget = max_steps;
  p.te = s->te;
  p.tol = s->tol;
  p.timeout_ns = (unsigned long long)(s->opt.wait_timeout_s * 1e9);
  for (int i = 0; i < kMaxStages * kMaxStages; ++i) {
    p.A[i] = s->A[i];
    p.nzA[i] = s->A[i] != 0.0;
  }
  for (int i = 0; i < kMaxStages; ++i) {
    p.b[i] = s->b[i];
    p.bh[i] = s->bh[i];
    p.nzb[i] = s->b[i] != 0.0;
    p.nzbh[i] = s->bh[i] != 0.0;
  }
  p.y[0] = s->y[0];
  p.y[1] = s->y[1];
  for (int l = 1; l < s->s; ++l) p.w[l] = s->stage + (size_t)(l - 1) * s->npairs;
  p.dy = s->stage + (size_t)(s->s - 1) * s->npairs;
  p.err = s->stage + (size_t)s->s * s->npairs;
  p.st = s->st;
  p.flags = s->flags;
  // automatic (0): neighbour progress flags, measured faster than a grid
  // barrier after every stage at every size tried
  p.schedule = s->opt.schedule == 1   ? rkcu::kScheduleGrid
               : s->opt.schedule == 3 ? rkcu::kScheduleFlow
                                      : rkcu::kScheduleNeighbour;
  // the row ring stages BRUSS2D-MIX grid rows in shared memory (N up to kRowRingMaxN)
  if (s->opt.schedule == 4 && s->prob.problem == RKCU_PROBLEM_BRUSS2D_MIX &&
      s->prob.grid_n <= rkcu::kRowRingMaxN)
    p.schedule = rkcu::kScheduleRowRing;
  flow_geometry(s, &p.flow_tile, &p.flow_ntiles, &p.flow_dep);
  p.flow_skew = s->opt.flow_skew;  // 0: chosen at launch from the grid size
  // the flow schedule's tile counters hold step * s + stage within a launch
  if (p.schedule == rkcu::kScheduleFlow && p.budget > (1 << 24)) p.budget = 1 << 24;
  p.trace_cap = s->trace_cap;
  p.trace_meta = s->trace_meta;
  p.trace_y = s->trace_y;
  p.pow_box = s->polling ? s->d_box : nullptr;
  p.bruss.N = s->prob.grid_n;
  p.bruss.coef = s->prob.problem == RKCU_PROBLEM_BRUSS2D_MIX ? bruss_coef(&s->prob) : 0.0;
  p.lvb.n = s->prob.n;
  p.lvb.r = s->lv_r;
  p.lvb.a = s->lv_a;
  p.extra_arrivals = s->extra_arrivals;
  int grid = 0;
  // FMA mode: the fused arithmetic with its plain products in software (same bits)
  const int mode = s->opt.precision == RKCU_FP64_EXACT        ? rkcu::kArithExactSoftMul
                   : s->opt.precision == RKCU_FP64_EXACT_HWMUL ? rkcu::kArithExact
                                                               : rkcu::kArithFusedSoftMul;
  cudaError_t e = rkcu::launch_plain(p, mode, 0, s->num_sms, s->stream, &grid);
  if (e != cudaSuccess) return cuda_fail(e, "plain kernel launch");
  s->last_grid = grid;
  ++s->launches;
  return RKCU_OK;
}

int rkcu_query(rkcu_solver *s, rkcu_stats *stats) {
  if (!s) return RKCU_ERR_INVALID;
  if (!s->begun) return RKCU_ERR_STATE;
  RKCU_CK(cudaSetDevice(s->opt.device));
  RKCU_CK(cudaMemcpyAsync(s->st_host, s->st, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
  RKCU_CK(cudaStreamSynchronize(s->stream));
  DevState *h = s->st_host;
  if (!h->error && h->pending) {
    // Finish the step-size update with the C library's pow, exactly as
    // include/tools.h:221-233 writes it, then the loop increment of
    // tools.h:196-197 and the loop test.
    const double f = h->pend_h * std::fmin(2.0, std::fmax(0.5, 0.9 * std::pow(s->tol / h->pend_err,
                                                                            1.0 / (s->ord + 1.0))));
    h->h = std::fmin(f, s->te - h->t);
    h->done = !(h->t < s->te) ||
              (s->opt.step_limit > 0 && h->steps_acc + h->steps_rej >= s->opt.step_limit);
    h->pending = 0;
    ++h->host_pow_steps;
    RKCU_CK(cudaMemcpyAsync(s->st, h, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
    RKCU_CK(cudaStreamSynchronize(s->stream));
  }
  if (stats) {
    stats->steps_acc = h->steps_acc;
    stats->steps_rej = h->steps_rej;
    stats->t = h->t;
    stats->h = h->h;
    stats->done = h->done;
    stats->step_limit_reached =
        s->opt.step_limit > 0 && h->steps_acc + h->steps_rej >= s->opt.step_limit;
    stats->host_pow_steps = h->host_pow_steps;
  }
  if (h->error) return rkcu::record_wait_timeout(h->error_site);
  return RKCU_OK;
}

int rkcu_get_y(rkcu_solver *s, double *y, int y_on_device) {
  if (!s || !y) return RKCU_ERR_INVALID;
  if (!s->begun) return RKCU_ERR_STATE;
  RKCU_CK(cudaSetDevice(s->opt.device));
  RKCU_CK(cudaMemcpyAsync(s->st_host, s->st, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
  RKCU_CK(cudaStreamSynchronize(s->stream));
  const int cur = s->st_host->cur & 1;
  RKCU_CK(cudaMemcpyAsync(y, s->y[cur], (size_t)s->prob.n * sizeof(double),
                          y_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                          s->stream));
  RKCU_CK(cudaStreamSynchronize(s->stream));
  return RKCU_OK;
}

// Answer a step-size update the running plain kernel posted to the mailbox:
// include/tools.h:221-233 with the C library's pow, exactly as rkcu_query
// finishes a pending update.
static void answer_mailbox(rkcu_solver *s) {
  rkcu::PowBox &x = *s->h_box;
  const unsigned req = __atomic_load_n(&x.req, __ATOMIC_ACQUIRE);
  if (req == x.ans) return;
  x.h_new = x.h * std::fmin(2.0, std::fmax(0.5, 0.9 * std::pow(s->tol / x.err, 1.0 / (s->ord + 1.0))));
  __atomic_store_n(&x.ans, req, __ATOMIC_RELEASE);
}

// One launch of up to max_steps steps while this thread answers the mailbox,
// then the counters (the launches that poll: rkcu_run and rkcu_solve).
static int advance_polling(rkcu_solver *s, int max_steps, rkcu_stats *st) {
  s->polling = true;
  int rc = rkcu_advance(s, max_steps);
  s->polling = false;
  if (rc != RKCU_OK) return rc;
  for (;;) {
    answer_mailbox(s);
    const cudaError_t q = cudaStreamQuery(s->stream);
    if (q == cudaSuccess) break;
    if (q != cudaErrorNotReady) return cuda_fail(q, "step loop");
  }
  return rkcu_query(s, st);
}

int rkcu_solve(rkcu_solver *s, double t0, double te, const double *y0, double *y, double tol,
               rkcu_stats *stats) {
  if (!s || !y0 || !y) return RKCU_ERR_INVALID;
  int rc = rkcu_begin(s, t0, te, y0, 0, tol);
  if (rc != RKCU_OK) return rc;
  rkcu_stats st{};
  if ((rc = rkcu_query(s, &st)) != RKCU_OK) return rc;
  while (!st.done)
    if ((rc = advance_polling(s, 1 << 20, &st)) != RKCU_OK) return rc;
  if ((rc = rkcu_get_y(s, y, 0)) != RKCU_OK) return rc;
  if (stats) *stats = st;
  return RKCU_OK;
}

int rkcu_run(rkcu_solver *s, int max_steps, rkcu_stats *stats) {
  if (!s) return RKCU_ERR_INVALID;
  if (!s->begun) return RKCU_ERR_STATE;
  rkcu_stats st{};
  int rc = rkcu_query(s, &st);
  if (rc != RKCU_OK) return rc;
  const long long target = (long long)st.steps_acc + st.steps_rej + (max_steps > 0 ? max_steps : 0);
  while (!st.done && (long long)st.steps_acc + st.steps_rej < target) {
    const long long left = target - st.steps_acc - st.steps_rej;
    if ((rc = advance_polling(s, (int)(left < (1 << 30) ? left : (1 << 30)), &st)) != RKCU_OK) return rc;
  }
  if (stats) *stats = st;
  return RKCU_OK;
}

double rkcu_step_size(double h, double err, double tol, int ord, int *host_pow) {
  bool hp = false;
  const double r = rkcu::step_factor_h(h, err, tol, ord, &hp);
  if (host_pow) *host_pow = hp ? 1 : 0;
  return r;
}

int rkcu_step_sizes_device(const double *h, const double *err, int count, double tol, int ord,
                           double *out, int *host_pow) {
  if (!h || !err || !out || count < 0) return RKCU_ERR_INVALID;
  if (count == 0) return RKCU_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return RKCU_ERR_NO_DEVICE;
  double *d = nullptr;
  const size_t bytes = (size_t)count * sizeof(double);
  double *flags = static_cast<double *>(std::malloc(bytes));
  if (!flags) return RKCU_ERR_NOMEM;
  cudaError_t e = cudaMalloc(&d, 4 * bytes);  // h, err, out, flags
  if (e == cudaSuccess) e = cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + count, err, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = rkcu::launch_step_sizes(d, d + count, count, tol, ord, d + 2 * count, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * count, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(flags, d + 3 * count, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && host_pow)
    for (int i = 0; i < count; ++i) host_pow[i] = flags[i] != 0.0;
  cudaFree(d);
  std::free(flags);
  return e == cudaSuccess ? RKCU_OK : cuda_fail(e, "rkcu_step_sizes_device");
}

int rkcu_debug_inject_wait_timeout(rkcu_solver *s, int extra_arrivals) {
  if (!s || extra_arrivals < 0) return RKCU_ERR_INVALID;
  s->extra_arrivals = extra_arrivals;
  return RKCU_OK;
}

int rkcu_set_rhs(rkcu_solver *s, rkcu_rhs_fn fn, void *user) {
  if (!s || !fn || s->prob.problem != RKCU_PROBLEM_RHS) return RKCU_ERR_INVALID;
  s->rhs = fn;
  s->rhs_user = user;
  s->begun = false;
  return RKCU_OK;
}

int rkcu_rhs_builtin(double t, const double *w, double *f, int n, void *stream, void *user) {
  (void)t;  // both modules are autonomous
  const rkcu_problem *prob = static_cast<const rkcu_problem *>(user);
  if (!prob || !w || !f || prob->n != n || check_problem(prob) != RKCU_OK ||
      prob->problem == RKCU_PROBLEM_LV_BANDED)
    return RKCU_ERR_INVALID;
  const rkcu::Bruss br{prob->grid_n, prob->problem == RKCU_PROBLEM_BRUSS2D_MIX ? bruss_coef(prob) : 0.0};
  const rkcu::LvBanded lvb{};
  const cudaError_t e = rkcu::launch_eval_rhs(prob->problem, br, lvb, (n + 1) / 2,
                                              reinterpret_cast<const double2 *>(w),
                                              reinterpret_cast<double2 *>(f), static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? RKCU_OK : cuda_fail(e, "built-in right-hand side");
}

int rkcu_set_trace(rkcu_solver *s, int capacity, int with_y) {
  if (!s || capacity < 0) return RKCU_ERR_INVALID;
  if (capacity > 0 && (s->opt.variant != RKCU_VARIANT_D || s->opt.precision == RKCU_MIXED ||
                       s->prob.problem == RKCU_PROBLEM_RHS))
    return RKCU_ERR_INVALID;
  RKCU_CK(cudaSetDevice(s->opt.device));
  RKCU_CK(cudaStreamSynchronize(s->stream));
  const long long old_bytes = (s->trace_meta ? 3LL * s->trace_cap * (long long)sizeof(double) : 0) +
                              (s->trace_y ? (long long)s->trace_cap * s->npairs * sizeof(double2) : 0);
  cudaFree(s->trace_meta);
  cudaFree(s->trace_y);
  s->trace_meta = nullptr;
  s->trace_y = nullptr;
  s->trace_cap = 0;
  s->dev_bytes -= old_bytes;
  if (capacity == 0) return RKCU_OK;
  RKCU_CK(cudaMalloc(&s->trace_meta, 3 * (size_t)capacity * sizeof(double)));
  long long bytes = 3LL * capacity * (long long)sizeof(double);
  if (with_y) {
    const size_t ybytes = (size_t)capacity * s->npairs * sizeof(double2);
    cudaError_t e = cudaMalloc(&s->trace_y, ybytes);
    if (e != cudaSuccess) {
      cudaFree(s->trace_meta);
      s->trace_meta = nullptr;
      cudaGetLastError();
      return e == cudaErrorMemoryAllocation ? RKCU_ERR_NOMEM : cuda_fail(e, "trace allocation");
    }
    bytes += (long long)ybytes;
  }
  s->trace_cap = capacity;
  s->dev_bytes += bytes;
  return RKCU_OK;
}

int rkcu_get_trace(rkcu_solver *s, double *t, double *h, double *err, double *y, int capacity,
                   int *count) {
  if (!s || capacity < 0) return RKCU_ERR_INVALID;
  if (!s->begun) return RKCU_ERR_STATE;
  rkcu_stats st{};
  int rc = rkcu_query(s, &st);
  if (rc != RKCU_OK) return rc;
  const long long attempted = (long long)st.steps_acc + st.steps_rej;
  const int rec = (int)(attempted < s->trace_cap ? attempted : s->trace_cap);
  if (count) *count = rec;
  const int k = rec < capacity ? rec : capacity;
  if (k == 0) return RKCU_OK;
  if (t || h || err) {
    std::vector<double> meta(3 * (size_t)k);
    RKCU_CK(cudaMemcpy(meta.data(), s->trace_meta, meta.size() * sizeof(double),
                       cudaMemcpyDeviceToHost));
    for (int i = 0; i < k; ++i) {
      if (t) t[i] = meta[3 * i];
      if (h) h[i] = meta[3 * i + 1];
      if (err) err[i] = meta[3 * i + 2];
    }
  }
  if (y) {
    if (!s->trace_y) return RKCU_ERR_INVALID;
    const size_t n = (size_t)s->prob.n;
    if (n % 2 == 0) {
      RKCU_CK(cudaMemcpy(y, s->trace_y, (size_t)k * n * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
      // odd n: each stored step is padded to npairs pairs
      for (int i = 0; i < k; ++i)
        RKCU_CK(cudaMemcpy(y + (size_t)i * n, s->trace_y + (size_t)i * s->npairs,
                           n * sizeof(double), cudaMemcpyDeviceToHost));
    }
  }
  return RKCU_OK;
}

void *rkcu_stream(rkcu_solver *s) { return s ? (void *)s->stream : nullptr; }
long long rkcu_launch_count(rkcu_solver *s) { return s ? s->launches : -1; }
long long rkcu_device_bytes(rkcu_solver *s) { return s ? s->dev_bytes : -1; }

int rkcu_ode_acc_dist(const rkcu_problem *prob) {
  if (check_problem(prob) != RKCU_OK) return RKCU_ERR_INVALID;
  switch (prob->problem) {
    case RKCU_PROBLEM_BRUSS2D_MIX: return 2 * prob->grid_n;  // bruss2d-mix.c:718-721
    case RKCU_PROBLEM_LV_PAIRS: return 1;                    // lv.c:127-130
    default: return 2;                                       // band half-width
  }
}

int rkcu_ode_start(const rkcu_problem *prob, double t, double *y0) {
  (void)t;
  if (!y0 || check_problem(prob) != RKCU_OK) return RKCU_ERR_INVALID;
  if (prob->problem == RKCU_PROBLEM_BRUSS2D_MIX) {  // bruss2d-mix.c:51-59
    const int N = prob->grid_n;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        y0[2 * N * i + 2 * j] = 0.5 + (double)j / (double)(N - 1);
        y0[2 * N * i + 2 * j + 1] = 1.0 + (5.0 * (double)i) / (double)(N - 1);
      }
    return RKCU_OK;
  }
  if (prob->problem == RKCU_PROBLEM_LV_PAIRS) {  // lv.c:56-60
    for (int i = 0; i + 1 < prob->n; i += 2) {
      y0[i] = 0.2;
      y0[i + 1] = 1.1;
    }
    return RKCU_OK;
  }
  return RKCU_ERR_INVALID;  // the banded chain's initial values are given by the caller
}

int rkcu_ode_eval_rng(const rkcu_problem *prob, int i, int j, double t, const double *y,
                      double *f) {
  (void)t;
  if (!y || !f || check_problem(prob) != RKCU_OK || i < 0 || j >= prob->n) return RKCU_ERR_INVALID;
  if (j < i) return RKCU_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return RKCU_ERR_NO_DEVICE;
  const size_t np = pairs_of(prob->n);
  double2 *dy = nullptr, *df = nullptr;
  double *r = nullptr, *a = nullptr;
  int rc = RKCU_OK;
  cudaError_t e = cudaSuccess;
  rkcu::Bruss br{prob->grid_n, prob->problem == RKCU_PROBLEM_BRUSS2D_MIX ? bruss_coef(prob) : 0.0};
  rkcu::LvBanded lvb{prob->n, nullptr, nullptr};
  if ((e = cudaMalloc(&dy, np * sizeof(double2))) != cudaSuccess) goto done;
  if ((e = cudaMalloc(&df, np * sizeof(double2))) != cudaSuccess) goto done;
  if ((e = cudaMemset(dy, 0, np * sizeof(double2))) != cudaSuccess) goto done;
  if ((e = cudaMemcpy(dy, y, prob->n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
    goto done;
  if (prob->problem == RKCU_PROBLEM_LV_BANDED) {
    if ((e = cudaMalloc(&r, 2 * np * sizeof(double))) != cudaSuccess) goto done;
    if ((e = cudaMalloc(&a, 10 * np * sizeof(double))) != cudaSuccess) goto done;
    cudaMemset(r, 0, 2 * np * sizeof(double));
    cudaMemset(a, 0, 10 * np * sizeof(double));
    if ((e = cudaMemcpy(r, prob->lv_r, prob->n * sizeof(double), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      goto done;
    if ((e = cudaMemcpy(a, prob->lv_a, 5 * (size_t)prob->n * sizeof(double),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
      goto done;
    lvb.r = r;
    lvb.a = a;
  }
  if ((e = rkcu::launch_eval_rhs(prob->problem, br, lvb, (int)np, dy, df, 0)) != cudaSuccess)
    goto done;
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) goto done;
  // ode_eval_rng writes f[i..j] with global indexing (ode.h:34, block-inline.h:338)
  e = cudaMemcpy(f + i, reinterpret_cast<double *>(df) + i, (size_t)(j - i + 1) * sizeof(double),
                 cudaMemcpyDeviceToHost);
done:
  if (e != cudaSuccess) rc = cuda_fail(e, "rkcu_ode_eval_rng");
  cudaFree(dy);
  cudaFree(df);
  cudaFree(r);
  cudaFree(a);
  return rc;
}

}  // extern "C"
