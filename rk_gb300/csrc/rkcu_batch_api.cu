// Host side of the batched / served step loop (include/rkcu.h, rkcu_batch_*):
// a device arena with first-fit allocation (admission by HBM footprint),
// instance slots, the finished list, a CUDA-graph-captured launch, and the
// autotuner that picks block and chunk shapes from timed sweeps.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "rkcu.h"
#include "rkcu_arena.h"
#include "rkcu_batch.cuh"

using rkcu::BatchParams;
using rkcu::DevState;
using rkcu::InstCoef;
using rkcu::InstDesc;
using rkcu::kMaxStages;

namespace {

constexpr size_t kAlign = 256;

struct SlotInfo {
  int state = 0;  // 0 free, 1 active, 2 finished (result not taken yet)
  size_t off = 0, size = 0;
  int n = 0, npairs = 0;
  long long host_id = -1;
  double tol = 0.0;
  long long host_pow = 0;  // step-size updates answered by the host
};

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

}  // namespace

struct rkcu_batch {
  rkcu_options opt{};
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int s = 0, ord = 0;
  double A[kMaxStages * kMaxStages] = {}, b[kMaxStages] = {}, bh[kMaxStages] = {};
  int max_slots = 0;
  InstDesc *d_desc = nullptr;
  InstCoef *d_coef = nullptr;
  int2 *d_chunks = nullptr;
  size_t chunk_cap = 0;
  int *d_ints = nullptr;  // [0] nslots, [1] nchunks, [2] rebuild, [3] done_count, [4] chunk
                          // length, [5] sweeps of the next launch
  int *d_done = nullptr;
  DevState *d_st = nullptr;
  rkcu::PowBox *h_box = nullptr;  // mapped, pinned host memory: one mailbox per slot
  rkcu::PowBox *d_box = nullptr;  // its device address
  char *arena = nullptr;
  size_t arena_bytes = 0;
  rkcu::ArenaList free_list;  // free byte ranges of the arena
  std::vector<SlotInfo> slots;
  int nslots_high = 0;
  std::vector<int> finished;
  int active = 0;
  // tuning
  int threads = 256, chunk_pairs = 1024, blocks_per_sm = 0;
  int grid = 0;
  // graph
  cudaGraphExec_t graph_exec = nullptr;
  int budget = 0;  // sweeps of the launch being set up (the source of the copy to d_ints[5])
  bool use_graph = true;
  long long launches = 0;
  char err[256] = "";
};

namespace {

int fail(rkcu_batch *b, cudaError_t e, const char *what) {
  std::snprintf(b->err, sizeof(b->err), "%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? RKCU_ERR_NOMEM : RKCU_ERR_CUDA;
}

#define BCK(call)                                  \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return fail(b, e_, #call); \
  } while (0)

BatchParams make_params(rkcu_batch *b) {
  BatchParams p;
  std::memset(&p, 0, sizeof(p));
  p.s = b->s;
  p.ord = b->ord;
  for (int i = 0; i < kMaxStages * kMaxStages; ++i) {
    p.A[i] = b->A[i];
    p.nzA[i] = b->A[i] != 0.0;
  }
  for (int i = 0; i < kMaxStages; ++i) {
    p.b[i] = b->b[i];
    p.bh[i] = b->bh[i];
    p.nzb[i] = b->b[i] != 0.0;
    p.nzbh[i] = b->bh[i] != 0.0;
  }
  p.desc = b->d_desc;
  p.coef = b->d_coef;
  p.nslots = b->d_ints;
  p.nchunks = b->d_ints + 1;
  p.rebuild = b->d_ints + 2;
  p.done_count = b->d_ints + 3;
  p.chunk_len = b->d_ints + 4;
  p.done_list = b->d_done;
  p.chunks = b->d_chunks;
  p.chunk_pairs = b->chunk_pairs;
  p.budget = b->d_ints + 5;
  p.timeout_ns = (unsigned long long)(b->opt.wait_timeout_s * 1e9);
  p.st = b->d_st;
  p.pow_box = b->d_box;
  return p;
}

// Answer the step-size updates the kernel posted: include/tools.h:221-233 with
// the C library's pow, as the reference computes every update.
void serve(rkcu_batch *b) {
  for (int i = 0; i < b->nslots_high; ++i) {
    SlotInfo &si = b->slots[i];
    if (si.state != 1) continue;
    rkcu::PowBox &x = b->h_box[i];
    const unsigned req = __atomic_load_n(&x.req, __ATOMIC_ACQUIRE);
    if (req == x.ans) continue;  // nothing new (only the host writes ans)
    const double err = x.err, h = x.h;
    x.h_new = h * std::fmin(2.0, std::fmax(0.5, 0.9 * std::pow(si.tol / err, 1.0 / (b->ord + 1.0))));
    __atomic_store_n(&x.ans, req, __ATOMIC_RELEASE);
    ++si.host_pow;
  }
}

// Wait for the batch's stream, answering posted step-size updates meanwhile
// (the kernel never waits for an answer: an instance with an update pending
// sits out the sweeps until the answer is there).
int wait_serving(rkcu_batch *b) {
  for (;;) {
    serve(b);
    const cudaError_t q = cudaStreamQuery(b->stream);
    if (q == cudaSuccess) break;
    if (q != cudaErrorNotReady) return fail(b, q, "batch launch");
  }
  serve(b);
  return RKCU_OK;
}

void drop_graph(rkcu_batch *b) {
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  b->graph_exec = nullptr;
}

// One launch of `budget` sweeps: the chunk-list rebuild then the persistent
// kernel, replayed from a captured CUDA graph when the shape is unchanged (the
// sweep count is a device word written before each replay).
int launch(rkcu_batch *b, int budget);
int launch(rkcu_batch *b, int budget) {
  const bool exact = b->opt.precision != RKCU_FP64_FMA;
  b->budget = budget;
  BCK(cudaMemcpyAsync(b->d_ints + 5, &b->budget, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  if (b->use_graph) {
    if (!b->graph_exec) {
      BatchParams p = make_params(b);
      p.nblocks = rkcu::batch_grid(exact, b->threads, b->blocks_per_sm, b->num_sms);
      cudaGraph_t g = nullptr;
      BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e1 = rkcu::launch_batch_rebuild(p, b->stream);
      int grid = 0;
      cudaError_t e2 = e1 == cudaSuccess ? rkcu::launch_batch(p, exact, b->threads, b->blocks_per_sm,
                                                              b->num_sms, b->stream, &grid)
                                         : e1;
      cudaError_t e3 = cudaStreamEndCapture(b->stream, &g);
      cudaError_t e4 = cudaErrorUnknown;
      if (e2 == cudaSuccess && e3 == cudaSuccess) e4 = cudaGraphInstantiate(&b->graph_exec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e4 != cudaSuccess) {
        // the platform refused to capture the cooperative launch: launch it directly
        std::snprintf(b->err, sizeof(b->err), "graph capture unavailable: %s / %s / %s",
                      cudaGetErrorString(e2), cudaGetErrorString(e3), cudaGetErrorString(e4));
        cudaGetLastError();
        b->graph_exec = nullptr;
        b->use_graph = false;
        return launch(b, budget);
      }
      b->grid = grid;
    }
    BCK(cudaGraphLaunch(b->graph_exec, b->stream));
  } else {
    BatchParams p = make_params(b);
    p.nblocks = rkcu::batch_grid(exact, b->threads, b->blocks_per_sm, b->num_sms);
    BCK(rkcu::launch_batch_rebuild(p, b->stream));
    int grid = 0;
    BCK(rkcu::launch_batch(p, exact, b->threads, b->blocks_per_sm, b->num_sms, b->stream, &grid));
    b->grid = grid;
  }
  b->launches += 2;
  return RKCU_OK;
}

// Collect the slots that finished during the last launch.
int collect(rkcu_batch *b) {
  int cnt = 0;
  BCK(cudaMemcpyAsync(&cnt, b->d_ints + 3, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  DevState st;
  BCK(cudaMemcpy(&st, b->d_st, sizeof(st), cudaMemcpyDeviceToHost));
  if (st.error) {
    std::snprintf(b->err, sizeof(b->err), "device wait timed out at site %d", st.error_site);
    return RKCU_ERR_TIMEOUT;
  }
  if (cnt > 0) {
    std::vector<int> ids(cnt);
    BCK(cudaMemcpy(ids.data(), b->d_done, cnt * sizeof(int), cudaMemcpyDeviceToHost));
    for (int id : ids) {
      if (id >= 0 && id < b->max_slots && b->slots[id].state == 1) {
        b->slots[id].state = 2;
        --b->active;
        b->finished.push_back(id);
      }
    }
    BCK(cudaMemsetAsync(b->d_ints + 3, 0, sizeof(int), b->stream));
  }
  return RKCU_OK;
}

}  // namespace

extern "C" {

long long rkcu_batch_footprint(const rkcu_problem *prob, int stages) {
  if (!prob || prob->n <= 0 || stages < 2 || stages > kMaxStages) return -1;
  const size_t np = ((size_t)prob->n + 1) / 2;
  size_t bytes = align_up((size_t)(stages + 3) * np * sizeof(double2));
  if (prob->problem == RKCU_PROBLEM_LV_BANDED) bytes += align_up(2 * np * 6 * sizeof(double));
  return (long long)bytes;
}

int rkcu_batch_create(rkcu_batch **out, long long arena_bytes, int max_instances, const char *method,
                      const rkcu_options *opt) {
  if (!out || arena_bytes <= 0 || max_instances <= 0 || !method) return RKCU_ERR_INVALID;
  *out = nullptr;
  rkcu_options o;
  if (opt)
    o = *opt;
  else
    rkcu_options_default(&o);
  if (o.precision != RKCU_FP64_EXACT && o.precision != RKCU_FP64_FMA) return RKCU_ERR_INVALID;
  if (!(o.wait_timeout_s > 0.0)) o.wait_timeout_s = 10.0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= o.device || o.device < 0)
    return RKCU_ERR_NO_DEVICE;
  double Am[kMaxStages * kMaxStages], bm[16], bhm[16], cm[16];
  int st = 0, ord = 0, emb = 0;
  if (rkcu_builtin_method(method, Am, bm, bhm, cm, &st, &ord, &emb) != RKCU_OK) return RKCU_ERR_INVALID;

  rkcu_batch *b = new (std::nothrow) rkcu_batch();
  if (!b) return RKCU_ERR_NOMEM;
  b->opt = o;
  b->s = st;
  b->ord = ord;
  for (int i = 0; i < st; ++i) {
    for (int j = 0; j < i; ++j) b->A[i * kMaxStages + j] = Am[i * st + j];
    b->b[i] = bm[i];
    b->bh[i] = bm[i] - bhm[i];  // src/impl/seq/D.c:40-41
  }
  b->max_slots = max_instances;
  b->slots.resize(max_instances);
  auto bail = [&](int rc) {
    rkcu_batch_destroy(b);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(o.device)) != cudaSuccess) return bail(fail(b, e, "cudaSetDevice"));
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, o.device);
  if (o.stream) {
    b->stream = static_cast<cudaStream_t>(o.stream);
  } else {
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
      return bail(fail(b, e, "cudaStreamCreate"));
    b->own_stream = true;
  }
  b->arena_bytes = align_up((size_t)arena_bytes);
  if ((e = cudaMalloc(&b->arena, b->arena_bytes)) != cudaSuccess) return bail(fail(b, e, "arena"));
  b->free_list.reset(b->arena_bytes);
  if ((e = cudaMalloc(&b->d_desc, sizeof(InstDesc) * max_instances)) != cudaSuccess)
    return bail(fail(b, e, "desc"));
  if ((e = cudaMemset(b->d_desc, 0, sizeof(InstDesc) * max_instances)) != cudaSuccess)
    return bail(fail(b, e, "desc"));
  if ((e = cudaMalloc(&b->d_coef, sizeof(InstCoef) * max_instances)) != cudaSuccess)
    return bail(fail(b, e, "coef"));
  // every pair of the arena in chunks of at least 128 pairs, plus one partial chunk per slot
  b->chunk_cap = b->arena_bytes / (sizeof(double2) * 128) + (size_t)max_instances + 1;
  if ((e = cudaMalloc(&b->d_chunks, sizeof(int2) * b->chunk_cap)) != cudaSuccess)
    return bail(fail(b, e, "chunks"));
  if ((e = cudaMalloc(&b->d_ints, 6 * sizeof(int))) != cudaSuccess) return bail(fail(b, e, "ints"));
  if ((e = cudaMemset(b->d_ints, 0, 6 * sizeof(int))) != cudaSuccess) return bail(fail(b, e, "ints"));
  if ((e = cudaMalloc(&b->d_done, sizeof(int) * max_instances)) != cudaSuccess)
    return bail(fail(b, e, "done list"));
  if ((e = cudaMalloc(&b->d_st, sizeof(DevState))) != cudaSuccess) return bail(fail(b, e, "state"));
  if ((e = cudaMemset(b->d_st, 0, sizeof(DevState))) != cudaSuccess) return bail(fail(b, e, "state"));
  if ((e = cudaHostAlloc(&b->h_box, sizeof(rkcu::PowBox) * max_instances,
                         cudaHostAllocMapped | cudaHostAllocPortable)) != cudaSuccess)
    return bail(fail(b, e, "step-size mailboxes"));
  std::memset(b->h_box, 0, sizeof(rkcu::PowBox) * max_instances);
  if ((e = cudaHostGetDevicePointer(&b->d_box, b->h_box, 0)) != cudaSuccess)
    return bail(fail(b, e, "step-size mailboxes"));
  *out = b;
  return RKCU_OK;
}

int rkcu_batch_destroy(rkcu_batch *b) {
  if (!b) return RKCU_ERR_INVALID;
  cudaSetDevice(b->opt.device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  cudaFree(b->arena);
  cudaFree(b->d_desc);
  cudaFree(b->d_coef);
  cudaFree(b->d_chunks);
  cudaFree(b->d_ints);
  cudaFree(b->d_done);
  cudaFree(b->d_st);
  if (b->h_box) cudaFreeHost(b->h_box);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return RKCU_OK;
}

int rkcu_batch_add(rkcu_batch *b, const rkcu_problem *prob, double t0, double te, double tol,
                   const double *y0, long long host_id, int *slot_out) {
  if (!b || !prob || !y0 || prob->n <= 0) return RKCU_ERR_INVALID;
  if (prob->problem == RKCU_PROBLEM_BRUSS2D_MIX &&
      (prob->grid_n < 2 || (long long)prob->n != 2LL * prob->grid_n * prob->grid_n))
    return RKCU_ERR_INVALID;
  if (prob->problem == RKCU_PROBLEM_LV_PAIRS && prob->n % 2) return RKCU_ERR_INVALID;
  if (prob->problem == RKCU_PROBLEM_LV_BANDED && (!prob->lv_r || !prob->lv_a)) return RKCU_ERR_INVALID;
  if (prob->problem < 0 || prob->problem > RKCU_PROBLEM_LV_BANDED) return RKCU_ERR_INVALID;
  if (tol <= 0.0 && b->opt.step_limit <= 0) return RKCU_ERR_INVALID;
  int slot = -1;
  for (int i = 0; i < b->max_slots; ++i)
    if (b->slots[i].state == 0) {
      slot = i;
      break;
    }
  if (slot < 0) return RKCU_ERR_NOMEM;  // no free slot: admission refused
  const long long fp = rkcu_batch_footprint(prob, b->s);
  size_t off = 0;
  if (fp < 0 || !b->free_list.alloc((size_t)fp, &off)) return RKCU_ERR_NOMEM;  // does not fit in HBM now
  BCK(cudaSetDevice(b->opt.device));
  const size_t np = ((size_t)prob->n + 1) / 2;
  double2 *vec = reinterpret_cast<double2 *>(b->arena + off);
  const double *lr = nullptr, *la = nullptr;
  if (prob->n % 2) BCK(cudaMemsetAsync(vec, 0, np * sizeof(double2), b->stream));
  BCK(cudaMemcpyAsync(vec, y0, (size_t)prob->n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  if (prob->problem == RKCU_PROBLEM_LV_BANDED) {
    double *par = reinterpret_cast<double *>(b->arena + off + align_up((size_t)(b->s + 3) * np * sizeof(double2)));
    BCK(cudaMemsetAsync(par, 0, 2 * np * 6 * sizeof(double), b->stream));
    BCK(cudaMemcpyAsync(par, prob->lv_r, (size_t)prob->n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(par + 2 * np, prob->lv_a, 5 * (size_t)prob->n * sizeof(double),
                        cudaMemcpyHostToDevice, b->stream));
    lr = par;
    la = par + 2 * np;
  }
  InstDesc d;
  std::memset(&d, 0, sizeof(d));
  d.kind = prob->problem;
  d.n = prob->n;
  d.npairs = (int)np;
  d.grid_n = prob->grid_n;
  if (prob->problem == RKCU_PROBLEM_BRUSS2D_MIX) {
    const double n1 = (double)prob->grid_n - 1.0;
    d.coef = prob->alpha * n1 * n1;
  }
  d.lv_r = lr;
  d.lv_a = la;
  d.vec = vec;
  d.t = t0;
  const double H = te - t0;
  const double lim = H / static_cast<double>(b->opt.step_limit);  // src/tools.c:25-36
  d.h = b->opt.h_init > 0.0 ? b->opt.h_init : tol > 0.0 ? std::fmin(10.0 * tol, lim) : lim;
  d.te = te;
  d.tol = tol;
  d.active = 1;
  d.done = !(t0 < te);
  d.step_limit = b->opt.step_limit;
  d.host_id = host_id;
  InstCoef k;
  std::memset(&k, 0, sizeof(k));
  for (int r = 1; r < b->s; ++r)
    for (int c = 0; c < r; ++c) k.hA[r * kMaxStages + c] = d.h * b->A[r * kMaxStages + c];
  for (int r = 0; r < b->s; ++r) {
    k.hb[r] = d.h * b->b[r];
    k.hbh[r] = d.h * b->bh[r];
  }
  b->h_box[slot] = rkcu::PowBox{};  // no request outstanding (d.pend_seq = 0)
  BCK(cudaMemcpyAsync(b->d_desc + slot, &d, sizeof(d), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_coef + slot, &k, sizeof(k), cudaMemcpyHostToDevice, b->stream));
  if (slot + 1 > b->nslots_high) {
    b->nslots_high = slot + 1;
    BCK(cudaMemcpyAsync(b->d_ints, &b->nslots_high, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  BCK(cudaStreamSynchronize(b->stream));  // the host-side d, k and nslots must outlive the copies
  SlotInfo &si = b->slots[slot];
  si.state = d.done ? 2 : 1;
  si.off = off;
  si.size = (size_t)fp;
  si.n = prob->n;
  si.npairs = (int)np;
  si.host_id = host_id;
  si.tol = tol;
  si.host_pow = 0;
  if (d.done)
    b->finished.push_back(slot);
  else
    ++b->active;
  if (slot_out) *slot_out = slot;
  return RKCU_OK;
}

int rkcu_batch_run(rkcu_batch *b, int max_sweeps, int *active_left) {
  if (!b || max_sweeps <= 0) return RKCU_ERR_INVALID;
  BCK(cudaSetDevice(b->opt.device));
  if (b->active > 0) {
    int rc = launch(b, max_sweeps);
    if (rc != RKCU_OK) return rc;
    if ((rc = wait_serving(b)) != RKCU_OK) return rc;
    if ((rc = collect(b)) != RKCU_OK) return rc;
  }
  if (active_left) *active_left = b->active;
  return RKCU_OK;
}

int rkcu_batch_finished(rkcu_batch *b, int *slots, int capacity, int *count) {
  if (!b || !count || (capacity > 0 && !slots)) return RKCU_ERR_INVALID;
  const int k = std::min<int>(capacity, (int)b->finished.size());
  for (int i = 0; i < k; ++i) slots[i] = b->finished[i];
  b->finished.erase(b->finished.begin(), b->finished.begin() + k);
  *count = k;
  return RKCU_OK;
}

int rkcu_batch_take(rkcu_batch *b, int slot, double *y, rkcu_stats *stats, long long *host_id) {
  if (!b || slot < 0 || slot >= b->max_slots) return RKCU_ERR_INVALID;
  SlotInfo &si = b->slots[slot];
  if (si.state != 2) return RKCU_ERR_STATE;
  BCK(cudaSetDevice(b->opt.device));
  InstDesc d;
  BCK(cudaMemcpyAsync(&d, b->d_desc + slot, sizeof(d), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (y) {
    const double2 *src = d.vec + (d.cur ? (size_t)si.npairs : 0);
    BCK(cudaMemcpyAsync(y, src, (size_t)si.n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  }
  InstDesc cleared;
  std::memset(&cleared, 0, sizeof(cleared));
  BCK(cudaMemcpyAsync(b->d_desc + slot, &cleared, sizeof(cleared), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (stats) {
    stats->steps_acc = d.steps_acc;
    stats->steps_rej = d.steps_rej;
    stats->t = d.t;
    stats->h = d.h;
    stats->done = d.done;
    stats->step_limit_reached = d.step_limit > 0 && d.steps_acc + d.steps_rej >= d.step_limit;
    stats->host_pow_steps = si.host_pow;
  }
  if (host_id) *host_id = si.host_id;
  b->free_list.release(si.off, si.size);
  si = SlotInfo();
  return RKCU_OK;
}

int rkcu_batch_set_tuning(rkcu_batch *b, int threads, int chunk_pairs, int blocks_per_sm,
                          int use_graph) {
  if (!b || (threads != 128 && threads != 256 && threads != 512) || chunk_pairs < 128 ||
      chunk_pairs % 32)
    return RKCU_ERR_INVALID;
  b->threads = threads;
  b->chunk_pairs = chunk_pairs;
  b->blocks_per_sm = blocks_per_sm;
  b->use_graph = use_graph != 0;
  drop_graph(b);
  return RKCU_OK;
}

int rkcu_batch_get_tuning(rkcu_batch *b, int *threads, int *chunk_pairs, int *blocks_per_sm) {
  if (!b) return RKCU_ERR_INVALID;
  if (threads) *threads = b->threads;
  if (chunk_pairs) *chunk_pairs = b->chunk_pairs;
  if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
  return RKCU_OK;
}

int rkcu_batch_tune(rkcu_batch *b, int sweeps_per_trial, double *best_ns_per_pair_step) {
  // Time real sweeps (they advance the solves exactly as untimed ones would: the
  // arithmetic per component does not depend on the shape) for every
  // candidate shape, twice (the first pass also takes each kernel's first-launch
  // cost), and keep the shape with the fastest per active pair-step.
  if (!b || sweeps_per_trial <= 0) return RKCU_ERR_INVALID;
  BCK(cudaSetDevice(b->opt.device));
  static const int kThreads[] = {128, 256, 512};
  static const int kChunks[] = {256, 512, 1024, 2048, 4096};
  double best = 1e300;
  int bt = b->threads, bc = b->chunk_pairs;
  cudaEvent_t e0, e1;
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  const bool graph = b->use_graph;
  for (int pass = 0; pass < 2; ++pass) {
    for (int t : kThreads) {
      for (int c : kChunks) {
        if (c < t) continue;
        if (b->active == 0) break;
        long long pairs = 0;
        for (int i = 0; i < b->nslots_high; ++i)
          if (b->slots[i].state == 1) pairs += b->slots[i].npairs;
        b->threads = t;
        b->chunk_pairs = c;
        b->use_graph = false;
        BCK(cudaEventRecord(e0, b->stream));
        int rc = launch(b, sweeps_per_trial);
        if (rc != RKCU_OK) return rc;
        BCK(cudaEventRecord(e1, b->stream));
        if ((rc = wait_serving(b)) != RKCU_OK) return rc;
        BCK(cudaEventSynchronize(e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        if ((rc = collect(b)) != RKCU_OK) return rc;
        const double per = ms * 1e6 / ((double)pairs * sweeps_per_trial);
        if (per < best) {
          best = per;
          bt = t;
          bc = c;
        }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->threads = bt;
  b->chunk_pairs = bc;
  b->use_graph = graph;
  drop_graph(b);
  if (best_ns_per_pair_step) *best_ns_per_pair_step = best < 1e300 ? best : -1.0;
  return RKCU_OK;
}

int rkcu_batch_info(rkcu_batch *b, int *active, long long *free_bytes, long long *launches) {
  if (!b) return RKCU_ERR_INVALID;
  if (active) *active = b->active;
  if (free_bytes) {
    *free_bytes = (long long)b->free_list.free_bytes();
  }
  if (launches) *launches = b->launches;
  return RKCU_OK;
}

void *rkcu_batch_stream(rkcu_batch *b) { return b ? (void *)b->stream : nullptr; }

}  // extern "C"
