// Allocation-free solve: the plain FP64 step loop with all of its scratch in one
// file-scope device array, for callers that must not allocate device memory.
//
// Who needs it: a host application that owns every byte of device memory
// through its own pool or a fixed budget (a simulation code that reserves HBM
// at start-up, or a plugin running inside another framework's context), and a
// latency-critical loop that cannot afford cudaFree's implicit device-wide
// synchronisation.  Such callers pass their own device buffers for the input
// and the output; everything else the solve needs (the two state buffers, the
// stage vectors, the error vectors and the step-control state) lives in
// g_noalloc_scratch below, which every GPU that loads this library holds until
// the process exits.
#include <cmath>
#include <cstring>
#include <mutex>

#include "rkcu.h"
#include "rkcu_plain.cuh"

namespace {

using rkcu::DevState;
using rkcu::kMaxStages;

// Largest system the allocation-free entry point accepts, in components.
constexpr int kNoAllocMaxComponents = 1 << 16;
constexpr size_t kPairs = kNoAllocMaxComponents / 2;
// y[2], w[1..s-1] (at most kMaxStages-1), dy, err
constexpr size_t kVectors = 2 + (kMaxStages - 1) + 2;
// the step-control state occupies the first 256 bytes, the plain kernel's
// per-CTA progress words the next kMaxPlainGrid * 4 bytes
constexpr size_t kStatePairs = 16;
constexpr size_t kFlagPairs = rkcu::kMaxPlainGrid * sizeof(unsigned int) / sizeof(double2);
static_assert(sizeof(DevState) <= kStatePairs * sizeof(double2), "state does not fit");

constexpr int kMaxDevices = 64;
double2 *g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

}  // namespace

// All scratch of rkcu_solve_noalloc, per device: 256 B of step-control state,
// 8 KiB of progress words and 16 vectors of 32768 pairs (8 MiB).
static __device__ __align__(256) double2 g_noalloc_scratch[kStatePairs + kFlagPairs + kVectors * kPairs];

namespace {

// The array's name in host code stands for a host-side shadow, not a device
// address; the device address is fetched once per device, with that device
// current, and cached.
int scratch_for_current_device(double2 **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RKCU_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    double2 *p = nullptr;
    e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch);
    if (e != cudaSuccess) return rkcu::record_cuda_error(e, "cudaGetSymbolAddress of the scratch array");
    if (!p) return RKCU_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return RKCU_OK;
}

// A failed CUDA call: its text goes where rkcu_last_cuda_error() reads it.
int fail_cuda(cudaError_t e, const char *what) { return rkcu::record_cuda_error(e, what); }

}  // namespace

extern "C" int rkcu_solve_noalloc(const rkcu_problem *prob, const char *method, int precision,
                                  int step_limit, double t0, double te, const double *y0_dev,
                                  double *y_dev, double tol, void *stream, rkcu_stats *stats) {
  if (!prob || !method || !y0_dev || !y_dev || step_limit < 0) return RKCU_ERR_INVALID;
  if (precision != RKCU_FP64_EXACT && precision != RKCU_FP64_FMA) return RKCU_ERR_INVALID;
  if (prob->problem == RKCU_PROBLEM_BRUSS2D_MIX) {
    if (prob->grid_n < 2 || (long long)prob->n != 2LL * prob->grid_n * prob->grid_n)
      return RKCU_ERR_INVALID;
  } else if (prob->problem == RKCU_PROBLEM_LV_PAIRS) {
    if (prob->n <= 0 || prob->n % 2) return RKCU_ERR_INVALID;
  } else {
    return RKCU_ERR_INVALID;  // problems with parameter arrays need device copies of them
  }
  if (prob->n > kNoAllocMaxComponents) return RKCU_ERR_TOO_LARGE;
  if (tol <= 0.0 && step_limit <= 0) return RKCU_ERR_INVALID;

  double A[kMaxStages * kMaxStages], b[16], bh[16], c[16];
  int s = 0, ord = 0, emb = 0;
  if (rkcu_builtin_method(method, A, b, bh, c, &s, &ord, &emb) != RKCU_OK) return RKCU_ERR_INVALID;

  double2 *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != RKCU_OK) return rc;
  int dev = 0, num_sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail_cuda(e, "device query");
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  const int npairs = prob->n / 2;
  DevState *dstate = reinterpret_cast<DevState *>(scratch);
  unsigned int *flags = reinterpret_cast<unsigned int *>(scratch + kStatePairs);
  double2 *vec = scratch + kStatePairs + kFlagPairs;
  rkcu::PlainParams p;
  std::memset(&p, 0, sizeof(p));
  p.npairs = npairs;
  p.n = prob->n;
  p.s = s;
  p.ord = ord;
  p.problem = prob->problem;
  p.step_limit = step_limit;
  p.te = te;
  p.tol = tol;
  p.timeout_ns = 10ull * 1000000000ull;
  for (int i = 0; i < s; ++i) {
    for (int j = 0; j < i; ++j) {
      p.A[i * kMaxStages + j] = A[i * s + j];
      p.nzA[i * kMaxStages + j] = A[i * s + j] != 0.0;
    }
    p.b[i] = b[i];
    p.bh[i] = b[i] - bh[i];  // src/impl/seq/D.c:40-41
    p.nzb[i] = p.b[i] != 0.0;
    p.nzbh[i] = p.bh[i] != 0.0;
  }
  p.y[0] = vec;
  p.y[1] = vec + kPairs;
  for (int l = 1; l < s; ++l) p.w[l] = vec + (size_t)(1 + l) * kPairs;
  p.dy = vec + (size_t)(1 + s) * kPairs;
  p.err = vec + (size_t)(2 + s) * kPairs;
  p.st = dstate;
  p.flags = flags;
  p.schedule = rkcu::kScheduleGrid;
  p.bruss.N = prob->grid_n;
  if (prob->problem == RKCU_PROBLEM_BRUSS2D_MIX) {
    const double n1 = static_cast<double>(prob->grid_n) - 1.0;
    p.bruss.coef = prob->alpha * n1 * n1;
  }

  // The array keeps the previous call's contents: the state is written afresh
  // (counters, error slots and barrier words start at zero), y[0] receives y0;
  // the stage vectors are written before they are read.
  DevState hs;
  std::memset(&hs, 0, sizeof(hs));
  const double H = te - t0;
  const double lim = H / static_cast<double>(step_limit);
  hs.t = t0;
  hs.h = tol > 0.0 ? std::fmin(10.0 * tol, lim) : lim;  // src/tools.c:25-36
  hs.done = !(t0 < te);
  if ((e = cudaMemcpyAsync(dstate, &hs, sizeof(hs), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return fail_cuda(e, "state upload");
  if ((e = cudaMemcpyAsync(p.y[0], y0_dev, (size_t)prob->n * sizeof(double),
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
    return fail_cuda(e, "y0 copy");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "synchronize");

  for (;;) {
    if (hs.done) break;
    p.budget = 1 << 20;
    int grid = 0;
    // the arithmetic rkcu_advance uses for the same precision (same bits either way)
    const int mode = precision == RKCU_FP64_EXACT ? rkcu::kArithExactSoftMul : rkcu::kArithFusedSoftMul;
    if ((e = rkcu::launch_plain(p, mode, 0, num_sms, st, &grid)) != cudaSuccess)
      return fail_cuda(e, "step-loop launch");
    if ((e = cudaMemcpyAsync(&hs, dstate, sizeof(hs), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return fail_cuda(e, "state download");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "synchronize");
    if (hs.error) return rkcu::record_wait_timeout(hs.error_site);
    if (hs.pending) {
      // the step-size update the device left to the C library's pow (tools.h:221-233)
      const double f =
          hs.pend_h * std::fmin(2.0, std::fmax(0.5, 0.9 * std::pow(tol / hs.pend_err, 1.0 / (ord + 1.0))));
      hs.h = std::fmin(f, te - hs.t);
      hs.done = !(hs.t < te) || (step_limit > 0 && hs.steps_acc + hs.steps_rej >= step_limit);
      hs.pending = 0;
      ++hs.host_pow_steps;
      if ((e = cudaMemcpyAsync(dstate, &hs, sizeof(hs), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail_cuda(e, "state upload");
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "synchronize");
    }
  }
  if ((e = cudaMemcpyAsync(y_dev, p.y[hs.cur & 1], (size_t)prob->n * sizeof(double),
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
    return fail_cuda(e, "y copy");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(e, "synchronize");
  if (stats) {
    stats->steps_acc = hs.steps_acc;
    stats->steps_rej = hs.steps_rej;
    stats->t = hs.t;
    stats->h = hs.h;
    stats->done = hs.done;
    stats->step_limit_reached = step_limit > 0 && hs.steps_acc + hs.steps_rej >= step_limit;
    stats->host_pow_steps = hs.host_pow_steps;
  }
  return RKCU_OK;
}
