/*
 * rkcu -- C ABI of the GB300 embedded Runge-Kutta step loop.
 *
 * The reference binds its hot path through plain C: the solver entry
 *   void solver(double t0, double te, double *y0, double *y, double tol);
 * (include/solver.h:47), the problem module of include/ode.h:29-36
 * (ode_size, ode_start, ode_eval_comp, ode_eval_rng, ode_acc_dist) and the
 * tableau constructors of type rk_method_t (include/methods.h:92-93,
 * src/methods.c:62-724).  A CUDA solver variant placed in the reference tree
 * (src/impl/cuda/<Variant>.c) calls the entry points below; nothing here
 * takes or returns a torch type, and every entry point returns an int status
 * (the reference's solver() is void and only asserts).
 *
 * All state lives on one GPU.  Calls on one rkcu_solver are not thread-safe
 * (the reference's solver() is not re-entrant either: it uses the globals
 * ode_size and threads, src/main.c:30-36).
 */
#ifndef RKCU_H_
#define RKCU_H_

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define RKCU_OK                0
#define RKCU_ERR_INVALID      -1   /* bad argument or unsupported combination */
#define RKCU_ERR_CUDA         -2   /* a CUDA runtime call failed (rkcu_last_cuda_error) */
#define RKCU_ERR_NOMEM        -3   /* device or pinned allocation failed */
#define RKCU_ERR_TIMEOUT      -4   /* a device-side wait reached its time limit */
#define RKCU_ERR_STATE        -5   /* call out of order (e.g. advance before begin) */
#define RKCU_ERR_NO_DEVICE    -6   /* no CUDA device, or not an sm_103 device */
#define RKCU_ERR_TOO_LARGE    -7   /* system larger than rkcu_solve_noalloc accepts */
#define RKCU_ERR_RHS          -8   /* the caller's right-hand side (rkcu_set_rhs) failed */

/* ---- problems (include/ode.h modules) ---------------------------------- */
#define RKCU_PROBLEM_BRUSS2D_MIX  0   /* src/problems/bruss2d-mix.c */
#define RKCU_PROBLEM_LV_PAIRS     1   /* src/problems/lv.c */
#define RKCU_PROBLEM_LV_BANDED    2   /* banded Lotka-Volterra chain (no reference module) */
#define RKCU_PROBLEM_RHS          3   /* any ode_eval_rng: a device function the caller supplies
                                         through rkcu_set_rhs (only n is used) */

/* ---- arithmetic -------------------------------------------------------- */
#define RKCU_FP64_EXACT  0   /* reference evaluation order, no contraction, and the C
                                library's pow for step sizes: bit-identical to the
                                reference compiled without FMA contraction on the same
                                platform (same step counts, same h, same y) */
#define RKCU_FP64_FMA    1   /* FP64 with fused multiply-adds (fewer FP64 instructions);
                                differs from the reference in the last bits, which can
                                change accept/reject decisions of stiff problems */
#define RKCU_MIXED       2   /* BRUSS2D-MIX: F0 in double-float, FP32 stage increments,
                                FP64 state; the update and the error estimate in
                                double-float, the error norm reduced in FP64 */
#define RKCU_FP64_EXACT_HWMUL 3 /* RKCU_FP64_EXACT with every product on the FP64 pipe (the
                                default exact mode computes products on the integer pipe,
                                bit for bit the same; this one exists to compare them) */

/* ---- solver variants (src/impl/seq/D.c, src/impl/seq/PipeDls.c) ------- */
#define RKCU_VARIANT_D           0   /* stage vectors w_1..w_{s-1}, dy, err in HBM */
#define RKCU_VARIANT_LOWSTORAGE  1   /* PipeDls idea: wavefront over row blocks, stage
                                        vectors in ring buffers (2n + O(s^2 B) doubles);
                                        BRUSS2D-MIX, FP64 */

typedef struct rkcu_solver rkcu_solver;

/* Problem description; replaces the compile-time macros of include/config.h:30-44
   (BRUSS_GRID_SIZE, BRUSS_ALPHA, LV_COUNT) and the global ode_size (ode.h:29). */
typedef struct
{
  int problem;          /* RKCU_PROBLEM_* */
  int n;                /* ode_size; for BRUSS2D-MIX must equal 2*grid_n*grid_n */
  int grid_n;           /* BRUSS_GRID_SIZE (>= 2) */
  double alpha;         /* BRUSS_ALPHA */
  const double *lv_r;   /* banded LV: r[n] (host memory, copied by rkcu_create) */
  const double *lv_a;   /* banded LV: a[n][5] for offsets -2..2 (host, copied) */
} rkcu_problem;

typedef struct
{
  int precision;        /* RKCU_FP64_EXACT (default), RKCU_FP64_FMA, RKCU_MIXED */
  int variant;          /* RKCU_VARIANT_D (default) */
  int step_limit;       /* STEP_LIMIT (config.h:71, tools.h:191-198); 0 = no limit */
  int device;           /* CUDA device ordinal */
  void *stream;         /* cudaStream_t to run on; NULL = a stream owned by the solver */
  double wait_timeout_s;/* limit of every device-side wait; <= 0 selects 10 s */
  double h_init;        /* initial step size; 0 = initial_stepsize() of src/tools.c:25-36
                           (pass the reference's own initial_stepsize() result or H_INIT) */
  int block_rows;       /* RKCU_VARIANT_LOWSTORAGE: grid rows per pipeline block (the
                           reference's BLOCKSIZE in rows, config.h:97-98); 0 = automatic */
  int schedule;         /* plain form, stage synchronisation: 0 = automatic (neighbour
                           flags), 1 = grid barrier after every stage, 2 = neighbour
                           progress flags, 3 = dataflow over (stage, tile) in wavefront
                           order, 4 = neighbour flags with each stage input's grid
                           rows staged in shared memory by bulk copies (BRUSS2D-MIX,
                           N <= 3600; others use 2); mixed form: 0 = automatic (3 where it runs: even
                           N, at most 8 stages; else 2), 1 = one stage at a time
                           over tiles with plain loads, 2 = the same with TMA-staged
                           tiles, 3 = all FP32 stages of a step per tile in shared
                           memory;
                           low-storage form: 1 = grid barrier after every wavefront
                           step, else neighbour progress flags */
  int flow_skew;        /* schedule 3: tiles by which stage i trails stage i-1 in the
                           wavefront; 0 = automatic (tiles are block_rows grid rows) */
} rkcu_options;

/* Progress of a solve: the counters of src/tools.c:62-79 plus the current t, h. */
typedef struct
{
  int steps_acc;
  int steps_rej;
  double t;
  double h;
  int done;             /* t >= te, or the step limit was reached */
  int step_limit_reached;
  long long host_pow_steps; /* step-size updates finished on the host (rkcu_step_size) */
} rkcu_stats;

void rkcu_options_default(rkcu_options *opt);

/* Create a solver for one problem on one device.  Allocates nothing large yet. */
int rkcu_create(rkcu_solver **out, const rkcu_problem *prob, const rkcu_options *opt);
int rkcu_destroy(rkcu_solver *s);

/* Install a tableau exactly as an rk_method_t fills it (methods.h:31-42,92-93):
   A given as `stages` row pointers, b, b_hat (the embedded weights, not yet
   transformed; b - b_hat is formed here as seq/D.c:40-41 does), c, order. */
int rkcu_set_method(rkcu_solver *s, double **A, const double *b, const double *b_hat,
                    const double *c, int stages, int ord);
/* Same, for the tableaux of src/methods.c by name: "HEUN2", "RK4", "SSPRK3",
   "RKF23", "DOPRI54", "VERNER65", "DOPRI87". */
int rkcu_set_method_by_name(rkcu_solver *s, const char *name);

/* General right-hand side, for problems whose ode_eval_rng reaches beyond a
   limited access distance (the reference's A/E/F variants, src/impl/seq/A.c,
   serve those; the fused kernels here need the BRUSS2D-MIX/LV stencils).  The
   function evaluates f(t, w) for all n components on the device: w and f are
   device arrays of n doubles (16-byte aligned, with one spare element when n
   is odd), and the work must be enqueued on `stream` (the solver's
   cudaStream_t).  It returns 0, or nonzero to stop the solve with RKCU_ERR_RHS.
   A solver for RKCU_PROBLEM_RHS runs the step loop of src/impl/seq/A.c:57-85
   around it: per stage a combine kernel w_l = y + sum_j h a_lj F_j, the call
   f(t + h c_l, w_l), then an output kernel for dy, err, y and the error max and
   a one-thread step-control kernel; the host reads the state back once per
   step.  FP64 modes only (RKCU_FP64_EXACT: the reference's rounding), plain
   variant. */
typedef int (*rkcu_rhs_fn)(double t, const double *w, double *f, int n, void *stream, void *user);
int rkcu_set_rhs(rkcu_solver *s, rkcu_rhs_fn fn, void *user);
/* A right-hand side of that form for the built-in modules, with `user` a
   const rkcu_problem * of RKCU_PROBLEM_BRUSS2D_MIX or RKCU_PROBLEM_LV_PAIRS
   (ode_eval_rng of src/problems/bruss2d-mix.c:670-712, src/problems/lv.c:89-121,
   in the reference's rounding). */
int rkcu_rhs_builtin(double t, const double *w, double *f, int n, void *stream, void *user);
/* Read a built-in tableau: A row-major [stages*stages]; arrays need 16 entries.
   Returns RKCU_ERR_INVALID for an unknown name.  HAS_EMB_SOL (methods.h:95-118)
   is returned in *embedded. */
int rkcu_builtin_method(const char *name, double *A, double *b, double *b_hat, double *c,
                        int *stages, int *ord, int *embedded);

/* Whole integration with host buffers: the solver() contract of
   include/solver.h:47.  y0 and y are host arrays of n doubles (may alias).
   Copies y0 in once and y out once; the step loop stays on the GPU. */
int rkcu_solve(rkcu_solver *s, double t0, double te, const double *y0, double *y,
               double tol, rkcu_stats *stats);

/* Device-resident flow, for callers that keep y in HBM:
   begin  -- set t=t0, h=initial_stepsize (src/tools.c:25-36), y=y0 (y0 is a host
             pointer if y0_on_device == 0, else a device pointer)
   advance-- enqueue up to max_steps attempted steps on the solver's stream (async);
             the device stops by itself at te, at the step limit, or after a step
             whose size update is left to the host (see rkcu_step_size; rkcu_run and
             rkcu_solve answer such updates while the launch runs, so their launches
             go on)
   query  -- wait for the stream, finish such an update, read the counters
   get_y  -- copy the current y out (host or device destination) */
int rkcu_begin(rkcu_solver *s, double t0, double te, const double *y0, int y0_on_device,
               double tol);
int rkcu_advance(rkcu_solver *s, int max_steps);
int rkcu_query(rkcu_solver *s, rkcu_stats *stats);
int rkcu_get_y(rkcu_solver *s, double *y, int y_on_device);

/* Per-step trace, the device counterpart of the reference's -DDUMP output
   (step_control in include/tools.h:239-256 prints t, h and the candidate y of
   every attempted step).  set_trace reserves room for the first `capacity`
   attempted steps after each rkcu_begin (capacity 0 turns tracing off); with_y
   also keeps each step's candidate state (capacity * n doubles).  Plain
   FP64 form only (RKCU_VARIANT_D, not RKCU_MIXED): RKCU_ERR_INVALID otherwise.
   get_trace copies the recorded steps: t[k], h[k] (the step's start and size),
   err[k] (its error max) and y[k * n ..] (host arrays; any may be NULL) for k <
   min(capacity, recorded), and sets *count to the number recorded. */
int rkcu_set_trace(rkcu_solver *s, int capacity, int with_y);
int rkcu_get_trace(rkcu_solver *s, double *t, double *h, double *err, double *y, int capacity,
                   int *count);

/* The device stream the solver runs on (cudaStream_t), for event timing. */
void *rkcu_stream(rkcu_solver *s);
/* Number of kernels this solver has launched so far. */
long long rkcu_launch_count(rkcu_solver *s);
/* Bytes of device memory this solver holds. */
long long rkcu_device_bytes(rkcu_solver *s);

/* Problem-module entry points of include/ode.h:31-35, for one problem instance:
   ode_start (host arithmetic, bruss2d-mix.c:35-60 / lv.c:43-62), and a
   device evaluation of the right-hand side over components [i, j]
   (ode_eval_rng semantics: f[i..j] written, global indexing) computed by the
   same device evaluator the step loop uses, in exact arithmetic. */
int rkcu_ode_start(const rkcu_problem *prob, double t, double *y0);
int rkcu_ode_eval_rng(const rkcu_problem *prob, int i, int j, double t, const double *y,
                      double *f);
int rkcu_ode_acc_dist(const rkcu_problem *prob);

/* Step-size update of include/tools.h:221-233, h * min(2, max(0.5,
   0.9 (tol/err)^(1/(ord+1)))), as the device controller computes it: with a
   correctly rounded pow.  *host_pow (may be NULL) is set to 1 when the power
   lies within 0.03 ulp of a rounding boundary -- there the C library's pow,
   which the reference uses and which may be off by up to 0.52 ulp, can round
   the other way, so the solver finishes such an update on the host with that
   pow.  rkcu_step_size evaluates on the host, rkcu_step_sizes_device evaluates
   count updates on the GPU (host arrays in and out). */
double rkcu_step_size(double h, double err, double tol, int ord, int *host_pow);
int rkcu_step_sizes_device(const double *h, const double *err, int count, double tol, int ord,
                           double *out, int *host_pow);

/* Run up to max_steps attempted steps and wait for them (advance + query until
   that many steps are done or the solve is done).  stats may be NULL. */
int rkcu_run(rkcu_solver *s, int max_steps, rkcu_stats *stats);

/* Test hook: make every later launch of this solver wait at its first grid
   barrier for `extra_arrivals` CTAs that do not exist, so the bounded device
   wait runs out and the call reports RKCU_ERR_TIMEOUT.  0 switches it off.
   It lets tests exercise the timeout path without faulting or hanging a GPU. */
int rkcu_debug_inject_wait_timeout(rkcu_solver *s, int extra_arrivals);

/* ---- batched and served solves ------------------------------------------
   Many independent instances (each its own problem size and parameters, t,
   h, tolerance) advanced together by one persistent kernel: a sweep is one
   attempted step of every active instance, stages run over equal-size chunks
   of all instances, the step control runs on the device per instance.  The
   reference solves one instance per process (src/main.c:92); these entry
   points batch its solver() over instances.  Device memory comes from one
   arena sized at creation; rkcu_batch_add admits an instance only if its
   footprint (rkcu_batch_footprint) fits, and returns RKCU_ERR_NOMEM without
   side effects otherwise, so a serving loop can queue it and retry after
   finished instances are taken.  Arithmetic per instance is the exact (or
   FMA) FP64 step loop of rkcu_solve, step sizes included: a step-size factor
   within 0.03 ulp of a rounding boundary is posted to the host, which answers
   with the C library's pow while the launch runs (the instance sits out the
   sweeps until the answer is there), so in the exact mode every instance
   reproduces the reference bit for bit; an instance's result does not depend
   on which other instances share the batch. */
typedef struct rkcu_batch rkcu_batch;

long long rkcu_batch_footprint(const rkcu_problem *prob, int stages);
int rkcu_batch_create(rkcu_batch **out, long long arena_bytes, int max_instances,
                      const char *method, const rkcu_options *opt);
int rkcu_batch_destroy(rkcu_batch *b);
/* Admit an instance (host y0 of n doubles, integrate t0..te with tol); *slot
   receives its slot.  RKCU_ERR_NOMEM: no room (arena or slots) right now. */
int rkcu_batch_add(rkcu_batch *b, const rkcu_problem *prob, double t0, double te, double tol,
                   const double *y0, long long host_id, int *slot);
/* Run up to max_sweeps sweeps (one launch, replayed from a CUDA graph) and
   wait for them; the calling thread answers posted step-size updates
   meanwhile.  *active_left receives the number of instances still
   integrating. */
int rkcu_batch_run(rkcu_batch *b, int max_sweeps, int *active_left);
/* Slots that finished since the last call (up to capacity). */
int rkcu_batch_finished(rkcu_batch *b, int *slots, int capacity, int *count);
/* Copy a finished instance's y out (host, may be NULL), its counters and id,
   and free its slot and arena space. */
int rkcu_batch_take(rkcu_batch *b, int slot, double *y, rkcu_stats *stats, long long *host_id);
/* Autotuner: time real sweeps for each block size x chunk size candidate and
   keep the fastest per active pair-step (results are unaffected: the
   arithmetic per component does not depend on the shape). */
int rkcu_batch_tune(rkcu_batch *b, int sweeps_per_trial, double *best_ns_per_pair_step);
int rkcu_batch_set_tuning(rkcu_batch *b, int threads, int chunk_pairs, int blocks_per_sm,
                          int use_graph);
int rkcu_batch_get_tuning(rkcu_batch *b, int *threads, int *chunk_pairs, int *blocks_per_sm);
int rkcu_batch_info(rkcu_batch *b, int *active, long long *free_bytes, long long *launches);
void *rkcu_batch_stream(rkcu_batch *b);

/* Allocation-free solve.  This entry point has no counterpart in the reference;
   it serves callers that must not allocate device memory: an application that
   owns all device memory through its own pool or a fixed budget (a simulation
   that reserves HBM at start-up, a plugin inside another framework's context)
   or a latency-critical loop that cannot take cudaFree's device-wide
   synchronisation.  It runs the same FP64 step loop as rkcu_solve for
   BRUSS2D-MIX or LV pairs with a built-in tableau (method name), reading y0
   from and writing y to the caller's DEVICE buffers (n doubles each), and calls
   no cudaMalloc, cudaFree or other allocating routine: every piece of scratch
   (state vectors, stage vectors, step-control state) lives in one static device
   array of 8 MiB + 8.25 KiB (16 vectors of 32768 double pairs, 256 B of state,
   8 KiB of per-CTA progress words) that each GPU loading the library holds
   until the process exits.  Limit: n <= 65536 components (e.g. BRUSS2D-MIX up to N = 181);
   larger systems return RKCU_ERR_TOO_LARGE.  The first call on a device looks up
   the array's device address (once per device, with that device current); make
   that first call before any stream capture.  All calls share the one array, so
   calls whose GPU work overlaps in time (other host threads, other streams)
   race and corrupt each other; serialise them.  stream is a cudaStream_t
   (NULL = the default stream); stats may be NULL. */
int rkcu_solve_noalloc(const rkcu_problem *prob, const char *method, int precision,
                       int step_limit, double t0, double te, const double *y0_dev,
                       double *y_dev, double tol, void *stream, rkcu_stats *stats);

const char *rkcu_strerror(int status);
const char *rkcu_last_cuda_error(void);

#ifdef __cplusplus
}
#endif

#endif /* RKCU_H_ */
