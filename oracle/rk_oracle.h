/*
 * CPU oracle for the embedded Runge-Kutta step loop -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's sequential D solver
 * (src/impl/seq/D.c:23-90 with the scatter stage kernels of
 * include/block-inline.h:253-320), its step control (include/tools.h:191-288,
 * src/tools.c:25-36), its tableaux (src/methods.c:43-724) and its problem
 * modules (src/problems/bruss2d-mix.c:35-206, src/problems/lv.c:43-121), with
 * the problem size and parameters taken at run time instead of from macros.
 * It also defines the banded Lotka-Volterra chain, which has no reference
 * module.  Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it; the GPU product never calls it.
 *
 * Parity: pinned bit for bit against reference binaries compiled from the
 * reference sources (oracle/Makefile, tests/golden/make_golden.py) for
 * BRUSS2D-MIX and LV pairs.  The banded LV chain is pinned only through the
 * reference's solver algorithm (it has no reference module).
 */
#ifndef RK_ORACLE_H_
#define RK_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

#define ORK_MAX_STAGES 16

enum { ORK_BRUSS2D_MIX = 0, ORK_LV_PAIRS = 1, ORK_LV_BANDED = 2 };

typedef struct
{
  int s, ord, embedded;
  double A[ORK_MAX_STAGES][ORK_MAX_STAGES];
  double b[ORK_MAX_STAGES], b_hat[ORK_MAX_STAGES], c[ORK_MAX_STAGES];
} ork_tableau;

typedef struct
{
  int kind;
  int n;                 /* number of components */
  int grid_n;            /* BRUSS2D-MIX grid size N (n = 2 N^2) */
  double alpha;          /* BRUSS2D-MIX diffusion parameter */
  const double *lv_r;    /* banded LV: r[n] */
  const double *lv_a;    /* banded LV: a[n][5], offsets -2..2 */
} ork_problem;

typedef struct
{
  int steps_acc, steps_rej;
  double t, h;
} ork_stats;

/* Tableau by the reference's method name; returns 0 on success. */
int ork_tableau_get(const char *name, ork_tableau *tab);

void ork_bruss_start(int grid_n, double *y0);
void ork_lv_pairs_start(int n, double *y0);
double ork_eval_comp(const ork_problem *p, int i, const double *y);
void ork_eval_all(const ork_problem *p, const double *y, double *f);

/* Step-size update of include/tools.h:221-233 with the C library's pow. */
double ork_h_new(double h, double err, double tol, int ord);

/*
 * Integrate from t0 to te (the reference's solver() contract).
 * step_limit <= 0 means no limit (the reference's STEP_LIMIT=0).
 * h_trace (optional, capacity trace_cap) receives the h of every attempted step.
 * nthreads > 1 runs the same arithmetic on a pthreads team (identical results).
 * Returns 0 on success, negative on bad arguments or allocation failure.
 */
int ork_solve(const ork_problem *p, const ork_tableau *tab, double t0, double te,
              const double *y0, double *y, double tol, int step_limit,
              ork_stats *stats, double *h_trace, int trace_cap, int nthreads);

/* Same step loop with the pipelined schedule (BRUSS2D-MIX, rows > 0): each
   thread sweeps a slab of grid rows diagonally, slab edges are finished after
   one barrier; bit-identical results, the stage vectors of a few rows stay in
   cache (the idea of the reference's PipeD variants).  rows <= 0 selects the
   D schedule.  Threads are limited to grid_n / (2 s). */
int ork_solve_pipelined(const ork_problem *p, const ork_tableau *tab, double t0, double te,
                        const double *y0, double *y, double tol, int step_limit,
                        ork_stats *stats, double *h_trace, int trace_cap, int nthreads,
                        int rows);

#ifdef __cplusplus
}
#endif

#endif /* RK_ORACLE_H_ */
