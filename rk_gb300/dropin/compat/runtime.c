/*
 * Driver runtime for the drop-in D.c outside the reference tree: main() with
 * the reference's stdout contract (src/main.c:40-124), the problem module's
 * ode_size/ode_start (BRUSS2D-MIX by default, LV pairs with -DRKCU_PROBLEM_LV),
 * the rk_method_t constructors (backed by the library's built-in tableaux of
 * src/methods.c), initial_stepsize and print_statistics (src/tools.c:25-79).
 * Inside the reference tree the reference's own main.c, tools.c, methods.c and
 * problem module are linked instead and this file is not used.
 */
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "solver.h"
#include "rkcu.h"

int threads;

#ifdef RKCU_PROBLEM_LV
int ode_size = 2 * LV_COUNT;
#else
int ode_size = 2 * BRUSS_GRID_SIZE * BRUSS_GRID_SIZE;
#endif

static rkcu_problem compat_problem(void)
{
  rkcu_problem p;
  memset(&p, 0, sizeof(p));
  p.n = ode_size;
#ifdef RKCU_PROBLEM_LV
  p.problem = RKCU_PROBLEM_LV_PAIRS;
#else
  p.problem = RKCU_PROBLEM_BRUSS2D_MIX;
  p.grid_n = BRUSS_GRID_SIZE;
  p.alpha = BRUSS_ALPHA;
#endif
  return p;
}

void ode_start(double t, double *y0)
{
  rkcu_problem p = compat_problem();
#ifdef RKCU_PROBLEM_LV
  printf("ODE: LV (Lotka-Volterra, scaled)\n");
  printf("System size: %d\n", ode_size);
#else
  printf("ODE: BRUSS2D-MIX (2D Brusselator with mixed row-oriented ordering)\n");
  printf("Grid size: %d\n", BRUSS_GRID_SIZE);
  printf("Alpha: %.2e\n", BRUSS_ALPHA);
#endif
  if (rkcu_ode_start(&p, t, y0) != RKCU_OK)
  {
    fprintf(stderr, "ode_start failed\n");
    exit(EXIT_FAILURE);
  }
}

/* One block of (s+3)*s doubles: rows of A, then b, b_hat, c (methods.h:31-42). */
static void make_method(const char *name, const char *title, double ***A, double **b,
                        double **b_hat, double **c, int *s, int *ord)
{
  double a[256], bb[16], bh[16], cc[16];
  int st, o, emb, i;
  if (rkcu_builtin_method(name, a, bb, bh, cc, &st, &o, &emb) != RKCU_OK)
  {
    fprintf(stderr, "unknown method %s\n", name);
    exit(EXIT_FAILURE);
  }
  printf("Method: %s (order %d, %d stages)\n", title, o, st);
  *A = (double **) malloc((size_t) st * sizeof(double *));
  (*A)[0] = (double *) malloc((size_t) (st + 3) * st * sizeof(double));
  for (i = 1; i < st; i++)
    (*A)[i] = (*A)[i - 1] + st;
  memcpy((*A)[0], a, (size_t) st * st * sizeof(double));
  *b = (*A)[st - 1] + st;
  *b_hat = *b + st;
  *c = *b_hat + st;
  memcpy(*b, bb, (size_t) st * sizeof(double));
  memcpy(*b_hat, bh, (size_t) st * sizeof(double));
  memcpy(*c, cc, (size_t) st * sizeof(double));
  *s = st;
  *ord = o;
}

void free_emb_rk_method(double ***A, double **b, double **b_hat, double **c, int s)
{
  (void) s;
  free((*A)[0]);
  free(*A);
  *A = NULL;
  *b = *b_hat = *c = NULL;
}

void HEUN2(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("HEUN2", "HEUN2", A, b, bh, c, s, o); }
void RK4(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("RK4", "RK4", A, b, bh, c, s, o); }
void SSPRK3(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("SSPRK3", "SSPRK3", A, b, bh, c, s, o); }
void RKF23(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("RKF23", "RKF 2(3)", A, b, bh, c, s, o); }
void DOPRI54(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("DOPRI54", "DOPRI 5(4)", A, b, bh, c, s, o); }
void VERNER65(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("VERNER65", "VERNER65", A, b, bh, c, s, o); }
void DOPRI87(double ***A, double **b, double **bh, double **c, int *s, int *o)
{ make_method("DOPRI87", "DOPRI 8(7)", A, b, bh, c, s, o); }

double initial_stepsize(double t0, double H, const double *y_0, int ord, double tol)
{
  double h;
  (void) t0;
  (void) y_0;
  (void) ord;
#ifdef H_INIT
  h = H_INIT;
#else
  h = tol > 0.0 ? fmin(10.0 * tol, H / (STEP_LIMIT)) : H / (STEP_LIMIT);
#endif
  printf("Initial step size: %.e\n", h);
  return h;
}

void timer_start(double *T)
{
  struct timeval tv;
  gettimeofday(&tv, NULL);
  *T = (double) tv.tv_sec + (double) tv.tv_usec * 1E-6;
}

void timer_stop(double *T)
{
  double now;
  timer_start(&now);
  *T = now - *T;
}

void print_statistics(double timer, int steps_acc, int steps_rej)
{
  printf("Number of steps: %d (%d accepted, %d rejected)\n", steps_acc + steps_rej, steps_acc,
         steps_rej);
  if (STEP_LIMIT > 0 && steps_acc + steps_rej >= STEP_LIMIT)
    printf("Step limit reached.\n");
  printf("Kernel time: %.2e s (%.2e s per step)\n", timer,
         timer / (double) (steps_acc + steps_rej));
}

int main(void)
{
  double *y0, *y, lo, hi, timer;
  const char *env = getenv("NUM_THREADS");
  double tol = HAS_EMB_SOL(METHOD) ? TOL : 0.0;
  int i;

  threads = env ? atoi(env) : 1;
  if (threads < 1)
    threads = 1;
  y0 = (double *) malloc((size_t) ode_size * sizeof(double));
  y = (double *) malloc((size_t) ode_size * sizeof(double));
  if (!y0 || !y)
    return EXIT_FAILURE;
  ode_start(T_START, y0);

  for (lo = hi = y0[0], i = 1; i < ode_size; i++)
    if (y0[i] < lo)
      lo = y0[i];
    else if (y0[i] > hi)
      hi = y0[i];
  printf("Integration interval: [%.2e,%.2e]\n", T_START, T_END);
  printf("Initial value: y0[0] = %e, ..., y0[%d] = %e; min = %e, max = %e\n", y0[0],
         ode_size - 1, y0[ode_size - 1], lo, hi);
  printf("Tolerance: %.2e\n", tol);
#if LOCKTYPE == SPINLOCK
  printf("Lock type: spin\n");
#else
  printf("Lock type: mutex\n");
#endif
  printf("Pad size: %d\n", PAD_SIZE);

  timer_start(&timer);
  solver(T_START, T_END, y0, y, tol);
  timer_stop(&timer);
  printf("Total time:  %.2e s\n", timer);

  for (lo = hi = y[0], i = 1; i < ode_size; i++)
    if (y[i] < lo)
      lo = y[i];
    else if (y[i] > hi)
      hi = y[i];
  printf("Result: y[0] = %.20e, ..., y[%d] = %.20e; min = %.20e, max = %.20e\n", y[0],
         ode_size - 1, y[ode_size - 1], lo, hi);
  free(y0);
  free(y);
  return 0;
}
