/*
 * GB300 solver variant for the reference tree: copy to src/impl/cuda/D.c.
 *
 * It defines the reference's entry point
 *   void solver(double t0, double te, double *y0, double *y, double tol);
 * (include/solver.h:47) on top of the rkcu C ABI (include/rkcu.h): the tableau
 * comes from the same rk_method_t constructor the CPU variants call (METHOD,
 * include/config.h:88-90), the initial step size from the reference's own
 * initial_stepsize() (src/tools.c:25-36), and the statistics go through
 * print_statistics() (src/tools.c:62-79), so the stdout contract read by
 * log2tab is unchanged.  The whole step loop runs on the GPU; y0 is copied in
 * once and y out once.
 *
 * Problem selection: the reference links one problem module per binary; the
 * GPU needs to know which device evaluator to run, so the Makefile's cuda
 * family passes -DRKCU_PROBLEM_LV for the LV binaries (BRUSS2D-MIX otherwise).
 * -DRKCU_PRECISION=RKCU_FP64_FMA selects the fused arithmetic.
 */
#include <stdio.h>
#include <stdlib.h>

#include "solver.h"
#include "rkcu.h"

#ifdef RKCU_PROBLEM_LV
#define RKCU_DROPIN_PROBLEM RKCU_PROBLEM_LV_PAIRS
#else
#define RKCU_DROPIN_PROBLEM RKCU_PROBLEM_BRUSS2D_MIX
#endif

#ifndef RKCU_PRECISION
#define RKCU_PRECISION RKCU_FP64_EXACT
#endif

static void rkcu_check(int rc, const char *what)
{
  if (rc != RKCU_OK)
  {
    fprintf(stderr, "%s failed: %s (%s)\n", what, rkcu_strerror(rc), rkcu_last_cuda_error());
    exit(EXIT_FAILURE);
  }
}

void solver(double t0, double te, double *y0, double *y, double tol)
{
  double **A, *b, *b_hat, *c;
  int s, ord;
  double h, timer;
  rkcu_problem prob = {0};
  rkcu_options opt;
  rkcu_solver *gpu = NULL;
  rkcu_stats st;

  printf("Solver type: CUDA embedded Runge-Kutta method (GB300)\n");
  printf("Implementation variant: D (persistent GPU step loop)\n");

  METHOD(&A, &b, &b_hat, &c, &s, &ord);
  h = initial_stepsize(t0, te - t0, y0, ord, tol);

  prob.problem = RKCU_DROPIN_PROBLEM;
  prob.n = ode_size;
#if !defined(RKCU_PROBLEM_LV)
  prob.grid_n = BRUSS_GRID_SIZE;
  prob.alpha = BRUSS_ALPHA;
#endif
  rkcu_options_default(&opt);
  opt.precision = RKCU_PRECISION;
  opt.step_limit = STEP_LIMIT;
  opt.h_init = h;

  rkcu_check(rkcu_create(&gpu, &prob, &opt), "rkcu_create");
  rkcu_check(rkcu_set_method(gpu, A, b, b_hat, c, s, ord), "rkcu_set_method");

  timer_start(&timer);
  rkcu_check(rkcu_solve(gpu, t0, te, y0, y, tol, &st), "rkcu_solve");
  timer_stop(&timer);

  rkcu_destroy(gpu);
  free_emb_rk_method(&A, &b, &b_hat, &c, s);

  print_statistics(timer, st.steps_acc, st.steps_rej);
}
