/*
 * A stand-in solver() for a CPU check of the drop-in runtime's stdout
 * contract (rk_gb300/dropin/compat/runtime.c): it prints the solver lines the
 * GPU variant prints, takes the tableau and the initial step size through the
 * same calls, "integrates" by copying y0 to y and reports the step counts of
 * the configuration's golden run, so every line log2tab reads can be compared
 * with the reference's own output without a GPU.
 */
#include <stdio.h>
#include <string.h>

#include "solver.h"

void solver(double t0, double te, double *y0, double *y, double tol)
{
  double **A, *b, *b_hat, *c;
  int s, ord;
  double timer;

  printf("Solver type: CUDA embedded Runge-Kutta method (GB300)\n");
  printf("Implementation variant: D (persistent GPU step loop)\n");
  METHOD(&A, &b, &b_hat, &c, &s, &ord);
  (void) initial_stepsize(t0, te - t0, y0, ord, tol);
  timer_start(&timer);
  memcpy(y, y0, (size_t) ode_size * sizeof(double));
  timer_stop(&timer);
  free_emb_rk_method(&A, &b, &b_hat, &c, s);
  print_statistics(timer, FAKE_ACC, FAKE_REJ);
}
