/*
 * Harness main for reference solver binaries (test infrastructure only).
 *
 * It plays the role of the reference's src/main.c:40-124 (same stdout lines for
 * the "Number of steps" / "Result:" contract) and additionally writes the final
 * state vector as raw little-endian doubles to the file named by RK_DUMP_Y, so
 * that golden fixtures can pin every component bit for bit.  It is compiled
 * together with the reference's own tools.c, methods.c, threads.c, one problem
 * module and one solver variant by oracle/Makefile.
 */
#include <stdio.h>
#include <stdlib.h>

#include "solver.h"

int threads;

int main(void)
{
  const char *env_threads = getenv("NUM_THREADS");
  const char *dump = getenv("RK_DUMP_Y");
  double tol = HAS_EMB_SOL(METHOD) ? TOL : 0.0;
  double *y0, *y, lo, hi;
  int i;

  threads = env_threads ? imin(imax(1, atoi(env_threads)), ode_size) : 1;
  y0 = MALLOC(ode_size, double);
  y = MALLOC(ode_size, double);
  ode_start(T_START, y0);
  printf("Tolerance: %.2e\n", tol);

  solver(T_START, T_END, y0, y, tol);

  for (lo = hi = y[0], i = 1; i < ode_size; i++)
    if (y[i] < lo)
      lo = y[i];
    else if (y[i] > hi)
      hi = y[i];
  printf("Result: y[0] = %.20e, ..., y[%d] = %.20e; min = %.20e, max = %.20e\n",
         y[0], ode_size - 1, y[ode_size - 1], lo, hi);

  if (dump)
  {
    FILE *f = fopen(dump, "wb");
    if (!f || fwrite(y, sizeof(double), ode_size, f) != (size_t) ode_size)
    {
      fprintf(stderr, "cannot write %s\n", dump);
      return 1;
    }
    fclose(f);
  }
  FREE(y0);
  FREE(y);
  return 0;
}
