/*
 * Stand-in declarations for building the drop-in D.c outside the reference
 * tree.  They declare the parts of the reference's interface D.c uses
 * (include/solver.h:47, ode.h:29-32, methods.h:31-50,92-118, tools.h:164-179,
 * 204-205, 294) with the same names and signatures; runtime.c implements them.
 * Inside the reference tree the real headers are used instead.
 */
#ifndef RKCU_COMPAT_SOLVER_H_
#define RKCU_COMPAT_SOLVER_H_

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "config.h"

extern int ode_size;
extern int threads;
void ode_start(double t, double *y0);

typedef void (rk_method_t) (double ***A, double **b, double **b_hat, double **c, int *s, int *ord);
rk_method_t HEUN2, RK4, SSPRK3, RKF23, DOPRI54, VERNER65, DOPRI87;

#define HAS_EMB_SOL(MNAME) HAS_EMB_SOL_I(MNAME)
#define HAS_EMB_SOL_I(MNAME) HAS_EMB_SOL_ ## MNAME()
#define HAS_EMB_SOL_HEUN2() 0
#define HAS_EMB_SOL_RK4() 0
#define HAS_EMB_SOL_SSPRK3() 0
#define HAS_EMB_SOL_RKF23() 1
#define HAS_EMB_SOL_DOPRI54() 1
#define HAS_EMB_SOL_VERNER65() 1
#define HAS_EMB_SOL_DOPRI87() 1

void free_emb_rk_method(double ***A, double **b, double **b_hat, double **c, int s);
double initial_stepsize(double t0, double H, const double *y_0, int ord, double tol);
void print_statistics(double timer, int steps_acc, int steps_rej);
void timer_start(double *T);
void timer_stop(double *T);

void solver(double t0, double te, double *y0, double *y, double tol);

#endif
