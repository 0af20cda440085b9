/*
 * CPU oracle for the embedded Runge-Kutta step loop -- TEST INFRASTRUCTURE ONLY.
 * See rk_oracle.h for what it restates and how it is pinned.  Only tests/,
 * the smoke check and the benchmark's CPU-baseline leg load this file's
 * library; the GPU product never links or calls it.
 *
 * All arithmetic keeps the reference's evaluation order and is compiled with
 * -ffp-contract=off (oracle/Makefile), so its results are bit-identical to the
 * reference built without FMA contraction.
 */
#define _GNU_SOURCE
#include "rk_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Tableaux: src/methods.c:62-724.  Each entry is a quotient of two integers */
/* exactly representable as doubles, so num/den evaluated at run time gives  */
/* the same correctly rounded double as the reference's constant expression. */
/* ------------------------------------------------------------------------- */

typedef struct { int r, c; double num, den; } q_entry;     /* A[r][c] = num/den */
typedef struct { double num, den; } q_val;

typedef struct
{
  const char *name;
  int s, ord, embedded;
  const q_entry *A; int nA;
  const q_val *b, *b_hat, *c;                               /* length s each */
} method_def;

/* HEUN2, methods.c:62-102 */
static const q_entry heun2_A[] = { {1, 0, 1, 1} };
static const q_val heun2_b[] = { {1, 2}, {1, 2} };
static const q_val heun2_c[] = { {0, 1}, {1, 1} };
static const q_val zero13[] = { {0, 1}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {0, 1},
  {0, 1}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {0, 1}, {0, 1} };

/* RK4, methods.c:106-166 */
static const q_entry rk4_A[] = { {1, 0, 1, 2}, {2, 1, 1, 2}, {3, 2, 1, 1} };
static const q_val rk4_b[] = { {1, 6}, {2, 6}, {2, 6}, {1, 6} };
static const q_val rk4_c[] = { {0, 1}, {1, 2}, {1, 2}, {1, 1} };

/* SSPRK3, methods.c:170-219 */
static const q_entry ssprk3_A[] = { {1, 0, 1, 1}, {2, 0, 1, 4}, {2, 1, 1, 4} };
static const q_val ssprk3_b[] = { {1, 6}, {1, 6}, {2, 3} };
static const q_val ssprk3_c[] = { {0, 1}, {1, 1}, {1, 2} };

/* RKF23, methods.c:223-268 */
static const q_entry rkf23_A[] = { {1, 0, 1, 1}, {2, 0, 1, 4}, {2, 1, 1, 4} };
static const q_val rkf23_b[] = { {1, 2}, {1, 2}, {0, 1} };
static const q_val rkf23_bh[] = { {1, 6}, {1, 6}, {4, 6} };
static const q_val rkf23_c[] = { {0, 1}, {1, 1}, {1, 2} };

/* DOPRI54, methods.c:273-378 */
static const q_entry dopri54_A[] = {
  {1, 0, 1, 5},
  {2, 0, 3, 40}, {2, 1, 9, 40},
  {3, 0, 44, 45}, {3, 1, -56, 15}, {3, 2, 32, 9},
  {4, 0, 19372, 6561}, {4, 1, -25360, 2187}, {4, 2, 64448, 6561}, {4, 3, -212, 729},
  {5, 0, 9017, 3168}, {5, 1, -355, 33}, {5, 2, 46732, 5247}, {5, 3, 49, 176},
  {5, 4, -5103, 18656},
  {6, 0, 35, 384}, {6, 2, 500, 1113}, {6, 3, 125, 192}, {6, 4, -2187, 6784},
  {6, 5, 11, 84} };
static const q_val dopri54_b[] = { {35, 384}, {0, 1}, {500, 1113}, {125, 192},
  {-2187, 6784}, {11, 84}, {0, 1} };
static const q_val dopri54_bh[] = { {5179, 57600}, {0, 1}, {7571, 16695},
  {393, 640}, {-92097, 339200}, {187, 2100}, {1, 40} };
static const q_val dopri54_c[] = { {0, 1}, {1, 5}, {3, 10}, {4, 5}, {8, 9},
  {1, 1}, {1, 1} };

/* VERNER65, methods.c:382-472.  A[6][5] is never written by the reference
   (its zeroing loop only clears j >= i); fresh heap memory makes it 0. */
static const q_entry verner65_A[] = {
  {1, 0, 1, 18},
  {2, 0, -1, 12}, {2, 1, 1, 4},
  {3, 0, -2, 81}, {3, 1, 4, 27}, {3, 2, 8, 81},
  {4, 0, 40, 33}, {4, 1, -4, 11}, {4, 2, -56, 11}, {4, 3, 54, 11},
  {5, 0, -369, 73}, {5, 1, 72, 73}, {5, 2, 5380, 219}, {5, 3, -12285, 584},
  {5, 4, 2695, 1752},
  {6, 0, -8716, 891}, {6, 1, 656, 297}, {6, 2, 39520, 891}, {6, 3, -416, 11},
  {6, 4, 52, 27},
  {7, 0, 3015, 256}, {7, 1, -9, 4}, {7, 2, -4219, 78}, {7, 3, 5985, 128},
  {7, 4, -539, 384}, {7, 6, 693, 3328} };
static const q_val verner65_b[] = { {3, 80}, {0, 1}, {4, 25}, {243, 1120},
  {77, 160}, {73, 700}, {0, 1}, {0, 1} };
static const q_val verner65_bh[] = { {57, 640}, {0, 1}, {-16, 65}, {1377, 2240},
  {121, 320}, {0, 1}, {891, 8320}, {2, 35} };
static const q_val verner65_c[] = { {0, 1}, {1, 18}, {1, 6}, {2, 9}, {2, 3},
  {1, 1}, {8, 9}, {1, 1} };

/* DOPRI87, methods.c:476-724 */
static const q_entry dopri87_A[] = {
  {1, 0, 1, 18},
  {2, 0, 1, 48}, {2, 1, 1, 16},
  {3, 0, 1, 32}, {3, 2, 3, 32},
  {4, 0, 5, 16}, {4, 2, -75, 64}, {4, 3, 75, 64},
  {5, 0, 3, 80}, {5, 3, 3, 16}, {5, 4, 3, 20},
  {6, 0, 29443841., 614563906.}, {6, 3, 77736583., 692538347.},
  {6, 4, -28693883., 1125000000.}, {6, 5, 23124283., 1800000000.},
  {7, 0, 16016141., 946692911.}, {7, 3, 61564180., 158732637.},
  {7, 4, 22789713., 633445777.}, {7, 5, 545815736., 2771057229.},
  {7, 6, -180193667., 1043307555.},
  {8, 0, 39632708., 573591083.}, {8, 3, -433636366., 683701615.},
  {8, 4, -421739975., 2616292301.}, {8, 5, 100302831., 723423059.},
  {8, 6, 790204164., 839813087.}, {8, 7, 800635310., 3783071287.},
  {9, 0, 246121993., 1340847787.}, {9, 3, -37695042795., 15268766246.},
  {9, 4, -309121744., 1061227803.}, {9, 5, -12992083., 490766935.},
  {9, 6, 6005943493., 2108947869.}, {9, 7, 393006217., 1396673457.},
  {9, 8, 123872331., 1001029789.},
  {10, 0, -1028468189., 846180014.}, {10, 3, 8478235783., 508512852.},
  {10, 4, 1311729495., 1432422823.}, {10, 5, -10304129995., 1701304382.},
  {10, 6, -48777925059., 3047939560.}, {10, 7, 15336726248., 1032824649.},
  {10, 8, -45442868181., 3398467696.}, {10, 9, 3065993473., 597172653.},
  {11, 0, 185892177., 718116043.}, {11, 3, -3185094517., 667107341.},
  {11, 4, -477755414., 1098053517.}, {11, 5, -703635378., 230739211.},
  {11, 6, 5731566787., 1027545527.}, {11, 7, 5232866602., 850066563.},
  {11, 8, -4093664535., 808688257.}, {11, 9, 3962137247., 1805957418.},
  {11, 10, 65686358., 487910083.},
  {12, 0, 403863854., 491063109.}, {12, 3, -5068492393., 434740067.},
  {12, 4, -411421997., 543043805.}, {12, 5, 652783627., 914296604.},
  {12, 6, 11173962825., 925320556.}, {12, 7, -13158990841., 6184727034.},
  {12, 8, 3936647629., 1978049680.}, {12, 9, -160528059., 685178525.},
  {12, 10, 248638103., 1413531060.} };
static const q_val dopri87_b[] = { {14005451., 335480064.}, {0, 1}, {0, 1},
  {0, 1}, {0, 1}, {-59238493., 1068277825.}, {181606767., 758867731.},
  {561292985., 797845732.}, {-1041891430., 1371343529.},
  {760417239., 1151165299.}, {118820643., 751138087.},
  {-528747749., 2220607170.}, {1, 4} };
static const q_val dopri87_bh[] = { {13451932., 455176623.}, {0, 1}, {0, 1},
  {0, 1}, {0, 1}, {-808719846., 976000145.}, {1757004468., 5645159321.},
  {656045339., 265891186.}, {-3867574721., 1518517206.},
  {465885868., 322736535.}, {53011238., 667516719.}, {2, 45}, {0, 1} };
static const q_val dopri87_c[] = { {0, 1}, {1, 18}, {1, 12}, {1, 8}, {5, 16},
  {3, 8}, {59, 400}, {93, 200}, {5490023248., 9719169821.}, {13, 20},
  {1201146811., 1299019798.}, {1, 1}, {1, 1} };

#define NE(a) ((int) (sizeof(a) / sizeof((a)[0])))

static const method_def methods[] = {
  {"HEUN2", 2, 2, 0, heun2_A, NE(heun2_A), heun2_b, zero13, heun2_c},
  {"RK4", 4, 4, 0, rk4_A, NE(rk4_A), rk4_b, zero13, rk4_c},
  {"SSPRK3", 3, 3, 0, ssprk3_A, NE(ssprk3_A), ssprk3_b, zero13, ssprk3_c},
  {"RKF23", 3, 2, 1, rkf23_A, NE(rkf23_A), rkf23_b, rkf23_bh, rkf23_c},
  {"DOPRI54", 7, 5, 1, dopri54_A, NE(dopri54_A), dopri54_b, dopri54_bh, dopri54_c},
  {"VERNER65", 8, 6, 1, verner65_A, NE(verner65_A), verner65_b, verner65_bh,
   verner65_c},
  {"DOPRI87", 13, 8, 1, dopri87_A, NE(dopri87_A), dopri87_b, dopri87_bh, dopri87_c},
};

int ork_tableau_get(const char *name, ork_tableau *tab)
{
  int m, i;
  for (m = 0; m < NE(methods); m++)
  {
    const method_def *d = &methods[m];
    if (strcmp(d->name, name) != 0)
      continue;
    memset(tab, 0, sizeof(*tab));
    tab->s = d->s;
    tab->ord = d->ord;
    tab->embedded = d->embedded;
    for (i = 0; i < d->nA; i++)
      tab->A[d->A[i].r][d->A[i].c] = d->A[i].num / d->A[i].den;
    for (i = 0; i < d->s; i++)
    {
      tab->b[i] = d->b[i].num / d->b[i].den;
      tab->b_hat[i] = d->b_hat[i].num / d->b_hat[i].den;
      tab->c[i] = d->c[i].num / d->c[i].den;
    }
    return 0;
  }
  return -1;
}

/* ------------------------------------------------------------------------- */
/* Problems                                                                  */
/* ------------------------------------------------------------------------- */

/* bruss2d-mix.c:51-59: u at [2N i + 2j] = 0.5 + j/(N-1), v at +1 = 1 + 5i/(N-1). */
void ork_bruss_start(int N, double *y0)
{
  int i, j;
  for (i = 0; i < N; i++)
    for (j = 0; j < N; j++)
    {
      y0[2 * N * i + 2 * j] = 0.5 + (double) j / (double) (N - 1);
      y0[2 * N * i + 2 * j + 1] = 1.0 + (5.0 * (double) i) / (double) (N - 1);
    }
}

/* lv.c:43-62: pairs (0.2, 1.1). */
void ork_lv_pairs_start(int n, double *y0)
{
  int i;
  for (i = 0; i + 1 < n; i += 2)
  {
    y0[i] = 0.2;
    y0[i + 1] = 1.1;
  }
}

/*
 * BRUSS2D-MIX component i (bruss2d-mix.c:66-206).  The nine boundary cases of
 * the reference reduce to: a vertical pair sum (the missing neighbour replaced
 * by the present one, so "2.0*y" becomes "y+y", which is exact), then either
 * "(vert + west) + east" in interior columns or "vert + (2*inward)" in the
 * first/last column -- the same roundings as the reference's expressions.
 */
static double bruss_comp(int N, double coef, int i, const double *y)
{
  const int N2 = N + N;
  const int k = i / N2;
  const int j = (i - k * N2) / 2;
  const int isv = i & 1;
  const double u = y[i - isv], v = y[i - isv + 1];
  const double up = (k == 0) ? y[i + N2] : y[i - N2];
  const double dn = (k == N - 1) ? y[i - N2] : y[i + N2];
  const double vert = up + dn;
  double lap, react;

  if (j == 0)
    lap = vert + 2.0 * y[i + 2];
  else if (j == N - 1)
    lap = vert + 2.0 * y[i - 2];
  else
    lap = vert + y[i - 2] + y[i + 2];
  lap = lap - 4.0 * y[i];

  if (isv)
    react = 3.4 * u - u * u * v;
  else
    react = 1.0 + u * u * v - 4.4 * u;
  return react + coef * lap;
}

/* lv.c:66-87 */
static double lv_pairs_comp(int i, const double *y)
{
  if (i & 1)
    return 0.4 * y[i - 1] * y[i] - 0.2 * y[i];
  return 0.1 * y[i] - 0.2 * y[i] * y[i + 1];
}

/*
 * Banded LV chain (no reference module): f_i = y_i * (r_i + sum_{d=-2..2}
 * a_i,d * y_{i+d}), band truncated at the ends, terms summed in order of d.
 */
static double lv_banded_comp(const ork_problem *p, int i, const double *y)
{
  double acc = p->lv_r[i];
  int d;
  for (d = -2; d <= 2; d++)
  {
    int jj = i + d;
    if (jj < 0 || jj >= p->n)
      continue;
    acc = acc + p->lv_a[5 * i + (d + 2)] * y[jj];
  }
  return y[i] * acc;
}

static double bruss_coef(const ork_problem *p)
{
  const double N1 = (double) p->grid_n - 1.0;
  return p->alpha * N1 * N1;
}

double ork_eval_comp(const ork_problem *p, int i, const double *y)
{
  switch (p->kind)
  {
  case ORK_BRUSS2D_MIX:
    return bruss_comp(p->grid_n, bruss_coef(p), i, y);
  case ORK_LV_PAIRS:
    return lv_pairs_comp(i, y);
  default:
    return lv_banded_comp(p, i, y);
  }
}

void ork_eval_all(const ork_problem *p, const double *y, double *f)
{
  int i;
  for (i = 0; i < p->n; i++)
    f[i] = ork_eval_comp(p, i, y);
}

/* ------------------------------------------------------------------------- */
/* Step loop: seq/D.c:23-90, block-inline.h:253-320, tools.h:191-288.        */
/* ------------------------------------------------------------------------- */

typedef struct
{
  const ork_problem *p;
  int s, ord, n, nthreads, step_limit;
  double t0, te, tol, coef;
  double A[ORK_MAX_STAGES][ORK_MAX_STAGES], b[ORK_MAX_STAGES], bh[ORK_MAX_STAGES],
    c[ORK_MAX_STAGES];
  double *y, *w[ORK_MAX_STAGES], *dy, *err;
  double *slot;                 /* per-thread err_max, padded */
  pthread_barrier_t bar;
  int rows;                     /* > 0: low-storage pipelined schedule */
  double *edge[ORK_MAX_STAGES + 1];   /* per slab edge: 2s rows of w_1..w_{s-1}, err */
  double *ls_work;              /* per thread: one row of f, then the rings */
  size_t ls_per_thread;
  ork_stats *stats;
  double *h_trace;
  int trace_cap;
} solve_ctx;

typedef struct { solve_ctx *ctx; int id; } thread_arg;

static inline double eval_at(const solve_ctx *x, int j, const double *arg)
{
  if (x->p->kind == ORK_BRUSS2D_MIX)
    return bruss_comp(x->p->grid_n, x->coef, j, arg);
  return ork_eval_comp(x->p, j, arg);
}

/*
 * BRUSS2D-MIX components [c0, c1) of f(y) into F[0 .. c1-c0): bruss_comp's
 * expressions with the grid position stepped along instead of divided out.
 */
static void bruss_range(int N, double coef, int c0, int c1, const double *y, double *F)
{
  const int N2 = N + N;
  int k = c0 / N2, r = c0 - k * N2, i;
  for (i = c0; i < c1; i++)
  {
    const int j = r >> 1, isv = r & 1;
    const double u = y[i - isv], v = y[i - isv + 1];
    const double up = (k == 0) ? y[i + N2] : y[i - N2];
    const double dn = (k == N - 1) ? y[i - N2] : y[i + N2];
    const double vert = up + dn;
    double lap, react;
    if (j == 0)
      lap = vert + 2.0 * y[i + 2];
    else if (j == N - 1)
      lap = vert + 2.0 * y[i - 2];
    else
      lap = vert + y[i - 2] + y[i + 2];
    lap = lap - 4.0 * y[i];
    if (isv)
      react = 3.4 * u - u * u * v;
    else
      react = 1.0 + u * u * v - 4.4 * u;
    F[i - c0] = react + coef * lap;
    if (++r == N2)
    {
      r = 0;
      k++;
    }
  }
}

/* f(arg) on components [c0, c1) into F[0 .. c1-c0) */
static void eval_range(const solve_ctx *x, int c0, int c1, const double *arg, double *F)
{
  int j;
  if (x->p->kind == ORK_BRUSS2D_MIX)
  {
    bruss_range(x->p->grid_n, x->coef, c0, c1, arg, F);
    return;
  }
  for (j = c0; j < c1; j++)
    F[j - c0] = ork_eval_comp(x->p, j, arg);
}

/* components per chunk of the stage loops (F of one chunk stays in L1) */
#define ORK_CHUNK 512

/* tools.h:221-233 */
static double h_new(double h, double err, double tol, int ord)
{
  if (tol <= 0.0)
    return h;
  return h * fmin(2.0, fmax(0.5, 0.9 * pow(tol / err, 1.0 / (ord + 1.0))));
}

double ork_h_new(double h, double err, double tol, int ord)
{
  return h_new(h, err, tol, ord);
}

/* block-inline.h:253-272, components [c0, c1) */
static void stage_first(solve_ctx *x, double hA[][ORK_MAX_STAGES], const double *hb,
                        const double *hbh, int c0, int c1)
{
  const int s = x->s;
  double *y = x->y, *dy = x->dy, *err = x->err;
  double F[ORK_CHUNK];
  int a, j, l;
  for (a = c0; a < c1; a += ORK_CHUNK)
  {
    const int e = c1 - a < ORK_CHUNK ? c1 : a + ORK_CHUNK;
    eval_range(x, a, e, y, F);
    for (l = 1; l < s; l++)
    {
      const double al = hA[l][0];
      double *wl = x->w[l];
      for (j = a; j < e; j++)
        wl[j] = y[j] + al * F[j - a];
    }
    for (j = a; j < e; j++)
    {
      dy[j] = hb[0] * F[j - a];
      err[j] = hbh[0] * F[j - a];
    }
  }
}

/* block-inline.h:276-294 */
static void stage_mid(solve_ctx *x, int i, double hA[][ORK_MAX_STAGES], const double *hb,
                      const double *hbh, int c0, int c1)
{
  const int s = x->s;
  const double *wi = x->w[i];
  double *dy = x->dy, *err = x->err;
  double F[ORK_CHUNK];
  int a, j, l;
  for (a = c0; a < c1; a += ORK_CHUNK)
  {
    const int e = c1 - a < ORK_CHUNK ? c1 : a + ORK_CHUNK;
    eval_range(x, a, e, wi, F);
    for (l = i + 1; l < s; l++)
    {
      const double al = hA[l][i];
      double *wl = x->w[l];
      for (j = a; j < e; j++)
        wl[j] += al * F[j - a];
    }
    for (j = a; j < e; j++)
    {
      dy[j] += hb[i] * F[j - a];
      err[j] += hbh[i] * F[j - a];
    }
  }
}

/* block-inline.h:298-320, tools.h:280-288 */
static void stage_last(solve_ctx *x, const double *hb, const double *hbh, int c0, int c1,
                       double *emax)
{
  const int i = x->s - 1;
  const double *wl = x->w[i];
  double *y = x->y, *dy = x->dy, *err = x->err;
  double F[ORK_CHUNK];
  int a, j;
  for (a = c0; a < c1; a += ORK_CHUNK)
  {
    const int e = c1 - a < ORK_CHUNK ? c1 : a + ORK_CHUNK;
    eval_range(x, a, e, wl, F);
    for (j = a; j < e; j++)
    {
      double yold, div;
      dy[j] += hb[i] * F[j - a];
      err[j] += hbh[i] * F[j - a];
      yold = y[j];
      y[j] += dy[j];
      dy[j] = yold;
      div = fmax(fabs(y[j]), fabs(yold));
      if (div == 0.0)
        *emax = 1.7E308;
      else
        *emax = fmax(*emax, fabs(err[j]) / div);
    }
  }
}

/* Stage i over components [c0, c1) */
static void stage_range(solve_ctx *x, int i, double hA[][ORK_MAX_STAGES], const double *hb,
                        const double *hbh, int c0, int c1, double *emax)
{
  if (i == 0)
    stage_first(x, hA, hb, hbh, c0, c1);
  else if (i < x->s - 1)
    stage_mid(x, i, hA, hb, hbh, c0, c1);
  else
    stage_last(x, hb, hbh, c0, c1, emax);
}

/*
 * Low-storage pipelined form (BRUSS2D-MIX).  y and dy are full vectors; the
 * argument vectors w_1 .. w_{s-1} and err are kept per grid row: a row near a
 * slab edge (within s rows of it) lives in that edge's store, every other row
 * in a ring of the owning thread (l + 2 rows for w_l, s rows for err), since
 * in the diagonal sweep row k of w_l is written at sweep step k and last read
 * at step k + l + 1, and row k of err is last read at step k + s - 1.
 */
typedef struct
{
  solve_ctx *x;
  int id, r0, r1, top, bot;
  double *ring[ORK_MAX_STAGES + 1];   /* [1 .. s-1]: w_l, [s]: err */
  int ring_rows[ORK_MAX_STAGES + 1];
  double *F;                          /* one row of f values */
} ls_thread;

/* row k of vector v (1 .. s-1: w_v, s: err) */
static double *ls_row(const ls_thread *T, int v, int k)
{
  const solve_ctx *x = T->x;
  const int s = x->s, rowc = 2 * x->p->grid_n;
  if (T->top && k < T->r0 + s)
    return x->edge[v] + ((size_t) (T->id - 1) * 2 * s + (size_t) (k - (T->r0 - s))) * rowc;
  if (T->bot && k >= T->r1 - s)
    return x->edge[v] + ((size_t) T->id * 2 * s + (size_t) (k - (T->r1 - s))) * rowc;
  return T->ring[v] + (size_t) (k % T->ring_rows[v]) * rowc;
}

/* bruss_comp on one grid row, from three row pointers (bruss2d-mix.c:66-206);
   interior columns in a branch-free loop over (u, v) pairs */
static void bruss_row(int N, double coef, const double *upr, const double *cr,
                      const double *dnr, double *F)
{
  const int last = N - 1;
  int j;
  for (j = 0; j < N; j += last > 0 ? last : 1)   /* first and last column */
  {
    const int c = 2 * j, in = j == 0 ? c + 2 : c - 2;
    const double u = cr[c], v = cr[c + 1];
    const double lu = (upr[c] + dnr[c] + 2.0 * cr[in]) - 4.0 * u;
    const double lv = (upr[c + 1] + dnr[c + 1] + 2.0 * cr[in + 1]) - 4.0 * v;
    F[c] = (1.0 + u * u * v - 4.4 * u) + coef * lu;
    F[c + 1] = (3.4 * u - u * u * v) + coef * lv;
    if (last == 0)
      break;
  }
  for (j = 1; j < last; j++)
  {
    const int c = 2 * j;
    const double u = cr[c], v = cr[c + 1];
    const double lu = (upr[c] + dnr[c] + cr[c - 2] + cr[c + 2]) - 4.0 * u;
    const double lv = (upr[c + 1] + dnr[c + 1] + cr[c - 1] + cr[c + 3]) - 4.0 * v;
    F[c] = (1.0 + u * u * v - 4.4 * u) + coef * lu;
    F[c + 1] = (3.4 * u - u * u * v) + coef * lv;
  }
}

/* stage i on grid row k: stage_first / stage_mid / stage_last restricted to
   one row, with the same operations in the same order */
static void ls_row_stage(ls_thread *T, int i, int k, double hA[][ORK_MAX_STAGES],
                         const double *hb, const double *hbh, double *emax)
{
  solve_ctx *x = T->x;
  const int s = x->s, N = x->p->grid_n, rowc = 2 * N;
  const int ku = k == 0 ? k + 1 : k - 1, kd = k == N - 1 ? k - 1 : k + 1;
  double *y = x->y + (size_t) k * rowc, *dy = x->dy + (size_t) k * rowc;
  double *F = T->F, *err = ls_row(T, s, k);
  int c, l;
  if (i == 0)
    bruss_row(N, x->coef, x->y + (size_t) ku * rowc, y, x->y + (size_t) kd * rowc, F);
  else
    bruss_row(N, x->coef, ls_row(T, i, ku), ls_row(T, i, k), ls_row(T, i, kd), F);
  if (i == 0)
  {
    for (l = 1; l < s; l++)
    {
      const double al = hA[l][0];
      double *wl = ls_row(T, l, k);
      for (c = 0; c < rowc; c++)
        wl[c] = y[c] + al * F[c];
    }
    for (c = 0; c < rowc; c++)
    {
      dy[c] = hb[0] * F[c];
      err[c] = hbh[0] * F[c];
    }
  }
  else if (i < s - 1)
  {
    for (l = i + 1; l < s; l++)
    {
      const double al = hA[l][i];
      double *wl = ls_row(T, l, k);
      for (c = 0; c < rowc; c++)
        wl[c] += al * F[c];
    }
    for (c = 0; c < rowc; c++)
    {
      dy[c] += hb[i] * F[c];
      err[c] += hbh[i] * F[c];
    }
  }
  else
  {
    for (c = 0; c < rowc; c++)
    {
      double yold, div;
      dy[c] += hb[i] * F[c];
      err[c] += hbh[i] * F[c];
      yold = y[c];
      y[c] += dy[c];
      dy[c] = yold;
      div = fmax(fabs(y[c]), fabs(yold));
      if (div == 0.0)
        *emax = 1.7E308;
      else
        *emax = fmax(*emax, fabs(err[c]) / div);
    }
  }
}

/*
 * The step of one thread.  Schedule D (x->rows == 0): stage by stage over the
 * thread's block of components, a barrier between stages (pthreads/D.c).
 * Low-storage pipelined schedule (x->rows != 0, BRUSS2D-MIX; the reference's
 * PipeD4ls idea, pthreads/PipeD4ls.c, seq/PipeDls.c:49-131): every thread owns
 * a slab of grid rows and sweeps it diagonally, stage i on row tau - i, with
 * the argument vectors and err in row rings (ls_row), so the working set of a
 * thread stays in its cache and only y and dy stream through memory.
 * Row-stages whose stencil reaches into the neighbouring slab are skipped
 * and, after one barrier, the thread above each slab edge finishes that edge's
 * diamond (stage i on the 2i rows around the edge) stage by stage.  Each row
 * still receives its stages in order, so all schedules apply the same
 * operations in the same order to every component and give bit-identical
 * results.  Slabs need at least 2s rows.
 */
static void *solve_thread(void *argp)
{
  thread_arg *ta = (thread_arg *) argp;
  solve_ctx *x = ta->ctx;
  const int s = x->s, n = x->n, id = ta->id, P = x->nthreads;
  const int q = n / P, r = n % P;       /* tools.c:42-56 block distribution */
  const int lo = id < r ? id * (q + 1) : r * (q + 1) + (id - r) * q;
  const int hi = lo + (id < r ? q + 1 : q);
  double hA[ORK_MAX_STAGES][ORK_MAX_STAGES], hb[ORK_MAX_STAGES], hbh[ORK_MAX_STAGES];
  double *y = x->y, *dy = x->dy;
  double t = x->t0, h;
  int acc = 0, rej = 0, i, j;
  ls_thread T;

  memset(&T, 0, sizeof(T));
  if (x->rows > 0)
  {
    /* slab of grid rows [r0, r1) of this thread and its rings */
    const int N = x->p->grid_n, P_ = x->nthreads, rowc = 2 * N;
    const int qr = N / P_, rr = N % P_;
    T.x = x;
    T.id = id;
    T.r0 = id < rr ? id * (qr + 1) : rr * (qr + 1) + (id - rr) * qr;
    T.r1 = T.r0 + (id < rr ? qr + 1 : qr);
    T.top = id > 0;
    T.bot = id < P_ - 1;
    T.F = x->ls_work + (size_t) id * x->ls_per_thread;
    {
      double *at = T.F + rowc;
      for (i = 1; i <= s; i++)
      {
        T.ring_rows[i] = i < s ? i + 2 : s;
        T.ring[i] = at;
        at += (size_t) T.ring_rows[i] * rowc;
      }
    }
  }

  /* tools.c:25-36 (H_INIT unset); step_limit <= 0 means H/0 = +inf */
  {
    const double H = x->te - x->t0;
    const double lim = x->step_limit > 0 ? H / (double) x->step_limit : H / 0.0;
    h = x->tol > 0.0 ? fmin(10.0 * x->tol, lim) : lim;
  }

  for (t = x->t0; t < x->te && (x->step_limit <= 0 || acc + rej < x->step_limit);
       h = fmin(h, x->te - t))
  {
    double emax = 0.0, gmax;

    for (i = 0; i < s; i++)     /* methods.c:43-58 */
    {
      for (j = 0; j < i; j++)
        hA[i][j] = h * x->A[i][j];
      hb[i] = h * x->b[i];
      hbh[i] = h * x->bh[i];
    }

    if (x->rows <= 0)
    {
      for (i = 0; i < s; i++)
      {
        stage_range(x, i, hA, hb, hbh, lo, hi, &emax);
        if (P > 1 && i < s - 1)
          pthread_barrier_wait(&x->bar);
      }
    }
    else
    {
      /* a row-stage (i, k) whose stencil reaches the neighbouring slab is
         deferred: rows r0 .. r0+i-1 below the top edge and r1-i .. r1-1
         above the bottom edge (no edge at the grid's own first and last row) */
      const int r0 = T.r0, r1 = T.r1, top = T.top, bot = T.bot;
      int tau;
      /* phase 1: diagonal sweep over the slab, stage i on row tau - i */
      for (tau = r0; tau < r1 + s - 1; tau++)
        for (i = 0; i < s; i++)
        {
          const int k = tau - i;
          if (k < r0 + (top ? i : 0) || k > r1 - 1 - (bot ? i : 0))
            continue;
          ls_row_stage(&T, i, k, hA, hb, hbh, &emax);
        }
      if (P > 1)
        pthread_barrier_wait(&x->bar);
      /* phase 2: the deferred diamond around this slab's bottom edge, stage
         by stage (stage i on rows r1-i .. r1+i-1) */
      if (bot)
        for (i = 1; i < s; i++)
          for (j = r1 - i; j < r1 + i; j++)
            ls_row_stage(&T, i, j, hA, hb, hbh, &emax);
    }

    /* Every thread combines the per-thread maxima in thread order, so all
       threads take the same step-control decision. */
    x->slot[16 * id] = emax;
    if (P > 1)
      pthread_barrier_wait(&x->bar);
    gmax = x->slot[0];
    for (j = 1; j < P; j++)
      gmax = fmax(gmax, x->slot[16 * j]);

    if (id == 0 && x->h_trace && acc + rej < x->trace_cap)
      x->h_trace[acc + rej] = h;

    /* tools.h:235-278 */
    if (x->tol <= 0.0)
    {
      t += h;
      acc++;
    }
    else if (gmax <= x->tol)
    {
      t += h;
      h = h_new(h, gmax, x->tol, x->ord);
      acc++;
    }
    else
    {
      memcpy(y + lo, dy + lo, (size_t) (hi - lo) * sizeof(double));
      h = h_new(h, gmax, x->tol, x->ord);
      rej++;
    }
    if (P > 1)
      pthread_barrier_wait(&x->bar);
  }

  if (id == 0)
  {
    x->stats->steps_acc = acc;
    x->stats->steps_rej = rej;
    x->stats->t = t;
    x->stats->h = h;
  }
  return NULL;
}

int ork_solve(const ork_problem *p, const ork_tableau *tab, double t0, double te,
              const double *y0, double *y, double tol, int step_limit,
              ork_stats *stats, double *h_trace, int trace_cap, int nthreads)
{
  return ork_solve_pipelined(p, tab, t0, te, y0, y, tol, step_limit, stats, h_trace,
                             trace_cap, nthreads, 0);
}

int ork_solve_pipelined(const ork_problem *p, const ork_tableau *tab, double t0, double te,
                        const double *y0, double *y, double tol, int step_limit,
                        ork_stats *stats, double *h_trace, int trace_cap, int nthreads,
                        int rows)
{
  solve_ctx x;
  thread_arg *args;
  pthread_t *tids;
  double *work;
  int i, s;

  if (!p || !tab || !y0 || !y || !stats || p->n <= 0 || tab->s < 2
      || tab->s > ORK_MAX_STAGES)
    return -1;
  if (p->kind == ORK_BRUSS2D_MIX && (p->grid_n < 2 || p->n != 2 * p->grid_n * p->grid_n))
    return -1;
  if (p->kind == ORK_LV_BANDED && (!p->lv_r || !p->lv_a))
    return -1;
  if (tol <= 0.0 && step_limit <= 0)
    return -1;                  /* fixed step size needs a step limit */
  if (nthreads < 1)
    nthreads = 1;
  if (nthreads > p->n)
    nthreads = p->n;
  if (p->kind == ORK_BRUSS2D_MIX && rows > 0 && nthreads > p->grid_n / (2 * tab->s))
    nthreads = p->grid_n / (2 * tab->s) > 0 ? p->grid_n / (2 * tab->s) : 1;

  memset(&x, 0, sizeof(x));
  x.p = p;
  x.s = s = tab->s;
  x.ord = tab->ord;
  x.n = p->n;
  x.nthreads = nthreads;
  x.step_limit = step_limit;
  x.t0 = t0;
  x.te = te;
  x.tol = tol;
  x.coef = p->kind == ORK_BRUSS2D_MIX ? bruss_coef(p) : 0.0;
  x.stats = stats;
  x.rows = (p->kind == ORK_BRUSS2D_MIX && rows > 0) ? 1 : 0;
  x.h_trace = h_trace;
  x.trace_cap = trace_cap;
  memcpy(x.A, tab->A, sizeof(x.A));
  memcpy(x.b, tab->b, sizeof(x.b));
  memcpy(x.c, tab->c, sizeof(x.c));
  for (i = 0; i < s; i++)       /* seq/D.c:40-41 */
    x.bh[i] = tab->b[i] - tab->b_hat[i];

  if (x.rows > 0)
  {
    /* dy as a full vector; per thread one row of f and the rings; per slab
       edge 2s rows of w_1 .. w_{s-1} and err */
    const size_t rowc = 2 * (size_t) p->grid_n, edges = (size_t) nthreads - 1;
    size_t ring_rows = 1 + (size_t) s, edge_sz = edges * 2 * (size_t) s * rowc;
    for (i = 1; i < s; i++)
      ring_rows += (size_t) i + 2;
    x.ls_per_thread = ring_rows * rowc;
    work = (double *) malloc(((size_t) p->n + (size_t) nthreads * x.ls_per_thread
                              + (size_t) s * edge_sz) * sizeof(double));
    if (work)
    {
      x.dy = work;
      x.ls_work = work + p->n;
      for (i = 1; i <= s; i++)
        x.edge[i] = x.ls_work + (size_t) nthreads * x.ls_per_thread + (size_t) (i - 1) * edge_sz;
    }
  }
  else
  {
    work = (double *) malloc((size_t) (s + 1) * (size_t) p->n * sizeof(double));
    if (work)
    {
      for (i = 1; i < s; i++)
        x.w[i] = work + (size_t) (i - 1) * p->n;
      x.dy = work + (size_t) (s - 1) * p->n;
      x.err = work + (size_t) s * p->n;
    }
  }
  x.slot = (double *) calloc((size_t) nthreads * 16, sizeof(double));
  args = (thread_arg *) calloc((size_t) nthreads, sizeof(thread_arg));
  tids = (pthread_t *) calloc((size_t) nthreads, sizeof(pthread_t));
  if (!work || !x.slot || !args || !tids)
  {
    free(work);
    free(x.slot);
    free(args);
    free(tids);
    return -2;
  }
  x.y = y;
  memcpy(y, y0, (size_t) p->n * sizeof(double));

  if (nthreads > 1)
    pthread_barrier_init(&x.bar, NULL, (unsigned) nthreads);
  for (i = 0; i < nthreads; i++)
  {
    args[i].ctx = &x;
    args[i].id = i;
  }
  for (i = 1; i < nthreads; i++)
    pthread_create(&tids[i], NULL, solve_thread, &args[i]);
  solve_thread(&args[0]);
  for (i = 1; i < nthreads; i++)
    pthread_join(tids[i], NULL);
  if (nthreads > 1)
    pthread_barrier_destroy(&x.bar);

  free(work);
  free(x.slot);
  free(args);
  free(tids);
  return 0;
}
