// Accuracy check of the double-float BRUSS2D-MIX right-hand side and its
// helpers (rkcu_dfloat.cuh) against long double arithmetic on the host.
// Compiled with -ffp-contract=off.  Usage: dfloat_check <count> <seed>.
// Prints the worst error over the bound per case kind and exits non-zero if a
// check fails:
//   * dbl_of(float) is the exact conversion (bit patterns of all kinds);
//   * df_of(x): hi is x truncated to 24 bits and |x - hi - lo| <= 2^-46 |x|;
//   * bruss_rhs_df: |F_df - F| <= 2^-42 T + 2^-53 |coef| M, where T is the sum
//     of the magnitudes of the terms 1, u^2 v, 4.4 u (3.4 u), coef lap, and M
//     the largest stencil operand; no fallback inside its documented range.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#include "rkcu_dfloat.cuh"

using namespace rkcu::dfl;
using rkcu::softfp::bits_of;
using rkcu::softfp::double_of;
using rkcu::softfp::float_of;

static uint64_t s_state;
static uint64_t next() {  // splitmix64
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unif() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }

struct pr {
  double x, y;
};

int main(int argc, char **argv) {
  const long long count = argc > 1 ? atoll(argv[1]) : 1000000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  int fails = 0;

  // float -> double from the bit fields: every kind of pattern
  long long bad_cvt = 0;
  for (long long i = 0; i < count; ++i) {
    const uint32_t b = static_cast<uint32_t>(next());
    const float f = float_of(b);
    const double want = static_cast<double>(f), got = dbl_of(f);
    if (f == f && bits_of(want) != bits_of(got) && bad_cvt++ < 5) printf("dbl_of %a: %a vs %a\n", f, got, want);
  }
  for (float f : {0.0f, -0.0f, 1.0f, -1.0f, 1e-40f, -1e-45f, 3.4e38f, INFINITY, -INFINITY}) {
    if (bits_of(dbl_of(f)) != bits_of(static_cast<double>(f)) && bad_cvt++ < 5) printf("dbl_of %a\n", f);
  }
  printf("dbl_of mismatches: %lld\n", bad_cvt);
  fails += bad_cvt != 0;

  // double -> hi + lo
  long long bad_split = 0;
  for (long long i = 0; i < count; ++i) {
    const int ex = 943 + static_cast<int>(next() % (1150 - 943 + 1));
    const double x = double_of((next() & 0x800fffffffffffffull) | (static_cast<uint64_t>(ex) << 52));
    df d;
    if (!df_of(x, &d)) {
      if (bad_split++ < 5) printf("df_of refused %a\n", x);
      continue;
    }
    const double hi_want = double_of(bits_of(x) & ~((1ull << 29) - 1));
    const long double r = static_cast<long double>(x) - d.hi - d.lo;
    if (static_cast<double>(d.hi) != hi_want || std::fabs(static_cast<double>(r)) > std::ldexp(std::fabs(x), -46)) {
      if (bad_split++ < 5) printf("df_of %a: %a + %a\n", x, d.hi, d.lo);
    }
  }
  for (double x : {0.0, 1e-30, 1e40, static_cast<double>(INFINITY), static_cast<double>(NAN)}) {
    df d;
    if (df_of(x, &d) && bad_split++ < 5) printf("df_of accepted %a\n", x);
  }
  printf("df_of failures: %lld\n", bad_split);
  fails += bad_split != 0;

  // the right-hand side: smooth stencils (neighbours within a relative
  // perturbation of the centre, as on a resolved grid), rough ones, the
  // boundary form (one neighbour twice), and values far from 1
  const char *kinds[4] = {"smooth", "rough", "boundary", "wide"};
  double worst[4] = {0, 0, 0, 0};
  long long refused[4] = {0, 0, 0, 0};
  for (long long i = 0; i < count; ++i) {
    const int kind = static_cast<int>(i % 4);
    const double scale = kind == 3 ? std::ldexp(1.0, static_cast<int>(next() % 60) - 30) : 1.0;
    const pr c = {scale * (0.05 + 6.0 * unif()), scale * (0.05 + 6.0 * unif())};
    const double pert = std::ldexp(1.0, -static_cast<int>(next() % 40));
    pr n[4];
    for (int k = 0; k < 4; ++k) {
      if (kind == 1) {
        n[k] = {scale * (0.05 + 6.0 * unif()), scale * (0.05 + 6.0 * unif())};
      } else {
        n[k] = {c.x * (1.0 + pert * (2.0 * unif() - 1.0)), c.y * (1.0 + pert * (2.0 * unif() - 1.0))};
      }
    }
    if (kind == 2) n[3] = n[2];
    const double coef = std::ldexp(1.0 + unif(), static_cast<int>(next() % 40));
    df cf;
    df_of(coef, &cf);
    df fu, fv;
    if (!bruss_rhs_df(c, n[0], n[1], n[2], n[3], cf, &fu, &fv)) {
      if (refused[kind]++ < 3) printf("refused %s: u %a v %a\n", kinds[kind], c.x, c.y);
      continue;
    }
    typedef long double ld;
    const ld u = c.x, v = c.y;
    const ld lu = (static_cast<ld>(n[0].x) + n[1].x + n[2].x + n[3].x) - 4.0L * u;
    const ld lv = (static_cast<ld>(n[0].y) + n[1].y + n[2].y + n[3].y) - 4.0L * v;
    const ld u2v = u * u * v;
    const ld k44 = static_cast<ld>(4.4), k34 = static_cast<ld>(3.4);
    const ld Fu = 1.0L + u2v - k44 * u + static_cast<ld>(coef) * lu;
    const ld Fv = k34 * u - u2v + static_cast<ld>(coef) * lv;
    double M = std::fabs(c.x) > std::fabs(c.y) ? std::fabs(c.x) : std::fabs(c.y);
    for (int k = 0; k < 4; ++k) M = std::fmax(M, std::fmax(std::fabs(n[k].x), std::fabs(n[k].y)));
    const double Tu = 1.0 + std::fabs(static_cast<double>(u2v)) + 4.4 * std::fabs(c.x) +
                      coef * std::fabs(static_cast<double>(lu));
    const double Tv = 3.4 * std::fabs(c.x) + std::fabs(static_cast<double>(u2v)) +
                      coef * std::fabs(static_cast<double>(lv));
    const double eu = std::fabs(static_cast<double>(static_cast<ld>(fu.hi) + fu.lo - Fu));
    const double ev = std::fabs(static_cast<double>(static_cast<ld>(fv.hi) + fv.lo - Fv));
    const double bu = std::ldexp(Tu, -42) + std::ldexp(coef * M, -53);
    const double bv = std::ldexp(Tv, -42) + std::ldexp(coef * M, -53);
    worst[kind] = std::fmax(worst[kind], std::fmax(eu / bu, ev / bv));
  }
  for (int k = 0; k < 4; ++k) {
    printf("bruss_rhs_df %-8s worst error / bound %.3f, refused %lld\n", kinds[k], worst[k], refused[k]);
    fails += worst[k] > 1.0 || refused[k] != 0;
  }
  return fails != 0;
}
