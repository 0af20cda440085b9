// Correctly rounded x^y for the step-size controller, host and device.
//
// The controller's factor 0.9 * (tol/err)^(1/(ord+1)) (include/tools.h:226)
// decides every later step size, and near the stability limit of an explicit
// method a one-ulp change of h can turn an accepted step into a rejected one.
// The reference evaluates it with glibc's pow, which is correctly rounded
// except in rare near-halfway cases, so a correctly rounded pow reproduces the
// reference's step sizes.  CUDA's pow() (up to 2 ulp) does not.
//
// Method (double-double arithmetic, about 100 bits):
//   log x  = k ln2 + 2 atanh(s),  x = 2^k m, m in [1/sqrt2, sqrt2), s = (m-1)/(m+1),
//            atanh(s) = s (1 + z/3 + z^2/5 + ...), z = s^2 (|s| <= 0.1716)
//   exp t  = 2^j exp(f)^(2^8) ... with f = (t - j ln2) / 2^8, Taylor series of
//            exp(f) (|f| <= 0.00136), then eight double-double squarings
// and one final rounding of the double-double result.  Error-free
// transformations (TwoSum, FMA-based TwoProd) follow Dekker/Knuth; the host
// build must not contract a*b+c (compiled with -ffp-contract=off).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define RKCU_HD __host__ __device__ __forceinline__
#else
#define RKCU_HD inline
#endif

namespace rkcu {
namespace crpow {

RKCU_HD double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
RKCU_HD double sub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
RKCU_HD double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
RKCU_HD double fma_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
RKCU_HD double div_(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
RKCU_HD int64_t bits(double x) {
  int64_t b;
#ifdef __CUDA_ARCH__
  b = __double_as_longlong(x);
#else
  std::memcpy(&b, &x, 8);
#endif
  return b;
}
RKCU_HD double from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}
// 2^e for -1022 <= e <= 1023
RKCU_HD double pow2i(int e) { return from_bits(static_cast<int64_t>(e + 1023) << 52); }

struct dd {
  double hi, lo;
};

RKCU_HD dd two_sum(double a, double b) {
  const double s = add(a, b);
  const double bb = sub(s, a);
  const double e = add(sub(a, sub(s, bb)), sub(b, bb));
  return {s, e};
}
RKCU_HD dd fast_two_sum(double a, double b) {  // |a| >= |b|
  const double s = add(a, b);
  return {s, sub(b, sub(s, a))};
}
RKCU_HD dd two_prod(double a, double b) {
  const double p = mul(a, b);
  return {p, fma_(a, b, -p)};
}
RKCU_HD dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  const dd t = two_sum(a.lo, b.lo);
  s.lo = add(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = add(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
RKCU_HD dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo = add(p.lo, add(mul(a.hi, b.lo), mul(a.lo, b.hi)));
  return fast_two_sum(p.hi, p.lo);
}
RKCU_HD dd dd_mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo = fma_(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
RKCU_HD dd dd_div(dd a, dd b) {
  const double q1 = div_(a.hi, b.hi);
  dd r = dd_add(a, dd_mul_d(b, -q1));
  const double q2 = div_(r.hi, b.hi);
  r = dd_add(r, dd_mul_d(b, -q2));
  const double q3 = div_(r.hi, b.hi);
  dd q = fast_two_sum(q1, q2);
  return dd_add(q, dd{q3, 0.0});
}
// 1/d as a double-double, d a small integer
RKCU_HD dd dd_recip(double d) {
  const double h = div_(1.0, d);
  return {h, div_(fma_(-h, d, 1.0), d)};
}
RKCU_HD dd ln2() {  // ln 2 = 0.69314718055994530941723212145817656807550013436...
  return {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
}

// log x for a normal x > 0, as a double-double
RKCU_HD dd log_dd(double x) {
  const int64_t b = bits(x);
  int k = static_cast<int>((b >> 52) & 0x7ff) - 1023;
  double m = from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);  // [1, 2)
  if (m > 1.4142135623730951) {
    m = mul(m, 0.5);
    ++k;
  }
  const double num = sub(m, 1.0);  // exact (Sterbenz)
  const dd s = dd_div(dd{num, 0.0}, two_sum(m, 1.0));
  const dd z = dd_mul(s, s);
  // tail 1/9 + z/11 + ... + z^12/33 in double (its contribution is below 2^-23)
  double tail = div_(1.0, 33.0);
  for (int d = 31; d >= 9; d -= 2) tail = add(div_(1.0, static_cast<double>(d)), mul(z.hi, tail));
  dd q = dd_mul_d(z, tail);
  q = dd_mul(dd_add(q, dd_recip(7.0)), z);
  q = dd_mul(dd_add(q, dd_recip(5.0)), z);
  q = dd_mul(dd_add(q, dd_recip(3.0)), z);
  q = dd_add(q, dd{1.0, 0.0});
  dd lm = dd_mul(s, q);
  lm.hi = mul(lm.hi, 2.0);
  lm.lo = mul(lm.lo, 2.0);
  return dd_add(dd_mul_d(ln2(), static_cast<double>(k)), lm);
}

// exp t for |t| <= 700, rounded once to double.  *near_half is set when the
// exact value lies within 0.03 ulp of a rounding boundary (halfway between two
// doubles), i.e. where a pow with up to 0.52 ulp error may round the other way.
RKCU_HD double exp_dd(dd t, bool *near_half) {
  const double j = rint(mul(t.hi, 1.4426950408889634));
  dd f = dd_add(t, dd_mul_d(ln2(), -j));
  f.hi = mul(f.hi, 0x1p-8);
  f.lo = mul(f.lo, 0x1p-8);
  // exp(f) = 1 + f + f^2/2 + f^3 (1/6 + f/24 + ... + f^6/362880 ...), |f| < 0.00136
  const double g = f.hi;
  double p = div_(1.0, 362880.0);
  p = add(div_(1.0, 40320.0), mul(g, p));
  p = add(div_(1.0, 5040.0), mul(g, p));
  p = add(div_(1.0, 720.0), mul(g, p));
  p = add(div_(1.0, 120.0), mul(g, p));
  p = add(div_(1.0, 24.0), mul(g, p));
  dd e = dd_add(dd_recip(6.0), dd{mul(g, p), 0.0});
  const dd f2 = dd_mul(f, f);
  e = dd_mul(e, dd_mul(f2, f));
  dd half_f2 = {mul(f2.hi, 0.5), mul(f2.lo, 0.5)};
  e = dd_add(e, half_f2);
  e = dd_add(e, f);
  e = dd_add(e, dd{1.0, 0.0});
  for (int r = 0; r < 8; ++r) e = dd_mul(e, e);
  const double v = add(e.hi, e.lo);
  {
    // distance of the exact value from v, in ulps of v (v is within 1 ulp of e.hi,
    // so e.hi - v is exact); a power of two straddles two ulp sizes: call it hard
    const double r = add(sub(e.hi, v), e.lo);
    const int64_t vb = bits(v);
    const double ulp = from_bits(vb & 0x7ff0000000000000LL) * 0x1p-52;
    const bool pow2 = (vb & 0x000fffffffffffffLL) == 0;
    *near_half = pow2 || fabs(r) > 0.47 * ulp;
  }
  const int ji = static_cast<int>(j);
  // scale by 2^j in two exact steps so that no intermediate overflows
  return mul(mul(v, pow2i(ji / 2)), pow2i(ji - ji / 2));
}

}  // namespace crpow

// x^y, correctly rounded for x in [2^-60, 2^60] and |y| <= 1 (the range in which
// the controller's clamp to [0.5, 2] does not hide the value); outside it the
// platform pow is used.  *near_half as in exp_dd (false outside the range).
RKCU_HD double pow_cr(double x, double y, bool *near_half) {
  *near_half = false;
  if (!(x >= 0x1p-60 && x <= 0x1p60) || !(y >= -1.0 && y <= 1.0)) return pow(x, y);
  if (y == 0.0 || x == 1.0) return 1.0;
  const crpow::dd l = crpow::log_dd(x);
  return crpow::exp_dd(crpow::dd_mul_d(l, y), near_half);
}

// Step-size update of include/tools.h:221-233 (AMAX 2, AMIN 0.5, ASAF 0.9):
// h * min(2, max(0.5, 0.9 * (tol/err)^(1/(ord+1)))).  *host_pow is set when the
// power is so close to a rounding boundary that the C library's pow (the
// reference's) may round it differently and the clamp does not hide it; the
// caller then finishes the update with that pow on the host.
RKCU_HD double step_factor_h(double h, double err, double tol, int ord, bool *host_pow) {
  *host_pow = false;
  if (tol <= 0.0) return h;
  const double q = crpow::div_(tol, err);
  const double e = crpow::div_(1.0, crpow::add(static_cast<double>(ord), 1.0));
  bool near_half = false;
  const double p = crpow::mul(0.9, pow_cr(q, e, &near_half));
  *host_pow = near_half && p > 0.49 && p < 2.01;
  return crpow::mul(h, fmin(2.0, fmax(0.5, p)));
}

}  // namespace rkcu
