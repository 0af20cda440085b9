// Double-float (pairs of FP32) arithmetic and a fixed-point stencil sum on
// 32-bit integer instructions -- host and device.
//
// On GB300 the FP64 pipe issues 2 instructions per SM per clock against 128
// FP32 or integer lanes.  The mixed-precision form needs F0 = f(y) to about
// 1e-13 relative (it enters y through h F0 every step), which FP32 alone does
// not give: alpha (N-1)^2 multiplies the Laplacian of y, so the Laplacian must
// be formed from y without FP32 rounding.  Here
//   * the five-point sum n0 + n1 + n2 + n3 - 4c is exact in 64-bit fixed point
//     at the scale of the largest operand (6 guard bits; each operand loses at
//     most 2^-58 of that scale in the alignment), then split into an FP32 pair;
//   * everything else (products, sums) is double-float arithmetic on the FP32
//     pipe: a value is hi + lo with |lo| < ulp(hi), about 46 significant bits;
//   * conversions between double and float are built from the bit fields with
//     integer instructions (a conversion instruction runs on the FP64 pipe).
// Inputs outside the ranges these handle (zeros, subnormals, infinities, NaNs,
// magnitudes outside [2^-80, 2^127)) make the functions return false; the
// caller then uses FP64 arithmetic for that point.
//
// Methods: Dekker's and Knuth's error-free transformations (TwoSum,
// Fast2Sum, and TwoProduct through a fused multiply-add), with the "sloppy"
// double-float sum and product of Hida, Li and Bailey's QD library (2001):
// absolute error a few units of 2^-46 of the operands' magnitudes.
// All FP32 operations are explicitly rounded (no contraction), so the host and
// the device give the same bits.
#pragma once

#include <cmath>

#include "rkcu_softfp64.cuh"

namespace rkcu {
namespace dfl {

struct df {
  float hi, lo;
};

SFP_HD float f_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
SFP_HD float f_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
SFP_HD float f_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
SFP_HD float f_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

SFP_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return b;
#endif
}

// s + e = a + b exactly (Knuth's TwoSum)
SFP_HD df two_sum(float a, float b) {
  const float s = f_add(a, b);
  const float bb = f_sub(s, a);
  const float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
  return {s, e};
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Fast2Sum)
SFP_HD df fast_two_sum(float a, float b) {
  const float s = f_add(a, b);
  return {s, f_sub(b, f_sub(s, a))};
}

// p + e = a * b exactly (TwoProduct with a fused multiply-add)
SFP_HD df two_prod(float a, float b) {
  const float p = f_mul(a, b);
  return {p, f_fma(a, b, -p)};
}

SFP_HD df df_neg(df a) { return {-a.hi, -a.lo}; }

SFP_HD df df_add(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, f_add(s.lo, f_add(a.lo, b.lo)));
}

SFP_HD df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

SFP_HD df df_mul(df a, df b) {
  const df p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, f_add(p.lo, f_fma(a.hi, b.lo, f_mul(a.lo, b.hi))));
}

// x (a double) as a float exactly, from the bit fields: float -> double is
// exact, and the conversion instruction would use the FP64 pipe.  Zeros are
// built here as well; subnormal floats, infinities and NaNs use the
// instruction (out of line, so it is not if-converted into every lane).
SFP_HD double dbl_of(float x) {
  const uint32_t b = fbits(x);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) {
    if ((b & 0x7fffffffu) == 0u) return softfp::double_of(static_cast<uint64_t>(b) << 32);
    return softfp::hw_to_double(x);
  }
  const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
  return softfp::double_of((static_cast<uint64_t>(hi) << 32) | (static_cast<uint64_t>(b & 7u) << 29));
}

// x (a double) as hi + lo: hi = x truncated to 24 significant bits, lo = the
// next 23 bits (truncated); |x - hi - lo| < 2^-46 |x|.  False unless
// 2^-80 <= |x| < 2^128 (so that hi and lo are normal floats).
SFP_HD bool df_of(double x, df *out) {
  const uint64_t b = softfp::bits_of(x);
  const uint32_t hw = static_cast<uint32_t>(b >> 32), lw = static_cast<uint32_t>(b);
  const int ex = static_cast<int>((hw >> 20) & 0x7ffu);
  if (ex < 943 || ex > 1150) return false;
  const uint32_t sg = hw & 0x80000000u;
  const float hi =
      softfp::float_of(sg | (static_cast<uint32_t>(ex - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  // the remaining 29 significand bits, top 23 of them as an integer-valued
  // float (2^23 + r - 2^23 is exact), times 2^(ex - 1069)
  const uint32_t r = (lw & 0x1fffffffu) >> 6;
  const float lo = f_mul(f_sub(softfp::float_of(0x4b000000u | r), 8388608.0f),
                         softfp::float_of(sg | (static_cast<uint32_t>(ex - 942) << 23)));
  *out = {hi, lo};
  return true;
}

// n0 + n1 + n2 + n3 - 4 c through 64-bit fixed point at the scale 2^(E-1081)
// of the largest operand's exponent field E: each significand is shifted to
// that scale (at most 2^-58 of 2^(E-1023) is lost per operand), the sum is
// exact (|sum| < 2^62), and the result is split into hi (24 bits) + lo (the
// next 23 bits).  False for zero, subnormal, infinite or NaN operands, or a
// nonzero result outside the normal float range.
// General case: operands of any signs and exponents; E < 0 when an operand is
// zero, subnormal, infinite or NaN.  Out of line (by value, so that the fast
// path keeps its operands in registers).
struct LapAcc {
  int64_t acc;
  int E;
};
SFP_HD LapAcc lap_acc_general(uint64_t b0, uint64_t b1, uint64_t b2, uint64_t b3, uint64_t b4) {
  const uint64_t b[5] = {b0, b1, b2, b3, b4};
  int e[5];
  int E = 0, emin = 0x7ff;
  for (int k = 0; k < 5; ++k) {
    e[k] = static_cast<int>((b[k] >> 52) & 0x7ff);
    E = e[k] > E ? e[k] : E;
    emin = e[k] < emin ? e[k] : emin;
  }
  if (emin == 0 || E == 0x7ff) return {0, -1};
  int64_t acc = 0;
  for (int k = 0; k < 5; ++k) {
    const int sh = E - e[k];
    uint64_t m = ((b[k] & 0x000fffffffffffffull) | 0x0010000000000000ull) << 6;  // < 2^59
    m = sh < 64 ? (m >> sh) : 0ull;
    if (k == 4) m <<= 2;  // 4 c, < 2^61
    const bool neg = ((b[k] >> 63) != 0) != (k == 4);
    acc += neg ? -static_cast<int64_t>(m) : static_cast<int64_t>(m);
  }
  return {acc, E};
}

SFP_HD bool lap_fixed(double c, double n0, double n1, double n2, double n3, df *out) {
  const uint64_t b[5] = {softfp::bits_of(n0), softfp::bits_of(n1), softfp::bits_of(n2), softfp::bits_of(n3),
                         softfp::bits_of(c)};
  // Fast path (a resolved field: all five of one sign and one binade): the
  // significands are already at one scale, so the sum needs no alignment;
  // 2^(E-1075) units, |sum| < 2^56, shifted up by 6 to the general path's scale.
  const uint32_t top = static_cast<uint32_t>(b[4] >> 52);
  int64_t acc;
  int E;
  if (static_cast<uint32_t>(b[0] >> 52) == top && static_cast<uint32_t>(b[1] >> 52) == top &&
      static_cast<uint32_t>(b[2] >> 52) == top && static_cast<uint32_t>(b[3] >> 52) == top &&
      (top & 0x7ffu) != 0u && (top & 0x7ffu) != 0x7ffu) {
    constexpr uint64_t kF = 0x000fffffffffffffull;
    const int64_t s = static_cast<int64_t>(((b[0] & kF) + (b[1] & kF)) + ((b[2] & kF) + (b[3] & kF))) -
                      static_cast<int64_t>((b[4] & kF) << 2);  // the hidden bits cancel (4 - 4)
    acc = (top & 0x800u) ? -s : s;
    acc *= 64;
    E = static_cast<int>(top & 0x7ffu);
  } else {
    const LapAcc g = lap_acc_general(b[0], b[1], b[2], b[3], b[4]);
    if (g.E < 0) return false;
    acc = g.acc;
    E = g.E;
  }
  if (acc == 0) {
    *out = {0.0f, 0.0f};
    return true;
  }
  const uint32_t sg = acc < 0 ? 0x80000000u : 0u;
  const uint64_t a = acc < 0 ? static_cast<uint64_t>(-acc) : static_cast<uint64_t>(acc);
  const int lz = softfp::clz64(a);
  const uint64_t m = a << lz;  // value = m * 2^(E - 1081 - lz), m in [2^63, 2^64)
  const int fe = E - 891 - lz;  // float exponent field of hi = (m >> 40) * 2^(E - 1041 - lz)
  const int ls = E - 937 - lz;  // of 2^(E - 1064 - lz), the unit of lo = bits 39..17 of m
  if (fe > 254 || fe < 1) return false;
  const float hi = softfp::float_of(sg | (static_cast<uint32_t>(fe) << 23) |
                                    (static_cast<uint32_t>(m >> 40) & 0x7fffffu));
  // lo is dropped where its unit is below the normal floats (then |lo| <
  // 2^-102 |hi|)
  const uint32_t r = static_cast<uint32_t>(m >> 17) & 0x7fffffu;
  const float lo = ls < 1 ? 0.0f
                          : f_mul(f_sub(softfp::float_of(0x4b000000u | r), 8388608.0f),
                                  softfp::float_of(sg | (static_cast<uint32_t>(ls) << 23)));
  *out = {hi, lo};
  return true;
}

// Constants of the BRUSS2D-MIX reaction terms as double-float pairs of the
// doubles 4.4 and 3.4 (folded at compile time).
constexpr float k44h = 4.4f;
constexpr float k44l = static_cast<float>(4.4 - static_cast<double>(k44h));
constexpr float k34h = 3.4f;
constexpr float k34l = static_cast<float>(3.4 - static_cast<double>(k34h));

// BRUSS2D-MIX right-hand side at one grid point (the formulas of
// src/problems/bruss2d-mix.c:66-206 and 579-667):
//   U: 1 + u^2 v - 4.4 u + coef lap(u),   V: 3.4 u - u^2 v + coef lap(v)
// with c = (u, v) at the point and its four neighbours' pairs (a boundary
// passes the inner neighbour twice).  Absolute error a few units of 2^-46 of
// the terms' magnitudes (plus 2^-55 coef max|y| from the fixed-point sum).
// P: any pair type with members x (u) and y (v), e.g. double2.
template <class P>
SFP_HD bool bruss_rhs_df(P c, P n0, P n1, P n2, P n3, df coef, df *fu, df *fv) {
  df lu, lv, u, v;
  if (!lap_fixed(c.x, n0.x, n1.x, n2.x, n3.x, &lu) || !lap_fixed(c.y, n0.y, n1.y, n2.y, n3.y, &lv) ||
      !df_of(c.x, &u) || !df_of(c.y, &v))
    return false;
  const df u2v = df_mul(df_mul(u, u), v);
  const df ru = df_sub(df_add(u2v, df{1.0f, 0.0f}), df_mul(df{k44h, k44l}, u));
  const df rv = df_sub(df_mul(df{k34h, k34l}, u), u2v);
  *fu = df_add(ru, df_mul(coef, lu));
  *fv = df_add(rv, df_mul(coef, lv));
  return true;
}

}  // namespace dfl
}  // namespace rkcu
