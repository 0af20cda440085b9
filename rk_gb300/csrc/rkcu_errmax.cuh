// The error norm's maximum, include/tools.h:280-288, per thread of a step
// loop: host and device (the host build is what tests/native checks against
// the reference's fmax chain).
#pragma once

#include <cmath>
#include <cstdint>

#include "rkcu_softfp64.cuh"

#ifdef __CUDACC__
#define EMX_HD __host__ __device__ __forceinline__
#define EMX_NOINLINE __host__ __device__ __noinline__
#else
#define EMX_HD inline
#define EMX_NOINLINE inline
#endif

namespace rkcu {

// Per-thread maximum of |e| / max(|y_new|, |y_old|) (include/tools.h:280-288)
// kept as a quotient num / den that is divided once, when it is read.  Rounding
// to nearest is monotonic, so the largest exact quotient rounds to the largest
// rounded one, which is what the reference's fmax chain keeps.  Two tests on
// the integer pipe decide whether a component raises the maximum.  The high
// word of a positive double, (exponent << 20) | top mantissa bits, is 2^20
// (log2 x + 1023) to within 0.086 * 2^20 (from below), so hi(|e|) - hi(divisor)
// estimates 2^20 log2(ratio) to within 0.086 * 2^20 either way; a component
// whose estimate is more than kMargin below the key of the current maximum
// cannot exceed it.  A component that passes is compared exactly
// (softfp::quotients_greater: |e| den > num divisor with the 106-bit products in
// integers) and, if larger, becomes the maximum without a division.  Zero or
// subnormal divisors and numerators, infinities and NaNs, and a maximum that is
// still zero or subnormal, take the division path, which stores its rounded
// quotient over 1.  The result is the largest of the quotients, a zero divisor
// counting as 1.7E308 and a NaN quotient ignored, as the reference's fmax chain
// gives it; the chain differs only where an infinite quotient comes before a
// zero divisor in its order (it then ends at 1.7E308, this at infinity), and
// the step control takes the same decision from either.
struct ErrMax {
  static constexpr int kMargin = 1 << 19;  // 0.5 in log2 units
  static constexpr uint64_t kMinNormal = 0x0010000000000000ull;
  static constexpr uint64_t kInf = 0x7ff0000000000000ull;
  static constexpr uint64_t kOne = 0x3ff0000000000000ull;
  static constexpr uint64_t kAbs = 0x7fffffffffffffffull;
  double num = 0.0, den = 1.0;
  uint64_t num_bits = 0, den_bits = kOne;
  int best_key = -0x40000000;

  // the maximum, rounded once
  EMX_HD double value() const { return den_bits == kOne ? num : num / den; }

  EMX_HD void add(double e, double yn, double yo) {
    const uint64_t ae = softfp::bits_of(e) & kAbs;
    const uint64_t an = softfp::bits_of(yn) & kAbs;
    const uint64_t ao = softfp::bits_of(yo) & kAbs;
    const uint64_t d = an > ao ? an : ao;  // an infinity or a NaN bit pattern if either is one
    const bool normal_d = d >= kMinNormal && d < kInf;
    if (ae == 0 && normal_d) return;  // a zero quotient never raises the maximum
    // Infinities and NaNs, zero or subnormal divisors and numerators (whose bit
    // patterns are no log estimate), and a maximum that is still zero or
    // subnormal: the division decides.
    if (!normal_d || ae < kMinNormal || ae >= kInf || num_bits < kMinNormal) {
      update(e, yn, yo);
      return;
    }
    const int key = static_cast<int>(ae >> 32) - static_cast<int>(d >> 32);
    if (key > best_key - kMargin && num_bits < kInf &&
        softfp::quotients_greater(ae, d, num_bits, den_bits)) {
      num = softfp::double_of(ae);
      den = softfp::double_of(d);
      num_bits = ae;
      den_bits = d;
      best_key = key;
    }
  }

  // the division path, kept out of line so that the division is not
  // if-converted (run for every lane) by the compiler
  EMX_NOINLINE void update(double e, double yn, double yo) {
    const double div = fmax(fabs(yn), fabs(yo));
    const double r = div == 0.0 ? 1.7E308 : fabs(e) / div;
    if (r > value()) {  // false for NaN, as fmax would ignore it
      num = r;
      den = 1.0;
      num_bits = softfp::bits_of(r);
      den_bits = kOne;
      best_key = static_cast<int>(num_bits >> 32) - 0x3ff00000;
    }
  }
};

}  // namespace rkcu
