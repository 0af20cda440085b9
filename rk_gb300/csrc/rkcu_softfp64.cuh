// IEEE-754 binary64 multiply and add, round to nearest even, on 32-bit integer
// instructions -- host and device.
//
// On GB300 the FP64 pipe issues 2 instructions per SM per clock while the SM
// issues 128 integer instructions per clock, so a double product or sum built
// from about 30-50 integer instructions costs less issue time than the FP64
// pipe spends on the hardware instruction, and both can run at once.  These
// functions give exactly the hardware's result: the fast path covers normal
// operands with a normal result, everything else (zeros, subnormals,
// infinities, NaNs, results that overflow or underflow) is handed to the
// hardware instruction.
//
// Method: the 53-bit significands are multiplied exactly as four 32x32->64
// partial products (106-bit product) or aligned with guard and sticky bits
// and added in 64-bit registers; the result is rounded to 53 bits, ties to
// even, and the exponent and significand are assembled with one addition of
// (exponent - 1) << 52, so that a rounding carry into 2^53 moves the exponent
// up by itself.
//
// Also here: the BRUSS2D-MIX Laplacian's four rounded sums computed exactly in
// 64-bit integers when the five operands share one binade (lap_same_binade),
// about 70 integer instructions in place of 4 on the FP64 pipe.  The measured
// balance: the products pay in the plain kernel's exact mode (tableau
// products) and the Laplacian pays everywhere; a general software sum does not
// (its alignment and normalisation cost more issue slots than the FP64 pipe
// time it frees).  And the exact comparison of two quotients a / d > c / e by
// their 106-bit cross products (quotients_greater), which lets the error norm's
// maximum be found without a division per candidate.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SFP_HD __host__ __device__ __forceinline__
#else
#define SFP_HD inline
#endif

namespace rkcu {
namespace softfp {

SFP_HD uint64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}

SFP_HD double double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(b));
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

SFP_HD int clz64(uint64_t x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll(static_cast<long long>(x));
#else
  return __builtin_clzll(x);
#endif
}

// The rare paths are real calls, not inlined: inlined, the compiler would
// if-convert them and run the FP64 instruction for every lane, which would
// defeat the purpose of moving the product off the FP64 pipe.
#ifdef __CUDACC__
static __host__ __device__ __noinline__ double hw_mul(double a, double b) {
#else
inline double hw_mul(double a, double b) {
#endif
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__ double hw_add(double a, double b) {
#else
inline double hw_add(double a, double b) {
#endif
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__ float hw_to_float(double x) {
#else
inline float hw_to_float(double x) {
#endif
#ifdef __CUDA_ARCH__
  return __double2float_rn(x);
#else
  return static_cast<float>(x);
#endif
}

#ifdef __CUDACC__
static __host__ __device__ __noinline__ double hw_to_double(float x) {
#else
inline double hw_to_double(float x) {
#endif
  return static_cast<double>(x);
}

SFP_HD float float_of(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, 4);
  return x;
#endif
}

// x rounded to the nearest float, ties to even (a double -> float conversion
// runs on the FP64 pipe on this part).  Results outside the normal float range
// (and zeros, infinities, NaNs) come from the hardware conversion.
SFP_HD float to_float(double x) {
  const uint64_t bx = bits_of(x);
  const uint32_t hi = static_cast<uint32_t>(bx >> 32);
  const int e = static_cast<int>((hi >> 20) & 0x7ff) - 1023 + 127;  // float exponent field
  if (e <= 0 || e >= 255) return hw_to_float(x);
  const uint64_t m = bx & 0x000fffffffffffffull;
  uint32_t r = static_cast<uint32_t>(m >> 29);   // the 23 kept significand bits
  const uint64_t rest = m & 0x1fffffffull;       // the 29 dropped ones
  r += static_cast<uint32_t>(rest > 0x10000000ull) | (static_cast<uint32_t>(rest == 0x10000000ull) & (r & 1u));
  // a carry out of the significand moves the exponent up (to infinity past the range)
  return float_of(((hi & 0x80000000u) | (static_cast<uint32_t>(e) << 23)) + r);
}

// a * b rounded to nearest even
SFP_HD double mul(double a, double b) {
  const uint64_t ab = bits_of(a), bb = bits_of(b);
  const uint32_t ahi = static_cast<uint32_t>(ab >> 32), alo = static_cast<uint32_t>(ab);
  const uint32_t bhi = static_cast<uint32_t>(bb >> 32), blo = static_cast<uint32_t>(bb);
  const int ea = static_cast<int>((ahi >> 20) & 0x7ff);
  const int eb = static_cast<int>((bhi >> 20) & 0x7ff);
  const uint32_t ma = (ahi & 0xfffffu) | 0x100000u;  // high 21 significand bits
  const uint32_t mb = (bhi & 0xfffffu) | 0x100000u;
  // 106-bit product  ma:alo * mb:blo = up * 2^64 + mid * 2^32 + low
  const uint64_t t0 = static_cast<uint64_t>(alo) * blo;
  const uint64_t t1 = static_cast<uint64_t>(ma) * blo + (t0 >> 32);
  const uint64_t mm = static_cast<uint64_t>(alo) * mb + t1;  // < 2^55
  const uint64_t up = static_cast<uint64_t>(ma) * mb + (mm >> 32);  // in [2^40, 2^42)
  const uint32_t mid = static_cast<uint32_t>(mm);
  const uint32_t low = static_cast<uint32_t>(t0);
  const int norm = static_cast<int>(up >> 41);  // product >= 2^105
  const int e = ea + eb - 1023 + norm;          // biased exponent of the result
  if (ea == 0 || ea == 0x7ff || eb == 0 || eb == 0x7ff || e < 1 || e > 2046) return hw_mul(a, b);
  // significand = product >> (52 + norm), 53 bits
  const int sh = 20 + norm;
  uint64_t m = (up << (32 - sh)) | (mid >> sh);
  const uint32_t rbit = (mid >> (sh - 1)) & 1u;
  const uint32_t sticky = (mid & ((1u << (sh - 1)) - 1u)) | low;
  m += rbit & ((sticky != 0u) | static_cast<uint32_t>(m & 1u));
  const uint64_t sign = (ab ^ bb) & 0x8000000000000000ull;
  return double_of(sign | ((static_cast<uint64_t>(e - 1) << 52) + m));
}

// a + b rounded to nearest even
SFP_HD double add(double a, double b) {
  uint64_t ab = bits_of(a), bb = bits_of(b);
  // order by magnitude: |a| >= |b|
  if ((ab & 0x7fffffffffffffffull) < (bb & 0x7fffffffffffffffull)) {
    const uint64_t t = ab;
    ab = bb;
    bb = t;
  }
  const int ea = static_cast<int>((ab >> 52) & 0x7ff);
  const int eb = static_cast<int>((bb >> 52) & 0x7ff);
  if (ea == 0 || ea == 0x7ff || eb == 0 || eb == 0x7ff) return hw_add(a, b);
  // significands with the hidden bit at 2^62 (10 guard bits below the 53)
  const uint64_t ma = ((ab & 0x000fffffffffffffull) | 0x0010000000000000ull) << 10;
  uint64_t mb = ((bb & 0x000fffffffffffffull) | 0x0010000000000000ull) << 10;
  const int d = ea - eb;
  if (d >= 64) {
    mb = 1;  // only a sticky bit remains
  } else if (d > 0) {
    mb = (mb >> d) | static_cast<uint64_t>((mb << (64 - d)) != 0);
  }
  const bool subtract = ((ab ^ bb) >> 63) != 0;
  uint64_t s;
  int e = ea;
  if (!subtract) {
    s = ma + mb;  // < 2^64
    if (s >> 63) {
      s = (s >> 1) | (s & 1u);
      ++e;
    }
  } else {
    s = ma - mb;
    if (s == 0) return hw_add(a, b);  // exact cancellation: +0 (sign rules) from the hardware
    const int lz = clz64(s) - 1;        // bring the leading bit to 2^62
    s <<= lz;
    e -= lz;
  }
  if (e < 1 || e > 2046) return hw_add(a, b);
  // round 63-bit s to 53 bits: drop 10 bits
  const uint64_t rbit = (s >> 9) & 1u;
  const uint64_t sticky = s & 0x1ffu;
  uint64_t m = s >> 10;
  m += rbit & ((sticky != 0u) | (m & 1u));
  const uint64_t sign = ab & 0x8000000000000000ull;
  return double_of(sign | ((static_cast<uint64_t>(e - 1) << 52) + m));
}

// The high 64 bits of the 128-bit product a * b.
SFP_HD uint64_t mul_hi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

// Whether a / d > c / e holds exactly, for positive normal doubles given as
// bit patterns: a e > c d with both 106-bit products of the significands in
// integers.  With t = (ea + ee) - (ec + ed) the products scale as ma me 2^t
// against mc md, both in [2^104, 2^106), so |t| >= 2 decides by itself.
SFP_HD bool quotients_greater(uint64_t ba, uint64_t bd, uint64_t bc, uint64_t be) {
  constexpr uint64_t kF = 0x000fffffffffffffull, kH = 0x0010000000000000ull;
  const int t = static_cast<int>(ba >> 52) + static_cast<int>(be >> 52) - static_cast<int>(bc >> 52) -
                static_cast<int>(bd >> 52);
  if (t >= 2) return true;
  if (t <= -2) return false;
  const uint64_t ma = (ba & kF) | kH, md = (bd & kF) | kH, mc = (bc & kF) | kH, me = (be & kF) | kH;
  uint64_t h1 = mul_hi64(ma, me), l1 = ma * me, h2 = mul_hi64(mc, md), l2 = mc * md;
  if (t == 1) {
    h1 = (h1 << 1) | (l1 >> 63);
    l1 <<= 1;
  } else if (t == -1) {
    h2 = (h2 << 1) | (l2 >> 63);
    l2 <<= 1;
  }
  return h1 > h2 || (h1 == h2 && l1 > l2);
}

// s rounded to a multiple of 2^k (k = 1, 2), ties to an even multiple of 2^k:
// the rounding of a sum of same-binade significands to the binade above.
SFP_HD uint64_t round_units(uint64_t s, int k) {
  const uint64_t q = s >> k, r = s & ((1ull << k) - 1u), half = 1ull << (k - 1);
  return (q + static_cast<uint64_t>((r > half) | ((r == half) & ((q & 1u) != 0u)))) << k;
}

// The five-point Laplacian of BRUSS2D-MIX in the order of its FP64 code,
//   interior (jcase 0):        ((n + s) + w) + e - 4 c
//   first/last column (1, 2):  (n + s) + 2 t - 4 c      (t = the inner neighbour)
// each operation rounded to nearest even, computed exactly in 64-bit integers
// when all operands have one sign and one exponent field (a resolved field):
// the significands then share one unit, n + s rounds to the binade above, the
// next sum to the binade above that or the one after, and the final difference
// is exact (Sterbenz: both operands lie in [2^54, 2^55] units).  Returns
// false, leaving *out unset, for any other operands.
SFP_HD bool lap_same_binade(double n, double s, double w, double e, double c, int jcase, double *out) {
  const uint64_t bn = bits_of(n), bs = bits_of(s), bw = bits_of(w), be = bits_of(e), bc = bits_of(c);
  const uint32_t top = static_cast<uint32_t>(bc >> 52);  // sign and exponent field
  const uint32_t ef = top & 0x7ffu;
  if (static_cast<uint32_t>(bn >> 52) != top || static_cast<uint32_t>(bs >> 52) != top ||
      static_cast<uint32_t>(bw >> 52) != top || static_cast<uint32_t>(be >> 52) != top || ef == 0u || ef > 2043u)
    return false;  // (the partial sums reach three binades up: no overflow below 2044)
  constexpr uint64_t kF = 0x000fffffffffffffull, kH = 0x0010000000000000ull;
  const uint64_t r1 = round_units(((bn & kF) | kH) + ((bs & kF) | kH), 1);  // in [2^53, 2^54]
  uint64_t r;
  if (jcase == 0) {
    const uint64_t s2 = r1 + ((bw & kF) | kH);                  // in [3 2^52, 3 2^53)
    const uint64_t r2 = round_units(s2, s2 >= (1ull << 54) ? 2 : 1);
    r = round_units(r2 + ((be & kF) | kH), 2);                   // in [2^54, 2^55]
  } else {
    const uint64_t t = jcase == 1 ? be : bw;
    r = round_units(r1 + (((t & kF) | kH) << 1), 2);              // in [2^54, 2^55]
  }
  const int64_t L = static_cast<int64_t>(r) - static_cast<int64_t>(((bc & kF) | kH) << 2);  // exact
  if (L == 0) {
    *out = 0.0;  // x - x is +0 in round to nearest
    return true;
  }
  const uint64_t a = L < 0 ? static_cast<uint64_t>(-L) : static_cast<uint64_t>(L);  // a multiple of 4, <= 2^54
  const int p = 63 - clz64(a);                     // value = a 2^(ef - 1075) = 1.f 2^(p + ef - 1075)
  const int f = p + static_cast<int>(ef) - 52;     // biased exponent of the result
  if (f < 1) return false;                          // subnormal: not on this path
  const uint64_t m = p >= 52 ? (a >> (p - 52)) : (a << (52 - p));  // exact: a's low 2 bits are 0
  const uint64_t sign = (static_cast<uint64_t>(top & 0x800u) << 52) ^ (L < 0 ? 0x8000000000000000ull : 0ull);
  *out = double_of(sign | ((static_cast<uint64_t>(f - 1) << 52) + m));
  return true;
}

}  // namespace softfp
}  // namespace rkcu
