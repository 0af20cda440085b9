// Bit-exactness check of the software binary64 multiply/add, the same-binade
// Laplacian and the exact quotient comparison (rkcu_softfp64.cuh) against the host's
// IEEE round-to-nearest arithmetic, and the error norm's maximum built on them
// (rkcu_errmax.cuh) against the fmax chain it replaces.  Compiled with
// -ffp-contract=off.  Usage: softfp64_check <count> <seed>; prints mismatches.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "rkcu_errmax.cuh"
#include "rkcu_softfp64.cuh"

using rkcu::softfp::add;
using rkcu::softfp::bits_of;
using rkcu::softfp::double_of;
using rkcu::softfp::mul;
using rkcu::softfp::to_float;

static uint64_t s_state;
static uint64_t next() {  // splitmix64
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// a random double of a chosen kind: any bit pattern, values near 1, a given
// exponent band, or a neighbour of another value (cancellation, near ties)
static double draw(int kind, double other) {
  const uint64_t r = next();
  switch (kind) {
    case 0: return double_of(r);
    case 1: return double_of((r & 0x800fffffffffffffull) | (static_cast<uint64_t>(1023 + (int)(r >> 53) % 8 - 4) << 52));
    case 2: return double_of((r & 0x800fffffffffffffull) | (static_cast<uint64_t>(1 + (r >> 52) % 2046) << 52));
    case 3: return double_of(bits_of(other) + (static_cast<int64_t>(r % 64) - 32));
    case 4: return -double_of(bits_of(other) + (r % 5));
    case 5: return double_of((r & 0x800fffffffffffffull) | (static_cast<uint64_t>((r >> 52) % 2) ? 1ull : 2045ull) << 52);
    default: return double_of((r & 0xfff0000000000000ull) | (r & 0x7));  // few mantissa bits: ties
  }
}

int main(int argc, char **argv) {
  const long long count = argc > 1 ? atoll(argv[1]) : 10000000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  long long bad_mul = 0, bad_add = 0, bad_cvt = 0;
  for (long long i = 0; i < count; ++i) {
    const int ka = static_cast<int>(next() % 7);
    const double a = draw(ka == 3 || ka == 4 ? 1 : ka, 0.0);
    const double b = draw(static_cast<int>(next() % 7), a);
    const double pm = a * b, sm = mul(a, b);
    const double pa = a + b, sa = add(a, b);
    const bool nan_m = pm != pm && sm != sm, nan_a = pa != pa && sa != sa;
    if (!nan_m && bits_of(pm) != bits_of(sm)) {
      if (bad_mul++ < 5)
        printf("mul %a * %a: hw %a sw %a\n", a, b, pm, sm);
    }
    if (!nan_a && bits_of(pa) != bits_of(sa)) {
      if (bad_add++ < 5)
        printf("add %a + %a: hw %a sw %a\n", a, b, pa, sa);
    }
    // double -> float rounding: the operands, the sum, doubles at the float
    // range edges, and exact halfway cases
    const uint64_t r = next();
    const int ee = (r >> 40) % 2 ? 1023 - 126 - static_cast<int>(r % 3) : 1023 + 127 - static_cast<int>(r % 2);
    const double cv[4] = {a, pa, double_of((next() & 0x800fffffffffffffull) | (static_cast<uint64_t>(ee) << 52)),
                          double_of((bits_of(a) & ~0x1fffffffull) | 0x10000000ull)};
    for (double x : cv) {
      const float hf = static_cast<float>(x), sf = to_float(x);
      uint32_t hb, sb;
      std::memcpy(&hb, &hf, 4);
      std::memcpy(&sb, &sf, 4);
      if (!(hf != hf && sf != sf) && hb != sb) {
        if (bad_cvt++ < 5)
          printf("to_float %a: hw %a sw %a\n", x, static_cast<double>(hf), static_cast<double>(sf));
      }
    }
  }
  printf("mismatches mul %lld add %lld to_float %lld of %lld\n", bad_mul, bad_add, bad_cvt, count);

  // the same-binade Laplacian against the FP64 sequence it replaces: operands
  // of one exponent field (random significands, significands near the top of
  // the binade, few-bit significands for ties), both signs, all three forms;
  // and operands of different binades, which it must refuse
  long long bad_lap = 0, taken = 0;
  for (long long i = 0; i < count; ++i) {
    const uint64_t r = next();
    const uint64_t ef = 1 + (r >> 11) % 2046;
    const uint64_t sg = (r >> 63) << 63;
    double v[5];
    for (int k = 0; k < 5; ++k) {
      const uint64_t q = next();
      uint64_t f;
      switch ((r >> (2 * k)) & 3) {
        case 0: f = q & 0x000fffffffffffffull; break;
        case 1: f = 0x000fffffffffffffull - (q & 0xff); break;               // near the top
        case 2: f = (q & 0xf) << ((q >> 8) % 49); break;                      // few bits: ties
        default: f = (q & 0x000fffffffffffffull) | 0x000ffffff0000000ull; break;
      }
      v[k] = double_of(sg | (ef << 52) | f);
    }
    if ((r >> 20) % 8 == 0) v[(r >> 24) % 5] = draw(2, 0.0);  // a different binade (usually)
    const int jcase = static_cast<int>((r >> 30) % 3);
    const double n = v[0], sv = v[1], w = jcase == 1 ? v[3] : v[2], e = jcase == 2 ? v[2] : v[3], c = v[4];
    double want = n + sv;
    if (jcase == 0)
      want = (want + w) + e;
    else
      want = std::fma(2.0, jcase == 1 ? e : w, want);
    want = std::fma(-4.0, c, want);
    double got = 0.0;
    const bool same = (bits_of(n) >> 52) == (bits_of(c) >> 52) && (bits_of(sv) >> 52) == (bits_of(c) >> 52) &&
                      (bits_of(w) >> 52) == (bits_of(c) >> 52) && (bits_of(e) >> 52) == (bits_of(c) >> 52) &&
                      ef <= 2043;
    const bool ok = rkcu::softfp::lap_same_binade(n, sv, w, e, c, jcase, &got);
    if (ok) ++taken;
    const bool sub = (bits_of(want) & 0x7ff0000000000000ull) == 0;  // subnormal or zero results may refuse
    if ((ok && bits_of(got) != bits_of(want) && want == want) || (ok && !same) || (!ok && same && !sub && want == want &&
                                                                                   std::fabs(want) < 1e300)) {
      if (bad_lap++ < 5) printf("lap %d: %a %a %a %a %a: fp64 %a int %a (ok %d)\n", jcase, n, sv, w, e, c, want, got, ok);
    }
  }
  printf("lap mismatches %lld (fast path taken %lld of %lld)\n", bad_lap, taken, count);

  // the exact comparison of two quotients a / d > c / e against the products
  // a e and c d and their FMA error terms: random operands, equal quotients
  // (c, e the same multiple of a, d) and their neighbours, and quotients one
  // rounding apart
  long long bad_q2 = 0, greater = 0;
  for (long long i = 0; i < count; ++i) {
    const uint64_t r0 = next(), r1 = next(), r2 = next(), r3 = next();
    auto band = [](uint64_t q, int lo, int span) {
      return double_of((q & 0x000fffffffffffffull) | (static_cast<uint64_t>(1023 + lo + static_cast<int>((q >> 52) % span)) << 52));
    };
    double a = band(r0, -250, 500), d = band(r1, -250, 500), c, e;
    switch (r3 % 4) {
      case 0: c = band(r2, -250, 500); e = band(r3, -250, 500); break;
      case 1: {  // c / e == a / d exactly, then moved by up to one unit in c or e
        a = double_of(bits_of(a) & ~0x00000000000fffffull);
        d = double_of(bits_of(d) & ~0x00000000000fffffull);
        const double k = double_of((static_cast<uint64_t>(1023 + static_cast<int>(r2 % 40) - 20) << 52) | ((r2 >> 8) & 0xffff00000000ull));
        c = a * k;
        e = d * k;
        const int64_t nudge = static_cast<int64_t>((r3 >> 8) % 3) - 1;
        if ((r3 >> 16) & 1) c = double_of(bits_of(c) + nudge); else e = double_of(bits_of(e) + nudge);
        break;
      }
      case 2: c = a / d * band(r2, 0, 1); e = band(r2, 0, 1); break;  // c / e near a / d
      default: c = double_of(bits_of(a / d) + (static_cast<int64_t>((r2 >> 8) % 5) - 2)); e = 1.0; break;
    }
    const double p1 = a * e, e1 = std::fma(a, e, -p1), p2 = c * d, e2 = std::fma(c, d, -p2);
    const bool want = p1 > p2 || (p1 == p2 && e1 > e2);
    const bool got = rkcu::softfp::quotients_greater(bits_of(a), bits_of(d), bits_of(c), bits_of(e));
    greater += want;
    if (got != want && bad_q2++ < 5) printf("quotients %a / %a > %a / %a: want %d got %d\n", a, d, c, e, want, got);
  }
  printf("quotient comparison mismatches %lld (greater %lld of %lld)\n", bad_q2, greater, count);

  // the error norm's maximum (ErrMax) against the fmax chain of rounded
  // quotients, a zero divisor counting as 1.7E308: sequences of up to 64
  // components of smooth fields (quotients within a few binades, many close
  // to the maximum) mixed with zeros, subnormals, infinities and NaNs
  long long bad_em = 0;
  const long long seqs = count / 16;
  for (long long i = 0; i < seqs; ++i) {
    const uint64_t r = next();
    const int len = 1 + static_cast<int>(r % 64);
    const int special_rate = static_cast<int>((r >> 8) % 4);  // 0: none ... 3: often
    const int spread = static_cast<int>((r >> 16) % 6);      // binades of the quotients
    rkcu::ErrMax em;
    double want = 0.0;
    for (int k = 0; k < len; ++k) {
      const uint64_t q = next(), q2 = next();
      auto pick = [&](uint64_t z, int base) {
        if (special_rate && (z >> 40) % (16 >> special_rate) == 0) {
          switch ((z >> 50) % 6) {
            case 0: return 0.0;
            case 1: return double_of(z & 0x000fffffffffffffull);            // subnormal
            case 2: return double_of(0x7ff0000000000000ull);                // infinity
            case 3: return double_of(0x7ff8000000000000ull | (z & 0xffff)); // NaN
            case 4: return double_of((z & 0x000fffffffffffffull) | 0x0010000000000000ull);  // smallest binade
            default: return double_of((z & 0x000fffffffffffffull) | (2046ull << 52));       // largest binade
          }
        }
        const int ex = base + static_cast<int>((z >> 52) % (spread + 1));
        return double_of((z & 0x800fffffffffffffull) | (static_cast<uint64_t>(1023 + ex) << 52));
      };
      const double e = pick(q, -30), yn = pick(q2, 0), yo = (q2 >> 39) & 1 ? pick(next(), 0) : yn;
      const double div = std::fmax(std::fabs(yn), std::fabs(yo));
      want = std::fmax(want, div == 0.0 ? 1.7E308 : std::fabs(e) / div);
      em.add(e, yn, yo);
    }
    const double got = em.value();
    if (bits_of(got) != bits_of(want) && bad_em++ < 5) printf("error max of %d: want %a got %a\n", len, want, got);
  }
  printf("error max mismatches %lld of %lld sequences\n", bad_em, seqs);
  return (bad_mul || bad_add || bad_cvt || bad_lap || bad_q2 || bad_em) ? 1 : 0;
}
