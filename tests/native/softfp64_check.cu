// Device check of the software binary64 multiply/add, double -> float
// rounding, the same-binade Laplacian and the exact quotient comparison
// (rkcu_softfp64.cuh) against the FP64 pipe's __dmul_rn/__dadd_rn/__fma_rn/
// __double2float_rn on random and adversarial operands.  Usage: softfp64_check_gpu <count> <seed>; prints mismatches.
#include <cstdio>
#include <cstdlib>

#include "rkcu_softfp64.cuh"

using namespace rkcu::softfp;

__device__ __forceinline__ uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ double draw(uint64_t r, int kind, double other) {
  switch (kind) {
    case 0: return double_of(r);
    case 1: return double_of((r & 0x800fffffffffffffull) | ((uint64_t)(1023 + (int)(r >> 53) % 8 - 4) << 52));
    case 2: return double_of((r & 0x800fffffffffffffull) | ((uint64_t)(1 + (r >> 52) % 2046) << 52));
    case 3: return double_of(bits_of(other) + ((int64_t)(r % 64) - 32));
    case 4: return -double_of(bits_of(other) + (r % 5));
    case 5: return double_of((r & 0x800fffffffffffffull) | ((uint64_t)(((r >> 52) % 2) ? 1 : 2045) << 52));
    default: return double_of((r & 0xfff0000000000000ull) | (r & 0x7));
  }
}

__global__ void check(long long count, unsigned long long seed, unsigned long long *bad) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long bm = 0, ba = 0, bf = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t r0 = mix(seed + 4 * i), r1 = mix(seed + 4 * i + 1), r2 = mix(seed + 4 * i + 2),
                   r3 = mix(seed + 4 * i + 3);
    int ka = (int)(r0 % 7);
    if (ka == 3 || ka == 4) ka = 1;
    const double a = draw(r1, ka, 0.0);
    const double b = draw(r3, (int)(r2 % 7), a);
    const double pm = __dmul_rn(a, b), sm = mul(a, b);
    const double pa = __dadd_rn(a, b), sa = add(a, b);
    if (!(pm != pm && sm != sm) && bits_of(pm) != bits_of(sm)) ++bm;
    if (!(pa != pa && sa != sa) && bits_of(pa) != bits_of(sa)) ++ba;
    // conversions: the operands, the sum, and doubles near the float range edges
    // and halfway cases (the 29 dropped bits exactly 0x10000000)
    const double near_edge = double_of((r2 & 0x800fffffffffffffull) |
                                       ((uint64_t)((r0 >> 40) % 2 ? 1023 - 126 - (int)(r1 % 3) : 1023 + 127 - (int)(r1 % 2)) << 52));
    const double tie = double_of((bits_of(a) & ~0x1fffffffull) | 0x10000000ull);
    const double cv[4] = {a, pa, near_edge, tie};
    for (int q = 0; q < 4; ++q) {
      const float hf = __double2float_rn(cv[q]), sf = to_float(cv[q]);
      if (!(hf != hf && sf != sf) && __float_as_uint(hf) != __float_as_uint(sf)) ++bf;
    }
  }
  if (bm) atomicAdd(&bad[0], bm);
  if (ba) atomicAdd(&bad[1], ba);
  if (bf) atomicAdd(&bad[2], bf);
}

// the same-binade Laplacian against the FP64 sequence it replaces, on the
// device: one exponent field per operand set (random significands, tops of the
// binade, few-bit significands for ties), both signs, all three stencil forms
__global__ void check_lap(long long count, unsigned long long seed, unsigned long long *bad) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long bl = 0, taken = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t r = mix(seed + 8 * i);
    const uint64_t ef = 1 + (r >> 11) % 2043;
    const uint64_t sg = (r >> 63) << 63;
    double v[5];
    for (int k = 0; k < 5; ++k) {
      const uint64_t q = mix(seed + 8 * i + 1 + k);
      uint64_t f;
      switch ((r >> (2 * k)) & 3) {
        case 0: f = q & 0x000fffffffffffffull; break;
        case 1: f = 0x000fffffffffffffull - (q & 0xff); break;
        case 2: f = (q & 0xf) << ((q >> 8) % 49); break;
        default: f = (q & 0x000fffffffffffffull) | 0x000ffffff0000000ull; break;
      }
      v[k] = double_of(sg | (ef << 52) | f);
    }
    const int jcase = (int)((r >> 30) % 3);
    const double n = v[0], s = v[1], w = jcase == 1 ? v[3] : v[2], e = jcase == 2 ? v[2] : v[3], c = v[4];
    double want = __dadd_rn(n, s);
    want = jcase == 0 ? __dadd_rn(__dadd_rn(want, w), e) : __fma_rn(2.0, jcase == 1 ? e : w, want);
    want = __fma_rn(-4.0, c, want);
    double got = 0.0;
    if (lap_same_binade(n, s, w, e, c, jcase, &got)) {
      ++taken;
      if (bits_of(got) != bits_of(want)) ++bl;
    } else if ((bits_of(want) & 0x7ff0000000000000ull) != 0) {
      ++bl;  // a normal result must take the integer path
    }
  }
  if (bl) atomicAdd(&bad[3], bl);
  atomicAdd(&bad[4], taken);
}

// the exact comparison of two quotients a / d > c / e against the products a e
// and c d and their FMA error terms, on the device: random operands, equal
// quotients (c, e the same multiple of a, d) moved by up to one unit, and
// quotients one rounding apart
__device__ double band(uint64_t q) {
  return double_of((q & 0x000fffffffffffffull) | ((uint64_t)(1023 - 250 + (int)((q >> 52) % 500)) << 52));
}

__global__ void check_quot(long long count, unsigned long long seed, unsigned long long *bad) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long bq = 0, greater = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t r0 = mix(seed + 4 * i + 11), r1 = mix(seed + 4 * i + 12), r2 = mix(seed + 4 * i + 13),
                   r3 = mix(seed + 4 * i + 14);
    double a = band(r0), d = band(r1), c, e;
    switch (r3 % 4) {
      case 0:
        c = band(r2);
        e = band(r3);
        break;
      case 1: {
        a = double_of(bits_of(a) & ~0x00000000000fffffull);
        d = double_of(bits_of(d) & ~0x00000000000fffffull);
        const double k = double_of(((uint64_t)(1023 + (int)(r2 % 40) - 20) << 52) | ((r2 >> 8) & 0xffff00000000ull));
        c = __dmul_rn(a, k);
        e = __dmul_rn(d, k);
        const int64_t nudge = (int64_t)((r3 >> 8) % 3) - 1;
        if ((r3 >> 16) & 1)
          c = double_of(bits_of(c) + nudge);
        else
          e = double_of(bits_of(e) + nudge);
        break;
      }
      default:
        c = double_of(bits_of(__ddiv_rn(a, d)) + ((int64_t)((r2 >> 8) % 5) - 2));
        e = 1.0;
        break;
    }
    const double p1 = __dmul_rn(a, e), e1 = __fma_rn(a, e, -p1), p2 = __dmul_rn(c, d), e2 = __fma_rn(c, d, -p2);
    const bool want = p1 > p2 || (p1 == p2 && e1 > e2);
    greater += want;
    if (quotients_greater(bits_of(a), bits_of(d), bits_of(c), bits_of(e)) != want) ++bq;
  }
  if (bq) atomicAdd(&bad[5], bq);
  atomicAdd(&bad[6], greater);
}

int main(int argc, char **argv) {
  const long long count = argc > 1 ? atoll(argv[1]) : (1ll << 28);
  const unsigned long long seed = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  unsigned long long *bad = nullptr, h[7] = {0, 0, 0, 0, 0, 0, 0};
  if (cudaMalloc(&bad, sizeof(h)) != cudaSuccess) return 2;
  cudaMemset(bad, 0, sizeof(h));
  check<<<152 * 8, 256>>>(count, seed, bad);
  check_lap<<<152 * 8, 256>>>(count / 4, seed, bad);
  check_quot<<<152 * 8, 256>>>(count / 4, seed, bad);
  if (cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  printf("mismatches mul %llu add %llu to_float %llu of %lld; lap %llu of %lld (integer path %llu); "
         "quotient comparison %llu of %lld (greater %llu)\n",
         h[0], h[1], h[2], count, h[3], count / 4, h[4], h[5], count / 4, h[6]);
  cudaFree(bad);
  return (h[0] || h[1] || h[2] || h[3] || h[5]) ? 1 : 0;
}
