// Device check of the double-float helpers (rkcu_dfloat.cuh): the device
// gives the same bits as the host for bruss_rhs_df, df_of and dbl_of on the
// same random stencils (smooth, rough, boundary and wide-range kinds) and float
// bit patterns, and dbl_of matches the conversion instruction.
// Usage: dfloat_check_gpu <count> <seed>; prints mismatches, exits non-zero on any.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rkcu_dfloat.cuh"

using namespace rkcu::dfl;
using rkcu::softfp::bits_of;

struct Out {
  float fu_hi, fu_lo, fv_hi, fv_lo;
  float sx_hi, sx_lo;  // df_of(c.x)
  double cvt;          // dbl_of of a float bit pattern
  int ok, ok_split;
};

__global__ void eval(int count, const double2 *in, const float *fl, double coef, Out *out, unsigned long long *bad_cvt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const double2 *s = in + 5 * i;
  df cf;
  df_of(coef, &cf);
  df fu = {0, 0}, fv = {0, 0}, sx = {0, 0};
  Out o;
  o.ok = bruss_rhs_df(s[0], s[1], s[2], s[3], s[4], cf, &fu, &fv);
  o.ok_split = df_of(s[0].x, &sx);
  o.fu_hi = fu.hi;
  o.fu_lo = fu.lo;
  o.fv_hi = fv.hi;
  o.fv_lo = fv.lo;
  o.sx_hi = sx.hi;
  o.sx_lo = sx.lo;
  o.cvt = dbl_of(fl[i]);
  const double hw = static_cast<double>(fl[i]);
  if (hw == hw && __double_as_longlong(hw) != __double_as_longlong(o.cvt)) atomicAdd(bad_cvt, 1ull);
  out[i] = o;
}

static uint64_t s_state;
static uint64_t next() {  // splitmix64
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unif() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }

int main(int argc, char **argv) {
  const int count = argc > 1 ? atoi(argv[1]) : (1 << 20);
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  const double coef = 0.002 * 3999.0 * 3999.0;
  std::vector<double2> in(5 * static_cast<size_t>(count));
  std::vector<float> fl(count);
  for (int i = 0; i < count; ++i) {
    const int kind = i % 4;
    const double scale = kind == 3 ? std::ldexp(1.0, static_cast<int>(next() % 60) - 30) : 1.0;
    double2 c = make_double2(scale * (0.05 + 6.0 * unif()), scale * (0.05 + 6.0 * unif()));
    const double pert = std::ldexp(1.0, -static_cast<int>(next() % 40));
    in[5 * i] = c;
    for (int k = 1; k <= 4; ++k)
      in[5 * i + k] = kind == 1 ? make_double2(scale * (0.05 + 6.0 * unif()), scale * (0.05 + 6.0 * unif()))
                                : make_double2(c.x * (1.0 + pert * (2.0 * unif() - 1.0)),
                                               c.y * (1.0 + pert * (2.0 * unif() - 1.0)));
    if (kind == 2) in[5 * i + 4] = in[5 * i + 3];
    fl[i] = rkcu::softfp::float_of(static_cast<uint32_t>(next()));
  }
  double2 *d_in = nullptr;
  float *d_fl = nullptr;
  Out *d_out = nullptr;
  unsigned long long *d_bad = nullptr, bad_cvt_hw = 0;
  if (cudaMalloc(&d_in, in.size() * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&d_fl, fl.size() * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&d_out, count * sizeof(Out)) != cudaSuccess || cudaMalloc(&d_bad, 8) != cudaSuccess)
    return 2;
  cudaMemcpy(d_in, in.data(), in.size() * sizeof(double2), cudaMemcpyHostToDevice);
  cudaMemcpy(d_fl, fl.data(), fl.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(d_bad, 0, 8);
  eval<<<(count + 255) / 256, 256>>>(count, d_in, d_fl, coef, d_out, d_bad);
  std::vector<Out> out(count);
  if (cudaMemcpy(out.data(), d_out, count * sizeof(Out), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  cudaMemcpy(&bad_cvt_hw, d_bad, 8, cudaMemcpyDeviceToHost);

  long long bad = 0, refused = 0;
  df cf;
  df_of(coef, &cf);
  for (int i = 0; i < count; ++i) {
    const double2 *s = &in[5 * static_cast<size_t>(i)];
    df fu = {0, 0}, fv = {0, 0}, sx = {0, 0};
    const int ok = bruss_rhs_df(s[0], s[1], s[2], s[3], s[4], cf, &fu, &fv);
    const int ok_split = df_of(s[0].x, &sx);
    const double cvt = dbl_of(fl[i]);
    const Out &o = out[i];
    refused += !ok;
    const bool same = ok == o.ok && ok_split == o.ok_split && fu.hi == o.fu_hi && fu.lo == o.fu_lo &&
                      fv.hi == o.fv_hi && fv.lo == o.fv_lo && sx.hi == o.sx_hi && sx.lo == o.sx_lo &&
                      (cvt != cvt ? o.cvt != o.cvt : bits_of(cvt) == bits_of(o.cvt));
    if (!same && bad++ < 5)
      printf("mismatch %d: host %a %a device %a %a\n", i, fu.hi, fu.lo, o.fu_hi, o.fu_lo);
  }
  printf("host/device mismatches %lld, dbl_of vs conversion %llu, refused %lld of %d\n", bad, bad_cvt_hw, refused,
         count);
  cudaFree(d_in);
  cudaFree(d_fl);
  cudaFree(d_out);
  cudaFree(d_bad);
  return (bad || bad_cvt_hw) ? 1 : 0;
}
