// fp64_math.cuh -- table-driven FP64 exp and log for the FP64-starved GB300.
//
// GB300 executes FP64 at 1/64 of its FP32 rate; the local rheology update is bound
// by that pipe and spends most of it in exp and log.  These follow P. T. P. Tang's
// table-driven method (ACM TOMS 15(2):144-157, 1989 for exp; 16(4):378-400, 1990
// for log): a reduction by a 256-entry table leaves an argument small enough for a
// short polynomial, and all index, exponent and range work is done with integer
// operations on the bit pattern, off the FP64 pipe.  Cost: 10 FP64 instructions for
// exp and 12 for log.  Accuracy is about 1 ulp (checked against CUDA's exp/log by
// tests/test_gpu_fp64_math.py).  Arguments outside the fast range (|x| >= 700 for
// exp; zero, negative, subnormal, inf or NaN for log) take the CUDA library function,
// so special values behave exactly as exp/log do.
#pragma once
#include <cuda_runtime.h>

#include "fp64_tables.inc"

namespace mdz {

struct MathTables {
  double exp2j[256];  // 2^(j/256)
  double invF[193];   // 256/j, j = 192..384  (F = j/256 in [0.75, 1.5])
  double logF[193];   // log(j/256)
};

// The tables live in global memory and are read through the read-only cache: each
// lane indexes its own entry, which a constant-bank read would serialise.
__device__ const MathTables g_math = {MDZ_EXP2J_TABLE, MDZ_INVF_TABLE, MDZ_LOGF_TABLE};

__device__ __forceinline__ double fast_exp(double x) {
  const int ahi = __double2hiint(x) & 0x7fffffff;
  if (ahi >= 0x4085e000) return exp(x);  // |x| >= 700, inf, NaN
  // x = (256 m + j) ln2/256 + r,  |r| <= ln2/512
  const double t = x * MDZ_INV_LN2_256;
  const double s = t + 6755399441055744.0;  // 1.5 * 2^52: round t to an integer
  const int k = __double2loint(s);
  const double kd = s - 6755399441055744.0;
  double r = fma(-kd, MDZ_LN2_256_HI, x);
  r = fma(-kd, MDZ_LN2_256_LO, r);
  const double T = __ldg(&g_math.exp2j[k & 255]);
  // exp(r) = 1 + r (1 + r/2 + r^2/6 + r^3/24) + O(r^5/120),  |r^5/120| < 4e-17
  double a = fma(r, 4.1666666666666666667e-02, 1.6666666666666666667e-01);
  a = fma(a, r, 0.5);
  a = fma(a, r, 1.0);
  const double res = fma(T * r, a, T);  // in [0.998, 2): scale by 2^m on the exponent field
  return __hiloint2double(__double2hiint(res) + ((k >> 8) << 20), __double2loint(res));
}

__device__ __forceinline__ double fast_log(double x) {
  const int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  if (hi < 0x00100000 || hi >= 0x7ff00000) return log(x);  // <= 0 or subnormal, inf, NaN
  int m = (hi >> 20) - 1023;
  const int frac = hi & 0x000fffff;
  // mantissa mx in [0.75, 1.5) and the nearest table point F = j/256, built from bits
  int mh, j, Fh;
  if (frac >= 0x00080000) {  // [1.5, 2) -> halve into [0.75, 1)
    m += 1;
    mh = 0x3fe00000 | frac;
    j = 128 + ((frac + 0x1000) >> 13);        // in [192, 256]
    Fh = (j == 256) ? 0x3ff00000 : (0x3fe00000 | ((j - 128) << 13));
  } else {                   // [1, 1.5)
    mh = 0x3ff00000 | frac;
    j = 256 + ((frac + 0x800) >> 12);         // in [256, 384]
    Fh = 0x3ff00000 | ((j - 256) << 12);
  }
  const double mx = __hiloint2double(mh, lo);
  const double F = __hiloint2double(Fh, 0);
  const double u = (mx - F) * __ldg(&g_math.invF[j - 192]);  // mx - F is exact (Sterbenz)
  // log1p(u) = u - u^2/2 + u^3/3 - u^4/4 + u^5/5 - u^6/6 + O(u^7/7),  |u| <= 1/383
  double q = fma(u, -1.6666666666666666667e-01, 2.0e-01);
  q = fma(q, u, -0.25);
  q = fma(q, u, 3.3333333333333333333e-01);
  q = fma(q, u, -0.5);
  const double p = fma(q * u, u, u);
  const double md = __hiloint2double(0x43300000, m ^ 0x80000000) - 4503601774854144.0;  // (double)m
  const double res = fma(md, MDZ_LN2_HI, __ldg(&g_math.logF[j - 192]));
  return fma(md, MDZ_LN2_LO, p) + res;
}

}  // namespace mdz
