// fp64_div.cuh -- correctly rounded division by a divisor known in advance.
//
// The grid kernels divide many numerators by the same mesh spacing.  With
// y = RN(1/b) computed once on the host (an IEEE division), a / b is formed from one
// multiply and four fused multiply-adds:
//   q0 = RN(a y)                 within 1.5 ulp of a/b (y is within half an ulp of 1/b);
//   q1 = RN(q0 + RN(a - b q0) y) within half an ulp plus a tiny term: faithful;
//   q2 = RN(q1 + (a - b q1) y)   the remainder is exact for a faithful q1, and the
//                                result is RN(a/b) by Markstein's theorem (P. Markstein,
//                                IBM J. Res. Develop. 34(1):111-119, 1990; also
//                                Muller et al., Handbook of Floating-Point Arithmetic,
//                                section on Newton-Raphson based division).
// The theorem holds without underflow or overflow; the fast form is used for
// 2^-500 <= |a| <= 2^500 and a divisor in [2^-400, 2^400] (so every intermediate is a
// normal number), and the plain division otherwise (zero, subnormal, huge, Inf, NaN).
// Checked bit for bit against CUDA's division by mdz_rheo_div_selftest.
#pragma once
#include <cuda_runtime.h>

#include "fp64_bits.cuh"

namespace mdz {

// a divisor b, its rounded reciprocal and whether the fast form may be used with it
struct Divisor {
  double b, y;
  int fast;
};

// host side: the divisor as the kernels use it
inline Divisor make_divisor(double b) {
  Divisor d;
  d.b = b;
  d.y = 1.0 / b;
  const double m = b < 0 ? -b : b;
  d.fast = (m >= 0x1p-400 && m <= 0x1p400) ? 1 : 0;
  return d;
}

__device__ __forceinline__ double div_by(double a, const Divisor &d) {
  if (d.fast && fp64_exponent(a) - (1023u - 500u) <= 1000u) {
    double q = __dmul_rn(a, d.y);
    q = __fma_rn(__fma_rn(-q, d.b, a), d.y, q);
    return __fma_rn(__fma_rn(-q, d.b, a), d.y, q);
  }
  return a / d.b;
}

// r / den for a Newton update, where a correctly rounded quotient is not needed (the
// iteration corrects a step's error on the next evaluation): the hardware reciprocal
// estimate (PTX rcp.approx.ftz.f64) refined by one Newton step, y (2 - den y), then
// r y -- three FP64 instructions in place of the general division.  den outside
// [2^-1000, 2^1000] (zero, subnormal, huge, Inf, NaN) takes the IEEE division.
__device__ __forceinline__ double newton_quotient(double r, double den) {
  if (fp64_exponent(den) - 23u > 2000u) return r / den;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(den));
  y = __fma_rn(y, __fma_rn(-den, y, 1.0), y);
  return __dmul_rn(r, y);
}

}  // namespace mdz
