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
// The second correction is mostly a no-op: q1 already is RN(a/b) whenever the remainder
// r1 = a - b q1 (exact, q1 being faithful) is below half an ulp of q1 times |b|, that is
// |r1| < |b| 2^(e(q1) - 53), the bound of the rounding interval around a q1 that is not a
// power of two.  That test runs on the integer pipe (b's significand with the exponent
// e(b) + e(q1) - 53, compared with |r1| as bit patterns), so the common case costs one
// multiply and three fused multiply-adds; ties, powers of two, and thresholds outside
// the normal range take the full second correction.
// Checked bit for bit against CUDA's division by mdz_rheo_div_selftest.
#pragma once
#include <cuda_runtime.h>
#include <string.h>

#include "fp64_bits.cuh"

namespace mdz {

// a divisor b, its rounded reciprocal, whether the fast form may be used with it, and
// the biased exponent and significand field of |b| (for the remainder test)
struct Divisor {
  double b, y;
  int fast, eb;
  unsigned long long bman;
};

// host side: the divisor as the kernels use it
inline Divisor make_divisor(double b) {
  Divisor d;
  d.b = b;
  d.y = 1.0 / b;
  const double m = b < 0 ? -b : b;
  d.fast = (m >= 0x1p-400 && m <= 0x1p400) ? 1 : 0;
  unsigned long long bits;
  memcpy(&bits, &m, sizeof(bits));
  d.eb = (int)((bits >> 52) & 0x7ffu);
  d.bman = bits & 0xfffffffffffffull;
  return d;
}

// the second correction, out of line: taken where the remainder test cannot decide
static __device__ __noinline__ double div_by_correct(double r1, double y, double q1) { return __fma_rn(r1, y, q1); }

__device__ __forceinline__ double div_by(double a, const Divisor &d) {
  if (d.fast && fp64_exponent(a) - (1023u - 500u) <= 1000u) {
    const double q0 = __dmul_rn(a, d.y);
    const double q1 = __fma_rn(__fma_rn(-q0, d.b, a), d.y, q0);
    const double r1 = __fma_rn(-q1, d.b, a);
    unsigned lo, hi;
    fp64_words(q1, lo, hi);
    const int te = d.eb + (int)((hi >> 20) & 0x7ffu) - 1023 - 53;  // exponent of |b| ulp(q1) / 2
    const bool pow2 = ((hi & 0xfffffu) | lo) == 0u;
    if (!pow2 && te > 0 && te < 0x7ff &&
        (fp64_bits(r1) & kFp64AbsMask) < (((unsigned long long)te << 52) | d.bman))
      return q1;
    return div_by_correct(r1, d.y, q1);
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

// r / den within a couple of ulp, for a result that is an output but need not be
// correctly rounded (the parity bar is 1e-12 relative): the same reciprocal estimate
// refined by two Newton steps, y <- y + y (1 - den y), each of which squares the relative
// error of y until the rounding of the last step dominates, then r y -- five FP64
// instructions in place of the general division.  den outside [2^-1000, 2^1000] takes the
// IEEE division.  Checked against IEEE division by mdz_rheo_quotient_selftest.
__device__ __forceinline__ double quotient(double r, double den) {
  if (fp64_exponent(den) - 23u > 2000u) return r / den;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(den));
  y = __fma_rn(y, __fma_rn(-den, y, 1.0), y);
  y = __fma_rn(y, __fma_rn(-den, y, 1.0), y);
  return __dmul_rn(r, y);
}

}  // namespace mdz
