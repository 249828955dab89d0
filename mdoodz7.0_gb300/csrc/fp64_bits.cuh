// fp64_bits.cuh -- tests on the bits of a double that stay on the integer pipe.
//
// GB300 runs FP64 instructions, compares included, at 1/64 of the FP32 rate, and the
// grid kernels of this library are bound by that pipe.  A test such as "x is finite" or
// "x is zero" written on the bit pattern is cheap integer work, but a compiler that sees
// the bitcast may turn it back into an FP64 compare (DSETP).  The two 32-bit words are
// therefore taken through an opaque register move, after which the tests are plain
// integer operations.
#pragma once
#include <cuda_runtime.h>

namespace mdz {

__device__ __forceinline__ void fp64_words(double x, unsigned &lo, unsigned &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}

__device__ __forceinline__ unsigned fp64_hi(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  return hi;
}

// biased exponent field, 0..2047
__device__ __forceinline__ unsigned fp64_exponent(double x) { return (fp64_hi(x) >> 20) & 0x7ffu; }

// not Inf or NaN
__device__ __forceinline__ bool fp64_finite(double x) { return fp64_exponent(x) != 0x7ffu; }

// +0 or -0
__device__ __forceinline__ bool fp64_is_zero(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  return ((hi << 1) | lo) == 0u;
}

// +Inf or -Inf
__device__ __forceinline__ bool fp64_is_inf(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  return (hi & 0x7fffffffu) == 0x7ff00000u && lo == 0u;
}

// NaN
__device__ __forceinline__ bool fp64_is_nan(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  return (hi & 0x7fffffffu) > 0x7ff00000u || ((hi & 0x7fffffffu) == 0x7ff00000u && lo != 0u);
}

// -0 exactly
__device__ __forceinline__ bool fp64_is_negative_zero(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  return hi == 0x80000000u && lo == 0u;
}

// for x, y not NaN: x < y exactly when fp64_order_key(x) < fp64_order_key(y) (unsigned);
// -0 and +0 share a key, as they compare equal
__device__ __forceinline__ unsigned long long fp64_order_key(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  unsigned long long b = ((unsigned long long)hi << 32) | lo;
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// The 64-bit pattern of x (through the same opaque unpack).
__device__ __forceinline__ unsigned long long fp64_bits(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  return ((unsigned long long)hi << 32) | lo;
}

constexpr unsigned long long kFp64AbsMask = 0x7fffffffffffffffull, kFp64InfBits = 0x7ff0000000000000ull;

__device__ __forceinline__ unsigned long long fp64_key_of_bits(unsigned long long b) {
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// IEEE comparisons of two doubles on the integer pipe, with the IEEE results for every
// input: false when either side is NaN, -0 equal to +0.
__device__ __forceinline__ bool fp64_lt(double a, double b) {
  const unsigned long long ba = fp64_bits(a), bb = fp64_bits(b);
  if ((ba & kFp64AbsMask) > kFp64InfBits || (bb & kFp64AbsMask) > kFp64InfBits) return false;
  return fp64_key_of_bits(ba) < fp64_key_of_bits(bb);
}
__device__ __forceinline__ bool fp64_le(double a, double b) {
  const unsigned long long ba = fp64_bits(a), bb = fp64_bits(b);
  if ((ba & kFp64AbsMask) > kFp64InfBits || (bb & kFp64AbsMask) > kFp64InfBits) return false;
  return fp64_key_of_bits(ba) <= fp64_key_of_bits(bb);
}
__device__ __forceinline__ bool fp64_gt(double a, double b) { return fp64_lt(b, a); }
__device__ __forceinline__ bool fp64_ge(double a, double b) { return fp64_le(b, a); }

// |x| < t, IEEE, for any x and t
__device__ __forceinline__ bool fp64_abs_lt(double x, double t) {
  const unsigned long long ax = fp64_bits(x) & kFp64AbsMask, bt = fp64_bits(t);
  if (ax > kFp64InfBits || (bt & kFp64AbsMask) > kFp64InfBits) return false;
  return fp64_key_of_bits(ax) < fp64_key_of_bits(bt);
}
// |x| > t, IEEE, for any x and t
__device__ __forceinline__ bool fp64_abs_gt(double x, double t) {
  const unsigned long long ax = fp64_bits(x) & kFp64AbsMask, bt = fp64_bits(t);
  if (ax > kFp64InfBits || (bt & kFp64AbsMask) > kFp64InfBits) return false;
  return fp64_key_of_bits(ax) > fp64_key_of_bits(bt);
}

// x == y as IEEE numbers, for a y that is neither NaN nor zero (bit equality then)
__device__ __forceinline__ bool fp64_eq_nonzero(double x, double y) { return fp64_bits(x) == fp64_bits(y); }

// fmax(a, b) on the integer pipe: a NaN operand yields the other one, +0 wins a tie with
// -0, otherwise the larger by order key
__device__ __forceinline__ double fp64_fmax(double a, double b) {
  const unsigned long long ba = fp64_bits(a), bb = fp64_bits(b);
  if ((ba & kFp64AbsMask) > kFp64InfBits) return b;
  if ((bb & kFp64AbsMask) > kFp64InfBits) return a;
  const unsigned long long ka = fp64_key_of_bits(ba), kb = fp64_key_of_bits(bb);
  return (ka > kb || (ka == kb && (ba >> 63) == 0ull)) ? a : b;
}

constexpr int kFp64CeilSat = 1 << 30;

// ceil(q) as an int, from the fields of q: |q| = m 2^(e-52) with m the 53-bit
// significand, so for 0 <= e < 30 the integer part is m >> (52 - e) and any bit below
// it is a fraction.  |q| >= 2^30 and Inf saturate to +-2^30 and NaN to +2^30 -- the
// same decisions as the FP64 ceil and int conversion for every cell index of a grid,
// without an FP64 instruction.
__device__ __forceinline__ int fp64_ceil_int(double q) {
  unsigned lo, hi;
  fp64_words(q, lo, hi);
  const bool neg = (hi >> 31) != 0u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
  if (e >= 30) {
    const bool nan = (hi & 0x7fffffffu) > 0x7ff00000u || ((hi & 0x7fffffffu) == 0x7ff00000u && lo != 0u);
    return (neg && !nan) ? -kFp64CeilSat : kFp64CeilSat;
  }
  if (e < 0) return (!neg && ((hi << 1) | lo) != 0u) ? 1 : 0;  // (0, 1) -> 1; (-1, 0] and -0 -> 0
  const unsigned long long m = ((unsigned long long)(hi & 0xfffffu) << 32 | lo) | (1ull << 52);
  const int sh = 52 - e;
  const int ip = (int)(m >> sh);
  const bool frac = (m & ((1ull << sh) - 1ull)) != 0ull;
  return neg ? -ip : ip + (frac ? 1 : 0);
}

}  // namespace mdz
