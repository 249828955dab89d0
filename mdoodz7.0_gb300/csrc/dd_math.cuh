// dd_math.cuh -- double-float arithmetic (a value carried as an unevaluated sum hi + lo
// of two FP32 numbers, about 48 significant bits) for the start of the local solve.
//
// GB300 runs FP32 at 64 times its FP64 rate, and the local rheology update leaves the
// FP32, integer and conversion pipes nearly idle while its FP64 pipe is saturated.  A
// double-float value carries enough bits (relative error about 2^-46 after a few
// operations) to put the local Newton's start within a few 1e-15 of its root, so the
// FP64 iteration that follows meets its stopping test at its first evaluation.
//
// The error-free transformations are the classical ones: Knuth's two-sum, Dekker's
// fast two-sum, and the two-product through a fused multiply-add (J.-M. Muller et al.,
// Handbook of Floating-Point Arithmetic, 2nd ed., 2018, ch. 4 and 14; T. J. Dekker,
// Numer. Math. 18:224-242, 1971).  Every such step is written with round-to-nearest
// intrinsics, which the compiler neither contracts nor reorders.  exp and log follow the
// same table-driven reductions as fp64_math.cuh (Tang's methods, with 256-entry tables of
// 2^(j/256) and log(j/256) stored as FP32 pairs), with short polynomials in
// double-float.
// Conversions between double and double-float run on the integer pipe (bit fields), so
// that they cost no FP64 instruction.
#pragma once
#include <cuda_runtime.h>

#include "fp64_bits.cuh"
#include "fp64_tables.inc"

namespace mdz {

struct f2 {
  float hi, lo;
};

struct DdTables {
  float2 exp2j[256];  // 2^(j/256) as (hi, lo)
  float2 logF[193];   // log(j/256), j = 192..384, as (hi, lo)
  float invF[193];    // 256/j rounded to FP32
};

// Global memory through the read-only cache: each lane indexes its own entry.
__device__ const DdTables g_dd = {MDZ_EXP2J_DD_TABLE, MDZ_LOGF_DD_TABLE, MDZ_INVF_F32_TABLE};

__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ f2 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ f2 dd_add(f2 x, f2 y) {
  f2 s = two_sum(x.hi, y.hi);
  const f2 t = two_sum(x.lo, y.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ f2 dd_neg(f2 x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ f2 dd_add_f(f2 x, float y) {
  f2 s = two_sum(x.hi, y);
  s.lo = __fadd_rn(s.lo, x.lo);
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ f2 dd_mul(f2 x, f2 y) {
  f2 p = two_prod(x.hi, y.hi);
  p.lo = __fmaf_rn(x.hi, y.lo, p.lo);
  p.lo = __fmaf_rn(x.lo, y.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ f2 dd_mul_f(f2 x, float y) {
  f2 p = two_prod(x.hi, y);
  p.lo = __fmaf_rn(x.lo, y, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// ---------------------------------------------------------------------------------------
// conversions (integer pipe)
// ---------------------------------------------------------------------------------------

// x truncated to its leading 24 significant bits as an FP32 number, from the bit fields;
// values beyond the FP32 range become +-FLT_MAX (NaN too), values below it 0.
__device__ __forceinline__ float f32_trunc(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f7fffffu);
  return __uint_as_float(sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// x as a double, exactly, from the bits of a normal x; zero, subnormal, Inf and NaN take
// the conversion instruction, out of line so that the common case does not execute it too
static __device__ __noinline__ double f64_of_f32_rare(float x) { return (double)x; }

__device__ __forceinline__ double f64_of_f32(float x) {
  const unsigned b = __float_as_uint(x), e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return f64_of_f32_rare(x);
  return __hiloint2double((int)((b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3)), (int)(b << 29));
}

// x as a double-float: hi = the leading 24 significant bits (truncated), lo = the next 24
// bits of the remaining 29 (rounded by the integer-to-float conversion).  Relative error
// below 2^-47.  |x| below 2^-74 keeps only hi; beyond the FP32 range hi is +-FLT_MAX.
__device__ __forceinline__ f2 dd_of_f64(double x) {
  unsigned lo, hi;
  fp64_words(x, lo, hi);
  const unsigned sign = hi & 0x80000000u;
  const int E = (int)((hi >> 20) & 0x7ffu);
  const int e = E - 1023 + 127;
  if (e <= 0) return {__uint_as_float(sign), 0.0f};
  if (e >= 255) return {__uint_as_float(sign | 0x7f7fffffu), 0.0f};
  const float h = __uint_as_float(sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
  const unsigned rem = lo & 0x1fffffffu;  // value rem * 2^(E - 1075)
  if (rem == 0u || E < 949) return {h, 0.0f};
  const unsigned rb = __float_as_uint(__uint2float_rn(rem));  // exponent field 127 .. 155
  const int le = (int)(rb >> 23) + E - 1075;                   // >= 1 for E >= 949
  return {h, __uint_as_float(sign | ((unsigned)le << 23) | (rb & 0x7fffffu))};
}

// hi + lo as a double: two exact conversions and one FP64 addition
__device__ __forceinline__ double f64_of_dd(f2 x) { return f64_of_f32(x.hi) + f64_of_f32(x.lo); }

// ---------------------------------------------------------------------------------------
// exp and log
// ---------------------------------------------------------------------------------------

// exp(x) for a double-float x; results below about 1e-35 are returned as 0, and x is
// taken as at most 80.  Relative error about 2^-46.
__device__ __forceinline__ f2 dd_exp(f2 x) {
  if (!(x.hi > -80.0f)) return {0.0f, 0.0f};  // also NaN
  const float xh = fminf(x.hi, 80.0f);
  // x = (256 m + j) ln2/256 + r,  |r| <= ln2/512
  const float t = __fmaf_rn(xh, MDZ_INV_LN2_256_F, 12582912.0f);  // 1.5 * 2^23: round to an integer
  const int k = __float_as_int(t) - 0x4b400000;
  const float kf = __fsub_rn(t, 12582912.0f);
  const float r1 = __fmaf_rn(-kf, MDZ_LN2_256_F1, xh);  // exact: kf * F1 has at most 23 bits
  // r = r1 - kf F2 - kf F3 + x.lo; the low word of x is added exactly (it may be as large
  // as half an ulp of x.hi, far above the rounding error that r can carry)
  const f2 p = two_prod(kf, MDZ_LN2_256_F2);
  f2 r = two_sum(r1, -p.hi);
  const f2 u = two_sum(r.hi, x.hi == xh ? x.lo : 0.0f);
  r.lo = __fadd_rn(u.lo, __fadd_rn(r.lo, __fsub_rn(-p.lo, kf * MDZ_LN2_256_F3)));
  r = fast_two_sum(u.hi, r.lo);
  // exp(r) = 1 + r + r^2/2 + r^3/6 + r^4/24 + O(r^5/120), |r^5/120| < 4e-17
  const float rh = r.hi;
  const f2 q = two_prod(rh, rh);
  const float poly = __fmul_rn(__fmul_rn(q.hi, rh), __fmaf_rn(rh, 4.16666679e-2f, 1.66666672e-1f));
  f2 m = two_sum(rh, 0.5f * q.hi);
  m.lo = __fadd_rn(m.lo, __fadd_rn(__fadd_rn(r.lo, 0.5f * q.lo), __fmaf_rn(rh, r.lo, poly)));
  f2 e = fast_two_sum(1.0f, m.hi);
  e.lo = __fadd_rn(e.lo, m.lo);
  e = fast_two_sum(e.hi, e.lo);
  const float2 T = __ldg(&g_dd.exp2j[k & 255]);
  e = dd_mul(e, f2{T.x, T.y});  // in [0.998, 2)
  const int mexp = k >> 8;       // in [-116, 116]
  const float sc = __int_as_float((mexp + 127) << 23);
  return {__fmul_rn(e.hi, sc), __fmul_rn(e.lo, sc)};
}

// log(s) for a positive normal FP32 s, as a double-float; absolute error about 2^-47
// (|log s| + 1).
__device__ __forceinline__ f2 dd_log_f(float s) {
  const unsigned b = __float_as_uint(s);
  int m = (int)(b >> 23) - 127;
  const unsigned frac = b & 0x7fffffu;
  // mantissa mx in [0.75, 1.5) and the nearest table point F = j/256
  float mx;
  int j;
  if (frac >= 0x400000u) {  // [1.5, 2) -> halve into [0.75, 1)
    m += 1;
    mx = __uint_as_float(0x3f000000u | frac);
    j = 128 + (int)((frac + 0x8000u) >> 16);  // in [192, 256]
  } else {                  // [1, 1.5)
    mx = __uint_as_float(0x3f800000u | frac);
    j = 256 + (int)((frac + 0x4000u) >> 15);  // in [256, 384]
  }
  const float F = __fmul_rn(__int2float_rn(j), 0.00390625f);
  const float d = __fsub_rn(mx, F);  // exact (Sterbenz)
  const float iF = __ldg(&g_dd.invF[j - 192]);
  const float uh = __fmul_rn(d, iF);
  const float ul = __fmul_rn(__fmaf_rn(-uh, F, d), iF);  // the remainder d - uh F is exact
  // log1p(u) = u - u^2/2 + u^3/3 - u^4/4 + u^5/5 + O(u^6/6),  |u| <= 1/383
  const f2 q = two_prod(uh, uh);
  const float poly = __fmul_rn(__fmul_rn(q.hi, uh),
                               __fmaf_rn(uh, __fmaf_rn(uh, 0.2f, -0.25f), 3.33333343e-1f));
  f2 l = two_sum(uh, -0.5f * q.hi);
  l.lo = __fadd_rn(l.lo, __fadd_rn(__fsub_rn(ul, 0.5f * q.lo), __fmaf_rn(-uh, ul, poly)));
  l = fast_two_sum(l.hi, l.lo);
  const float2 LF = __ldg(&g_dd.logF[j - 192]);
  l = dd_add(l, f2{LF.x, LF.y});
  if (m != 0) {
    const float mf = __int2float_rn(m);
    f2 ml = two_prod(mf, MDZ_LN2_F2);
    ml.lo = __fmaf_rn(mf, MDZ_LN2_F3, ml.lo);
    ml = dd_add_f(ml, __fmul_rn(mf, MDZ_LN2_F1));  // exact product: 16 x 8 bits
    l = dd_add(l, ml);
  }
  return l;
}

}  // namespace mdz
