// tpls_pair.cuh -- FP64 values as FP32 pairs by integer operations.
//
// On GB300 FP64 arithmetic and FP64<->FP32 conversions share a pipe 64x
// slower than FP32.  The FP32 parts of the FP32-mixed form therefore read
// FP64 values as a pair (hi = the value truncated to 24 significant bits,
// lo = the FP32 rounding of the remainder, hi + lo within 2^-47 of the
// value) built with integer instructions only, and form differences of
// nearby values as (hi_a - hi_b) + (lo_a - lo_b), which carries FP32
// precision relative to the difference itself rather than to the values.
#pragma once
#include "tpls_common.cuh"

namespace tpls {

struct F2 {
  float h, l;
};

__device__ __forceinline__ F2 split_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int top = (unsigned int)(b >> 32), sgn = top & 0x80000000u;
  const int e = (int)((top >> 20) & 0x7ffu);  // biased FP64 exponent
  const unsigned int m23 = (unsigned int)(b >> 29) & 0x7fffffu, rem = (unsigned int)b & 0x1fffffffu;
  F2 p;
  if (e >= 897 && e <= 1150) {  // 2^-126 <= |x| < 2^128: hi is an FP32 normal
    p.h = __uint_as_float(sgn | ((unsigned int)(e - 896) << 23) | m23);
    // lo = rem * 2^(e - 1075); that power of two is an FP32 normal for e >= 949
    const float sc = __uint_as_float((unsigned int)max(e - 948, 0) << 23);
    const float lo = (e >= 949) ? __uint2float_rn(rem) * sc : 0.0f;
    p.l = __uint_as_float(__float_as_uint(lo) | sgn);
  } else if (e == 2047) {  // inf / NaN stay inf / NaN
    p.h = __uint_as_float(sgn | 0x7f800000u | ((m23 | rem) ? 0x400000u : 0u));
    p.l = 0.0f;
  } else {  // |x| < 2^-126 (taken as zero) or beyond the FP32 range (inf)
    p.h = __uint_as_float(sgn | (e > 1150 ? 0x7f800000u : 0u));
    p.l = 0.0f;
  }
  return p;
}

// exact FP32 -> FP64 widening by integer operations (FP32 subnormals,
// never produced by these stencils' magnitudes, become signed zero)
__device__ __forceinline__ double widen_bits(float v) {
  const unsigned int b = __float_as_uint(v), e = (b >> 23) & 0xffu;
  const unsigned long long s = (unsigned long long)(b & 0x80000000u) << 32;
  const unsigned long long m = (unsigned long long)(b & 0x7fffffu) << 29;
  unsigned long long r;
  if (e == 0) r = s;
  else if (e == 255) r = s | 0x7ff0000000000000ull | m;
  else r = s | ((unsigned long long)(e + 896) << 52) | m;
  return __longlong_as_double((long long)r);
}

__device__ __forceinline__ float dif(F2 a, F2 b) { return (a.h - b.h) + (a.l - b.l); }

// the pair's value rounded to FP32 (hi alone is truncated, biased toward
// zero by up to an ulp: sums and products take the rounded value)
__device__ __forceinline__ float val(F2 a) { return a.h + a.l; }
__device__ __forceinline__ float round_bits(double x) { return val(split_bits(x)); }

// order of two pairs of the same normalisation (both from split_bits, or
// both from an error-free sum): by hi, then by lo
__device__ __forceinline__ F2 pmin(F2 a, F2 b) { return (b.h < a.h || (b.h == a.h && b.l < a.l)) ? b : a; }
__device__ __forceinline__ F2 pmax(F2 a, F2 b) { return (b.h > a.h || (b.h == a.h && b.l > a.l)) ? b : a; }

// FP64 min and max by integer operations.  The key maps the bit pattern of
// a double to a signed integer with the same order (negative values have
// their magnitude bits flipped), so for non-NaN a, b: a < b iff
// dkey(a) < dkey(b), with -0 just below +0.  That differs from fmin/fmax
// only in which zero a (+0, -0) tie returns; every use here squares the
// result or subtracts it from a value and squares that, where the sign of
// a zero does not survive.  The key and the sign tests work on the two
// 32-bit words of the double (no 64-bit integer shift).
__device__ __forceinline__ long long dkey(double a) {
  const int hi = __double2hiint(a), s = hi >> 31;
  return __double_as_longlong(__hiloint2double(hi ^ (s & 0x7fffffff), __double2loint(a) ^ s));
}
__device__ __forceinline__ double dmin_bits(double a, double b) { return (dkey(b) < dkey(a)) ? b : a; }
__device__ __forceinline__ double dmax_bits(double a, double b) { return (dkey(a) < dkey(b)) ? b : a; }
// max(a, 0) for a not NaN: +0 for a <= 0 (the sign bit decides)
__device__ __forceinline__ double dpos_bits(double a) { return (__double2hiint(a) < 0) ? 0.0 : a; }

}  // namespace tpls
