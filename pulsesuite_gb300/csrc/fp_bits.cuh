// FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 the FP64 pipe (which also executes the F2F conversions between double
// and float) runs at about 1/64 of the FP32 rate, so a per-element (float)x or
// (double)f in an O(Nk^2) kernel costs as much as an FP64 FMA.  These helpers do
// the same IEEE conversions with integer instructions.
#pragma once
#include <cstdint>

namespace sbe {

// round-to-nearest-even of x * 2^e to FP32 (e is added to the exponent, so the
// scaling is exact).  Results below the FP32 normal range (|x 2^e| < 2^-126)
// become signed zero; overflow gives infinity; NaN stays NaN.  The 52-bit
// mantissa is rounded to 23 bits with one 64-bit integer add (ties to even); a
// carry out of the mantissa runs into the exponent field.
__device__ __forceinline__ float f64_to_f32(double x, int e = 0) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const unsigned long long a = u & 0x7FFFFFFFFFFFFFFFull;
  if (a >= 0x7FF0000000000000ull)   // infinity or NaN
    return __uint_as_float(sign | 0x7F800000u | (a != 0x7FF0000000000000ull ? 0x400000u : 0u));
  const unsigned long long r = (a + 0x0FFFFFFFull + ((a >> 29) & 1ull)) >> 29;
  const int fe = (int)(r >> 23) - (1023 - 127) + e;
  if (fe >= 255) return __uint_as_float(sign | 0x7F800000u);
  if (fe <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | ((unsigned)fe << 23) | ((unsigned)r & 0x7FFFFFu));
}

// x * 2^e for FP32 by two exact power-of-two multiplies (|e| <= 252, result in
// the normal range)
__device__ __forceinline__ float f32_ldexp(float x, int e) {
  const int e1 = e / 2, e2 = e - e1;
  return x * __int_as_float((127 + e1) << 23) * __int_as_float((127 + e2) << 23);
}

// exact widening of an FP32 value to FP64
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  unsigned ex = (u >> 23) & 0xFFu;
  unsigned m = u & 0x7FFFFFu;
  if (ex == 0xFFu) {
    return __hiloint2double((int)(sign | 0x7FF00000u | (m ? 0x80000u : 0u)), 0);
  }
  if (ex == 0) {
    if (m == 0) return __hiloint2double((int)sign, 0);
    // FP32 subnormal m 2^-149: normalise the leading bit to bit 23
    const int sh = __clz((int)m) - 8;
    m = (m << sh) & 0x7FFFFFu;
    const unsigned e64 = (unsigned)(1 - 127 + 1023 - sh);
    return __hiloint2double((int)(sign | (e64 << 20) | (m >> 3)), (int)(m << 29));
  }
  return __hiloint2double((int)(sign | ((ex - 127u + 1023u) << 20) | (m >> 3)), (int)(m << 29));
}

// f * 2^e exactly in FP64 (f finite; the result is assumed to stay normal)
__device__ __forceinline__ double f32_to_f64_scaled(float f, int e) {
  const double d = f32_to_f64(f);
  if (f == 0.f) return d;
  return __hiloint2double(__double2hiint(d) + (e << 20), __double2loint(d));
}

__device__ __forceinline__ float2 f64_to_f32(double2 v, int e = 0) {
  return make_float2(f64_to_f32(v.x, e), f64_to_f32(v.y, e));
}

__device__ __forceinline__ double2 f32_to_f64(float2 v) {
  return make_double2(f32_to_f64(v.x), f32_to_f64(v.y));
}

// |x| as an ordered integer (the bit pattern of a non-negative double grows with
// its value), for maxima without floating-point instructions
__device__ __forceinline__ unsigned long long absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// the unsigned pattern of max(|re|, |im|) rounded to FP32, for atomicMax on
// non-negative floats
__device__ __forceinline__ unsigned bits_to_fmax(unsigned long long b) {
  return __float_as_uint(f64_to_f32(__longlong_as_double((long long)b)));
}

}  // namespace sbe
