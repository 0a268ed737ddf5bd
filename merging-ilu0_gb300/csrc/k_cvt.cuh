// FP64 <-> FP32 conversions by integer operations, bit for bit equal to the
// hardware's round-to-nearest-even conversions (cvt.rn.f32.f64 and
// cvt.f64.f32).
//
// Why: on GB300 a hardware conversion between double and float issues at about
// the FP64 FMA rate (measured: ~1.9 conversions per clock per SM against 1.6
// DFMA), so the four conversions per row and iteration of the FP32-ISAI solver
// take FP64-unit slots from A*x and the inner products.  The integer forms run
// on the integer/FP32 issue slots (a round trip measured at 5.0 per clock per
// SM).
//
// Method (IEEE 754 binary64 -> binary32, round to nearest even): for a double
// of biased exponent e in [897, 1150] the float has exponent e - 896, whose low
// 8 bits are (e & 0xff) ^ 0x80 because 896 = 3 * 256 + 128; its 23 mantissa
// bits are the top 23 of the double's 52, and the 29 dropped bits r round up
// when r > 2^28, or r == 2^28 with an odd kept mantissa, i.e. when
// r + lsb + (2^28 - 1) >= 2^29.  A carry out of the mantissa moves into the
// exponent, and 0x7f7fffff + 1 is infinity, as rounding requires.  e <= 872
// (|x| < 2^-150) gives a signed zero, 1151 <= e <= 2046 (|x| >= 2^128) a signed
// infinity.  binary32 -> binary64 is exact: exponent + 896, mantissa shifted
// into place.  What is left (results that are float subnormals, infinities and
// NaNs as inputs, float subnormals widened) is reported as not handled and
// converted by the hardware in a call that is not inlined: a hardware
// conversion in the caller under a branch can be if-converted into a
// predicated instruction, which still costs its issue slot on the FP64 unit
// (measured), while a call runs only on the lanes that take it.
#pragma once

namespace bilu {
namespace cvt {
namespace {

__device__ __noinline__ float f32_slow(double x) { return __double2float_rn(x); }
__device__ __noinline__ double f64_slow(float y) { return (double)y; }

// x rounded to float; ok = false where the result is not handled here.
__device__ __forceinline__ float to_f32(double x, bool& ok) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned h = (unsigned)(u >> 32), l = (unsigned)u;
  const unsigned e = (h >> 20) & 0x7ffu;
  const unsigned sign = h & 0x80000000u;
  const unsigned t = __funnelshift_l(l, h, 3);  // (h << 3) | (l >> 29): exponent bits 7..0 and 23 mantissa bits
  unsigned f = ((t & 0x7fffffffu) ^ 0x40000000u) | sign;
  f += ((l & 0x1fffffffu) + (f & 1u) + 0x0fffffffu) >> 29;
  f = e < 897u ? sign : (e > 1150u ? (sign | 0x7f800000u) : f);
  ok = (e - 873u) >= 24u && e != 0x7ffu;
  return __uint_as_float(f);
}

// y widened to double; ok = false for float subnormals, infinities and NaNs.
__device__ __forceinline__ double to_f64(float y, bool& ok) {
  const unsigned f = __float_as_uint(y);
  const unsigned e = (f >> 23) & 0xffu;
  const unsigned sign = f & 0x80000000u;
  const bool zero = (f & 0x7fffffffu) == 0u;
  const unsigned hi = zero ? sign : ((((f & 0x7fffffffu) >> 3) + 0x38000000u) | sign);
  ok = zero || (e - 1u) < 254u;
  return __longlong_as_double((long long)(((unsigned long long)hi << 32) | (f << 29)));
}

// The conversions for any value: the integer forms, and the hardware's for
// what they leave (in a call, so that only the lanes that need it run it).
__device__ __forceinline__ float f32(double x) {
  bool ok;
  float f = to_f32(x, ok);
  if (!ok) f = f32_slow(x);
  return f;
}

__device__ __forceinline__ double f64(float y) {
  bool ok;
  double d = to_f64(y, ok);
  if (!ok) d = f64_slow(y);
  return d;
}

}  // namespace
}  // namespace cvt
}  // namespace bilu
