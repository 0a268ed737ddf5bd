// FP64 operations done exactly with integer arithmetic, bit for bit equal to
// the hardware's: the FP64 <-> FP32 conversions (round to nearest even,
// cvt.rn.f32.f64, and cvt.f64.f32) and the correctly rounded FP64 reciprocal
// (__drcp_rn).
//
// Why: GB300's FP64 unit is the bound of the factorisation and solver kernels
// (about 1.6 FP64 FMAs per clock per SM), and these operations run there too;
// their integer forms run on the integer and FP32 issue slots instead and
// overlap with the FP64 work (measured: a 1:1 mix of integer reciprocals and
// DFMAs runs at the integer reciprocal's own rate).
//
// Conversions.
// On GB300 a hardware conversion between double and float issues at about
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
namespace ifp {
namespace {

__device__ __noinline__ float f32_slow(double x) { return __double2float_rn(x); }
__device__ __noinline__ double f64_slow(float y) { return (double)y; }
__device__ __noinline__ double rcp_slow(double u) { return __drcp_rn(u); }

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

// Reciprocal.  RN(1/u) for a double u = m 2^(e-1075) with biased exponent
// e in [1, 2044] (the result is then a normal double), by Newton-Raphson
// iteration on integers (the textbook reciprocal iteration x' = x (2 - M x),
// here in 64-bit fixed point) and an exact remainder for the rounding:
//   * m = 2^52 (u a power of two): 1/u = 2^(1023-(e-1023)), biased exponent
//     2046 - e, mantissa 0;
//   * otherwise 2^105 / m lies in (2^52, 2^53), 1/u = (2^105 / m) 2^(970-e),
//     biased exponent 2045 - e, and the 53-bit significand is
//     Y = RN(2^105 / m).  With m64 = m 2^11 in (2^63, 2^64), x approximates
//     R = 2^127 / m64 in (2^63, 2^64): a seed from the FP32 approximate
//     reciprocal of the top 24 bits of the significand (clamped to
//     [2^63, 2^64 - 1]: relative error below 2^-21), then two steps
//     x += x (2^127 - m64 x) / 2^127, the error term's high word (below 2^44
//     in magnitude after the seed) times x, (a few units of 2^0 after two
//     steps).  q = x >> 11 is within one of floor(2^105 / m); the remainder
//     2^105 - q m (|.| < 2^54, so exact in 64-bit two's complement, 2^105 being
//     0 modulo 2^64) corrects q to the floor, and Y = q + (2 rem > m) (no ties:
//     2^105 / m is never an odd multiple of 1/2 for m not a power of two).
// Other u (zero, subnormal, infinite, NaN, or e >= 2045, whose reciprocal is
// subnormal) are reported as not handled.
__device__ __forceinline__ double to_rcp(double u, bool& ok) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(u);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  const unsigned long long sign = b & 0x8000000000000000ull;
  const unsigned long long f = b & 0xfffffffffffffull;
  ok = (e - 1u) < 2044u;
  const unsigned long long m = f | (1ull << 52);
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(0x3f800000u | (unsigned)(f >> 29))));
  const unsigned rb = __float_as_uint(r);
  unsigned long long x = rb >= 0x3f800000u ? ~0ull
                         : rb < 0x3f000000u ? (1ull << 63)
                                            : ((unsigned long long)((rb & 0x7fffffu) | 0x800000u) << 40);
  const unsigned long long m64 = m << 11;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const unsigned long long th = __umul64hi(m64, x), tl = m64 * x;
    const long long eh = (long long)(0x8000000000000000ull - th - (tl != 0ull ? 1ull : 0ull));
    const unsigned long long ae = eh < 0 ? (unsigned long long)(-eh) : (unsigned long long)eh;
    const unsigned long long c = __umul64hi(x, ae << 1);
    x = eh < 0 ? x - c : x + c;
  }
  unsigned long long q = x >> 11;
  long long rem = (long long)(0ull - q * m);
  if (rem < 0) {
    q -= 1;
    rem += (long long)m;
  } else if (rem >= (long long)m) {
    q += 1;
    rem -= (long long)m;
  }
  q += (2ull * (unsigned long long)rem > m) ? 1ull : 0ull;
  const unsigned long long mant = f == 0ull ? 0ull : (q & 0xfffffffffffffull);
  const unsigned long long ex = f == 0ull ? (2046ull - e) : (2045ull - e);
  return __longlong_as_double((long long)(sign | (ex << 52) | mant));
}

// RN(1/u) for any u: the integer form, the hardware's for what it leaves.
__device__ __forceinline__ double rcp(double u) {
  bool ok;
  double y = to_rcp(u, ok);
  if (!ok) y = rcp_slow(u);
  return y;
}

}  // namespace
}  // namespace ifp
}  // namespace bilu
