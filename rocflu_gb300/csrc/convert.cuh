// Conversions between float and double with integer and FP32 instructions,
// bit-identical to the hardware conversions (round to nearest even) for every
// input: zeros, denormals, overflow, infinities and NaNs (any NaN maps to a
// NaN).  In the mixed update they would otherwise occupy a large part of the
// FP64 pipe, the kernel's bound there.  rflu_gpu_check_conversions compares
// them with the hardware's on the device.
#pragma once

namespace rflu {

__device__ inline double f2d(float f) {
  // denormals are scaled into the normal range first (exact: a power of 2)
  const bool den = (__float_as_uint(f) & 0x7F800000u) == 0u && f != 0.f;
  const unsigned u = __float_as_uint(den ? f * 18446744073709551616.f : f);
  const unsigned ex = (u >> 23) & 0xFFu;
  unsigned long long dex = ex == 0u ? 0ull : (ex == 255u ? 2047ull : (unsigned long long)(ex + 896u));
  if (den) dex -= 64ull;
  const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) | (dex << 52) |
                                  ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)bits);
}
__device__ inline float d2f(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FFull);
  const unsigned long long man = b & 0xFFFFFFFFFFFFFull;
  const int fex = e - 896;  // the float's biased exponent
  if ((unsigned)(fex - 1) < 254u) {
    const unsigned m = (unsigned)(man >> 29);
    const unsigned rem = (unsigned)(man & 0x1FFFFFFFull);
    // the mantissa carry of the rounding increments the exponent, as it must
    const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | ((((unsigned)fex << 23) | m) + up));
  }
  if (e == 0x7FF) return __uint_as_float(sign | (man ? 0x7FC00000u : 0x7F800000u));  // nan, inf
  if (fex >= 255) return __uint_as_float(sign | 0x7F800000u);                        // overflow
  if (e == 0) return __uint_as_float(sign);  // zero and double denormals
  // a float denormal (or zero): (2^52 + man) * 2^-(30 - fex) units of 2^-149
  const int sh = 30 - fex;
  if (sh >= 54) return __uint_as_float(sign);
  const unsigned long long M = man | (1ull << 52);
  const unsigned long long q = M >> sh, rem = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  return __uint_as_float(sign | ((unsigned)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u)));
}

}  // namespace rflu
