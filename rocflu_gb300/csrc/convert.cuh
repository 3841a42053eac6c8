// Conversions between float and double with integer and FP32 instructions,
// bit-identical to the hardware conversions (round to nearest even) for every
// input: zeros, denormals, overflow, infinities and NaNs (any NaN maps to a
// NaN).  In the mixed update they would otherwise occupy a large part of the
// FP64 pipe, the kernel's bound there.  rflu_gpu_check_conversions compares
// them with the hardware's on the device; the same source compiles for the
// host (the bit casts through memcpy), where tests/convert_check.cpp compares
// them with C casts.
#pragma once

#if defined(__CUDACC__)
#define RFLU_CVT_FN __device__ inline
#else
#include <cstring>
#define RFLU_CVT_FN inline
#endif

namespace rflu {

namespace cvt {
#if defined(__CUDACC__)
RFLU_CVT_FN unsigned bits(float f) { return __float_as_uint(f); }
RFLU_CVT_FN float fromBits(unsigned u) { return __uint_as_float(u); }
RFLU_CVT_FN unsigned long long bits(double d) { return (unsigned long long)__double_as_longlong(d); }
RFLU_CVT_FN double fromBits(unsigned long long u) { return __longlong_as_double((long long)u); }
#else
RFLU_CVT_FN unsigned bits(float f) { unsigned u; std::memcpy(&u, &f, sizeof u); return u; }
RFLU_CVT_FN float fromBits(unsigned u) { float f; std::memcpy(&f, &u, sizeof f); return f; }
RFLU_CVT_FN unsigned long long bits(double d) { unsigned long long u; std::memcpy(&u, &d, sizeof u); return u; }
RFLU_CVT_FN double fromBits(unsigned long long u) { double d; std::memcpy(&d, &u, sizeof d); return d; }
#endif
}  // namespace cvt

RFLU_CVT_FN double f2d(float f) {
  // denormals are scaled into the normal range first (exact: a power of 2)
  const bool den = (cvt::bits(f) & 0x7F800000u) == 0u && f != 0.f;
  const unsigned u = cvt::bits(den ? f * 18446744073709551616.f : f);
  const unsigned ex = (u >> 23) & 0xFFu;
  unsigned long long dex = ex == 0u ? 0ull : (ex == 255u ? 2047ull : (unsigned long long)(ex + 896u));
  if (den) dex -= 64ull;
  const unsigned long long bits = ((unsigned long long)(u & 0x80000000u) << 32) | (dex << 52) |
                                  ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return cvt::fromBits(bits);
}
RFLU_CVT_FN float d2f(double d) {
  const unsigned long long b = cvt::bits(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FFull);
  const unsigned long long man = b & 0xFFFFFFFFFFFFFull;
  const int fex = e - 896;  // the float's biased exponent
  if ((unsigned)(fex - 1) < 254u) {
    const unsigned m = (unsigned)(man >> 29);
    const unsigned rem = (unsigned)(man & 0x1FFFFFFFull);
    // the mantissa carry of the rounding increments the exponent, as it must
    const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return cvt::fromBits(sign | ((((unsigned)fex << 23) | m) + up));
  }
  if (e == 0x7FF) return cvt::fromBits(sign | (man ? 0x7FC00000u : 0x7F800000u));  // nan, inf
  if (fex >= 255) return cvt::fromBits(sign | 0x7F800000u);                        // overflow
  if (e == 0) return cvt::fromBits(sign);  // zero and double denormals
  // a float denormal (or zero): (2^52 + man) * 2^-(30 - fex) units of 2^-149
  const int sh = 30 - fex;
  if (sh >= 54) return cvt::fromBits(sign);
  const unsigned long long M = man | (1ull << 52);
  const unsigned long long q = M >> sh, rem = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  return cvt::fromBits(sign | ((unsigned)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u)));
}

}  // namespace rflu
