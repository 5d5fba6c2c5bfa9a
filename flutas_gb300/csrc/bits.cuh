// bits.cuh -- FP64 <-> FP32 conversions by integer bit operations.
//
// A conversion instruction between FP64 and FP32 issues on the FP64 pipe, the
// scarce unit of the part (about 1/57 of the FP32 rate); these run on the
// integer ALUs instead.  __host__ __device__ so the CPU tests run the same code.
//
// f32_of truncates the mantissa toward zero (relative error < 2^-23), flushes
// magnitudes below 2^-126 to a signed zero and turns finite values above the
// FP32 range into infinities; NaN stays NaN.  f64_of is exact for normal FP32
// values (FP32 subnormals become a signed zero).
#pragma once
#include <cstring>

#ifndef FG_HD
#define FG_HD __host__ __device__ __forceinline__
#endif

namespace fg {

FG_HD unsigned hi_word(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2hiint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, 8);
  return (unsigned)(b >> 32);
#endif
}
FG_HD unsigned lo_word(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2loint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, 8);
  return (unsigned)b;
#endif
}
FG_HD double from_words(unsigned hi, unsigned lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const unsigned long long b = ((unsigned long long)hi << 32) | lo;
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
FG_HD float float_of_bits(unsigned f) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(f);
#else
  float x;
  memcpy(&x, &f, 4);
  return x;
#endif
}
FG_HD unsigned bits_of_float(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned f;
  memcpy(&f, &x, 4);
  return f;
#endif
}

// General form: every exponent (subnormal results flushed, overflow to inf, NaN kept).
FG_HD float f32_of_any(unsigned hi, unsigned lo) {
  const unsigned sign = hi & 0x80000000u, ex = (hi >> 20) & 0x7ffu;
  const int e = (int)ex - 896;  // FP32 biased exponent
  unsigned f = sign | ((unsigned)e << 23) | (((hi << 3) | (lo >> 29)) & 0x7fffffu);
  if (e <= 0) f = sign;
  if (e >= 255) f = sign | 0x7f800000u | ((ex == 0x7ffu && ((hi & 0xfffffu) | lo)) ? 0x400000u : 0u);
  return float_of_bits(f);
}

// For |x| in FP32's normal range (double exponent 897..1150) the FP32 bit
// pattern is the double's top 32 bits shifted left by 3 (exponent field and
// the top 23 mantissa bits), with the FP32 exponent = double exponent - 896:
// in that range the low 8 bits of the double exponent are the FP32 exponent
// with bit 7 flipped, so one XOR rebiases.  Four integer instructions; other
// values take the general form above.
FG_HD float f32_of(double x) {
  const unsigned hi = hi_word(x), lo = lo_word(x);
  if ((hi & 0x7fffffffu) - 0x38100000u < 0x47f00000u - 0x38100000u)
    return float_of_bits(((((hi << 3) | (lo >> 29)) & 0x7fffffffu) ^ 0x40000000u) | (hi & 0x80000000u));
  return f32_of_any(hi, lo);
}

FG_HD double f64_of(float x) {
  const unsigned f = bits_of_float(x);
  if ((f & 0x7fffffffu) - 0x00800000u < 0x7f000000u)  // normal: rebias the exponent by +896, spread the mantissa
    return from_words((((f & 0x7fffffffu) >> 3) + 0x38000000u) | (f & 0x80000000u), f << 29);
  const unsigned e = (f >> 23) & 0xffu;
  unsigned hi = (f & 0x80000000u) | ((e + 896u) << 20) | ((f >> 3) & 0xfffffu), lo = f << 29;
  if (e == 0) {
    hi = f & 0x80000000u;
    lo = 0u;
  }
  if (e == 255) hi = (f & 0x80000000u) | 0x7ff00000u | ((f >> 3) & 0xfffffu);
  return from_words(hi, lo);
}

// x = h + l with h = f32_of(x) (x truncated to FP32) and l the next 23 bits of
// x's significand: both are exact FP32 values and |x - h - l| < 2^-46 |x|.
// Valid for x = +-0 and 2^-103 <= |x| < 2^128 (double exponent 920..1150),
// which split_ok tells.  l is the difference of two floats of one binade
// (exact, Sterbenz): the remainder bits under a power of two, minus it.  No
// FP64 instruction.
FG_HD bool split_ok(double x) {
  const unsigned hi = hi_word(x), lo = lo_word(x);
  return (hi & 0x7fffffffu) - 0x39800000u < 0x47f00000u - 0x39800000u || ((hi << 1) | lo) == 0u;
}
FG_HD void split32(double x, float &h, float &l) {
  const unsigned hi = hi_word(x), lo = lo_word(x), s = hi & 0x80000000u;
  const unsigned b = ((((hi >> 20) & 0x7ffu) - 919u) << 23) | s;
  const bool zero = ((hi << 1) | lo) == 0u;
  h = zero ? float_of_bits(s) : float_of_bits(((((hi << 3) | (lo >> 29)) & 0x7fffffffu) ^ 0x40000000u) | s);
  l = zero ? float_of_bits(s) : float_of_bits(b | ((lo >> 6) & 0x7fffffu)) - float_of_bits(b);
}
// The forms for values already known to be nonzero and inside split32's range
// (split_range: three integer instructions), without the zero case.
FG_HD bool split_range(double x) { return (hi_word(x) & 0x7fffffffu) - 0x39800000u < 0x47f00000u - 0x39800000u; }
FG_HD void split32_in(double x, float &h, float &l) {
  const unsigned hi = hi_word(x), lo = lo_word(x), s = hi & 0x80000000u;
  const unsigned b = ((((hi >> 20) & 0x7ffu) - 919u) << 23) | s;
  h = float_of_bits(((((hi << 3) | (lo >> 29)) & 0x7fffffffu) ^ 0x40000000u) | s);
  l = float_of_bits(b | ((lo >> 6) & 0x7fffffu)) - float_of_bits(b);
}
FG_HD float f32_in(double x) {  // f32_of's fast path (split_range lies inside it)
  const unsigned hi = hi_word(x), lo = lo_word(x);
  return float_of_bits(((((hi << 3) | (lo >> 29)) & 0x7fffffffu) ^ 0x40000000u) | (hi & 0x80000000u));
}
// a - b from the splits of a and b: (ha - hb) is exact when ha and hb are
// within a factor 2 of each other (the cancelling case), so the result is the
// FP32 rounding of a - b to within 2^-46 (|a| + |b|) and one more rounding.
FG_HD float diff32(float ha, float la, float hb, float lb) { return (ha - hb) + (la - lb); }

}  // namespace fg
