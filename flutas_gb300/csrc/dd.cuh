// dd.cuh -- double-float arithmetic: a value as the unevaluated sum h + l of
// two FP32 numbers (about 48 significant bits).
//
// The FP64 solver's x/y transforms run in it.  On this part one FP64
// instruction costs about as much issue time as 57 FP32 ones, and an FFT is
// sums and products only, which double-float arithmetic builds from a handful
// of FP32 operations each (error-free two-sum and fused multiply-add):
//   two_sum(a, b)      s + e = a + b exactly (Knuth, 6 operations)
//   fast_two_sum(a, b) the same for |a| >= |b| (Dekker, 3 operations)
//   a + b (dd)         two_sum of the high parts, the low parts added, renormalised
//   a * b (dd)         the high product and its exact rounding error by FMA, the
//                      cross terms by FMA, renormalised
// The sum is the "sloppy" double-float addition: its error is bounded by about
// 2^-47 of the larger operand, not of the result, which is the bound a linear
// transform needs (the error of each output relative to the input's norm).
// Conversions from and to FP64 go through bits.cuh (integer instructions) and
// one FP64 addition, so the transforms issue almost nothing on the FP64 pipe.
//
// The z sweeps, stencils, residuals and updates stay in FP64.
#pragma once
#include <cmath>

#include "bits.cuh"

namespace fg {

struct dd {
  float h, l;
  dd() = default;
  FG_HD constexpr dd(float h_, float l_) : h(h_), l(l_) {}
  // For constants (folded at compile time); runtime FP64 values go through dd_of.
  FG_HD constexpr dd(double x) : h((float)x), l((float)(x - (double)(float)x)) {}
  FG_HD constexpr dd(int x) : h((float)x), l(0.0f) {}
  // Host-side reading (tests, tables); device code uses double_of (no FP32 -> FP64 convert instruction).
  FG_HD explicit constexpr operator double() const { return (double)h + (double)l; }
};

FG_HD dd dd_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dd(s, b - (s - a));
}
FG_HD dd dd_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return dd(s, (a - (s - bb)) + (b - bb));
}
FG_HD dd operator+(dd a, dd b) {
  const dd s = dd_two_sum(a.h, b.h);
  return dd_fast_two_sum(s.h, s.l + (a.l + b.l));
}
FG_HD dd operator-(dd a) { return dd(-a.h, -a.l); }
FG_HD dd operator-(dd a, dd b) { return a + dd(-b.h, -b.l); }
FG_HD dd operator*(dd a, dd b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return dd_fast_two_sum(p, e);
}

// FP64 -> double-float: the exact split of bits.cuh where it applies (no FP64
// instruction), the truncated high part alone outside its range.
FG_HD dd dd_of(double x) {
  float h, l;
  if (split_ok(x)) {
    split32(x, h, l);
  } else {
    h = f32_of(x);
    l = 0.0f;
  }
  return dd(h, l);
}
// double-float -> FP64: both parts exactly, one FP64 addition.
FG_HD double double_of(dd v) { return f64_of(v.h) + f64_of(v.l); }

}  // namespace fg
