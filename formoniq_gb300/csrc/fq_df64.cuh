// Float-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi)/2, a 48-bit significand (relative rounding error
// about 2^-48 = 3.6e-15 per operation) computed entirely on the FP32 pipe.
//
// Why: GB300 executes FP64 at 1/62 of its FP32 rate (1.25 vs 78 TFLOP/s,
// measured). The element kernels and the scatter are FP64-pipe bound in plain
// double; their results only need 1e-12 relative accuracy, which float-float
// provides at a few FP32 operations per double operation.
//
// The building blocks are the classical error-free transformations (Knuth's
// TwoSum, Dekker's FastTwoSum, and the FMA form of TwoProduct). Each of them is
// exact only if every addition and product rounds on its own, so on the device
// they are written with the _rn intrinsics, which the compiler never fuses into
// an FMA (a plain `a * b + c` may be contracted, and a contracted TwoSum or
// FastTwoSum no longer returns the rounding error). Host builds compile the same
// code with contraction switched off.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "fq_combinatorics.cuh"

namespace fq {

FQ_HDI float f_add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
FQ_HDI float f_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
FQ_HDI float f_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
FQ_HDI float f_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
FQ_HDI float f_from_double(double d) {
#if defined(__CUDA_ARCH__)
  return __double2float_rn(d);
#else
  return static_cast<float>(d);
#endif
}

struct df64 {
  float hi, lo;

  FQ_HDI df64() : hi(0.f), lo(0.f) {}
  FQ_HDI df64(float h, float l) : hi(h), lo(l) {}
  // Split a double into the nearest float and the float nearest the remainder
  // (d - hi is exact in double: hi carries d's leading 24 bits).
  FQ_HDI explicit df64(double d) {
    hi = f_from_double(d);
    lo = f_from_double(d - double(hi));
  }
  FQ_HDI explicit df64(int i) : hi(float(i)), lo(0.f) {}
  FQ_HDI double to_double() const { return double(hi) + double(lo); }
};

FQ_HDI df64 two_sum(float a, float b) {
  const float s = f_add(a, b);
  const float bb = f_sub(s, a);
  const float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
  return df64(s, e);
}

FQ_HDI df64 fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = f_add(a, b);
  const float e = f_sub(b, f_sub(s, a));
  return df64(s, e);
}

FQ_HDI df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  const df64 t = two_sum(a.lo, b.lo);
  s.lo = f_add(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = f_add(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}

FQ_HDI df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
FQ_HDI df64 operator-(df64 a, df64 b) { return a + (-b); }

FQ_HDI df64 operator*(df64 a, df64 b) {
  const float p = f_mul(a.hi, b.hi);
  float e = f_fma(a.hi, b.hi, -p);
  e = f_fma(a.hi, b.lo, e);
  e = f_fma(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

FQ_HDI df64& operator+=(df64& a, df64 b) {
  a = a + b;
  return a;
}
FQ_HDI df64& operator-=(df64& a, df64 b) {
  a = a - b;
  return a;
}

FQ_HDI bool is_zero(df64 a) { return a.hi == 0.f && a.lo == 0.f; }

// Storage: a df64 occupies the same 8 bytes as a double.
static_assert(sizeof(df64) == 8, "df64 must pack into 8 bytes");

}  // namespace fq
