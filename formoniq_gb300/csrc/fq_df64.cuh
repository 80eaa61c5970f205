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
// TwoSum, Dekker's FastTwoSum, and the FMA form of TwoProduct), written with
// explicit fmaf where a product's rounding error is needed, so contraction by
// the compiler cannot change their meaning (none of the additions multiplies).
#pragma once

#include <cuda_runtime.h>

namespace fq {

struct df64 {
  float hi, lo;

  __device__ __forceinline__ df64() : hi(0.f), lo(0.f) {}
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  // Split a double into the nearest float and the float nearest the remainder.
  __device__ __forceinline__ explicit df64(double d) {
    hi = __double2float_rn(d);
    lo = __double2float_rn(d - double(hi));
  }
  __device__ __forceinline__ explicit df64(int i) : hi(float(i)), lo(0.f) {}
  __device__ __forceinline__ double to_double() const { return double(hi) + double(lo); }
};

__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df64(s, e);
}

__device__ __forceinline__ df64 fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  const float e = b - (s - a);
  return df64(s, e);
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  const df64 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) {
  a = a + b;
  return a;
}
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) {
  a = a - b;
  return a;
}

__device__ __forceinline__ bool is_zero(df64 a) { return a.hi == 0.f && a.lo == 0.f; }

// Storage: a df64 occupies the same 8 bytes as a double.
static_assert(sizeof(df64) == 8, "df64 must pack into 8 bytes");

}  // namespace fq
