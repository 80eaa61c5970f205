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
#include <cstdint>
#include <cstring>

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

// ---------------------------------------------------------------------------
// Conversions between double and float pairs by integer operations on the IEEE
// bit layouts (binary64: 1/11/52, binary32: 1/8/23). GB300 issues two FP64
// instructions per SM and clock, and the double<->float conversions run on that
// pipe; these run on the integer and FP32 pipes. Values outside the range where
// both float parts are normal take the conversion instructions instead.
// ---------------------------------------------------------------------------
FQ_HDI uint64_t bits_of(double d) {
#if defined(__CUDA_ARCH__)
  return uint64_t(__double_as_longlong(d));
#else
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return u;
#endif
}
FQ_HDI double double_of(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d;
  std::memcpy(&d, &u, 8);
  return d;
#endif
}
FQ_HDI uint32_t bits_of(float f) {
#if defined(__CUDA_ARCH__)
  return uint32_t(__float_as_uint(f));
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
FQ_HDI float float_of(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
// 2^k for -126 <= k <= 127
FQ_HDI float pow2f(int k) { return float_of(uint32_t(k + 127) << 23); }

// The rare ranges of the conversions below (|exponent| > 60, subnormals, inf,
// nan) take the conversion instructions, which run on the FP64 pipe. They stay
// out of line: inlined, the compiler if-converts the short fallback and issues
// its conversions for every value.
#if defined(__CUDACC__)
#define FQ_NOINLINE __noinline__
#else
#define FQ_NOINLINE __attribute__((noinline))
#endif
// (hi, lo) packed into one 64-bit word: returned in registers, no stack
static FQ_HD FQ_NOINLINE uint64_t split_rare(double d) {
  const float hi = f_from_double(d);
  const float lo = f_from_double(d - double(hi));
  return (uint64_t(bits_of(lo)) << 32) | bits_of(hi);
}
static FQ_HD FQ_NOINLINE double widen_rare(float f) { return double(f); }

// float -> double, exact.
FQ_HDI double widen(float f) {
  const uint32_t u = bits_of(f);
  const uint32_t ex = (u >> 23) & 0xffu;
  if (ex == 0u || ex == 0xffu) {
    if ((u & 0x7fffffffu) == 0u) return double_of(uint64_t(u) << 32);  // signed zero
    return widen_rare(f);                                             // subnormal, inf, nan
  }
  return double_of((uint64_t(u & 0x80000000u) << 32) | (uint64_t(ex + 896u) << 52) |
                   (uint64_t(u & 0x7fffffu) << 29));
}

// 8-byte aligned like float2: one 64-bit load or store moves a value, where a
// 4-byte-aligned pair takes two 32-bit accesses.
struct alignas(8) df64 {
  float hi, lo;

  FQ_HDI df64() : hi(0.f), lo(0.f) {}
  FQ_HDI df64(float h, float l) : hi(h), lo(l) {}
  // Split a double into the nearest float (ties to even) and the float nearest
  // the remainder d - hi, which is exact: the 53-bit significand m is divided
  // into its leading 24 bits (rounded) and a signed remainder of at most 29 bits.
  FQ_HDI explicit df64(double d) {
    const uint64_t u = bits_of(d);
    if ((u << 1) == 0u) {  // signed zero
      hi = float_of(uint32_t(u >> 32));
      lo = 0.f;
      return;
    }
    const int e = int((u >> 52) & 0x7ffu) - 1023;  // unbiased exponent
    if (e < -60 || e > 60) {
      const uint64_t p = split_rare(d);
      hi = float_of(uint32_t(p));
      lo = float_of(uint32_t(p >> 32));
      return;
    }
    const uint64_t m = (u & 0xfffffffffffffull) | (1ull << 52);  // d = +-m 2^(e-52)
    uint32_t h = uint32_t(m >> 29);                             // 24 bits
    const uint32_t r = uint32_t(m & 0x1fffffffu);
    if (r > 0x10000000u || (r == 0x10000000u && (h & 1u))) ++h;
    const int32_t rem = int32_t(int64_t(m) - (int64_t(h) << 29));  // |rem| <= 2^28
    const uint32_t sign = uint32_t(u >> 63) << 31;
    // hi = h 2^(e-23): h is 2^23..2^24 (2^24 after a carry: one binade up)
    hi = h == (1u << 24) ? float_of(sign | (uint32_t(e + 1 + 127) << 23))
                         : float_of(sign | (uint32_t(e + 127) << 23) | (h & 0x7fffffu));
    // lo = rem 2^(e-52), rounded once by the int -> float conversion, scaled
    // exactly (|e| <= 60 keeps both factors and the product normal)
    const float lr = float(rem) * pow2f(-60) * pow2f(e + 8);
    lo = sign ? -lr : lr;
  }
  FQ_HDI explicit df64(int i) : hi(float(i)), lo(0.f) {}
  // hi + lo rounded to double: both parts widened exactly, one FP64 add.
  FQ_HDI double to_double() const { return widen(hi) + widen(lo); }
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

// Dekker's float-float add (T. J. Dekker, "A floating-point technique for
// extending the available precision", 1971; the "sloppy" add of the QD
// library): one TwoSum of the leading parts, the trailing parts added in FP32,
// one renormalisation. 11 FP32 operations against the accurate add's 20; its
// error is bounded by about 2^-44 (|a| + |b|), relative to the operands rather
// than to the sum.
FQ_HDI df64 dd_add_dekker(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  const float e = f_add(s.lo, f_add(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
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

FQ_HDI df64 dd_abs(df64 a) { return a.hi < 0.f ? -a : a; }

// Square root: the FP32 root of the leading part, corrected once by the Newton
// step of Karp and Markstein, s = q + (a - q^2) / (2 q) with the residual in
// float-float and the division in FP32 (the correction only needs 24 bits).
FQ_HDI df64 dd_sqrt(df64 a) {
  if (!(a.hi > 0.f)) return df64(0.f, 0.f);
  const float q = sqrtf(a.hi);
  const df64 qq(q, 0.f);
  const df64 res = a - qq * qq;
  return fast_two_sum(q, res.hi / (q + q));
}

// Storage: a df64 occupies the same 8 bytes as a double, with its alignment.
static_assert(sizeof(df64) == 8, "df64 must pack into 8 bytes");
static_assert(alignof(df64) == 8, "df64 must be 8-byte aligned");

}  // namespace fq
