// df32.cuh -- double-float arithmetic (an unevaluated sum hi + lo of two
// FP32 numbers, about 48 significant bits) for the mixed path's increment
// solve.  GB300 runs FP32 at roughly 60x its FP64 rate, so a double-float
// operation (7-20 FP32 instructions) still costs less than one FP64
// instruction's share of the FP64 pipe.
//
// The operations are the classical error-free transformations: Knuth's
// TwoSum (exact a + b = s + e with six additions), Dekker's Fast2Sum
// (|a| >= |b|) and the FMA-based TwoProd (exact a * b = p + e with
// e = fma(a, b, -p)), combined as in the double-double algorithms of
// Dekker (1971) and Hida, Li and Bailey (2001).  Relative error of + and *
// is a few units of 2^-48.  Nothing here may be reassociated, so this file
// relies on the default (IEEE) FP32 compilation: no fast-math.
#pragma once
#include <cuda_runtime.h>

namespace chf {

struct df32 {
  float hi, lo;
  df32() = default;
  // exact split of a double (hi = nearest float, lo = nearest float of the
  // remainder); constant-folded for literals
  __host__ __device__ constexpr df32(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr df32(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr df32(int i) : hi((float)i), lo(0.f) {}
  __host__ __device__ double to_double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ df32 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df32(s, e);
}

__device__ __forceinline__ df32 df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df32(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df32 operator+(df32 a, df32 b) {
  df32 s = df_two_sum(a.hi, b.hi);
  const df32 t = df_two_sum(a.lo, b.lo);
  s = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

__device__ __forceinline__ df32 operator-(df32 a) { return df32(-a.hi, -a.lo); }

__device__ __forceinline__ df32 operator-(df32 a, df32 b) { return a + (-b); }

__device__ __forceinline__ df32 operator*(df32 a, df32 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return df_fast_two_sum(p, e);
}

}  // namespace chf
