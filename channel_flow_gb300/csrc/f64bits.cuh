// f64bits.cuh -- FP64 <-> FP32 moves by integer operations on the IEEE-754
// bit patterns.
//
// On GB300 the FP64 pipe retires about 2 lane-operations per clock per SM
// (FP32 FMA: about 115), and double <-> float conversions execute on that same
// pipe at the same rate, so a conversion costs as much as a DFMA.  The
// mixed path moves FP64 state into FP32 arithmetic and back at every step;
// these helpers do it with integer instructions (ALU pipe, half the FP32
// rate) instead.  Only the binary64 / binary32 layouts are used:
//   binary64: sign 1 | exponent 11 (bias 1023) | fraction 52
//   binary32: sign 1 | exponent 8  (bias 127)  | fraction 23
// Magnitudes below 2^-126 (binary32 subnormals) are flushed to signed zero,
// magnitudes of 2^128 and above become infinity, NaN stays NaN.
#pragma once
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace chf {
namespace bits {

__host__ __device__ __forceinline__ uint64_t d2u(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
__host__ __device__ __forceinline__ double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ uint32_t f2u(float x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

// binary32 with the given sign bit (0 / 1), biased exponent and fraction;
// the biased exponent is clamped: <= 0 gives signed zero, >= 255 infinity.
__host__ __device__ __forceinline__ float make_f(uint32_t sign, int ebias, uint32_t frac23) {
  if (ebias <= 0) return u2f(sign << 31);
  if (ebias >= 255) return u2f((sign << 31) | 0x7f800000u);
  return u2f((sign << 31) | ((uint32_t)ebias << 23) | frac23);
}

// x truncated to its leading 24 significant bits (hi) and the next 23 bits
// (lo, same sign): hi + lo equals x to 2^-46 relative, |lo| < ulp(hi).  For
// |x| < 2^-80 lo would be a binary32 subnormal and is zero (hi alone: 2^-23).
__host__ __device__ __forceinline__ void split(double x, float& hi, float& lo) {
  const uint64_t u = d2u(x);
  const uint32_t sign = (uint32_t)(u >> 63);
  const int e = (int)((u >> 52) & 0x7ff);
  if (e == 0x7ff) {  // infinity or NaN
    hi = u2f((sign << 31) | 0x7f800000u | (uint32_t)((u >> 29) & 0x7fffffu) | ((u & 0xfffffffffffffull) ? 1u : 0u));
    lo = 0.f;
    return;
  }
  hi = make_f(sign, e - 896, (uint32_t)(u >> 29) & 0x7fffffu);
  // remainder: fraction bits 28..6 as an integer n < 2^23, weight 2^(e - 1069)
  const uint32_t n = (uint32_t)(u >> 6) & 0x7fffffu;
  const float nf = u2f(0x4b000000u | n) - 8388608.0f;  // exact: 2^23 + n - 2^23
  const int pe = e - 1069 + 127;                       // biased exponent of 2^(e - 1069)
  lo = (e == 0 || pe <= 0 || e - 896 <= 0) ? 0.f : nf * u2f((uint32_t)pe << 23);
  if (sign) lo = -lo;
}

// x rounded to the nearest binary32 (ties away from zero).
__host__ __device__ __forceinline__ float narrow(double x) {
  const uint64_t u = d2u(x);
  const uint32_t sign = (uint32_t)(u >> 63);
  const int e = (int)((u >> 52) & 0x7ff);
  if (e == 0x7ff) return u2f((sign << 31) | 0x7f800000u | ((u & 0xfffffffffffffull) ? 0x400000u : 0u));
  // adding half an ulp of the 24-bit result to the magnitude bits carries into
  // the exponent when the fraction overflows, which is the correct result
  const uint64_t r = (u & 0x7fffffffffffffffull) + (1ull << 28);
  const int er = (int)(r >> 52);
  return make_f(sign, e == 0 ? 0 : er - 896, (uint32_t)(r >> 29) & 0x7fffffu);
}

// x rounded to the nearest binary32, ties to even (the hardware conversion's
// result wherever that is a normal binary32); magnitudes below 2^-126 give
// signed zero, 2^128 and above infinity, NaN stays NaN.
__host__ __device__ __forceinline__ float narrow_rn(double x) {
  const uint64_t u = d2u(x);
  const uint32_t sign = (uint32_t)(u >> 63);
  const int e = (int)((u >> 52) & 0x7ff);
  if (e == 0x7ff) return u2f((sign << 31) | 0x7f800000u | ((u & 0xfffffffffffffull) ? 0x400000u : 0u));
  // half an ulp of the 24-bit result minus one, plus the kept part's last
  // bit: a tie carries only from an odd significand
  const uint64_t m = u & 0x7fffffffffffffffull;
  const uint64_t r = m + 0x0fffffffull + ((m >> 29) & 1ull);
  return make_f(sign, e == 0 ? 0 : (int)(r >> 52) - 896, (uint32_t)(r >> 29) & 0x7fffffu);
}

// the binary64 of a binary32 (exact; binary32 subnormals give signed zero)
__host__ __device__ __forceinline__ double widen(float f) {
  const uint32_t v = f2u(f);
  const uint64_t sign = (uint64_t)(v >> 31) << 63;
  const uint32_t ef = (v >> 23) & 0xffu;
  if (ef == 0) return u2d(sign);
  const uint64_t ed = ef == 0xffu ? 0x7ffull : (uint64_t)(ef + 896u);
  return u2d(sign | (ed << 52) | ((uint64_t)(v & 0x7fffffu) << 29));
}

// x / 2 by decrementing the exponent (exact for |x| >= 2^-1021; smaller
// magnitudes give signed zero)
__host__ __device__ __forceinline__ double half(double x) {
  const uint64_t u = d2u(x);
  return ((u >> 52) & 0x7ff) > 1 ? u2d(u - (1ull << 52)) : u2d(u & 0x8000000000000000ull);
}

// the binary64 of an integer 1 <= n < 2^31 (exact)
__host__ __device__ __forceinline__ double from_int(uint32_t n) {
#ifdef __CUDA_ARCH__
  const int top = 31 - __clz(n);
#else
  const int top = 31 - __builtin_clz(n);
#endif
  return u2d(((uint64_t)(1023 + top) << 52) | (((uint64_t)n << (52 - top)) & 0xfffffffffffffull));
}

__host__ __device__ __forceinline__ int clz64(uint64_t a) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)a);
#else
  return __builtin_clzll(a);
#endif
}

// t 2^n as a binary64, exact for |t| < 2^53 (results below 2^-1022 give
// signed zero, above the binary64 range infinity)
__host__ __device__ __forceinline__ double scaled_i64(long long t, int n) {
  if (t == 0) return 0.0;
  const uint64_t sign = t < 0 ? 0x8000000000000000ull : 0ull;
  const uint64_t a = t < 0 ? (uint64_t)(-t) : (uint64_t)t;
  const int top = 63 - clz64(a);  // a in [2^top, 2^(top+1)), top <= 52
  const int eb = 1023 + top + n;
  if (eb <= 0) return u2d(sign);
  if (eb >= 2047) return u2d(sign | 0x7ff0000000000000ull);
  return u2d(sign | ((uint64_t)eb << 52) | ((a << (52 - top)) & 0xfffffffffffffull));
}

// t 2^n rounded to the nearest binary32 (ties to even), |t| < 2^62 (results
// below 2^-126 give signed zero, above the binary32 range infinity)
__host__ __device__ __forceinline__ float scaled_i64_f(long long t, int n) {
  if (t == 0) return 0.f;
  const uint32_t sign = t < 0 ? 1u : 0u;
  const uint64_t a = t < 0 ? (uint64_t)(-t) : (uint64_t)t;
  int top = 63 - clz64(a);
  uint64_t m;  // 24-bit significand
  if (top <= 23) {
    m = a << (23 - top);
  } else {
    const int sh = top - 23;
    const uint64_t r = a + ((1ull << (sh - 1)) - 1) + ((a >> sh) & 1);  // round to nearest even
    m = r >> sh;
    if (m >> 24) {  // rounding carried into a new leading bit
      m >>= 1;
      ++top;
    }
  }
  return make_f(sign, 127 + top + n, (uint32_t)m & 0x7fffffu);
}

}  // namespace bits
}  // namespace chf
