// Host check of channel_flow_gb300/csrc/f64bits.cuh against the compiler's
// own IEEE conversions.  Prints "ok" and exits 0, or the first mismatch.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <random>

#include "../channel_flow_gb300/csrc/f64bits.cuh"

using namespace chf::bits;

static int fail(const char* what, double x, double a, double b) {
  std::printf("%s: x=%.17g got=%.17g want=%.17g\n", what, x, a, b);
  return 1;
}

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> mant(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-125, 120);
  for (int i = 0; i < 2000000; ++i) {
    const double x = std::ldexp(mant(rng), ex(rng));
    // narrow: nearest binary32 (random values are never exact ties)
    const float n = narrow(x);
    const float nref = std::fabs(x) >= std::ldexp(1.0, -126) ? static_cast<float>(x) : 0.f;  // flush
    if (n != nref) return fail("narrow", x, n, nref);
    if (narrow_rn(x) != nref) return fail("narrow_rn", x, narrow_rn(x), nref);
    // split: hi is x truncated to 24 bits, lo the next 23 bits
    float hi, lo;
    split(x, hi, lo);
    const double hd = std::fabs(x) >= std::ldexp(1.0, -126) ? u2d(d2u(x) & ~((1ull << 29) - 1)) : 0.0;
    if ((double)hi != hd) return fail("split hi", x, hi, hd);
    const double err = std::fabs(x - ((double)hi + (double)lo));
    const int rel = std::fabs(x) >= std::ldexp(1.0, -80) ? -46 : -23;
    if (hd != 0.0 && err > std::ldexp(std::fabs(x), rel)) return fail("split lo", x, (double)hi + (double)lo, x);
    if (lo != 0.f && (std::signbit(lo) != std::signbit(x))) return fail("split lo sign", x, lo, x);
    // widen: exact
    const float f = static_cast<float>(x);
    const double wref = std::fabs(f) >= std::ldexp(1.0f, -126) ? static_cast<double>(f) : 0.0;  // flush
    if (widen(f) != wref) return fail("widen", f, widen(f), wref);
  }
  // edge cases
  const double zeros[] = {0.0, -0.0, 1e-300, -1e-300, std::ldexp(1.0, -127), std::ldexp(-1.0, -130)};
  for (double z : zeros) {
    float hi, lo;
    split(z, hi, lo);
    if (hi != 0.f || lo != 0.f || narrow(z) != 0.f) return fail("flush", z, hi, 0.0);
  }
  if (!std::isinf(narrow(1e300)) || !std::isinf(narrow(-1e300)) || narrow(-1e300) > 0) return fail("inf", 1e300, narrow(1e300), 0);
  if (!std::isnan(narrow(std::nan(""))) || !std::isnan(widen(std::nanf("")))) return fail("nan", 0, 0, 0);
  if (!std::isinf(widen(INFINITY)) || widen(1.5f) != 1.5) return fail("widen edge", 0, 0, 0);
  // rounding carry into the exponent and the smallest normal
  const double up = std::nextafter(2.0, 0.0);  // rounds up to 2.0f
  if (narrow(up) != 2.0f) return fail("carry", up, narrow(up), 2.0);
  if (narrow_rn(up) != static_cast<float>(up)) return fail("carry rn", up, narrow_rn(up), static_cast<float>(up));
  // exact ties go to the even significand, as the compiler's conversion does
  for (double t : {1.0 + std::ldexp(1.0, -24), 1.0 + 3.0 * std::ldexp(1.0, -24), -(1.0 + 3.0 * std::ldexp(1.0, -24)),
                   std::ldexp(1.0 + std::ldexp(1.0, -24), 100), 2.0 - std::ldexp(1.0, -25)})
    if (narrow_rn(t) != static_cast<float>(t)) return fail("tie rn", t, narrow_rn(t), static_cast<float>(t));
  if (!std::isinf(narrow_rn(1e300)) || !std::isnan(narrow_rn(std::nan(""))) || narrow_rn(1e-300) != 0.f)
    return fail("special rn", 0, 0, 0);
  const double tiny = std::ldexp(1.0, -126);
  if (narrow(tiny) != static_cast<float>(tiny)) return fail("min normal", tiny, narrow(tiny), tiny);
  for (double x : {1.0, -3.5, 1e-300, -7e200, 0.0, std::ldexp(1.0, -1021)})
    if (half(x) != x * 0.5) return fail("half", x, half(x), x * 0.5);
  for (uint32_t n = 1; n < (1u << 20); ++n)
    if (from_int(n) != (double)n) return fail("from_int", n, from_int(n), n);
  if (from_int(0x7fffffffu) != 2147483647.0) return fail("from_int max", 0, 0, 0);
  // scaled integers (the exact-GEMM epilogue): t 2^n
  std::uniform_int_distribution<long long> ti(-(1ll << 46), (1ll << 46));
  std::uniform_int_distribution<int> sh(-60, 10);
  for (int i = 0; i < 2000000; ++i) {
    long long t = ti(rng);
    if (i % 4 == 1) t >>= (i % 40);  // small magnitudes too
    const int n = sh(rng);
    const double want = std::ldexp((double)t, n);
    if (scaled_i64(t, n) != want) return fail("scaled_i64", (double)t, scaled_i64(t, n), want);
    const float wf = static_cast<float>(std::ldexp((double)static_cast<float>(t), n));  // RN-even once
    if (scaled_i64_f(t, n) != wf) return fail("scaled_i64_f", (double)t, scaled_i64_f(t, n), wf);
  }
  if (scaled_i64_f((1ll << 24) + 1, 0) != 16777216.f || scaled_i64_f((1ll << 24) + 3, 0) != 16777220.f ||
      scaled_i64_f(-((1ll << 25) - 1), 0) != -33554432.f)
    return fail("ties", 0, 0, 0);
  std::printf("ok\n");
  return 0;
}
