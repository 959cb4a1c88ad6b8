// tc_dev.cuh -- device helpers shared by the tcgen05 GEMM kernels: shared
// addresses, bounded mbarrier waits on %globaltimer, the no-swizzle K-major
// shared-memory descriptor and the bf16 x bf16 -> f32 instruction
// descriptor for 128 x 128 tiles, and the fixed-point digit split of
// k_tcgemm.cu.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace chf {
namespace tc {

constexpr int TC_THREADS = 128;
constexpr long WAIT_NS = 1000000000L;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// wait for the phase with parity `phase` to complete, at most limit_ns of
// wall time (false on timeout)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, long limit_ns = WAIT_NS) {
  const uint64_t t0 = gtimer();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    if (ok) return true;
    if ((long)(gtimer() - t0) > limit_ns) return false;
  }
}

// no-swizzle K-major shared-memory matrix descriptor
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: D = F32, A = B = BF16, both K-major, M = 128, N = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);


// NP digits of x * 2^-e (|x| < 2^e), each the rint of the scaled remainder,
// exact in float: NP = 4, radix 2^7 (d_0 in [-128, 128], then [-64, 64]);
// NP = 3, radix 2^8 (d_0 in [-256, 256], then [-128, 128])
template <int NP>
__device__ __forceinline__ void fx_digits_np(float x, int e, float* dg) {
  constexpr int RB = NP == 4 ? 7 : 8;
  float y = scalbnf(x, RB - e);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    const float di = rintf(y);
    dg[i] = di;
    y = (y - di) * (float)(1 << RB);
  }
}
__device__ __forceinline__ void fx_digits_f(float x, int e, float* dg) { fx_digits_np<4>(x, e, dg); }

// one element of an extra output row: the level sums lev[L] += sum_{i+j=L}
// a_i b_j of the row's digits a (plane-major, kpad each, at k) and the
// column's digits b; every product and level sum is an integer below 2^24,
// so the FP32 FMAs are exact
__device__ __forceinline__ void fx_tail_mac(const float* __restrict__ adig, int kpad, int k, const float* b,
                                            float* lev) {
  const float a0 = adig[k], a1 = adig[kpad + k], a2 = adig[2 * kpad + k], a3 = adig[3 * kpad + k];
  lev[0] = fmaf(a0, b[0], lev[0]);
  lev[1] = fmaf(a0, b[1], fmaf(a1, b[0], lev[1]));
  lev[2] = fmaf(a0, b[2], fmaf(a1, b[1], fmaf(a2, b[0], lev[2])));
  lev[3] = fmaf(a0, b[3], fmaf(a1, b[2], fmaf(a2, b[1], fmaf(a3, b[0], lev[3]))));
}

// the four level sums combined exactly (t = lev0 2^21 + lev1 2^14 + lev2 2^7
// + lev3 in 64 bits) and scaled by 2^n, exactly in FP64 (|t| < 2^46)
__device__ __forceinline__ double fx_tail_value(const float* lev, int n) {
  const long long t = ((long long)__float2int_rn(lev[0]) << 21) + ((long long)__float2int_rn(lev[1]) << 14) +
                      ((long long)__float2int_rn(lev[2]) << 7) + (long long)__float2int_rn(lev[3]);
  return (double)t * __longlong_as_double((long long)(1023 + n) << 52);
}

__device__ __forceinline__ uint16_t bf16_bits(float f) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(f));  // exact: |f| <= 128, integer
}

}  // namespace tc
}  // namespace chf
