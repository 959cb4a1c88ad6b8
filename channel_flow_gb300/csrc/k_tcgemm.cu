// k_tcgemm.cu -- the wall-normal Chebyshev transforms of the mixed path
// as tcgen05 GEMMs with exact accumulation (fixed-point bf16 digits).
//
//   C_f[m][col] = sum_k A[m][k] * B_f[k][col]
//
// Why: the curl of the Lamb vector differentiates the z-transform's output
// (h_v = k^2 H2 + i alpha D H1 + i beta D H3), and D amplifies an error
// floor that is flat across the Chebyshev index by up to N^2.  With operands
// split into floating bf16 planes and one FP32 accumulator, that floor is
// the FP32 rounding of every partial sum (relative to the largest term): it
// dominated the mixed path's error against FP64 (2.5e-5 velocity rel-L2
// after 1000 steps at 128^3; 1.2e-6 with these exact transforms, the same
// as with the z transforms done in FP64).
//
// How: every row m of A is scaled by 2^-f_m and every column c of B by
// 2^-e_c (powers of two, so exactly) into (-1, 1), then written as NP digit
// planes (each digit the rint of the scaled remainder, so all steps are
// exact; digits are integers of at most 9 bits, exact in bf16):
//   NP = 4:  x = sum_i d_i 2^(-7 (i + 1)),  d_0 in [-128, 128], d_i in [-64, 64]
//   NP = 3:  x = sum_i d_i 2^(-8 (i + 1)),  d_0 in [-256, 256], d_i in [-128, 128]
// The products of one level L = i + j summed over K stay integers below 2^24
// (K <= 680 for NP = 4, K <= 204 for NP = 3; the launcher checks), so
// tensor-core FP32 accumulation of a level is EXACT.  B data are taken as
// FP32 (FP64 coefficients are rounded to FP32 first: a relative error per
// coefficient, not a flat floor).  Levels 0..NP-1 (ten or six products) go
// to NP TMEM accumulators; the epilogue combines
//   NP = 4:  t = acc_0 2^21 + acc_1 2^14 + acc_2 2^7 + acc_3,   |t| < 2^46
//   NP = 3:  t = acc_0 2^16 + acc_1 2^8 + acc_2,                 |t| < 2^41
// for FP64 outputs exactly, as one 64-bit integer converted once (the levels
// can cancel), for FP32 outputs by FMAs on the levels (within about 2^-24 of
// the maxima below), and scales by 2^(f_m + e_c - 35) or 2^(f_m + e_c - 32).
// What is dropped -- the higher
// levels and the digit remainders -- is below 2^-28 (NP = 4) or 2^-24
// (NP = 3) of max|A row| * max|B column| per term, instead of 2^-24 of each
// running FP32 sum.  The 4-plane format serves the transforms whose output
// is differentiated (Z2, GL); Z1, whose values go to FP32 products, uses 3
// planes (six MMAs per K16 slice instead of ten).
//
// Operand images: each 128-row tile of A and each 64-column tile of B is
// stored in HBM already in the shared-memory "core matrix" layout that
// tcgen05.mma reads with a no-swizzle K-major descriptor (8 rows x 16 bytes
// per core matrix; core (g = row/8, c = k/8) at (c * G + g) * 128 bytes with
// G = 16 for A and 8 for B).  K is cut into chunks of TC_KC; every (tile,
// chunk, plane) image is one contiguous block moved by one cp.async.bulk,
// completion signalled on an mbarrier.  The GEMM kernel below is persistent
// and warp-specialised (its section says how); every wait in it is bounded
// (1 s of wall time), and on timeout it records an error code, stops issuing
// work, waits (bounded) for the copies and MMAs in flight and frees its
// tensor memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "chf_internal.h"
#include "f64bits.cuh"
#include "tc_dev.cuh"

namespace chf {

namespace {

using namespace tc;

// np digits of x * 2^-e on the host (exact in double), the format of
// fx_digits_np: radix 2^7 for 4 planes, 2^8 for 3
void fx_digits_host(double x, int e, double* dg, int np) {
  const int rb = np == 4 ? 7 : 8;
  double y = std::scalbn(x, rb - e);
  for (int i = 0; i < np; ++i) {
    const double di = std::rint(y);
    dg[i] = di;
    y = (y - di) * (double)(1 << rb);
  }
}


}  // namespace

// ---------------------------------------------------------------------------
// GEMM: persistent and warp-specialised, one CTA per SM (all 512 TMEM
// columns).  CTA c works on the 128-row tile mt = c % mtiles and deals the
// (field, 64-column tile) items of that tile round-robin with the other CTAs
// of the same mt.  Shared memory holds either
//   resident: the CTA's whole A tile image (loaded once) plus a ring of
//             WS_STAGES B chunk stages (K chunks of TC_KC), or
//   streamed: a ring of WS_STAGES stages each holding the A and B chunks
// (resident when it fits: A is the transform matrix, the same for every item,
// and re-reading it per item would make the GEMM L2-bound).
//   warp 0    producer: per K chunk of an item waits for a free stage, then
//             moves the chunk's plane images with cp.async.bulk (completion
//             counted in bytes on the stage's "full" barrier);
//   warps 1-2 MMA issuers (4 planes: levels {0, 3} and {1, 2}, 5 of the 10
//             products each; 3 planes: levels {0, 1} and {2}, 3 of the 6):
//             wait for a free accumulator set (two sets of NP 64-column level
//             accumulators, so one item's epilogue
//             overlaps the next item's MMAs), per chunk wait for "full", issue
//             their level MMAs per K16 slice (descriptors formed once per chunk,
//             advanced by a constant per slice) and commit to the stage's
//             "empty" barrier; after the last chunk they commit to "tfull";
//   warps 3-10 epilogue: wait for "tfull", read the levels back with
//             tcgen05.ld (warp w reads TMEM lanes 32 (w % 4) .., columns
//             32 ((w - 3) / 4) ..), release the set on "tempty" and form the
//             outputs from the exact 64-bit level sum.
// Every wait is bounded (1 s of wall time); a role that times out records
// the failure, the others see it and stop, the producer waits for its copies
// in flight and the MMA issuer drains its outstanding MMAs (both bounded)
// before the tensor memory is freed.
// ---------------------------------------------------------------------------
// instruction descriptor: D = F32, A = B = BF16, both K-major, M = 128, N = 64
constexpr uint32_t IDESC_FX = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr int WS_STAGES = 4;
constexpr int WS_MMA_WARPS = 2;  // issuers on disjoint level accumulators
constexpr int WS_EPI_WARPS = 8;
constexpr int WS_EPI0 = 1 + WS_MMA_WARPS;  // first epilogue warp
constexpr int WS_THREADS = 32 * (WS_EPI0 + WS_EPI_WARPS);
constexpr uint32_t WS_A_PLANE = 128u * TC_KC * 2u;
constexpr uint32_t WS_B_PLANE = (uint32_t)FX_NT * TC_KC * 2u;
// one stage of the ring: the B planes of a K chunk (A resident), or A and B
__host__ __device__ constexpr uint32_t ws_b_stage(int np) { return (uint32_t)np * WS_B_PLANE; }
__host__ __device__ constexpr uint32_t ws_ab_stage(int np) { return (uint32_t)np * (WS_A_PLANE + WS_B_PLANE); }
// two accumulator sets of np 64-column level accumulators (allocation: all 512)
constexpr uint32_t WS_TMEM_COLS = 512u;
constexpr size_t WS_SMEM_LIMIT = 225u * 1024u;  // dynamic, below the 227 KB opt-in

__host__ __device__ inline size_t ws_a_resident_bytes(const FxPlan& p) { return (p.a_tile_bytes + 1023) / 1024 * 1024; }
__host__ __device__ inline bool ws_resident(const FxPlan& p) {
  return ws_a_resident_bytes(p) + (size_t)WS_STAGES * ws_b_stage(p.planes) <= WS_SMEM_LIMIT;
}

// one output from the exact level sums: t 2^n with
//   4 planes: t = acc_0 2^21 + acc_1 2^14 + acc_2 2^7 + acc_3,  |t| < 2^46
//   3 planes: t = acc_0 2^16 + acc_1 2^8 + acc_2,              |t| < 2^41
// (the levels can cancel, so t is formed exactly before the single rounding)
template <int NP>
__device__ __forceinline__ long long fx_level_sum(const uint32_t* acc) {
  if (NP == 4)
    return ((long long)__float2int_rn(__uint_as_float(acc[0])) << 21) +
           ((long long)__float2int_rn(__uint_as_float(acc[1])) << 14) +
           ((long long)__float2int_rn(__uint_as_float(acc[2])) << 7) +
           (long long)__float2int_rn(__uint_as_float(acc[NP - 1]));
  return ((long long)__float2int_rn(__uint_as_float(acc[0])) << 16) +
         ((long long)__float2int_rn(__uint_as_float(acc[1])) << 8) + (long long)__float2int_rn(__uint_as_float(acc[2]));
}
// the power of two of t: 2^(f_m + e_c - FX_SHIFT) (two digit radices for the
// first digits, one per level)
template <int NP>
__host__ __device__ constexpr int fx_shift() { return NP == 4 ? 35 : 32; }
template <typename OutT, int NP>
__device__ __forceinline__ OutT fx_out(const uint32_t* acc, int n);
// FP32: the levels are exact integers below 2^24 held in binary32, so the
// sum is formed by FMAs on them directly, lowest level first (3 planes: two
// FMAs, 4 planes: three), without conversions to integers (which run at a
// quarter of the FMA rate).  Each FMA rounds once: the result is within one
// unit in the last place of t where the levels do not cancel, and within
// 2^-23 max|A row| max|B column| where they do (the format's own truncation
// is 2^-24 of that); the scaling by 2^n is two exact power-of-two multiplies
template <>
__device__ __forceinline__ float fx_out<float, 4>(const uint32_t* acc, int n) {
  const float v = __fmaf_rn(__uint_as_float(acc[0]), 2097152.0f,
                            __fmaf_rn(__uint_as_float(acc[1]), 16384.0f,
                                      __fmaf_rn(__uint_as_float(acc[2]), 128.0f, __uint_as_float(acc[3]))));
  const int h = n / 2;  // two factors keep each power of two in range
  return __fmul_rn(__fmul_rn(v, __int_as_float((127 + h) << 23)), __int_as_float((127 + n - h) << 23));
}
template <>
__device__ __forceinline__ float fx_out<float, 3>(const uint32_t* acc, int n) {
  const float v = __fmaf_rn(__uint_as_float(acc[0]), 65536.0f,
                            __fmaf_rn(__uint_as_float(acc[1]), 256.0f, __uint_as_float(acc[2])));
  const int h = n / 2;  // two factors keep each power of two in range
  return __fmul_rn(__fmul_rn(v, __int_as_float((127 + h) << 23)), __int_as_float((127 + n - h) << 23));
}
// FP64: exact, built from the 64-bit integer by bit operations (off the
// narrow FP64 pipe)
template <>
__device__ __forceinline__ double fx_out<double, 4>(const uint32_t* acc, int n) {
  return bits::scaled_i64(fx_level_sum<4>(acc), n);
}
template <>
__device__ __forceinline__ double fx_out<double, 3>(const uint32_t* acc, int n) {
  return bits::scaled_i64(fx_level_sum<3>(acc), n);
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

template <typename OutT, int NP>
__global__ void __launch_bounds__(WS_THREADS, 1) k_tc_gemm_fx(const __grid_constant__ FxPlan plan,
                                                              const uint8_t* __restrict__ aimg,
                                                              const int* __restrict__ aexp,
                                                              const uint8_t* __restrict__ bimg,
                                                              const int* __restrict__ bexp,
                                                              const __grid_constant__ Ptr8<OutT> outs,
                                                              size_t ldc, int nfields, int* status,
                                                              long wait_ns, int skip_first) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[WS_STAGES], empty[WS_STAGES], tfull[2], tempty[2], drain[WS_MMA_WARPS], abar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t SET_COLS = (uint32_t)FX_NT * NP;  // one accumulator set: NP levels
  const bool resident = ws_resident(plan);
  const int mt = (int)(blockIdx.x % plan.mtiles);
  const long j0 = blockIdx.x / plan.mtiles, jstep = gridDim.x / plan.mtiles;
  const long njobs = (long)nfields * plan.ntiles;  // (field, column tile) items of this row tile
  uint8_t* sAres = smem;                                            // resident A tile
  uint8_t* ring = resident ? smem + ws_a_resident_bytes(plan) : smem;  // stages
  const uint32_t stage_bytes = resident ? ws_b_stage(NP) : ws_ab_stage(NP);
  if (tid == 0) {
    s_fail = 0;
    for (int i = 0; i < WS_STAGES; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&empty[i])), "r"(WS_MMA_WARPS));
    }
    for (int i = 0; i < 2; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tfull[i])), "r"(WS_MMA_WARPS));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tempty[i])), "r"(32 * WS_EPI_WARPS));
    }
    for (int i = 0; i < WS_MMA_WARPS; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&drain[i])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&abar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(WS_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  volatile int* fail = &s_fail;
  const uint8_t* atile = aimg + (size_t)mt * plan.a_tile_bytes;
  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      if (resident) {
        expect_tx(smem_u32(&abar), (uint32_t)plan.a_tile_bytes);
        bulk_copy(smem_u32(sAres), atile, (uint32_t)plan.a_tile_bytes, smem_u32(&abar));
      }
      uint32_t g = 0;  // chunks issued by this CTA
      for (long j = j0; j < njobs && !*fail; j += jstep) {
        const int f = (int)(j / plan.ntiles), nt = (int)(j % plan.ntiles);
        const uint8_t* btile = bimg + (size_t)f * plan.b_field_bytes() + (size_t)nt * plan.b_tile_bytes;
        for (int ch = 0; ch < plan.nchunks; ++ch, ++g) {
          const uint32_t s = g % WS_STAGES, ph = (g / WS_STAGES) & 1u;
          if (!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, wait_ns)) {
            *fail = 1;
            break;
          }
          // test of the bounded waits (chf_test_wait_timeout): the first
          // chunk's copies are not issued, so its stage never fills and the
          // waits on it run out
          if (skip_first && g == 0) continue;
          const int kc = plan.kc[ch];
          const uint32_t apb = 128u * kc * 2u, bpb = (uint32_t)FX_NT * kc * 2u;
          uint8_t* st = ring + (size_t)s * stage_bytes;
          uint8_t* sB = resident ? st : st + NP * WS_A_PLANE;
          const uint32_t fb = smem_u32(&full[s]);
          expect_tx(fb, NP * (bpb + (resident ? 0u : apb)));
          for (int pl = 0; pl < NP; ++pl) {
            if (!resident) bulk_copy(smem_u32(st + pl * WS_A_PLANE), atile + plan.a_chunk_off[ch] + (size_t)pl * apb, apb, fb);
            bulk_copy(smem_u32(sB + pl * WS_B_PLANE), btile + plan.b_chunk_off[ch] + (size_t)pl * bpb, bpb, fb);
          }
        }
      }
      // no copy may still be landing when the CTA exits: the last chunk
      // issued into each stage (and the resident A tile) has arrived (a no-op
      // after a normal run, where the MMA issuer consumed everything)
      for (uint32_t k = g > (uint32_t)WS_STAGES ? g - WS_STAGES : 0; k < g; ++k)
        if (!mbar_wait(smem_u32(&full[k % WS_STAGES]), (k / WS_STAGES) & 1u, wait_ns)) *fail = 6;
      if (resident && !mbar_wait(smem_u32(&abar), 0, wait_ns)) *fail = 7;
    }
  } else if (warp < WS_EPI0) {
    // ---------------- MMA issuers ----------------
    // the two issuers own disjoint level accumulators (see the selection
    // below), with equal numbers of products per K16 slice
    const int mw = warp - 1;
    if (lane == 0) {
      // K-adjacent core matrices: 16 (A, 128 rows) or 8 (B, 64 columns)
      // groups of 8 rows x 16 bytes apart; adjacent 8-row groups 128 B apart.
      // One K16 slice advances the start address by 2 core matrices: 256 / 128
      // in the descriptor's 16-byte units.
      const uint32_t lbo_a = 16u * 128u, lbo_b = 8u * 128u, sbo = 128u;
      bool ok = !resident || mbar_wait(smem_u32(&abar), 0, wait_ns);
      if (!ok) *fail = 3;
      uint32_t g = 0, tc = 0;
      for (long j = j0; ok && j < njobs && !*fail; j += jstep, ++tc) {
        const uint32_t b = tc & 1u, tph = (tc >> 1) & 1u;
        if (!mbar_wait(smem_u32(&tempty[b]), tph ^ 1u, wait_ns)) {
          *fail = 2;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t tacc = tmem + b * SET_COLS;
        for (int ch = 0; ch < plan.nchunks; ++ch, ++g) {
          const uint32_t s = g % WS_STAGES, ph = (g / WS_STAGES) & 1u;
          if (!mbar_wait(smem_u32(&full[s]), ph, wait_ns)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const int kc = plan.kc[ch];
          const uint8_t* st = ring + (size_t)s * stage_bytes;
          const uint8_t* sA = resident ? sAres + plan.a_chunk_off[ch] : st;
          const uint32_t aplane = resident ? 128u * kc * 2u : WS_A_PLANE;
          const uint8_t* sB = resident ? st : st + NP * WS_A_PLANE;
          uint64_t da[NP], db[NP];
#pragma unroll
          for (int pl = 0; pl < NP; ++pl) {
            da[pl] = sdesc(smem_u32(sA + pl * aplane), lbo_a, sbo);
            db[pl] = sdesc(smem_u32(sB + pl * WS_B_PLANE), lbo_b, sbo);
          }
          for (int k16 = 0; k16 < kc / 16; ++k16) {
            const bool first = (ch == 0 && k16 == 0);
            // products d_i e_(L-i) in rounds over i, so that consecutive MMAs
            // accumulate into different levels (no read-after-write on one
            // accumulator between neighbours); each level's first MMA (i = 0)
            // comes in round 0
#pragma unroll
            for (int i = 0; i < NP; ++i) {
#pragma unroll
              for (int L = i; L < NP; ++L) {
                // issuer 0: levels {0, 3} (4 planes) or {0, 1} (3 planes)
                if ((NP == 4 ? (L == 0 || L == 3) : L < 2) != (mw == 0)) continue;
                const uint32_t accum = (first && i == 0) ? 0u : 1u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tacc + (uint32_t)(L * FX_NT)),
                    "l"(da[i] + (uint64_t)(k16 * 256)), "l"(db[L - i] + (uint64_t)(k16 * 128)), "r"(IDESC_FX),
                    "r"(accum));
              }
            }
          }
          mma_commit(smem_u32(&empty[s]));  // the stage is free once these MMAs have read it
        }
        if (!ok) {
          *fail = 3;
          break;
        }
        mma_commit(smem_u32(&tfull[b]));
      }
      // every MMA this thread issued has completed once "drain" arrives
      mma_commit(smem_u32(&drain[mw]));
      if (!mbar_wait(smem_u32(&drain[mw]), 0, wait_ns)) *fail = 4;
    }
  } else {
    // ---------------- epilogue ----------------
    const int q = warp & 3;                     // the TMEM lane quarter this warp may access
    const int cbase = 32 * ((warp - WS_EPI0) / 4);  // its 32 of the 64 columns
    const int row = q * 32 + lane;
    const int m = mt * 128 + row;
    const bool mrow = m < plan.mvalid;
    const int fm = mrow ? aexp[m] : 0;
    uint32_t tc = 0;
    for (long j = j0; j < njobs; j += jstep, ++tc) {
      // decisions stay warp-uniform: tcgen05.ld needs the whole warp
      if (__shfl_sync(0xffffffffu, *fail, 0)) break;
      const uint32_t b = tc & 1u, tph = (tc >> 1) & 1u;
      const int f = (int)(j / plan.ntiles), nt = (int)(j % plan.ntiles);
      // column exponents of this warp's 32 columns, one per lane (loaded
      // before the wait for the accumulators, so the load's latency overlaps it)
      const int ecl = bexp[(size_t)f * plan.bexp_stride() + (size_t)nt * FX_NT + cbase + lane];
      if (!__all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull[b]), tph, wait_ns))) {
        if (lane == 0) *fail = 5;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      OutT* out = outs.p[f];
#pragma unroll
      for (int g2 = 0; g2 < 2; ++g2) {
        const int c0 = cbase + 16 * g2;
        uint32_t r[NP][16];
#pragma unroll
        for (int L = 0; L < NP; ++L) {
          const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + b * SET_COLS + (uint32_t)(L * FX_NT + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
              "[%16];"
              : "=r"(r[L][0]), "=r"(r[L][1]), "=r"(r[L][2]), "=r"(r[L][3]), "=r"(r[L][4]), "=r"(r[L][5]),
                "=r"(r[L][6]), "=r"(r[L][7]), "=r"(r[L][8]), "=r"(r[L][9]), "=r"(r[L][10]), "=r"(r[L][11]),
                "=r"(r[L][12]), "=r"(r[L][13]), "=r"(r[L][14]), "=r"(r[L][15])
              : "r"(taddr));
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        if (g2 == 1) {  // this warp's part of the set is in registers: release it
          asm volatile("tcgen05.fence::before_thread_sync;");
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
        }
        int ec[16];
#pragma unroll
        for (int qq = 0; qq < 16; ++qq) ec[qq] = __shfl_sync(0xffffffffu, ecl, 16 * g2 + qq);
        if (mrow) {
          const size_t col = (size_t)nt * FX_NT + c0;
          OutT* dst = out + (size_t)m * ldc + col;
          OutT v[16];
#pragma unroll
          for (int qq = 0; qq < 16; ++qq) {
            uint32_t acc[NP];
#pragma unroll
            for (int L = 0; L < NP; ++L) acc[L] = r[L][qq];
            v[qq] = fx_out<OutT, NP>(acc, fm + ec[qq] - fx_shift<NP>());
          }
          // a thread's 16 outputs are consecutive in its row: 16-byte stores
          // when the group is whole and aligned, element stores otherwise
          if (col + 16 <= (size_t)plan.ncols && (reinterpret_cast<uintptr_t>(dst) & 15u) == 0) {
            uint4* d4 = reinterpret_cast<uint4*>(dst);
            const uint4* v4 = reinterpret_cast<const uint4*>(v);
#pragma unroll
            for (int k = 0; k < (int)(16 * sizeof(OutT) / 16); ++k) d4[k] = v4[k];
          } else {
#pragma unroll
            for (int qq = 0; qq < 16; ++qq)
              if (col + qq < (size_t)plan.ncols) dst[qq] = v[qq];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (tid == 0 && s_fail) atomicExch(status, 10 + s_fail);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(WS_TMEM_COLS));
}

// ---------------------------------------------------------------------------
// Split a field [K rows][ncols] (rows >= kvalid are zero) into NP digit
// planes and write the K-major 64-column tile images plus the column
// exponents.  grid (2 ntiles, 1, nfields): a CTA takes 32 columns (half a B
// tile) with one warp per slot q = 0 .. Q-1 (blockDim 32 Q); warp q takes
// the 8-row groups q, q + Q, ... of the 32 columns (one coalesced row
// segment per load).  Q = ceil(groups / SG) keeps every thread's rows in
// registers as FP32 (SG = 2 groups for FP64 input, 3 for FP32: all loads in
// flight at once) between the column maximum and the digits; columns longer
// than 32 SG groups re-read the rest.  The column's largest |value|
// (max < 2^e_c) is combined in shared memory; the digits of 8 rows go out as
// one 16-byte store per plane, consecutive columns filling consecutive
// core-matrix rows.
// ---------------------------------------------------------------------------
constexpr int SP_COLS = 32;  // columns per CTA
template <typename InT>
struct SplitGroups {
  static constexpr int value = sizeof(InT) == 8 ? 2 : 3;  // 8-row groups per thread in registers
};

// FP64 inputs are rounded to FP32 (to nearest even) by integer operations:
// the FP64 pipe, which would execute the conversions, retires about 2 per
// clock per SM
__device__ __forceinline__ float to_f32(float x) { return x; }
__device__ __forceinline__ float to_f32(double x) { return bits::narrow_rn(x); }

// digits of the 8 rows of group g of one column (exponent e, position r in
// its 64-column tile): the tile image stores and, with a tail, the row's
// level sums
template <int NP>
__device__ __forceinline__ void split_group(const FxPlan& plan, uint8_t* __restrict__ tile, int r, int g,
                                            const float* v, int e, const FxTail& tail, float* lev, bool live) {
  uint16_t h[NP][8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    float dg[FX_PLANES];
    fx_digits_np<NP>(v[u], e, dg);
#pragma unroll
    for (int i = 0; i < NP; ++i) h[i][u] = bf16_bits(dg[i]);
    if (NP == 4 && tail.adig) fx_tail_mac(tail.adig, plan.kpad, 8 * g + u, dg, lev);
  }
  if (!live) return;
  const int ch = (8 * g) / TC_KC;
  const int kl = 8 * g - ch * TC_KC;
  const uint32_t pbytes = (uint32_t)FX_NT * plan.kc[ch] * 2u;
  uint8_t* base = tile + plan.b_chunk_off[ch];
  // core matrix (column group r / 8, k group kl / 8) of a 64-column tile
  const size_t off = ((size_t)(kl / 8) * (FX_NT / 8) + r / 8) * 128 + (r % 8) * 16;
#pragma unroll
  for (int pl = 0; pl < NP; ++pl) {
    uint4 w;
    w.x = (uint32_t)h[pl][0] | ((uint32_t)h[pl][1] << 16);
    w.y = (uint32_t)h[pl][2] | ((uint32_t)h[pl][3] << 16);
    w.z = (uint32_t)h[pl][4] | ((uint32_t)h[pl][5] << 16);
    w.w = (uint32_t)h[pl][6] | ((uint32_t)h[pl][7] << 16);
    *reinterpret_cast<uint4*>(base + (size_t)pl * pbytes + off) = w;
  }
}

// tail (optional): one more output row that the GEMM's plan leaves out,
// computed exactly as the GEMM would (the row's digit planes tail.adig, its
// exponent tail.aexp; levels i + j <= 3 summed exactly in FP32 -- the
// threads' partial sums and their total are integers below 2^24, so adding
// them in shared memory is exact in any order -- combined in 64 bits),
// written as FP64 to tail.out.p[f][col].  Tails are for 4-plane plans.
template <typename InT, int NP>
__global__ void __launch_bounds__(1024) k_tc_split_fx(const __grid_constant__ FxPlan plan,
                                                      const __grid_constant__ Ptr8<const InT> ins, int kvalid,
                                                      uint8_t* __restrict__ bimg, int* __restrict__ bexp,
                                                      const __grid_constant__ FxTail tail) {
  constexpr int SG = SplitGroups<InT>::value;
  __shared__ int s_max[SP_COLS];  // column maxima as float bits (non-negative floats order as integers)
  __shared__ float s_lev[FX_PLANES][SP_COLS];
  const int f = blockIdx.z;
  const int lane = threadIdx.x & 31, q = threadIdx.x >> 5, Q = blockDim.x >> 5;
  const InT* in = ins.p[f];
  const long col = (long)blockIdx.x * SP_COLS + lane;
  const int nt = blockIdx.x >> 1, r = (blockIdx.x & 1) * SP_COLS + lane;  // tile, column in the tile
  const bool live = col < plan.ncols;
  const int ng = plan.kpad / 8;
  if (threadIdx.x < SP_COLS) {
    s_max[threadIdx.x] = 0;
#pragma unroll
    for (int i = 0; i < FX_PLANES; ++i) s_lev[i][threadIdx.x] = 0.f;
  }
  // all of a thread's loads first, then their FP32 values
  InT raw[SG][8];
#pragma unroll
  for (int j = 0; j < SG; ++j) {
    const int g = q + Q * j;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = 8 * g + u;
      raw[j][u] = (live && g < ng && k < kvalid) ? in[(size_t)k * plan.ncols + col] : (InT)0;
    }
  }
  float x[SG][8];
  float mx = 0.f;
#pragma unroll
  for (int j = 0; j < SG; ++j)
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      x[j][u] = to_f32(raw[j][u]);
      mx = fmaxf(mx, fabsf(x[j][u]));
    }
  for (int g = q + Q * SG; g < ng; g += Q)
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = 8 * g + u;
      if (live && k < kvalid) mx = fmaxf(mx, fabsf(to_f32(in[(size_t)k * plan.ncols + col])));
    }
  __syncthreads();
  atomicMax(&s_max[lane], __float_as_int(mx));
  __syncthreads();
  int e = 0;
  const float cm = __int_as_float(s_max[lane]);
  if (cm > 0.f) (void)frexpf(cm, &e);  // cm = m 2^e, m in [0.5, 1)
  if (q == 0) bexp[(size_t)f * plan.bexp_stride() + col] = e;
  uint8_t* tile = bimg + (size_t)f * plan.b_field_bytes() + (size_t)nt * plan.b_tile_bytes;
  float lev[FX_PLANES] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int j = 0; j < SG; ++j) {
    const int g = q + Q * j;
    if (g < ng) split_group<NP>(plan, tile, r, g, x[j], e, tail, lev, live);
  }
  for (int g = q + Q * SG; g < ng; g += Q) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = 8 * g + u;
      v[u] = (live && k < kvalid) ? to_f32(in[(size_t)k * plan.ncols + col]) : 0.f;
    }
    split_group<NP>(plan, tile, r, g, v, e, tail, lev, live);
  }
  if (NP == 4 && tail.adig) {
#pragma unroll
    for (int i = 0; i < FX_PLANES; ++i) atomicAdd(&s_lev[i][lane], lev[i]);
    __syncthreads();
    if (q == 0 && live) {
      const float tot[FX_PLANES] = {s_lev[0][lane], s_lev[1][lane], s_lev[2][lane], s_lev[3][lane]};
      tail.out.p[f][col] = fx_tail_value(tot, tail.aexp + e - 35);
    }
  }
}

FxPlan make_fx_plan(int mvalid, int kvalid, long ncols, int planes) {
  FxPlan p{};
  p.planes = planes;
  p.mvalid = mvalid;
  p.mtiles = (mvalid + 127) / 128;
  p.kpad = (kvalid + 15) / 16 * 16;
  p.ncols = ncols;
  p.ntiles = (int)((ncols + FX_NT - 1) / FX_NT);
  p.nchunks = (p.kpad + TC_KC - 1) / TC_KC;
  size_t oa = 0, ob = 0;
  for (int c = 0; c < p.nchunks; ++c) {
    p.kc[c] = std::min(TC_KC, p.kpad - c * TC_KC);
    p.a_chunk_off[c] = oa;
    p.b_chunk_off[c] = ob;
    oa += (size_t)p.planes * 128 * p.kc[c] * 2;
    ob += (size_t)p.planes * FX_NT * p.kc[c] * 2;
  }
  p.a_tile_bytes = oa;
  p.b_tile_bytes = ob;
  return p;
}

// Host: the A image of a dense row-major M x K double matrix, and its row
// exponents (max |A[m][.]| < 2^row_exp[m]; 0 for zero and padding rows).
std::vector<uint8_t> make_a_image_fx(const FxPlan& p, const std::vector<double>& a, int M, int K,
                                     std::vector<int>& row_exp) {
  std::vector<uint8_t> img((size_t)p.mtiles * p.a_tile_bytes, 0);
  row_exp.assign((size_t)p.mtiles * 128, 0);
  for (int m = 0; m < M; ++m) {
    double mx = 0.0;
    for (int k = 0; k < K; ++k) mx = std::max(mx, std::fabs(a[(size_t)m * K + k]));
    int e = 0;
    if (mx > 0) (void)std::frexp(mx, &e);
    row_exp[m] = e;
  }
  for (int m = 0; m < p.mtiles * 128; ++m)
    for (int k = 0; k < p.kpad; ++k) {
      const double x = (m < M && k < K) ? a[(size_t)m * K + k] : 0.0;
      double dg[FX_PLANES];
      fx_digits_host(x, row_exp[m], dg, p.planes);
      const int mt = m / 128, r = m % 128, ch = k / TC_KC, kl = k - ch * TC_KC;
      const size_t pbytes = (size_t)128 * p.kc[ch] * 2;
      const size_t off = (size_t)mt * p.a_tile_bytes + p.a_chunk_off[ch] +
                         ((size_t)(kl / 8) * 16 + r / 8) * 128 + (r % 8) * 16 + (kl % 8) * 2;
      for (int pl = 0; pl < p.planes; ++pl) {
        // digits are integers with |d| <= 256: their bf16 pattern is the top
        // half of the float's
        const float fd = (float)dg[pl];
        uint32_t w;
        std::memcpy(&w, &fd, 4);
        const uint16_t b = (uint16_t)(w >> 16);
        std::memcpy(&img[off + pl * pbytes], &b, 2);
      }
    }
  return img;
}

// Host: the digit planes (plane-major, kpad each) and exponent of row `row` of a
// dense row-major M x K double matrix, as make_a_image_fx would cut it.
std::vector<float> a_row_digits(const FxPlan& p, const std::vector<double>& a, int K, int row, int& row_exp) {
  double mx = 0.0;
  for (int k = 0; k < K; ++k) mx = std::max(mx, std::fabs(a[(size_t)row * K + k]));
  row_exp = 0;
  if (mx > 0) (void)std::frexp(mx, &row_exp);
  std::vector<float> dig((size_t)FX_PLANES * p.kpad, 0.f);
  for (int k = 0; k < K; ++k) {
    double dg[FX_PLANES];
    fx_digits_host(a[(size_t)row * K + k], row_exp, dg, FX_PLANES);
    for (int i = 0; i < FX_PLANES; ++i) dig[(size_t)i * p.kpad + k] = (float)dg[i];
  }
  return dig;
}

template <typename OutT>
int launch_tc_gemm_fx(Handle* h, const FxPlan& p, const uint8_t* aimg, const int* aexp, const uint8_t* bimg,
                      const int* bexp, const Ptr8<OutT>& outs, int nfields, size_t ldc, int kid) {
  // exactness of a level's FP32 sum, the largest level's products per k times
  // kpad below 2^24: 4 planes (2 * 128 * 64 + 2 * 64 * 64) * kpad, 3 planes
  // (2 * 256 * 128 + 128 * 128) * kpad
  if ((p.planes == 4 && p.kpad > 680) || (p.planes == 3 && p.kpad > 204) || (p.planes != 3 && p.planes != 4)) {
    h->err = "k_tc_gemm_fx: K is too long for exact sums";
    return CHF_E_INVALID;
  }
  if (p.planes == 3 && sizeof(OutT) != 4) {
    h->err = "k_tc_gemm_fx: 3-plane digits are for FP32 outputs";
    return CHF_E_INVALID;
  }
  auto kern = p.planes == 4 ? k_tc_gemm_fx<OutT, 4> : k_tc_gemm_fx<OutT, 3>;
  const size_t smem = ws_resident(p) ? ws_a_resident_bytes(p) + (size_t)WS_STAGES * ws_b_stage(p.planes)
                                     : (size_t)WS_STAGES * ws_ab_stage(p.planes);
  if (!cuda_ok(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "k_tc_gemm_fx smem"))
    return CHF_E_CUDA;
  // whole multiples of the row tiles, each CTA on one row tile
  const long items = (long)nfields * p.ntiles * p.mtiles;
  const int grid = (int)(std::min<long>(items, (long)std::max(h->num_sms, p.mtiles)) / p.mtiles * p.mtiles);
  cudaEvent_t ev;
  prof_begin(h, kid, &ev);
  // the bounded-wait test (chf_test_wait_timeout) applies to one launch
  const long wait_ns = h->test_skip ? h->test_wait_ns : tc::WAIT_NS;
  const int skip = h->test_skip;
  h->test_skip = 0;
  kern<<<grid, WS_THREADS, smem, h->stream>>>(p, aimg, aexp, bimg, bexp, outs, ldc, nfields, h->dev_status,
                                              wait_ns, skip);
  prof_end(h, kid, ev);
  return cuda_ok(h, cudaGetLastError(), "k_tc_gemm_fx") ? CHF_OK : CHF_E_CUDA;
}

template <typename InT>
int launch_tc_split_fx(Handle* h, const FxPlan& p, const Ptr8<const InT>& ins, int kvalid, uint8_t* bimg,
                       int* bexp, int nfields, int kid, const FxTail& tail) {
  if (tail.adig && p.planes != 4) {
    h->err = "k_tc_split_fx: row tails need 4-plane digits";
    return CHF_E_INVALID;
  }
  // warps per CTA: enough that each thread's groups fit in registers, at
  // most 32 (longer columns re-read their remaining groups)
  const int ng = p.kpad / 8, sg = SplitGroups<InT>::value;
  const int nq = std::min(32, (ng + sg - 1) / sg);
  dim3 grid(2 * p.ntiles, 1, nfields);
  cudaEvent_t ev;
  prof_begin(h, kid, &ev);
  if (p.planes == 4)
    k_tc_split_fx<InT, 4><<<grid, 32 * nq, 0, h->stream>>>(p, ins, kvalid, bimg, bexp, tail);
  else
    k_tc_split_fx<InT, 3><<<grid, 32 * nq, 0, h->stream>>>(p, ins, kvalid, bimg, bexp, tail);
  prof_end(h, kid, ev);
  return cuda_ok(h, cudaGetLastError(), "k_tc_split_fx") ? CHF_OK : CHF_E_CUDA;
}

template int launch_tc_gemm_fx<float>(Handle*, const FxPlan&, const uint8_t*, const int*, const uint8_t*,
                                      const int*, const Ptr8<float>&, int, size_t, int);
template int launch_tc_gemm_fx<double>(Handle*, const FxPlan&, const uint8_t*, const int*, const uint8_t*,
                                       const int*, const Ptr8<double>&, int, size_t, int);
template int launch_tc_split_fx<float>(Handle*, const FxPlan&, const Ptr8<const float>&, int, uint8_t*, int*,
                                       int, int, const FxTail&);
template int launch_tc_split_fx<double>(Handle*, const FxPlan&, const Ptr8<const double>&, int, uint8_t*,
                                        int*, int, int, const FxTail&);

}  // namespace chf
