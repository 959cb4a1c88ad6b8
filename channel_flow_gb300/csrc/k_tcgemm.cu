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
// 2^-e_c (powers of two, so exactly) into (-1, 1), then written as
// FX_PLANES digits of 7 bits:
//     x = sum_i d_i 2^(-7 (i + 1)),   d_0 in [-128, 128], d_i in [-64, 64]
// (each digit is rint of the scaled remainder, so all steps are exact).
// Digits are integers of at most 8 bits, exact in bf16.  The products of
// one level L = i + j (at most four planes pairs) summed over K <= 680 stay
// integers below 2^24, so tensor-core FP32 accumulation of a level is EXACT
// (the launcher checks K).  B data are taken as FP32 (FP64 coefficients are
// rounded to FP32 first: a relative error per coefficient, not a flat floor).  Levels
// 0..3 (ten products) go to four TMEM accumulators; the epilogue forms
//     C = 2^(f_m + e_c - 14) * sum_L 2^(-7 L) acc_L
// exactly: the four levels combine into one 64-bit integer
//     t = acc_0 2^21 + acc_1 2^14 + acc_2 2^7 + acc_3,   |t| < 2^46,
// converted once (exactly to FP64, correctly rounded to FP32) and scaled by
// 2^(f_m + e_c - 35).  What is dropped -- levels >= 4 and the digit
// remainders -- is below 2^-28 of max|A row| * max|B column| per term,
// instead of 2^-24 of each running FP32 sum.
//
// Operand images: each 128-row tile of A and each 64-column tile of B is
// stored in HBM already in the shared-memory "core matrix" layout that
// tcgen05.mma reads with a no-swizzle K-major descriptor (8 rows x 16 bytes
// per core matrix; core (g = row/8, c = k/8) at (c * G + g) * 128 bytes with
// G = 16 for A and 8 for B).  K is cut into chunks of TC_KC; every (tile,
// chunk, plane) image is one contiguous block moved by one cp.async.bulk,
// completion signalled on an mbarrier.  One thread issues the MMAs and
// tcgen05.commit arrives on a second mbarrier; four warps read the
// accumulators back with tcgen05.ld.  Every wait is bounded (1 s of wall
// time); on timeout the kernel records an error code, stops issuing work,
// waits (bounded) for the MMAs it issued and frees its tensor memory.  The
// four accumulators take 4 x 64 TMEM columns and the operands 96 KB of
// shared memory, so two CTAs share an SM and one's copies overlap the
// other's MMAs and epilogue.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "chf_internal.h"
#include "tc_dev.cuh"

namespace chf {

namespace {

using namespace tc;

constexpr int FX_LEVELS = 4;  // products d_i e_j with i + j <= 3
constexpr uint32_t FX_TMEM_COLS = (uint32_t)FX_NT * FX_LEVELS;

// FX_PLANES digits of x * 2^-e on the host (exact in double)
void fx_digits_host(double x, int e, double* dg) {
  double y = std::scalbn(x, 7 - e);
  for (int i = 0; i < FX_PLANES; ++i) {
    const double di = std::rint(y);
    dg[i] = di;
    y = (y - di) * 128.0;
  }
}


}  // namespace

// ---------------------------------------------------------------------------
// GEMM.  grid (ntiles, mtiles, nfields), 128 threads, dynamic shared memory
// FX_PLANES planes of 128 x TC_KC (A) and of 64 x TC_KC (B) bf16.
// ---------------------------------------------------------------------------
// instruction descriptor: D = F32, A = B = BF16, both K-major, M = 128, N = 64
constexpr uint32_t IDESC_FX = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

template <typename OutT>
__device__ __forceinline__ void store_fx(OutT* p, long long t, int n);
// t 2^n, correctly rounded to FP32 (n in the normal exponent range)
template <>
__device__ __forceinline__ void store_fx<float>(float* p, long long t, int n) {
  const float v = __ll2float_rn(t);
  const int h = n / 2;  // two exact power-of-two factors keep each in range
  *p = v * __int_as_float((127 + h) << 23) * __int_as_float((127 + n - h) << 23);
}
// t 2^n exactly in FP64 (|t| < 2^46)
template <>
__device__ __forceinline__ void store_fx<double>(double* p, long long t, int n) {
  *p = (double)t * __longlong_as_double((long long)(1023 + n) << 52);
}

template <typename OutT>
__global__ void __launch_bounds__(TC_THREADS) k_tc_gemm_fx(const __grid_constant__ FxPlan plan,
                                                           const uint8_t* __restrict__ aimg,
                                                           const int* __restrict__ aexp,
                                                           const uint8_t* __restrict__ bimg,
                                                           const int* __restrict__ bexp,
                                                           const __grid_constant__ Ptr8<OutT> outs,
                                                           size_t ldc, int* status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nt = blockIdx.x, mt = blockIdx.y, f = blockIdx.z;
  constexpr int NP = FX_PLANES;
  constexpr uint32_t a_plane_max = 128u * TC_KC * 2u;
  constexpr uint32_t b_plane_max = (uint32_t)FX_NT * TC_KC * 2u;
  uint8_t* sA = smem;
  uint8_t* sB = smem + NP * a_plane_max;
  if (tid == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_load)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_mma)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(FX_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint8_t* atile = aimg + (size_t)mt * plan.a_tile_bytes;
  const uint8_t* btile = bimg + (size_t)f * plan.b_field_bytes() + (size_t)nt * plan.b_tile_bytes;
  for (int ch = 0; ch < plan.nchunks; ++ch) {
    const int kc = plan.kc[ch];
    const uint32_t apb = 128u * kc * 2u, bpb = (uint32_t)FX_NT * kc * 2u;
    if (tid == 0 && !s_fail) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar_load)),
                   "r"(NP * (apb + bpb))
                   : "memory");
      for (int pl = 0; pl < NP; ++pl) {
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(sA + pl * a_plane_max)),
            "l"(atile + plan.a_chunk_off[ch] + (size_t)pl * apb), "r"(apb), "r"(smem_u32(&bar_load))
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(sB + pl * b_plane_max)),
            "l"(btile + plan.b_chunk_off[ch] + (size_t)pl * bpb), "r"(bpb), "r"(smem_u32(&bar_load))
            : "memory");
      }
      if (!mbar_wait(smem_u32(&bar_load), ch & 1)) {
        s_fail = 1;
      } else {
        // K-adjacent core matrices: 16 (A, 128 rows) or 8 (B, 64 columns)
        // groups of 8 rows x 16 bytes apart; adjacent 8-row groups 128 B apart
        const uint32_t lbo_a = 16u * 128u, lbo_b = 8u * 128u, sbo = 128u;
        for (int s = 0; s < kc / 16; ++s) {
#pragma unroll
          for (int L = 0; L < FX_LEVELS; ++L) {
#pragma unroll
            for (int i = 0; i <= L; ++i) {
              const int j = L - i;
              uint64_t da = sdesc(smem_u32(sA + i * a_plane_max) + s * 2 * lbo_a, lbo_a, sbo);
              uint64_t db = sdesc(smem_u32(sB + j * b_plane_max) + s * 2 * lbo_b, lbo_b, sbo);
              uint32_t acc = (ch > 0 || s > 0 || i > 0) ? 1u : 0u;
              asm volatile(
                  "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(
                      tmem + (uint32_t)(L * FX_NT)),
                  "l"(da), "l"(db), "r"(IDESC_FX), "r"(acc));
            }
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&bar_mma))
            : "memory");
        // the next chunk overwrites the operands: wait until the MMAs read them
        if (!mbar_wait(smem_u32(&bar_mma), ch & 1)) s_fail = 2;
      }
    }
    __syncthreads();
    if (s_fail) break;
  }
  const bool ok = !s_fail;
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    const int row = warp * 32 + (tid & 31);
    const int m = mt * 128 + row;
    const bool mrow = m < plan.mvalid;
    const int fm = mrow ? aexp[m] : 0;
    OutT* out = outs.p[f];
    const int* ecol = bexp + (size_t)f * plan.bexp_stride() + (size_t)nt * FX_NT;
    for (int c0 = 0; c0 < FX_NT; c0 += 16) {
      uint32_t r[FX_LEVELS][16];
#pragma unroll
      for (int L = 0; L < FX_LEVELS; ++L) {
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(L * FX_NT + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];"
            : "=r"(r[L][0]), "=r"(r[L][1]), "=r"(r[L][2]), "=r"(r[L][3]), "=r"(r[L][4]), "=r"(r[L][5]),
              "=r"(r[L][6]), "=r"(r[L][7]), "=r"(r[L][8]), "=r"(r[L][9]), "=r"(r[L][10]), "=r"(r[L][11]),
              "=r"(r[L][12]), "=r"(r[L][13]), "=r"(r[L][14]), "=r"(r[L][15])
            : "r"(taddr));
      }
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (mrow) {
        const size_t col = (size_t)nt * FX_NT + c0;
        OutT* dst = out + (size_t)m * ldc + col;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          if (col + q < (size_t)plan.ncols) {
            // each level holds an integer below 2^24 exactly
            const long long t = ((long long)__float2int_rn(__uint_as_float(r[0][q])) << 21) +
                                ((long long)__float2int_rn(__uint_as_float(r[1][q])) << 14) +
                                ((long long)__float2int_rn(__uint_as_float(r[2][q])) << 7) +
                                (long long)__float2int_rn(__uint_as_float(r[3][q]));
            store_fx(dst + q, t, fm + ecol[c0 + q] - 35);
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(status, s_fail == 1 ? 11 : 12);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(FX_TMEM_COLS));
}

// ---------------------------------------------------------------------------
// Split a field [K rows][ncols] (rows >= kvalid are zero) into FX_PLANES digit
// planes and write the K-major 64-column tile images plus the column
// exponents.  One thread per column: pass 1 finds the column's largest
// |value| (its exponent e_c: max < 2^e_c), pass 2 writes the digits of 8 rows
// at a time as one 16-byte store per plane (consecutive threads fill
// consecutive core-matrix rows).  grid (ntiles, 1, nfields), FX_NT threads.
// ---------------------------------------------------------------------------
template <typename InT>
__global__ void __launch_bounds__(FX_NT) k_tc_split_fx(const __grid_constant__ FxPlan plan,
                                                       const __grid_constant__ Ptr8<const InT> ins, int kvalid,
                                                       uint8_t* __restrict__ bimg, int* __restrict__ bexp) {
  const int nt = blockIdx.x, f = blockIdx.z, r = threadIdx.x;
  const InT* in = ins.p[f];
  const long col = (long)nt * FX_NT + r;
  const bool live = col < plan.ncols;
  float mx = 0.f;
  if (live)
    for (int k = 0; k < kvalid; ++k) mx = fmaxf(mx, fabsf((float)in[(size_t)k * plan.ncols + col]));
  int e = 0;
  if (mx > 0.f) (void)frexpf(mx, &e);  // mx = m 2^e, m in [0.5, 1)
  bexp[(size_t)f * plan.bexp_stride() + col] = e;
  uint8_t* tile = bimg + (size_t)f * plan.b_field_bytes() + (size_t)nt * plan.b_tile_bytes;
  for (int g = 0; g < plan.kpad / 8; ++g) {
    uint16_t h[FX_PLANES][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = 8 * g + q;
      const float x = (live && k < kvalid) ? (float)in[(size_t)k * plan.ncols + col] : 0.f;
      float dg[FX_PLANES];
      fx_digits_f(x, e, dg);
#pragma unroll
      for (int i = 0; i < FX_PLANES; ++i) h[i][q] = bf16_bits(dg[i]);
    }
    const int ch = (8 * g) / TC_KC;
    const int kl = 8 * g - ch * TC_KC;
    const uint32_t pbytes = (uint32_t)FX_NT * plan.kc[ch] * 2u;
    uint8_t* base = tile + plan.b_chunk_off[ch];
    // core matrix (column group r / 8, k group kl / 8) of a 64-column tile
    const size_t off = ((size_t)(kl / 8) * (FX_NT / 8) + r / 8) * 128 + (r % 8) * 16;
#pragma unroll
    for (int pl = 0; pl < FX_PLANES; ++pl) {
      uint4 v;
      v.x = (uint32_t)h[pl][0] | ((uint32_t)h[pl][1] << 16);
      v.y = (uint32_t)h[pl][2] | ((uint32_t)h[pl][3] << 16);
      v.z = (uint32_t)h[pl][4] | ((uint32_t)h[pl][5] << 16);
      v.w = (uint32_t)h[pl][6] | ((uint32_t)h[pl][7] << 16);
      *reinterpret_cast<uint4*>(base + (size_t)pl * pbytes + off) = v;
    }
  }
}

FxPlan make_fx_plan(int mvalid, int kvalid, long ncols) {
  FxPlan p{};
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
    oa += (size_t)FX_PLANES * 128 * p.kc[c] * 2;
    ob += (size_t)FX_PLANES * FX_NT * p.kc[c] * 2;
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
      fx_digits_host(x, row_exp[m], dg);
      const int mt = m / 128, r = m % 128, ch = k / TC_KC, kl = k - ch * TC_KC;
      const size_t pbytes = (size_t)128 * p.kc[ch] * 2;
      const size_t off = (size_t)mt * p.a_tile_bytes + p.a_chunk_off[ch] +
                         ((size_t)(kl / 8) * 16 + r / 8) * 128 + (r % 8) * 16 + (kl % 8) * 2;
      for (int pl = 0; pl < FX_PLANES; ++pl) {
        // digits are integers with |d| <= 128: their bf16 pattern is the top
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

template <typename OutT>
int launch_tc_gemm_fx(Handle* h, const FxPlan& p, const uint8_t* aimg, const int* aexp, const uint8_t* bimg,
                      const int* bexp, const Ptr8<OutT>& outs, int nfields, size_t ldc, int kid) {
  // exactness of a level's FP32 sum: (2 * 128 * 64 + 2 * 64 * 64) * kpad < 2^24
  if (p.kpad > 680) {
    h->err = "k_tc_gemm_fx: K is too long for exact sums";
    return CHF_E_INVALID;
  }
  const size_t smem = (size_t)FX_PLANES * (128 + FX_NT) * TC_KC * 2;
  if (!cuda_ok(h, cudaFuncSetAttribute(k_tc_gemm_fx<OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem),
               "k_tc_gemm_fx smem"))
    return CHF_E_CUDA;
  dim3 grid(p.ntiles, p.mtiles, nfields);
  cudaEvent_t ev;
  prof_begin(h, kid, &ev);
  k_tc_gemm_fx<OutT><<<grid, TC_THREADS, smem, h->stream>>>(p, aimg, aexp, bimg, bexp, outs, ldc, h->dev_status);
  prof_end(h, kid, ev);
  return cuda_ok(h, cudaGetLastError(), "k_tc_gemm_fx") ? CHF_OK : CHF_E_CUDA;
}

template <typename InT>
int launch_tc_split_fx(Handle* h, const FxPlan& p, const Ptr8<const InT>& ins, int kvalid, uint8_t* bimg,
                       int* bexp, int nfields, int kid) {
  dim3 grid(p.ntiles, 1, nfields);
  cudaEvent_t ev;
  prof_begin(h, kid, &ev);
  k_tc_split_fx<InT><<<grid, FX_NT, 0, h->stream>>>(p, ins, kvalid, bimg, bexp);
  prof_end(h, kid, ev);
  return cuda_ok(h, cudaGetLastError(), "k_tc_split_fx") ? CHF_OK : CHF_E_CUDA;
}

template int launch_tc_gemm_fx<float>(Handle*, const FxPlan&, const uint8_t*, const int*, const uint8_t*,
                                      const int*, const Ptr8<float>&, int, size_t, int);
template int launch_tc_gemm_fx<double>(Handle*, const FxPlan&, const uint8_t*, const int*, const uint8_t*,
                                       const int*, const Ptr8<double>&, int, size_t, int);
template int launch_tc_split_fx<float>(Handle*, const FxPlan&, const Ptr8<const float>&, int, uint8_t*, int*,
                                       int, int);
template int launch_tc_split_fx<double>(Handle*, const FxPlan&, const Ptr8<const double>&, int, uint8_t*,
                                        int*, int, int);

}  // namespace chf
