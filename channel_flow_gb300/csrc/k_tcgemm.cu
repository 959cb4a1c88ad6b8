// k_tcgemm.cu -- wall-normal Chebyshev transforms of the mixed-precision path
// as tcgen05 tensor-core GEMMs (sm_103a).
//
//   C_f[m][col] = sum_k A[m][k] * B_f[k][col]          (f = field)
//
// A is a constant transform matrix (Chebyshev evaluation cos(pi n p / M),
// the Gauss-Lobatto DCT-I weights, ...), B_f the data of one field with the
// columns = (spectral mode, re/im) and rows = wall-normal index.  Both are
// split into three bf16 planes x = x0 + x1 + x2 (8 significant bits each,
// together exact to FP32) and the six products x_a y_b with a + b <= 2 are
// accumulated in FP32 in tensor memory; the dropped terms are below 2^-24
// relative.  Differentiating the result (the curl of the Lamb vector)
// amplifies value errors by ~100x, which is why a two-plane split (2^-17)
// is not enough.
//
// Operand images: each 128-row tile of A and each 128-column tile of B is
// stored in HBM already in the shared-memory "core matrix" layout that
// tcgen05.mma reads with a no-swizzle K-major descriptor (8 rows x 16 bytes
// per core matrix; core (g = row/8, c = k/8) at (c * 16 + g) * 128 bytes).
// The K dimension is cut into chunks of at most KC = 64; every
// (tile, chunk, plane) image is one contiguous block moved by a single
// cp.async.bulk into shared memory, completion signalled on an mbarrier.
// One thread issues the MMAs; tcgen05.commit arrives on a second mbarrier;
// four warps read the 128 x 128 FP32 accumulator back with tcgen05.ld.
// Every wait is bounded (1 s of wall time); on timeout the kernel records an
// error code, stops issuing work, waits (bounded) for the MMAs it issued and
// frees its tensor memory.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "chf_internal.h"

namespace chf {

namespace {

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

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
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
    if ((long)(gtimer() - t0) > WAIT_NS) return false;
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

template <typename OutT>
__device__ __forceinline__ void store_out(OutT* p, float v);
template <>
__device__ __forceinline__ void store_out<float>(float* p, float v) { *p = v; }
template <>
__device__ __forceinline__ void store_out<double>(double* p, float v) { *p = (double)v; }

}  // namespace

// ---------------------------------------------------------------------------
// GEMM kernel.  grid (ntiles, mtiles, nfields), 128 threads.
// ---------------------------------------------------------------------------
template <typename OutT>
__global__ void __launch_bounds__(TC_THREADS) k_tc_gemm(const __grid_constant__ TcPlan plan,
                                                        const uint8_t* __restrict__ aimg,
                                                        const uint8_t* __restrict__ bimg,
                                                        size_t bfield_stride,
                                                        const __grid_constant__ Ptr8<OutT> outs,
                                                        size_t ldc, int* status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nt = blockIdx.x, mt = blockIdx.y, f = blockIdx.z;
  const int NS = TC_SPLITS;
  const uint32_t plane_max = 128u * TC_KC * 2u;  // bytes of one plane image at full chunk
  uint8_t* sA = smem;                            // NS planes
  uint8_t* sB = smem + NS * plane_max;           // NS planes
  if (tid == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_load)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_mma)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
        smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint8_t* atile = aimg + (size_t)mt * plan.tile_bytes;
  const uint8_t* btile = bimg + (size_t)f * bfield_stride + (size_t)nt * plan.tile_bytes;
  bool issued = false;
  for (int ch = 0; ch < plan.nchunks; ++ch) {
    const int kc = plan.kc[ch];
    const uint32_t pbytes = 128u * kc * 2u;
    const size_t coff = plan.chunk_off[ch];
    if (tid == 0 && !s_fail) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar_load)),
                   "r"(2u * NS * pbytes)
                   : "memory");
      for (int pl = 0; pl < NS; ++pl) {
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(sA + pl * plane_max)),
            "l"(atile + coff + (size_t)pl * pbytes), "r"(pbytes), "r"(smem_u32(&bar_load))
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(sB + pl * plane_max)),
            "l"(btile + coff + (size_t)pl * pbytes), "r"(pbytes), "r"(smem_u32(&bar_load))
            : "memory");
      }
    }
    if (tid == 0 && !s_fail) {
      if (!mbar_wait(smem_u32(&bar_load), ch & 1)) {
        s_fail = 1;
      } else {
        const uint32_t lbo = 16u * 128u;  // K-adjacent core matrices (16 row groups of 128 B)
        const uint32_t sbo = 128u;        // adjacent 8-row groups
        for (int s = 0; s < kc / 16; ++s) {
          // products a + b <= 2, smallest first
          const int pa[6] = {2, 1, 0, 1, 0, 0};
          const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            uint64_t da = sdesc(smem_u32(sA + pa[q] * plane_max) + s * 2 * lbo, lbo, sbo);
            uint64_t db = sdesc(smem_u32(sB + pb[q] * plane_max) + s * 2 * lbo, lbo, sbo);
            uint32_t acc = (ch > 0 || s > 0 || q > 0) ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                "l"(da), "l"(db), "r"(IDESC), "r"(acc));
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&bar_mma))
            : "memory");
        issued = true;
        // the next chunk overwrites the operands: wait until the MMAs read them
        if (!mbar_wait(smem_u32(&bar_mma), ch & 1)) s_fail = 2;
      }
    }
    __syncthreads();
    if (s_fail) break;
  }
  (void)issued;
  const bool ok = !s_fail;
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    const int row = warp * 32 + (tid & 31);
    const int m = mt * 128 + row;
    OutT* out = outs.p[f];
    for (int c0 = 0; c0 < 128; c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
            "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
            "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
            "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (m < plan.mvalid) {
        const size_t col = (size_t)nt * 128 + c0;
        OutT* dst = out + (size_t)m * ldc + col;
#pragma unroll
        for (int q = 0; q < 32; ++q)
          if (col + q < (size_t)plan.ncols) store_out(dst + q, __uint_as_float(r[q]));
      }
    }
  } else if (tid == 0) {
    atomicExch(status, s_fail == 1 ? 11 : 12);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// Split a field [K rows][ncols] (row stride ncols, rows >= kvalid are zero)
// into three bf16 planes and write the K-major tile images.  Thread (r, g):
// column r of a 128-column tile, k-group g of 8 rows -> one 16-byte store per
// plane.  grid (ntiles, ceil(kgroups * 128 / 256), nfields), 256 threads.
// ---------------------------------------------------------------------------
template <typename InT>
__global__ void __launch_bounds__(256) k_tc_split(const __grid_constant__ TcPlan plan,
                                                  const __grid_constant__ Ptr8<const InT> ins, int kvalid,
                                                  uint8_t* __restrict__ bimg, size_t bfield_stride) {
  const int nt = blockIdx.x, f = blockIdx.z;
  const int t = blockIdx.y * blockDim.x + threadIdx.x;
  const int r = t % 128, g = t / 128;  // column in tile, 8-row group
  if (8 * g >= plan.kpad) return;
  const InT* in = ins.p[f];
  const long col = (long)nt * 128 + r;
  uint16_t h[3][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int k = 8 * g + q;
    float x = 0.f;
    if (k < kvalid && col < plan.ncols) x = (float)in[(size_t)k * plan.ncols + col];
    __nv_bfloat16 b0 = __float2bfloat16_rn(x);
    float r1 = x - __bfloat162float(b0);
    __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    float r2 = r1 - __bfloat162float(b1);
    __nv_bfloat16 b2 = __float2bfloat16_rn(r2);
    h[0][q] = __bfloat16_as_ushort(b0);
    h[1][q] = __bfloat16_as_ushort(b1);
    h[2][q] = __bfloat16_as_ushort(b2);
  }
  const int ch = (8 * g) / TC_KC;
  const int kl = 8 * g - ch * TC_KC;
  const uint32_t pbytes = 128u * plan.kc[ch] * 2u;
  uint8_t* base = bimg + (size_t)f * bfield_stride + (size_t)nt * plan.tile_bytes + plan.chunk_off[ch];
  const size_t off = ((size_t)(kl / 8) * 16 + r / 8) * 128 + (r % 8) * 16;
#pragma unroll
  for (int pl = 0; pl < 3; ++pl) {
    uint4 v;
    v.x = (uint32_t)h[pl][0] | ((uint32_t)h[pl][1] << 16);
    v.y = (uint32_t)h[pl][2] | ((uint32_t)h[pl][3] << 16);
    v.z = (uint32_t)h[pl][4] | ((uint32_t)h[pl][5] << 16);
    v.w = (uint32_t)h[pl][6] | ((uint32_t)h[pl][7] << 16);
    *reinterpret_cast<uint4*>(base + (size_t)pl * pbytes + off) = v;
  }
}

TcPlan make_tc_plan(int mvalid, int kvalid, long ncols) {
  TcPlan p{};
  p.mvalid = mvalid;
  p.mtiles = (mvalid + 127) / 128;
  p.kpad = (kvalid + 15) / 16 * 16;
  p.ncols = ncols;
  p.ntiles = (int)((ncols + 127) / 128);
  p.nchunks = (p.kpad + TC_KC - 1) / TC_KC;
  size_t off = 0;
  for (int c = 0; c < p.nchunks; ++c) {
    p.kc[c] = std::min(TC_KC, p.kpad - c * TC_KC);
    p.chunk_off[c] = off;
    off += (size_t)TC_SPLITS * 128 * p.kc[c] * 2;
  }
  p.tile_bytes = off;
  return p;
}

// Host: split a dense row-major M x K double matrix into the A image.
std::vector<uint8_t> make_a_image(const TcPlan& p, const std::vector<double>& a, int M, int K) {
  std::vector<uint8_t> img((size_t)p.mtiles * p.tile_bytes, 0);
  auto bf = [](float f) -> uint16_t {
    __nv_bfloat16 b = __float2bfloat16_rn(f);
    return __bfloat16_as_ushort(b);
  };
  auto fb = [](uint16_t u) -> double {
    uint32_t w = (uint32_t)u << 16;
    float f;
    memcpy(&f, &w, 4);
    return (double)f;
  };
  for (int m = 0; m < p.mtiles * 128; ++m)
    for (int k = 0; k < p.kpad; ++k) {
      double x = (m < M && k < K) ? a[(size_t)m * K + k] : 0.0;
      uint16_t h[3];
      double rest = x;
      for (int pl = 0; pl < 3; ++pl) {
        h[pl] = bf((float)rest);
        rest -= fb(h[pl]);
      }
      const int mt = m / 128, r = m % 128, ch = k / TC_KC, kl = k - ch * TC_KC;
      const size_t pbytes = (size_t)128 * p.kc[ch] * 2;
      size_t off = (size_t)mt * p.tile_bytes + p.chunk_off[ch] +
                   ((size_t)(kl / 8) * 16 + r / 8) * 128 + (r % 8) * 16 + (kl % 8) * 2;
      for (int pl = 0; pl < 3; ++pl) memcpy(&img[off + pl * pbytes], &h[pl], 2);
    }
  return img;
}

template <typename OutT>
int launch_tc_gemm(Handle* h, const TcPlan& p, const uint8_t* aimg, const uint8_t* bimg,
                   size_t bfield_stride, const Ptr8<OutT>& outs, int nfields, size_t ldc, int kid) {
  const size_t smem = (size_t)2 * TC_SPLITS * 128 * TC_KC * 2;
  if (!cuda_ok(h, cudaFuncSetAttribute(k_tc_gemm<OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem),
               "k_tc_gemm smem"))
    return CHF_E_CUDA;
  dim3 grid(p.ntiles, p.mtiles, nfields);
  cudaEvent_t ev;
  prof_begin(h, kid, &ev);
  k_tc_gemm<OutT><<<grid, TC_THREADS, smem, h->stream>>>(p, aimg, bimg, bfield_stride, outs, ldc,
                                                         h->dev_status);
  prof_end(h, kid, ev);
  return cuda_ok(h, cudaGetLastError(), "k_tc_gemm") ? CHF_OK : CHF_E_CUDA;
}

template <typename InT>
int launch_tc_split(Handle* h, const TcPlan& p, const Ptr8<const InT>& ins, int kvalid, uint8_t* bimg,
                    size_t bfield_stride, int nfields, int kid) {
  const int groups = p.kpad / 8;
  dim3 grid(p.ntiles, (groups * 128 + 255) / 256, nfields);
  cudaEvent_t ev;
  prof_begin(h, kid, &ev);
  k_tc_split<InT><<<grid, 256, 0, h->stream>>>(p, ins, kvalid, bimg, bfield_stride);
  prof_end(h, kid, ev);
  return cuda_ok(h, cudaGetLastError(), "k_tc_split") ? CHF_OK : CHF_E_CUDA;
}

template int launch_tc_gemm<float>(Handle*, const TcPlan&, const uint8_t*, const uint8_t*, size_t,
                                   const Ptr8<float>&, int, size_t, int);
template int launch_tc_gemm<double>(Handle*, const TcPlan&, const uint8_t*, const uint8_t*, size_t,
                                    const Ptr8<double>&, int, size_t, int);
template int launch_tc_split<float>(Handle*, const TcPlan&, const Ptr8<const float>&, int, uint8_t*,
                                    size_t, int, int);
template int launch_tc_split<double>(Handle*, const TcPlan&, const Ptr8<const double>&, int, uint8_t*,
                                     size_t, int, int);

}  // namespace chf
