// k_mixed.cu -- getnonlinear (poiseuilleflow.f90:1380-1612) in mixed precision.
//
// The state and the implicit solves stay FP64 (k_solve.cu).  The nonlinear
// term is formed with FP32 FFTs/products and tcgen05 tensor-core GEMMs for
// the wall-normal Chebyshev transforms, accumulated exactly on fixed-point
// digits (k_tcgemm.cu):
//
//   k_tc_split_z1   six FP64 fields [NZ][2 modes] -> fixed-point digit images
//   k_tc_gemm_z1    values on the product grid: V = T1 C, T1[p][n] = cos(pi n p / MZ)
//   k_yinv/xprod/yfwd (FP32)   as in the FP64 path (k_nonlinear.cu)
//   k_tc_split_z2   the three Lamb components [MP][2 modes] -> digit images
//   k_tc_gemm_z2    Chebyshev coefficients in FP64: L = W V, W = DCT-I weights
//                   on the product grid, rows 0..N (truncation, REF:1686-1704)
//   k_curl          h_v = k^2 H2 + D (i a H1 + i b H3) with one FP64 recurrence
//                   per (mode, re/im) column,
//                   h_g = i a H3 - i b H1 (REF:1502-1540), written as tile images
//   k_tc_gemm_gl    Gauss-Lobatto values T0 h (REF:1573-1609) into the FP64
//                   history buffers
//   k_meanfix       the (0,0) histories clamb1n/clamb3n (REF:1482-1487, 1560-1609)
//
// Differences from the FP64 path: omega_x / omega_z keep their values in the
// spanwise Nyquist slots (the FP64 path, like the reference, leaves H1 / H3
// there; no step reads them).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "chf_internal.h"
#include "f64bits.cuh"
#include "tc_dev.cuh"

namespace chf {

namespace {

constexpr int CURL_THREADS = 64;  // 16 (mode, re/im) columns per CTA: warp 0 h_v, warp 1 h_g
constexpr int CURL_COLS = 16;

// Grid ceil(ncols / CURL_COLS), CURL_THREADS threads: warp f of a CTA forms
// field f (0 = h_v, 1 = h_g) of the CTA's 16 (mode, re/im) columns, two lanes
// per column (lanes 2c and 2c + 1).  lc: 3 fields [NZ][ncols] FP64 (H1, H2,
// H3 coefficients from the exact z transform); hs: FP32 scratch
// [2][NZ][ncols]; out: fixed-point digit images and column exponents for the
// GL GEMM (k_tcgemm.cu layout), field 0 = h_v, field 1 = h_g (mode (0,0)
// carries H1, H3).  FP64 up to h_v, h_g: h_v is a small remainder of
// k^2 H2 + D G with G = i a H1 + i b H3 (the gradient part of the Lamb vector
// cancels), so FP32 derivatives would leave an error ~100x FP32 rounding in
// it.  Only G is differentiated, by dz's backward recurrence (REF:570-599)
//   (D G)_k = (D G)_{k+2} + 2 (k+1) G_{k+1},
// whose even-k and odd-k chains are independent: lane p of a pair runs the
// rows k = p (mod 2), forming the G values of the other parity it needs;
// h_g = i a H3 - i b H1 is pointwise.  Multiplying by i folds into the signs
// of the per-thread coefficients, the partner component is read directly.
// Pass 1 (descending, CURL_PF rows of H loaded ahead) rounds the field to
// FP32 by integer operations into hs; the pair combines its column maxima
// (their powers of two).  Pass 2 (the pair splits the 8-row groups) writes
// the digits, 8 rows per 16-byte store, and the exact level sums of the GL
// row N (the wall z = -1), which the GL GEMM leaves out (it covers 0..N-1).
constexpr int CURL_PF = 4;  // own rows of H loaded ahead of the recurrence

__global__ void __launch_bounds__(CURL_THREADS, 16) k_curl(const double* __restrict__ lc,
                                                       const double* __restrict__ iapha,
                                                       const double* __restrict__ ibeta, Dims d,
                                                       const __grid_constant__ FxPlan plan, float* __restrict__ hs,
                                                       uint8_t* __restrict__ bimg, int* __restrict__ bexp,
                                                       const float* __restrict__ gl_tail, int gl_tail_exp,
                                                       double* __restrict__ glv_n, double* __restrict__ glg_n) {
  const long modes = d.modes(), ncols = 2 * modes;
  const int f = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long col = (long)blockIdx.x * CURL_COLS + (lane >> 1);
  const int par = lane & 1;
  const bool live = col < ncols;  // every lane takes part in the pair's shuffles
  const long cl = live ? col : 0;
  const long m = cl >> 1;
  const int N = d.N, NZ = d.NZ;
  const double a = iapha[m % d.KX], b = ibeta[m / d.KX], k2 = a * a + b * b;
  const double s = (cl & 1) ? 1.0 : -1.0;  // (i z)_re = -z_im, (i z)_im = z_re
  const double sa = s * a, sb = s * b;
  const bool mean = (m % d.chm == 0);  // a channel's (0,0) mode
  // the mean column reads its own H1, H3 and passes them through
  const long pcol = mean ? cl : (cl ^ 1);
  const double* H1 = lc;
  const double* H2 = lc + (size_t)NZ * ncols;
  const double* H3 = lc + (size_t)2 * NZ * ncols;
  float* out = hs + (size_t)f * NZ * ncols;
  double dg2 = 0.0;  // D G at k+2 (this parity)
  float mx = 0.f;    // column maximum of |field| over this parity's rows
  const int ktop = (N - par) & ~1 | par;  // the largest k <= N with k = par (mod 2)
  for (int k0 = ktop; k0 >= 0; k0 -= 2 * CURL_PF) {
    // h_v: H2 (H1 for the mean) at row k, H1 and H3 at row k + 1;
    // h_g: H1 and H3 at row k
    double x1[CURL_PF], x2[CURL_PF], x3[CURL_PF];
#pragma unroll
    for (int i = 0; i < CURL_PF; ++i) {
      const int k = max(k0 - 2 * i, 0);
      const size_t base = (size_t)k * ncols, up = (size_t)min(k + 1, N) * ncols;
      if (f == 0) {
        x2[i] = mean ? H1[base + cl] : H2[base + cl];
        x1[i] = H1[up + pcol];
        x3[i] = H3[up + pcol];
      } else {
        x2[i] = 0.0;
        x1[i] = H1[base + pcol];
        x3[i] = H3[base + pcol];
      }
    }
#pragma unroll
    for (int i = 0; i < CURL_PF; ++i) {
      const int k = k0 - 2 * i;
      if (k < 0) break;
      float o;
      if (f == 0) {
        double dg = 0.0;
        if (k < N) {
          const double gk1 = fma(sa, x1[i], sb * x3[i]);  // (i a H1 + i b H3) at row k + 1
          dg = fma(bits::from_int(2u * (uint32_t)(k + 1)), gk1, dg2);
        }
        dg2 = dg;
        if (k == 0) dg = bits::half(dg);  // dz halves b_0
        o = bits::narrow(mean ? x2[i] : fma(k2, x2[i], dg));  // h_v = k^2 H2 + D G
      } else {
        o = bits::narrow(mean ? x3[i] : fma(sa, x3[i], -(sb * x1[i])));  // h_g = i a H3 - i b H1
      }
      if (live) out[(size_t)k * ncols + col] = o;
      mx = fmaxf(mx, fabsf(o));
    }
  }
  mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
  int e = 0;
  if (mx > 0.f) (void)frexpf(mx, &e);
  if (live && par == 0) bexp[(size_t)f * plan.bexp_stride() + col] = e;
  __syncwarp();  // the partner's rows of the field are visible from here on
  // pass 2: digits, groups of 8 rows (rows >= NZ are zero), the pair taking
  // alternate groups, and the level sums of the GL row N
  const int nt = (int)(cl / FX_NT), r = (int)(cl % FX_NT);
  float lev[FX_PLANES] = {0.f, 0.f, 0.f, 0.f};
  uint8_t* fimg = bimg + (size_t)f * plan.b_field_bytes() + (size_t)nt * plan.b_tile_bytes;
  for (int g = par; g < plan.kpad / 8; g += 2) {
    const int ch = (8 * g) / TC_KC, kl = 8 * g - ch * TC_KC;
    const uint32_t pbytes = (uint32_t)FX_NT * plan.kc[ch] * 2u;
    const size_t off = ((size_t)(kl / 8) * (FX_NT / 8) + r / 8) * 128 + (r % 8) * 16;
    uint16_t hd[FX_PLANES][8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = 8 * g + q;
      const float x = (live && k <= N) ? out[(size_t)k * ncols + col] : 0.f;
      float dg[FX_PLANES];
      tc::fx_digits_f(x, e, dg);
#pragma unroll
      for (int i = 0; i < FX_PLANES; ++i) hd[i][q] = tc::bf16_bits(dg[i]);
      tc::fx_tail_mac(gl_tail, plan.kpad, k, dg, lev);
    }
    if (live) {
      uint8_t* base = fimg + plan.b_chunk_off[ch];
#pragma unroll
      for (int pl = 0; pl < FX_PLANES; ++pl) {
        uint4 u4;
        u4.x = (uint32_t)hd[pl][0] | ((uint32_t)hd[pl][1] << 16);
        u4.y = (uint32_t)hd[pl][2] | ((uint32_t)hd[pl][3] << 16);
        u4.z = (uint32_t)hd[pl][4] | ((uint32_t)hd[pl][5] << 16);
        u4.w = (uint32_t)hd[pl][6] | ((uint32_t)hd[pl][7] << 16);
        *reinterpret_cast<uint4*>(base + (size_t)pl * pbytes + off) = u4;
      }
    }
  }
  // the pair's partial level sums are exact integers: their sum is exact
#pragma unroll
  for (int i = 0; i < FX_PLANES; ++i) lev[i] += __shfl_xor_sync(0xffffffffu, lev[i], 1);
  if (live && par == 0) (f == 0 ? glv_n : glg_n)[col] = tc::fx_tail_value(lev, gl_tail_exp + e - 35);
}

// (0,0)-mode histories: the GL GEMM left the GL values of H1(0,0), H3(0,0)
// in mode 0 of the h_v / h_g buffers.  clamb*nm1 <- clamb*n (REF:1560-1569),
// clamb*n <- those values, mode 0 of h_v / h_g <- 0 (k^2 = 0 there).  One
// CTA per stacked channel c: its mode c chm, its mean arrays at c * 2 NZ.
__global__ void k_meanfix(cd* __restrict__ hv, cd* __restrict__ hg, double* cl1n, double* cl1nm1,
                          double* cl3n, double* cl3nm1, int NZ, long modes, long chm) {
  const long c = blockIdx.x;
  hv += c * chm;
  hg += c * chm;
  cl1n += c * 2 * NZ;
  cl1nm1 += c * 2 * NZ;
  cl3n += c * 2 * NZ;
  cl3nm1 += c * 2 * NZ;
  for (int p = threadIdx.x; p < NZ; p += blockDim.x) {
    cd a = hv[(size_t)p * modes], b = hg[(size_t)p * modes];
    cl1nm1[2 * p] = cl1n[2 * p];
    cl1nm1[2 * p + 1] = cl1n[2 * p + 1];
    cl3nm1[2 * p] = cl3n[2 * p];
    cl3nm1[2 * p + 1] = cl3n[2 * p + 1];
    cl1n[2 * p] = a.re;
    cl1n[2 * p + 1] = a.im;
    cl3n[2 * p] = b.re;
    cl3n[2 * p + 1] = b.im;
    hv[(size_t)p * modes] = cd{0.0, 0.0};
    hg[(size_t)p * modes] = cd{0.0, 0.0};
  }
}

constexpr double kPi = 3.14159265358979323846;

double cospi_ratio(long num, long den) {
  // cos(pi num / den) with the argument reduced exactly
  long r = num % (2 * den);
  return std::cos(kPi * (double)r / (double)den);
}

}  // namespace

int setup_mixed(Handle* h) {
  const Dims& d = h->d;
  const long cols = 2 * d.modes();
  const int N = d.N, NZ = d.NZ, MZ = d.MZ, MP = d.MP;
  // z transforms with exact accumulation (fixed-point digits, k_tcgemm.cu):
  // Z2 and GL on four planes of 7-bit digits, Z1 on three of 8 bits (below)
  // Z2 and GL cover rows 0..N-1 (one 128-row tile for nnz = 128): row N, the
  // last coefficient / the wall point z = -1, is formed beside the digits by
  // k_tc_split_fx and k_curl with the same exact level sums, instead of by a
  // second row tile of MMAs
  // Z1's values go to FP32 products: 3-plane digits (about 2^-24 of the row
  // and column maxima, as an FP32 GEMM) suffice there, where their level sums
  // stay exact (K padded to at most 204); 4 planes beyond that
  h->tz1 = make_fx_plan(MP, NZ, cols, (NZ + 15) / 16 * 16 <= 204 ? 3 : 4);
  h->tz2 = make_fx_plan(N, MP, cols);
  h->tgl = make_fx_plan(N, NZ, cols);
  std::vector<double> a1((size_t)MP * NZ), a2((size_t)NZ * MP), a3((size_t)NZ * NZ);
  for (int p = 0; p < MP; ++p)
    for (int n = 0; n < NZ; ++n) a1[(size_t)p * NZ + n] = cospi_ratio((long)n * p, MZ);
  for (int n = 0; n < NZ; ++n)
    for (int q = 0; q < MP; ++q) {
      double w = (q == 0 || q == MZ) ? 0.5 : 1.0;
      double v = (2.0 / MZ) * w * cospi_ratio((long)n * q, MZ);
      if (n == 0) v *= 0.5;
      a2[(size_t)n * MP + q] = v;
    }
  for (int p = 0; p < NZ; ++p)
    for (int n = 0; n < NZ; ++n) a3[(size_t)p * NZ + n] = cospi_ratio((long)n * p, N);
  auto upload = [h](uint8_t** dst, const std::vector<uint8_t>& img, const char* what) {
    if (!cuda_ok(h, cudaMalloc((void**)dst, img.size()), what)) return false;
    return cuda_ok(h, cudaMemcpy(*dst, img.data(), img.size(), cudaMemcpyHostToDevice), what);
  };
  std::vector<int> e1, e2, e3;
  auto upload_int = [h](int** dst, const std::vector<int>& v, const char* what) {
    if (!cuda_ok(h, cudaMalloc((void**)dst, sizeof(int) * v.size()), what)) return false;
    return cuda_ok(h, cudaMemcpy(*dst, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice), what);
  };
  if (!upload(&h->az1, make_a_image_fx(h->tz1, a1, MP, NZ, e1), "A image z1") ||
      !upload(&h->az2, make_a_image_fx(h->tz2, a2, N, MP, e2), "A image z2") ||
      !upload(&h->agl, make_a_image_fx(h->tgl, a3, N, NZ, e3), "A image gl") ||
      !upload_int(&h->aexp1, e1, "A exponents z1") || !upload_int(&h->aexp2, e2, "A exponents z2") ||
      !upload_int(&h->aexp3, e3, "A exponents gl"))
    return CHF_E_NOMEM;
  {  // row N of Z2 and GL as digit planes, computed beside the split / curl
    auto up_digits = [h](float** dst, const std::vector<float>& v, const char* what) {
      if (!cuda_ok(h, cudaMalloc((void**)dst, sizeof(float) * v.size()), what)) return false;
      return cuda_ok(h, cudaMemcpy(*dst, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice), what);
    };
    if (!up_digits(&h->z2_tail, a_row_digits(h->tz2, a2, MP, N, h->z2_tail_exp), "z2 row N") ||
        !up_digits(&h->gl_tail, a_row_digits(h->tgl, a3, NZ, N, h->gl_tail_exp), "GL row N"))
      return CHF_E_CUDA;
  }
  if (!cuda_ok(h, cudaMalloc((void**)&h->bexp,
                            sizeof(int) * 6 * std::max(h->tz1.bexp_stride(), h->tz2.bexp_stride())),
               "B exponents"))
    return CHF_E_NOMEM;
  h->bimg_bytes = std::max({(size_t)6 * h->tz1.b_field_bytes(), (size_t)3 * h->tz2.b_field_bytes(),
                            (size_t)2 * h->tgl.b_field_bytes()});
  if (!cuda_ok(h, cudaMalloc((void**)&h->bimg, h->bimg_bytes), "B images") ||
      !cuda_ok(h, cudaMemsetAsync(h->bimg, 0, h->bimg_bytes, h->stream), "B images") ||
      !cuda_ok(h, cudaMalloc((void**)&h->wz32, sizeof(cf) * 6 * (size_t)MP * d.modes()), "wz32") ||
      !cuda_ok(h, cudaMalloc((void**)&h->wy32, sizeof(cf) * 6 * (size_t)fft_view(d).MP * d.PY * d.KX), "wy32") ||
      !cuda_ok(h, cudaMalloc((void**)&h->lc64, sizeof(double) * 3 * (size_t)NZ * cols), "lc64"))
    return CHF_E_NOMEM;
  // FP32 twiddles
  struct {
    cf** dst;
    int L;
  } tws[] = {{&h->twf_py, d.PY}, {&h->twf_px, d.PX}};
  for (auto& t : tws) {
    std::vector<cf> v(t.L);
    for (int k = 0; k < t.L; ++k) {
      double a = -2.0 * kPi * (double)k / (double)t.L;
      v[k] = cf{(float)std::cos(a), (float)std::sin(a)};
    }
    if (!cuda_ok(h, cudaMalloc((void**)t.dst, sizeof(cf) * v.size()), "twiddles") ||
        !cuda_ok(h, cudaMemcpy(*t.dst, v.data(), sizeof(cf) * v.size(), cudaMemcpyHostToDevice), "twiddles"))
      return CHF_E_CUDA;
  }
  return CHF_OK;
}

int launch_nonlinear_mixed(Handle* h, const cudaEvent_t* field_ready) {
  const Dims& d = h->d;
  const long modes = d.modes(), cols = 2 * modes;
  int rc;
  // z: coefficients -> values on the product grid (tensor cores)
  Ptr8<const double> in6{};
  const int order[6] = {F_U, F_V, F_W, F_OX, F_OY, F_OZ};
  for (int i = 0; i < 6; ++i) in6.p[i] = reinterpret_cast<const double*>(h->f[order[i]]);
  Ptr8<float> o6{};
  for (int i = 0; i < 6; ++i) o6.p[i] = reinterpret_cast<float*>(h->wz32 + (size_t)i * d.MP * modes);
  if (field_ready && xy_register_path(d)) {
    // field by field as the inputs land: digits, product-grid values and the
    // inverse y transform of field i need field i only
    for (int i = 0; i < 6; ++i) {
      if (!cuda_ok(h, cudaStreamWaitEvent(h->stream, field_ready[i], 0), "field wait")) return CHF_E_CUDA;
      Ptr8<const double> in1{};
      in1.p[0] = in6.p[i];
      Ptr8<float> o1{};
      o1.p[0] = o6.p[i];
      uint8_t* bimg = h->bimg + (size_t)i * h->tz1.b_field_bytes();
      int* bexp = h->bexp + (size_t)i * h->tz1.bexp_stride();
      if ((rc = launch_tc_split_fx<double>(h, h->tz1, in1, d.NZ, bimg, bexp, 1, K_SPLIT_Z1)) != CHF_OK ||
          (rc = launch_tc_gemm_fx<float>(h, h->tz1, h->az1, h->aexp1, bimg, bexp, o1, 1, cols, K_GEMM_Z1)) !=
              CHF_OK ||
          (rc = launch_yinv_fields(h, h->wz32, h->wy32, h->twf_py, i, 1)) != CHF_OK)
        return rc;
    }
    if ((rc = launch_xprod_yfwd(h, h->wz32, h->wy32, h->twf_py, h->twf_px)) != CHF_OK) return rc;
  } else {
    if (field_ready)
      for (int i = 0; i < 6; ++i)
        if (!cuda_ok(h, cudaStreamWaitEvent(h->stream, field_ready[i], 0), "field wait")) return CHF_E_CUDA;
    if ((rc = launch_tc_split_fx<double>(h, h->tz1, in6, d.NZ, h->bimg, h->bexp, 6, K_SPLIT_Z1)) != CHF_OK)
      return rc;
    if ((rc = launch_tc_gemm_fx<float>(h, h->tz1, h->az1, h->aexp1, h->bimg, h->bexp, o6, 6, cols,
                                       K_GEMM_Z1)) != CHF_OK)
      return rc;
    // y and x transforms with the products, FP32
    if ((rc = launch_xy<float>(h, h->wz32, h->wy32, h->twf_py, h->twf_px)) != CHF_OK) return rc;
  }
  // z: values -> coefficients 0..N
  Ptr8<const float> in3{};
  for (int i = 0; i < 3; ++i) in3.p[i] = reinterpret_cast<const float*>(h->wz32 + (size_t)i * d.MP * modes);
  Ptr8<double> o3{}, row_n{};
  for (int i = 0; i < 3; ++i) {
    o3.p[i] = h->lc64 + (size_t)i * d.NZ * cols;
    row_n.p[i] = o3.p[i] + (size_t)d.N * cols;
  }
  FxTail tail;
  tail.adig = h->z2_tail;
  tail.aexp = h->z2_tail_exp;
  tail.out = row_n;
  if ((rc = launch_tc_split_fx<float>(h, h->tz2, in3, d.MP, h->bimg, h->bexp, 3, K_SPLIT_Z2, tail)) != CHF_OK)
    return rc;
  if ((rc = launch_tc_gemm_fx<double>(h, h->tz2, h->az2, h->aexp2, h->bimg, h->bexp, o3, 3, cols,
                                      K_GEMM_Z2)) != CHF_OK)
    return rc;
  // curl / projection -> digit images for the GL transform
  {
    cudaEvent_t ev;
    prof_begin(h, K_CURL32, &ev);
    // FP32 scratch for h_v, h_g: the product-grid buffer, free once the z2
    // digits are formed (2 NZ <= 6 MP rows of modes complex values)
    k_curl<<<(unsigned)((cols + CURL_COLS - 1) / CURL_COLS), CURL_THREADS, 0, h->stream>>>(
        h->lc64, h->iapha, h->ibeta, d, h->tgl, reinterpret_cast<float*>(h->wz32), h->bimg, h->bexp,
        h->gl_tail, h->gl_tail_exp, reinterpret_cast<double*>(h->f[F_U]) + (size_t)d.N * cols,
        reinterpret_cast<double*>(h->f[F_W]) + (size_t)d.N * cols);
    prof_end(h, K_CURL32, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_curl")) return CHF_E_CUDA;
  }
  // Gauss-Lobatto values of h_v, h_g -> the unp1 / wnp1 buffers (FP64)
  Ptr8<double> o2{};
  o2.p[0] = reinterpret_cast<double*>(h->f[F_U]);
  o2.p[1] = reinterpret_cast<double*>(h->f[F_W]);
  if ((rc = launch_tc_gemm_fx<double>(h, h->tgl, h->agl, h->aexp3, h->bimg, h->bexp, o2, 2, cols,
                                      K_GEMM_GL)) != CHF_OK)
    return rc;
  {
    cudaEvent_t ev;
    prof_begin(h, K_MEANFIX, &ev);
    k_meanfix<<<d.nch, 256, 0, h->stream>>>(h->f[F_U], h->f[F_W], h->mean[M_CL1N], h->mean[M_CL1NM1],
                                            h->mean[M_CL3N], h->mean[M_CL3NM1], d.NZ, modes, d.chm);
    prof_end(h, K_MEANFIX, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_meanfix")) return CHF_E_CUDA;
  }
  std::swap(h->f[F_U], h->f[F_RV]);
  std::swap(h->f[F_W], h->f[F_RG]);
  return CHF_OK;
}

}  // namespace chf
