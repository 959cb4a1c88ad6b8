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
//   k_curl          dz of H1, H3 by FP64 warp scans, h_v = k^2 H2 + i a D H1 + i b D H3,
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
#include "tc_dev.cuh"

namespace chf {

namespace {

constexpr int CM = 8;           // modes per CTA in k_curl
constexpr int CURL_THREADS = 256;

// dz (REF:570-599) of a[0..N] (stride as) into b (stride bs) by one warp, in
// FP64: suffix sums per parity class, lane-local then a warp scan (the scheme
// of k_solve.cu)
__device__ __forceinline__ void warp_deriv_d(const double* a, int as, double* b, int bs, int N) {
  const int lane = threadIdx.x & 31;
  const int E = (N + 32) / 32;
  const int i0 = lane * E;
  double te = 0.0, to = 0.0;
  for (int q = 0; q < E; ++q) {
    int j = i0 + q;
    if (j <= N) {
      double g = 2.0 * (double)j * a[j * as];
      if (j & 1) to += g; else te += g;
    }
  }
  double se = te, so = to;
  for (int off = 1; off < 32; off <<= 1) {
    double ue = __shfl_down_sync(0xffffffffu, se, off);
    double uo = __shfl_down_sync(0xffffffffu, so, off);
    if (lane + off < 32) { se += ue; so += uo; }
  }
  double re_ = se - te, ro = so - to;
  for (int q = E - 1; q >= 0; --q) {
    int i = i0 + q;
    if (i <= N) {
      double bi = (i & 1) ? re_ : ro;
      if (i == 0) bi *= 0.5;
      b[i * bs] = bi;
      double g = 2.0 * (double)i * a[i * as];
      if (i & 1) ro += g; else re_ += g;
    }
  }
  __syncwarp();
}

// grid (ceil(modes / CM)), CURL_THREADS threads.
// lc: 3 fields [NZ][ncols] FP64 (H1, H2, H3 coefficients from the exact z
// transform); out: fixed-point digit images and column exponents for the GL
// GEMM (k_tcgemm.cu layout), field 0 = h_v, field 1 = h_g (mode (0,0)
// carries H1, H3).  FP64 up to h_v, h_g: h_v is a small remainder of
// k^2 H2 + i a D H1 + i b D H3 (the gradient part of the Lamb vector
// cancels), so FP32 derivatives would leave an error ~100x FP32 rounding in
// it.  h_v, h_g are then rounded to FP32 (a relative error per coefficient)
// and split into digits below their column's power of two.
__global__ void __launch_bounds__(CURL_THREADS) k_curl(const double* __restrict__ lc,
                                                       const double* __restrict__ iapha,
                                                       const double* __restrict__ ibeta, Dims d,
                                                       const __grid_constant__ FxPlan plan,
                                                       uint8_t* __restrict__ bimg, int* __restrict__ bexp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NZ = d.NZ, N = d.N;
  const long modes = d.modes(), ncols = 2 * modes;
  double* L = reinterpret_cast<double*>(smem_raw);     // [3][NZ][CM][2]
  double* D = L + 3 * NZ * CM * 2;                     // [4][CM][NZ]: D H1.re, D H1.im, D H3.re, D H3.im
  float* Hs = reinterpret_cast<float*>(D + 4 * CM * NZ);  // [2][NZ][CM][2]: h_v, h_g
  __shared__ int s_e[2][CM * 2];
  const long m0 = (long)blockIdx.x * CM;
  for (int t = threadIdx.x; t < 3 * NZ * CM * 2; t += blockDim.x) {
    int c = t % (CM * 2), n = (t / (CM * 2)) % NZ, f = t / (CM * 2 * NZ);
    long col = 2 * m0 + c;
    L[t] = col < ncols ? lc[(size_t)f * NZ * ncols + (size_t)n * ncols + col] : 0.0;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  for (int task = warp; task < 4 * CM; task += CURL_THREADS / 32) {
    int comp = task / CM, l = task % CM;
    int f = comp < 2 ? 0 : 2, reim = comp & 1;
    warp_deriv_d(L + (size_t)f * NZ * CM * 2 + l * 2 + reim, CM * 2, D + ((size_t)comp * CM + l) * NZ, 1, N);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < NZ * CM * 2; t += blockDim.x) {
    const int c = t % (CM * 2), n = t / (CM * 2);
    const int l = c / 2, reim = c % 2;
    const long m = m0 + l;
    float v = 0.f, w = 0.f;
    if (m < modes) {
      const int kx = (int)(m % d.KX), ky = (int)(m / d.KX);
      const double a = iapha[kx], b = ibeta[ky], k2 = a * a + b * b;
      const double* h1 = L + ((size_t)0 * NZ + n) * CM * 2 + l * 2;
      const double* h2 = L + ((size_t)1 * NZ + n) * CM * 2 + l * 2;
      const double* h3 = L + ((size_t)2 * NZ + n) * CM * 2 + l * 2;
      const double d1r = D[(0 * CM + l) * NZ + n], d1i = D[(1 * CM + l) * NZ + n];
      const double d3r = D[(2 * CM + l) * NZ + n], d3i = D[(3 * CM + l) * NZ + n];
      if (m == 0) {
        v = (float)h1[reim];
        w = (float)h3[reim];
      } else if (reim == 0) {
        v = (float)(k2 * h2[0] - a * d1i - b * d3i);   // h_v = k2 H2 + i a D H1 + i b D H3
        w = (float)(-a * h3[1] + b * h1[1]);           // h_g = i a H3 - i b H1
      } else {
        v = (float)(k2 * h2[1] + a * d1r + b * d3r);
        w = (float)(a * h3[0] - b * h1[0]);
      }
    }
    Hs[(size_t)n * CM * 2 + c] = v;
    Hs[(size_t)(NZ + n) * CM * 2 + c] = w;
  }
  __syncthreads();
  // column exponents: max |value| < 2^e
  if (threadIdx.x < 2 * CM * 2) {
    const int f = threadIdx.x / (CM * 2), c = threadIdx.x % (CM * 2);
    float mx = 0.f;
    for (int n = 0; n < NZ; ++n) mx = fmaxf(mx, fabsf(Hs[(size_t)(f * NZ + n) * CM * 2 + c]));
    int e = 0;
    if (mx > 0.f) (void)frexpf(mx, &e);
    s_e[f][c] = e;
    const long col = 2 * m0 + c;
    if (col < ncols) bexp[(size_t)f * plan.bexp_stride() + col] = e;
  }
  __syncthreads();
  // one thread per (column c of this CTA, 8-row group g): 8 digits per plane
  // and field, one 16-byte store each
  const int groups = plan.kpad / 8;
  for (int t = threadIdx.x; t < CM * 2 * groups; t += blockDim.x) {
    const int c = t % (CM * 2), g = t / (CM * 2);
    const long col = 2 * m0 + c;
    if (col >= ncols) continue;
    const int nt = (int)(col / FX_NT), r = (int)(col % FX_NT);
    const int ch = (8 * g) / TC_KC, kl = 8 * g - ch * TC_KC;
    const uint32_t pbytes = (uint32_t)FX_NT * plan.kc[ch] * 2u;
    const size_t off = ((size_t)(kl / 8) * (FX_NT / 8) + r / 8) * 128 + (r % 8) * 16;
    for (int f = 0; f < 2; ++f) {
      uint16_t hd[FX_PLANES][8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int n = 8 * g + q;
        const float x = n < NZ ? Hs[(size_t)(f * NZ + n) * CM * 2 + c] : 0.f;
        float dg[FX_PLANES];
        tc::fx_digits_f(x, s_e[f][c], dg);
#pragma unroll
        for (int i = 0; i < FX_PLANES; ++i) hd[i][q] = tc::bf16_bits(dg[i]);
      }
      uint8_t* base = bimg + (size_t)f * plan.b_field_bytes() + (size_t)nt * plan.b_tile_bytes + plan.b_chunk_off[ch];
#pragma unroll
      for (int pl = 0; pl < FX_PLANES; ++pl) {
        uint4 u;
        u.x = (uint32_t)hd[pl][0] | ((uint32_t)hd[pl][1] << 16);
        u.y = (uint32_t)hd[pl][2] | ((uint32_t)hd[pl][3] << 16);
        u.z = (uint32_t)hd[pl][4] | ((uint32_t)hd[pl][5] << 16);
        u.w = (uint32_t)hd[pl][6] | ((uint32_t)hd[pl][7] << 16);
        *reinterpret_cast<uint4*>(base + (size_t)pl * pbytes + off) = u;
      }
    }
  }
}

// (0,0)-mode histories: the GL GEMM left the GL values of H1(0,0), H3(0,0)
// in mode 0 of the h_v / h_g buffers.  clamb*nm1 <- clamb*n (REF:1560-1569),
// clamb*n <- those values, mode 0 of h_v / h_g <- 0 (k^2 = 0 there).
__global__ void k_meanfix(cd* __restrict__ hv, cd* __restrict__ hg, double* cl1n, double* cl1nm1,
                          double* cl3n, double* cl3nm1, int NZ, long modes) {
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
  // z transforms with exact accumulation (fixed-point digits, k_tcgemm.cu);
  // the GL evaluation of h_v, h_g is not differentiated afterwards and keeps
  // the floating bf16x3 split
  h->tz1 = make_fx_plan(MP, NZ, cols);
  h->tz2 = make_fx_plan(NZ, MP, cols);
  h->tgl = make_fx_plan(NZ, NZ, cols);
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
      !upload(&h->az2, make_a_image_fx(h->tz2, a2, NZ, MP, e2), "A image z2") ||
      !upload(&h->agl, make_a_image_fx(h->tgl, a3, NZ, NZ, e3), "A image gl") ||
      !upload_int(&h->aexp1, e1, "A exponents z1") || !upload_int(&h->aexp2, e2, "A exponents z2") ||
      !upload_int(&h->aexp3, e3, "A exponents gl"))
    return CHF_E_NOMEM;
  if (!cuda_ok(h, cudaMalloc((void**)&h->bexp,
                            sizeof(int) * 6 * std::max(h->tz1.bexp_stride(), h->tz2.bexp_stride())),
               "B exponents"))
    return CHF_E_NOMEM;
  h->bimg_bytes = std::max({(size_t)6 * h->tz1.b_field_bytes(), (size_t)3 * h->tz2.b_field_bytes(),
                            (size_t)2 * h->tgl.b_field_bytes()});
  if (!cuda_ok(h, cudaMalloc((void**)&h->bimg, h->bimg_bytes), "B images") ||
      !cuda_ok(h, cudaMemsetAsync(h->bimg, 0, h->bimg_bytes, h->stream), "B images") ||
      !cuda_ok(h, cudaMalloc((void**)&h->wz32, sizeof(cf) * 6 * (size_t)MP * d.modes()), "wz32") ||
      !cuda_ok(h, cudaMalloc((void**)&h->wy32, sizeof(cf) * 6 * (size_t)MP * d.PY * d.KX), "wy32") ||
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

int launch_nonlinear_mixed(Handle* h) {
  const Dims& d = h->d;
  const long modes = d.modes(), cols = 2 * modes;
  int rc;
  // z: coefficients -> values on the product grid (tensor cores)
  Ptr8<const double> in6{};
  const int order[6] = {F_U, F_V, F_W, F_OX, F_OY, F_OZ};
  for (int i = 0; i < 6; ++i) in6.p[i] = reinterpret_cast<const double*>(h->f[order[i]]);
  if ((rc = launch_tc_split_fx<double>(h, h->tz1, in6, d.NZ, h->bimg, h->bexp, 6, K_SPLIT_Z1)) != CHF_OK)
    return rc;
  Ptr8<float> o6{};
  for (int i = 0; i < 6; ++i) o6.p[i] = reinterpret_cast<float*>(h->wz32 + (size_t)i * d.MP * modes);
  if ((rc = launch_tc_gemm_fx<float>(h, h->tz1, h->az1, h->aexp1, h->bimg, h->bexp, o6, 6, cols,
                                     K_GEMM_Z1)) != CHF_OK)
    return rc;
  // y and x transforms with the products, FP32
  if ((rc = launch_xy<float>(h, h->wz32, h->wy32, h->twf_py, h->twf_px)) != CHF_OK) return rc;
  // z: values -> coefficients 0..N
  Ptr8<const float> in3{};
  for (int i = 0; i < 3; ++i) in3.p[i] = reinterpret_cast<const float*>(h->wz32 + (size_t)i * d.MP * modes);
  if ((rc = launch_tc_split_fx<float>(h, h->tz2, in3, d.MP, h->bimg, h->bexp, 3, K_SPLIT_Z2)) != CHF_OK)
    return rc;
  Ptr8<double> o3{};
  for (int i = 0; i < 3; ++i) o3.p[i] = h->lc64 + (size_t)i * d.NZ * cols;
  if ((rc = launch_tc_gemm_fx<double>(h, h->tz2, h->az2, h->aexp2, h->bimg, h->bexp, o3, 3, cols,
                                      K_GEMM_Z2)) != CHF_OK)
    return rc;
  // curl / projection -> digit images for the GL transform
  {
    size_t smem = sizeof(double) * ((size_t)3 * d.NZ * CM * 2 + (size_t)4 * CM * d.NZ) +
                  sizeof(float) * (size_t)2 * d.NZ * CM * 2;
    if (smem > 48 * 1024 &&
        !cuda_ok(h, cudaFuncSetAttribute(k_curl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "k_curl smem"))
      return CHF_E_CUDA;
    cudaEvent_t ev;
    prof_begin(h, K_CURL32, &ev);
    k_curl<<<(unsigned)((modes + CM - 1) / CM), CURL_THREADS, smem, h->stream>>>(
        h->lc64, h->iapha, h->ibeta, d, h->tgl, h->bimg, h->bexp);
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
    k_meanfix<<<1, 256, 0, h->stream>>>(h->f[F_U], h->f[F_W], h->mean[M_CL1N], h->mean[M_CL1NM1],
                                        h->mean[M_CL3N], h->mean[M_CL3NM1], d.NZ, modes);
    prof_end(h, K_MEANFIX, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_meanfix")) return CHF_E_CUDA;
  }
  std::swap(h->f[F_U], h->f[F_RV]);
  std::swap(h->f[F_W], h->f[F_RG]);
  return CHF_OK;
}

}  // namespace chf
