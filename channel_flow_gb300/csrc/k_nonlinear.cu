// k_nonlinear.cu -- getnonlinear (poiseuilleflow.f90:1380-1612) on one GB300.
//
// The reference forms each of the six products of the Lamb vector separately
// (getlamb/getlamb1, poiseuilleflow.f90:1625-1815), transforming both factors
// to the 3/2-padded physical grid every time (12 inverse + 6 forward 3D
// transforms, 36 MPI transposes).  Here each of the six fields u, v, w,
// omega_x, omega_y, omega_z goes to physical space once and the three
// components
//     H1 = omega_y w - re_p - omega_z v,  H2 = omega_z u - omega_x w,
//     H3 = omega_x v - omega_y u
// come back once (6 inverse + 3 forward transforms).  Products of truncated
// series are exact on the padded grids, so the result equals the reference's
// to rounding.
//
// Pass order (each a kernel; the pencil transposes of the reference become
// the choice of which index is contiguous in each pass):
//   k_zc2v   z: Chebyshev coefficients -> values on the MZ-interval product
//            grid, per spectral mode, for the six fields   [REF:1657-1680]
//   k_yinv   y: 3/2 zero-padding and backward DFT of length PY per (plane, kx)
//            [REF:1051-1083 with expand, REF:721-765]
//   k_xprod  x: Hermitian c2r of length PX (two fields per complex DFT),
//            the three products at every point, forward r2c (two products per
//            DFT), truncation to kx < nnx/2      [REF:1094-1145, 1683, 1787]
//   k_yfwd   y: forward DFT of length PY, truncation, 1/(PX PY)
//            [REF:1152-1181]
//   k_zcurl  z: values -> coefficients 0..N, the curl/projection
//            h_v = k^2 H2 + i alpha D H1 + i beta D H3, h_g = i alpha H3 - i beta H1
//            (REF:1502-1540), the (0,0)-mode histories (REF:1482-1487, 1560-1569)
//            and coefficients -> Gauss-Lobatto values (REF:1573-1609).
// The history swap of REF:1542-1558 is a pointer exchange on the host.
#include <algorithm>
#include <cstdio>

#include "chf_internal.h"
#include "fft_warp.cuh"

namespace chf {

namespace {

// Modes per CTA in the z kernels (ZL) and (plane, y) rows per CTA in k_xprod
// (XR) are template parameters: the launchers take the largest of 8, 4, 2
// (and 1 for XR) whose FFT work fits the per-thread butterfly bound, so long
// lines (600-point z lines, 576-point x rows) run with fewer lines per CTA.
constexpr int ZC_THREADS = 512;
constexpr int Y_THREADS = 256;
constexpr int X_THREADS = 256;
// the shared-memory y / x kernels hold two buffers (out-of-place FFT stages,
// smem_fft_pp); the rules take the most lines per CTA whose buffers fit this
// much, so that four CTAs share an SM
constexpr size_t kXYSmemTarget = 56 * 1024;

struct SixPtr {
  const cd* p[6];
};

// ---------------------------------------------------------------------------
// z: coefficients -> values at z'_p = cos(pi p / MZ), p = 0..MZ.
// Even extension of length 2 MZ with doubled first entry, forward DFT, /2
// (the packed evaluation of getlamb, REF:1672-1683, applied per field).
// ZL modes per CTA, grid (ceil(modes / ZL), 6)
// ---------------------------------------------------------------------------
template <int MB2, int ZL>
__global__ void __launch_bounds__(ZC_THREADS) k_zc2v(SixPtr in, cd* __restrict__ out, Dims d,
                                                     const __grid_constant__ FftPlan pz, const cd* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int L = 2 * d.MZ, ls = L;
  const long modes = d.modes();
  const long m0 = (long)blockIdx.x * ZL;
  const int f = blockIdx.y;
  const cd* __restrict__ src = in.p[f];
  for (int t = threadIdx.x; t < ZL * L; t += blockDim.x) s[t] = cd{0.0, 0.0};
  __syncthreads();
  for (int t = threadIdx.x; t < ZL * d.NZ; t += blockDim.x) {
    int l = t % ZL, n = t / ZL;
    long m = m0 + l;
    cd c{0.0, 0.0};
    if (m < modes) c = src[(size_t)n * modes + m];
    if (n == 0) {
      s[l * ls] = cd{2.0 * c.re, 2.0 * c.im};
    } else {
      s[l * ls + n] = c;
      s[l * ls + L - n] = c;
    }
  }
  __syncthreads();
  smem_fft<double, -1, MB2>(s, ZL, ls, pz, tw);
  cd* __restrict__ dst = out + (size_t)f * d.MP * modes;
  for (int t = threadIdx.x; t < ZL * d.MP; t += blockDim.x) {
    int l = t % ZL, p = t / ZL;
    long m = m0 + l;
    if (m < modes) {
      cd v = s[l * ls + p];
      dst[(size_t)p * modes + m] = cd{0.5 * v.re, 0.5 * v.im};
    }
  }
}

// ---------------------------------------------------------------------------
// y inverse: per (field, plane p, group of kxb streamwise modes).
// grid (KX / kxb, MP, 6)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(Y_THREADS, 4) k_yinv(const cplx<T>* __restrict__ wz, cplx<T>* __restrict__ wy,
                                                       Dims d, int kxb, const __grid_constant__ FftPlan py,
                                                       const cplx<T>* __restrict__ stab) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s2 = s + kxb * (d.PY + 1);
  const int ls = d.PY + 1;
  const int f = blockIdx.z, p = blockIdx.y, kx0 = blockIdx.x * kxb;
  const long modes = d.modes();
  const cplx<T>* __restrict__ src = wz + ((size_t)f * d.MP + p) * modes;
  for (int t = threadIdx.x; t < kxb * ls; t += blockDim.x) s[t] = cplx<T>{(T)0, (T)0};
  __syncthreads();
  for (int t = threadIdx.x; t < kxb * d.KY; t += blockDim.x) {
    int l = t % kxb, ky = t / kxb;
    if (ky == d.NYQ) continue;  // expand(1) zeroes the spanwise Nyquist
    int slot = ky < d.NYQ ? ky : d.PY - d.KY + ky;
    s[l * ls + slot] = src[(size_t)ky * d.KX + kx0 + l];
  }
  __syncthreads();
  const cplx<T>* r = smem_fft_pp<T, +1>(s, s2, kxb, ls, py, stab);
  cplx<T>* __restrict__ dst = wy + ((size_t)f * d.MP + p) * (size_t)d.PY * d.KX;
  for (int t = threadIdx.x; t < kxb * d.PY; t += blockDim.x) {
    int l = t % kxb, yp = t / kxb;
    dst[(size_t)yp * d.KX + kx0 + l] = r[l * ls + yp];
  }
}

// ---------------------------------------------------------------------------
// x: fused c2r, products, r2c.  Rows r = p * PY + yp; each row holds KX modes
// of six fields (u, v, w, ox, oy, oz), written back in place as H1, H2, H3
// into field slots 0, 1, 2.  XR rows per CTA, grid (ceil(MP * PY / XR))
// ---------------------------------------------------------------------------
template <typename T, int XR>
__global__ void __launch_bounds__(X_THREADS, 4) k_xprod(cplx<T>* __restrict__ wy, Dims d, T re_p,
                                                        const __grid_constant__ FftPlan px, const cplx<T>* __restrict__ stab) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using C = cplx<T>;
  C* s = reinterpret_cast<C*>(smem_raw);
  const int PX = d.PX, KX = d.KX, ls = PX + 1;
  C* s2 = s + XR * 3 * ls;  // second buffer of the out-of-place FFT stages
  const long nrows = (long)d.MP * d.PY;
  const long r0 = (long)blockIdx.x * XR;
  const size_t fstride = (size_t)d.MP * d.PY * KX;
  // lines: row q, pair c (0: u+iv, 1: w+i ox, 2: oy+i oz) at (c*XR + q) * ls
  for (int t = threadIdx.x; t < XR * 3 * ls; t += blockDim.x) s[t] = C{(T)0, (T)0};
  __syncthreads();
  for (int t = threadIdx.x; t < XR * 3 * KX; t += blockDim.x) {
    int k = t % KX, c = (t / KX) % 3, q = t / (3 * KX);
    long r = r0 + q;
    if (r >= nrows) continue;
    C F = wy[(size_t)(2 * c) * fstride + (size_t)r * KX + k];
    C G = wy[(size_t)(2 * c + 1) * fstride + (size_t)r * KX + k];
    C* line = s + (c * XR + q) * ls;
    if (k == 0) {
      line[0] = C{F.re, G.re};  // imaginary part of the streamwise mean dropped
    } else {
      line[k] = C{F.re - G.im, F.im + G.re};        // F + i G
      line[PX - k] = C{F.re + G.im, G.re - F.im};   // conj(F) + i conj(G)
    }
  }
  __syncthreads();
  s = smem_fft_pp<T, +1>(s, s2, XR * 3, ls, px, stab);  // s: the physical lines
  s2 = (s == reinterpret_cast<C*>(smem_raw)) ? s + XR * 3 * ls : reinterpret_cast<C*>(smem_raw);
  // products at every physical point; write (H1 + i H2) to pair 0, (H3 + 0i) to pair 1
  for (int t = threadIdx.x; t < XR * PX; t += blockDim.x) {
    int x = t % PX, q = t / PX;
    C a = s[(0 * XR + q) * ls + x];  // u, v
    C b = s[(1 * XR + q) * ls + x];  // w, ox
    C c = s[(2 * XR + q) * ls + x];  // oy, oz
    T u = a.re, v = a.im, w = b.re, ox = b.im, oy = c.re, oz = c.im;
    T h1 = (oy * w - re_p) - oz * v;
    T h2 = oz * u - ox * w;
    T h3 = ox * v - oy * u;
    s[(0 * XR + q) * ls + x] = C{h1, h2};
    s[(1 * XR + q) * ls + x] = C{h3, (T)0};
  }
  __syncthreads();
  // forward DFT of the 2 * XR lines holding (H1 + i H2) and H3
  s = smem_fft_pp<T, -1>(s, s2, XR * 2, ls, px, stab);
  for (int t = threadIdx.x; t < XR * KX; t += blockDim.x) {
    int k = t % KX, q = t / KX;
    long r = r0 + q;
    if (r >= nrows) continue;
    const C* z = s + (0 * XR + q) * ls;
    C A = z[k];
    C B = z[k == 0 ? 0 : PX - k];
    B.im = -B.im;  // conj(Z[-k])
    C H1{(T)0.5 * (A.re + B.re), (T)0.5 * (A.im + B.im)};
    C H2{(T)0.5 * (A.im - B.im), (T)-0.5 * (A.re - B.re)};
    C H3 = s[(1 * XR + q) * ls + k];
    wy[(size_t)0 * fstride + (size_t)r * KX + k] = H1;
    wy[(size_t)1 * fstride + (size_t)r * KX + k] = H2;
    wy[(size_t)2 * fstride + (size_t)r * KX + k] = H3;
  }
}

// ---------------------------------------------------------------------------
// y forward: per (component, plane, kx group); keeps ky = 0..NYQ (the Nyquist
// slot receives padded mode +NYQ as in expand(-1), REF:751-761) and the
// negative modes, scaled by 1/(PX PY).  grid (KX / kxb, MP, 3)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(Y_THREADS, 4) k_yfwd(const cplx<T>* __restrict__ wy, cplx<T>* __restrict__ wz,
                                                       Dims d, int kxb, const __grid_constant__ FftPlan py,
                                                       const cplx<T>* __restrict__ stab, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* s2 = s + kxb * (d.PY + 1);
  const int ls = d.PY + 1;
  const int f = blockIdx.z, p = blockIdx.y, kx0 = blockIdx.x * kxb;
  const long modes = d.modes();
  const cplx<T>* __restrict__ src = wy + ((size_t)f * d.MP + p) * (size_t)d.PY * d.KX;
  for (int t = threadIdx.x; t < kxb * d.PY; t += blockDim.x) {
    int l = t % kxb, yp = t / kxb;
    s[l * ls + yp] = src[(size_t)yp * d.KX + kx0 + l];
  }
  __syncthreads();
  const cplx<T>* r = smem_fft_pp<T, -1>(s, s2, kxb, ls, py, stab);
  cplx<T>* __restrict__ dst = wz + ((size_t)f * d.MP + p) * modes;
  for (int t = threadIdx.x; t < kxb * d.KY; t += blockDim.x) {
    int l = t % kxb, ky = t / kxb;
    int slot = ky <= d.NYQ ? ky : d.PY - d.KY + ky;
    cplx<T> v = r[l * ls + slot];
    dst[(size_t)ky * d.KX + kx0 + l] = cplx<T>{v.re * scale, v.im * scale};
  }
}

// Chebyshev derivative in coefficient space (dz, REF:570-599) by the backward
// recurrence b_{k-1} = b_{k+1} + 2 k a_k, b_0 halved.  Serial; a and b are
// strided real sequences (a = one component of interleaved complex data).
__device__ __forceinline__ void cheb_deriv_serial(const double* a, int as, double* b, int bs, int N) {
  double bp1 = 0.0, bp2 = 0.0;  // b_{k}, b_{k+1} of the previous iteration
  b[N * bs] = 0.0;
  for (int k = N; k >= 1; --k) {
    double bk1 = bp2 + 2.0 * (double)k * a[k * as];  // b_{k-1}
    if (k == 1) bk1 *= 0.5;
    b[(k - 1) * bs] = bk1;
    bp2 = bp1;
    bp1 = bk1;
  }
}

// ---------------------------------------------------------------------------
// z: values -> coefficients, curl, histories, coefficients -> GL values.
// ZL modes per CTA, grid (ceil(modes / ZL))
// shared: FFT buffer max(ZL x 2MZ, 2 ZL x 2N), coefficient store 3 x ZL x NZ,
//         derivative store 4 x ZL x NZ (doubles)
// ---------------------------------------------------------------------------
template <int MB2, int ZL>
__global__ void __launch_bounds__(ZC_THREADS) k_zcurl(
    const cd* __restrict__ wz, cd* __restrict__ out_hv, cd* __restrict__ out_hg,
    cd* __restrict__ ox_out, cd* __restrict__ oz_out, double* __restrict__ cl1n,
    double* __restrict__ cl1nm1, double* __restrict__ cl3n, double* __restrict__ cl3nm1,
    const double* __restrict__ iapha, const double* __restrict__ ibeta, Dims d, const __grid_constant__ FftPlan pzm,
    const cd* __restrict__ twm, const __grid_constant__ FftPlan pz2, const cd* __restrict__ tw2) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = 2 * d.MZ, ls = L;
  const int NZ = d.NZ, N = d.N;
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int L2 = 2 * N;
  const int fb = max(ZL * ls, 2 * ZL * L2);  // FFT buffer elements
  cd* coef = s + fb;                     // [3][ZL][NZ]
  double* der = reinterpret_cast<double*>(coef + 3 * ZL * NZ);  // [4][ZL][NZ]
  const long modes = d.modes();
  const long m0 = (long)blockIdx.x * ZL;
  const double inv_mz = 1.0 / (double)d.MZ;
  for (int f = 0; f < 3; ++f) {
    const cd* __restrict__ src = wz + (size_t)f * d.MP * modes;
    for (int t = threadIdx.x; t < ZL * d.MP; t += blockDim.x) {
      int l = t % ZL, p = t / ZL;
      long m = m0 + l;
      cd v{0.0, 0.0};
      if (m < modes) v = src[(size_t)p * modes + m];
      s[l * ls + p] = v;
      if (p > 0 && p < d.MZ) s[l * ls + L - p] = v;
    }
    __syncthreads();
    smem_fft<double, -1, MB2>(s, ZL, ls, pzm, twm);
    for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
      int l = t % ZL, n = t / ZL;
      cd v = s[l * ls + n];
      double sc = (n == 0) ? 0.5 * inv_mz : inv_mz;
      coef[(f * ZL + l) * NZ + n] = cd{v.re * sc, v.im * sc};
    }
    __syncthreads();
  }
  // omega_x <- H1, omega_z <- H3 (the reference leaves them there, REF:1489-1496)
  for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
    int l = t % ZL, n = t / ZL;
    long m = m0 + l;
    if (m >= modes) continue;
    ox_out[(size_t)n * modes + m] = coef[(0 * ZL + l) * NZ + n];
    oz_out[(size_t)n * modes + m] = coef[(2 * ZL + l) * NZ + n];
  }
  // derivatives of H1 and H3 (re, im): 4 serial recurrences per line
  if (threadIdx.x < 4 * ZL) {
    int l = threadIdx.x % ZL, which = threadIdx.x / ZL;  // 0:H1re 1:H1im 2:H3re 3:H3im
    const cd* c = coef + ((which < 2 ? 0 : 2) * ZL + l) * NZ;
    const double* a = reinterpret_cast<const double*>(c) + (which & 1);
    cheb_deriv_serial(a, 2, der + (which * ZL + l) * NZ, 1, N);
  }
  __syncthreads();
  // (0,0)-mode histories: nm1 <- old n (the swap of REF:1560-1569), n <- new
  // coefficients (converted to GL values below)
  const bool has00 = (m0 == 0);
  if (has00) {
    for (int t = threadIdx.x; t < 2 * NZ; t += blockDim.x) {
      cl1nm1[t] = cl1n[t];
      cl3nm1[t] = cl3n[t];
    }
  }
  // h_v, h_g in coefficient space -> FFT buffer lines 2l (h_v) and 2l+1 (h_g)
  // of length 2N (even extension with doubled end points, REF:1573-1581)
  for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
    int l = t % ZL, n = t / ZL;
    long m = m0 + l;
    int kx = (int)(m % d.KX), ky = (int)(m / d.KX);
    double a = 0.0, b = 0.0;
    if (m < modes) { a = iapha[kx]; b = ibeta[ky]; }
    double k2 = a * a + b * b;
    cd h1 = coef[(0 * ZL + l) * NZ + n];
    cd h2 = coef[(1 * ZL + l) * NZ + n];
    cd h3 = coef[(2 * ZL + l) * NZ + n];
    double d1r = der[(0 * ZL + l) * NZ + n], d1i = der[(1 * ZL + l) * NZ + n];
    double d3r = der[(2 * ZL + l) * NZ + n], d3i = der[(3 * ZL + l) * NZ + n];
    // h_v = k2 H2 + i a D H1 + i b D H3
    cd hv{k2 * h2.re - a * d1i - b * d3i, k2 * h2.im + a * d1r + b * d3r};
    // h_g = i a H3 - i b H1
    cd hg{-a * h3.im + b * h1.im, a * h3.re - b * h1.re};
    if (has00 && l == 0) {  // the (0,0) mode's H1, H3 become clamb1n / clamb3n
      hv = h1;
      hg = h3;
    }
    cd* lv = s + (2 * l) * L2;
    cd* lg = s + (2 * l + 1) * L2;
    double dbl = (n == 0 || n == N) ? 2.0 : 1.0;
    lv[n] = cd{dbl * hv.re, dbl * hv.im};
    lg[n] = cd{dbl * hg.re, dbl * hg.im};
    if (n > 0 && n < N) {
      lv[L2 - n] = hv;
      lg[L2 - n] = hg;
    }
  }
  __syncthreads();
  smem_fft<double, -1, MB2>(s, ZL * 2, L2, pz2, tw2);
  for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
    int l = t % ZL, n = t / ZL;
    long m = m0 + l;
    if (m >= modes) continue;
    cd v = s[(2 * l) * L2 + n];
    cd g = s[(2 * l + 1) * L2 + n];
    v = cd{0.5 * v.re, 0.5 * v.im};
    g = cd{0.5 * g.re, 0.5 * g.im};
    if (has00 && l == 0) {
      cl1n[2 * n] = v.re;
      cl1n[2 * n + 1] = v.im;
      cl3n[2 * n] = g.re;
      cl3n[2 * n + 1] = g.im;
      v = cd{0.0, 0.0};
      g = cd{0.0, 0.0};
    }
    out_hv[(size_t)n * modes + m] = v;
    out_hg[(size_t)n * modes + m] = g;
  }
}


// ---------------------------------------------------------------------------
// z forward only: the Lamb vector H1, H2, H3 on the product grid ->
// Chebyshev coefficients 0..N (the first part of k_zcurl), for the pressure.
// ZL modes per CTA, grid (ceil(modes / ZL), 3); out: 3 x [NZ][modes].
// ---------------------------------------------------------------------------
template <int MB2, int ZL>
__global__ void __launch_bounds__(ZC_THREADS) k_zfwd(const cd* __restrict__ wz, cd* __restrict__ out, Dims d,
                                                     const __grid_constant__ FftPlan pzm,
                                                     const cd* __restrict__ twm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = 2 * d.MZ, ls = L;
  const int NZ = d.NZ;
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const long modes = d.modes();
  const long m0 = (long)blockIdx.x * ZL;
  const int f = blockIdx.y;
  const double inv_mz = 1.0 / (double)d.MZ;
  const cd* __restrict__ src = wz + (size_t)f * d.MP * modes;
  for (int t = threadIdx.x; t < ZL * d.MP; t += blockDim.x) {
    int l = t % ZL, p = t / ZL;
    long m = m0 + l;
    cd v{0.0, 0.0};
    if (m < modes) v = src[(size_t)p * modes + m];
    s[l * ls + p] = v;
    if (p > 0 && p < d.MZ) s[l * ls + L - p] = v;
  }
  __syncthreads();
  smem_fft<double, -1, MB2>(s, ZL, ls, pzm, twm);
  cd* __restrict__ dst = out + (size_t)f * NZ * modes;
  for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
    int l = t % ZL, n = t / ZL;
    long m = m0 + l;
    if (m >= modes) continue;
    cd v = s[l * ls + n];
    double sc = (n == 0) ? 0.5 * inv_mz : inv_mz;
    dst[(size_t)n * modes + m] = cd{v.re * sc, v.im * sc};
  }
}

// ---------------------------------------------------------------------------
// Length-192 specialisations (3/2-padded 128-point directions), FP32, one
// warp per line with the packed register FFT of fft_warp.cuh.  Rows written
// by k_yinv_w and read by k_xprod_w / k_yfwd_w are in the permuted order
// 32 k1 + lane of that header; every consumer is row-wise, so the order never
// matters.
// ---------------------------------------------------------------------------
constexpr int W_WARPS = 8;    // warps (lines) per CTA in the x kernel
constexpr int YW_COLS = 16;   // kx columns (one warp each) per CTA in the y kernels

// Element t of a pass over a [rows][YW_COLS] tile (rows a multiple of 32,
// row stride YW_COLS + 1 floats): a warp takes the 16 columns of rows r and
// r + 16, whose banks are disjoint (17 * 16 = 16 mod 32), and each half-warp
// one 128-byte row segment in global memory.
__device__ __forceinline__ void tile_rc(int t, int& row, int& col) {
  const int lane = t & 31, wi = t >> 5;
  col = lane & 15;
  row = (wi >> 4) * 32 + (lane >> 4) * 16 + (wi & 15);
}

// x: c2r (three packed pairs), Lamb products, r2c; KX = 64, PX = 192.
// grid ceil(nrows / W_WARPS), W_WARPS * 32 threads.
__global__ void __launch_bounds__(W_WARPS * 32) k_xprod_w(cf* __restrict__ wy, long nrows, size_t fstride,
                                                         float re_p, const cf* __restrict__ tw) {
  using C = cf;
  __shared__ Fft192Table s_inv, s_fwd;
  fft192_table<+1>(&s_inv, tw);
  fft192_table<-1>(&s_fwd, tw);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long r = (long)blockIdx.x * W_WARPS + (threadIdx.x >> 5);
  if (r >= nrows) return;
  Line6 pk3[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const C* F = wy + (size_t)(2 * c) * fstride + (size_t)r * 64;
    const C* G = wy + (size_t)(2 * c + 1) * fstride + (size_t)r * 64;
    C f0 = F[lane], f1 = F[32 + lane], g0 = G[lane], g1 = G[32 + lane];
    // Hermitian partners: positions 128 + l -> mode 64 - l, 160 + l -> mode 32 - l
    const int src = (32 - lane) & 31;
    C f1s = shfl_i(f1, src), g1s = shfl_i(g1, src);
    C f0s = shfl_i(f0, src), g0s = shfl_i(g0, src);
    C f32 = shfl_i(f1, 0), g32 = shfl_i(g1, 0);  // mode 32 (for lane 0)
    // F + iG (mean: real parts) at positions l, 32 + l; zero at 64 .. 127;
    // conj F + i conj G at 128 + l, 160 + l
    const C v0 = lane == 0 ? C{f0.re, g0.re} : C{f0.re - g0.im, f0.im + g0.re};
    const C v1{f1.re - g1.im, f1.im + g1.re};
    const C v4 = lane == 0 ? C{0.f, 0.f} : C{f1s.re + g1s.im, g1s.re - f1s.im};
    const C v5 = lane == 0 ? C{f32.re + g32.im, g32.re - f32.im} : C{f0s.re + g0s.im, g0s.re - f0s.im};
    Line6& a = pk3[c];
    a.r[0] = pk(v0.re, v1.re);
    a.i[0] = pk(v0.im, v1.im);
    a.r[1] = a.i[1] = 0ull;
    a.r[2] = pk(v4.re, v5.re);
    a.i[2] = pk(v4.im, v5.im);
    fft192_natural_to_perm_x2<+1, true>(a, s_inv);
  }
  // products, two elements per instruction:
  //   H1 + i H2 = (oy w - re_p - oz v) + i (oz u - ox w),  H3 = ox v - oy u
  Line6 z1, z2;
  const f32x2 nrp = pk(-re_p, -re_p);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const f32x2 u = pk3[0].r[j], v = pk3[0].i[j], w = pk3[1].r[j], ox = pk3[1].i[j];
    const f32x2 oy = pk3[2].r[j], oz = pk3[2].i[j];
    z1.r[j] = sub2(fma2(oy, w, nrp), mul2(oz, v));
    z1.i[j] = sub2(mul2(oz, u), mul2(ox, w));
    z2.r[j] = sub2(mul2(ox, v), mul2(oy, u));
    z2.i[j] = 0ull;
  }
  fft192_perm_to_natural_x2<-1>(z1, s_fwd);
  fft192_perm_to_natural_x2<-1>(z2, s_fwd);
  // unpack H1, H2 from Z = FFT(H1 + i H2): Z[-k] for k = l (element 0) and 32 + l (element 1)
  const int src = (32 - lane) & 31;
  const C z10 = line_get(z1, 0), z11 = line_get(z1, 1), z14 = line_get(z1, 4), z15 = line_get(z1, 5);
  C m5 = shfl_i(z15, src), m4 = shfl_i(z14, src), m50 = shfl_i(z15, 0);
  C A0 = z10, B0 = lane == 0 ? z10 : m5;   // Z[192 - l]
  C A1 = z11, B1 = lane == 0 ? m50 : m4;   // Z[160 - l]
  C* o0 = wy + (size_t)r * 64;
  C* o1 = wy + fstride + (size_t)r * 64;
  C* o2 = wy + 2 * fstride + (size_t)r * 64;
  const float h = 0.5f;
  o0[lane] = C{h * (A0.re + B0.re), h * (A0.im - B0.im)};
  o1[lane] = C{h * (A0.im + B0.im), -h * (A0.re - B0.re)};
  o0[32 + lane] = C{h * (A1.re + B1.re), h * (A1.im - B1.im)};
  o1[32 + lane] = C{h * (A1.im + B1.im), -h * (A1.re - B1.re)};
  o2[lane] = line_get(z2, 0);
  o2[32 + lane] = line_get(z2, 1);
}

// y inverse: per (field, plane, 16 kx columns); KY = 128, PY = 192.
// grid (KX / 16, MP, 6), 512 threads.  The tile holds real and imaginary
// parts in separate planes (the packed lines pair elements, not re / im).
__global__ void __launch_bounds__(YW_COLS * 32, 4) k_yinv_w(const cf* __restrict__ wz, cf* __restrict__ wy, Dims d,
                                                        const cf* __restrict__ tw) {
  __shared__ Fft192Table s_t;
  __shared__ float tre[192][YW_COLS + 1], tim[192][YW_COLS + 1];
  fft192_table<+1>(&s_t, tw);
  const int f = blockIdx.z, p = blockIdx.y, kx0 = blockIdx.x * YW_COLS;
  const long modes = d.modes();
  const cf* src = wz + ((size_t)f * d.MP + p) * modes;
  for (int t = threadIdx.x; t < 128 * YW_COLS; t += blockDim.x) {
    int ky, c;
    tile_rc(t, ky, c);
    const cf x = src[(size_t)ky * d.KX + kx0 + c];
    tre[ky][c] = x.re;
    tim[ky][c] = x.im;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  // ky = l, 32 + l; 64 (Nyquist, zeroed) and padding; 64 + l (negative modes, l > 0), 96 + l
  Line6 a;
  a.r[0] = pk(tre[lane][c], tre[32 + lane][c]);
  a.i[0] = pk(tim[lane][c], tim[32 + lane][c]);
  a.r[1] = a.i[1] = 0ull;
  a.r[2] = pk(lane == 0 ? 0.f : tre[64 + lane][c], tre[96 + lane][c]);
  a.i[2] = pk(lane == 0 ? 0.f : tim[64 + lane][c], tim[96 + lane][c]);
  fft192_natural_to_perm_x2<+1, true>(a, s_t);
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    upk(a.r[j], tre[64 * j + lane][c], tre[64 * j + 32 + lane][c]);
    upk(a.i[j], tim[64 * j + lane][c], tim[64 * j + 32 + lane][c]);
  }
  __syncthreads();
  cf* dst = wy + ((size_t)f * d.MP + p) * (size_t)192 * d.KX;
  for (int t = threadIdx.x; t < 192 * YW_COLS; t += blockDim.x) {
    int q, cc;
    tile_rc(t, q, cc);
    dst[(size_t)q * d.KX + kx0 + cc] = cf{tre[q][cc], tim[q][cc]};
  }
}

// y forward: per (component, plane, 16 kx columns); keeps ky = 0..64 and
// the negative modes, scaled by 1/(PX PY).  grid (KX / 16, MP, 3), 512 threads.
__global__ void __launch_bounds__(YW_COLS * 32, 4) k_yfwd_w(const cf* __restrict__ wy, cf* __restrict__ wz, Dims d,
                                                        const cf* __restrict__ tw, float scale) {
  __shared__ Fft192Table s_t;
  __shared__ float tre[192][YW_COLS + 1], tim[192][YW_COLS + 1];
  fft192_table<-1>(&s_t, tw);
  const int f = blockIdx.z, p = blockIdx.y, kx0 = blockIdx.x * YW_COLS;
  const long modes = d.modes();
  const cf* src = wy + ((size_t)f * d.MP + p) * (size_t)192 * d.KX;
  for (int t = threadIdx.x; t < 192 * YW_COLS; t += blockDim.x) {
    int q, c;
    tile_rc(t, q, c);
    const cf x = src[(size_t)q * d.KX + kx0 + c];
    tre[q][c] = x.re;
    tim[q][c] = x.im;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  Line6 a;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    a.r[j] = pk(tre[64 * j + lane][c], tre[64 * j + 32 + lane][c]);
    a.i[j] = pk(tim[64 * j + lane][c], tim[64 * j + 32 + lane][c]);
  }
  fft192_perm_to_natural_x2<-1>(a, s_t);
  const f32x2 sc = pk(scale, scale);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    a.r[j] = mul2(a.r[j], sc);
    a.i[j] = mul2(a.i[j], sc);
  }
  __syncthreads();
  // natural spectral position 32 j + l -> ky slot
  const cf v0 = line_get(a, 0), v1 = line_get(a, 1), v2 = line_get(a, 2), v4 = line_get(a, 4),
           v5 = line_get(a, 5);
  tre[lane][c] = v0.re;  // ky = l
  tim[lane][c] = v0.im;
  tre[32 + lane][c] = v1.re;  // ky = 32 + l
  tim[32 + lane][c] = v1.im;
  if (lane == 0) {  // ky = 64 <- padded mode +64
    tre[64][c] = v2.re;
    tim[64][c] = v2.im;
  } else {  // ky = 64 + l
    tre[64 + lane][c] = v4.re;
    tim[64 + lane][c] = v4.im;
  }
  tre[96 + lane][c] = v5.re;  // ky = 96 + l
  tim[96 + lane][c] = v5.im;
  __syncthreads();
  cf* dst = wz + ((size_t)f * d.MP + p) * modes;
  for (int t = threadIdx.x; t < 128 * YW_COLS; t += blockDim.x) {
    int ky, cc;
    tile_rc(t, ky, cc);
    dst[(size_t)ky * d.KX + kx0 + cc] = cf{tre[ky][cc], tim[ky][cc]};
  }
}

template <typename K>
bool set_smem(Handle* h, K kernel, size_t bytes) {
  // the shared-memory FFT kernels want several CTAs per SM: the largest
  // shared-memory carveout (the default heuristic can pick 32 KB, one CTA)
  if (!cuda_ok(h, cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared),
               "cudaFuncSetAttribute"))
    return false;
  if (bytes > 48 * 1024)
    return cuda_ok(h, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes),
                   "cudaFuncSetAttribute");
  return true;
}

constexpr size_t kMaxSmem = 227 * 1024;  // dynamic shared memory per CTA

// streamwise modes per CTA in the generic y kernels: the largest power of two
// up to 16 that divides KX and whose two line buffers fit kXYSmemTarget (1
// if none does); any b whose buffers fit the SM is valid (autotuner)
template <typename T>
size_t y_smem(const Dims& d, int b) { return 2 * sizeof(cplx<T>) * b * (d.PY + 1); }

template <typename T>
int pick_kxb(const Dims& d) {
  for (int b = 16; b > 1; b /= 2)
    if (d.KX % b == 0 && y_smem<T>(d, b) <= kXYSmemTarget) return b;
  return y_smem<T>(d, 1) <= kMaxSmem ? 1 : 0;
}

template <typename T>
size_t xprod_smem(const Dims& d, int xr) { return 2 * sizeof(cplx<T>) * xr * 3 * (d.PX + 1); }

template <typename T>
int pick_xr(const Dims& d) {
  for (int r = 8; r > 1; r /= 2)
    if (xprod_smem<T>(d, r) <= kXYSmemTarget) return r;
  return xprod_smem<T>(d, 1) <= kMaxSmem ? 1 : 0;
}

size_t zc2v_smem(const Dims& d, int zl) { return sizeof(cd) * zl * 2 * d.MZ; }

size_t zcurl_smem(const Dims& d, int zl) {
  const size_t fb = (size_t)std::max(zl * 2 * d.MZ, 2 * zl * 2 * d.N);
  return sizeof(cd) * fb + sizeof(cd) * 3 * zl * d.NZ + sizeof(double) * 4 * zl * d.NZ;
}

int pick_zl_c2v(const Dims& d) {
  for (int l = 8; l >= 2; l /= 2)
    if (fft_fits(l, 2 * d.MZ, ZC_THREADS, 4) && zc2v_smem(d, l) <= kMaxSmem) return l;
  return 0;
}

int pick_zl_curl(const Dims& d) {
  for (int l = 8; l >= 2; l /= 2)
    if (fft_fits(l, 2 * d.MZ, ZC_THREADS, 4) && fft_fits(2 * l, 2 * d.N, ZC_THREADS, 4) &&
        zcurl_smem(d, l) <= kMaxSmem)
      return l;
  return 0;
}

template <typename T, int XR>
int run_xprod(Handle* h, cplx<T>* wy, const FftPlan& px, const cplx<T>* tw_px) {
  const Dims d = fft_view(h->d);
  const size_t smem = xprod_smem<T>(d, XR);
  if (!set_smem(h, k_xprod<T, XR>, smem)) return CHF_E_CUDA;
  const long nrows = (long)d.MP * d.PY;
  dim3 grid((unsigned)((nrows + XR - 1) / XR));
  cudaEvent_t ev;
  prof_begin(h, K_XPROD, &ev);
  k_xprod<T, XR><<<grid, X_THREADS, smem, h->stream>>>(wy, d, (T)h->cfg.re_p, px, tw_px);
  prof_end(h, K_XPROD, ev);
  return cuda_ok(h, cudaGetLastError(), "k_xprod") ? CHF_OK : CHF_E_CUDA;
}

template <int ZL>
int run_zc2v(Handle* h) {
  const Dims& d = h->d;
  SixPtr in{{h->f[F_U], h->f[F_V], h->f[F_W], h->f[F_OX], h->f[F_OY], h->f[F_OZ]}};
  const size_t smem = zc2v_smem(d, ZL);
  if (!set_smem(h, k_zc2v<4, ZL>, smem)) return CHF_E_CUDA;
  dim3 grid((unsigned)((d.modes() + ZL - 1) / ZL), 6);
  cudaEvent_t ev;
  prof_begin(h, K_ZC2V, &ev);
  k_zc2v<4, ZL><<<grid, ZC_THREADS, smem, h->stream>>>(in, h->wz, d, h->pzm, h->tw_zm);
  prof_end(h, K_ZC2V, ev);
  return cuda_ok(h, cudaGetLastError(), "k_zc2v") ? CHF_OK : CHF_E_CUDA;
}

template <int ZL>
int run_zcurl(Handle* h) {
  const Dims& d = h->d;
  const size_t smem = zcurl_smem(d, ZL);
  if (!set_smem(h, k_zcurl<4, ZL>, smem)) return CHF_E_CUDA;
  dim3 grid((unsigned)((d.modes() + ZL - 1) / ZL));
  // h_v -> the unp1 buffer, h_g -> the wnp1 buffer; swapped with rhsvn /
  // rhsomegayn by the caller (REF:1542-1558)
  cudaEvent_t ev;
  prof_begin(h, K_ZCURL, &ev);
  k_zcurl<4, ZL><<<grid, ZC_THREADS, smem, h->stream>>>(
      h->wz, h->f[F_U], h->f[F_W], h->f[F_OX], h->f[F_OZ], h->mean[M_CL1N], h->mean[M_CL1NM1],
      h->mean[M_CL3N], h->mean[M_CL3NM1], h->iapha, h->ibeta, d, h->pzm, h->tw_zm, h->pz2,
      h->tw_z2);
  prof_end(h, K_ZCURL, ev);
  return cuda_ok(h, cudaGetLastError(), "k_zcurl") ? CHF_OK : CHF_E_CUDA;
}

}  // namespace

// Launch shapes the autotuner may try (chf_tune.cu): every shape the rules
// above accept, largest first.  y / x candidates for the handle's FFT-pass
// dimensions and arithmetic (fp32: the mixed path's FP32 transforms).
std::vector<int> shape_candidates(const Handle* h, int knob) {
  const Dims d = fft_view(h->d);
  const bool f32 = h->cfg.precision != CHF_FP64;
  std::vector<int> out;
  if (knob == 0) {  // kxb
    for (int b = 16; b >= 1; b /= 2) {
      const size_t bytes = f32 ? y_smem<float>(d, b) : y_smem<double>(d, b);
      if (d.KX % b == 0 && bytes <= kMaxSmem) out.push_back(b);
    }
  } else if (knob == 1) {  // xr
    for (int r = 8; r >= 1; r /= 2) {
      const size_t bytes = f32 ? xprod_smem<float>(d, r) : xprod_smem<double>(d, r);
      if (bytes <= kMaxSmem) out.push_back(r);
    }
  } else if (knob == 2) {  // zl_c2v
    for (int l = 8; l >= 2; l /= 2)
      if (fft_fits(l, 2 * d.MZ, ZC_THREADS, 4) && zc2v_smem(d, l) <= kMaxSmem) out.push_back(l);
  } else if (knob == 3) {  // zl_curl
    for (int l = 8; l >= 2; l /= 2)
      if (fft_fits(l, 2 * d.MZ, ZC_THREADS, 4) && fft_fits(2 * l, 2 * d.N, ZC_THREADS, 4) &&
          zcurl_smem(d, l) <= kMaxSmem)
        out.push_back(l);
  }
  return out;
}

// The FP32 register-FFT path of the x/y transforms, in two parts so that a
// caller can run the inverse y transform field by field (fields f0 ..
// f0 + nf - 1 of the six) and the products and forward transforms once.
bool xy_register_path(const Dims& d) { return d.PX == 192 && d.PY == 192 && d.KX % YW_COLS == 0; }

int launch_yinv_fields(Handle* h, cf* wz, cf* wy, const cf* tw_py, int f0, int nf) {
  const Dims d = fft_view(h->d);
  constexpr int YC = YW_COLS;
  cudaEvent_t ev;
  prof_begin(h, K_YINV, &ev);
  k_yinv_w<<<dim3(d.KX / YC, d.MP, nf), YC * 32, 0, h->stream>>>(
      wz + (size_t)f0 * d.MP * d.modes(), wy + (size_t)f0 * d.MP * d.PY * d.KX, d, tw_py);
  prof_end(h, K_YINV, ev);
  return cuda_ok(h, cudaGetLastError(), "k_yinv_w") ? CHF_OK : CHF_E_CUDA;
}

int launch_xprod_yfwd(Handle* h, cf* wz, cf* wy, const cf* tw_py, const cf* tw_px) {
  const Dims d = fft_view(h->d);
  constexpr int YC = YW_COLS;
  cudaStream_t st = h->stream;
  cudaEvent_t ev;
  const long nrows = (long)d.MP * d.PY;
  prof_begin(h, K_XPROD, &ev);
  k_xprod_w<<<(unsigned)((nrows + W_WARPS - 1) / W_WARPS), W_WARPS * 32, 0, st>>>(
      wy, nrows, (size_t)d.MP * d.PY * d.KX, (float)h->cfg.re_p, tw_px);
  prof_end(h, K_XPROD, ev);
  if (!cuda_ok(h, cudaGetLastError(), "k_xprod_w")) return CHF_E_CUDA;
  const float scale = (float)(1.0 / ((double)d.PX * (double)d.PY));
  prof_begin(h, K_YFWD, &ev);
  k_yfwd_w<<<dim3(d.KX / YC, d.MP, 3), YC * 32, 0, st>>>(wy, wz, d, tw_py, scale);
  prof_end(h, K_YFWD, ev);
  return cuda_ok(h, cudaGetLastError(), "k_yfwd_w") ? CHF_OK : CHF_E_CUDA;
}

template <typename T>
int launch_xy(Handle* h, cplx<T>* wz, cplx<T>* wy, const cplx<T>* tw_py, const cplx<T>* tw_px) {
  const Dims d = fft_view(h->d);
  cudaStream_t st = h->stream;
  if (sizeof(T) == 4 && xy_register_path(d)) {
    // register-FFT specialisation of the 128-point directions, FP32 only: in
    // FP64 (the FP64 pipe is the bound) the cross-lane radix-2 network costs
    // more FP64 instructions than the radix-4 shared-memory stages below
    cf* wzf = reinterpret_cast<cf*>(wz);
    cf* wyf = reinterpret_cast<cf*>(wy);
    const cf* twy = reinterpret_cast<const cf*>(tw_py);
    const cf* twx = reinterpret_cast<const cf*>(tw_px);
    const int rc = launch_yinv_fields(h, wzf, wyf, twy, 0, 6);
    return rc == CHF_OK ? launch_xprod_yfwd(h, wzf, wyf, twy, twx) : rc;
  }
  // the handle's own line precision takes the tuned plans and shapes; FP64
  // lines of a mixed handle take the FP64 rules
  const bool own = (sizeof(T) == 8) == !mixed_front(h);
  const FftPlan& py = own ? h->py : h->py64;
  const FftPlan& px = own ? h->px : h->px64;
  // the plans' stage twiddle tables (tw_py, tw_px serve the register path)
  const cplx<T>* stw_py = own ? static_cast<const cplx<T>*>(h->stw_py) : reinterpret_cast<const cplx<T>*>(h->stw_py64);
  const cplx<T>* stw_px = own ? static_cast<const cplx<T>*>(h->stw_px) : reinterpret_cast<const cplx<T>*>(h->stw_px64);
  if (sizeof(T) == 8)
    for (const FftPlan* p : {&py, &px})
      for (int s = 0; s < p->nst; ++s)
        if (p->R[s] > 9) {
          h->err = "x/y transforms: radix above 9 in an FP64 plan";
          return CHF_E_INVALID;
        }
  const int kxb = own && h->tune.kxb ? h->tune.kxb : pick_kxb<T>(d);
  const int xr = own && h->tune.xr ? h->tune.xr : pick_xr<T>(d);
  if (!kxb || !xr) {
    h->err = "x/y transforms: FFT length too large for the launch shapes";
    return CHF_E_INVALID;
  }
  {
    const size_t smem = y_smem<T>(d, kxb);
    if (!set_smem(h, k_yinv<T>, smem)) return CHF_E_CUDA;
    dim3 grid(d.KX / kxb, d.MP, 6);
    cudaEvent_t ev;
    prof_begin(h, K_YINV, &ev);
    k_yinv<T><<<grid, Y_THREADS, smem, st>>>(wz, wy, d, kxb, py, stw_py);
    prof_end(h, K_YINV, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_yinv")) return CHF_E_CUDA;
  }
  {
    int rc = xr == 8 ? run_xprod<T, 8>(h, wy, px, stw_px)
           : xr == 4 ? run_xprod<T, 4>(h, wy, px, stw_px)
           : xr == 2 ? run_xprod<T, 2>(h, wy, px, stw_px)
                     : run_xprod<T, 1>(h, wy, px, stw_px);
    if (rc != CHF_OK) return rc;
  }
  {
    const size_t smem = y_smem<T>(d, kxb);
    if (!set_smem(h, k_yfwd<T>, smem)) return CHF_E_CUDA;
    dim3 grid(d.KX / kxb, d.MP, 3);
    T scale = (T)(1.0 / ((double)d.PX * (double)d.PY));
    cudaEvent_t ev;
    prof_begin(h, K_YFWD, &ev);
    k_yfwd<T><<<grid, Y_THREADS, smem, st>>>(wy, wz, d, kxb, py, stw_py, scale);
    prof_end(h, K_YFWD, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_yfwd")) return CHF_E_CUDA;
  }
  return CHF_OK;
}

template int launch_xy<double>(Handle*, cd*, cd*, const cd*, const cd*);
template int launch_xy<float>(Handle*, cf*, cf*, const cf*, const cf*);

int launch_nonlinear_fp64(Handle* h) {
  const Dims& d = h->d;
  // z inverse of the six fields u, v, w, ox, oy, oz
  const int zl = h->tune.zl_c2v ? h->tune.zl_c2v : pick_zl_c2v(d);
  const int zc = h->tune.zl_curl ? h->tune.zl_curl : pick_zl_curl(d);
  if (!zl || !zc) {
    h->err = "z transforms: FFT length too large for the launch shapes";
    return CHF_E_INVALID;
  }
  int rc = zl == 8 ? run_zc2v<8>(h) : zl == 4 ? run_zc2v<4>(h) : run_zc2v<2>(h);
  if (rc != CHF_OK) return rc;
  rc = launch_xy<double>(h, h->wz, h->wy, h->tw_py, h->tw_px);
  if (rc != CHF_OK) return rc;
  rc = zc == 8 ? run_zcurl<8>(h) : zc == 4 ? run_zcurl<4>(h) : run_zcurl<2>(h);
  if (rc != CHF_OK) return rc;
  std::swap(h->f[F_U], h->f[F_RV]);
  std::swap(h->f[F_W], h->f[F_RG]);
  return CHF_OK;
}

// The Lamb vector of the current state (velocities and vorticities, as
// after a solve) as Chebyshev coefficients hc = 3 x [NZ][modes], FP64; the
// work buffers wz / wy must exist.  For the pressure (chf_pressure).
int launch_lamb_fp64(Handle* h, cd* hc) {
  const Dims& d = h->d;
  const int zl = h->tune.zl_c2v ? h->tune.zl_c2v : pick_zl_c2v(d);
  if (!zl) {
    h->err = "z transforms: FFT length too large for the launch shapes";
    return CHF_E_INVALID;
  }
  int rc = zl == 8 ? run_zc2v<8>(h) : zl == 4 ? run_zc2v<4>(h) : run_zc2v<2>(h);
  if (rc != CHF_OK) return rc;
  rc = launch_xy<double>(h, h->wz, h->wy, h->tw_py, h->tw_px);
  if (rc != CHF_OK) return rc;
  const size_t smem = zc2v_smem(d, zl);
  auto kern = zl == 8 ? k_zfwd<4, 8> : zl == 4 ? k_zfwd<4, 4> : k_zfwd<4, 2>;
  if (!set_smem(h, kern, smem)) return CHF_E_CUDA;
  dim3 grid((unsigned)((d.modes() + zl - 1) / zl), 3);
  kern<<<grid, ZC_THREADS, smem, h->stream>>>(h->wz, hc, d, h->pzm, h->tw_zm);
  return cuda_ok(h, cudaGetLastError(), "k_zfwd") ? CHF_OK : CHF_E_CUDA;
}

}  // namespace chf
