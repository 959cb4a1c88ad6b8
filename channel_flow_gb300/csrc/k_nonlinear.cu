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

namespace chf {

namespace {

constexpr int ZC_LINES = 8;      // modes per CTA in the z kernels
constexpr int ZC_THREADS = 512;
constexpr int Y_THREADS = 256;
constexpr int X_ROWS = 8;        // (plane, y) rows per CTA in k_xprod
constexpr int X_THREADS = 512;

struct SixPtr {
  const cd* p[6];
};

// ---------------------------------------------------------------------------
// z: coefficients -> values at z'_p = cos(pi p / MZ), p = 0..MZ.
// Even extension of length 2 MZ with doubled first entry, forward DFT, /2
// (the packed evaluation of getlamb, REF:1672-1683, applied per field).
// grid (ceil(modes / ZC_LINES), 6)
// ---------------------------------------------------------------------------
template <int MB2>
__global__ void __launch_bounds__(ZC_THREADS) k_zc2v(SixPtr in, cd* __restrict__ out, Dims d,
                                                     const __grid_constant__ FftPlan pz, const cd* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int L = 2 * d.MZ, ls = L;
  const long modes = d.modes();
  const long m0 = (long)blockIdx.x * ZC_LINES;
  const int f = blockIdx.y;
  const cd* __restrict__ src = in.p[f];
  for (int t = threadIdx.x; t < ZC_LINES * L; t += blockDim.x) s[t] = cd{0.0, 0.0};
  __syncthreads();
  for (int t = threadIdx.x; t < ZC_LINES * d.NZ; t += blockDim.x) {
    int l = t % ZC_LINES, n = t / ZC_LINES;
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
  smem_fft<double, -1, MB2>(s, ZC_LINES, ls, pz, tw);
  cd* __restrict__ dst = out + (size_t)f * d.MP * modes;
  for (int t = threadIdx.x; t < ZC_LINES * d.MP; t += blockDim.x) {
    int l = t % ZC_LINES, p = t / ZC_LINES;
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
template <typename T, int MB2>
__global__ void __launch_bounds__(Y_THREADS) k_yinv(const cplx<T>* __restrict__ wz, cplx<T>* __restrict__ wy,
                                                    Dims d, int kxb, const __grid_constant__ FftPlan py,
                                                    const cplx<T>* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smem_raw);
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
  smem_fft<T, +1, MB2>(s, kxb, ls, py, tw);
  cplx<T>* __restrict__ dst = wy + ((size_t)f * d.MP + p) * (size_t)d.PY * d.KX;
  for (int t = threadIdx.x; t < kxb * d.PY; t += blockDim.x) {
    int l = t % kxb, yp = t / kxb;
    dst[(size_t)yp * d.KX + kx0 + l] = s[l * ls + yp];
  }
}

// ---------------------------------------------------------------------------
// x: fused c2r, products, r2c.  Rows r = p * PY + yp; each row holds KX modes
// of six fields (u, v, w, ox, oy, oz), written back in place as H1, H2, H3
// into field slots 0, 1, 2.  grid (ceil(MP * PY / X_ROWS))
// ---------------------------------------------------------------------------
template <typename T, int MB2>
__global__ void __launch_bounds__(X_THREADS) k_xprod(cplx<T>* __restrict__ wy, Dims d, T re_p,
                                                     const __grid_constant__ FftPlan px, const cplx<T>* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using C = cplx<T>;
  C* s = reinterpret_cast<C*>(smem_raw);
  const int PX = d.PX, KX = d.KX, ls = PX + 1;
  const long nrows = (long)d.MP * d.PY;
  const long r0 = (long)blockIdx.x * X_ROWS;
  const size_t fstride = (size_t)d.MP * d.PY * KX;
  // lines: row q, pair c (0: u+iv, 1: w+i ox, 2: oy+i oz) at (c*X_ROWS + q) * ls
  for (int t = threadIdx.x; t < X_ROWS * 3 * ls; t += blockDim.x) s[t] = C{(T)0, (T)0};
  __syncthreads();
  for (int t = threadIdx.x; t < X_ROWS * 3 * KX; t += blockDim.x) {
    int k = t % KX, c = (t / KX) % 3, q = t / (3 * KX);
    long r = r0 + q;
    if (r >= nrows) continue;
    C F = wy[(size_t)(2 * c) * fstride + (size_t)r * KX + k];
    C G = wy[(size_t)(2 * c + 1) * fstride + (size_t)r * KX + k];
    C* line = s + (c * X_ROWS + q) * ls;
    if (k == 0) {
      line[0] = C{F.re, G.re};  // imaginary part of the streamwise mean dropped
    } else {
      line[k] = C{F.re - G.im, F.im + G.re};        // F + i G
      line[PX - k] = C{F.re + G.im, G.re - F.im};   // conj(F) + i conj(G)
    }
  }
  __syncthreads();
  smem_fft<T, +1, MB2>(s, X_ROWS * 3, ls, px, tw);
  // products at every physical point; write (H1 + i H2) to pair 0, (H3 + 0i) to pair 1
  for (int t = threadIdx.x; t < X_ROWS * PX; t += blockDim.x) {
    int x = t % PX, q = t / PX;
    C a = s[(0 * X_ROWS + q) * ls + x];  // u, v
    C b = s[(1 * X_ROWS + q) * ls + x];  // w, ox
    C c = s[(2 * X_ROWS + q) * ls + x];  // oy, oz
    T u = a.re, v = a.im, w = b.re, ox = b.im, oy = c.re, oz = c.im;
    T h1 = (oy * w - re_p) - oz * v;
    T h2 = oz * u - ox * w;
    T h3 = ox * v - oy * u;
    s[(0 * X_ROWS + q) * ls + x] = C{h1, h2};
    s[(1 * X_ROWS + q) * ls + x] = C{h3, (T)0};
  }
  __syncthreads();
  // forward DFT of the 2 * X_ROWS lines holding (H1 + i H2) and H3
  smem_fft<T, -1, MB2>(s, X_ROWS * 2, ls, px, tw);
  for (int t = threadIdx.x; t < X_ROWS * KX; t += blockDim.x) {
    int k = t % KX, q = t / KX;
    long r = r0 + q;
    if (r >= nrows) continue;
    const C* z = s + (0 * X_ROWS + q) * ls;
    C A = z[k];
    C B = z[k == 0 ? 0 : PX - k];
    B.im = -B.im;  // conj(Z[-k])
    C H1{(T)0.5 * (A.re + B.re), (T)0.5 * (A.im + B.im)};
    C H2{(T)0.5 * (A.im - B.im), (T)-0.5 * (A.re - B.re)};
    C H3 = s[(1 * X_ROWS + q) * ls + k];
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
template <typename T, int MB2>
__global__ void __launch_bounds__(Y_THREADS) k_yfwd(const cplx<T>* __restrict__ wy, cplx<T>* __restrict__ wz,
                                                    Dims d, int kxb, const __grid_constant__ FftPlan py,
                                                    const cplx<T>* __restrict__ tw, T scale) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* s = reinterpret_cast<cplx<T>*>(smem_raw);
  const int ls = d.PY + 1;
  const int f = blockIdx.z, p = blockIdx.y, kx0 = blockIdx.x * kxb;
  const long modes = d.modes();
  const cplx<T>* __restrict__ src = wy + ((size_t)f * d.MP + p) * (size_t)d.PY * d.KX;
  for (int t = threadIdx.x; t < kxb * d.PY; t += blockDim.x) {
    int l = t % kxb, yp = t / kxb;
    s[l * ls + yp] = src[(size_t)yp * d.KX + kx0 + l];
  }
  __syncthreads();
  smem_fft<T, -1, MB2>(s, kxb, ls, py, tw);
  cplx<T>* __restrict__ dst = wz + ((size_t)f * d.MP + p) * modes;
  for (int t = threadIdx.x; t < kxb * d.KY; t += blockDim.x) {
    int l = t % kxb, ky = t / kxb;
    int slot = ky <= d.NYQ ? ky : d.PY - d.KY + ky;
    cplx<T> v = s[l * ls + slot];
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
// grid (ceil(modes / ZC_LINES))
// shared: FFT buffer ZC_LINES x 2MZ, coefficient store 3 x ZC_LINES x NZ,
//         derivative store 2 x ZC_LINES x NZ
// ---------------------------------------------------------------------------
template <int MB2>
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
  const int fb = max(ZC_LINES * ls, 2 * ZC_LINES * L2);  // FFT buffer elements
  cd* coef = s + fb;                     // [3][ZC_LINES][NZ]
  double* der = reinterpret_cast<double*>(coef + 3 * ZC_LINES * NZ);  // [4][ZC_LINES][NZ]
  const long modes = d.modes();
  const long m0 = (long)blockIdx.x * ZC_LINES;
  const double inv_mz = 1.0 / (double)d.MZ;
  for (int f = 0; f < 3; ++f) {
    const cd* __restrict__ src = wz + (size_t)f * d.MP * modes;
    for (int t = threadIdx.x; t < ZC_LINES * d.MP; t += blockDim.x) {
      int l = t % ZC_LINES, p = t / ZC_LINES;
      long m = m0 + l;
      cd v{0.0, 0.0};
      if (m < modes) v = src[(size_t)p * modes + m];
      s[l * ls + p] = v;
      if (p > 0 && p < d.MZ) s[l * ls + L - p] = v;
    }
    __syncthreads();
    smem_fft<double, -1, MB2>(s, ZC_LINES, ls, pzm, twm);
    for (int t = threadIdx.x; t < ZC_LINES * NZ; t += blockDim.x) {
      int l = t % ZC_LINES, n = t / ZC_LINES;
      cd v = s[l * ls + n];
      double sc = (n == 0) ? 0.5 * inv_mz : inv_mz;
      coef[(f * ZC_LINES + l) * NZ + n] = cd{v.re * sc, v.im * sc};
    }
    __syncthreads();
  }
  // omega_x <- H1, omega_z <- H3 (the reference leaves them there, REF:1489-1496)
  for (int t = threadIdx.x; t < ZC_LINES * NZ; t += blockDim.x) {
    int l = t % ZC_LINES, n = t / ZC_LINES;
    long m = m0 + l;
    if (m >= modes) continue;
    ox_out[(size_t)n * modes + m] = coef[(0 * ZC_LINES + l) * NZ + n];
    oz_out[(size_t)n * modes + m] = coef[(2 * ZC_LINES + l) * NZ + n];
  }
  // derivatives of H1 and H3 (re, im): 4 serial recurrences per line
  if (threadIdx.x < 4 * ZC_LINES) {
    int l = threadIdx.x % ZC_LINES, which = threadIdx.x / ZC_LINES;  // 0:H1re 1:H1im 2:H3re 3:H3im
    const cd* c = coef + ((which < 2 ? 0 : 2) * ZC_LINES + l) * NZ;
    const double* a = reinterpret_cast<const double*>(c) + (which & 1);
    cheb_deriv_serial(a, 2, der + (which * ZC_LINES + l) * NZ, 1, N);
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
  for (int t = threadIdx.x; t < ZC_LINES * NZ; t += blockDim.x) {
    int l = t % ZC_LINES, n = t / ZC_LINES;
    long m = m0 + l;
    int kx = (int)(m % d.KX), ky = (int)(m / d.KX);
    double a = 0.0, b = 0.0;
    if (m < modes) { a = iapha[kx]; b = ibeta[ky]; }
    double k2 = a * a + b * b;
    cd h1 = coef[(0 * ZC_LINES + l) * NZ + n];
    cd h2 = coef[(1 * ZC_LINES + l) * NZ + n];
    cd h3 = coef[(2 * ZC_LINES + l) * NZ + n];
    double d1r = der[(0 * ZC_LINES + l) * NZ + n], d1i = der[(1 * ZC_LINES + l) * NZ + n];
    double d3r = der[(2 * ZC_LINES + l) * NZ + n], d3i = der[(3 * ZC_LINES + l) * NZ + n];
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
  smem_fft<double, -1, MB2>(s, ZC_LINES * 2, L2, pz2, tw2);
  for (int t = threadIdx.x; t < ZC_LINES * NZ; t += blockDim.x) {
    int l = t % ZC_LINES, n = t / ZC_LINES;
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

template <typename K>
bool set_smem(Handle* h, K kernel, size_t bytes) {
  if (bytes > 48 * 1024)
    return cuda_ok(h, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes),
                   "cudaFuncSetAttribute");
  return true;
}

int pick_kxb(int KX) {
  for (int b = 16; b > 1; b /= 2)
    if (KX % b == 0) return b;
  return 1;
}

}  // namespace

template <typename T>
int launch_xy(Handle* h, cplx<T>* wz, cplx<T>* wy, const cplx<T>* tw_py, const cplx<T>* tw_px) {
  const Dims& d = h->d;
  cudaStream_t st = h->stream;
  const int kxb = pick_kxb(d.KX);
  {
    if (!fft_fits(kxb, d.PY, Y_THREADS, 6)) {
      h->err = "k_yinv: FFT length too large for the launch shape";
      return CHF_E_INVALID;
    }
    size_t smem = sizeof(cplx<T>) * kxb * (d.PY + 1);
    if (!set_smem(h, k_yinv<T, 6>, smem)) return CHF_E_CUDA;
    dim3 grid(d.KX / kxb, d.MP, 6);
    cudaEvent_t ev;
    prof_begin(h, K_YINV, &ev);
    k_yinv<T, 6><<<grid, Y_THREADS, smem, st>>>(wz, wy, d, kxb, h->py, tw_py);
    prof_end(h, K_YINV, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_yinv")) return CHF_E_CUDA;
  }
  {
    if (!fft_fits(X_ROWS * 3, d.PX, X_THREADS, 5)) {
      h->err = "k_xprod: FFT length too large for the launch shape";
      return CHF_E_INVALID;
    }
    size_t smem = sizeof(cplx<T>) * X_ROWS * 3 * (d.PX + 1);
    if (!set_smem(h, k_xprod<T, 5>, smem)) return CHF_E_CUDA;
    long nrows = (long)d.MP * d.PY;
    dim3 grid((unsigned)((nrows + X_ROWS - 1) / X_ROWS));
    cudaEvent_t ev;
    prof_begin(h, K_XPROD, &ev);
    k_xprod<T, 5><<<grid, X_THREADS, smem, st>>>(wy, d, (T)h->cfg.re_p, h->px, tw_px);
    prof_end(h, K_XPROD, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_xprod")) return CHF_E_CUDA;
  }
  {
    size_t smem = sizeof(cplx<T>) * kxb * (d.PY + 1);
    if (!set_smem(h, k_yfwd<T, 6>, smem)) return CHF_E_CUDA;
    dim3 grid(d.KX / kxb, d.MP, 3);
    T scale = (T)(1.0 / ((double)d.PX * (double)d.PY));
    cudaEvent_t ev;
    prof_begin(h, K_YFWD, &ev);
    k_yfwd<T, 6><<<grid, Y_THREADS, smem, st>>>(wy, wz, d, kxb, h->py, tw_py, scale);
    prof_end(h, K_YFWD, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_yfwd")) return CHF_E_CUDA;
  }
  return CHF_OK;
}

template int launch_xy<double>(Handle*, cd*, cd*, const cd*, const cd*);
template int launch_xy<float>(Handle*, cf*, cf*, const cf*, const cf*);

int launch_nonlinear_fp64(Handle* h) {
  const Dims& d = h->d;
  cudaStream_t st = h->stream;
  const long modes = d.modes();
  // z inverse, six fields: u, v, w, ox, oy, oz
  {
    SixPtr in{{h->f[F_U], h->f[F_V], h->f[F_W], h->f[F_OX], h->f[F_OY], h->f[F_OZ]}};
    const int L = 2 * d.MZ;
    if (!fft_fits(ZC_LINES, L, ZC_THREADS, 4)) {
      h->err = "k_zc2v: FFT length too large for the launch shape";
      return CHF_E_INVALID;
    }
    size_t smem = sizeof(cd) * ZC_LINES * L;
    if (!set_smem(h, k_zc2v<4>, smem)) return CHF_E_CUDA;
    dim3 grid((unsigned)((modes + ZC_LINES - 1) / ZC_LINES), 6);
    cudaEvent_t ev;
    prof_begin(h, K_ZC2V, &ev);
    k_zc2v<4><<<grid, ZC_THREADS, smem, st>>>(in, h->wz, d, h->pzm, h->tw_zm);
    prof_end(h, K_ZC2V, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_zc2v")) return CHF_E_CUDA;
  }
  {
    int rc = launch_xy<double>(h, h->wz, h->wy, h->tw_py, h->tw_px);
    if (rc != CHF_OK) return rc;
  }
  {
    const int L = 2 * d.MZ;
    if (!fft_fits(ZC_LINES, L, ZC_THREADS, 4) || !fft_fits(2 * ZC_LINES, 2 * d.N, ZC_THREADS, 4)) {
      h->err = "k_zcurl: FFT length too large for the launch shape";
      return CHF_E_INVALID;
    }
    size_t fb = (size_t)std::max(ZC_LINES * L, 2 * ZC_LINES * 2 * d.N);
    size_t smem = sizeof(cd) * fb + sizeof(cd) * 3 * ZC_LINES * d.NZ +
                  sizeof(double) * 4 * ZC_LINES * d.NZ;
    if (!set_smem(h, k_zcurl<4>, smem)) return CHF_E_CUDA;
    dim3 grid((unsigned)((modes + ZC_LINES - 1) / ZC_LINES));
    // h_v -> the unp1 buffer, h_g -> the wnp1 buffer; swapped with rhsvn /
    // rhsomegayn below (REF:1542-1558)
    cudaEvent_t ev;
    prof_begin(h, K_ZCURL, &ev);
    k_zcurl<4><<<grid, ZC_THREADS, smem, st>>>(
        h->wz, h->f[F_U], h->f[F_W], h->f[F_OX], h->f[F_OZ], h->mean[M_CL1N], h->mean[M_CL1NM1],
        h->mean[M_CL3N], h->mean[M_CL3NM1], h->iapha, h->ibeta, d, h->pzm, h->tw_zm, h->pz2,
        h->tw_z2);
    prof_end(h, K_ZCURL, ev);
    if (!cuda_ok(h, cudaGetLastError(), "k_zcurl")) return CHF_E_CUDA;
  }
  std::swap(h->f[F_U], h->f[F_RV]);
  std::swap(h->f[F_W], h->f[F_RG]);
  return CHF_OK;
}

}  // namespace chf
