// chf_stats.cu -- flow statistics on the GPU (statistics, poiseuilleflow.f90:2666-3198).
//
// The reference transforms u, v, w to the physical nnx x nny x (nz+1) grid
// (transform(1), unpadded) at every outputstep and forms, per Gauss-Lobatto
// plane z_k, the plane means <u>, <v>, <w> and the covariances
// <u'u'>, <v'v'>, <w'w'>, <u'v'>, <u'w'>, <v'w'> (:2945-3060), the physical
// kinetic energy sum (:2786-2800) and from these the wall shear velocities,
// Re_tau, Re_c and Re_b (:3150-3190).  Plane averages of products of
// band-limited fields are exact spectral sums (Parseval; the products
// cannot alias onto the zero mode because the spanwise Nyquist slot is
// empty), so here they are computed without any in-plane transform:
//   <f'g'>(z_k) = sum over modes (kx, ky) != (0, 0) of w_kx Re(f^(z_k) conj(g^(z_k))),
// with w_kx = 1 for kx = 0 and 2 for kx > 0 (the half spectrum in x), and
// <f>(z_k) = Re f^_{00}(z_k).  The only transform is Chebyshev coefficients
// -> Gauss-Lobatto values, one 2N-point DFT per (field, mode) line.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

namespace {

constexpr int ST_LINES = 4;    // (field, mode) lines per CTA
constexpr int ST_THREADS = 256;
constexpr int NSTAT = 10;      // per plane: <u>,<v>,<w>, uu,vv,ww, uv,uw,vw, energy density

// GL values of u, v, w (fields 0..2) for every mode: out[f][k][mode]
template <int MB2>
__global__ void __launch_bounds__(ST_THREADS) k_stat_gl(const cd* __restrict__ u, const cd* __restrict__ v,
                                                       const cd* __restrict__ w, cd* __restrict__ out, Dims d,
                                                       const __grid_constant__ FftPlan pz2,
                                                       const cd* __restrict__ tw2) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int N = d.N, NZ = d.NZ, L2 = 2 * N;
  const long modes = d.modes(), lines = 3 * modes;
  const long l0 = (long)blockIdx.x * ST_LINES;
  for (int t = threadIdx.x; t < ST_LINES * NZ; t += blockDim.x) {
    const int l = t / NZ, n = t % NZ;
    const long line = l0 + l;
    cd c{0.0, 0.0};
    if (line < lines) {
      const int f = (int)(line / modes);
      const long m = line % modes;
      const cd* src = f == 0 ? u : f == 1 ? v : w;
      c = src[(size_t)n * modes + m];
    }
    // even extension with doubled end coefficients: 0.5 DFT = values at z_k
    const double dbl = (n == 0 || n == N) ? 2.0 : 1.0;
    s[l * L2 + n] = cd{dbl * c.re, dbl * c.im};
    if (n > 0 && n < N) s[l * L2 + L2 - n] = c;
  }
  __syncthreads();
  smem_fft<double, -1, MB2>(s, ST_LINES, L2, pz2, tw2);
  for (int t = threadIdx.x; t < ST_LINES * NZ; t += blockDim.x) {
    const int l = t / NZ, k = t % NZ;
    const long line = l0 + l;
    if (line >= lines) continue;
    const int f = (int)(line / modes);
    const long m = line % modes;
    const cd x = s[l * L2 + k];
    out[((size_t)f * NZ + k) * modes + m] = cd{0.5 * x.re, 0.5 * x.im};
  }
}

// one CTA per plane k: means, covariances and sum_modes w (|u|^2+|v|^2+|w|^2)
__global__ void __launch_bounds__(ST_THREADS) k_stat_sum(const cd* __restrict__ gl, Dims d, double* __restrict__ out) {
  const int k = blockIdx.x, NZ = d.NZ;
  const long modes = d.modes();
  const cd* U = gl + ((size_t)0 * NZ + k) * modes;
  const cd* V = gl + ((size_t)1 * NZ + k) * modes;
  const cd* W = gl + ((size_t)2 * NZ + k) * modes;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};  // uu vv ww uv uw vw energy
  for (long m = threadIdx.x; m < modes; m += blockDim.x) {
    const int kx = (int)(m % d.KX), ky = (int)(m / d.KX);
    if (ky == d.NYQ) continue;
    const double wt = kx == 0 ? 1.0 : 2.0;
    const cd a = U[m], b = V[m], c = W[m];
    const double ea = a.re * a.re + a.im * a.im, eb = b.re * b.re + b.im * b.im, ec = c.re * c.re + c.im * c.im;
    acc[6] += wt * (ea + eb + ec);
    if (m == 0) continue;  // the mean mode is not a fluctuation
    acc[0] += wt * ea;
    acc[1] += wt * eb;
    acc[2] += wt * ec;
    acc[3] += wt * (a.re * b.re + a.im * b.im);
    acc[4] += wt * (a.re * c.re + a.im * c.im);
    acc[5] += wt * (b.re * c.re + b.im * c.im);
  }
  __shared__ double red[ST_THREADS / 32][7];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    double x = acc[q];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    double x = 0.0;
    for (int q = 0; q < ST_THREADS / 32; ++q) x += red[q][threadIdx.x];
    out[(size_t)k * NSTAT + 3 + threadIdx.x] = x;
  }
  if (threadIdx.x == 0) {
    out[(size_t)k * NSTAT + 0] = U[0].re;
    out[(size_t)k * NSTAT + 1] = V[0].re;
    out[(size_t)k * NSTAT + 2] = W[0].re;
  }
}

}  // namespace

extern "C" int chf_statistics(chf_handle* h, double* profiles, chf_stats* out) {
  if (!h || !out) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = "chf_statistics before chf_upload_state";
    return CHF_E_STATE;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  const Dims& d = h->d;
  const int N = d.N, NZ = d.NZ;
  const long modes = d.modes();
  const size_t gl_elems = (size_t)3 * NZ * modes;
  if (!h->stats_buf) {  // first call: GL values of three fields + plane sums
    const size_t bytes = sizeof(cd) * gl_elems + sizeof(double) * (size_t)NZ * NSTAT;
    if (!cuda_ok(h, cudaMalloc(&h->stats_buf, bytes), "statistics buffer")) return CHF_E_NOMEM;
  }
  cd* gl = static_cast<cd*>(h->stats_buf);
  double* sums = reinterpret_cast<double*>(gl + gl_elems);
  const int mb2 = fft_fits(ST_LINES, 2 * N, ST_THREADS, 2) ? 2 : 4;
  if (!fft_fits(ST_LINES, 2 * N, ST_THREADS, mb2)) {
    h->err = "chf_statistics: nnz too large";
    return CHF_E_INVALID;
  }
  const size_t smem = sizeof(cd) * ST_LINES * 2 * N;
  auto kern = mb2 == 2 ? k_stat_gl<2> : k_stat_gl<4>;
  if (smem > 48 * 1024 &&
      !cuda_ok(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "stats smem"))
    return CHF_E_CUDA;
  const long lines = 3 * modes;
  kern<<<(unsigned)((lines + ST_LINES - 1) / ST_LINES), ST_THREADS, smem, h->stream>>>(
      h->f[F_U], h->f[F_V], h->f[F_W], gl, d, h->pz2, h->tw_z2);
  k_stat_sum<<<NZ, ST_THREADS, 0, h->stream>>>(gl, d, sums);
  if (!cuda_ok(h, cudaGetLastError(), "statistics kernels")) return CHF_E_CUDA;
  std::vector<double> S((size_t)NZ * NSTAT), au0(2 * (size_t)NZ);
  if (!cuda_ok(h, cudaMemcpyAsync(S.data(), sums, sizeof(double) * S.size(), cudaMemcpyDeviceToHost, h->stream),
               "statistics download") ||
      !cuda_ok(h, cudaMemcpyAsync(au0.data(), h->mean[M_AU0], sizeof(double) * au0.size(),
                                  cudaMemcpyDeviceToHost, h->stream),
               "statistics download") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "statistics sync"))
    return CHF_E_CUDA;
  const double re = h->cfg.re, pi = 3.14159265358979323846;
  std::vector<double> z(NZ);
  for (int k = 0; k < NZ; ++k) z[k] = std::cos(pi * k / N);
  // wall stress: d<u>/dz / re at z = +1 (k = 0) and z = -1 (k = nz), where the
  // Reynolds stress vanishes; T_n'(1) = n^2, T_n'(-1) = (-1)^(n+1) n^2
  double dtop = 0.0, dbot = 0.0, ub = 0.0;
  for (int n = 0; n < NZ; ++n) {
    const double a = au0[2 * n], n2 = (double)n * n;
    dtop += a * n2;
    dbot += ((n % 2) ? a : -a) * n2;
    if (n % 2 == 0) ub += a / (1.0 - n2);
  }
  out->u_tau_top = std::sqrt(std::fabs(dtop / re));
  out->u_tau_bottom = std::sqrt(std::fabs(dbot / re));
  out->re_tau_top = out->u_tau_top * re;
  out->re_tau_bottom = out->u_tau_bottom * re;
  out->re_centre = S[(size_t)(N / 2) * NSTAT + 0] * re;
  double ubr = 0.0;  // the reference's half-channel rectangle rule (:3176-3179)
  for (int k = N / 2; k <= N - 1; ++k) ubr += S[(size_t)k * NSTAT + 0] * std::fabs(z[k + 1] - z[k]);
  out->re_bulk = 2.0 * ubr * re;
  out->bulk_velocity = ub;
  double e = 0.0;
  for (int k = 0; k < NZ; ++k) e += S[(size_t)k * NSTAT + 9];
  out->energy = 0.5 * (double)d.nnx * (double)d.nny * e;
  if (profiles)
    for (int k = 0; k < NZ; ++k) {
      profiles[0 * NZ + k] = z[k];
      for (int q = 0; q < 9; ++q) profiles[(size_t)(q + 1) * NZ + k] = S[(size_t)k * NSTAT + q];
    }
  return CHF_OK;
}
