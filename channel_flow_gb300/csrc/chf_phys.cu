// chf_phys.cu -- the physical-space side of statistics, on the device.
//
//   chf_transform          transform (poiseuilleflow.f90:919-1005) with
//                          fourtrx_zcomp (poiseuilleflow.f90:774-913): one
//                          array between the spectral layout and the
//                          unpadded physical grid, in either direction
//   chf_cfl                CFL_X, CFL_Y, CFL_Z of statistics
//                          (poiseuilleflow.f90:2866-2934)
//   chf_physical_velocity  the instantaneous physical velocity of the
//                          3Ddata dump (poiseuilleflow.f90:2745-2764)
//   chf_write_velocity     that dump as the reference writes it, one file per
//                          rank, read by post-processing/post_poiseuilleflow.f90:63-70
//
// All FP64 for either precision of the handle.  The physical grid is the
// unpadded one of transform: x_i = 2 pi aphi i / nnx, y_j = 2 pi beta j / nny,
// z_k = cos(pi k / nz), stored [k][j][i] (Fortran (0:nx,0:ny,0:nz), one
// rank).  Three passes, each in place on one field-sized buffer:
//   z  per spectral mode: Chebyshev coefficients <-> Gauss-Lobatto values by
//      the even extension of length 2 nz and one forward DFT (REF:936-962,
//      971-1001);
//   y  per (plane, group of streamwise modes): backward DFT of length nny
//      with the spanwise Nyquist mode zeroed (REF:796-818), or forward DFT
//      and 1 / (nnx nny) (REF:888-911);
//   x  per pair of (plane, y) rows: Hermitian c2r of length nnx with the
//      streamwise Nyquist zeroed (getall, REF:836-852; two real rows per
//      complex DFT), or r2c keeping modes 0 .. nnx/2 - 1 (REF:868-879).
// The reference moves the data between ranks with its pencil transposes in
// between; on one GPU each pass walks the contiguous index of its layout
// instead.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

namespace {

constexpr int PH_THREADS = 256;
constexpr int PH_MB2 = 4;  // radix-2 butterflies per thread (fft_fits bound)
constexpr size_t kMaxSmem = 227 * 1024;

// ---------------------------------------------------------------------------
// z: per spectral mode m (ZL consecutive modes per CTA), in place on
// a[n * modes + m], n = 0..N.
//   DIR = +1: u_k = sum_n c_n cos(pi n k / N): sequence (2 c_0, c_1 .. c_{N-1},
//             2 c_N, c_{N-1} .. c_1), forward DFT, / 2
//   DIR = -1: c_k = (1 / N) sum over the even extension of u, forward DFT;
//             c_0 and c_N halved
// ---------------------------------------------------------------------------
template <int MB2, int ZL, int DIR>
__global__ void __launch_bounds__(PH_THREADS) k_ph_z(cd* __restrict__ a, long modes, int N,
                                                     const __grid_constant__ FftPlan pz, const cd* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int L = 2 * N, NZ = N + 1;
  const long m0 = (long)blockIdx.x * ZL;
  for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
    const int l = t % ZL, n = t / ZL;
    const long m = m0 + l;
    cd c{0.0, 0.0};
    if (m < modes) c = a[(size_t)n * modes + m];
    if (DIR > 0 && (n == 0 || n == N)) c = cd{2.0 * c.re, 2.0 * c.im};
    s[l * L + n] = c;
    if (n > 0 && n < N) s[l * L + L - n] = c;
  }
  __syncthreads();
  smem_fft<double, -1, MB2>(s, ZL, L, pz, tw);
  for (int t = threadIdx.x; t < ZL * NZ; t += blockDim.x) {
    const int l = t % ZL, n = t / ZL;
    const long m = m0 + l;
    if (m >= modes) continue;
    cd v = s[l * L + n];
    if (DIR > 0) {
      v = cd{v.re / 2.0, v.im / 2.0};
    } else {
      v = cd{v.re / (double)N, v.im / (double)N};
      if (n == 0 || n == N) v = cd{v.re / 2.0, v.im / 2.0};
    }
    a[(size_t)n * modes + m] = v;
  }
}

// ---------------------------------------------------------------------------
// y: per (plane k, kxb streamwise modes), in place on a[(k * nny + y) * KX + kx].
//   DIR = +1: backward DFT of length nny, spanwise Nyquist mode zeroed first
//   DIR = -1: forward DFT, / (nnx nny)
// grid (KX / kxb, NZ)
// ---------------------------------------------------------------------------
template <int MB2, int DIR>
__global__ void __launch_bounds__(PH_THREADS) k_ph_y(cd* __restrict__ a, int KX, int nny, int kxb, double norm,
                                                     const __grid_constant__ FftPlan py, const cd* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int ls = nny + 1;
  const int kx0 = blockIdx.x * kxb;
  cd* __restrict__ p = a + (size_t)blockIdx.y * nny * KX;
  for (int t = threadIdx.x; t < kxb * nny; t += blockDim.x) {
    const int l = t % kxb, y = t / kxb;
    cd c = p[(size_t)y * KX + kx0 + l];
    if (DIR > 0 && y == nny / 2) c = cd{0.0, 0.0};
    s[l * ls + y] = c;
  }
  __syncthreads();
  smem_fft<double, (DIR > 0 ? +1 : -1), MB2>(s, kxb, ls, py, tw);
  for (int t = threadIdx.x; t < kxb * nny; t += blockDim.x) {
    const int l = t % kxb, y = t / kxb;
    cd v = s[l * ls + y];
    if (DIR < 0) v = cd{v.re / norm, v.im / norm};
    p[(size_t)y * KX + kx0 + l] = v;
  }
}

// ---------------------------------------------------------------------------
// x: per pair of rows (2q, 2q + 1) of nnx doubles (XP pairs per CTA), in
// place.  A row holds KX = nnx / 2 complex modes (spectral side) or nnx real
// values (physical side); two real rows f, g travel as one complex line
// f + i g.
//   DIR = +1: line_j = F_j + i G_j, line_{nnx-j} = conj(F_j) + i conj(G_j),
//             line_0 = Re F_0 + i Re G_0, line_{KX} = 0; backward DFT;
//             f = Re, g = Im
//   DIR = -1: forward DFT Z of f + i g; F_j = (Z_j + conj Z_{-j}) / 2,
//             G_j = (Z_j - conj Z_{-j}) / 2i, j = 0 .. KX - 1
// ---------------------------------------------------------------------------
template <int MB2, int XP, int DIR>
__global__ void __launch_bounds__(PH_THREADS) k_ph_x(double* __restrict__ a, long npairs, int nnx,
                                                     const __grid_constant__ FftPlan px, const cd* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cd* s = reinterpret_cast<cd*>(smem_raw);
  const int KX = nnx / 2, ls = nnx + 1;
  const long p0 = (long)blockIdx.x * XP;
  if (DIR > 0) {
    for (int t = threadIdx.x; t < XP * KX; t += blockDim.x) {
      const int j = t % KX, q = t / KX;
      const long pr = p0 + q;
      if (pr >= npairs) continue;
      const cd f = reinterpret_cast<const cd*>(a + (size_t)(2 * pr) * nnx)[j];
      const cd g = reinterpret_cast<const cd*>(a + (size_t)(2 * pr + 1) * nnx)[j];
      cd* line = s + q * ls;
      if (j == 0) {
        line[0] = cd{f.re, g.re};
        line[KX] = cd{0.0, 0.0};
      } else {
        line[j] = cd{f.re - g.im, f.im + g.re};
        line[nnx - j] = cd{f.re + g.im, g.re - f.im};
      }
    }
  } else {
    for (int t = threadIdx.x; t < XP * nnx; t += blockDim.x) {
      const int x = t % nnx, q = t / nnx;
      const long pr = p0 + q;
      if (pr >= npairs) continue;
      s[q * ls + x] = cd{a[(size_t)(2 * pr) * nnx + x], a[(size_t)(2 * pr + 1) * nnx + x]};
    }
  }
  __syncthreads();
  smem_fft<double, (DIR > 0 ? +1 : -1), MB2>(s, XP, ls, px, tw);
  if (DIR > 0) {
    for (int t = threadIdx.x; t < XP * nnx; t += blockDim.x) {
      const int x = t % nnx, q = t / nnx;
      const long pr = p0 + q;
      if (pr >= npairs) continue;
      const cd v = s[q * ls + x];
      a[(size_t)(2 * pr) * nnx + x] = v.re;
      a[(size_t)(2 * pr + 1) * nnx + x] = v.im;
    }
  } else {
    for (int t = threadIdx.x; t < XP * KX; t += blockDim.x) {
      const int j = t % KX, q = t / KX;
      const long pr = p0 + q;
      if (pr >= npairs) continue;
      const cd A = s[q * ls + j];
      cd B = s[q * ls + (j == 0 ? 0 : nnx - j)];
      B.im = -B.im;
      reinterpret_cast<cd*>(a + (size_t)(2 * pr) * nnx)[j] = cd{0.5 * (A.re + B.re), 0.5 * (A.im + B.im)};
      reinterpret_cast<cd*>(a + (size_t)(2 * pr + 1) * nnx)[j] = cd{0.5 * (A.im - B.im), -0.5 * (A.re - B.re)};
    }
  }
}

// Per plane k (one CTA each): max |u|, max |v|, max |w| over the nnx x nny
// physical points of that plane -> mx[3 k + c].
__global__ void __launch_bounds__(PH_THREADS) k_ph_planemax(const double* __restrict__ u, const double* __restrict__ v,
                                                            const double* __restrict__ w, long plane,
                                                            double* __restrict__ mx) {
  const size_t base = (size_t)blockIdx.x * plane;
  double m[3] = {0.0, 0.0, 0.0};
  for (long i = threadIdx.x; i < plane; i += blockDim.x) {
    m[0] = fmax(m[0], fabs(u[base + i]));
    m[1] = fmax(m[1], fabs(v[base + i]));
    m[2] = fmax(m[2], fabs(w[base + i]));
  }
  __shared__ double sm[3][PH_THREADS / 32];
  for (int c = 0; c < 3; ++c) {
    for (int off = 16; off > 0; off >>= 1) m[c] = fmax(m[c], __shfl_down_sync(0xffffffffu, m[c], off));
    if ((threadIdx.x & 31) == 0) sm[c][threadIdx.x >> 5] = m[c];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double r = 0.0;
    for (int q = 0; q < PH_THREADS / 32; ++q) r = fmax(r, sm[threadIdx.x][q]);
    mx[3 * (size_t)blockIdx.x + threadIdx.x] = r;
  }
}

template <typename K>
bool set_smem(Handle* h, K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  return cuda_ok(h, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                 "physical-space smem");
}

// Launch shapes: the most lines per CTA whose butterflies fit PH_MB2 per
// thread and whose lines fit in shared memory.
int pick_zl(const Dims& d) {
  for (int l = 8; l >= 1; l /= 2)
    if (fft_fits(l, 2 * d.N, PH_THREADS, PH_MB2) && sizeof(cd) * l * 2 * d.N <= kMaxSmem) return l;
  return 0;
}
int pick_kxb(const Dims& d) {
  for (int b = 8; b >= 1; b /= 2)
    if (d.KX % b == 0 && fft_fits(b, d.nny, PH_THREADS, PH_MB2) && sizeof(cd) * b * (d.nny + 1) <= kMaxSmem)
      return b;
  return 0;
}
int pick_xp(const Dims& d) {
  for (int p = 4; p >= 1; p /= 2)
    if (fft_fits(p, d.nnx, PH_THREADS, PH_MB2) && sizeof(cd) * p * (d.nnx + 1) <= kMaxSmem) return p;
  return 0;
}

template <int DIR, int ZL>
int run_z(Handle* h, cd* buf) {
  const Dims& d = h->d;
  const size_t smem = sizeof(cd) * ZL * 2 * d.N;
  if (!set_smem(h, k_ph_z<PH_MB2, ZL, DIR>, smem)) return CHF_E_CUDA;
  k_ph_z<PH_MB2, ZL, DIR><<<(unsigned)((d.modes() + ZL - 1) / ZL), PH_THREADS, smem, h->stream>>>(
      buf, d.modes(), d.N, h->pz2, h->tw_z2);
  return cuda_ok(h, cudaGetLastError(), "k_ph_z") ? CHF_OK : CHF_E_CUDA;
}

template <int DIR>
int run_y(Handle* h, cd* buf) {
  const Dims& d = h->d;
  const int kxb = pick_kxb(d);
  const size_t smem = sizeof(cd) * kxb * (d.nny + 1);
  if (!set_smem(h, k_ph_y<PH_MB2, DIR>, smem)) return CHF_E_CUDA;
  k_ph_y<PH_MB2, DIR><<<dim3(d.KX / kxb, d.NZ), PH_THREADS, smem, h->stream>>>(
      buf, d.KX, d.nny, kxb, (double)d.nnx * (double)d.nny, h->pyu, h->tw_pyu);
  return cuda_ok(h, cudaGetLastError(), "k_ph_y") ? CHF_OK : CHF_E_CUDA;
}

template <int DIR, int XP>
int run_x(Handle* h, cd* buf) {
  const Dims& d = h->d;
  const long npairs = (long)d.NZ * d.nny / 2;
  const size_t smem = sizeof(cd) * XP * (d.nnx + 1);
  if (!set_smem(h, k_ph_x<PH_MB2, XP, DIR>, smem)) return CHF_E_CUDA;
  k_ph_x<PH_MB2, XP, DIR><<<(unsigned)((npairs + XP - 1) / XP), PH_THREADS, smem, h->stream>>>(
      reinterpret_cast<double*>(buf), npairs, d.nnx, h->pxu, h->tw_pxu);
  return cuda_ok(h, cudaGetLastError(), "k_ph_x") ? CHF_OK : CHF_E_CUDA;
}

template <int DIR>
int run_zl(Handle* h, cd* buf, int zl) {
  return zl == 8 ? run_z<DIR, 8>(h, buf) : zl == 4 ? run_z<DIR, 4>(h, buf) : zl == 2 ? run_z<DIR, 2>(h, buf)
                                                                                       : run_z<DIR, 1>(h, buf);
}
template <int DIR>
int run_xp(Handle* h, cd* buf, int xp) {
  return xp == 4 ? run_x<DIR, 4>(h, buf) : xp == 2 ? run_x<DIR, 2>(h, buf) : run_x<DIR, 1>(h, buf);
}

// transform(isign) in place on one field-sized device buffer
int transform_dev(Handle* h, int isign, cd* buf) {
  const Dims& d = h->d;
  const int zl = pick_zl(d), kxb = pick_kxb(d), xp = pick_xp(d);
  if (!zl || !kxb || !xp) {
    h->err = "physical transform: line length too large for the launch shapes";
    return CHF_E_INVALID;
  }
  int rc;
  if (isign > 0) {
    if ((rc = run_zl<+1>(h, buf, zl)) != CHF_OK || (rc = run_y<+1>(h, buf)) != CHF_OK) return rc;
    return run_xp<+1>(h, buf, xp);
  }
  if ((rc = run_xp<-1>(h, buf, xp)) != CHF_OK || (rc = run_y<-1>(h, buf)) != CHF_OK) return rc;
  return run_zl<-1>(h, buf, zl);
}

// First use: three field-sized buffers and NZ x 3 plane maxima, the nnx- and
// nny-point plans and their twiddles.
int ensure_phys(Handle* h) {
  if (h->phys_buf) return CHF_OK;
  const Dims& d = h->d;
  const size_t fb = sizeof(cd) * d.field_elems();
  if (!cuda_ok(h, cudaMalloc(&h->phys_buf, 3 * fb + sizeof(double) * 3 * (size_t)d.NZ), "physical buffers"))
    return CHF_E_NOMEM;
  h->pxu = make_plan(d.nnx);
  h->pyu = make_plan(d.nny);
  struct {
    cd** dst;
    int L;
  } tws[] = {{&h->tw_pxu, d.nnx}, {&h->tw_pyu, d.nny}};
  for (auto& t : tws) {
    std::vector<cd> v = twiddles(t.L);
    if (!cuda_ok(h, cudaMalloc((void**)t.dst, sizeof(cd) * v.size()), "twiddle alloc") ||
        !cuda_ok(h, cudaMemcpy(*t.dst, v.data(), sizeof(cd) * v.size(), cudaMemcpyHostToDevice), "twiddle upload"))
      return CHF_E_CUDA;
  }
  return CHF_OK;
}

cd* phys_field(Handle* h, int i) {
  return reinterpret_cast<cd*>(static_cast<char*>(h->phys_buf) + (size_t)i * sizeof(cd) * h->d.field_elems());
}

// u, v, w of the resident state on the physical grid in phys_field 0, 1, 2
int velocity_to_physical(Handle* h) {
  int rc = ensure_phys(h);
  if (rc != CHF_OK) return rc;
  const size_t fb = sizeof(cd) * h->d.field_elems();
  const int src[3] = {F_U, F_V, F_W};
  for (int i = 0; i < 3; ++i) {
    if (!cuda_ok(h, cudaMemcpyAsync(phys_field(h, i), h->f[src[i]], fb, cudaMemcpyDeviceToDevice, h->stream),
                 "physical copy"))
      return CHF_E_CUDA;
    if ((rc = transform_dev(h, +1, phys_field(h, i))) != CHF_OK) return rc;
  }
  return CHF_OK;
}

int begin(chf_handle* h, const char* what) {
  if (!h) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = std::string(what) + " before chf_upload_state";
    return CHF_E_STATE;
  }
  return cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice") ? CHF_OK : CHF_E_CUDA;
}

// host: (u + u0(k), w, v) of the physical grid into out[(m, k, j, i)], the
// order of the reference's ftmp(i, j, k, m) (Fortran, i fastest)
int physical_velocity_host(Handle* h, const double* u0, double* out) {
  const Dims& d = h->d;
  const size_t n = 2 * d.field_elems();  // doubles per field = nnx nny NZ
  int rc = velocity_to_physical(h);
  if (rc != CHF_OK) return rc;
  const int order[3] = {0, 2, 1};  // u, w, v
  for (int m = 0; m < 3; ++m)
    if (!cuda_ok(h, cudaMemcpyAsync(out + m * n, phys_field(h, order[m]), sizeof(double) * n,
                                    cudaMemcpyDeviceToHost, h->stream),
                 "physical download"))
      return CHF_E_CUDA;
  if (!cuda_ok(h, cudaStreamSynchronize(h->stream), "physical sync")) return CHF_E_CUDA;
  if (u0) {
    const size_t plane = (size_t)d.nnx * d.nny;
    for (int k = 0; k < d.NZ; ++k)
      for (size_t i = 0; i < plane; ++i) out[(size_t)k * plane + i] += u0[k];
  }
  return CHF_OK;
}

}  // namespace

extern "C" {

int chf_transform(chf_handle* h, int isign, double* u) {
  if (!h || !u || (isign != 1 && isign != -1)) {
    if (h) h->err = "chf_transform: isign must be 1 or -1 and u non-NULL";
    return CHF_E_INVALID;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  int rc = ensure_phys(h);
  if (rc != CHF_OK) return rc;
  const size_t fb = sizeof(cd) * h->d.field_elems();
  cd* buf = phys_field(h, 0);
  if (!cuda_ok(h, cudaMemcpyAsync(buf, u, fb, cudaMemcpyHostToDevice, h->stream), "transform upload")) return CHF_E_CUDA;
  if ((rc = transform_dev(h, isign, buf)) != CHF_OK) return rc;
  if (!cuda_ok(h, cudaMemcpyAsync(u, buf, fb, cudaMemcpyDeviceToHost, h->stream), "transform download") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "transform sync"))
    return CHF_E_CUDA;
  return CHF_OK;
}

int chf_cfl(chf_handle* h, double* cfl_x, double* cfl_y, double* cfl_z) {
  int rc = begin(h, "chf_cfl");
  if (rc != CHF_OK) return rc;
  if ((rc = velocity_to_physical(h)) != CHF_OK) return rc;
  const Dims& d = h->d;
  double* mx = reinterpret_cast<double*>(phys_field(h, 3));
  k_ph_planemax<<<d.NZ, PH_THREADS, 0, h->stream>>>(
      reinterpret_cast<const double*>(phys_field(h, 0)), reinterpret_cast<const double*>(phys_field(h, 1)),
      reinterpret_cast<const double*>(phys_field(h, 2)), (long)d.nnx * d.nny, mx);
  if (!cuda_ok(h, cudaGetLastError(), "k_ph_planemax")) return CHF_E_CUDA;
  std::vector<double> m(3 * (size_t)d.NZ);
  if (!cuda_ok(h, cudaMemcpyAsync(m.data(), mx, sizeof(double) * m.size(), cudaMemcpyDeviceToHost, h->stream),
               "cfl download") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "cfl sync"))
    return CHF_E_CUDA;
  // spacings of statistics (REF:2868-2876): dx, ddz (spanwise) uniform; the
  // Gauss-Lobatto spacing dy(k) = cos((k-1) pi / nz) - cos(k pi / nz),
  // k = 1..nz/2, mirrored
  const double pi2 = 8.0 * std::atan(1.0), ddy = 4.0 * std::atan(1.0) / (double)d.N;
  const double dx = h->cfg.aphi * pi2 / (double)d.nnx, ddz = h->cfg.beta * pi2 / (double)d.nny;
  const double dt = h->cfg.dt;
  std::vector<double> dy(d.N + 1, 0.0);
  for (int k = 1; k <= d.N / 2; ++k) {
    dy[k] = -(std::cos((double)k * ddy) - std::cos((double)(k - 1) * ddy));
    dy[d.N - k] = dy[k];
  }
  double umax = 0.0, wmax = 0.0, cy = 0.0;
  for (int k = 0; k <= d.N; ++k) {
    umax = std::fmax(umax, m[3 * (size_t)k + 0]);
    wmax = std::fmax(wmax, m[3 * (size_t)k + 2]);
    if (k >= 1 && k <= d.N - 1) cy = std::fmax(cy, m[3 * (size_t)k + 1] * dt / dy[k]);
  }
  if (cfl_x) *cfl_x = umax * dt / dx;
  if (cfl_y) *cfl_y = cy;
  if (cfl_z) *cfl_z = wmax * dt / ddz;
  return CHF_OK;
}

int chf_physical_velocity(chf_handle* h, const double* u0, double* out) {
  int rc = begin(h, "chf_physical_velocity");
  if (rc != CHF_OK) return rc;
  if (!out) {
    h->err = "chf_physical_velocity: out is NULL";
    return CHF_E_INVALID;
  }
  return physical_velocity_host(h, u0, out);
}

int chf_write_velocity(chf_handle* h, const char* dir, int nproc, int istep, const double* u0) {
  int rc = begin(h, "chf_write_velocity");
  if (rc != CHF_OK) return rc;
  const Dims& d = h->d;
  if (nproc < 1 || nproc > 999 || istep < 0 || istep > 99999999) {
    h->err = "chf_write_velocity: nproc must be 1..999 and istep 0..99999999";
    return CHF_E_INVALID;
  }
  // the reference's decomposition (paraandcons.f90:5-8): nnx / nproc
  // physical x points per rank, nny / 2 divisible by nproc
  if (d.nnx % (2 * nproc) != 0 || (d.nny / 2) % nproc != 0) {
    h->err = "chf_write_velocity: nnx must be a multiple of 2 nproc and nny / 2 a multiple of nproc";
    return CHF_E_INVALID;
  }
  const int w = d.nnx / nproc;
  const uint64_t rec = 3ull * (uint64_t)w * d.nny * d.NZ * sizeof(double);
  if (rec > 0x7FFFFFF0ull) {
    h->err = "chf_write_velocity: a record above 2 GiB needs more ranks (subrecords are not written)";
    return CHF_E_INVALID;
  }
  const size_t n = 2 * d.field_elems();
  std::vector<double> all(3 * n);
  if ((rc = physical_velocity_host(h, u0, all.data())) != CHF_OK) return rc;
  std::string base = dir && *dir ? dir : ".";
  if (base.back() != '/') base += '/';
  for (int r = 0; r < nproc; ++r) {
    char name[64];
    std::snprintf(name, sizeof name, "velocity%08d.%03d.dat", istep, r);  // format 212, REF:2750
    const std::string path = base + name;
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
      h->err = "chf_write_velocity: cannot create " + path;
      return CHF_E_INVALID;
    }
    const uint32_t mark = (uint32_t)rec;  // 4-byte record length, little-endian host
    bool ok = std::fwrite(&mark, 4, 1, f) == 1;
    for (int m = 0; ok && m < 3; ++m)
      for (int k = 0; ok && k < d.NZ; ++k)
        for (int j = 0; ok && j < d.nny; ++j) {
          const double* row = all.data() + m * n + ((size_t)k * d.nny + j) * d.nnx + (size_t)r * w;
          ok = std::fwrite(row, sizeof(double), w, f) == (size_t)w;
        }
    ok = ok && std::fwrite(&mark, 4, 1, f) == 1;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
      h->err = "chf_write_velocity: write failed on " + path;
      return CHF_E_INVALID;
    }
  }
  return CHF_OK;
}

}  // extern "C"
