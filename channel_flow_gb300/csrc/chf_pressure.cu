// chf_pressure.cu -- pressure recovery from the current velocity field.
//
// The reference's pressure routine (instantp, poiseuilleflow.f90:3701-3890)
// is never called and works with finite differences; this is a spectral
// replacement in the discretisation of the time step.  The momentum
// equation of the time step is u_t = -H - grad P + (1/re) lap u, with H the
// Lamb vector of getnonlinear (REF:1380-1612, including -re_p in H1) and P
// the total head p + |u|^2 / 2 (rotational form).  Its divergence and its
// wall-normal component at the walls (u = 0) give, per Fourier mode,
//   (D^2 - k^2) P = -(i alpha H1 + D H2 + i beta H3)        at the interior
//   D P = -H2 + (1/re) (D^2 - k^2) v                        at z = +1, -1
// solved by Chebyshev collocation at the Gauss-Lobatto points (the grid of
// the implicit solves), in the even / odd blocks of the mirror symmetry
// z -> -z.  The (0,0) mode has D P = -H2 (no mean wall-normal velocity):
// P_00 is its Chebyshev antiderivative with zero mean over the channel.
// All FP64, for either precision of the handle; the FP64 nonlinear-term
// kernels supply H.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

namespace {

constexpr int PL = 4;          // modes per CTA in the right-hand-side kernel
constexpr int P_THREADS = 256;
constexpr int PCH = 8;         // modes per elimination pass in the solve kernel

// b = dz a (REF:570-599), serial recurrence, real sequences with strides
__device__ void deriv_serial(const double* a, int as, double* b, int bs, int N) {
  double bp1 = 0.0, bp2 = 0.0;  // b_{k+1}, b_{k+2}
  for (int k = N; k >= 0; --k) {
    const double bk = (k == N) ? 0.0 : bp2 + 2.0 * (double)(k + 1) * a[(k + 1) * as];
    b[k * bs] = bk;
    bp2 = bp1;
    bp1 = bk;
  }
  b[0] *= 0.5;
}

// right-hand sides at the Gauss-Lobatto points; R[0] and R[N] carry the
// Neumann data of z = +1 and z = -1.  grid (ceil(modes / PL))
template <int MB2>
__global__ void __launch_bounds__(P_THREADS) k_p_rhs(const cd* __restrict__ hc, const cd* __restrict__ v,
                                                     const double* __restrict__ iapha,
                                                     const double* __restrict__ ibeta, double nu, Dims d,
                                                     const __grid_constant__ FftPlan pz2,
                                                     const cd* __restrict__ tw2, cd* __restrict__ R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = d.N, NZ = d.NZ, L2 = 2 * N;
  const long modes = d.modes();
  cd* lines = reinterpret_cast<cd*>(smem_raw);  // [PL][2N]
  cd* C = lines + PL * L2;                       // [4][PL][NZ]: H1, H2, H3, v
  cd* Dh2 = C + 4 * PL * NZ;                     // [PL][NZ]
  cd* Dv = Dh2 + PL * NZ;                        // [PL][NZ]
  cd* D2v = Dv + PL * NZ;                        // [PL][NZ]
  __shared__ double bc[PL][4];                   // top re, top im, bottom re, bottom im
  const long m0 = (long)blockIdx.x * PL;
  for (int t = threadIdx.x; t < 4 * PL * NZ; t += blockDim.x) {
    const int f = t / (PL * NZ), l = (t / NZ) % PL, n = t % NZ;
    const long m = m0 + l;
    cd x{0.0, 0.0};
    if (m < modes) x = (f < 3 ? hc + (size_t)f * NZ * modes : v)[(size_t)n * modes + m];
    C[t] = x;
  }
  __syncthreads();
  if (threadIdx.x < 2 * PL) {  // (mode, re/im): D H2 and D^2 v
    const int l = threadIdx.x / 2, c = threadIdx.x % 2;
    const double* h2 = reinterpret_cast<const double*>(C + (1 * PL + l) * NZ) + c;
    const double* vv = reinterpret_cast<const double*>(C + (3 * PL + l) * NZ) + c;
    deriv_serial(h2, 2, reinterpret_cast<double*>(Dh2 + l * NZ) + c, 2, N);
    deriv_serial(vv, 2, reinterpret_cast<double*>(Dv + l * NZ) + c, 2, N);
    deriv_serial(reinterpret_cast<const double*>(Dv + l * NZ) + c, 2,
                 reinterpret_cast<double*>(D2v + l * NZ) + c, 2, N);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < PL * NZ; t += blockDim.x) {
    const int l = t / NZ, n = t % NZ;
    const long m = m0 + l;
    double a = 0.0, b = 0.0;
    if (m < modes) {
      a = iapha[m % d.KX];
      b = ibeta[m / d.KX];
    }
    const cd h1 = C[(0 * PL + l) * NZ + n], h3 = C[(2 * PL + l) * NZ + n], dh2 = Dh2[l * NZ + n];
    // g = -(i a H1 + D H2 + i b H3)
    const cd g{a * h1.im - dh2.re + b * h3.im, -a * h1.re - dh2.im - b * h3.re};
    const double dbl = (n == 0 || n == N) ? 2.0 : 1.0;
    lines[l * L2 + n] = cd{dbl * g.re, dbl * g.im};
    if (n > 0 && n < N) lines[l * L2 + L2 - n] = g;
  }
  if (threadIdx.x < 4 * PL) {  // Neumann data: sums over n with (+1)^n and (-1)^n
    const int l = threadIdx.x / 4, q = threadIdx.x % 4, c = q & 1, bottom = q >> 1;
    const long m = m0 + l;
    double k2 = 0.0;
    if (m < modes) {
      const double a = iapha[m % d.KX], b = ibeta[m / d.KX];
      k2 = a * a + b * b;
    }
    double s = 0.0;
    for (int n = 0; n < NZ; ++n) {
      const double sg = (bottom && (n & 1)) ? -1.0 : 1.0;
      const double h2 = reinterpret_cast<const double*>(C + (1 * PL + l) * NZ + n)[c];
      const double vn = reinterpret_cast<const double*>(C + (3 * PL + l) * NZ + n)[c];
      const double d2 = reinterpret_cast<const double*>(D2v + l * NZ + n)[c];
      s += sg * (-h2 + nu * (d2 - k2 * vn));
    }
    bc[l][q] = s;
  }
  __syncthreads();
  smem_fft<double, -1, MB2>(lines, PL, L2, pz2, tw2);
  for (int t = threadIdx.x; t < PL * NZ; t += blockDim.x) {
    const int l = t / NZ, j = t % NZ;
    const long m = m0 + l;
    if (m >= modes) continue;
    cd r;
    if (j == 0) r = cd{bc[l][0], bc[l][1]};
    else if (j == N) r = cd{bc[l][2], bc[l][3]};
    else r = cd{0.5 * lines[l * L2 + j].re, 0.5 * lines[l * L2 + j].im};
    R[(size_t)j * modes + m] = r;
  }
}

// Gauss-Jordan elimination with partial pivoting of the augmented n x (n + w)
// matrix A (row-major, row stride ld) by the whole CTA; the solution replaces
// the last w columns.  Returns false (CTA-uniform) on a zero pivot.
__device__ bool gauss_jordan(double* A, int n, int w, int ld) {
  __shared__ int s_piv;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(A[k * ld + k]);
      for (int r = k + 1; r < n; ++r)
        if (fabs(A[r * ld + k]) > best) {
          best = fabs(A[r * ld + k]);
          p = r;
        }
      s_piv = best > 0.0 ? p : -1;
    }
    __syncthreads();
    const int p = s_piv;
    if (p < 0) return false;
    if (p != k)
      for (int c = threadIdx.x; c < n + w; c += blockDim.x) {
        const double t = A[k * ld + c];
        A[k * ld + c] = A[p * ld + c];
        A[p * ld + c] = t;
      }
    __syncthreads();
    const double inv = 1.0 / A[k * ld + k];
    __syncthreads();
    for (int c = k + threadIdx.x; c < n + w; c += blockDim.x) A[k * ld + c] *= inv;
    __syncthreads();
    // columns right of k (the multipliers A[r][k] stay unchanged meanwhile),
    // then column k itself
    const int wc = n + w - k - 1;
    for (int t = threadIdx.x; t < n * wc; t += blockDim.x) {
      const int r = t / wc, c = k + 1 + t % wc;
      if (r != k) A[r * ld + c] -= A[r * ld + k] * A[k * ld + c];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x)
      if (r != k) A[r * ld + k] = 0.0;
    __syncthreads();
  }
  return true;
}

// one CTA per k^2 group (modes sharing the operator), PCH modes per pass
__global__ void __launch_bounds__(P_THREADS) k_p_solve(const cd* __restrict__ R, cd* __restrict__ P,
                                                       const double* __restrict__ t0, const double* __restrict__ t2,
                                                       const double* __restrict__ k2vals,
                                                       const int* __restrict__ group_start,
                                                       const int* __restrict__ group_modes, Dims d,
                                                       int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = d.N, Z = d.NZ, ne = N / 2 + 1, no = N / 2, w = 2 * PCH;
  const long modes = d.modes();
  double* Ae = reinterpret_cast<double*>(smem_raw);  // [ne][ne + w]
  double* Ao = Ae + (size_t)ne * (ne + w);           // [no][no + w]
  const int g = blockIdx.x;
  const double k2 = k2vals[g];
  const int gs = group_start[g], ge = group_start[g + 1];
  auto op = [&](int j, int n) { return t2[j + (size_t)Z * n] - k2 * t0[j + (size_t)Z * n]; };
  for (int base = gs; base < ge; base += PCH) {
    const int nm = min(PCH, ge - base);
    // even block: rows j = 1..N/2 (sums of the mirror rows), then D P(+1) - D P(-1)
    for (int t = threadIdx.x; t < ne * (ne + w); t += blockDim.x) {
      const int i = t / (ne + w), c = t % (ne + w);
      double x = 0.0;
      if (c < ne) {
        x = (i < ne - 1) ? op(i + 1, 2 * c) : (double)(2 * c) * (double)(2 * c);
      } else {
        const int q = (c - ne) / 2, part = (c - ne) % 2;
        if (q < nm) {
          const int m = group_modes[base + q];
          const double* r = reinterpret_cast<const double*>(R + m);
          const size_t st = (size_t)2 * modes;  // doubles between GL points
          x = (i < ne - 1) ? 0.5 * (r[(size_t)(i + 1) * st + part] + r[(size_t)(N - i - 1) * st + part])
                           : 0.5 * (r[part] - r[(size_t)N * st + part]);
        }
      }
      Ae[t] = x;
    }
    // odd block: rows j = 1..N/2 - 1 (differences), then D P(+1) + D P(-1)
    for (int t = threadIdx.x; t < no * (no + w); t += blockDim.x) {
      const int i = t / (no + w), c = t % (no + w);
      double x = 0.0;
      if (c < no) {
        x = (i < no - 1) ? op(i + 1, 2 * c + 1) : (double)(2 * c + 1) * (double)(2 * c + 1);
      } else {
        const int q = (c - no) / 2, part = (c - no) % 2;
        if (q < nm) {
          const int m = group_modes[base + q];
          const double* r = reinterpret_cast<const double*>(R + m);
          const size_t st = (size_t)2 * modes;
          x = (i < no - 1) ? 0.5 * (r[(size_t)(i + 1) * st + part] - r[(size_t)(N - i - 1) * st + part])
                           : 0.5 * (r[part] + r[(size_t)N * st + part]);
        }
      }
      Ao[t] = x;
    }
    __syncthreads();
    const bool ok = gauss_jordan(Ae, ne, w, ne + w) && gauss_jordan(Ao, no, w, no + w);
    if (!ok) {
      if (threadIdx.x == 0) atomicExch(status, 1);
      return;
    }
    for (int t = threadIdx.x; t < nm * Z; t += blockDim.x) {
      const int q = t / Z, n = t % Z;
      const int m = group_modes[base + q];
      const double* row = (n % 2 == 0) ? Ae + (size_t)(n / 2) * (ne + w) + ne : Ao + (size_t)(n / 2) * (no + w) + no;
      P[(size_t)n * modes + m] = cd{row[2 * q], row[2 * q + 1]};
    }
    __syncthreads();
  }
}

// (0,0) mode: P = -antiderivative of H2_00, zero mean over z
__global__ void k_p_mean(const cd* __restrict__ hc, cd* __restrict__ P, Dims d) {
  if (threadIdx.x >= 2) return;
  const int N = d.N, c = threadIdx.x;
  const long modes = d.modes();
  const double* a = reinterpret_cast<const double*>(hc + (size_t)1 * d.NZ * modes) + c;  // H2, mode 0
  const size_t st = (size_t)2 * modes;
  double* out = reinterpret_cast<double*>(P) + c;
  double mean = 0.0;
  for (int n = 1; n <= N; ++n) {
    const double am1 = a[(size_t)(n - 1) * st] * (n == 1 ? 2.0 : 1.0);
    const double ap1 = n + 1 <= N ? a[(size_t)(n + 1) * st] : 0.0;
    const double b = -(am1 - ap1) / (2.0 * n);
    out[(size_t)n * st] = b;
    if (n % 2 == 0) mean += b / (1.0 - (double)n * n);
  }
  out[0] = -mean;
}

}  // namespace

extern "C" int chf_pressure(chf_handle* h, double* p_out) {
  if (!h || !p_out) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = "chf_pressure before chf_upload_state";
    return CHF_E_STATE;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  const Dims& d = h->d;
  const int N = d.N, NZ = d.NZ;
  const long modes = d.modes();
  // FP64 work buffers of the nonlinear term (a mixed handle has none yet)
  if (!h->wz && !cuda_ok(h, cudaMalloc((void**)&h->wz, sizeof(cd) * 6 * (size_t)d.MP * modes), "pressure work"))
    return CHF_E_NOMEM;
  if (!h->wy &&
      !cuda_ok(h, cudaMalloc((void**)&h->wy, sizeof(cd) * 6 * (size_t)d.MP * d.PY * d.KX), "pressure work"))
    return CHF_E_NOMEM;
  if (!h->pres_buf &&
      !cuda_ok(h, cudaMalloc(&h->pres_buf, sizeof(cd) * 5 * (size_t)NZ * modes + sizeof(int)), "pressure buffer"))
    return CHF_E_NOMEM;
  cd* hc = static_cast<cd*>(h->pres_buf);  // 3 x [NZ][modes]
  cd* R = hc + (size_t)3 * NZ * modes;
  cd* P = R + (size_t)NZ * modes;
  int* status = reinterpret_cast<int*>(P + (size_t)NZ * modes);
  int rc = launch_lamb_fp64(h, hc);
  if (rc != CHF_OK) return rc;
  const int mb2 = fft_fits(PL, 2 * N, P_THREADS, 2) ? 2 : 4;
  if (!fft_fits(PL, 2 * N, P_THREADS, mb2)) {
    h->err = "chf_pressure: nnz too large";
    return CHF_E_INVALID;
  }
  const size_t smem1 = sizeof(cd) * ((size_t)PL * 2 * N + 7 * (size_t)PL * NZ);
  auto rk = mb2 == 2 ? k_p_rhs<2> : k_p_rhs<4>;
  const int ne = N / 2 + 1, no = N / 2;
  const size_t smem2 = sizeof(double) * ((size_t)ne * (ne + 2 * PCH) + (size_t)no * (no + 2 * PCH));
  if (!cuda_ok(h, cudaFuncSetAttribute(rk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1), "p smem") ||
      !cuda_ok(h, cudaFuncSetAttribute(k_p_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2),
               "p smem") ||
      !cuda_ok(h, cudaMemsetAsync(P, 0, sizeof(cd) * (size_t)NZ * modes + sizeof(int), h->stream), "p clear"))
    return CHF_E_CUDA;
  rk<<<(unsigned)((modes + PL - 1) / PL), P_THREADS, smem1, h->stream>>>(
      hc, h->f[F_V], h->iapha, h->ibeta, 1.0 / h->cfg.re, d, h->pz2, h->tw_z2, R);
  k_p_solve<<<h->nk2, P_THREADS, smem2, h->stream>>>(R, P, h->t0, h->t2, h->k2vals, h->group_start,
                                                     h->group_modes, d, status);
  k_p_mean<<<1, 32, 0, h->stream>>>(hc, P, d);
  if (!cuda_ok(h, cudaGetLastError(), "pressure kernels")) return CHF_E_CUDA;
  int st = 0;
  if (!cuda_ok(h, cudaMemcpyAsync(p_out, P, sizeof(cd) * (size_t)NZ * modes, cudaMemcpyDeviceToHost, h->stream),
               "pressure download") ||
      !cuda_ok(h, cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "pressure status") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "pressure sync"))
    return CHF_E_CUDA;
  if (st) {
    h->err = "pressure operator is singular for some k^2";
    return CHF_E_NUMERIC;
  }
  return CHF_OK;
}
