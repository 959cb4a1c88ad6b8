// k_solve_mixed.cu -- the implicit solve of the mixed path.
//
// The per-mode solve (poiseuilleflow.f90:242-394) for every (kx, ky) but the
// (0,0) mode, written as an FP64 state plus an increment:
//   x = c + delta,   delta = A^-1 (B - A) c + A^-1 r,
//   r = dt (3/2 N^n - 1/2 N^{n-1})
// on the collocation rows and 0 on the wall rows, with B - A =
// (dt/re) (D^2 - k^2)^2 for v and (dt/re) (D^2 - k^2) for omega_y (the CN
// operators of get_coef_v / get_coef_omegay and of get_coef_rhs /
// get_rhs_omegay, REF:3348-3489) and A^-1 the even/odd inverses of
// k_solve.cu.  Forming (B - A) c at the collocation points cancels heavily
// (fourth derivatives of the coefficients against an O(c) result), so the
// set-up multiplies it into the inverse once per k^2 in FP64:
// M = A^-1 (B - A) maps coefficients to coefficients and has no such
// cancellation (its rows sum to within ~10x of the result).  A step is then
//   k_inc_solve    one CTA per k^2 group: delta = M c (compensated FP32 on
//                  (hi, lo) splits of M and c, about 2^-44 relative) + A^-1 r
//                  (FP32), x = c + delta in FP64
//   k_inc_recover  u, w, omega_x, omega_z from v and omega_y (getvelocityandvorticity,
//                  REF:2347-2407), FP64, one thread per (mode, re/im)
// The (0,0) mode (REF:401-474) stays with k_solve (FP64, one CTA).
#include <cuda_runtime.h>

#include <algorithm>

#include "chf_internal.h"
#include "df32.cuh"

namespace chf {

namespace {

constexpr int I_THREADS = 256;
constexpr int MV_THREADS = 288;  // threads over the 2 NZ rows of one group's four blocks
constexpr int MCH = 4;           // modes per pass in k_inc_solve

// Chebyshev derivative recurrence (dz, REF:570-599), descending in k:
//   b_k = b_{k+2} + 2 (k+1) a_{k+1}   (b_0 is halved by the caller)
struct Rec {  // one recurrence: values at k+1 and k+2
  double b1 = 0.0, b2 = 0.0;
  __device__ __forceinline__ double step(double src_k1, int k, bool top) {
    const double b = top ? 0.0 : b2 + 2.0 * (double)(k + 1) * src_k1;
    b2 = b1;
    b1 = b;
    return b;
  }
};

constexpr int TM = 16;  // modes per CTA in k_inc_recover

// ---------------------------------------------------------------------------
// Set-up of the increment operators, grid (nk2, 4 blocks): with X = A^-1 the
// block's inverse (k_solve.cu, FP64) and W the folded rows of B - A,
//   W[q][c] = (dt/re) (T4 - 2 k^2 T2 + k^4 T0)(z_q, T_j)   (v)
//   W[q][c] = (dt/re) (T2 - k^2 T0)(z_q, T_j)               (omega_y)
// for q >= r0 (0 on the wall rows), j = 2c or 2c + 1, the kernel forms
// M = X W in FP64 (W staged BW columns at a time, X read through L1) and
// stores it as (hi, lo) float pairs, and X as floats; both column-major,
// M[c * n + r], at the inverses' block offsets.
// ---------------------------------------------------------------------------
constexpr int BW = 32;  // columns of W staged per pass in k_build_incr

__global__ void __launch_bounds__(256) k_build_incr(const double* __restrict__ t0,
                                                    const double* __restrict__ t2,
                                                    const double* __restrict__ t4,
                                                    const double* __restrict__ k2vals,
                                                    const double* __restrict__ xinv, SolveLayout sl, int N,
                                                    double dt_re, float2* __restrict__ incm,
                                                    float* __restrict__ incx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int g = blockIdx.x, blk = blockIdx.y, NZ = N + 1;
  const bool isv = blk < 2, even = (blk % 2) == 0;
  const int n = isv ? (even ? sl.ne_v : sl.no_v) : (even ? sl.ne_w : sl.no_w);
  const int r0 = isv ? 2 : 1;
  const BlockOffsets bo = block_offsets(sl);
  const size_t off = (size_t)g * sl.stride + (blk == 0 ? bo.ve : blk == 1 ? bo.vo : blk == 2 ? bo.we : bo.wo);
  const double* X = xinv + off;                     // column-major X[q * n + r]
  double* W = reinterpret_cast<double*>(smem_raw);  // W[q * BW + cc], column c0 + cc
  const double k2 = k2vals[g];
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) incx[off + t] = (float)X[t];
  for (int c0 = 0; c0 < n; c0 += BW) {
    const int nc = min(BW, n - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < n * BW; t += blockDim.x) {
      const int q = t / BW, cc = t % BW, j = even ? 2 * (c0 + cc) : 2 * (c0 + cc) + 1;
      double w = 0.0;
      if (q >= r0 && cc < nc) {
        const size_t p = (size_t)q + (size_t)NZ * j;
        w = isv ? dt_re * (t4[p] - 2.0 * k2 * t2[p] + k2 * k2 * t0[p]) : dt_re * (t2[p] - k2 * t0[p]);
      }
      W[t] = w;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * nc; t += blockDim.x) {
      const int cc = t / n, r = t % n;
      double acc = 0.0;
      for (int q = r0; q < n; ++q) acc = fma(X[(size_t)q * n + r], W[q * BW + cc], acc);
      const float hi = (float)acc;
      incm[off + (size_t)(c0 + cc) * n + r] = make_float2(hi, (float)(acc - (double)hi));
    }
  }
}

// ---------------------------------------------------------------------------
// k_inc_solve: one CTA per k^2 group (mean excluded), MCH modes of the group
// per pass.  Per mode the CTA stages in shared memory
//   * the coefficients c of v and omega_y as (hi, lo) floats, ordered as the
//     four blocks' columns (v even j, v odd j, omega even j, omega odd j);
//   * the AB2 term r = dt (3/2 N^n - 1/2 N^{n-1}) at the Gauss-Lobatto
//     points, folded (even rows 1/2 (r_p + r_{N-p}), odd rows
//     1/2 (r_p - r_{N-p}), p = row) with the wall rows zero, as floats;
// then one thread per block row forms
//   delta = M c + X r
// M c with compensated FP32 arithmetic (the exact product of the high parts
// added by TwoSum, the cross terms and rounding errors into a second
// accumulator; about 2^-44 relative), X r in plain FP32 (r is O(dt) and
// X r has no cancellation), and writes x = c + delta in FP64.
// ---------------------------------------------------------------------------
struct CoefHL {
  float hr, hi, lr, li;  // high and low parts of the real and imaginary parts
};

constexpr int CB = 4;  // matrix columns per load batch (two batches in flight)

// S + C += (mh + ml)(ch + cl), compensated: p + e = mh ch exactly, the cross
// terms join e, TwoSum keeps the rounding error of S + p.
__device__ __forceinline__ void comp_mac(float mh, float ml, float ch, float cl, float& S, float& C) {
  const float p = __fmul_rn(mh, ch);
  float e = __fmaf_rn(mh, ch, -p);
  e = __fmaf_rn(mh, cl, e);
  e = __fmaf_rn(ml, ch, e);
  const df32 sm = df_two_sum(S, p);
  S = sm.hi;
  C = __fadd_rn(C, __fadd_rn(sm.lo, e));
}

__global__ void __launch_bounds__(MV_THREADS, 3) k_inc_solve(cd* __restrict__ v, cd* __restrict__ g,
                                                             const cd* __restrict__ rv, const cd* __restrict__ uh,
                                                             const cd* __restrict__ rg, const cd* __restrict__ wh,
                                                             const float2* __restrict__ incm,
                                                             const float* __restrict__ incx, SolveLayout sl,
                                                             const int* __restrict__ group_start,
                                                             const int* __restrict__ group_modes, Dims d,
                                                             double c3, double c1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = d.N, NZ = d.NZ, ne = N / 2 + 1;
  const long modes = d.modes();
  cd* Cd = reinterpret_cast<cd*>(smem_raw);                   // [MCH][2 NZ] FP64 coefficients
  CoefHL* Cs = reinterpret_cast<CoefHL*>(Cd + MCH * 2 * NZ);  // [MCH][2 NZ] their (hi, lo) splits
  float2* Rs = reinterpret_cast<float2*>(Cs + MCH * 2 * NZ);  // [MCH][2 NZ] folded AB2 term
  __shared__ int s_mode[MCH];
  const int grp = blockIdx.x;
  const int gs = group_start[grp], ge = group_start[grp + 1];
  const int nev = sl.ne_v, nov = sl.no_v, new_ = sl.ne_w, now_ = sl.no_w;
  const int rows = nev + nov + new_ + now_;
  const BlockOffsets bo = block_offsets(sl);
  const float2* Mg = incm + (size_t)grp * sl.stride;
  const float* Xg = incx + (size_t)grp * sl.stride;
  for (int base = gs; base < ge; base += MCH) {
    const int nm = min(MCH, ge - base);
    if (threadIdx.x < nm) s_mode[threadIdx.x] = group_modes[base + threadIdx.x];
    __syncthreads();
    for (int e = threadIdx.x; e < nm * 2 * NZ; e += blockDim.x) {
      const int q = e / (2 * NZ), i = e % (2 * NZ), f = i / NZ, k = i % NZ;
      const cd x = (f == 0 ? v : g)[(size_t)k * modes + s_mode[q]];
      const float hr = (float)x.re, hi = (float)x.im;
      const int slot = q * 2 * NZ + f * NZ + ((k & 1) ? ne + k / 2 : k / 2);
      Cd[slot] = x;
      Cs[slot] = CoefHL{hr, hi, (float)(x.re - (double)hr), (float)(x.im - (double)hi)};
    }
    for (int e = threadIdx.x; e < nm * 2 * ne; e += blockDim.x) {
      const int q = e / (2 * ne), i = e % (2 * ne), f = i / ne, r = i % ne;
      const long m = s_mode[q];
      const cd* H = f == 0 ? rv : rg;   // N^n (GL values)
      const cd* Ho = f == 0 ? uh : wh;  // N^{n-1}
      const size_t ip = (size_t)r * modes + m, iq = (size_t)(N - r) * modes + m;
      const cd hp = H[ip], hq = H[iq], op = Ho[ip], oq = Ho[iq];
      const double pr = c3 * hp.re - c1 * op.re, pi = c3 * hp.im - c1 * op.im;
      const double qr = c3 * hq.re - c1 * oq.re, qi = c3 * hq.im - c1 * oq.im;
      const bool wall = (f == 0) ? (r < 2) : (r < 1);
      float2* out = Rs + q * 2 * NZ + f * NZ;
      out[r] = wall ? make_float2(0.f, 0.f) : make_float2((float)(0.5 * (pr + qr)), (float)(0.5 * (pi + qi)));
      if (r < N / 2)
        out[ne + r] = wall ? make_float2(0.f, 0.f) : make_float2((float)(0.5 * (pr - qr)), (float)(0.5 * (pi - qi)));
    }
    __syncthreads();
    for (int t = threadIdx.x; t < rows; t += blockDim.x) {
      int b, row, n;
      size_t boff;
      if (t < nev) { b = 0; row = t; n = nev; boff = bo.ve; }
      else if (t < nev + nov) { b = 1; row = t - nev; n = nov; boff = bo.vo; }
      else if (t < nev + nov + new_) { b = 2; row = t - nev - nov; n = new_; boff = bo.we; }
      else { b = 3; row = t - nev - nov - new_; n = now_; boff = bo.wo; }
      // offset of block b inside a mode's 2 NZ staged entries
      const int roff = b == 0 ? 0 : b == 1 ? nev : b == 2 ? NZ : NZ + new_;
      const float2* Mb = Mg + boff + row;
      const float* Xb = Xg + boff + row;
      float S[MCH][2], C[MCH][2], A[MCH][2];
#pragma unroll
      for (int q = 0; q < MCH; ++q)
        S[q][0] = S[q][1] = C[q][0] = C[q][1] = A[q][0] = A[q][1] = 0.f;
      // columns c < r0 of X meet the zero wall entries of the staged rhs
      float2 ma[CB];
      float xa[CB];
#pragma unroll
      for (int u = 0; u < CB; ++u) {
        ma[u] = u < n ? __ldg(Mb + (size_t)u * n) : make_float2(0.f, 0.f);
        xa[u] = u < n ? __ldg(Xb + (size_t)u * n) : 0.f;
      }
      for (int c0 = 0; c0 < n; c0 += CB) {
        float2 mb[CB];
        float xb[CB];
#pragma unroll
        for (int u = 0; u < CB; ++u) {
          const int c = c0 + CB + u;
          mb[u] = c < n ? __ldg(Mb + (size_t)c * n) : make_float2(0.f, 0.f);
          xb[u] = c < n ? __ldg(Xb + (size_t)c * n) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < CB; ++u) {
          if (c0 + u < n) {
#pragma unroll
            for (int q = 0; q < MCH; ++q) {
              if (q < nm) {
                const int si = q * 2 * NZ + roff + c0 + u;
                const CoefHL cc = Cs[si];
                const float2 rr = Rs[si];
                comp_mac(ma[u].x, ma[u].y, cc.hr, cc.lr, S[q][0], C[q][0]);
                comp_mac(ma[u].x, ma[u].y, cc.hi, cc.li, S[q][1], C[q][1]);
                A[q][0] = __fmaf_rn(xa[u], rr.x, A[q][0]);
                A[q][1] = __fmaf_rn(xa[u], rr.y, A[q][1]);
              }
            }
          }
        }
#pragma unroll
        for (int u = 0; u < CB; ++u) {
          ma[u] = mb[u];
          xa[u] = xb[u];
        }
      }
      const int j = (b == 0 || b == 2) ? 2 * row : 2 * row + 1;
      cd* dst = b < 2 ? v : g;
#pragma unroll
      for (int q = 0; q < MCH; ++q) {
        if (q < nm) {
          const cd c0 = Cd[q * 2 * NZ + roff + row];
          const double dr = (double)S[q][0] + ((double)C[q][0] + (double)A[q][0]);
          const double di = (double)S[q][1] + ((double)C[q][1] + (double)A[q][1]);
          dst[(size_t)j * modes + s_mode[q]] = cd{c0.re + dr, c0.im + di};
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// k_inc_recover: grid (ceil(modes / TM)); tiles of v and omega_y in shared
// memory, one thread per (mode, re/im) running one descending pass (the
// derivative recurrence), the other component from its partner lane:
//   Dv_k -> u_k = (i a Dv - i b g) / k^2, w_k = (i b Dv + i a g) / k^2
//   Du_k, Dw_k (from u, w at k+1) -> omega_z = -Du + i a v, omega_x = Dw - i b v
// for every solved mode (not (0,0), not the spanwise Nyquist slot).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(I_THREADS) k_inc_recover(const cd* __restrict__ v, const cd* __restrict__ g,
                                                           cd* __restrict__ u, cd* __restrict__ w,
                                                           cd* __restrict__ ox, cd* __restrict__ oz,
                                                           const double* __restrict__ iapha,
                                                           const double* __restrict__ ibeta, Dims d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = d.N, NZ = d.NZ, C2 = 2 * TM;
  const long modes = d.modes();
  double* V = reinterpret_cast<double*>(smem_raw);  // [NZ][C2]
  double* G = V + (size_t)NZ * C2;                  // [NZ][C2]
  const long m0 = (long)blockIdx.x * TM;
  for (int t = threadIdx.x; t < NZ * C2; t += blockDim.x) {
    const int c = t % C2, n = t / C2;
    const long col = 2 * m0 + c;
    const bool in = col < 2 * modes;
    V[t] = in ? reinterpret_cast<const double*>(v)[(size_t)n * 2 * modes + col] : 0.0;
    G[t] = in ? reinterpret_cast<const double*>(g)[(size_t)n * 2 * modes + col] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x >= C2) return;  // one warp: lanes 2l (re) and 2l+1 (im) of mode m0 + l
  const int c = threadIdx.x, comp = c & 1;
  const long m = m0 + c / 2;
  const bool live = m > 0 && m < modes && (m / d.KX) != d.NYQ;
  double a = 0.0, b = 0.0, ik2 = 0.0;
  if (live) {
    a = iapha[m % d.KX];
    b = ibeta[m / d.KX];
    ik2 = 1.0 / (a * a + b * b);
  }
  const double s = comp ? 1.0 : -1.0;  // multiplying by i: re <- -im, im <- +re
  Rec rv, ru, rw;
  double vk1 = 0.0, uk1 = 0.0, wk1 = 0.0;
  double* ud = reinterpret_cast<double*>(u);
  double* wd = reinterpret_cast<double*>(w);
  double* oxd = reinterpret_cast<double*>(ox);
  double* ozd = reinterpret_cast<double*>(oz);
  for (int k = N; k >= 0; --k) {
    const bool top = (k == N);
    const double vk = V[k * C2 + c], gk = G[k * C2 + c];
    const double h = k == 0 ? 0.5 : 1.0;
    const double dv = h * rv.step(vk1, k, top);
    const double du = h * ru.step(uk1, k, top);
    const double dw = h * rw.step(wk1, k, top);
    // partner components (the other of re / im of the same mode)
    const double dv_p = __shfl_xor_sync(0xffffffffu, dv, 1);
    const double g_p = __shfl_xor_sync(0xffffffffu, gk, 1);
    const double v_p = __shfl_xor_sync(0xffffffffu, vk, 1);
    // u = (i a Dv - i b g) / k^2, w = (i b Dv + i a g) / k^2: i x -> s x_partner
    const double uk = s * (a * dv_p - b * g_p) * ik2;
    const double wk = s * (b * dv_p + a * g_p) * ik2;
    if (live) {
      const size_t idx = ((size_t)k * modes + m) * 2 + comp;
      ud[idx] = uk;
      wd[idx] = wk;
      ozd[idx] = -du + s * a * v_p;  // omega_z = -Du + i a v
      oxd[idx] = dw - s * b * v_p;   // omega_x = Dw - i b v
    }
    vk1 = vk;
    uk1 = uk;
    wk1 = wk;
  }
}

}  // namespace

int setup_solver_mixed(Handle* h) {
  const SolveLayout& sl = h->sl;
  const size_t n = sl.stride * (size_t)h->nk2;
  if (n == 0) return CHF_OK;
  if (!cuda_ok(h, cudaMalloc((void**)&h->incm, sizeof(float2) * n), "increment operators") ||
      !cuda_ok(h, cudaMalloc((void**)&h->incx, sizeof(float) * n), "increment operators"))
    return CHF_E_NOMEM;
  const int nmax = std::max(sl.ne_v, sl.ne_w);
  const size_t smem = sizeof(double) * (size_t)nmax * BW;
  if (smem > 48 * 1024 &&
      !cuda_ok(h, cudaFuncSetAttribute(k_build_incr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "k_build_incr smem"))
    return CHF_E_CUDA;
  k_build_incr<<<dim3(h->nk2, 4), 256, smem, h->stream>>>(h->t0, h->t2, h->t4, h->k2vals, h->xinv, sl, h->d.N,
                                                          h->cfg.dt / h->cfg.re, h->incm, h->incx);
  if (!cuda_ok(h, cudaGetLastError(), "k_build_incr") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "k_build_incr sync"))
    return CHF_E_CUDA;
  return CHF_OK;
}

int launch_solve_mixed(Handle* h) {
  const Dims& d = h->d;
  const int NZ = d.NZ;
  const long modes = d.modes();
  const double dt = h->cfg.dt;
  cudaStream_t st = h->stream;
  cudaEvent_t ev;
  if (h->nk2 > 0) {
    const size_t smem = (sizeof(cd) + sizeof(CoefHL) + sizeof(float2)) * MCH * 2 * (size_t)NZ;
    if (smem > 48 * 1024 &&
        !cuda_ok(h, cudaFuncSetAttribute(k_inc_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "k_inc_solve smem"))
      return CHF_E_CUDA;
    prof_begin(h, K_INC_SOLVE, &ev);
    k_inc_solve<<<h->nk2, MV_THREADS, smem, st>>>(h->f[F_V], h->f[F_OY], h->f[F_RV], h->f[F_U], h->f[F_RG],
                                                   h->f[F_W], h->incm, h->incx, h->sl, h->group_start,
                                                   h->group_modes, d, 1.5 * dt, 0.5 * dt);
    prof_end(h, K_INC_SOLVE, ev);
  }
  {
    prof_begin(h, K_INC_RECOVER, &ev);
    const size_t smem = sizeof(double) * 2 * (size_t)NZ * 2 * TM;
    if (smem > 48 * 1024 &&
        !cuda_ok(h, cudaFuncSetAttribute(k_inc_recover, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "k_inc_recover smem"))
      return CHF_E_CUDA;
    k_inc_recover<<<(unsigned)((modes + TM - 1) / TM), I_THREADS, smem, st>>>(
        h->f[F_V], h->f[F_OY], h->f[F_U], h->f[F_W], h->f[F_OX], h->f[F_OZ], h->iapha, h->ibeta, d);
    prof_end(h, K_INC_RECOVER, ev);
  }
  if (!cuda_ok(h, cudaGetLastError(), "mixed solve")) return CHF_E_CUDA;
  // the (0,0) mode: the FP64 solve kernel, its last CTA only
  return launch_solve_mean(h);
}

}  // namespace chf
