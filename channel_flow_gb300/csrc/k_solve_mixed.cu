// k_solve_mixed.cu -- the implicit solve of the mixed path as four kernels.
//
// The per-mode solve (poiseuilleflow.f90:242-394) for every (kx, ky) but the
// (0,0) mode, written as an FP64 state plus an increment:
//   x = c + delta,   A delta = r,   r = (B - A) c + dt (3/2 N^n - 1/2 N^{n-1})
// on the collocation rows and 0 on the wall rows, with B - A =
// (dt/re) (D^2 - k^2)^2 for v and (dt/re) (D^2 - k^2) for omega_y (the CN
// operators of get_coef_v / get_coef_omegay and of get_coef_rhs /
// get_rhs_omegay, REF:3348-3489), A^-1 the even/odd inverses of k_solve.cu.
// delta is O(dt) smaller than x, so the DFT of (B - A) c runs in double-float
// arithmetic (df32.cuh) and the matvec A^-1 r multiplies (hi, lo) float
// splits with compensated FP32 accumulation, both about 2^-44 accurate, on
// the FP32 pipe; derivative scans and x = c + delta stay FP64.  Split so that
// every stage runs at full occupancy without CTA-wide phases:
//   k_inc_expl     w_v = (dt/re)(D^2-k^2)^2 c_v, w_g = (dt/re)(D^2-k^2) c_g, FP64, one
//                  thread per column running the derivative recurrences in registers
//   k_inc_fold     double-float 2N-point DFT of w -> Gauss-Lobatto values, + AB2 term,
//                  folded into even / odd right-hand sides, split into (hi, lo)
//   k_inc_matvec   one CTA per k^2 group: delta = A^-1 r, x = c + delta
//   k_inc_recover  u, w, omega_x, omega_z from v and omega_y (getvelocityandvorticity,
//                  REF:2347-2407), FP64, one thread per (mode, re/im)
// The (0,0) mode (REF:401-474) stays with k_solve (FP64, one CTA).
#include <cuda_runtime.h>

#include "chf_internal.h"
#include "df32.cuh"

namespace chf {

namespace {

constexpr int I_THREADS = 256;
constexpr int FL = 4;            // modes per CTA in the DFT kernel (2 lines each)
constexpr int MV_THREADS = 288;  // threads over the 2 NZ rows of one group's four blocks
constexpr int MCH = 4;           // modes per pass in the matvec kernel

struct RhsHL {
  float hr, hi, lr, li;
};

// ---------------------------------------------------------------------------
// k_inc_expl: grid (ceil(modes / TM)).  The Chebyshev derivatives follow
// dz's backward recurrence (REF:570-599)
//   b_k = b_{k+2} + 2 (k+1) a_{k+1},  b_0 halved,
// and since order j+1 at index k needs order j only at index k+1, one
// descending pass per column carries D1..D4 of v (D1, D2 of omega_y) in
// registers and emits w at every k.
// ---------------------------------------------------------------------------
struct Rec {  // one recurrence: values at k+1 and k+2
  double b1 = 0.0, b2 = 0.0;
  __device__ __forceinline__ double step(double src_k1, int k, bool top) {
    const double b = top ? 0.0 : b2 + 2.0 * (double)(k + 1) * src_k1;
    b2 = b1;
    b1 = b;
    return b;
  }
};

// TM modes per CTA: the tile [2 fields][NZ][TM][re, im] is loaded by all
// threads (coalesced), 4 TM threads (one per field and column) run the
// recurrences from shared memory and overwrite the tile with w, which all
// threads then store.
constexpr int TM = 16;

__global__ void __launch_bounds__(I_THREADS) k_inc_expl(const cd* __restrict__ v, const cd* __restrict__ g,
                                                        cd* __restrict__ wv, cd* __restrict__ wg,
                                                        const double* __restrict__ iapha,
                                                        const double* __restrict__ ibeta, Dims d, double dt_re) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = d.N, NZ = d.NZ, C2 = 2 * TM;
  const long modes = d.modes();
  double* T = reinterpret_cast<double*>(smem_raw);  // [2][NZ][C2]
  const long m0 = (long)blockIdx.x * TM;
  for (int t = threadIdx.x; t < 2 * NZ * C2; t += blockDim.x) {
    const int c = t % C2, n = (t / C2) % NZ, f = t / (C2 * NZ);
    const long col = 2 * m0 + c;
    const double* src = reinterpret_cast<const double*>(f == 0 ? v : g);
    T[t] = col < 2 * modes ? src[(size_t)n * 2 * modes + col] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < 2 * C2) {
    const int f = threadIdx.x / C2, c = threadIdx.x % C2;
    const long m = m0 + c / 2;
    double k2 = 0.0;
    if (m < modes) {
      const double a = iapha[m % d.KX], b = ibeta[m / d.KX];
      k2 = a * a + b * b;
    }
    double* col = T + (size_t)f * NZ * C2 + c;  // stride C2
    Rec r1, r2, r3, r4;
    double ck1 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;  // c, D1, D2, D3 at k+1
    for (int k = N; k >= 0; --k) {
      const bool top = (k == N);
      const double ck = col[k * C2];
      const double d1 = r1.step(ck1, k, top);
      const double d2 = r2.step(p1, k, top);
      double out;
      if (f == 0) {
        const double d3 = r3.step(p2, k, top);
        const double d4 = r4.step(p3, k, top);
        p3 = d3;
        const double h = k == 0 ? 0.5 : 1.0;  // only the k = 0 outputs halve
        out = dt_re * (h * d4 - 2.0 * k2 * h * d2 + k2 * k2 * ck);
      } else {
        out = dt_re * ((k == 0 ? 0.5 : 1.0) * d2 - k2 * ck);
      }
      p1 = d1;
      p2 = d2;
      ck1 = ck;
      col[k * C2] = out;  // c_k is kept in ck1 for the next step
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * NZ * C2; t += blockDim.x) {
    const int c = t % C2, n = (t / C2) % NZ, f = t / (C2 * NZ);
    const long col = 2 * m0 + c;
    if (col < 2 * modes) reinterpret_cast<double*>(f == 0 ? wv : wg)[(size_t)n * 2 * modes + col] = T[t];
  }
}

// ---------------------------------------------------------------------------
// k_inc_fold: grid (ceil(modes / FL)).  2 FL double-float lines of 2N points
// (even extension of w with doubled end coefficients), forward DFT, then
// R = 1/2 DFT + AB2 term at the Gauss-Lobatto points, folded:
//   even rows 1/2 (R_p + R_{N-p}), odd rows 1/2 (R_p - R_{N-p}), p = 0..N/2,
// wall rows (v: p < 2, omega_y: p < 1) zero.  Out: rb[mode][2 NZ] (hi, lo)
// in the order v-even (ne), v-odd (no), omega-even (ne), omega-odd (no).
// ---------------------------------------------------------------------------
template <int MB2>
__global__ void __launch_bounds__(I_THREADS) k_inc_fold(const cd* __restrict__ wv, const cd* __restrict__ wg,
                                                        const cd* __restrict__ rv, const cd* __restrict__ uh,
                                                        const cd* __restrict__ rg, const cd* __restrict__ wh,
                                                        Dims d, double c3, double c1,
                                                        const __grid_constant__ FftPlan pz2,
                                                        const cplx<df32>* __restrict__ tw, RhsHL* __restrict__ rb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using C = cplx<df32>;
  C* lines = reinterpret_cast<C*>(smem_raw);  // [2 FL][2N]: line 2l = v, 2l+1 = omega_y
  const int N = d.N, NZ = d.NZ, L2 = 2 * N, ne = N / 2 + 1;
  const long modes = d.modes();
  const long m0 = (long)blockIdx.x * FL;
  for (int t = threadIdx.x; t < 2 * FL * NZ; t += blockDim.x) {
    const int ln = t / NZ, n = t % NZ, l = ln / 2, f = ln % 2;
    const long m = m0 + l;
    cd x{0.0, 0.0};
    if (m < modes) x = (f == 0 ? wv : wg)[(size_t)n * modes + m];
    const double dbl = (n == 0 || n == N) ? 2.0 : 1.0;
    lines[ln * L2 + n] = C{df32(dbl * x.re), df32(dbl * x.im)};
    if (n > 0 && n < N) lines[ln * L2 + L2 - n] = C{df32(x.re), df32(x.im)};
  }
  __syncthreads();
  smem_fft<df32, -1, MB2>(lines, 2 * FL, L2, pz2, tw);
  for (int t = threadIdx.x; t < 2 * FL * ne; t += blockDim.x) {
    const int ln = t / ne, r = t % ne, l = ln / 2, f = ln % 2;
    const long m = m0 + l;
    if (m >= modes) continue;
    const int p = r, q = N - r;
    const C* line = lines + ln * L2;
    const cd* H = f == 0 ? rv : rg;   // N^n (GL values)
    const cd* Ho = f == 0 ? uh : wh;  // N^{n-1}
    const cd hp = H[(size_t)p * modes + m], hq = H[(size_t)q * modes + m];
    const cd op = Ho[(size_t)p * modes + m], oq = Ho[(size_t)q * modes + m];
    const double Rp_re = 0.5 * line[p].re.to_double() + (c3 * hp.re - c1 * op.re);
    const double Rp_im = 0.5 * line[p].im.to_double() + (c3 * hp.im - c1 * op.im);
    const double Rq_re = 0.5 * line[q].re.to_double() + (c3 * hq.re - c1 * oq.re);
    const double Rq_im = 0.5 * line[q].im.to_double() + (c3 * hq.im - c1 * oq.im);
    const bool wall = (f == 0) ? (r < 2) : (r < 1);
    const double er = wall ? 0.0 : 0.5 * (Rp_re + Rq_re), ei = wall ? 0.0 : 0.5 * (Rp_im + Rq_im);
    const double orr = wall ? 0.0 : 0.5 * (Rp_re - Rq_re), oi = wall ? 0.0 : 0.5 * (Rp_im - Rq_im);
    auto hl = [](double xr, double xi) {
      const float hr = (float)xr, hi = (float)xi;
      return RhsHL{hr, hi, (float)(xr - (double)hr), (float)(xi - (double)hi)};
    };
    RhsHL* out = rb + (size_t)m * 2 * NZ + (f == 0 ? 0 : NZ);
    out[r] = hl(er, ei);                       // even block, row r (r < ne)
    if (r < N / 2) out[ne + r] = hl(orr, oi);  // odd block, row r (r < no)
  }
}

// ---------------------------------------------------------------------------
// k_inc_matvec: one CTA per k^2 group (mean excluded), threads over the rows
// of the four blocks; MCH modes of the group per pass.  Compensated FP32: the
// exact product xh rh = p + pe is added by TwoSum into S (error into C),
// xh rl + xl rh + pe into C.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(MV_THREADS) k_inc_matvec(const RhsHL* __restrict__ rb,
                                                           const float2* __restrict__ xinv2, SolveLayout sl,
                                                           const int* __restrict__ group_start,
                                                           const int* __restrict__ group_modes,
                                                           cd* __restrict__ v, cd* __restrict__ g, Dims d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RhsHL* R = reinterpret_cast<RhsHL*>(smem_raw);  // [MCH][2 NZ]
  const int NZ = d.NZ;
  const long modes = d.modes();
  const int grp = blockIdx.x;
  const int gs = group_start[grp], ge = group_start[grp + 1];
  const int nev = sl.ne_v, nov = sl.no_v, new_ = sl.ne_w, now_ = sl.no_w;
  const int rows = nev + nov + new_ + now_;
  const BlockOffsets bo = block_offsets(sl);
  const float2* Xg = xinv2 + (size_t)grp * sl.stride;
  for (int base = gs; base < ge; base += MCH) {
    const int nm = min(MCH, ge - base);
    for (int e = threadIdx.x; e < nm * 2 * NZ; e += blockDim.x) {
      const int q = e / (2 * NZ), i = e % (2 * NZ);
      R[e] = rb[(size_t)group_modes[base + q] * 2 * NZ + i];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < rows; t += blockDim.x) {
      int b, row, n, r0;
      size_t boff;
      if (t < nev) { b = 0; row = t; n = nev; r0 = 2; boff = bo.ve; }
      else if (t < nev + nov) { b = 1; row = t - nev; n = nov; r0 = 2; boff = bo.vo; }
      else if (t < nev + nov + new_) { b = 2; row = t - nev - nov; n = new_; r0 = 1; boff = bo.we; }
      else { b = 3; row = t - nev - nov - new_; n = now_; r0 = 1; boff = bo.wo; }
      // offset of block b inside a mode's 2 NZ right-hand-side entries
      const int roff = b == 0 ? 0 : b == 1 ? nev : b == 2 ? NZ : NZ + new_;
      const float2* X = Xg + boff;
      float S[MCH][2], C[MCH][2];
#pragma unroll
      for (int q = 0; q < MCH; ++q) S[q][0] = S[q][1] = C[q][0] = C[q][1] = 0.f;
#pragma unroll 2
      for (int c = r0; c < n; ++c) {
        const float2 x = __ldg(X + (size_t)c * n + row);
#pragma unroll
        for (int q = 0; q < MCH; ++q) {
          if (q < nm) {
            const RhsHL rr = R[q * 2 * NZ + roff + c];
            const float rh[2] = {rr.hr, rr.hi}, rl[2] = {rr.lr, rr.li};
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              const float p = __fmul_rn(x.x, rh[k]);
              const float pe = __fmaf_rn(x.x, rh[k], -p);
              const df32 s = df_two_sum(S[q][k], p);
              S[q][k] = s.hi;
              C[q][k] = __fadd_rn(C[q][k],
                                  __fadd_rn(__fadd_rn(s.lo, pe), __fmaf_rn(x.x, rl[k], __fmul_rn(x.y, rh[k]))));
            }
          }
        }
      }
      const int j = (b == 0 || b == 2) ? 2 * row : 2 * row + 1;
      cd* dst = b < 2 ? v : g;
#pragma unroll
      for (int q = 0; q < MCH; ++q) {
        if (q < nm) {
          const size_t idx = (size_t)j * modes + group_modes[base + q];
          const cd c0 = dst[idx];
          dst[idx] = cd{c0.re + ((double)S[q][0] + (double)C[q][0]), c0.im + ((double)S[q][1] + (double)C[q][1])};
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// k_inc_recover: grid (ceil(modes / TM)); tiles of v and omega_y in shared
// memory, one thread per (mode, re/im) running one descending pass (the
// recurrence of k_inc_expl), the other component from its partner lane:
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

int launch_solve_mixed(Handle* h) {
  const Dims& d = h->d;
  const int N = d.N, NZ = d.NZ;
  const long modes = d.modes();
  const double dt = h->cfg.dt, re = h->cfg.re;
  if (!h->inc_buf) {  // w_v, w_g (FP64 coefficients) and the folded right-hand sides
    const size_t bytes = sizeof(cd) * 2 * (size_t)NZ * modes + sizeof(RhsHL) * 2 * (size_t)NZ * modes;
    if (!cuda_ok(h, cudaMalloc(&h->inc_buf, bytes), "increment buffers")) return CHF_E_NOMEM;
  }
  cd* wv = static_cast<cd*>(h->inc_buf);
  cd* wg = wv + (size_t)NZ * modes;
  RhsHL* rb = reinterpret_cast<RhsHL*>(wg + (size_t)NZ * modes);
  cudaStream_t st = h->stream;
  cudaEvent_t ev;
  {
    prof_begin(h, K_INC_EXPL, &ev);
    const size_t smem = sizeof(double) * 2 * (size_t)NZ * 2 * TM;
    if (smem > 48 * 1024 &&
        !cuda_ok(h, cudaFuncSetAttribute(k_inc_expl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "k_inc_expl smem"))
      return CHF_E_CUDA;
    k_inc_expl<<<(unsigned)((modes + TM - 1) / TM), I_THREADS, smem, st>>>(
        h->f[F_V], h->f[F_OY], wv, wg, h->iapha, h->ibeta, d, dt / re);
    prof_end(h, K_INC_EXPL, ev);
  }
  {
    const int mb2 = fft_fits(2 * FL, 2 * N, I_THREADS, 2) ? 2 : fft_fits(2 * FL, 2 * N, I_THREADS, 4) ? 4 : 8;
    if (!fft_fits(2 * FL, 2 * N, I_THREADS, mb2)) {
      h->err = "mixed solve: nnz too large for the DFT launch shape";
      return CHF_E_INVALID;
    }
    const size_t smem = sizeof(cplx<df32>) * 2 * FL * 2 * N;
    auto kern = mb2 == 2 ? k_inc_fold<2> : mb2 == 4 ? k_inc_fold<4> : k_inc_fold<8>;
    if (smem > 48 * 1024 &&
        !cuda_ok(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "k_inc_fold smem"))
      return CHF_E_CUDA;
    prof_begin(h, K_INC_FOLD, &ev);
    kern<<<(unsigned)((modes + FL - 1) / FL), I_THREADS, smem, st>>>(
        wv, wg, h->f[F_RV], h->f[F_U], h->f[F_RG], h->f[F_W], d, 1.5 * dt, 0.5 * dt, h->pz2, h->twd_z2, rb);
    prof_end(h, K_INC_FOLD, ev);
  }
  {
    const size_t smem = sizeof(RhsHL) * MCH * 2 * NZ;
    prof_begin(h, K_INC_MATVEC, &ev);
    k_inc_matvec<<<h->nk2, MV_THREADS, smem, st>>>(rb, h->xinv2, h->sl, h->group_start, h->group_modes,
                                                   h->f[F_V], h->f[F_OY], d);
    prof_end(h, K_INC_MATVEC, ev);
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
