// k_solve_mixed.cu -- the implicit solve of the mixed path.
//
// The per-mode solve (poiseuilleflow.f90:242-394) for every (kx, ky) but the
// (0,0) mode, written as an FP64 state plus an increment:
//   x = c + delta,   delta = A^-1 (B - A) c + A^-1 r,
//   r = dt (3/2 N^n - 1/2 N^{n-1})
// on the collocation rows and 0 on the wall rows, with B - A =
// (dt/re) (D^2 - k^2)^2 for v and (dt/re) (D^2 - k^2) for omega_y on the
// collocation rows (the CN operators of get_coef_v / get_coef_omegay and of
// get_coef_rhs / get_rhs_omegay, REF:3348-3489) and minus the wall rows of A
// on the wall rows (the reference's right-hand side holds the boundary
// values, 0, there), and A^-1 the even/odd inverses of k_solve.cu.  Then
// A x = B c + r with B's wall rows 0: the equations the reference solves,
// for any c (also one that does not satisfy the walls, e.g. an uploaded
// initial field).  Forming (B - A) c at the collocation points cancels
// heavily (fourth derivatives of the coefficients against an O(c) result),
// so the set-up multiplies it into the inverse once per k^2 in FP64:
// M = A^-1 (B - A) = A^-1 B - I maps coefficients to coefficients and has no
// such cancellation (its rows sum to within ~10x of the result; at 128^3
// the largest row sum is ~150, the median ~2).  A step is then
//   k_inc_solve    one CTA per run of at most 4 (or 2) modes of one k^2
//                  group: delta = M c (compensated FP32 on (hi, lo) splits of
//                  M and c, summed against a power-of-two offset) + A^-1 r
//                  (FP32), x = c + delta in FP64
//   k_inc_recover  u, w, omega_x, omega_z from v and omega_y (getvelocityandvorticity,
//                  REF:2347-2407), four threads per mode, in double-float
//                  (k_inc_recover) or FP64 (k_inc_recover64)
// FP64 arithmetic and double <-> float conversions share GB300's narrow FP64
// pipe, so the conversions here are integer operations (f64bits.cuh).
// The (0,0) mode (REF:401-474) stays with k_solve (FP64, one CTA).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "chf_internal.h"
#include "f32x2.cuh"
#include "f64bits.cuh"

namespace chf {

namespace {

constexpr int MV_THREADS = 288;  // threads over the 2 NZ rows of one group's four blocks
// modes per CTA (MCH), matrix columns per load batch (CB) and rows per thread
// of k_inc_solve are template parameters: the defaults 4, 4 and 1, others
// picked by the autotuner (chf_tune.cu)

// Chebyshev derivative recurrence (dz, REF:570-599), descending in k:
//   b_k = b_{k+2} + 2 (k+1) a_{k+1}   (b_0 halved on output)

// ---------------------------------------------------------------------------
// Set-up of the increment operators, grid (nk2, 4 blocks): with X = A^-1 the
// block's inverse (k_solve.cu, FP64) and W the folded rows of B - A,
//   W[q][c] = (dt/re) (T4 - 2 k^2 T2 + k^4 T0)(z_q, T_j)   (v)
//   W[q][c] = (dt/re) (T2 - k^2 T0)(z_q, T_j)               (omega_y)
// for q >= r0 and minus the folded wall rows of A (k_invert: -1 for the
// value rows, -j^2 for the slope row of v) for q < r0, j = 2c or 2c + 1, the
// kernel forms
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
      } else if (cc < nc) {
        w = (isv && q == 1) ? -(double)j * (double)j : -1.0;
      }
      W[t] = w;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n * nc; t += blockDim.x) {
      const int cc = t / n, r = t % n;
      double acc = 0.0;
      for (int q = 0; q < n; ++q) acc = fma(X[(size_t)q * n + r], W[q * BW + cc], acc);
      const float hi = (float)acc;
      incm[off + (size_t)(c0 + cc) * n + r] = make_float2(hi, (float)(acc - (double)hi));
    }
  }
}

// Row exponents of the increment operators, grid (nk2, 4 blocks): for row r
// of a block of M, sum_c |hi(r, c)| < 2^e (e = -100 for a zero row), as a
// signed byte at the row's place among the group's 2 NZ rows (v even, v odd,
// omega even, omega odd).
__global__ void __launch_bounds__(128) k_incr_rowexp(const float2* __restrict__ incm, SolveLayout sl,
                                                     signed char* __restrict__ rowexp) {
  const int g = blockIdx.x, blk = blockIdx.y;
  const int n = blk == 0 ? sl.ne_v : blk == 1 ? sl.no_v : blk == 2 ? sl.ne_w : sl.no_w;
  const int roff = blk == 0 ? 0 : blk == 1 ? sl.ne_v : blk == 2 ? sl.ne_v + sl.no_v : sl.ne_v + sl.no_v + sl.ne_w;
  const BlockOffsets bo = block_offsets(sl);
  const float2* M = incm + (size_t)g * sl.stride + (blk == 0 ? bo.ve : blk == 1 ? bo.vo : blk == 2 ? bo.we : bo.wo);
  const int rows = sl.ne_v + sl.no_v + sl.ne_w + sl.no_w;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    double sum = 0.0;
    for (int c = 0; c < n; ++c) sum += fabs((double)M[(size_t)c * n + r].x);
    int e = -100;
    if (sum > 0.0) (void)frexp(sum, &e);  // sum = m 2^e, m in [0.5, 1)
    rowexp[(size_t)g * rows + roff + r] = (signed char)max(-100, min(100, e));
  }
}

// ---------------------------------------------------------------------------
// k_inc_solve: one CTA per work item, up to MCH modes of one k^2 group (mean
// excluded; setup_inc_items).  Per mode the CTA stages in shared memory
//   * the coefficients c of v and omega_y as (hi, lo) floats, ordered as the
//     four blocks' columns (v even j, v odd j, omega even j, omega odd j);
//   * the AB2 term r = dt (3/2 N^n - 1/2 N^{n-1}) at the Gauss-Lobatto
//     points, folded (even rows 1/2 (r_p + r_{N-p}), odd rows
//     1/2 (r_p - r_{N-p}), p = row) with the wall rows zero, as floats;
// and per block the exponent e_c of the largest |hi| (max < 2^e_c); then one
// thread per block row forms
//   delta = M c + X r
// and writes x = c + delta in FP64.  M c is compensated: the products of the
// high parts p = mh ch are summed into S, which starts at the power of two
//   sigma = 2^(e_r + e_c + 3) >= 8 sum_c |mh ch|      (sum_c |mh| < 2^e_r),
// so that S and every S + p stay within (7/8, 9/8) sigma: s = S + p, then
// S - s is exact (Sterbenz) and fma(mh, ch, S - s) is the product's rounding
// error plus the part of p that S could not hold, rounded once.  That term
// and the cross products mh cl + ml ch go to a second FP32 accumulator C,
// with X r in plain FP32 (r is O(dt) and X r has no cancellation), and
// delta = (S - sigma) + C with S - sigma exact: M c to about
// 2^-38 sum_c |M_rc| max|c| (sigma is at most 2^5 of that; the dropped
// parts are 2^-43 of sigma), X r to FP32 rounding.
// ---------------------------------------------------------------------------
struct __align__(16) CoefHL {
  float hr, hi, lr, li;  // high and low parts of the real and imaginary parts
};

// CB matrix columns per load batch (two batches in flight)

// Packed FP32 pairs (f32x2.cuh): the real and imaginary parts of a
// coefficient travel together.

// S, C for one matrix entry (mh + ml) and one coefficient (ch + cl), real and
// imaginary parts as a pair: S += mh ch, C += (mh ch - (s - S)) + mh cl + ml ch
// (S against its offset sigma, so s - S is exact).  mh, ml broadcast.  The
// compiler may fuse the product into the first sum (ptxas contracts packed
// multiply-add pairs); u is then the error of that fused sum, rounded once,
// and the bound is the same.
__device__ __forceinline__ void sig_mac2(f32x2 mh, f32x2 ml, f32x2 ch, f32x2 cl, f32x2& S, f32x2& C) {
  const f32x2 s = add2(S, mul2(mh, ch));
  const f32x2 u = fma2(mh, ch, sub2(S, s));
  S = s;
  C = fma2(ml, ch, fma2(mh, cl, add2(C, u)));
}

// Rows of one pass of k_inc_solve for NM staged modes: each thread owns RPT
// adjacent rows of one of the four blocks (v even, v odd, omega even,
// omega odd), so that every staged coefficient and AB2 value read from
// shared memory serves RPT rows.  The staged values of entry e of mode q sit
// at e MS + q (MS = the kernel's modes per CTA), so one address per column
// reaches every mode by constant offsets; the matrix columns are walked by
// element offsets advanced per batch, and only the last batch checks the
// column count.  The arithmetic of a row does not depend on RPT.
template <int NM, int MS, int CB, int RPT>
__device__ __forceinline__ void inc_rows(cd* __restrict__ v, cd* __restrict__ g, const float2* __restrict__ Mg,
                                         const float* __restrict__ Xg, const SolveLayout& sl,
                                         const BlockOffsets& bo, int NZ, long modes, const cd* Cd,
                                         const CoefHL* Cs, const float2* Rs, const int* s_mode,
                                         const signed char* __restrict__ rexp, const int* s_cexp) {
  const int nev = sl.ne_v, nov = sl.no_v, new_ = sl.ne_w, now_ = sl.no_w;
  // slots (groups of RPT rows) per block
  const int sev = (nev + RPT - 1) / RPT, sov = (nov + RPT - 1) / RPT, sew = (new_ + RPT - 1) / RPT,
            sow = (now_ + RPT - 1) / RPT;
  const int slots = sev + sov + sew + sow;
  for (int t = threadIdx.x; t < slots; t += blockDim.x) {
    int b, slot, n;
    int boff;
    if (t < sev) { b = 0; slot = t; n = nev; boff = (int)bo.ve; }
    else if (t < sev + sov) { b = 1; slot = t - sev; n = nov; boff = (int)bo.vo; }
    else if (t < sev + sov + sew) { b = 2; slot = t - sev - sov; n = new_; boff = (int)bo.we; }
    else { b = 3; slot = t - sev - sov - sew; n = now_; boff = (int)bo.wo; }
    // offset of block b inside a mode's 2 NZ staged entries
    const int roff = b == 0 ? 0 : b == 1 ? nev : b == 2 ? NZ : NZ + new_;
    const int row0 = slot * RPT;
    bool live[RPT];
    int off[RPT];  // element offset of the row's current column in the group's blocks
    f32x2 S[RPT][NM], C[RPT][NM];  // (re, im) pairs
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      live[i] = row0 + i < n;
      const int row = live[i] ? row0 + i : row0;  // a dead row reads its live neighbour
      off[i] = boff + row;
      const int er = rexp[roff + row];
#pragma unroll
      for (int q = 0; q < NM; ++q) {  // S starts at sigma of mode q for this row
        const int e = max(-120, min(120, er + s_cexp[4 * q + b] + 3));
        const float sg = __int_as_float((127 + e) << 23);
        S[i][q] = pk(sg, sg);
        C[i][q] = 0ull;
      }
    }
    // columns c < r0 of X meet the zero wall entries of the staged rhs
    float2 ma[RPT][CB];
    float xa[RPT][CB];
#pragma unroll
    for (int u = 0; u < CB; ++u)
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        ma[i][u] = u < n ? __ldg(Mg + off[i] + u * n) : make_float2(0.f, 0.f);
        xa[i][u] = u < n ? __ldg(Xg + off[i] + u * n) : 0.f;
      }
#pragma unroll
    for (int i = 0; i < RPT; ++i) off[i] += CB * n;
    const float4* cc = reinterpret_cast<const float4*>(Cs) + roff * MS;  // column 0, mode 0
    const f32x2* rr = reinterpret_cast<const f32x2*>(Rs) + roff * MS;
    auto columns = [&](const float2(&mc)[RPT][CB], const float(&xc)[RPT][CB], int ncol) {
#pragma unroll
      for (int u = 0; u < CB; ++u) {
        if (u < ncol) {
          f32x2 mh[RPT], ml[RPT], xx[RPT];  // the column's entries, broadcast to (re, im)
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            mh[i] = pk(mc[i][u].x, mc[i][u].x);
            ml[i] = pk(mc[i][u].y, mc[i][u].y);
            xx[i] = pk(xc[i][u], xc[i][u]);
          }
#pragma unroll
          for (int q = 0; q < NM; ++q) {
            const float4 ch = cc[u * MS + q];  // one 16-byte load
            const f32x2 r2 = rr[u * MS + q];
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
              sig_mac2(mh[i], ml[i], pk(ch.x, ch.y), pk(ch.z, ch.w), S[i][q], C[i][q]);
              C[i][q] = fma2(xx[i], r2, C[i][q]);
            }
          }
        }
      }
    };
    int c0 = 0;
    for (; c0 + CB <= n; c0 += CB) {
      float2 mb[RPT][CB];
      float xb[RPT][CB];
      if (c0 + 2 * CB <= n) {  // the next batch is whole
#pragma unroll
        for (int u = 0; u < CB; ++u)
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            mb[i][u] = __ldg(Mg + off[i] + u * n);
            xb[i][u] = __ldg(Xg + off[i] + u * n);
          }
      } else {
#pragma unroll
        for (int u = 0; u < CB; ++u) {
          const bool in = c0 + CB + u < n;
#pragma unroll
          for (int i = 0; i < RPT; ++i) {
            mb[i][u] = in ? __ldg(Mg + off[i] + u * n) : make_float2(0.f, 0.f);
            xb[i][u] = in ? __ldg(Xg + off[i] + u * n) : 0.f;
          }
        }
      }
#pragma unroll
      for (int i = 0; i < RPT; ++i) off[i] += CB * n;
      columns(ma, xa, CB);
      cc += CB * MS;
      rr += CB * MS;
#pragma unroll
      for (int u = 0; u < CB; ++u)
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          ma[i][u] = mb[i][u];
          xa[i][u] = xb[i][u];
        }
    }
    columns(ma, xa, n - c0);  // the last n mod CB columns
    cd* dst = b < 2 ? v : g;
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      if (!live[i]) continue;
      const int row = row0 + i;
      const int j = (b == 0 || b == 2) ? 2 * row : 2 * row + 1;
#pragma unroll
      for (int q = 0; q < NM; ++q) {
        const cd c0v = Cd[q * 2 * NZ + roff + row];
        float Sv[2], Cv[2];
        upk(S[i][q], Sv[0], Sv[1]);
        upk(C[i][q], Cv[0], Cv[1]);
        double x[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          // S - sigma (exact): S lies within (7/8, 9/8) sigma, so sigma is S's
          // power of two, rounded up when S's significand is at least 1.5
          const float d = Sv[k] - __int_as_float((__float_as_int(Sv[k]) + 0x400000) & 0xff800000);
          // x = c + delta with two FP64 additions (the float -> double moves
          // are integer operations)
          x[k] = ((k == 0 ? c0v.re : c0v.im) + bits::widen(d)) + bits::widen(Cv[k]);
        }
        dst[(size_t)j * modes + s_mode[q]] = cd{x[0], x[1]};
      }
    }
  }
}

// block size and minimum CTAs per SM of k_inc_solve: one row per thread at
// MV_THREADS threads (RPT = 1; blocks of more rows loop), one row per thread
// with every row in one pass at up to MV_WIDE threads (RPT = 0, for
// wall-normal grids of more than MV_THREADS block rows), or two rows per
// thread at up to 256 threads (RPT = 2)
constexpr int MV_WIDE = 416;
template <int MCH, int RPT>
struct IncShape {
  static constexpr int threads = RPT == 1 ? MV_THREADS : RPT == 0 ? MV_WIDE : 256;
  static constexpr int min_ctas = RPT == 1 ? (MCH == 2 ? 4 : 3) : 2;
  static constexpr int rows = RPT == 0 ? 1 : RPT;  // block rows per thread
};

template <int MCH, int CB, int RPT>
__global__ void __launch_bounds__(IncShape<MCH, RPT>::threads, IncShape<MCH, RPT>::min_ctas)
    k_inc_solve(cd* __restrict__ v, cd* __restrict__ g,
                                                             const cd* __restrict__ rv, const cd* __restrict__ uh,
                                                             const cd* __restrict__ rg, const cd* __restrict__ wh,
                                                             const float2* __restrict__ incm,
                                                             const float* __restrict__ incx,
                                                             const signed char* __restrict__ rowexp, SolveLayout sl,
                                                             const int* __restrict__ group_start,
                                                             const int* __restrict__ group_modes,
                                                             const int2* __restrict__ items, Dims d,
                                                             float c3, float c1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = d.N, NZ = d.NZ, ne = N / 2 + 1;
  const long modes = d.modes();
  cd* Cd = reinterpret_cast<cd*>(smem_raw);                   // [MCH][2 NZ] FP64 coefficients
  CoefHL* Cs = reinterpret_cast<CoefHL*>(Cd + MCH * 2 * NZ);  // [2 NZ][MCH] their (hi, lo) splits
  float2* Rs = reinterpret_cast<float2*>(Cs + MCH * 2 * NZ);  // [2 NZ][MCH] folded AB2 term
  __shared__ int s_mode[MCH];
  __shared__ int s_cexp[MCH * 4];  // largest |hi| per (mode, block): float bits, then its exponent
  // work item: up to MCH modes of one k^2 group, from base
  const int2 it = items[blockIdx.x];
  const int grp = it.x, base = it.y;
  const BlockOffsets bo = block_offsets(sl);
  const float2* Mg = incm + (size_t)grp * sl.stride;
  const float* Xg = incx + (size_t)grp * sl.stride;
  {
    const int nm = min(MCH, group_start[grp + 1] - base);
    if (threadIdx.x < nm) s_mode[threadIdx.x] = group_modes[base + threadIdx.x];
    if (threadIdx.x < MCH * 4) s_cexp[threadIdx.x] = 0;
    __syncthreads();
    // (mode, entry) loops without divisions by the run-time sizes
    for (int q = 0; q < nm; ++q)
    for (int i = threadIdx.x; i < 2 * NZ; i += blockDim.x) {
      const int f = i >= NZ, k = i - f * NZ;
      const cd x = (f == 0 ? v : g)[(size_t)k * modes + s_mode[q]];
      const int en = f * NZ + ((k & 1) ? ne + k / 2 : k / 2);  // entry within the mode
      Cd[q * 2 * NZ + en] = x;
      CoefHL h;
      bits::split(x.re, h.hr, h.lr);
      bits::split(x.im, h.hi, h.li);
      Cs[en * MCH + q] = h;
      atomicMax(&s_cexp[4 * q + 2 * f + (k & 1)], __float_as_int(fmaxf(fabsf(h.hr), fabsf(h.hi))));
    }
    // the AB2 term in FP32 (X r is an FP32 product of an O(dt) term)
    for (int q = 0; q < nm; ++q)
    for (int i = threadIdx.x; i < 2 * ne; i += blockDim.x) {
      const int f = i >= ne, r = i - f * ne;
      const long m = s_mode[q];
      const cd* H = f == 0 ? rv : rg;   // N^n (GL values)
      const cd* Ho = f == 0 ? uh : wh;  // N^{n-1}
      const size_t ip = (size_t)r * modes + m, iq = (size_t)(N - r) * modes + m;
      const cd hp = H[ip], hq = H[iq], op = Ho[ip], oq = Ho[iq];
      const float pr = c3 * bits::narrow(hp.re) - c1 * bits::narrow(op.re);
      const float pi = c3 * bits::narrow(hp.im) - c1 * bits::narrow(op.im);
      const float qr = c3 * bits::narrow(hq.re) - c1 * bits::narrow(oq.re);
      const float qi = c3 * bits::narrow(hq.im) - c1 * bits::narrow(oq.im);
      const bool wall = (f == 0) ? (r < 2) : (r < 1);
      float2* out = Rs + (size_t)f * NZ * MCH + q;  // entry e of mode q at e MCH + q
      out[r * MCH] = wall ? make_float2(0.f, 0.f) : make_float2(0.5f * (pr + qr), 0.5f * (pi + qi));
      if (r < N / 2)
        out[(ne + r) * MCH] = wall ? make_float2(0.f, 0.f) : make_float2(0.5f * (pr - qr), 0.5f * (pi - qi));
    }
    __syncthreads();
    if (threadIdx.x < nm * 4) {  // max < 2^e
      int e = -60;
      const float mx = __int_as_float(s_cexp[threadIdx.x]);
      if (mx > 0.f) (void)frexpf(mx, &e);
      s_cexp[threadIdx.x] = max(-60, e);
    }
    __syncthreads();
    const signed char* rexp = rowexp + (size_t)grp * 2 * NZ;
    switch (nm) {
      case 1: inc_rows<1, MCH, CB, IncShape<MCH, RPT>::rows>(v, g, Mg, Xg, sl, bo, NZ, modes, Cd, Cs, Rs, s_mode, rexp, s_cexp); break;
      case 2: inc_rows<2, MCH, CB, IncShape<MCH, RPT>::rows>(v, g, Mg, Xg, sl, bo, NZ, modes, Cd, Cs, Rs, s_mode, rexp, s_cexp); break;
      default:
        if constexpr (MCH >= 4) {
          if (nm == 3) inc_rows<3, MCH, CB, IncShape<MCH, RPT>::rows>(v, g, Mg, Xg, sl, bo, NZ, modes, Cd, Cs, Rs, s_mode, rexp, s_cexp);
          else inc_rows<4, MCH, CB, IncShape<MCH, RPT>::rows>(v, g, Mg, Xg, sl, bo, NZ, modes, Cd, Cs, Rs, s_mode, rexp, s_cexp);
        }
        break;
    }
  }
}

// ---------------------------------------------------------------------------
// k_inc_recover: four threads per mode (lane = 4 mode + 2 parity + re/im),
// grid (ceil(4 modes / RC_THREADS)); u, w, omega_x, omega_z from v and
// omega_y (getvelocityandvorticity, REF:2347-2407) for every solved mode
// (not (0,0), not the spanwise Nyquist slot):
//   u = (i a Dv - i b g) / k^2,            w = (i b Dv + i a g) / k^2,
//   omega_z = -Du + i a v = (i b Dg - i a D^2 v) / k^2 + i a v,
//   omega_x =  Dw - i b v = (i b D^2 v + i a Dg) / k^2 - i b v.
// The dz recurrences (b_0 halved on output) run on descending rows; the
// even-k and odd-k chains of Dv and Dg are independent, so the pair of parity
// threads of a component runs them in lockstep (even rows 2s below the top,
// odd rows one below those); D^2 v at row k needs Dv at row k + 1 from the
// other chain, and Dv, Dg at row k need v, g at row k + 1, the other chain's
// row: both come by shuffle (the odd thread takes the even thread's current
// values, the even thread the odd thread's previous ones).  The other re/im
// component comes by shuffle too, and multiplying by i folds into the signs
// of the per-thread coefficients.
// Arithmetic: double-float (hi, lo) pairs of FP32.  v and omega_y enter as
// their (hi, lo) splits (bits::split: 2^-46 relative); a recurrence step
// t a + b (t = 2 (k + 1), an exact FP32 integer) is an exact product and an
// exact sum (Knuth's two-sum) plus the low parts, renormalised; an output is
// a sum of double-float products.  Every operation is a __f*_rn intrinsic,
// which the compiler never contracts into an FMA (a contracted
// multiply-subtract would break the two-sum).  Each output leaves as hi + lo
// in one FP64 addition (the only FP64 operations: 4 per element; the FP64
// pipe retires about 2 lane-operations per clock per SM, FP32 about 128).
// Relative to the largest term of each sum the result is within about
// 2^-44, against 2^-53 for FP64 throughout; RC_PF steps of v and omega_y are
// loaded ahead.
// ---------------------------------------------------------------------------
constexpr int RC_THREADS = 32;  // one warp: 1024 CTAs at 128^3, balanced over the SMs
constexpr int RC_PF = 8;  // steps of v, omega_y loaded ahead of the recurrences

// a double-float value h + l
struct DF {
  float h, l;
};

// s + e = a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// t a + b for an exact FP32 integer t, renormalised
__device__ __forceinline__ DF df_fma_int(float t, const DF& a, const DF& b) {
  const float p = __fmul_rn(t, a.h);
  const float pe = __fmaf_rn(t, a.h, -p);  // t a.h - p, exact
  float s, e;
  two_sum(b.h, p, s, e);
  const float lo = __fadd_rn(e, __fadd_rn(b.l, __fmaf_rn(t, a.l, pe)));
  DF r;
  two_sum(s, lo, r.h, r.l);
  return r;
}

// c x as (ph, pl), unnormalised: ph = RN(c.h x.h), pl = the rest
__device__ __forceinline__ void df_prod(const DF& c, const DF& x, float& ph, float& pl) {
  ph = __fmul_rn(c.h, x.h);
  pl = __fmaf_rn(c.h, x.l, __fmaf_rn(c.l, x.h, __fmaf_rn(c.h, x.h, -ph)));
}

__device__ __forceinline__ DF df_of(double x) {
  DF r;
  bits::split(x, r.h, r.l);
  return r;
}

// c1 x1 + c2 x2 (+ c3 x3) as FP64: the products' high parts summed exactly,
// the rest in FP32, hi + lo in one FP64 addition (the float -> double moves
// are integer operations)
__device__ __forceinline__ double df_dot2(const DF& c1, const DF& x1, const DF& c2, const DF& x2) {
  float p1, q1, p2, q2, s, e;
  df_prod(c1, x1, p1, q1);
  df_prod(c2, x2, p2, q2);
  two_sum(p1, p2, s, e);
  return bits::widen(s) + bits::widen(__fadd_rn(e, __fadd_rn(q1, q2)));
}
__device__ __forceinline__ double df_dot3(const DF& c1, const DF& x1, const DF& c2, const DF& x2, const DF& c3,
                                          const DF& x3) {
  float p1, q1, p2, q2, p3, q3, s, e, s2, e2;
  df_prod(c1, x1, p1, q1);
  df_prod(c2, x2, p2, q2);
  df_prod(c3, x3, p3, q3);
  two_sum(p1, p2, s, e);
  two_sum(s, p3, s2, e2);
  return bits::widen(s2) + bits::widen(__fadd_rn(__fadd_rn(e, e2), __fadd_rn(q1, __fadd_rn(q2, q3))));
}

__device__ __forceinline__ DF shfl_df(const DF& x, int m) {
  return DF{__shfl_xor_sync(0xffffffffu, x.h, m), __shfl_xor_sync(0xffffffffu, x.l, m)};
}

__global__ void __launch_bounds__(RC_THREADS) k_inc_recover(const cd* __restrict__ v, const cd* __restrict__ g,
                                                            cd* __restrict__ u, cd* __restrict__ w,
                                                            cd* __restrict__ ox, cd* __restrict__ oz,
                                                            const double* __restrict__ iapha,
                                                            const double* __restrict__ ibeta, Dims d) {
  const long modes = d.modes(), ncols = 2 * modes;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = (int)(t & 1), par = (int)((t >> 1) & 1);
  const long mt = t >> 2;
  const bool in = mt < modes;  // every lane takes part in the shuffles
  const long m = in ? mt : 0;
  const long col = 2 * m + comp;
  // not a channel's (0,0) mode nor its spanwise Nyquist slot
  const bool live = in && (m % d.chm) > 0 && ((m % d.chm) / d.KX) != d.NYQ;
  double sak = 0.0, sbk = 0.0, sa = 0.0, sb = 0.0;
  if (live) {
    // (i z)_re = -z_im, (i z)_im = z_re: the sign s of the partner term
    const double s = comp ? 1.0 : -1.0;
    const double a = iapha[m % d.KX], b = ibeta[m / d.KX], ik2 = 1.0 / (a * a + b * b);
    sa = s * a;
    sb = s * b;
    sak = sa * ik2;
    sbk = sb * ik2;
  }
  const DF c_ak = df_of(sak), c_bk = df_of(sbk), c_a = df_of(sa), c_b = df_of(sb);
  const DF c_nak = DF{-c_ak.h, -c_ak.l}, c_nbk = DF{-c_bk.h, -c_bk.l}, c_nb = DF{-c_b.h, -c_b.l};
  const double* vd = reinterpret_cast<const double*>(v);
  const double* gd = reinterpret_cast<const double*>(g);
  double* ud = reinterpret_cast<double*>(u);
  double* wd = reinterpret_cast<double*>(w);
  double* oxd = reinterpret_cast<double*>(ox);
  double* ozd = reinterpret_cast<double*>(oz);
  const int N = d.N;
  const int ktop = ((N - par) & ~1) | par;  // the largest k <= N with k = par (mod 2)
  const int nsteps = N / 2 + 1;             // the even chain's rows N, N-2, ..., 0 (N is even)
  // this chain's Dv, D^2 v, Dg at k + 2; the other chain's Dv at k + 1 and
  // v, g at row k + 1
  const DF zero{0.f, 0.f};
  DF dv2 = zero, d2v2 = zero, dg2 = zero, dvx = zero, vu = zero, gu = zero;
  for (int s0 = 0; s0 < nsteps; s0 += RC_PF) {
    double vk[RC_PF], gk[RC_PF];
#pragma unroll
    for (int i = 0; i < RC_PF; ++i) {
      const int k = min(max(ktop - 2 * (s0 + i), 0), N);
      const size_t idx = (size_t)k * ncols + col;
      vk[i] = vd[idx];
      gk[i] = gd[idx];
    }
#pragma unroll
    for (int i = 0; i < RC_PF; ++i) {
      const int st = s0 + i;
      if (st >= nsteps) break;
      const int k = ktop - 2 * st;  // -1 for the odd chain's last step
      const bool row = k >= 0;
      const DF vv = df_of(vk[i]), gg = df_of(gk[i]);  // v, g at row k
      // v, g at row k + 1: the even thread's current row for the odd thread,
      // the odd thread's previous row for the even thread
      const DF xv = shfl_df(vv, 2), xg = shfl_df(gg, 2);
      if (par == 1) vu = xv, gu = xg;
      const bool inner = row && k < N;
      const float tk = inner ? (float)(2 * (k + 1)) : 0.f;  // exact; 0 gives the b term alone
      DF dv = df_fma_int(tk, vu, dv2), dg = df_fma_int(tk, gu, dg2);
      if (!inner) dv = zero, dg = zero;
      if (par == 0) vu = xv, gu = xg;
      // exchange Dv with the other chain: the odd thread needs the even
      // thread's Dv of this step (row k + 1), the even thread keeps the odd
      // thread's for its next step (also its row k + 1 then)
      const DF xd = shfl_df(dv, 2);
      if (par == 1) dvx = xd;
      DF d2v = df_fma_int(tk, dvx, d2v2);
      if (!inner) d2v = zero;
      if (par == 0) dvx = xd;
      dv2 = dv;
      d2v2 = d2v;
      dg2 = dg;
      if (k == 0) {  // the k = 0 outputs of dz are halved (exact)
        dv = DF{__fmul_rn(0.5f, dv.h), __fmul_rn(0.5f, dv.l)};
        dg = DF{__fmul_rn(0.5f, dg.h), __fmul_rn(0.5f, dg.l)};
        d2v = DF{__fmul_rn(0.5f, d2v.h), __fmul_rn(0.5f, d2v.l)};
      }
      // the partner component's values
      const DF dv_p = shfl_df(dv, 1), dg_p = shfl_df(dg, 1), d2v_p = shfl_df(d2v, 1);
      const DF v_p = shfl_df(vv, 1), g_p = shfl_df(gg, 1);
      if (live && row) {
        const size_t idx = (size_t)k * ncols + col;
        ud[idx] = df_dot2(c_ak, dv_p, c_nbk, g_p);                  // sak Dv - sbk g
        wd[idx] = df_dot2(c_bk, dv_p, c_ak, g_p);                   // sbk Dv + sak g
        ozd[idx] = df_dot3(c_bk, dg_p, c_nak, d2v_p, c_a, v_p);     // sbk Dg - sak D^2 v + sa v
        oxd[idx] = df_dot3(c_bk, d2v_p, c_ak, dg_p, c_nb, v_p);     // sbk D^2 v + sak Dg - sb v
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_inc_recover64: the FP64 form of k_inc_recover (above), four threads per
// mode (lane = 4 mode + 2 parity + re/im),
// grid (ceil(4 modes / RC_THREADS)); u, w, omega_x, omega_z from v and
// omega_y (getvelocityandvorticity, REF:2347-2407) for every solved mode
// (not (0,0), not the spanwise Nyquist slot):
//   u = (i a Dv - i b g) / k^2,            w = (i b Dv + i a g) / k^2,
//   omega_z = -Du + i a v = (i b Dg - i a D^2 v) / k^2 + i a v,
//   omega_x =  Dw - i b v = (i b D^2 v + i a Dg) / k^2 - i b v.
// The dz recurrences (b_0 halved on output) run in FP64 registers on
// descending rows; the even-k and odd-k chains of Dv and Dg are independent,
// so the pair of parity threads of a component runs them in lockstep (even
// rows 2s below the top, odd rows one below those); D^2 v at row k needs Dv
// at row k + 1 from the other chain, exchanged by one shuffle per step (the
// odd thread takes the even thread's current value, the even thread the odd
// thread's previous one).  The other re/im component comes by shuffle, and
// multiplying by i folds into the signs of the per-thread coefficients.  13
// FP64 operations per element; the factors 2 (k + 1) are built by integer
// operations; RC_PF steps of v and omega_y loaded ahead.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(RC_THREADS) k_inc_recover64(const cd* __restrict__ v, const cd* __restrict__ g,
                                                            cd* __restrict__ u, cd* __restrict__ w,
                                                            cd* __restrict__ ox, cd* __restrict__ oz,
                                                            const double* __restrict__ iapha,
                                                            const double* __restrict__ ibeta, Dims d) {
  const long modes = d.modes(), ncols = 2 * modes;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int comp = (int)(t & 1), par = (int)((t >> 1) & 1);
  const long mt = t >> 2;
  const bool in = mt < modes;  // every lane takes part in the shuffles
  const long m = in ? mt : 0;
  const long col = 2 * m + comp;
  // not a channel's (0,0) mode nor its spanwise Nyquist slot
  const bool live = in && (m % d.chm) > 0 && ((m % d.chm) / d.KX) != d.NYQ;
  double sak = 0.0, sbk = 0.0, sa = 0.0, sb = 0.0;
  if (live) {
    // (i z)_re = -z_im, (i z)_im = z_re: the sign s of the partner term
    const double s = comp ? 1.0 : -1.0;
    const double a = iapha[m % d.KX], b = ibeta[m / d.KX], ik2 = 1.0 / (a * a + b * b);
    sa = s * a;
    sb = s * b;
    sak = sa * ik2;
    sbk = sb * ik2;
  }
  const double* vd = reinterpret_cast<const double*>(v);
  const double* gd = reinterpret_cast<const double*>(g);
  double* ud = reinterpret_cast<double*>(u);
  double* wd = reinterpret_cast<double*>(w);
  double* oxd = reinterpret_cast<double*>(ox);
  double* ozd = reinterpret_cast<double*>(oz);
  const int N = d.N;
  const int ktop = ((N - par) & ~1) | par;  // the largest k <= N with k = par (mod 2)
  const int nsteps = N / 2 + 1;             // the even chain's rows N, N-2, ..., 0 (N is even)
  // this chain's Dv, D^2 v, Dg at k + 2; the other chain's Dv at k + 1
  double dv2 = 0.0, d2v2 = 0.0, dg2 = 0.0, dvx = 0.0;
  for (int s0 = 0; s0 < nsteps; s0 += RC_PF) {
    double vk[RC_PF], gk[RC_PF], vu[RC_PF], gu[RC_PF];
#pragma unroll
    for (int i = 0; i < RC_PF; ++i) {
      const int k = min(max(ktop - 2 * (s0 + i), 0), N);
      const size_t idx = (size_t)k * ncols + col, iup = (size_t)min(k + 1, N) * ncols + col;
      vk[i] = vd[idx];
      gk[i] = gd[idx];
      vu[i] = vd[iup];
      gu[i] = gd[iup];
    }
#pragma unroll
    for (int i = 0; i < RC_PF; ++i) {
      const int st = s0 + i;
      if (st >= nsteps) break;
      const int k = ktop - 2 * st;  // -1 for the odd chain's last step
      const bool row = k >= 0;
      double dv = 0.0, dg = 0.0;
      if (row && k < N) {
        const double tk = bits::from_int(2u * (uint32_t)(k + 1));
        dv = fma(tk, vu[i], dv2);
        dg = fma(tk, gu[i], dg2);
      }
      // exchange with the other chain: the odd thread needs the even thread's
      // Dv of this step (row k + 1), the even thread keeps the odd thread's
      // for its next step (also its row k + 1 then)
      const double xv = __shfl_xor_sync(0xffffffffu, dv, 2);
      if (par == 1) dvx = xv;
      double d2v = 0.0;
      if (row && k < N) d2v = fma(bits::from_int(2u * (uint32_t)(k + 1)), dvx, d2v2);
      if (par == 0) dvx = xv;
      dv2 = dv;
      d2v2 = d2v;
      dg2 = dg;
      if (k == 0) {  // the k = 0 outputs of dz are halved
        dv = bits::half(dv);
        d2v = bits::half(d2v);
        dg = bits::half(dg);
      }
      const double dv_p = __shfl_xor_sync(0xffffffffu, dv, 1);
      const double d2v_p = __shfl_xor_sync(0xffffffffu, d2v, 1);
      const double dg_p = __shfl_xor_sync(0xffffffffu, dg, 1);
      const double v_p = __shfl_xor_sync(0xffffffffu, vk[i], 1);
      const double g_p = __shfl_xor_sync(0xffffffffu, gk[i], 1);
      if (live && row) {
        const size_t idx = (size_t)k * ncols + col;
        ud[idx] = fma(sak, dv_p, -(sbk * g_p));
        wd[idx] = fma(sbk, dv_p, sak * g_p);
        ozd[idx] = fma(sbk, dg_p, fma(-sak, d2v_p, sa * v_p));
        oxd[idx] = fma(sbk, d2v_p, fma(sak, dg_p, -(sb * v_p)));
      }
    }
  }
}

}  // namespace

int setup_solver_mixed(Handle* h) {
  const SolveLayout& sl = h->sl;
  const size_t n = sl.stride * (size_t)h->nk2;
  if (n == 0) return CHF_OK;
  if (!cuda_ok(h, cudaMalloc((void**)&h->incm, sizeof(float2) * n), "increment operators") ||
      !cuda_ok(h, cudaMalloc((void**)&h->incx, sizeof(float) * n), "increment operators") ||
      !cuda_ok(h, cudaMalloc((void**)&h->incr_exp, (size_t)2 * h->d.NZ * h->nk2), "increment operators"))
    return CHF_E_NOMEM;
  const int nmax = std::max(sl.ne_v, sl.ne_w);
  const size_t smem = sizeof(double) * (size_t)nmax * BW;
  if (smem > 48 * 1024 &&
      !cuda_ok(h, cudaFuncSetAttribute(k_build_incr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "k_build_incr smem"))
    return CHF_E_CUDA;
  k_build_incr<<<dim3(h->nk2, 4), 256, smem, h->stream>>>(h->t0, h->t2, h->t4, h->k2vals, h->xinv, sl, h->d.N,
                                                          h->cfg.dt / h->cfg.re, h->incm, h->incx);
  if (!cuda_ok(h, cudaGetLastError(), "k_build_incr")) return CHF_E_CUDA;
  k_incr_rowexp<<<dim3(h->nk2, 4), 128, 0, h->stream>>>(h->incm, sl, h->incr_exp);
  if (!cuda_ok(h, cudaGetLastError(), "k_incr_rowexp") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "k_build_incr sync"))
    return CHF_E_CUDA;
  // k_inc_recover's double-float form from 16 warps per SM on (measured on
  // GB300: at 7 warps per SM, 128^3, it is issue-bound and 14% slower than
  // the FP64 form; at 60, 384 x 193 x 384, 17% faster)
  int nsm = 0;
  if (!cuda_ok(h, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device), "SM count"))
    return CHF_E_CUDA;
  h->rec_df_rule = (4 * h->d.modes() + 31) / 32 >= 16L * nsm;
  return setup_inc_items(h);
}

// Work items of k_inc_solve, one CTA each: a k^2 group's modes in runs of at
// most 4 (the first n_inc_items[1] entries) or 2 (the next n_inc_items[0]).
// The runs of one group are adjacent in the list, so the CTAs that stream the
// same operators run at the same time and share them through L2 instead of a
// group's later runs reading them from HBM again.  Groups stay in k^2 order:
// modes next to each other in memory (kx, kx + 1) have nearby k^2, so the
// CTAs that gather them run close in time and the other half of each 32-byte
// sector of the mode-major fields is still in L2.
int setup_inc_items(Handle* h) {
  const int ng = h->nk2;
  std::vector<int> gs(ng + 1);
  if (!cuda_ok(h, cudaMemcpy(gs.data(), h->group_start, sizeof(int) * gs.size(), cudaMemcpyDeviceToHost),
               "increment solve items"))
    return CHF_E_CUDA;
  std::vector<int2> items;
  for (int mch : {4, 2}) {
    const size_t first = items.size();
    for (int g = 0; g < ng; ++g)
      for (int base = gs[g]; base < gs[g + 1]; base += mch) items.push_back(make_int2(g, base));
    h->n_inc_items[mch == 4 ? 1 : 0] = (int)(items.size() - first);
  }
  if (items.empty()) return CHF_OK;
  if (!cuda_ok(h, cudaMalloc((void**)&h->inc_items, sizeof(int2) * items.size()), "increment solve items") ||
      !cuda_ok(h, cudaMemcpy(h->inc_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice),
               "increment solve items"))
    return CHF_E_NOMEM;
  return CHF_OK;
}

int launch_solve_mixed(Handle* h) {
  const Dims& d = h->d;
  const int NZ = d.NZ;
  const long modes = d.modes();
  const double dt = h->cfg.dt;
  cudaStream_t st = h->stream;
  cudaEvent_t ev;
  // the (0,0) mode touches only mode-0 entries and the mean arrays, which
  // the kernels below neither write nor use: it runs beside them on the side
  // stream (in order on the handle's stream while kernels are being timed)
  const bool fork = h->side_stream && !h->profiling;
  if (fork) {
    if (!cuda_ok(h, cudaEventRecord(h->ev_fork, st), "solve fork") ||
        !cuda_ok(h, cudaStreamWaitEvent(h->side_stream, h->ev_fork, 0), "solve fork"))
      return CHF_E_CUDA;
    const int rc = launch_solve_mean(h, h->side_stream);
    if (rc != CHF_OK) return rc;
    if (!cuda_ok(h, cudaEventRecord(h->ev_join, h->side_stream), "solve join")) return CHF_E_CUDA;
  }
  if (h->nk2 > 0) {
    const SolveLayout& sl = h->sl;
    const int rows = sl.ne_v + sl.no_v + sl.ne_w + sl.no_w;
    const int mch = h->tune.inc_mch == 2 ? 2 : 4, cb = h->tune.inc_cb;
    // the wide block only where one row per thread at MV_THREADS would loop
    const int rpt = h->tune.inc_rpt == 2 ? 2 : h->tune.inc_wide && rows > MV_THREADS ? 0 : 1;
    auto kern = rpt == 2 ? (mch == 2 ? (cb == 2 ? k_inc_solve<2, 2, 2> : k_inc_solve<2, 3, 2>)
                                     : (cb == 2 ? k_inc_solve<4, 2, 2> : k_inc_solve<4, 3, 2>))
              : rpt == 0 ? (mch == 2 ? (cb == 2 ? k_inc_solve<2, 2, 0> : cb == 4 ? k_inc_solve<2, 4, 0> : k_inc_solve<2, 3, 0>)
                                     : (cb == 2 ? k_inc_solve<4, 2, 0> : cb == 4 ? k_inc_solve<4, 4, 0> : k_inc_solve<4, 3, 0>))
              : mch == 2 ? (cb == 2 ? k_inc_solve<2, 2, 1> : cb == 4 ? k_inc_solve<2, 4, 1> : k_inc_solve<2, 3, 1>)
                         : (cb == 2 ? k_inc_solve<4, 2, 1> : cb == 4 ? k_inc_solve<4, 4, 1> : k_inc_solve<4, 3, 1>);
    const int slots2 = (sl.ne_v + 1) / 2 + (sl.no_v + 1) / 2 + (sl.ne_w + 1) / 2 + (sl.no_w + 1) / 2;
    const int threads = rpt == 1 ? MV_THREADS
                      : rpt == 0 ? std::min(MV_WIDE, (rows + 31) / 32 * 32)
                                 : std::min(256, (slots2 + 31) / 32 * 32);
    const size_t smem = (sizeof(cd) + sizeof(CoefHL) + sizeof(float2)) * mch * 2 * (size_t)NZ;
    if (smem > 48 * 1024 &&
        !cuda_ok(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "k_inc_solve smem"))
      return CHF_E_CUDA;
    prof_begin(h, K_INC_SOLVE, &ev);
    const int nitems = h->n_inc_items[mch == 4 ? 1 : 0];
    const int2* items = h->inc_items + (mch == 4 ? 0 : h->n_inc_items[1]);
    kern<<<nitems, threads, smem, st>>>(h->f[F_V], h->f[F_OY], h->f[F_RV], h->f[F_U], h->f[F_RG],
                                           h->f[F_W], h->incm, h->incx, h->incr_exp, h->sl, h->group_start,
                                           h->group_modes, items, d, (float)(1.5 * dt), (float)(0.5 * dt));
    prof_end(h, K_INC_SOLVE, ev);
    if (h->after_inc && !cuda_ok(h, cudaEventRecord(h->after_inc, st), "increment solve event")) return CHF_E_CUDA;
  }
  {
    // the double-float form where the grid gives it enough warps to hide its
    // longer instruction stream, the FP64 form otherwise (fixed per grid)
    const bool df = h->tune.rec_form >= 0 ? h->tune.rec_form == 1 : h->rec_df_rule;
    auto kern = df ? k_inc_recover : k_inc_recover64;
    prof_begin(h, K_INC_RECOVER, &ev);
    kern<<<(unsigned)((4 * modes + RC_THREADS - 1) / RC_THREADS), RC_THREADS, 0, st>>>(
        h->f[F_V], h->f[F_OY], h->f[F_U], h->f[F_W], h->f[F_OX], h->f[F_OZ], h->iapha, h->ibeta, d);
    prof_end(h, K_INC_RECOVER, ev);
  }
  if (!cuda_ok(h, cudaGetLastError(), "mixed solve")) return CHF_E_CUDA;
  if (fork) return cuda_ok(h, cudaStreamWaitEvent(st, h->ev_join, 0), "solve join") ? CHF_OK : CHF_E_CUDA;
  // the (0,0) mode: the FP64 solve kernel, its last CTA only
  return launch_solve_mean(h, st);
}

}  // namespace chf
