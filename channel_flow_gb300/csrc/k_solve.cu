// k_solve.cu -- the implicit half of the time step on one GB300.
//
// Reference: the per-mode loop poiseuilleflow.f90:242-394 (AB2 + Crank-
// Nicolson collocation equations for v and omega_y, solved by applying the
// explicit inverse computed once with zgetrf/zgetri at poiseuilleflow.f90:
// 181-214), velocity/vorticity recovery getvelocityandvorticity
// (poiseuilleflow.f90:2347-2407) and the (0,0)-mode solve
// (poiseuilleflow.f90:401-474, gsij full-pivot elimination every step).
//
// Design:
//  * The operators depend on k^2 only (their alpha terms are switched off in
//    the reference, tmpi = 0 at poiseuilleflow.f90:3363-3365, 3445), so one
//    inverse is kept per distinct k^2 and modes are grouped by k^2: a CTA
//    loads each inverse once for all modes that share it.
//  * Collocation points z_p and z_{N-p} are mirror images and T_j, T_j'' and
//    T_j'''' have parity (-1)^j there, so sums/differences of mirrored rows
//    (and of the paired boundary rows) split each operator into an even-j and
//    an odd-j block of half size: half the FP64 multiply-adds and half the
//    matrix bytes of the dense inverse, same solution to rounding.
//  * The explicit right-hand side B c (get_coef_rhs, get_rhs_omegay,
//    get_rhs_u0; dense O(N^2) per mode in the reference) is evaluated as the
//    Gauss-Lobatto values of the Chebyshev series
//    (dt/2re) D^4 v + (1 - k^2 dt/re) D^2 v - k^2 (1 - k^2 dt/2re) v
//    (or (dt/2re) D^2 w + (1 - k^2 dt/2re) w), i.e. derivative recurrences and
//    one length-2N DFT per equation.
//  * The (0,0) operator equals the omega_y operator at k^2 = 0, so the mean
//    mode is the last "group" with k^2 = 0 and reuses the same code path; its
//    inverse replaces the per-step full-pivot elimination of gsij.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "chf_internal.h"

namespace chf {

namespace {

constexpr int S_THREADS = 256;
constexpr int INV_THREADS = 256;

// ---------------------------------------------------------------------------
// Set-up: assemble one even/odd block of the v or omega_y collocation
// operator (get_coef_v REF:3348-3381, get_coef_omegay REF:3432-3455) for one
// k^2 and invert it in place by Gauss-Jordan elimination with partial
// pivoting.  grid (nk2 + 1, 4): block 0 v-even, 1 v-odd, 2 w-even, 3 w-odd.
// Output column-major: X[c * n + r] is row r, column c.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(INV_THREADS) k_invert(const double* __restrict__ t0,
                                                        const double* __restrict__ t2,
                                                        const double* __restrict__ t4,
                                                        const double* __restrict__ k2vals,
                                                        double* __restrict__ xinv, SolveLayout sl,
                                                        int N, double dt, double re,
                                                        int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int g = blockIdx.x, blk = blockIdx.y;
  const int NZ = N + 1;
  const double k2 = k2vals[g];
  const bool isv = blk < 2, even = (blk % 2) == 0;
  const int n = isv ? (even ? sl.ne_v : sl.no_v) : (even ? sl.ne_w : sl.no_w);
  double* A = reinterpret_cast<double*>(smem_raw);  // row-major n x n: A[r*n + c]
  double* fcol = A + n * n;                          // n
  int* piv = reinterpret_cast<int*>(fcol + n);       // n
  __shared__ int s_p;
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    int r = t / n, c = t % n;
    int j = even ? 2 * c : 2 * c + 1;
    double val;
    if (isv) {
      if (r == 0) val = 1.0;
      else if (r == 1) val = (double)j * (double)j;
      else {
        size_t p = (size_t)r + (size_t)NZ * j;  // point p = r
        val = -(t4[p] * dt * 0.5 / re) + (1.0 + k2 * dt / re) * t2[p] -
              k2 * (1.0 + k2 * dt * 0.5 / re) * t0[p];
      }
    } else {
      if (r == 0) val = 1.0;
      else {
        size_t p = (size_t)r + (size_t)NZ * j;
        val = -(t2[p] * dt * 0.5 / re) + (1.0 + k2 * dt * 0.5 / re) * t0[p];
      }
    }
    A[r * n + c] = val;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot: first row of maximal |A[i][k]|, i >= k
    if (threadIdx.x < 32) {
      double best = -1.0;
      int bi = k;
      for (int i = k + threadIdx.x; i < n; i += 32) {
        double a = fabs(A[i * n + k]);
        if (a > best) { best = a; bi = i; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        double ob = __shfl_down_sync(0xffffffffu, best, off);
        int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (threadIdx.x == 0) {
        s_p = bi;
        piv[k] = bi;
        if (!(best > 0.0)) s_bad = 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (p != k)
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double tmp = A[k * n + c];
        A[k * n + c] = A[p * n + c];
        A[p * n + c] = tmp;
      }
    __syncthreads();
    const double inv = 1.0 / A[k * n + k];
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      double v = (c == k) ? 1.0 : A[k * n + c];
      A[k * n + c] = v * inv;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) fcol[i] = (i == k) ? 0.0 : A[i * n + k];
    __syncthreads();
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
      int i = t / n, c = t % n;
      if (i == k) continue;
      double f = fcol[i];
      double base = (c == k) ? 0.0 : A[i * n + c];
      A[i * n + c] = base - f * A[k * n + c];
    }
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last to first
  for (int k = n - 1; k >= 0; --k) {
    int p = piv[k];
    if (p != k)
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        double tmp = A[r * n + k];
        A[r * n + k] = A[r * n + p];
        A[r * n + p] = tmp;
      }
    __syncthreads();
  }
  BlockOffsets bo = block_offsets(sl);
  size_t off = blk == 0 ? bo.ve : blk == 1 ? bo.vo : blk == 2 ? bo.we : bo.wo;
  double* X = xinv + (size_t)g * sl.stride + off;
  for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
    int r = t / n, c = t % n;
    X[(size_t)c * n + r] = A[r * n + c];
  }
  if (threadIdx.x == 0 && s_bad) atomicExch(status, 1);
}

// ---------------------------------------------------------------------------
// Per-group solve: one CTA per distinct k^2 (plus one for the (0,0) mode),
// modes of the group processed CH at a time.
// ---------------------------------------------------------------------------
struct SolveArgs {
  cd *v, *oy, *u, *w, *ox, *oz;       // state (u, w hold the N^{n-1} histories on entry)
  const cd *rv, *rg;                  // N^n histories (GL values)
  double *cl1n, *cl1nm1, *cl3n, *cl3nm1, *au0, *w0;
  const double *iapha, *ibeta, *k2vals, *xinv;
  const int *group_start, *group_modes;
  SolveLayout sl;
  Dims d;
  double dt, re;
  FftPlan pz2;
  const cd* tw2;
  int nk2;
  int g0;  // group of CTA 0 (nk2: the (0,0) mode alone)
  // constant flow rate: influence function phi of a unit mean pressure
  // gradient over one step, its bulk velocity, and the device word
  // flow = {target bulk velocity (0: off), last correction, bulk before, bulk after}
  const double* phi;
  double ubphi;
  double* flow;
  // stacked channels (d.nch > 1): groups nk2 .. nk2 + nch - 1 are the
  // channels' (0,0) modes; per group Reynolds number, per channel phi
  // ([nch][NZ]), flow word ([nch][4]), mean arrays ([nch][2 NZ]) and bulk
  // velocity of phi; group_re NULL: re and ubphi above for every group
  const double* group_re;
  const double* ubphi_dev;
};


constexpr int CH = 2;          // modes per chunk
constexpr int S_WARPS = S_THREADS / 32;

// Chebyshev derivative (dz, REF:570-599) of a real sequence a[0..N] (stride
// as) into b (stride bs), by one warp: b_i = c_i sum_{j>i, j-i odd} 2 j a_j
// (c_0 = 1/2) evaluated as suffix sums over each parity class, lane-local
// then a warp scan.  Same sums as the serial recurrence, tree-ordered.
// tj[j] = 2 j (a per-CTA table, so no int-to-double conversion per element).
constexpr int WD_EMAX = 8;  // elements per lane: N + 1 <= 256
__device__ __forceinline__ void warp_deriv(const double* a, int as, double* b, int bs, int N,
                                           const double* __restrict__ tj) {
  const int lane = threadIdx.x & 31;
  const int E = (N + 32) / 32;  // elements per lane (N + 1 <= 32 * E)
  const int i0 = lane * E;
  double g[WD_EMAX];
  double te = 0.0, to = 0.0;    // lane totals of g_j over even / odd j
#pragma unroll
  for (int q = 0; q < WD_EMAX; ++q) {
    const int j = i0 + q;
    g[q] = 0.0;
    if (q < E && j <= N) {
      g[q] = tj[j] * a[j * as];
      if (j & 1) to += g[q]; else te += g[q];
    }
  }
  double se = te, so = to;      // inclusive suffix scan over lanes
  for (int off = 1; off < 32; off <<= 1) {
    double ue = __shfl_down_sync(0xffffffffu, se, off);
    double uo = __shfl_down_sync(0xffffffffu, so, off);
    if (lane + off < 32) { se += ue; so += uo; }
  }
  double re_ = se - te, ro = so - to;  // sums over lanes above this one
#pragma unroll
  for (int q = WD_EMAX - 1; q >= 0; --q) {
    const int i = i0 + q;
    if (q < E && i <= N) {
      double bi = (i & 1) ? re_ : ro;  // sum over j > i of the opposite parity
      if (i == 0) bi *= 0.5;
      b[i * bs] = bi;
      if (i & 1) ro += g[q]; else re_ += g[q];
    }
  }
  __syncwarp();
}

struct ChunkSmem {
  double* tj; // [NZ] 2 j
  cd* cv;     // [CH][NZ] v coefficients  -> new v
  cd* co;     // [CH][NZ] omega_y coeffs  -> new omega_y
  cd* rv;     // [CH][NZ] AB2 explicit term of the v equation (GL values)
  cd* rg;     // [CH][NZ] AB2 explicit term of the omega_y equation
  cd* fb;     // [2 CH][2N] DFT lines
  double* dd; // [CH][10][NZ] derivative scratch; also the even/odd rhs
};

__device__ __forceinline__ double* dslot(const ChunkSmem& s, int m, int q, int NZ) {
  return s.dd + ((size_t)m * 10 + q) * NZ;
}

// MB2 bounds the radix-2 butterflies per thread of the 2N-point DFTs (2 up
// to nnz = 128, 4 up to nnz = 256)
template <int MB2>
__global__ void __launch_bounds__(S_THREADS, 3) k_solve(const __grid_constant__ SolveArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Dims& d = a.d;
  const int N = d.N, NZ = d.NZ, L2 = 2 * N;
  const long modes = d.modes();
  const int tid = threadIdx.x, warp = tid >> 5;
  ChunkSmem s;
  {
    cd* p = reinterpret_cast<cd*>(smem_raw);
    s.cv = p; p += CH * NZ;
    s.co = p; p += CH * NZ;
    s.rv = p; p += CH * NZ;
    s.rg = p; p += CH * NZ;
    s.fb = p; p += 2 * CH * L2;
    s.dd = reinterpret_cast<double*>(p);
    s.tj = s.dd + (size_t)CH * 10 * NZ;
  }
  for (int j = threadIdx.x; j < NZ; j += blockDim.x) s.tj[j] = 2.0 * (double)j;
  __syncthreads();
  const int g = blockIdx.x + a.g0;
  const bool mean = (g >= a.nk2);
  const int mch = mean ? g - a.nk2 : 0;      // the channel of a (0,0) group
  const long mean_mode = (long)mch * d.chm;  // its (0,0) mode
  const double dt = a.dt, re = a.group_re ? a.group_re[g] : a.re;
  double* const au0 = a.au0 + (size_t)mch * 2 * NZ;
  double* const w0 = a.w0 + (size_t)mch * 2 * NZ;
  const double* const cl1n = a.cl1n + (size_t)mch * 2 * NZ;
  const double* const cl1nm1 = a.cl1nm1 + (size_t)mch * 2 * NZ;
  const double* const cl3n = a.cl3n + (size_t)mch * 2 * NZ;
  const double* const cl3nm1 = a.cl3nm1 + (size_t)mch * 2 * NZ;
  const double k2 = mean ? 0.0 : a.k2vals[g];
  const double* X = a.xinv + (size_t)g * a.sl.stride;
  const SolveLayout& sl = a.sl;
  BlockOffsets bo = block_offsets(sl);
  const int gs = mean ? 0 : a.group_start[g], ge = mean ? 2 : a.group_start[g + 1];
  const double c3 = 3.0 * dt / 2.0, c1 = dt / 2.0;
  for (int base = gs; base < ge; base += CH) {
    const int nm = min(CH, ge - base);
    // ---- A: load coefficients and explicit AB2 terms
    for (int t = tid; t < CH * NZ; t += blockDim.x) {
      int m = t / NZ, n = t % NZ;
      cd v{0.0, 0.0}, oy{0.0, 0.0}, rv{0.0, 0.0}, rg{0.0, 0.0};
      if (m < nm) {
        if (mean) {
          const double* am = m == 0 ? au0 : w0;
          const double* cln = m == 0 ? cl1n : cl3n;
          const double* clm = m == 0 ? cl1nm1 : cl3nm1;
          oy = cd{am[2 * n], am[2 * n + 1]};
          rg = cd{-1.0 * dt / 2.0 * (3.0 * cln[2 * n] - clm[2 * n]),
                  -1.0 * dt / 2.0 * (3.0 * cln[2 * n + 1] - clm[2 * n + 1])};
        } else {
          const int mode = a.group_modes[base + m];
          size_t idx = (size_t)n * modes + mode;
          v = a.v[idx];
          oy = a.oy[idx];
          cd x = a.rv[idx], y = a.u[idx];
          rv = cd{(c3 * x.re - c1 * y.re) * 1.0, (c3 * x.im - c1 * y.im) * 1.0};
          x = a.rg[idx];
          y = a.w[idx];
          rg = cd{(c3 * x.re - c1 * y.re) * 1.0, (c3 * x.im - c1 * y.im) * 1.0};
        }
      }
      s.cv[t] = v;
      s.co[t] = oy;
      s.rv[t] = rv;
      s.rg[t] = rg;
    }
    __syncthreads();
    // ---- B: derivatives, one warp per chain.  task (m, comp): comp 0/1 =
    // v re/im (D1..D4 into slots comp*4 + 0..3), comp 2/3 = omega_y re/im
    // (D1 into this mode's omega DFT line, free until phase C; D2 into slot
    // 8 + comp - 2)
    for (int task = warp; task < CH * 4; task += S_WARPS) {
      int m = task / 4, comp = task % 4;
      if (m >= nm) continue;
      if (comp < 2) {
        if (mean) continue;
        const double* src = reinterpret_cast<const double*>(s.cv + m * NZ) + comp;
        double* o = dslot(s, m, comp * 4, NZ);
        warp_deriv(src, 2, o, 1, N, s.tj);
        warp_deriv(o, 1, o + NZ, 1, N, s.tj);
        warp_deriv(o + NZ, 1, o + 2 * NZ, 1, N, s.tj);
        warp_deriv(o + 2 * NZ, 1, o + 3 * NZ, 1, N, s.tj);
      } else {
        const int c = comp - 2;
        const double* src = reinterpret_cast<const double*>(s.co + m * NZ) + c;
        double* t1 = reinterpret_cast<double*>(s.fb + (2 * m + 1) * L2) + c * NZ;
        warp_deriv(src, 2, t1, 1, N, s.tj);
        warp_deriv(t1, 1, dslot(s, m, 8 + c, NZ), 1, N, s.tj);
      }
    }
    __syncthreads();
    // ---- C: explicit right-hand sides as Chebyshev series -> DFT lines
    {
      const double v4 = dt * 0.5 / re, v2 = 1.0 - k2 * dt / re, v0 = -k2 * (1.0 - k2 * dt * 0.5 / re);
      const double w2 = dt * 0.5 / re, w0 = 1.0 - k2 * dt * 0.5 / re;
      for (int t = tid; t < CH * NZ; t += blockDim.x) {
        int m = t / NZ, n = t % NZ;
        cd* lv = s.fb + (2 * m) * L2;
        cd* lw = s.fb + (2 * m + 1) * L2;
        cd cv = s.cv[t], co = s.co[t];
        cd wv{0.0, 0.0}, ww{0.0, 0.0};
        if (m < nm) {
          if (!mean) {
            wv.re = v4 * dslot(s, m, 3, NZ)[n] + v2 * dslot(s, m, 1, NZ)[n] + v0 * cv.re;
            wv.im = v4 * dslot(s, m, 7, NZ)[n] + v2 * dslot(s, m, 5, NZ)[n] + v0 * cv.im;
          }
          ww.re = w2 * dslot(s, m, 8, NZ)[n] + w0 * co.re;
          ww.im = w2 * dslot(s, m, 9, NZ)[n] + w0 * co.im;
        }
        double dbl = (n == 0 || n == N) ? 2.0 : 1.0;
        // the omega line's first 2*NZ doubles held D1 scratch; all reads of
        // it finished before the barrier above
        lv[n] = cd{dbl * wv.re, dbl * wv.im};
        lw[n] = cd{dbl * ww.re, dbl * ww.im};
        if (n > 0 && n < N) {
          lv[L2 - n] = wv;
          lw[L2 - n] = ww;
        }
      }
    }
    __syncthreads();
    smem_fft<double, -1, MB2>(s.fb, 2 * CH, L2, a.pz2, a.tw2);
    // ---- D: fold the collocation rows into even / odd right-hand sides.
    // rhs storage reuses dd: [CH][4 blocks][NZ] complex (fits in 10*NZ doubles)
    const int nev = sl.ne_v, nov = sl.no_v, new_ = sl.ne_w, now_ = sl.no_w;
    cd* rhs = reinterpret_cast<cd*>(s.dd);  // rhs[(m*4 + b) * NZ + r]
    for (int t = tid; t < CH * NZ; t += blockDim.x) {
      int m = t / NZ, r = t % NZ;
      const cd* lv = s.fb + (2 * m) * L2;
      const cd* lw = s.fb + (2 * m + 1) * L2;
      cd ev{0.0, 0.0}, ovv{0.0, 0.0}, ew{0.0, 0.0}, ow{0.0, 0.0};
      if (m < nm && r <= N / 2) {
        int p = r, q = N - r;
        if (!mean && r >= 2) {
          cd Rp{0.5 * lv[p].re + s.rv[m * NZ + p].re, 0.5 * lv[p].im + s.rv[m * NZ + p].im};
          cd Rq{0.5 * lv[q].re + s.rv[m * NZ + q].re, 0.5 * lv[q].im + s.rv[m * NZ + q].im};
          ev = cd{0.5 * (Rp.re + Rq.re), 0.5 * (Rp.im + Rq.im)};
          ovv = cd{0.5 * (Rp.re - Rq.re), 0.5 * (Rp.im - Rq.im)};
        }
        if (r >= 1) {
          cd Rp{0.5 * lw[p].re + s.rg[m * NZ + p].re, 0.5 * lw[p].im + s.rg[m * NZ + p].im};
          cd Rq{0.5 * lw[q].re + s.rg[m * NZ + q].re, 0.5 * lw[q].im + s.rg[m * NZ + q].im};
          ew = cd{0.5 * (Rp.re + Rq.re), 0.5 * (Rp.im + Rq.im)};
          ow = cd{0.5 * (Rp.re - Rq.re), 0.5 * (Rp.im - Rq.im)};
        }
      }
      if (r < nev) rhs[(m * 4 + 0) * NZ + r] = ev;
      if (r < nov) rhs[(m * 4 + 1) * NZ + r] = ovv;
      if (r < new_) rhs[(m * 4 + 2) * NZ + r] = ew;
      if (r < now_) rhs[(m * 4 + 3) * NZ + r] = ow;
    }
    __syncthreads();
    // ---- E: block matvecs, each inverse element used for every mode of the chunk
    {
      const int rows = nev + nov + new_ + now_;
      for (int t = tid; t < rows; t += blockDim.x) {
        int b, row, n, r0;
        if (t < nev) { b = 0; row = t; n = nev; r0 = 2; }
        else if (t < nev + nov) { b = 1; row = t - nev; n = nov; r0 = 2; }
        else if (t < nev + nov + new_) { b = 2; row = t - nev - nov; n = new_; r0 = 1; }
        else { b = 3; row = t - nev - nov - new_; n = now_; r0 = 1; }
        if (mean && b < 2) continue;
        const double* Xb = X + (b == 0 ? bo.ve : b == 1 ? bo.vo : b == 2 ? bo.we : bo.wo);
        double acc[CH][2];
#pragma unroll
        for (int m = 0; m < CH; ++m) acc[m][0] = acc[m][1] = 0.0;
#pragma unroll 4
        for (int c = r0; c < n; ++c) {
          double xv = __ldg(Xb + (size_t)c * n + row);
#pragma unroll
          for (int m = 0; m < CH; ++m) {
            cd rr = rhs[(m * 4 + b) * NZ + c];
            acc[m][0] = fma(xv, rr.re, acc[m][0]);
            acc[m][1] = fma(xv, rr.im, acc[m][1]);
          }
        }
        int j = (b == 0 || b == 2) ? 2 * row : 2 * row + 1;
        cd* dst = b < 2 ? s.cv : s.co;
#pragma unroll
        for (int m = 0; m < CH; ++m)
          if (m < nm) dst[m * NZ + j] = cd{acc[m][0], acc[m][1]};
      }
    }
    __syncthreads();
    // ---- F: store, then getvelocityandvorticity (REF:2347-2407)
    if (mean) {
      // constant flow rate (no counterpart in the reference, which holds the
      // pressure gradient re_p fixed): add the multiple of phi that restores
      // the target bulk velocity U_b = sum_{n even} Re(au0_n) / (1 - n^2);
      // the multiple is this step's extra mean pressure gradient
      double* const flow = a.flow + 4 * mch;
      const double* const phi = a.phi + (size_t)mch * NZ;
      const double ubphi = a.ubphi_dev ? a.ubphi_dev[mch] : a.ubphi;
      const double target = flow[0];
      if (target > 0.0 && warp == 0) {
        const int lane = tid & 31;
        double ub = 0.0;
        for (int n = lane; n < NZ; n += 32)
          if (!(n & 1)) ub += s.co[n].re / (1.0 - (double)n * (double)n);
        for (int off = 16; off > 0; off >>= 1) ub += __shfl_xor_sync(0xffffffffu, ub, off);
        const double alpha = (target - ub) / ubphi;
        for (int n = lane; n < NZ; n += 32) s.co[n].re += alpha * phi[n];
        if (lane == 0) {
          flow[1] = alpha;
          flow[2] = ub;
          flow[3] = ub + alpha * ubphi;
        }
      }
      __syncthreads();
      for (int t = tid; t < nm * NZ; t += blockDim.x) {
        int m = t / NZ, n = t % NZ;
        cd x = s.co[t];
        double* am = m == 0 ? au0 : w0;
        am[2 * n] = x.re;
        am[2 * n + 1] = x.im;
        (m == 0 ? a.u : a.w)[(size_t)n * modes + mean_mode] = x;
      }
      for (int task = warp; task < nm * 2; task += S_WARPS) {
        int m = task / 2, comp = task % 2;
        warp_deriv(reinterpret_cast<const double*>(s.co + m * NZ) + comp, 2, dslot(s, m, comp, NZ), 1, N, s.tj);
      }
      __syncthreads();
      for (int t = tid; t < nm * NZ; t += blockDim.x) {
        int m = t / NZ, n = t % NZ;
        const double sg = m == 0 ? -1.0 : 1.0;  // omega_z = -D au0, omega_x = D w0
        (m == 0 ? a.oz : a.ox)[(size_t)n * modes + mean_mode] =
            cd{sg * dslot(s, m, 0, NZ)[n], sg * dslot(s, m, 1, NZ)[n]};
      }
      __syncthreads();
      continue;
    }
    for (int task = warp; task < nm * 2; task += S_WARPS) {  // Dv
      int m = task / 2, comp = task % 2;
      warp_deriv(reinterpret_cast<const double*>(s.cv + m * NZ) + comp, 2, dslot(s, m, comp, NZ), 1, N, s.tj);
    }
    __syncthreads();
    // u, w into rv / rg (free now); v and omega_y stored
    for (int t = tid; t < nm * NZ; t += blockDim.x) {
      int m = t / NZ, n = t % NZ;
      const int mode = a.group_modes[base + m];
      const int kx = mode % d.KX, ky = mode / d.KX;
      const double al = a.iapha[kx], be = a.ibeta[ky];
      const double ik2 = 1.0 / k2;
      cd vv = s.cv[t], oy = s.co[t];
      cd dv{dslot(s, m, 0, NZ)[n], dslot(s, m, 1, NZ)[n]};
      size_t idx = (size_t)n * modes + mode;
      a.v[idx] = vv;
      a.oy[idx] = oy;
      cd u{(-1.0 * al * dv.im) * ik2 + (be * oy.im) * ik2, (al * dv.re) * ik2 - (be * oy.re) * ik2};
      cd w{(-1.0 * dv.im * be) * ik2 - (1.0 * oy.im * al) * ik2, (be * dv.re) * ik2 + (al * oy.re) * ik2};
      s.rv[t] = u;
      s.rg[t] = w;
      a.u[idx] = u;
      a.w[idx] = w;
    }
    __syncthreads();
    for (int task = warp; task < nm * 4; task += S_WARPS) {  // Du (re, im), Dw (re, im)
      int m = task / 4, comp = task % 4;
      const cd* src = (comp < 2) ? s.rv + m * NZ : s.rg + m * NZ;
      warp_deriv(reinterpret_cast<const double*>(src) + (comp & 1), 2, dslot(s, m, 2 + comp, NZ), 1, N, s.tj);
    }
    __syncthreads();
    for (int t = tid; t < nm * NZ; t += blockDim.x) {
      int m = t / NZ, n = t % NZ;
      const int mode = a.group_modes[base + m];
      const int kx = mode % d.KX, ky = mode / d.KX;
      const double al = a.iapha[kx], be = a.ibeta[ky];
      cd vv = s.cv[t];
      size_t idx = (size_t)n * modes + mode;
      double dur = dslot(s, m, 2, NZ)[n], dui = dslot(s, m, 3, NZ)[n];
      double dwr = dslot(s, m, 4, NZ)[n], dwi = dslot(s, m, 5, NZ)[n];
      // omega_x = Dw - i be v ; omega_z = -Du + i al v
      a.ox[idx] = cd{dwr + be * vv.im, dwi - be * vv.re};
      a.oz[idx] = cd{-dur - al * vv.im, -dui + al * vv.re};
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Diagnostics: energy (REF:2322-2336 definition, spectral sum), max |value|,
// finiteness.  out[0] = energy sum, out[1] = max abs, out[2] = nonfinite count
// ---------------------------------------------------------------------------
__global__ void k_diag(const double* __restrict__ u, const double* __restrict__ v,
                       const double* __restrict__ w, const double* __restrict__ f4,
                       const double* __restrict__ f5, const double* __restrict__ f6, size_t n,
                       long modes, int KX, int NYQ, double* out) {
  double e = 0.0, mx = 0.0;
  unsigned long long bad = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    // the spanwise Nyquist slot is never part of the solution (it is zeroed
    // before every transform, REF:739, 811, 1358); skip it
    long mode = (long)((i >> 1) % (size_t)modes);
    if (mode / KX == NYQ) continue;
    double a = u[i], b = v[i], c = w[i];
    e += 0.5 * (a * a) + 0.5 * (b * b) + 0.5 * (c * c);
    const double vals[6] = {a, b, c, f4[i], f5[i], f6[i]};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      double x = vals[q];
      if (!isfinite(x)) ++bad;
      else mx = fmax(mx, fabs(x));
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    e += __shfl_down_sync(0xffffffffu, e, off);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
    bad += __shfl_down_sync(0xffffffffu, bad, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, e);
    atomicMax(reinterpret_cast<unsigned long long*>(out + 1), __double_as_longlong(mx));
    atomicAdd(reinterpret_cast<unsigned long long*>(out + 2), bad);
  }
}

// SCHEB (poiseuilleflow.f90:3272-3342) on the host with the reference's
// closed forms; column-major NZ x NZ, T(J, L) at J + NZ * L.
void scheb_host(int n2, std::vector<double>& t0, std::vector<double>& t2, std::vector<double>& t4) {
  const int Z = n2 + 1;
  t0.assign((size_t)Z * Z, 0.0);
  t2.assign((size_t)Z * Z, 0.0);
  t4.assign((size_t)Z * Z, 0.0);
  auto at = [Z](std::vector<double>& a, int J, int L) -> double& { return a[(size_t)J + (size_t)Z * L]; };
  const double h0 = 4.0 * std::atan(1.0) / (double)n2;
  for (int L = 0; L <= n2; ++L) {
    double Ld = (double)L, sg = (L % 2 == 0) ? 1.0 : -1.0;
    at(t0, 0, L) = 1.0;
    at(t0, n2, L) = sg;
    at(t2, 0, L) = Ld * Ld * (Ld * Ld - 1.0) / 3.0;
    at(t2, n2, L) = sg * (Ld * Ld) * (Ld * Ld - 1.0) / 3.0;
  }
  for (int J = 1; J <= n2 - 1; ++J) {
    double q = h0 * J, c1 = std::cos(q), c2 = c1 * c1, s1 = std::sin(q), s2 = s1 * s1;
    double ds1 = 1.0 / s1, ds3 = ds1 / s2, ds7 = ds3 / s2 / s2;
    for (int L = 0; L <= n2; ++L) {
      double bj = (double)L, qj = q * bj, sj = std::sin(qj), cj = std::cos(qj);
      double bs = bj * bj * s2, bc = bj * cj * s1;
      at(t0, J, L) = cj;
      at(t2, J, L) = bj * (sj * c1 - bc) * ds3;
      at(t4, J, L) = bj * (sj * c1 * (9.0 + 6.0 * (c2 - bs)) - bc * (4.0 + 11.0 * c2 - bs)) * ds7;
    }
  }
}

}  // namespace

int setup_solver(Handle* h) {
  const Dims& d = h->d;
  const int N = d.N, NZ = d.NZ;
  // wavenumbers, REF:123-134
  std::vector<double> ia(d.KX), ib(d.KY, 0.0);
  const int ny = d.KY - 1;
  for (int j = 0; j <= (ny + 1) / 2; ++j) {
    ib[j] = (double)j / h->cfg.beta;
    if (j <= (ny - 1) / 2 - 1) ib[ny - j] = (double)(-j - 1) / h->cfg.beta;
  }
  for (int i = 0; i < d.KX; ++i) ia[i] = (0.0 + (double)i) / h->cfg.aphi;
  // modes grouped by k^2 (skip the spanwise Nyquist and k^2 = 0, REF:246-249)
  std::map<double, std::vector<int>> groups;
  for (int ky = 0; ky < d.KY; ++ky)
    for (int kx = 0; kx < d.KX; ++kx) {
      double k2 = ia[kx] * ia[kx] + ib[ky] * ib[ky];
      if (ky == d.NYQ || k2 == 0.0) continue;
      groups[k2].push_back(ky * d.KX + kx);
    }
  h->nk2 = (int)groups.size();
  std::vector<double> k2v;
  std::vector<int> gstart, gmodes;
  for (auto& kv : groups) {
    gstart.push_back((int)gmodes.size());
    k2v.push_back(kv.first);
    for (int m : kv.second) gmodes.push_back(m);
  }
  gstart.push_back((int)gmodes.size());
  k2v.push_back(0.0);  // the (0,0)-mode operator
  h->nsolve = (int)gmodes.size();
  SolveLayout& sl = h->sl;
  sl.ne_v = N / 2 + 1;
  sl.no_v = N / 2;
  sl.ne_w = N / 2 + 1;
  sl.no_w = N / 2;
  sl.stride = (size_t)sl.ne_v * sl.ne_v + (size_t)sl.no_v * sl.no_v + (size_t)sl.ne_w * sl.ne_w +
              (size_t)sl.no_w * sl.no_w;
  std::vector<double> t0, t2, t4;
  scheb_host(N, t0, t2, t4);
  auto up = [h](void** dst, const void* src, size_t bytes, const char* what) {
    if (!cuda_ok(h, cudaMalloc(dst, bytes), what)) return false;
    return cuda_ok(h, cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), what);
  };
  if (!up((void**)&h->iapha, ia.data(), sizeof(double) * ia.size(), "iapha") ||
      !up((void**)&h->ibeta, ib.data(), sizeof(double) * ib.size(), "ibeta") ||
      !up((void**)&h->t0, t0.data(), sizeof(double) * t0.size(), "t0") ||
      !up((void**)&h->t2, t2.data(), sizeof(double) * t2.size(), "t2") ||
      !up((void**)&h->t4, t4.data(), sizeof(double) * t4.size(), "t4") ||
      !up((void**)&h->k2vals, k2v.data(), sizeof(double) * k2v.size(), "k2vals") ||
      !up((void**)&h->group_start, gstart.data(), sizeof(int) * gstart.size(), "group_start") ||
      !up((void**)&h->group_modes, gmodes.data(),
          sizeof(int) * std::max<size_t>(1, gmodes.size()), "group_modes"))
    return CHF_E_CUDA;
  // constant-flow-rate influence function: the mean-mode operator of
  // get_coef_u0 (REF:3493-3511) applied to phi equals a unit mean pressure
  // gradient over one step (dt on the collocation rows, as re_p enters the
  // right-hand side of REF:401-412), with phi = 0 at both walls
  {
    const int Z = NZ;
    const double dt = h->cfg.dt, re = h->cfg.re;
    std::vector<double> A((size_t)Z * Z), phi(Z, 0.0);
    for (int j = 0; j < Z; ++j) {
      A[j] = 1.0;
      A[(size_t)Z + j] = (j % 2 == 0) ? 1.0 : -1.0;
    }
    for (int i = 2; i < Z; ++i) {
      for (int j = 0; j < Z; ++j)
        A[(size_t)i * Z + j] = t0[(size_t)(i - 1) + (size_t)Z * j] - dt * 0.5 / re * t2[(size_t)(i - 1) + (size_t)Z * j];
      phi[i] = dt;
    }
    // Gaussian elimination with partial pivoting
    for (int k = 0; k < Z; ++k) {
      int p = k;
      for (int i = k + 1; i < Z; ++i)
        if (std::fabs(A[(size_t)i * Z + k]) > std::fabs(A[(size_t)p * Z + k])) p = i;
      if (A[(size_t)p * Z + k] == 0.0) {
        h->err = "mean-mode operator is singular";
        return CHF_E_NUMERIC;
      }
      if (p != k) {
        for (int j = 0; j < Z; ++j) std::swap(A[(size_t)k * Z + j], A[(size_t)p * Z + j]);
        std::swap(phi[k], phi[p]);
      }
      for (int i = k + 1; i < Z; ++i) {
        const double f = A[(size_t)i * Z + k] / A[(size_t)k * Z + k];
        for (int j = k; j < Z; ++j) A[(size_t)i * Z + j] -= f * A[(size_t)k * Z + j];
        phi[i] -= f * phi[k];
      }
    }
    for (int k = Z - 1; k >= 0; --k) {
      double acc = phi[k];
      for (int j = k + 1; j < Z; ++j) acc -= A[(size_t)k * Z + j] * phi[j];
      phi[k] = acc / A[(size_t)k * Z + k];
    }
    h->ubphi = 0.0;
    for (int n = 0; n < Z; n += 2) h->ubphi += phi[n] / (1.0 - (double)n * (double)n);
    const double zero4[4] = {0.0, 0.0, 0.0, 0.0};
    if (!up((void**)&h->phi, phi.data(), sizeof(double) * Z, "phi") ||
        !up((void**)&h->flow, zero4, sizeof(zero4), "flow"))
      return CHF_E_CUDA;
  }
  size_t xbytes = sizeof(double) * sl.stride * (size_t)(h->nk2 + 1);
  if (!cuda_ok(h, cudaMalloc((void**)&h->xinv, xbytes), "xinv")) return CHF_E_NOMEM;
  int* dstatus = nullptr;
  if (!cuda_ok(h, cudaMalloc((void**)&dstatus, sizeof(int)), "status")) return CHF_E_NOMEM;
  cudaMemsetAsync(dstatus, 0, sizeof(int), h->stream);
  const int nmax = sl.ne_v;
  size_t smem = sizeof(double) * ((size_t)nmax * nmax + nmax) + sizeof(int) * nmax + 16;
  if (smem > 48 * 1024 &&
      !cuda_ok(h, cudaFuncSetAttribute(k_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "k_invert smem"))
    return CHF_E_CUDA;
  dim3 grid(h->nk2 + 1, 4);
  k_invert<<<grid, INV_THREADS, smem, h->stream>>>(h->t0, h->t2, h->t4, h->k2vals, h->xinv, sl, N,
                                                   h->cfg.dt, h->cfg.re, dstatus);
  if (!cuda_ok(h, cudaGetLastError(), "k_invert")) return CHF_E_CUDA;
  int status = 0;
  if (!cuda_ok(h, cudaMemcpyAsync(&status, dstatus, sizeof(int), cudaMemcpyDeviceToHost, h->stream),
               "status") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "k_invert sync"))
    return CHF_E_CUDA;
  cudaFree(dstatus);
  if (status) {
    h->err = "implicit operator is singular for some k^2";
    return CHF_E_NUMERIC;
  }
  (void)NZ;
  return CHF_OK;
}

// groups g0 .. nk2 (the last CTA is the (0,0) mode)
static int launch_solve_from(Handle* h, int g0, cudaStream_t st) {
  const Dims& d = h->d;
  SolveArgs a;
  a.v = h->f[F_V];
  a.oy = h->f[F_OY];
  a.u = h->f[F_U];
  a.w = h->f[F_W];
  a.ox = h->f[F_OX];
  a.oz = h->f[F_OZ];
  a.rv = h->f[F_RV];
  a.rg = h->f[F_RG];
  a.cl1n = h->mean[M_CL1N];
  a.cl1nm1 = h->mean[M_CL1NM1];
  a.cl3n = h->mean[M_CL3N];
  a.cl3nm1 = h->mean[M_CL3NM1];
  a.au0 = h->mean[M_AU0];
  a.w0 = h->mean[M_W0];
  a.iapha = h->iapha;
  a.ibeta = h->ibeta;
  a.k2vals = h->k2vals;
  a.xinv = h->xinv;
  a.group_start = h->group_start;
  a.group_modes = h->group_modes;
  a.sl = h->sl;
  a.d = d;
  a.dt = h->cfg.dt;
  a.re = h->cfg.re;
  a.pz2 = h->pz2;
  a.tw2 = h->tw_z2;
  a.g0 = g0;
  a.phi = h->phi;
  a.ubphi = h->ubphi;
  a.flow = h->flow;
  a.nk2 = h->nk2;
  a.group_re = h->group_re;
  a.ubphi_dev = h->ubphi_dev;
  const int mb2 = fft_fits(2 * CH, 2 * d.N, S_THREADS, 2) ? 2 : 4;
  if (d.N + 1 > 32 * WD_EMAX || !fft_fits(2 * CH, 2 * d.N, S_THREADS, mb2)) {
    h->err = "k_solve: nnz too large for the launch shape";
    return CHF_E_INVALID;
  }
  size_t smem = sizeof(cd) * (4 * (size_t)CH * d.NZ + 2 * (size_t)CH * 2 * d.N) +
                sizeof(double) * (10 * (size_t)CH + 1) * d.NZ;
  auto kern = mb2 == 2 ? k_solve<2> : k_solve<4>;
  if (smem > 48 * 1024 &&
      !cuda_ok(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "k_solve smem"))
    return CHF_E_CUDA;
  cudaEvent_t ev;
  prof_begin(h, g0 == 0 ? K_SOLVE : K_SOLVE_MEAN, &ev);
  // groups g0 .. nk2 - 1 and the nch (0,0)-mode groups after them
  kern<<<h->nk2 + h->d.nch - g0, S_THREADS, smem, st>>>(a);
  prof_end(h, g0 == 0 ? K_SOLVE : K_SOLVE_MEAN, ev);
  if (!cuda_ok(h, cudaGetLastError(), "k_solve")) return CHF_E_CUDA;
  return CHF_OK;
}

int launch_solve_fp64(Handle* h) { return launch_solve_from(h, 0, h->stream); }

int launch_solve_mean(Handle* h, cudaStream_t st) { return launch_solve_from(h, h->nk2, st); }

int launch_diagnostics(Handle* h, chf_diag* out) {
  const Dims& d = h->d;
  double* s = reinterpret_cast<double*>(h->scratch);
  if (!cuda_ok(h, cudaMemsetAsync(s, 0, 3 * sizeof(double), h->stream), "diag memset"))
    return CHF_E_CUDA;
  size_t n = d.field_elems() * 2;
  k_diag<<<4 * 152, 256, 0, h->stream>>>(
      reinterpret_cast<const double*>(h->f[F_U]), reinterpret_cast<const double*>(h->f[F_V]),
      reinterpret_cast<const double*>(h->f[F_W]), reinterpret_cast<const double*>(h->f[F_OX]),
      reinterpret_cast<const double*>(h->f[F_OY]), reinterpret_cast<const double*>(h->f[F_OZ]), n,
      d.modes(), d.KX, d.NYQ, s);
  if (!cuda_ok(h, cudaGetLastError(), "k_diag")) return CHF_E_CUDA;
  double host[3];
  std::vector<double> au0(2 * (size_t)d.NZ);
  if (!cuda_ok(h, cudaMemcpyAsync(host, s, sizeof(host), cudaMemcpyDeviceToHost, h->stream), "diag") ||
      !cuda_ok(h, cudaMemcpyAsync(au0.data(), h->mean[M_AU0], sizeof(double) * au0.size(),
                                  cudaMemcpyDeviceToHost, h->stream), "diag au0") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "diag sync"))
    return CHF_E_CUDA;
  unsigned long long bad;
  memcpy(&bad, &host[2], sizeof(bad));
  out->energy = host[0];
  out->max_abs = host[1];
  out->finite = bad == 0 ? 1 : 0;
  // d<u>/dz at z = +1: sum n^2 c_n ; at z = -1: sum (-1)^(n+1) n^2 c_n
  double top = 0.0, bot = 0.0;
  for (int n = 0; n <= d.N; ++n) {
    double c = au0[2 * (size_t)n], n2 = (double)n * n;
    top += n2 * c;
    bot += ((n % 2) ? 1.0 : -1.0) * n2 * c;
  }
  out->wall_shear_top = top;
  out->wall_shear_bottom = bot;
  return out->finite ? CHF_OK : CHF_E_NUMERIC;
}

}  // namespace chf
