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

constexpr int S_THREADS = 128;
constexpr int INV_THREADS = 256;

// Offsets of the four blocks inside one k^2 entry of xinv.
struct BlockOffsets {
  size_t ve, vo, we, wo;
};

__host__ __device__ inline BlockOffsets block_offsets(const SolveLayout& s) {
  BlockOffsets b;
  b.ve = 0;
  b.vo = b.ve + (size_t)s.ne_v * s.ne_v;
  b.we = b.vo + (size_t)s.no_v * s.no_v;
  b.wo = b.we + (size_t)s.ne_w * s.ne_w;
  return b;
}

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
// Per-group solve.
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
};

// serial Chebyshev derivative of a strided real sequence (dz, REF:570-599)
__device__ __forceinline__ void dser(const double* a, int as, double* b, int bs, int N) {
  double bp1 = 0.0, bp2 = 0.0;
  b[N * bs] = 0.0;
  for (int k = N; k >= 1; --k) {
    double bk1 = bp2 + 2.0 * (double)k * a[k * as];
    if (k == 1) bk1 *= 0.5;
    b[(k - 1) * bs] = bk1;
    bp2 = bp1;
    bp1 = bk1;
  }
}

struct SolveSmem {
  cd* c;      // NZ coefficients of the current unknown
  cd* r;      // NZ explicit AB2 terms at GL points
  cd* fb;     // 2N FFT buffer
  double* dr; // 4 x NZ derivative scratch (re)
  double* di; // 4 x NZ derivative scratch (im)
  cd* e;      // ne rhs (even)
  cd* o;      // no rhs (odd)
  cd* x;      // NZ solution
};

// Values at the Gauss-Lobatto points of the series in s.fb[0..N] (already
// written as coefficients): even extension with doubled ends, forward DFT,
// halve.  Result in s.fb[p], p = 0..N.
__device__ void gl_values(SolveSmem& s, const SolveArgs& a) {
  const int N = a.d.N, L2 = 2 * N;
  for (int n = threadIdx.x; n <= N; n += blockDim.x) {
    cd v = s.fb[n];
    if (n > 0 && n < N) s.fb[L2 - n] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s.fb[0] = cd{2.0 * s.fb[0].re, 2.0 * s.fb[0].im};
    s.fb[N] = cd{2.0 * s.fb[N].re, 2.0 * s.fb[N].im};
  }
  __syncthreads();
  smem_fft<double, -1, 2>(s.fb, 1, L2, a.pz2, a.tw2);
  for (int n = threadIdx.x; n <= N; n += blockDim.x) s.fb[n] = cd{0.5 * s.fb[n].re, 0.5 * s.fb[n].im};
  __syncthreads();
}

// Solve one CN collocation equation for the unknown whose current
// coefficients are in s.c and whose explicit AB2 values are in s.r.
// isv: v equation (4th order, BC rows v(+-1) = v'(+-1) = 0) else 2nd order.
// On return the new coefficients are in s.x.
__device__ void solve_eq(SolveSmem& s, const SolveArgs& a, double k2, const double* X, bool isv) {
  const int N = a.d.N, NZ = N + 1;
  const double dt = a.dt, re = a.re;
  // derivatives: re by thread 0, im by thread 32 (different warps)
  const int nder = isv ? 4 : 2;
  if (threadIdx.x == 0 || threadIdx.x == 32) {
    const bool im = threadIdx.x == 32;
    const double* c = reinterpret_cast<const double*>(s.c) + (im ? 1 : 0);
    double* dd = im ? s.di : s.dr;
    dser(c, 2, dd, 1, N);
    for (int q = 1; q < nder; ++q) dser(dd + (q - 1) * NZ, 1, dd + q * NZ, 1, N);
  }
  __syncthreads();
  for (int n = threadIdx.x; n <= N; n += blockDim.x) {
    cd c = s.c[n];
    cd w;
    if (isv) {
      double c4 = dt * 0.5 / re, c2 = 1.0 - k2 * dt / re, c0 = -k2 * (1.0 - k2 * dt * 0.5 / re);
      w.re = c4 * s.dr[3 * NZ + n] + c2 * s.dr[NZ + n] + c0 * c.re;
      w.im = c4 * s.di[3 * NZ + n] + c2 * s.di[NZ + n] + c0 * c.im;
    } else {
      double c2 = dt * 0.5 / re, c0 = 1.0 - k2 * dt * 0.5 / re;
      w.re = c2 * s.dr[NZ + n] + c0 * c.re;
      w.im = c2 * s.di[NZ + n] + c0 * c.im;
    }
    s.fb[n] = w;
  }
  __syncthreads();
  gl_values(s, a);
  // right-hand side at the collocation points, folded into even/odd parts
  const SolveLayout& sl = a.sl;
  const int ne = isv ? sl.ne_v : sl.ne_w, no = isv ? sl.no_v : sl.no_w;
  const int r0 = isv ? 2 : 1;  // first interior row of the blocks
  for (int r = threadIdx.x; r < ne; r += blockDim.x) {
    cd e{0.0, 0.0}, o{0.0, 0.0};
    if (r >= r0) {
      int p = r, q = N - r;
      cd Rp{s.fb[p].re + s.r[p].re, s.fb[p].im + s.r[p].im};
      cd Rq{s.fb[q].re + s.r[q].re, s.fb[q].im + s.r[q].im};
      e = cd{0.5 * (Rp.re + Rq.re), 0.5 * (Rp.im + Rq.im)};
      o = cd{0.5 * (Rp.re - Rq.re), 0.5 * (Rp.im - Rq.im)};
    }
    s.e[r] = e;
    if (r < no) s.o[r] = o;
  }
  __syncthreads();
  // matvecs: even rows then odd rows; X blocks column-major
  BlockOffsets bo = block_offsets(sl);
  const double* Xe = X + (isv ? bo.ve : bo.we);
  const double* Xo = X + (isv ? bo.vo : bo.wo);
  for (int t = threadIdx.x; t < ne + no; t += blockDim.x) {
    const bool ev = t < ne;
    const int row = ev ? t : t - ne, n = ev ? ne : no;
    const double* Xb = ev ? Xe : Xo;
    const cd* rhs = ev ? s.e : s.o;
    double ar = 0.0, ai = 0.0;
    for (int c = r0; c < n; ++c) {
      double xv = __ldg(Xb + (size_t)c * n + row);
      ar = fma(xv, rhs[c].re, ar);
      ai = fma(xv, rhs[c].im, ai);
    }
    int j = ev ? 2 * row : 2 * row + 1;
    s.x[j] = cd{ar, ai};
  }
  __syncthreads();
}

__global__ void __launch_bounds__(S_THREADS) k_solve(const __grid_constant__ SolveArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Dims& d = a.d;
  const int N = d.N, NZ = d.NZ;
  const long modes = d.modes();
  SolveSmem s;
  {
    cd* p = reinterpret_cast<cd*>(smem_raw);
    s.c = p; p += NZ;
    s.r = p; p += NZ;
    s.fb = p; p += 2 * N;
    s.e = p; p += NZ;
    s.o = p; p += NZ;
    s.x = p; p += NZ;
    double* q = reinterpret_cast<double*>(p);
    s.dr = q; q += 4 * NZ;
    s.di = q; q += 4 * NZ;
  }
  const int g = blockIdx.x;
  const double dt = a.dt;
  const double* X = a.xinv + (size_t)g * a.sl.stride;
  if (g == a.nk2) {
    // (0,0) mode: au0 with clamb1, then w0 with clamb3 (REF:401-474)
    for (int comp = 0; comp < 2; ++comp) {
      const double* cln = comp == 0 ? a.cl1n : a.cl3n;
      const double* clm = comp == 0 ? a.cl1nm1 : a.cl3nm1;
      double* am = comp == 0 ? a.au0 : a.w0;
      for (int n = threadIdx.x; n <= N; n += blockDim.x) {
        s.c[n] = cd{am[2 * n], am[2 * n + 1]};
        s.r[n] = cd{-1.0 * dt / 2.0 * (3.0 * cln[2 * n] - clm[2 * n]),
                    -1.0 * dt / 2.0 * (3.0 * cln[2 * n + 1] - clm[2 * n + 1])};
      }
      __syncthreads();
      solve_eq(s, a, 0.0, X, false);
      cd* vel = comp == 0 ? a.u : a.w;
      cd* vort = comp == 0 ? a.oz : a.ox;
      const double sg = comp == 0 ? -1.0 : 1.0;
      for (int n = threadIdx.x; n <= N; n += blockDim.x) {
        cd x = s.x[n];
        am[2 * n] = x.re;
        am[2 * n + 1] = x.im;
        vel[(size_t)n * modes] = x;
      }
      if (threadIdx.x == 0 || threadIdx.x == 32) {
        const bool im = threadIdx.x == 32;
        dser(reinterpret_cast<const double*>(s.x) + (im ? 1 : 0), 2, im ? s.di : s.dr, 1, N);
      }
      __syncthreads();
      for (int n = threadIdx.x; n <= N; n += blockDim.x)
        vort[(size_t)n * modes] = cd{sg * s.dr[n], sg * s.di[n]};
      __syncthreads();
    }
    return;
  }
  const double k2 = a.k2vals[g];
  const double c3 = 3.0 * dt / 2.0, c1 = dt / 2.0;
  for (int gi = a.group_start[g]; gi < a.group_start[g + 1]; ++gi) {
    const int m = a.group_modes[gi];
    const int kx = m % d.KX, ky = m / d.KX;
    const double al = a.iapha[kx], be = a.ibeta[ky];
    // ---- v equation (REF:253-330)
    for (int n = threadIdx.x; n <= N; n += blockDim.x) {
      size_t idx = (size_t)n * modes + m;
      s.c[n] = a.v[idx];
      cd rv = a.rv[idx], un = a.u[idx];
      s.r[n] = cd{(c3 * rv.re - c1 * un.re) * 1.0, (c3 * rv.im - c1 * un.im) * 1.0};
    }
    __syncthreads();
    solve_eq(s, a, k2, X, true);
    for (int n = threadIdx.x; n <= N; n += blockDim.x) a.v[(size_t)n * modes + m] = s.x[n];
    // keep v^{n+1} for the recovery: Dv -> dr/di row 0 after the omega solve
    for (int n = threadIdx.x; n <= N; n += blockDim.x) s.r[n] = s.x[n];
    __syncthreads();
    if (threadIdx.x == 0 || threadIdx.x == 32) {
      const bool im = threadIdx.x == 32;
      // Dv into derivative slot 3 (not used by the second-order solve)
      dser(reinterpret_cast<const double*>(s.r) + (im ? 1 : 0), 2, (im ? s.di : s.dr) + 3 * NZ, 1, N);
    }
    __syncthreads();
    // park v^{n+1} and Dv in the even/odd rhs buffers' spare room is not
    // possible in general, so keep them in registers of the owning threads:
    // thread t owns coefficients n = t, t + blockDim.x, ...
    cd vkeep[3], dvkeep[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      int n = threadIdx.x + q * blockDim.x;
      if (n <= N) {
        vkeep[q] = s.r[n];
        dvkeep[q] = cd{s.dr[3 * NZ + n], s.di[3 * NZ + n]};
      }
    }
    __syncthreads();
    // ---- omega_y equation (REF:333-382)
    for (int n = threadIdx.x; n <= N; n += blockDim.x) {
      size_t idx = (size_t)n * modes + m;
      s.c[n] = a.oy[idx];
      cd rg = a.rg[idx], wn = a.w[idx];
      s.r[n] = cd{(c3 * rg.re - c1 * wn.re) * 1.0, (c3 * rg.im - c1 * wn.im) * 1.0};
    }
    __syncthreads();
    solve_eq(s, a, k2, X, false);
    // ---- getvelocityandvorticity (REF:2347-2407)
    // u = (i al Dv - i be oy) / k2, w = (i be Dv + i al oy) / k2
    const double ik2 = 1.0 / k2;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      int n = threadIdx.x + q * blockDim.x;
      if (n <= N) {
        cd oy = s.x[n];
        cd dv = dvkeep[q];
        a.oy[(size_t)n * modes + m] = oy;
        cd u{(-1.0 * al * dv.im) * ik2 + (be * oy.im) * ik2, (al * dv.re) * ik2 - (be * oy.re) * ik2};
        cd w{(-1.0 * dv.im * be) * ik2 - (1.0 * oy.im * al) * ik2, (be * dv.re) * ik2 + (al * oy.re) * ik2};
        s.c[n] = u;   // u coefficients
        s.e[n] = w;   // w coefficients (e has NZ room)
      }
    }
    __syncthreads();
    if (threadIdx.x < 64 && (threadIdx.x % 32) == 0) {
      // thread 0: Du (re, im); thread 32: Dw (re, im)
      const bool isw = threadIdx.x == 32;
      const double* src = reinterpret_cast<const double*>(isw ? s.e : s.c);
      double* dst_r = s.dr + (isw ? 1 : 0) * NZ;
      double* dst_i = s.di + (isw ? 1 : 0) * NZ;
      dser(src, 2, dst_r, 1, N);
      dser(src + 1, 2, dst_i, 1, N);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      int n = threadIdx.x + q * blockDim.x;
      if (n <= N) {
        size_t idx = (size_t)n * modes + m;
        cd v = vkeep[q];
        a.u[idx] = s.c[n];
        a.w[idx] = s.e[n];
        // omega_x = Dw - i be v ; omega_z = -Du + i al v
        a.ox[idx] = cd{s.dr[NZ + n] + be * v.im, s.di[NZ + n] - be * v.re};
        a.oz[idx] = cd{-s.dr[n] - al * v.im, -s.di[n] + al * v.re};
      }
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
                       double* out) {
  double e = 0.0, mx = 0.0;
  unsigned long long bad = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
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

int launch_solve_fp64(Handle* h) {
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
  a.nk2 = h->nk2;
  if (d.NZ > 3 * S_THREADS || !fft_fits(1, 2 * d.N, S_THREADS, 2)) {
    h->err = "k_solve: nnz too large for the launch shape";
    return CHF_E_INVALID;
  }
  size_t smem = sizeof(cd) * (5 * (size_t)d.NZ + 2 * (size_t)d.N) + sizeof(double) * 8 * (size_t)d.NZ;
  if (smem > 48 * 1024 &&
      !cuda_ok(h, cudaFuncSetAttribute(k_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "k_solve smem"))
    return CHF_E_CUDA;
  cudaEvent_t ev;
  prof_begin(h, K_SOLVE, &ev);
  k_solve<<<h->nk2 + 1, S_THREADS, smem, h->stream>>>(a);
  prof_end(h, K_SOLVE, ev);
  if (!cuda_ok(h, cudaGetLastError(), "k_solve")) return CHF_E_CUDA;
  return CHF_OK;
}

int launch_diagnostics(Handle* h, chf_diag* out) {
  const Dims& d = h->d;
  double* s = reinterpret_cast<double*>(h->scratch);
  if (!cuda_ok(h, cudaMemsetAsync(s, 0, 3 * sizeof(double), h->stream), "diag memset"))
    return CHF_E_CUDA;
  size_t n = d.field_elems() * 2;
  k_diag<<<4 * 152, 256, 0, h->stream>>>(
      reinterpret_cast<const double*>(h->f[F_U]), reinterpret_cast<const double*>(h->f[F_V]),
      reinterpret_cast<const double*>(h->f[F_W]), reinterpret_cast<const double*>(h->f[F_OX]),
      reinterpret_cast<const double*>(h->f[F_OY]), reinterpret_cast<const double*>(h->f[F_OZ]), n, s);
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
