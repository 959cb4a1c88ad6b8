// fft_dev.cuh -- batched complex DFTs in shared memory for sm_103a.
//
// Stockham auto-sort formulation (each stage reads stride L/R, writes
// blocks of Ns), radices 4, 2, 3 and 5.  The whole CTA cooperates on
// `nlines` lines that live in shared memory; each stage reads every
// butterfly's inputs into registers, synchronises, then writes, so one
// buffer suffices.  Twiddles come from a host-computed table
// tw[k] = exp(-2 pi i k / L) (accurate libm values, identical on every run).
//
// Sign convention: SIGN = -1 is FFTW_FORWARD, +1 is FFTW_BACKWARD
// (unnormalised), matching the reference's fftw_f77_one calls.
#pragma once
#include <cuda_runtime.h>

namespace chf {

template <typename T>
struct cplx {
  T re, im;
};

struct FftPlan {
  int L;
  int nst;
  int R[16];
  int Ns[16];
  // per stage, division by L / R[st] and by Ns[st] as a multiply-high and a
  // shift (fft_plan_divisors): q = (umulhi(n, m) + n) >> s for 0 <= n < 2^31
  unsigned int nr_m[16], ns_m[16];
  int nr_s[16], ns_s[16];
  // two-buffer stages (smem_fft_pp): offset of stage st's twiddles in the
  // plan's stage table, which holds w^(r jm L / (Ns R)) at (r - 1) Ns + jm
  // for r = 1 .. R - 1, jm = 0 .. Ns - 1 (L - 1 entries in all), so that the
  // threads of a stage read consecutive entries
  int twoff[16];
};

// m, s of the division by d (d >= 1) used in FftPlan: l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1 (the round-up method of Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994)
inline void fft_divisor(unsigned int d, unsigned int* m, int* s) {
  int l = 0;
  while ((1ull << l) < d) ++l;
  *m = (unsigned int)((((1ull << 32) * ((1ull << l) - d)) / d + 1) & 0xffffffffull);
  *s = l;
}

// fill the divisors of every stage of p (after R, Ns, nst, L are set)
inline void fft_plan_divisors(FftPlan& p) {
  int off = 0;
  for (int st = 0; st < p.nst; ++st) {
    fft_divisor((unsigned int)(p.L / p.R[st]), &p.nr_m[st], &p.nr_s[st]);
    fft_divisor((unsigned int)p.Ns[st], &p.ns_m[st], &p.ns_s[st]);
    p.twoff[st] = off;
    off += (p.R[st] - 1) * p.Ns[st];
  }
}

__device__ __forceinline__ int fft_div(int n, unsigned int m, int s) {
  return (int)((__umulhi((unsigned int)n, m) + (unsigned int)n) >> s);
}

template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  cplx<T> r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

template <typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) {
  return cplx<T>{a.re + b.re, a.im + b.im};
}

template <typename T>
__device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) {
  return cplx<T>{a.re - b.re, a.im - b.im};
}

// v[k] <- sum_r v[r] exp(SIGN 2 pi i r k / R)
template <typename T, int SIGN>
__device__ __forceinline__ void bfly2(cplx<T>* v) {
  cplx<T> a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <typename T, int SIGN>
__device__ __forceinline__ void bfly4(cplx<T>* v) {
  cplx<T> t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  cplx<T> t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
  cplx<T> st3;  // (SIGN i) * t3
  st3.re = (T)(-SIGN) * t3.im;
  st3.im = (T)(SIGN)*t3.re;
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, st3);
  v[3] = csub(t1, st3);
}

template <typename T, int SIGN>
__device__ __forceinline__ void bfly3(cplx<T>* v) {
  const T c = (T)0.86602540378443864676;  // sqrt(3)/2
  cplx<T> s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  cplx<T> a = v[0];
  cplx<T> m{a.re - (T)0.5 * s.re, a.im - (T)0.5 * s.im};
  cplx<T> e{(T)(-SIGN) * c * d.im, (T)(SIGN)*c * d.re};
  v[0] = cadd(a, s);
  v[1] = cadd(m, e);
  v[2] = csub(m, e);
}

template <typename T, int SIGN>
__device__ __forceinline__ void bfly5(cplx<T>* v) {
  // Direct 5-point DFT with the exact roots cos/sin(2 pi k / 5).
  const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
  const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
  cplx<T> a = v[0];
  cplx<T> p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]);
  cplx<T> p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
  cplx<T> r1{a.re + c1 * p1.re + c2 * p2.re, a.im + c1 * p1.im + c2 * p2.im};
  cplx<T> r2{a.re + c2 * p1.re + c1 * p2.re, a.im + c2 * p1.im + c1 * p2.im};
  // SIGN i (s1 m1 + s2 m2) and SIGN i (s2 m1 - s1 m2)
  cplx<T> i1{(T)(-SIGN) * (s1 * m1.im + s2 * m2.im), (T)(SIGN) * (s1 * m1.re + s2 * m2.re)};
  cplx<T> i2{(T)(-SIGN) * (s2 * m1.im - s1 * m2.im), (T)(SIGN) * (s2 * m1.re - s1 * m2.re)};
  v[0] = cplx<T>{a.re + p1.re + p2.re, a.im + p1.im + p2.im};
  v[1] = cadd(r1, i1);
  v[4] = csub(r1, i1);
  v[2] = cadd(r2, i2);
  v[3] = csub(r2, i2);
}

// Larger radices for the two-buffer stages (smem_fft_pp): fewer passes
// through shared memory.  Each is a two-level factorisation in registers,
// X[k1 + R1 k2] = sum_p W_R^(p k1) W_R2^(p k2) sum_m x[R2 m + p] W_R1^(m k1)
// (n = R2 m + p, R = R1 R2), with the exact roots cos / sin(2 pi q / R).
template <typename T, int SIGN>
__device__ __forceinline__ cplx<T> rot(cplx<T> a, T c, T s) {  // a * (c + SIGN i s)
  return cplx<T>{a.re * c - (T)SIGN * a.im * s, a.im * c + (T)SIGN * a.re * s};
}

// radix 8 = 4 x 2
template <typename T, int SIGN>
__device__ __forceinline__ void bfly8(cplx<T>* v) {
  const T h = (T)0.70710678118654752440;  // cos(pi / 4) = sin(pi / 4)
  cplx<T> e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  bfly4<T, SIGN>(e);
  bfly4<T, SIGN>(o);
  o[1] = rot<T, SIGN>(o[1], h, h);
  o[2] = cplx<T>{(T)(-SIGN) * o[2].im, (T)(SIGN)*o[2].re};  // * SIGN i
  o[3] = rot<T, SIGN>(o[3], -h, h);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// radix 9 = 3 x 3
template <typename T, int SIGN>
__device__ __forceinline__ void bfly9(cplx<T>* v) {
  const T c1 = (T)0.76604444311897803520, s1 = (T)0.64278760968653932632;  // 2 pi / 9
  const T c2 = (T)0.17364817766693034885, s2 = (T)0.98480775301220805936;  // 4 pi / 9
  const T c4 = (T)-0.93969262078590838405, s4 = (T)0.34202014332566873304;  // 8 pi / 9
  cplx<T> a[3][3];
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    a[p][0] = v[p];
    a[p][1] = v[3 + p];
    a[p][2] = v[6 + p];
    bfly3<T, SIGN>(a[p]);
  }
  a[1][1] = rot<T, SIGN>(a[1][1], c1, s1);
  a[1][2] = rot<T, SIGN>(a[1][2], c2, s2);
  a[2][1] = rot<T, SIGN>(a[2][1], c2, s2);
  a[2][2] = rot<T, SIGN>(a[2][2], c4, s4);
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    cplx<T> b[3] = {a[0][k1], a[1][k1], a[2][k1]};
    bfly3<T, SIGN>(b);
    v[k1] = b[0];
    v[k1 + 3] = b[1];
    v[k1 + 6] = b[2];
  }
}

// radix 16 = 4 x 4
template <typename T, int SIGN>
__device__ __forceinline__ void bfly16(cplx<T>* v) {
  const T ca = (T)0.92387953251128675613, sa = (T)0.38268343236508977173;  // pi / 8
  const T h = (T)0.70710678118654752440;                                    // pi / 4
  cplx<T> a[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
#pragma unroll
    for (int m = 0; m < 4; ++m) a[p][m] = v[4 * m + p];
    bfly4<T, SIGN>(a[p]);
  }
  // W16^(p k1): p = 1: k1 = 1, 2, 3 -> pi/8, pi/4, 3pi/8; p = 2: pi/4, pi/2, 3pi/4;
  // p = 3: 3pi/8, 3pi/4, 9pi/8
  a[1][1] = rot<T, SIGN>(a[1][1], ca, sa);
  a[1][2] = rot<T, SIGN>(a[1][2], h, h);
  a[1][3] = rot<T, SIGN>(a[1][3], sa, ca);
  a[2][1] = rot<T, SIGN>(a[2][1], h, h);
  a[2][2] = cplx<T>{(T)(-SIGN) * a[2][2].im, (T)(SIGN)*a[2][2].re};
  a[2][3] = rot<T, SIGN>(a[2][3], -h, h);
  a[3][1] = rot<T, SIGN>(a[3][1], sa, ca);
  a[3][2] = rot<T, SIGN>(a[3][2], -h, h);
  a[3][3] = rot<T, SIGN>(a[3][3], -ca, -sa);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cplx<T> b[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
    bfly4<T, SIGN>(b);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
  }
}

// One stage helper: load R inputs of butterfly (line, j), twiddle, butterfly.
// The first stage (Ns = 1, jm = 0) has every twiddle equal to 1 (tw[0] is
// exactly (1, 0)) and skips them.
template <typename T, int SIGN, int R>
__device__ __forceinline__ void stage_load(const cplx<T>* __restrict__ base, int j, int nr, int jm,
                                           int twstep, const cplx<T>* __restrict__ tw,
                                           cplx<T>* v, bool twiddled) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    cplx<T> x = base[j + r * nr];
    if (r > 0 && twiddled) {
      cplx<T> w = tw[r * jm * twstep];
      if (SIGN > 0) w.im = -w.im;
      x = cmul(x, w);
    }
    v[r] = x;
  }
  if (R == 2) bfly2<T, SIGN>(v);
  if (R == 3) bfly3<T, SIGN>(v);
  if (R == 4) bfly4<T, SIGN>(v);
  if (R == 5) bfly5<T, SIGN>(v);
  if (R == 8) bfly8<T, SIGN>(v);
  if (R == 9) bfly9<T, SIGN>(v);
  if (R == 16) bfly16<T, SIGN>(v);
}

// One Stockham stage with compile-time radix R; each thread owns up to MB
// butterflies (b = tid + k * blockDim.x).  Reads all inputs, synchronises,
// writes all outputs, synchronises.
template <typename T, int SIGN, int R, int MB>
__device__ __forceinline__ void fft_stage(cplx<T>* s, int nlines, int lstride, const FftPlan& p, int st,
                                          const cplx<T>* __restrict__ tw) {
  const int nt = blockDim.x, tid = threadIdx.x;
  const int L = p.L, Ns = p.Ns[st];
  const int nr = L / R;
  const int total = nlines * nr;
  const int twstep = L / (Ns * R);
  const unsigned int nrm = p.nr_m[st], nsm = p.ns_m[st];
  const int nrs = p.nr_s[st], nss = p.ns_s[st];
  cplx<T> v[MB][R];
  int off[MB];  // output position of butterfly b: line start + block start + jm
#pragma unroll
  for (int b = 0; b < MB; ++b) {
    int t = tid + b * nt;
    off[b] = 0;
    if (t < total) {
      const int line = fft_div(t, nrm, nrs), j = t - line * nr;
      const int q = fft_div(j, nsm, nss), jm = j - q * Ns;
      stage_load<T, SIGN, R>(s + line * lstride, j, nr, jm, twstep, tw, v[b], Ns > 1);
      off[b] = line * lstride + q * Ns * R + jm;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < MB; ++b) {
    int t = tid + b * nt;
    if (t < total) {
      cplx<T>* base = s + off[b];
#pragma unroll
      for (int r = 0; r < R; ++r) base[r * Ns] = v[b][r];
    }
  }
  __syncthreads();
}

// Batched in-place DFT of `nlines` lines of length p.L in shared memory,
// line l at s + l * lstride.  All threads of the CTA must call it.
// MB2 bounds the radix-2 butterflies per thread:
//   MB2 >= ceil(nlines * L / 2 / blockDim.x)   (checked by the launchers).
template <typename T, int SIGN, int MB2>
__device__ void smem_fft(cplx<T>* s, int nlines, int lstride, const FftPlan& p,
                         const cplx<T>* __restrict__ tw) {
  constexpr int MB4 = (MB2 + 1) / 2;
  constexpr int MB3 = (2 * MB2 + 2) / 3;
  constexpr int MB5 = (2 * MB2 + 4) / 5;
  for (int st = 0; st < p.nst; ++st) {
    const int R = p.R[st];
    if (R == 4) fft_stage<T, SIGN, 4, MB4>(s, nlines, lstride, p, st, tw);
    else if (R == 2) fft_stage<T, SIGN, 2, MB2>(s, nlines, lstride, p, st, tw);
    else if (R == 3) fft_stage<T, SIGN, 3, MB3>(s, nlines, lstride, p, st, tw);
    else fft_stage<T, SIGN, 5, MB5>(s, nlines, lstride, p, st, tw);
  }
}

// Out-of-place Stockham stages between two shared-memory buffers: each
// butterfly is read from one buffer, computed and written to the other at
// once, with one barrier per stage, so a thread holds a single butterfly's R
// values (few registers, no per-thread butterfly bound).  Line l of either
// buffer at l * lstride.  Call after a barrier that makes the input in `a`
// visible; returns the buffer holding the result (a or b), visible to every
// thread of the CTA.
template <typename T, int SIGN, int R>
__device__ __forceinline__ void fft_stage_pp(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                             int nlines, int lstride, const FftPlan& p, int st,
                                             const cplx<T>* __restrict__ stab) {
  const int L = p.L, Ns = p.Ns[st];
  const int nr = L / R;
  const int total = nlines * nr;
  const unsigned int nrm = p.nr_m[st], nsm = p.ns_m[st];
  const int nrs = p.nr_s[st], nss = p.ns_s[st];
  const cplx<T>* __restrict__ tws = stab + p.twoff[st];  // this stage's (r - 1) Ns + jm table
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int line = fft_div(t, nrm, nrs), j = t - line * nr;
    const int q = fft_div(j, nsm, nss), jm = j - q * Ns;
    cplx<T> v[R];
    const cplx<T>* in = src + line * lstride;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      cplx<T> x = in[j + r * nr];
      if (r > 0 && Ns > 1) {  // the first stage's twiddles are all 1
        cplx<T> w = tws[(r - 1) * Ns + jm];
        if (SIGN > 0) w.im = -w.im;
        x = cmul(x, w);
      }
      v[r] = x;
    }
    if (R == 2) bfly2<T, SIGN>(v);
    if (R == 3) bfly3<T, SIGN>(v);
    if (R == 4) bfly4<T, SIGN>(v);
    if (R == 5) bfly5<T, SIGN>(v);
    if (R == 8) bfly8<T, SIGN>(v);
    if (R == 9) bfly9<T, SIGN>(v);
    if (R == 16) bfly16<T, SIGN>(v);
    cplx<T>* base = dst + line * lstride + q * Ns * R + jm;
#pragma unroll
    for (int r = 0; r < R; ++r) base[r * Ns] = v[r];
  }
}

// stab: the plan's stage twiddle table (FftPlan::twoff, fft_stage_twiddles).
template <typename T, int SIGN>
__device__ cplx<T>* smem_fft_pp(cplx<T>* a, cplx<T>* b, int nlines, int lstride, const FftPlan& p,
                                const cplx<T>* __restrict__ stab) {
  for (int st = 0; st < p.nst; ++st) {
    const int R = p.R[st];
    if (R == 4) fft_stage_pp<T, SIGN, 4>(a, b, nlines, lstride, p, st, stab);
    else if (R == 8) fft_stage_pp<T, SIGN, 8>(a, b, nlines, lstride, p, st, stab);
    else if (R == 16) {  // FP32 lines only (16 FP64 values would not fit the registers)
      if constexpr (sizeof(T) == 4) fft_stage_pp<T, SIGN, 16>(a, b, nlines, lstride, p, st, stab);
    }
    else if (R == 9) fft_stage_pp<T, SIGN, 9>(a, b, nlines, lstride, p, st, stab);
    else if (R == 2) fft_stage_pp<T, SIGN, 2>(a, b, nlines, lstride, p, st, stab);
    else if (R == 3) fft_stage_pp<T, SIGN, 3>(a, b, nlines, lstride, p, st, stab);
    else fft_stage_pp<T, SIGN, 5>(a, b, nlines, lstride, p, st, stab);
    __syncthreads();
    cplx<T>* t = a;
    a = b;
    b = t;
  }
  return a;
}

// Host side: the stage twiddle table of plan p (L - 1 entries, FftPlan::twoff)
// from the length-L table tw[k] = exp(-2 pi i k / L), converted to T.
template <typename T, typename V>
inline void fft_stage_twiddles(const FftPlan& p, const V& tw, cplx<T>* out) {
  for (int st = 0; st < p.nst; ++st) {
    const int R = p.R[st], Ns = p.Ns[st], step = p.L / (Ns * R);
    for (int r = 1; r < R; ++r)
      for (int jm = 0; jm < Ns; ++jm) {
        const auto& w = tw[(size_t)r * jm * step];
        out[p.twoff[st] + (r - 1) * Ns + jm] = cplx<T>{(T)w.re, (T)w.im};
      }
  }
}

// Host-side check of the MB2 bound for a launch.
inline bool fft_fits(int nlines, int L, int nthreads, int mb2) {
  return (long)nlines * (L / 2) <= (long)mb2 * nthreads;
}

}  // namespace chf
