// fft_warp.cuh -- register-resident length-192 DFTs, one warp per line.
//
// 192 = 6 x 32.  Lane l holds six values; "natural" layout means register j
// of lane l is element 32 j + l.  With n = 32 j + l and k = k1 + 6 k2,
//   X[k1 + 6 k2] = sum_l W32^(l k2) W192^(l k1) sum_j W6^(j k1) x[32 j + l],
// so a 6-point DFT per lane, a twiddle W192^(l k1) and a 32-point DFT across
// lanes (radix-2 decimation in frequency over warp shuffles) give, in
// register k1 of lane l, element k1 + 6 bitrev5(l): the "permuted" layout.
// fft192_perm_to_natural runs the reverse factorisation (32-point decimation
// in time across lanes from bit-reversed input, twiddle, 6-point DFT per
// lane) and takes permuted input to natural output.  Physical-space values
// are consumed pointwise (products) or row by row, so they stay permuted and
// no reordering pass exists.
//
// tw[m] = exp(-2 pi i m / 192), m = 0..191 (shared memory); SIGN = -1 is the
// forward (FFTW_FORWARD) transform, +1 the backward one.
#pragma once
#include "fft_dev.cuh"

namespace chf {

template <typename T, int SIGN>
__device__ __forceinline__ cplx<T> twid(const cplx<T>* tw, int m) {
  cplx<T> w = tw[m];
  if (SIGN > 0) w.im = -w.im;
  return w;
}

// 6-point DFT in registers: X[k] = sum_j a[j] exp(SIGN 2 pi i j k / 6)
template <typename T, int SIGN>
__device__ __forceinline__ void dft6(cplx<T>* a) {
  cplx<T> e[3] = {a[0], a[2], a[4]};
  cplx<T> o[3] = {a[1], a[3], a[5]};
  bfly3<T, SIGN>(e);
  bfly3<T, SIGN>(o);
  // omega6^k = exp(SIGN i pi k / 3), k = 0, 1, 2
  const T c = (T)0.5, s = (T)0.86602540378443864676;
  cplx<T> w1{c, (T)SIGN * s};
  cplx<T> w2{-c, (T)SIGN * s};
  cplx<T> t0 = o[0], t1 = cmul(o[1], w1), t2 = cmul(o[2], w2);
  a[0] = cadd(e[0], t0);
  a[3] = csub(e[0], t0);
  a[1] = cadd(e[1], t1);
  a[4] = csub(e[1], t1);
  a[2] = cadd(e[2], t2);
  a[5] = csub(e[2], t2);
}

template <typename T>
__device__ __forceinline__ cplx<T> shfl_x(cplx<T> v, int mask) {
  return cplx<T>{__shfl_xor_sync(0xffffffffu, v.re, mask), __shfl_xor_sync(0xffffffffu, v.im, mask)};
}

template <typename T>
__device__ __forceinline__ cplx<T> shfl_i(cplx<T> v, int src) {
  return cplx<T>{__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src)};
}

// natural -> permuted
template <typename T, int SIGN>
__device__ __forceinline__ void fft192_natural_to_perm(cplx<T>* v, const cplx<T>* tw) {
  const int lane = threadIdx.x & 31;
  dft6<T, SIGN>(v);
#pragma unroll
  for (int k1 = 1; k1 < 6; ++k1) v[k1] = cmul(v[k1], twid<T, SIGN>(tw, lane * k1));
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool upper = (lane & h) != 0;
    const cplx<T> w = twid<T, SIGN>(tw, (lane & (h - 1)) * (96 / h));  // W_{2h}^t = W192^(t * 96/h)
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
      cplx<T> p = shfl_x(v[k1], h);
      v[k1] = upper ? cmul(csub(p, v[k1]), w) : cadd(v[k1], p);
    }
  }
}

// permuted -> natural
template <typename T, int SIGN>
__device__ __forceinline__ void fft192_perm_to_natural(cplx<T>* v, const cplx<T>* tw) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 1; h <= 16; h <<= 1) {
    const bool upper = (lane & h) != 0;
    const cplx<T> w = twid<T, SIGN>(tw, (lane & (h - 1)) * (96 / h));
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
      cplx<T> x = upper ? cmul(v[k1], w) : v[k1];
      cplx<T> p = shfl_x(x, h);
      v[k1] = upper ? csub(p, x) : cadd(x, p);
    }
  }
#pragma unroll
  for (int k1 = 1; k1 < 6; ++k1) v[k1] = cmul(v[k1], twid<T, SIGN>(tw, lane * k1));
  // 6-point DFT over k1 -> register j' holds element 32 j' + lane
  dft6<T, SIGN>(v);
}

}  // namespace chf
