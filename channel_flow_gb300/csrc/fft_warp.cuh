// fft_warp.cuh -- register-resident length-192 DFTs in FP32, one warp per
// line.
//
// 192 = 6 x 32.  Lane l holds six values; "natural" layout means value j of
// lane l is element 32 j + l.  With n = 32 j + l and k = k1 + 6 k2,
//   X[k1 + 6 k2] = sum_l W32^(l k2) W192^(l k1) sum_j W6^(j k1) x[32 j + l],
// so a 6-point DFT per lane, a twiddle W192^(l k1) and a 32-point DFT across
// lanes (radix-2 decimation in frequency over warp shuffles) give, as value
// k1 of lane l, element k1 + 6 bitrev5(l): the "permuted" layout.
// fft192_perm_to_natural_x2 runs the reverse factorisation (32-point
// decimation in time across lanes from bit-reversed input, twiddle, 6-point
// DFT per lane) and takes permuted input to natural output.  Physical-space
// values are consumed pointwise (products) or row by row, so they stay
// permuted and no reordering pass exists.
//
// tw[m] = exp(-2 pi i m / 192), m = 0..191; SIGN = -1 is the forward
// (FFTW_FORWARD) transform, +1 the backward one.
#pragma once
#include "f32x2.cuh"
#include "fft_dev.cuh"

namespace chf {

template <typename T, int SIGN>
__device__ __forceinline__ cplx<T> twid(const cplx<T>* tw, int m) {
  cplx<T> w = tw[m];
  if (SIGN > 0) w.im = -w.im;
  return w;
}

template <typename T>
__device__ __forceinline__ cplx<T> shfl_i(cplx<T> v, int src) {
  return cplx<T>{__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src)};
}

// ---------------------------------------------------------------------------
// Packed form: a lane's six values are held as three (element 2j, element
// 2j + 1) pairs of real parts and three of imaginary parts, so that each
// f32x2 instruction does one operation for two elements.  A cross-lane
// radix-2 stage is, per pair, four shuffles, y = p + S v (S = +1 on the lower
// lane of a butterfly, -1 on the upper one) and y W' (W' = the stage twiddle
// on the upper lane, 1 on the lower one): the lower lane's v + p and the
// upper lane's (p - v) W.  The per-lane constants come from a shared-memory table
// built once per CTA (fft192_table).
// ---------------------------------------------------------------------------
struct Line6 {
  f32x2 r[3], i[3];  // r[j] = (x[2j].re, x[2j+1].re), i[j] likewise
};

// per transform sign, lane-contiguous (conflict-free 8- and 16-byte loads):
// st[s][lane] = W', the twiddle of stage s (h = 16 >> s) on the upper lane
// of a butterfly and 1 on the lower one; tw6[j][lane] = W192^(lane k1) for
// k1 = 2j, 2j + 1 as {re, re', im, im'}.  The butterfly sign S comes from
// the lane bits.
struct Fft192Table {
  float2 st[5][32];
  float4 tw6[3][32];
};

template <int SIGN>
__device__ __forceinline__ void fft192_table(Fft192Table* t, const cplx<float>* __restrict__ tw) {
  for (int e = threadIdx.x; e < 8 * 32; e += blockDim.x) {
    const int s = e >> 5, lane = e & 31;
    if (s < 5) {
      const int h = 16 >> s;
      cplx<float> w = twid<float, SIGN>(tw, (lane & (h - 1)) * (96 / h));
      if ((lane & h) == 0) w = cplx<float>{1.f, 0.f};
      t->st[s][lane] = make_float2(w.re, w.im);
    } else {
      const int j = s - 5;
      const cplx<float> a = twid<float, SIGN>(tw, lane * 2 * j), b = twid<float, SIGN>(tw, lane * (2 * j + 1));
      t->tw6[j][lane] = make_float4(a.re, b.re, a.im, b.im);
    }
  }
}

// the packed constants of cross-lane stage s for this lane
struct StageK {
  f32x2 wr, wi, nwi, sg;
};
__device__ __forceinline__ StageK stage_k(const Fft192Table& t, int s, int lane) {
  const int h = 16 >> s;
  const float2 w = t.st[s][lane];
  const float sg = (lane & h) ? -1.f : 1.f;
  return StageK{pk(w.x, w.x), pk(w.y, w.y), pk(-w.y, -w.y), pk(sg, sg)};
}

// (r, i) <- (r, i) (wr, wi) for two elements; nwi = -wi
__device__ __forceinline__ void cmul_x2(f32x2& r, f32x2& i, f32x2 wr, f32x2 wi, f32x2 nwi) {
  const f32x2 nr = fma2(i, nwi, mul2(r, wr));
  i = fma2(r, wi, mul2(i, wr));
  r = nr;
}

__device__ __forceinline__ f32x2 shfl_x2(f32x2 v, int mask) {
  float a, b;
  upk(v, a, b);
  return pk(__shfl_xor_sync(0xffffffffu, a, mask), __shfl_xor_sync(0xffffffffu, b, mask));
}

// 6-point DFT of a lane's values, X[k] = sum_j x[j] exp(SIGN 2 pi i j k / 6):
// the pairs (x[2j], x[2j+1]) are (e_j, o_j), so one packed 3-point DFT over j
// does both halves.
// Z1: elements 2 and 3 are zero (zero-padded inverse transforms).
template <int SIGN, bool Z1 = false>
__device__ __forceinline__ void dft6_x2(Line6& a) {
  const float c = 0.86602540378443864676f;
  const f32x2 nh = pk(-0.5f, -0.5f);
  f32x2 sr, si, er, ei;
  if (Z1) {  // s = x2, d = -x2
    sr = a.r[2];
    si = a.i[2];
    er = mul2(pk(SIGN * c, SIGN * c), a.i[2]);
    ei = mul2(pk(-SIGN * c, -SIGN * c), a.r[2]);
  } else {
    sr = add2(a.r[1], a.r[2]);
    si = add2(a.i[1], a.i[2]);
    er = mul2(pk(-SIGN * c, -SIGN * c), sub2(a.i[1], a.i[2]));
    ei = mul2(pk(SIGN * c, SIGN * c), sub2(a.r[1], a.r[2]));
  }
  const f32x2 mr = fma2(nh, sr, a.r[0]), mi = fma2(nh, si, a.i[0]);
  float E0r, O0r, E0i, O0i, E1r, O1r, E1i, O1i, E2r, O2r, E2i, O2i;
  upk(add2(a.r[0], sr), E0r, O0r);
  upk(add2(a.i[0], si), E0i, O0i);
  upk(add2(mr, er), E1r, O1r);
  upk(add2(mi, ei), E1i, O1i);
  upk(sub2(mr, er), E2r, O2r);
  upk(sub2(mi, ei), E2i, O2i);
  // t_k = O_k omega6^k, omega6^k = exp(SIGN i pi k / 3)
  const float t1r = 0.5f * O1r - SIGN * c * O1i, t1i = 0.5f * O1i + SIGN * c * O1r;
  const float t2r = -0.5f * O2r - SIGN * c * O2i, t2i = -0.5f * O2i + SIGN * c * O2r;
  a.r[0] = pk(E0r + O0r, E1r + t1r);
  a.i[0] = pk(E0i + O0i, E1i + t1i);
  a.r[1] = pk(E2r + t2r, E0r - O0r);
  a.i[1] = pk(E2i + t2i, E0i - O0i);
  a.r[2] = pk(E1r - t1r, E2r - t2r);
  a.i[2] = pk(E1i - t1i, E2i - t2i);
}

// natural -> permuted, table of the same SIGN;
// Z1 as for dft6_x2
template <int SIGN, bool Z1 = false>
__device__ __forceinline__ void fft192_natural_to_perm_x2(Line6& a, const Fft192Table& t) {
  const int lane = threadIdx.x & 31;
  dft6_x2<SIGN, Z1>(a);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float4 p = t.tw6[j][lane];
    cmul_x2(a.r[j], a.i[j], pk(p.x, p.y), pk(p.z, p.w), pk(-p.z, -p.w));
  }
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = 16 >> s;
    const StageK k = stage_k(t, s, lane);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      a.r[j] = fma2(k.sg, a.r[j], shfl_x2(a.r[j], h));
      a.i[j] = fma2(k.sg, a.i[j], shfl_x2(a.i[j], h));
      if (h > 1) cmul_x2(a.r[j], a.i[j], k.wr, k.wi, k.nwi);  // W_2 = 1
    }
  }
}

// permuted -> natural, table of the same SIGN
template <int SIGN>
__device__ __forceinline__ void fft192_perm_to_natural_x2(Line6& a, const Fft192Table& t) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 4; s >= 0; --s) {
    const int h = 16 >> s;
    const StageK k = stage_k(t, s, lane);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (h > 1) cmul_x2(a.r[j], a.i[j], k.wr, k.wi, k.nwi);
      a.r[j] = fma2(k.sg, a.r[j], shfl_x2(a.r[j], h));
      a.i[j] = fma2(k.sg, a.i[j], shfl_x2(a.i[j], h));
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float4 p = t.tw6[j][lane];
    cmul_x2(a.r[j], a.i[j], pk(p.x, p.y), pk(p.z, p.w), pk(-p.z, -p.w));
  }
  dft6_x2<SIGN>(a);
}

// element k of a lane's six values
__device__ __forceinline__ cplx<float> line_get(const Line6& a, int k) {
  float r0, r1, i0, i1;
  upk(a.r[k >> 1], r0, r1);
  upk(a.i[k >> 1], i0, i1);
  return (k & 1) ? cplx<float>{r1, i1} : cplx<float>{r0, i0};
}

}  // namespace chf
