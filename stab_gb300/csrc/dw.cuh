// Double-word ("float-float") arithmetic for the seed spectra.
//
// A real value is an unevaluated sum h + l of two floats with |l| <= ulp(h)/2
// (Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971): about 48 significant bits, against 53
// for FP64.  GB300 issues FP32 at 59 times its FP64 rate, and one double-word
// multiply-add takes 15 FP32 instructions, so a complex update that is four
// FP64 FMAs costs about a quarter as long in double-word form.
//
// The building blocks are the error-free transformations of Knuth (TwoSum,
// TAOCP vol. 2, 4.2.2) and Dekker (FastTwoSum), and the exact product error
// fma(a, b, -a*b).  Additions follow "SloppyDWPlusDW" and products
// "DWTimesDW" of Joldes, Muller and Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", ACM TOMS 44 (2017):
// the error of a sum is at most a few u^2 (|x| + |y|) with u = 2^-24, which
// is the error model (no relative bound under cancellation) that Householder
// and QR backward-error analysis needs.
//
// Every FP32 operation of a transformation is written with an explicit
// rounding intrinsic, so the compiler cannot contract a product and a sum
// into an FMA and break the exactness the transformations rely on.
//
// Complex values are float4 {re.h, re.l, im.h, im.l} (16 bytes, the size of a
// complex128, so the same pools and shared buffers hold either).
#pragma once
#include "common.cuh"

typedef float2 dw;   // {h, l}
typedef float4 dz;   // {re.h, re.l, im.h, im.l}

__device__ __forceinline__ dw dw_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
// exact when |a| >= |b| (or a == 0)
__device__ __forceinline__ dw dw_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dw dw_neg(dw x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ dw dw_add(dw x, dw y) {
  const dw s = dw_two_sum(x.x, y.x);
  return dw_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(x.y, y.y)));
}
__device__ __forceinline__ dw dw_mul(dw x, dw y) {
  const float p = __fmul_rn(x.x, y.x);
  float e = fmaf(x.x, y.x, -p);
  e = fmaf(x.x, y.y, e);
  e = fmaf(x.y, y.x, e);
  return dw_fast_two_sum(p, e);
}
// x*y + c
__device__ __forceinline__ dw dw_fma(dw x, dw y, dw c) {
  const float p = __fmul_rn(x.x, y.x);
  float e = fmaf(x.x, y.x, -p);
  e = fmaf(x.x, y.y, e);
  e = fmaf(x.y, y.x, e);
  const dw s = dw_two_sum(p, c.x);
  return dw_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(e, c.y)));
}
__device__ __forceinline__ double dw_to64(dw x) { return (double)x.x + (double)x.y; }
__device__ __forceinline__ dw dw_from64(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

// ---- complex ---------------------------------------------------------------
__device__ __forceinline__ dw dz_re(dz a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ dw dz_im(dz a) { return make_float2(a.z, a.w); }
__device__ __forceinline__ dz dz_mk(dw re, dw im) { return make_float4(re.x, re.y, im.x, im.y); }

__device__ __forceinline__ dz zadd(dz a, dz b) { return dz_mk(dw_add(dz_re(a), dz_re(b)), dw_add(dz_im(a), dz_im(b))); }
__device__ __forceinline__ dz zsub(dz a, dz b) {
  return dz_mk(dw_add(dz_re(a), dw_neg(dz_re(b))), dw_add(dz_im(a), dw_neg(dz_im(b))));
}
__device__ __forceinline__ dz zconj(dz a) { return make_float4(a.x, a.y, -a.z, -a.w); }
// scaling by a power of two is exact
__device__ __forceinline__ dz zscale(dz a, float s) {
  return make_float4(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}
__device__ __forceinline__ float zabs1(dz a) { return fabsf(a.x) + fabsf(a.z); }
__device__ __forceinline__ dz zmul(dz a, dz b) {
  const dw ar = dz_re(a), ai = dz_im(a), br = dz_re(b), bi = dz_im(b);
  return dz_mk(dw_fma(ar, br, dw_mul(dw_neg(ai), bi)), dw_fma(ar, bi, dw_mul(ai, br)));
}
// a*b + c
__device__ __forceinline__ dz zfma(dz a, dz b, dz c) {
  const dw ar = dz_re(a), ai = dz_im(a), br = dz_re(b), bi = dz_im(b);
  return dz_mk(dw_fma(ar, br, dw_fma(dw_neg(ai), bi, dz_re(c))), dw_fma(ar, bi, dw_fma(ai, br, dz_im(c))));
}
// conj(a)*b + c
__device__ __forceinline__ dz zcfma(dz a, dz b, dz c) {
  const dw ar = dz_re(a), ai = dz_im(a), br = dz_re(b), bi = dz_im(b);
  return dz_mk(dw_fma(ar, br, dw_fma(ai, bi, dz_re(c))), dw_fma(ar, bi, dw_fma(dw_neg(ai), br, dz_im(c))));
}
// c - a*b
__device__ __forceinline__ dz zfnma(dz a, dz b, dz c) {
  const dw ar = dz_re(a), ai = dz_im(a), br = dz_re(b), bi = dz_im(b);
  return dz_mk(dw_fma(dw_neg(ar), br, dw_fma(ai, bi, dz_re(c))),
               dw_fma(dw_neg(ar), bi, dw_fma(dw_neg(ai), br, dz_im(c))));
}
// c - a*conj(b)
__device__ __forceinline__ dz zfnmac(dz a, dz b, dz c) {
  const dw ar = dz_re(a), ai = dz_im(a), br = dz_re(b), bi = dz_im(b);
  return dz_mk(dw_fma(dw_neg(ar), br, dw_fma(dw_neg(ai), bi, dz_re(c))),
               dw_fma(ar, bi, dw_fma(dw_neg(ai), br, dz_im(c))));
}
__device__ __forceinline__ zc dz_to64(dz a) { return zmk(dw_to64(dz_re(a)), dw_to64(dz_im(a))); }
__device__ __forceinline__ dz dz_from64(zc a) { return dz_mk(dw_from64(a.x), dw_from64(a.y)); }

// Exponent e of x (x ~ 2^e) for scaling by the exact power of two 2^-e,
// clamped so that 2^-e and 2^e stay finite floats: below 2^-126 (bulge
// entries of a nearly deflated stretch of a low-Mach operator reach that) the
// scaled value stays small instead of the factor overflowing to infinity.
// 0 for x == 0.
__device__ __forceinline__ int dw_scale_exponent(float x) {
  if (!(x > 0.f)) return 0;
  return min(max(ilogbf(x), -126), 126);
}

// ---- reciprocal and reciprocal square root ----------------------------------
// Newton steps in double-word arithmetic from a float seed: each step doubles
// the number of correct bits (reciprocal: y + y (1 - d y); reciprocal square
// root: r + r (1 - s r^2) / 2).  The reciprocal starts from the correctly
// rounded float reciprocal, so one step reaches the double-word precision;
// the reciprocal square root takes two (its float seed is a few ulps off).
__device__ __forceinline__ dw dw_rcp(dw d) {
  const dw y = make_float2(__frcp_rn(d.x), 0.f);
  const dw e = dw_fma(dw_neg(d), y, make_float2(1.f, 0.f));   // 1 - d y
  return dw_fma(y, e, y);
}
__device__ __forceinline__ dw dw_rsqrt(dw s) {
  float r0 = rsqrtf(s.x);
  r0 = __fmul_rn(r0, __fsub_rn(1.5f, __fmul_rn(__fmul_rn(0.5f, s.x), __fmul_rn(r0, r0))));   // float Newton step
  dw r = make_float2(r0, 0.f);
  for (int it = 0; it < 2; ++it) {
    const dw e = dw_fma(dw_neg(s), dw_mul(r, r), make_float2(1.f, 0.f));   // 1 - s r^2
    r = dw_fma(make_float2(0.5f * r.x, 0.f), e, r);
  }
  return r;
}

// ---- the LU / triangular-solve traits (cx<T> of common.cuh) -----------------
template <> struct cx<dz> {
  typedef float real;
  __device__ static dz make(float r, float i) { return make_float4(r, 0.f, i, 0.f); }
  __device__ static dz mul(dz a, dz b) { return zmul(a, b); }
  __device__ static dz fma_(dz a, dz b, dz c) { return zfma(a, b, c); }
  __device__ static dz sub(dz a, dz b) { return zsub(a, b); }
  __device__ static dz fnma(dz a, dz b, dz c) { return zfnma(a, b, c); }   // c - a*b
  // a conj(b) / |b|^2, with b first scaled by the power of two that brings
  // it near 1 (the squares stay inside the float exponent range)
  __device__ static dz div(dz a, dz b) {
    const float p = ldexpf(1.f, -dw_scale_exponent(zabs1(b)));
    const dz bs = zscale(b, p);
    const dw r = dw_rcp(dw_fma(dz_re(bs), dz_re(bs), dw_mul(dz_im(bs), dz_im(bs))));
    const dz q = zmul(a, zconj(bs));
    return zscale(dz_mk(dw_mul(dz_re(q), r), dw_mul(dz_im(q), r)), p);
  }
  __device__ static float abs1(dz a) { return zabs1(a); }
  __device__ static dz from(zc a) { return dz_from64(a); }
  __device__ static zc to64(dz a) { return dz_to64(a); }
};
