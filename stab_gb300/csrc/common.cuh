// Shared device definitions for the stab GB300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>

#include "../../include/stab_gb300.h"

#define STAB_NDOF 5

// ---------------------------------------------------------------------------
// complex arithmetic on double2 / float2 ({re, im}); column-major matrices
// ---------------------------------------------------------------------------
typedef double2 zc;   // complex128
typedef float2 cc;    // complex64

__host__ __device__ __forceinline__ zc zmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ zc zadd(zc a, zc b) { return zmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ zc zsub(zc a, zc b) { return zmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ zc zmul(zc a, zc b) { return zmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__host__ __device__ __forceinline__ zc zconj(zc a) { return zmk(a.x, -a.y); }
__host__ __device__ __forceinline__ zc zscale(zc a, double s) { return zmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double zabs1(zc a) { return fabs(a.x) + fabs(a.y); }
__host__ __device__ __forceinline__ double zabs(zc a) { return hypot(a.x, a.y); }
// a*b + c
__host__ __device__ __forceinline__ zc zfma(zc a, zc b, zc c) {
  return zmk(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// conj(a)*b + c
__host__ __device__ __forceinline__ zc zcfma(zc a, zc b, zc c) {
  return zmk(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
// c - a*b in four FMAs (a separate product and subtraction take six FP64
// instructions, and GB300 issues FP64 at 1/64 of the FP32 rate)
__host__ __device__ __forceinline__ zc zfnma(zc a, zc b, zc c) {
  return zmk(fma(-a.x, b.x, fma(a.y, b.y, c.x)), fma(-a.x, b.y, fma(-a.y, b.x, c.y)));
}
// c - a*conj(b)
__host__ __device__ __forceinline__ zc zfnmac(zc a, zc b, zc c) {
  return zmk(fma(-a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
// robust complex division a/b (Smith's method)
__host__ __device__ __forceinline__ zc zdiv(zc a, zc b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return zmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    double r = b.x / b.y, d = b.y + b.x * r;
    return zmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
// principal square root
__host__ __device__ __forceinline__ zc zsqrt(zc a) {
  double m = zabs(a);
  if (m == 0.0) return zmk(0.0, 0.0);
  double t = sqrt(0.5 * (m + fabs(a.x)));
  if (a.x >= 0.0) return zmk(t, 0.5 * a.y / t);
  return zmk(0.5 * fabs(a.y) / t, copysign(t, a.y));
}

__host__ __device__ __forceinline__ cc cmk(float r, float i) { return make_float2(r, i); }
__host__ __device__ __forceinline__ cc cmul(cc a, cc b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__host__ __device__ __forceinline__ cc cfma(cc a, cc b, cc c) {
  return cmk(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__host__ __device__ __forceinline__ float cabs1f(cc a) { return fabsf(a.x) + fabsf(a.y); }

// generic helpers for templated LU / solves
template <typename T> struct cx;
template <> struct cx<zc> {
  typedef double real;
  __device__ static zc make(double r, double i) { return zmk(r, i); }
  __device__ static zc mul(zc a, zc b) { return zmul(a, b); }
  __device__ static zc fma_(zc a, zc b, zc c) { return zfma(a, b, c); }
  __device__ static zc sub(zc a, zc b) { return zsub(a, b); }
  __device__ static zc fnma(zc a, zc b, zc c) { return zfnma(a, b, c); }   // c - a*b
  __device__ static zc div(zc a, zc b) { return zdiv(a, b); }
  __device__ static double abs1(zc a) { return zabs1(a); }
  __device__ static zc from(zc a) { return a; }
  __device__ static zc to64(zc a) { return a; }
};
template <> struct cx<cc> {
  typedef float real;
  __device__ static cc make(float r, float i) { return cmk(r, i); }
  __device__ static cc mul(cc a, cc b) { return cmul(a, b); }
  __device__ static cc fma_(cc a, cc b, cc c) { return cfma(a, b, c); }
  __device__ static cc sub(cc a, cc b) { return cmk(a.x - b.x, a.y - b.y); }
  __device__ static cc fnma(cc a, cc b, cc c) {   // c - a*b
    return cmk(fmaf(-a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(-a.x, b.y, fmaf(-a.y, b.x, c.y)));
  }
  __device__ static cc div(cc a, cc b) {
    // float Smith division
    if (fabsf(b.x) >= fabsf(b.y)) {
      float r = b.y / b.x, d = b.x + b.y * r;
      return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    } else {
      float r = b.x / b.y, d = b.y + b.x * r;
      return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
    }
  }
  __device__ static float abs1(cc a) { return cabs1f(a); }
  __device__ static cc from(zc a) { return cmk((float)a.x, (float)a.y); }
  __device__ static zc to64(cc a) { return zmk(a.x, a.y); }
};

// ---------------------------------------------------------------------------
// per-instance descriptor (device side).  Offsets index the batch pools.
// ---------------------------------------------------------------------------
struct InstDesc {
  int32_t ny, n;          // nodes, unknowns 5*ny
  int32_t itype, wallt, top, mattyp, navier, nym;
  int32_t dmat;           // index of the (D1, D2) table for this ny
  int32_t m;              // order of the standard eigenproblem: n (temporal), 2n (spatial)
  int32_t iprof;          // index of the mean profile (ProfDesc)
  int32_t ider;           // 1: mean derivatives by the collocation matrices; 0: from tables (getmean2)
  double Ma, Re, Pr, Te, yi, ymax;
  double ar, ai, br, bi, wr, wi;  // alpha, beta, omega
  int64_t off_prof;       // profile pool (doubles): nym*6, row-major y rho u v w T
  int64_t off_spl;        // spline second-derivative pool: nym*5
  int64_t off_node;       // node pool (doubles): NODE_STRIDE*ny
  int64_t off_blk;        // per-node operator blocks (complex): BLK_STRIDE*ny
  int64_t off_mat;        // dense complex128 matrix pool (elements)
  int64_t off_mat32;      // dense complex64 matrix pool (elements)
  int64_t off_vec;        // vector pool (complex128 elements): VEC_SLOTS*n
  // ider = 0: the first and second y-derivative tables of the profile
  // (getmean2.f90:99-175), profile entries like the mean's
  int32_t iprof_d1, iprof_d2;
  int64_t off_prof_d1, off_spl_d1, off_prof_d2, off_spl_d2;
  // curved wall (spatial, curve = 2): 1, and the arc-position scalars of the
  // circle's metric (dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1,
  // d2bn2) from which h(y) and its derivatives follow (circh.f90:190-199)
  int32_t curved;
  // finite-difference temporal solver (fd_temporal.f90, input itype 3):
  // ogengrid nodes on a uniform eta, node 0 at the wall; D tables are its
  // stencil matrices, and the mean derivatives use grad.f90's matrices
  int32_t fd;
  int32_t dmean, pad3_;   // index of the mean-derivative (D1, D2) table (= dmat for Chebyshev)
  double cw[8];
};
#define VEC_SLOTS 10

// one entry per distinct mean profile (a batch may share profiles)
struct ProfDesc {
  int64_t off_prof;       // profile pool (doubles): nym*6
  int64_t off_spl;        // spline pool (doubles): nym*6
  int32_t nym;
  int32_t three;          // 1: one of the three tables of an ider = 0 profile row
};

// node pool layout per node (doubles): y eta deta d2eta vm[5] g2[5] g22[5]
#define NODE_Y 0
#define NODE_ETA 1
#define NODE_DETA 2
#define NODE_D2ETA 3
#define NODE_VM 4
#define NODE_G2 9
#define NODE_G22 14
#define NODE_STRIDE 19

// per-node operator blocks (complex128 5x5, row-major [eq][var]):
// temporal (A0 row block i = P1 D1(i,:) - P2 D2(i,:) + delta P3; B0 block = Bb)
//   0: Bh (mapped, masked)   1: Vyy (mapped, masked)   2: Dh (masked)
//   3: B0 diagonal block     4: B0 diagonal block inverse
// spatial (C_k row block i = P1k D1(i,:) - P2k D2(i,:) + delta P3k):
//   0: Bh0  1: Vyy0  2: Dh0 (incl. -i omega G and BC diagonals)
//   3: Bh1  4: Dh1   5: C2 diagonal block (Vxx)
#define BLK_NB 6
#define BLK_STRIDE (BLK_NB * 25)

// ---------------------------------------------------------------------------
// error checking for host code
// ---------------------------------------------------------------------------
#define STAB_CUDA_OK(expr) ((expr) == cudaSuccess)
