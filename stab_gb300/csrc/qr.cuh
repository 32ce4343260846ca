// The QR part of the full-spectrum eigensolver, in either working precision:
// precision traits, reflectors, multi-bulge sweeps and the complex QR
// iteration on a packed Hessenberg matrix.  hqr.cu includes it inside
// namespace stab; the CPU test of the double-word QR compiles it on the host
// with the CUDA thread model replaced by threads of one process.
#pragma once

#define HQ_T 128        // block of the batched (persistent) eigensolver
#define HQ_WIDE 512     // block for a few large instances (latency)
#define HQ_MAXW (HQ_WIDE / 32)
// the device code runs with either block size
#define NTH ((int)blockDim.x)
#define NWA ((int)(blockDim.x >> 5))

// multi-bulge sweeps: at most MS_MAXB bulges; the trailing MS_MAXB x
// MS_MAXB block that supplies their shifts is kept packed in MS_SMALL entries
#define MS_MAXB 6
#define MS_SMALL 48

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ dw warp_sum(dw v) {
  for (int o = 16; o > 0; o >>= 1)
    v = dw_add(v, make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o)));
  return v;
}

// Working precision of the Hessenberg reduction and the QR iteration:
// complex128 (zc), or double-word complex (dz) for the seed spectra.  `real`
// is the type of magnitude tests, `sq` the accumulator of sums of squares.
// Scalar work of one thread per step (reflector and shift formulas) runs in
// FP64 on converted values in both precisions.
template <class C> struct ew;
template <> struct ew<zc> {
  typedef double real;
  typedef double sq;
  typedef zc S;        // one-thread shift formulas, and their real type
  typedef double SR;
  __device__ static zc to_s(zc a) { return a; }
  __device__ static zc from_s(zc a) { return a; }
  __device__ static zc smk(double r, double i) { return zmk(r, i); }
  __device__ static double ulp() { return 2.220446049250313e-16; }
  __device__ static double safmin() { return 2.2250738585072014e-308; }
  __device__ static zc zero() { return zmk(0.0, 0.0); }
  __device__ static zc one() { return zmk(1.0, 0.0); }
  __device__ static zc from64(zc a) { return a; }
  __device__ static zc to64(zc a) { return a; }
  __device__ static double mag2(zc a) { return a.x * a.x + a.y * a.y; }
  __device__ static double sq_zero() { return 0.0; }
  __device__ static void sq_add(double& acc, zc a) { acc = fma(a.x, a.x, fma(a.y, a.y, acc)); }
  __device__ static double sq_64(double v) { return v; }
  __device__ static zc warp_sum_c(zc a) { return zmk(warp_sum(a.x), warp_sum(a.y)); }
};
template <> struct ew<dz> {
  typedef float real;
  typedef double sq;
  // the shift formulas of one thread run in FP64: a complex64 shift carries an
  // absolute error of 2^-24 times the trailing block's entries, which stalls
  // the convergence of small clustered eigenvalues (spatial companion
  // matrices)
  typedef zc S;
  typedef double SR;
  __device__ static zc to_s(dz a) { return dz_to64(a); }
  __device__ static dz from_s(zc a) { return dz_from64(a); }
  __device__ static zc smk(double r, double i) { return zmk(r, i); }
  // deflation and start tests use 2^-44: a double-word multiply-add errs by
  // up to ~2^-46.5 of its operands, and the threshold keeps a few units of
  // margin above that (as FP64's 2^-52 is twice its unit roundoff).
  // Magnitudes in the tests are the high words.
  __device__ static float ulp() { return 5.68434189e-14f; }
  __device__ static float safmin() { return 1.17549435e-38f; }
  __device__ static dz zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  __device__ static dz one() { return make_float4(1.f, 0.f, 0.f, 0.f); }
  __device__ static dz from64(zc a) { return dz_from64(a); }
  __device__ static zc to64(dz a) { return dz_to64(a); }
  __device__ static float mag2(dz a) { return a.x * a.x + a.z * a.z; }
  // sums of squares (O(n) per Householder step) in FP64: squares of the
  // ~1e-20 entries of a balanced low-Mach operator underflow in float
  __device__ static double sq_zero() { return 0.0; }
  __device__ static void sq_add(double& acc, dz a) {
    const zc v = dz_to64(a);
    acc = fma(v.x, v.x, fma(v.y, v.y, acc));
  }
  __device__ static double sq_64(double v) { return v; }
  __device__ static dz warp_sum_c(dz a) { return dz_mk(warp_sum(dz_re(a)), warp_sum(dz_im(a))); }
};

// 2-element reflector in FP64, as formed by make_refl
struct Refl {
  double tr, ti, ur, ui, beta, v1r, v1i;
  int ident;
};
// the same reflector in the working precision: applied through tau and u2;
// bv is what the annihilated column keeps at the top (beta, or v1 for an
// identity reflector)
template <class C> struct ReflC {
  C tau, u2, bv;
  int ident;
};
template <class C>
__device__ __forceinline__ ReflC<C> pack_refl(const Refl& f) {
  ReflC<C> o;
  o.ident = f.ident;
  o.tau = ew<C>::from64(zmk(f.tr, f.ti));
  o.u2 = ew<C>::from64(zmk(f.ur, f.ui));
  o.bv = ew<C>::from64(f.ident ? zmk(f.v1r, f.v1i) : zmk(f.beta, 0.0));
  return o;
}

template <class C>
struct HqrSmem {
  double red[2 * HQ_MAXW];
  int flag;
  int found;
  int mp;
  int kk;
  int emax;
  double sc[8];        // broadcast FP64 scalars (gathered sums)
  C hc[3];             // Householder step of the reduction: tau, scale, beta
  C tsh;               // shift of a single-shift iteration
  ReflC<C> refl[2];    // reflector of the next bulge step, double buffered
  ReflC<C> srefl[2];   // the same for the small QR that supplies shifts
  // multi-bulge sweeps: shifts, the trailing block they come from (packed),
  // and one reflector per bulge
  zc shifts[MS_MAXB];
  C small[MS_SMALL];
  ReflC<C> mrefl[MS_MAXB];
};

// block sum of two values; result valid in all threads after return
template <class T, class SM>
__device__ void block_sum2(SM& s, T& a, T& b) {
  T* red = reinterpret_cast<T*>(s.red);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  __syncthreads();
  if (lane == 0) { red[warp] = a; red[HQ_MAXW + warp] = b; }
  __syncthreads();
  T ta = 0, tb = 0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { ta += red[q]; tb += red[HQ_MAXW + q]; }
  a = ta;
  b = tb;
  __syncthreads();
}
// block sum of a sum-of-squares accumulator, returned in FP64 to all threads
template <class C, class SM>
__device__ double block_sum_sq(SM& s, typename ew<C>::sq a) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = warp_sum(a);
  __syncthreads();
  if (lane == 0) s.red[warp] = ew<C>::sq_64(a);
  __syncthreads();
  double t = 0.0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += s.red[q];
  __syncthreads();
  return t;
}

// packed Hessenberg-plus-one storage: column c keeps rows 0 .. min(c + 2,
// mp - 1)
__host__ __device__ __forceinline__ int64_t hess_coff(int c, int mp) {
  return (int64_t)c * (c + 5) / 2 - ((c == mp - 1 && mp >= 2) ? 1 : 0);
}
__host__ __device__ __forceinline__ int64_t hess_packed_size(int mp) {
  return mp <= 0 ? 0 : hess_coff(mp - 1, mp) + mp;
}
template <class C>
struct SAcc {
  C* S;
  int mp;
  __device__ __forceinline__ C& operator()(int r, int c) const { return S[hess_coff(c, mp) + r]; }
};
// windows at least this wide use multi-bulge sweeps
#define MS_MIN_WINDOW 16

// 2-element reflector (as ZLARFG): (v1, v2) -> (beta, 0).  It sits on the
// serial path of every bulge step, where each FP64 instruction of a single
// thread costs a full warp issue of the 1/64-rate FP64 pipe, so it uses one
// reciprocal square root (|beta| and 1/beta from it) and one reciprocal.
__device__ __forceinline__ Refl make_refl(zc v1, zc v2) {
  Refl f;
  f.v1r = v1.x;
  f.v1i = v1.y;
  const double n2 = v2.x * v2.x + v2.y * v2.y;
  if (n2 == 0.0 && v1.y == 0.0) {
    f.ident = 1;
    f.tr = f.ti = f.ur = f.ui = 0.0;
    f.beta = v1.x;
    return f;
  }
  f.ident = 0;
  const double S = fma(v1.x, v1.x, fma(v1.y, v1.y, n2));
  const double r = rsqrt(S);
  const double beta = -copysign(S * r, v1.x);
  const double ib = -copysign(r, v1.x);                    // 1 / beta
  f.beta = beta;
  f.tr = (beta - v1.x) * ib;
  f.ti = -v1.y * ib;
  const double dr = v1.x - beta, di = v1.y;                // u2 = v2 / (v1 - beta)
  const double idd = __drcp_rn(fma(dr, dr, di * di));
  f.ur = fma(v2.x, dr, v2.y * di) * idd;
  f.ui = fma(v2.y, dr, -v2.x * di) * idd;
  return f;
}
// reflector that starts a bulge: (h11 - shift, h21), scaled
__device__ __forceinline__ Refl entry_refl(zc h11, zc h21, zc shift) {
  const zc h11s = zsub(h11, shift);
  double sc = zabs1(h11s) + zabs1(h21);
  if (sc == 0.0) sc = 1.0;
  return make_refl(zscale(h11s, 1.0 / sc), zscale(h21, 1.0 / sc));
}
__device__ __forceinline__ ReflC<zc> refl_of(zc v1, zc v2) { return pack_refl<zc>(make_refl(v1, v2)); }
__device__ __forceinline__ ReflC<zc> entry_of(zc h11, zc h21, zc shift) {
  return pack_refl<zc>(entry_refl(h11, h21, shift));
}

// The double-word reflector: the formulas of make_refl, with 1/|v| and the
// reciprocal from Newton steps in double-word arithmetic (dw_rsqrt, dw_rcp).
// It runs on the serial path of every bulge step, which then issues no FP64
// instruction at all.  The float exponent range is narrow: entries of a bulge
// passing a nearly deflated stretch are ~1e-20, whose squares underflow, so
// (v1, v2) is first scaled by the power of two that brings its larger part
// near 1 (tau and u2 do not depend on the scale; beta is scaled back).
__device__ __forceinline__ ReflC<dz> refl_of(dz v1in, dz v2in) {
  ReflC<dz> f;
  const float mx = fmaxf(zabs1(v1in), zabs1(v2in));
  const int ex = dw_scale_exponent(mx);
  const dz v1 = zscale(v1in, ldexpf(1.f, -ex)), v2 = zscale(v2in, ldexpf(1.f, -ex));
  const dw v1r = dz_re(v1), v1i = dz_im(v1), v2r = dz_re(v2), v2i = dz_im(v2);
  const dw n2 = dw_fma(v2r, v2r, dw_mul(v2i, v2i));
  if (n2.x == 0.f && v1i.x == 0.f) {
    f.ident = 1;
    f.tau = f.u2 = make_float4(0.f, 0.f, 0.f, 0.f);
    f.bv = v1in;
    return f;
  }
  f.ident = 0;
  const dw S = dw_fma(v1r, v1r, dw_fma(v1i, v1i, n2));
  const dw r = dw_rsqrt(S);
  const float sg = -copysignf(1.f, v1r.x);
  const dw ab = dw_mul(S, r);                                  // |beta|
  const dw beta = make_float2(sg * ab.x, sg * ab.y);
  const dw ib = make_float2(sg * r.x, sg * r.y);               // 1 / beta
  const dw tr = dw_mul(dw_add(beta, dw_neg(v1r)), ib);
  const dw ti = dw_neg(dw_mul(v1i, ib));
  const dw dr = dw_add(v1r, dw_neg(beta));                     // u2 = v2 / (v1 - beta)
  const dw idd = dw_rcp(dw_fma(dr, dr, dw_mul(v1i, v1i)));
  const dw ur = dw_mul(dw_fma(v2r, dr, dw_mul(v2i, v1i)), idd);
  const dw ui = dw_mul(dw_fma(v2i, dr, dw_neg(dw_mul(v2r, v1i))), idd);
  f.tau = dz_mk(tr, ti);
  f.u2 = dz_mk(ur, ui);
  f.bv = zscale(dz_mk(beta, make_float2(0.f, 0.f)), ldexpf(1.f, ex));
  return f;
}
// scaled by a power of two near 1 / (|h11 - shift| + |h21|), which is exact
__device__ __forceinline__ ReflC<dz> entry_of(dz h11, dz h21, dz shift) {
  const dz h11s = zsub(h11, shift);
  const float p = ldexpf(1.f, -dw_scale_exponent(zabs1(h11s) + zabs1(h21)));
  return refl_of(zscale(h11s, p), zscale(h21, p));
}

// left: rows k, k+1 of column j;  right: columns k, k+1 of row j
template <class C>
__device__ __forceinline__ void apply_left(const SAcc<C>& H, int k, int j, C tau, C u2) {
  C a = H(k, j), b = H(k + 1, j);
  C sm = zmul(zconj(tau), zcfma(u2, b, a));
  H(k, j) = zsub(a, sm);
  H(k + 1, j) = zfnma(sm, u2, b);
}
template <class C>
__device__ __forceinline__ void apply_right(const SAcc<C>& H, int k, int j, C tau, C u2) {
  C a = H(j, k), b = H(j, k + 1);
  C sm = zmul(tau, zfma(u2, b, a));
  H(j, k) = zsub(a, sm);
  H(j, k + 1) = zfnmac(sm, u2, b);
}

// One sweep of nb bulges over the active window [l, i] (i - l + 1 >=
// 3 nb + 2), with the shifts in s.shifts.  Bulge q enters at row l at step
// 3q and sits at row k = l + step - 3q.  Rows of different bulges are three
// apart, so within a step the left updates of all bulges (rows k, k+1) are
// disjoint, and so are the right updates (columns k, k+1).  Left and right
// updates commute, so a step runs all left updates, then all right updates,
// then forms every bulge's next reflector on lanes of warp 0, with a barrier
// between phases.  That puts the serial reflector work of nb bulges into
// the same warp instructions.
template <class C>
__device__ void multi_bulge_sweep(const SAcc<C>& H, int l, int i, int nb, HqrSmem<C>& s, long long& upd) {
  const int tid = threadIdx.x;
  const int steps = (i - l) + 3 * (nb - 1);
  // entering reflector of bulge 0
  if (tid == 0) s.mrefl[0] = entry_of(H(l, l), H(l + 1, l), ew<C>::from64(s.shifts[0]));
  __syncthreads();
  for (int st = 0; st < steps; ++st) {
    // active bulges: q with 0 <= st - 3q <= i - l - 1
    const int qhi = min(nb - 1, st / 3);
    const int qlo = max(0, (st - (i - l - 1) + 2) / 3);
    // phase L: annihilation writes (column k-1) and left updates of columns k..i
    int ltask = 0;
    for (int q = qlo; q <= qhi; ++q) ltask += 1 + (i - (l + st - 3 * q) + 1);
    if (tid == 0) upd += ltask;
    for (int t = tid; t < ltask; t += NTH) {
      int q = qlo, rem = t;
      for (;;) {
        const int cnt = 1 + (i - (l + st - 3 * q) + 1);
        if (rem < cnt) break;
        rem -= cnt;
        ++q;
      }
      const int k = l + st - 3 * q;
      const ReflC<C>& f = s.mrefl[q];
      if (rem == 0) {
        if (k > l) {
          H(k, k - 1) = f.bv;
          H(k + 1, k - 1) = ew<C>::zero();
        }
      } else if (!f.ident) {
        apply_left(H, k, k + rem - 1, f.tau, f.u2);
      }
    }
    __syncthreads();
    // phase R: right updates of rows l..min(k+2, i)
    int rtask = 0;
    for (int q = qlo; q <= qhi; ++q) {
      const int k = l + st - 3 * q;
      rtask += min(k + 2, i) - l + 1;
    }
    if (tid == 0) upd += rtask;
    for (int t = tid; t < rtask; t += NTH) {
      int q = qlo, rem = t;
      for (;;) {
        const int k = l + st - 3 * q;
        const int cnt = min(k + 2, i) - l + 1;
        if (rem < cnt) break;
        rem -= cnt;
        ++q;
      }
      const int k = l + st - 3 * q;
      const ReflC<C>& f = s.mrefl[q];
      if (!f.ident) apply_right(H, k, l + rem, f.tau, f.u2);
    }
    __syncthreads();
    // phase C: next reflector of every bulge that moves on, and the
    // entering reflector of the bulge that starts next step
    if (tid < 32) {
      const int q = tid;
      if (q < nb) {
        const int k = l + st - 3 * q;          // position this step
        if (k >= l && k + 1 <= i - 1) {
          s.mrefl[q] = refl_of(H(k + 1, k), H(k + 2, k));
        } else if (k + 1 == l) {               // enters next step
          s.mrefl[q] = entry_of(H(l, l), H(l + 1, l), ew<C>::from64(s.shifts[q]));
        }
      }
    }
    __syncthreads();
  }
}

// Complex QR on the mp x mp upper Hessenberg matrix behind H (single-shift
// steps, and multi-bulge sweeps when MULTI); writes the eigenvalues to
// ev[0..mp) in FP64.  refl is the double-buffered reflector slot of the
// single-shift chase; upd (thread 0) counts 2-element reflector applications
// in integers, so counting adds no FP64 instruction.  Returns 0 or
// STAB_ST_NOCONV.
template <class E, bool MULTI, class SM>
__device__ int qr_eigs(const SAcc<E> H, const int mp, zc* ev, SM& s, ReflC<E>* refl, long long& upd) {
  typedef typename ew<E>::real R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const R ulp = ew<E>::ulp();
  const R smlnum = ew<E>::safmin() * ((R)mp / ulp);
  const int its_cap = 40 * (mp > 10 ? mp : 10);
  int st = 0;
  int total_its = 0;
  int i = mp - 1;
  while (i >= 0 && st == 0) {
    int l = 0;
    int kdefl = 0;
    for (;;) {
      // largest k in [l+1, i] with a negligible subdiagonal; l if none
      if (tid == 0) s.kk = l;
      __syncthreads();
      for (int k = i - tid; k >= l + 1; k -= NTH) {
        const E h = H(k, k - 1);
        bool ok = zabs1(h) <= smlnum;
        if (!ok) {
          R tst = zabs1(H(k - 1, k - 1)) + zabs1(H(k, k));
          if (tst == (R)0) {
            if (k - 2 >= 0) tst += zabs1(H(k - 1, k - 2));
            if (k + 1 <= mp - 1) tst += zabs1(H(k + 1, k));
          }
          if (zabs1(h) <= ulp * tst) {
            const R h1 = zabs1(h), h2 = zabs1(H(k - 1, k));
            const R ab = max(h1, h2), ba = min(h1, h2);
            const R d1 = zabs1(H(k, k)), d2 = zabs1(zsub(H(k - 1, k - 1), H(k, k)));
            const R aa = max(d1, d2), bb = min(d1, d2);
            const R sm = aa + ab;
            ok = ba * (ab / sm) <= max(smlnum, ulp * (bb * (aa / sm)));
          }
        }
        if (ok) { atomicMax(&s.kk, k); break; }   // this thread's larger k's were tested first
      }
      __syncthreads();
      l = s.kk;
      __syncthreads();
      if (l > 0 && tid == 0) H(l, l - 1) = ew<E>::zero();
      if (l >= i) break;
      if (total_its >= its_cap) { st = STAB_ST_NOCONV; break; }
      ++kdefl;
      ++total_its;
      if constexpr (MULTI) {
        if ((i - l + 1) >= MS_MIN_WINDOW && kdefl % 10 != 0) {
          // shifts: eigenvalues of the trailing nb x nb block (a small
          // single-shift QR on a packed copy), then one sweep of nb bulges
          const int nb = (i - l + 1) >= 3 * MS_MAXB + 2 + 24 ? MS_MAXB : 2;
          const int o = i - nb + 1;
          for (int c = tid; c < nb; c += NTH)
            for (int r = 0; r <= min(c + 2, nb - 1); ++r)
              s.small[hess_coff(c, nb) + r] = (r <= c + 1) ? H(o + r, o + c) : ew<E>::zero();
          __syncthreads();
          long long su = 0;
          const int sst = qr_eigs<E, false>(SAcc<E>{s.small, nb}, nb, s.shifts, s, s.srefl, su);
          upd += su;
          if (sst == 0) {
            multi_bulge_sweep(H, l, i, nb, s, upd);
            total_its += nb - 1;
            continue;
          }
          // the small eigensolve did not converge: a single-shift iteration
        }
      }
      // shift (one thread)
      if (tid == 0) {
        typedef typename ew<E>::S S;
        typedef typename ew<E>::SR SR;
        S t;
        if (kdefl % 20 == 0) {
          t = zadd(ew<E>::smk(0.75 * zabs(ew<E>::to_s(H(i, i - 1))), 0.0), ew<E>::to_s(H(i, i)));
        } else if (kdefl % 10 == 0) {
          t = zadd(ew<E>::smk(0.75 * zabs(ew<E>::to_s(H(l + 1, l))), 0.0), ew<E>::to_s(H(l, l)));
        } else {
          t = ew<E>::to_s(H(i, i));
          const S u = zmul(zsqrt(ew<E>::to_s(H(i - 1, i))), zsqrt(ew<E>::to_s(H(i, i - 1))));
          const SR su = zabs1(u);
          if (su != (SR)0) {
            const S x = zscale(zsub(ew<E>::to_s(H(i - 1, i - 1)), t), (SR)0.5);
            const SR sx = zabs1(x);
            const SR sc = max(su, sx);
            const S xs = zscale(x, (SR)1 / sc), us = zscale(u, (SR)1 / sc);
            S y = zscale(zsqrt(zadd(zmul(xs, xs), zmul(us, us))), sc);
            if (sx > (SR)0) {
              const S xn = zscale(x, (SR)1 / sx);
              if (xn.x * y.x + xn.y * y.y < (SR)0) y = ew<E>::smk(-y.x, -y.y);
            }
            t = zsub(t, zmul(u, zdiv(u, zadd(x, y))));
          }
        }
        s.tsh = ew<E>::from_s(t);
        s.kk = l;
      }
      __syncthreads();
      const E te = s.tsh;
      // start row: largest m in [l+1, i-1] where two consecutive small
      // subdiagonals decouple the sweep; l otherwise
      for (int mm = i - 1 - tid; mm >= l + 1; mm -= NTH) {
        const E h11 = H(mm, mm), h22 = H(mm + 1, mm + 1);
        const E h11s = zsub(h11, te);
        const E h21 = H(mm + 1, mm);
        const R sc = zabs1(h11s) + zabs1(h21);
        if (sc == (R)0) continue;
        const R h10 = zabs1(H(mm, mm - 1));
        // |h10| |h21/sc| <= ulp |h11s/sc| (|h11| + |h22|), multiplied through by sc
        if (h10 * zabs1(h21) <= ulp * (zabs1(h11s) * (zabs1(h11) + zabs1(h22)))) {
          atomicMax(&s.kk, mm);
          break;
        }
      }
      __syncthreads();
      const int m0 = s.kk;
      if (tid == 0) refl[m0 & 1] = entry_of(H(m0, m0), H(m0 + 1, m0), te);
      __syncthreads();
      // bulge chase, one barrier per step.  The serial corner of a step is
      // reflector k on columns k, k+1, then on rows k, k+1, then reflector
      // k+1 formed from the new bulge.  It runs on lanes of warp 0 in three
      // dependent stages of one update each.  Every other update of the step
      // (columns k+2..i, rows l..k-1 and k+2) is independent of it and of the
      // others and runs on all threads.
      for (int k = m0; k < i; ++k) {
        const ReflC<E> f = refl[k & 1];
        const E tau = f.tau, u2 = f.u2;
        const int nleft = i - k - 1;        // columns k+2..i
        const int nrows = k - l;            // rows l..k-1
        const int ntask = 4 + nleft + nrows;
        if (tid == 0) upd += i - l + 4;
        for (int q = tid; q < ntask; q += NTH) {
          if (q == 0) {
            if (!f.ident) apply_left(H, k, k, tau, u2);
          } else if (q == 1) {
            if (!f.ident) apply_left(H, k, k + 1, tau, u2);
          } else if (q == 2) {
            if (!f.ident && k + 2 <= i) apply_right(H, k, k + 2, tau, u2);
          } else if (q == 3) {
            if (k > m0) {
              H(k, k - 1) = f.bv;
              H(k + 1, k - 1) = ew<E>::zero();
            }
            // a sweep started below l still applies the first reflector to
            // column m0-1: H(m0, m0-1) picks up (1 - conj(tau)); the fill-in
            // at H(m0+1, m0-1) is what the start test bounds
            if (!f.ident && k == m0 && m0 > l)
              H(m0, m0 - 1) = zmul(H(m0, m0 - 1), zsub(ew<E>::one(), zconj(tau)));
          } else if (!f.ident) {
            const int t = q - 4;
            if (t < nleft) apply_left(H, k, k + 2 + t, tau, u2);
            else apply_right(H, k, l + (t - nleft), tau, u2);
          }
        }
        if (warp == 0) {
          __syncwarp();
          if (lane < 2 && !f.ident) apply_right(H, k, k + lane, tau, u2);   // rows k, k+1
          __syncwarp();
          if (lane == 0 && k + 1 < i) refl[(k + 1) & 1] = refl_of(H(k + 1, k), H(k + 2, k));
        }
        __syncthreads();
      }
    }
    if (st) break;
    if (tid == 0) ev[i] = ew<E>::to64(H(i, i));
    i = l - 1;
    __syncthreads();
  }
  if (st)
    for (int q = tid; q <= i; q += NTH) ev[q] = zmk(nan(""), nan(""));
  __syncthreads();
  return st;
}
