// Plain FP64 full-spectrum eigensolver: the GPU replacement of ZGEEV
// (temporal.f90:803, spatial.f90:1043) for all eigenvalues.
//
// Per instance (one 256-thread CTA, instances taken from a work counter):
//   1. isolation: rows (columns) whose off-diagonal entries are exactly zero
//      within the active set give eigenvalue a_ii and are removed, repeated
//      until none is found (the permutation step of ZGEBAL).  The temporal
//      Dirichlet rows and the zero columns of the spatial companion matrix
//      leave this way, so they come out as exact zeros like in ZGEEV.
//   2. compaction of the active submatrix into H;
//   3. diagonal balancing by powers of two (the scaling step of ZGEBAL);
//   4. Householder reduction to upper Hessenberg form (as ZGEHD2);
//   5. single-shift complex QR with Wilkinson shifts, exceptional shifts
//      every 10th iteration and the conservative deflation test of Ahues and
//      Tisseur (the algorithm of ZLAHQR, eigenvalues only).  The 2-element
//      reflectors are general complex ones, so the subdiagonal need not be
//      kept real.
// All arithmetic is FP64.  Every loop has an iteration cap; an instance
// that hits it gets status STAB_ST_NOCONV and NaN for the missing values.
#include "common.cuh"
#include "kernels.cuh"
#include "hqr.cuh"

namespace stab {

#define HQ_T 256
#define HQ_W (HQ_T / 32)

struct HqrSmem {
  double red[2 * HQ_W];
  int ired[HQ_W];
  int flag;
  int found;
  int mp;
  int kk;
  double f;
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// block sum of two doubles; result valid in all threads after return
__device__ void block_sum2(HqrSmem& s, double& a, double& b) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  __syncthreads();
  if (lane == 0) { s.red[warp] = a; s.red[HQ_W + warp] = b; }
  __syncthreads();
  double ta = 0.0, tb = 0.0;
  for (int q = 0; q < HQ_W; ++q) { ta += s.red[q]; tb += s.red[HQ_W + q]; }
  a = ta;
  b = tb;
  __syncthreads();
}

__global__ void __launch_bounds__(HQ_T) k_eig_plain(int count, const int32_t* __restrict__ msz, zc* __restrict__ A,
                                                   const int64_t* __restrict__ a_off, zc* __restrict__ Hp,
                                                   const int64_t* __restrict__ h_off, zc* __restrict__ eig,
                                                   const int64_t* __restrict__ eig_off, int32_t* __restrict__ status,
                                                   int32_t* __restrict__ work_counter, const int32_t* __restrict__ order,
                                                   double* __restrict__ flops_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem s;
  __shared__ int s_inst;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double ulp = 2.220446049250313e-16;
  const double safmin = 2.2250738585072014e-308;
  for (;;) {
    if (tid == 0) s_inst = atomicAdd(work_counter, 1);
    __syncthreads();
    const int slot = s_inst;
    if (slot >= count) return;
    const int inst = order ? order[slot] : slot;
    const int m = msz[inst];
    zc* M = A + a_off[inst];
    zc* H = Hp + h_off[inst];
    zc* ev = eig + eig_off[inst];
    // shared scratch: active flags (m bytes, as int), act list (m ints), v, w, z (m complex each)
    int* active = reinterpret_cast<int*>(smraw);
    int* act = active + m;
    zc* v = reinterpret_cast<zc*>(smraw + ((2 * (size_t)m * sizeof(int) + 15) / 16) * 16);
    zc* w = v + m;
    zc* z = w + m;
    for (int i = tid; i < m; i += HQ_T) active[i] = 1;
    if (tid == 0) s.mp = 0;
    __syncthreads();
    // ---- 1. isolation -----------------------------------------------------
    int n_iso = 0;           // isolated eigenvalues are written from the top: ev[m-1-q]
    for (int pass = 0; pass < m; ++pass) {
      if (tid == 0) s.found = 0;
      __syncthreads();
      // rows: thread per row
      for (int r = tid; r < m; r += HQ_T) {
        if (!active[r]) continue;
        bool zero = true;
        for (int c = 0; c < m && zero; ++c) {
          if (c == r || !active[c]) continue;
          zc a = M[(size_t)c * m + r];
          zero = (a.x == 0.0 && a.y == 0.0);
        }
        if (zero) { active[r] = 2; atomicAdd(&s.found, 1); }   // 2 = isolated this pass (row)
      }
      // columns: warp per column
      for (int c = warp; c < m; c += HQ_W) {
        if (active[c] != 1) continue;
        bool zero = true;
        for (int r = lane; r < m; r += 32) {
          if (r == c || active[r] == 0) continue;
          zc a = M[(size_t)c * m + r];
          if (a.x != 0.0 || a.y != 0.0) zero = false;
        }
        zero = __all_sync(0xffffffffu, zero);
        if (zero && lane == 0) { active[c] = 3; atomicAdd(&s.found, 1); }
      }
      __syncthreads();
      const int found = s.found;
      if (found == 0) break;
      // record eigenvalues of the newly isolated indices (sequential, deterministic order)
      if (tid == 0) {
        int q = n_iso;
        for (int i = 0; i < m; ++i)
          if (active[i] >= 2) { ev[m - 1 - q] = M[(size_t)i * m + i]; active[i] = 0; ++q; }
        s.kk = q;
      }
      __syncthreads();
      n_iso = s.kk;
      __syncthreads();
    }
    // ---- 2. compaction ------------------------------------------------------
    if (tid == 0) {
      int q = 0;
      for (int i = 0; i < m; ++i)
        if (active[i]) act[q++] = i;
      s.mp = q;
    }
    __syncthreads();
    const int mp = s.mp;
    const int ld = mp;
    for (int c = warp; c < mp; c += HQ_W) {
      const int sc = act[c];
      for (int r = lane; r < mp; r += 32) H[(size_t)c * ld + r] = M[(size_t)sc * m + act[r]];
    }
    __syncthreads();
    // ---- 3. balancing -------------------------------------------------------
    for (int sweep = 0; sweep < 64; ++sweep) {
      if (tid == 0) s.flag = 0;
      __syncthreads();
      for (int i = 0; i < mp; ++i) {
        double cs = 0.0, rs = 0.0;
        for (int r = tid; r < mp; r += HQ_T) {
          if (r == i) continue;
          zc a = H[(size_t)i * ld + r];
          cs += a.x * a.x + a.y * a.y;
          zc b = H[(size_t)r * ld + i];
          rs += b.x * b.x + b.y * b.y;
        }
        block_sum2(s, cs, rs);
        double c = sqrt(cs), r = sqrt(rs);
        double f = 1.0;
        if (c != 0.0 && r != 0.0) {
          double g = r / 2.0, sum = c + r;
          int guard = 0;
          while (c < g && guard++ < 2000) { f *= 2.0; c *= 2.0; r /= 2.0; g /= 2.0; }
          g = c / 2.0;
          while (g >= r && guard++ < 4000) { f /= 2.0; c /= 2.0; g /= 2.0; r *= 2.0; }
          if (c + r >= 0.95 * sum) f = 1.0;
        }
        if (f != 1.0) {
          const double gi = 1.0 / f;
          for (int q = tid; q < mp; q += HQ_T) {
            zc* a = &H[(size_t)q * ld + i];    // row i
            *a = zscale(*a, gi);
          }
          __syncthreads();
          for (int q = tid; q < mp; q += HQ_T) {
            zc* a = &H[(size_t)i * ld + q];    // column i
            *a = zscale(*a, f);
          }
          if (tid == 0) s.flag = 1;
          __syncthreads();
        }
      }
      __syncthreads();
      if (!s.flag) break;
      __syncthreads();
    }
    // ---- 4. Hessenberg reduction -----------------------------------------
    double flops = 0.0;   // FP64 work of the reduction and the sweeps (thread 0)
    for (int k = 0; k + 2 < mp; ++k) {
      const int L = mp - k - 1;
      if (tid == 0) flops += 16.0 * (double)mp * L + 16.0 * (double)L * L;
      double ss = 0.0, dummy = 0.0;
      for (int r = tid; r < L; r += HQ_T) {
        zc x = H[(size_t)k * ld + k + 1 + r];
        v[r] = x;
        if (r >= 1) ss += x.x * x.x + x.y * x.y;
      }
      block_sum2(s, ss, dummy);
      const zc alpha = v[0];
      if (ss == 0.0 && alpha.y == 0.0) continue;   // H(k) = I
      const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + ss), alpha.x);
      const zc tau = zmk((beta - alpha.x) / beta, -alpha.y / beta);
      const zc scal = zdiv(zmk(1.0, 0.0), zmk(alpha.x - beta, alpha.y));
      __syncthreads();
      for (int r = tid; r < L; r += HQ_T) v[r] = (r == 0) ? zmk(1.0, 0.0) : zmul(v[r], scal);
      if (tid == 0) H[(size_t)k * ld + k + 1] = zmk(beta, 0.0);
      for (int r = 2 + tid; r <= L; r += HQ_T) H[(size_t)k * ld + k + r] = zmk(0.0, 0.0);
      __syncthreads();
      // right: w = H(:, k+1:) v
      for (int r = tid; r < mp; r += HQ_T) {
        zc acc = zmk(0.0, 0.0);
        for (int c = 0; c < L; ++c) acc = zfma(H[(size_t)(k + 1 + c) * ld + r], v[c], acc);
        w[r] = zmul(tau, acc);
      }
      __syncthreads();
      // right update fused with the left product z = v^H H(k+1:, k+1:), warp per column
      for (int c = warp; c < L; c += HQ_W) {
        const zc vc = zconj(v[c]);
        zc* col = H + (size_t)(k + 1 + c) * ld;
        zc acc = zmk(0.0, 0.0);
        for (int r = lane; r < mp; r += 32) {
          zc h = zsub(col[r], zmul(w[r], vc));
          col[r] = h;
          if (r >= k + 1) acc = zcfma(v[r - k - 1], h, acc);
        }
        acc.x = warp_sum(acc.x);
        acc.y = warp_sum(acc.y);
        if (lane == 0) z[c] = zmul(zconj(tau), acc);
      }
      __syncthreads();
      // left update: H(k+1:, k+1:) -= v z
      for (int c = warp; c < L; c += HQ_W) {
        const zc zc_ = z[c];
        zc* col = H + (size_t)(k + 1 + c) * ld + k + 1;
        for (int r = lane; r < L; r += 32) col[r] = zsub(col[r], zmul(v[r], zc_));
      }
      __syncthreads();
    }
    // ---- 5. QR iteration ----------------------------------------------------
    int st = 0;
    int total_its = 0;
    const int its_cap = 40 * (mp > 10 ? mp : 10);
    const double smlnum = safmin * ((double)mp / ulp);
    auto Hs = [&](int r, int c) -> zc& { return H[(size_t)c * ld + r]; };
    int i = mp - 1;
    while (i >= 0 && st == 0) {
      int l = 0;
      int kdefl = 0;
      for (;;) {
        // largest k in [l+1, i] with a negligible subdiagonal; l if none
        if (tid == 0) s.kk = l;
        __syncthreads();
        for (int k = i - tid; k >= l + 1; k -= HQ_T) {
          zc h = Hs(k, k - 1);
          bool ok = zabs1(h) <= smlnum;
          if (!ok) {
            double tst = zabs1(Hs(k - 1, k - 1)) + zabs1(Hs(k, k));
            if (tst == 0.0) {
              if (k - 2 >= 0) tst += zabs1(Hs(k - 1, k - 2));
              if (k + 1 <= mp - 1) tst += zabs1(Hs(k + 1, k));
            }
            if (zabs1(h) <= ulp * tst) {
              const double h1 = zabs1(h), h2 = zabs1(Hs(k - 1, k));
              const double ab = fmax(h1, h2), ba = fmin(h1, h2);
              const double d1 = zabs1(Hs(k, k)), d2 = zabs1(zsub(Hs(k - 1, k - 1), Hs(k, k)));
              const double aa = fmax(d1, d2), bb = fmin(d1, d2);
              const double sm = aa + ab;
              ok = ba * (ab / sm) <= fmax(smlnum, ulp * (bb * (aa / sm)));
            }
          }
          if (ok) { atomicMax(&s.kk, k); break; }   // larger k's of this thread were tested first
        }
        __syncthreads();
        l = s.kk;
        __syncthreads();
        if (l > 0 && tid == 0) Hs(l, l - 1) = zmk(0.0, 0.0);
        if (l >= i) break;
        if (total_its >= its_cap) { st = STAB_ST_NOCONV; break; }
        ++kdefl;
        ++total_its;
        // shift
        zc t;
        if (kdefl % 20 == 0) {
          t = zadd(zmk(0.75 * zabs(Hs(i, i - 1)), 0.0), Hs(i, i));
        } else if (kdefl % 10 == 0) {
          t = zadd(zmk(0.75 * zabs(Hs(l + 1, l)), 0.0), Hs(l, l));
        } else {
          t = Hs(i, i);
          zc u = zmul(zsqrt(Hs(i - 1, i)), zsqrt(Hs(i, i - 1)));
          double su = zabs1(u);
          if (su != 0.0) {
            zc x = zscale(zsub(Hs(i - 1, i - 1), t), 0.5);
            double sx = zabs1(x);
            double sc = fmax(su, sx);
            zc xs = zscale(x, 1.0 / sc), us = zscale(u, 1.0 / sc);
            zc y = zscale(zsqrt(zadd(zmul(xs, xs), zmul(us, us))), sc);
            if (sx > 0.0) {
              zc xn = zscale(x, 1.0 / sx);
              if (xn.x * y.x + xn.y * y.y < 0.0) y = zmk(-y.x, -y.y);
            }
            t = zsub(t, zmul(u, zdiv(u, zadd(x, y))));
          }
        }
        // start row: largest m in [l+1, i-1] where two consecutive small
        // subdiagonals decouple the sweep; l otherwise
        if (tid == 0) s.kk = l;
        __syncthreads();
        for (int mm = i - 1 - tid; mm >= l + 1; mm -= HQ_T) {
          zc h11 = Hs(mm, mm), h22 = Hs(mm + 1, mm + 1);
          zc h11s = zsub(h11, t);
          zc h21 = Hs(mm + 1, mm);
          double sc = zabs1(h11s) + zabs1(h21);
          if (sc == 0.0) continue;
          h11s = zscale(h11s, 1.0 / sc);
          h21 = zscale(h21, 1.0 / sc);
          zc h10 = Hs(mm, mm - 1);
          if (zabs1(h10) * zabs1(h21) <= ulp * (zabs1(h11s) * (zabs1(h11) + zabs1(h22)))) {
            atomicMax(&s.kk, mm);
            break;
          }
        }
        __syncthreads();
        const int m0 = s.kk;
        __syncthreads();
        zc v1, v2;
        {
          zc h11s = zsub(Hs(m0, m0), t);
          zc h21 = Hs(m0 + 1, m0);
          double sc = zabs1(h11s) + zabs1(h21);
          if (sc == 0.0) sc = 1.0;
          v1 = zscale(h11s, 1.0 / sc);
          v2 = zscale(h21, 1.0 / sc);
        }
        // bulge chase
        for (int k = m0; k < i; ++k) {
          if (k > m0) { v1 = Hs(k, k - 1); v2 = Hs(k + 1, k - 1); }
          // 2-element reflector (as ZLARFG): (v1, v2) -> (beta, 0)
          zc tau = zmk(0.0, 0.0), u2 = zmk(0.0, 0.0);
          double beta = v1.x;
          bool ident = false;
          {
            double xn = zabs(v2);
            if (xn == 0.0 && v1.y == 0.0) {
              ident = true;
            } else {
              beta = -copysign(sqrt(v1.x * v1.x + v1.y * v1.y + xn * xn), v1.x);
              tau = zmk((beta - v1.x) / beta, -v1.y / beta);
              u2 = zdiv(v2, zmk(v1.x - beta, v1.y));
            }
          }
          __syncthreads();   // everyone has read the column before it changes
          const int nleft = i - k - 1;        // columns k+2..i
          const int ntask = i - l;            // 1 corner + nleft + (k - l) right rows
          if (tid == 0) flops += 24.0 * (double)(ntask + 4);   // 24 flops per 2-element pair update
          for (int q = tid; q < ntask; q += HQ_T) {
            if (q == 0) {
              if (k > m0) { Hs(k, k - 1) = zmk(ident ? v1.x : beta, ident ? v1.y : 0.0); Hs(k + 1, k - 1) = zmk(0.0, 0.0); }
              if (k == m0 && m0 > l && !ident) {
                // a sweep started below l still applies the first reflector to
                // column m0-1: H(m0, m0-1) picks up the factor (1 - conj(tau));
                // the fill-in at H(m0+1, m0-1) is what the start test bounds.
                Hs(m0, m0 - 1) = zmul(Hs(m0, m0 - 1), zsub(zmk(1.0, 0.0), zconj(tau)));
              }
              if (!ident) {
                for (int j = k; j <= k + 1; ++j) {   // left on the 2x2 corner
                  zc a = Hs(k, j), b = Hs(k + 1, j);
                  zc sm = zmul(zconj(tau), zcfma(u2, b, a));
                  Hs(k, j) = zsub(a, sm);
                  Hs(k + 1, j) = zsub(b, zmul(sm, u2));
                }
                const int rmax = (k + 2 <= i) ? k + 2 : i;
                for (int j = k; j <= rmax; ++j) {   // right on rows k..k+2
                  zc a = Hs(j, k), b = Hs(j, k + 1);
                  zc sm = zmul(tau, zfma(u2, b, a));
                  Hs(j, k) = zsub(a, sm);
                  Hs(j, k + 1) = zsub(b, zmul(sm, zconj(u2)));
                }
              }
            } else if (!ident) {
              if (q <= nleft) {
                const int j = k + 1 + q;          // column
                zc a = Hs(k, j), b = Hs(k + 1, j);
                zc sm = zmul(zconj(tau), zcfma(u2, b, a));
                Hs(k, j) = zsub(a, sm);
                Hs(k + 1, j) = zsub(b, zmul(sm, u2));
              } else {
                const int j = l + (q - nleft - 1);   // row < k
                zc a = Hs(j, k), b = Hs(j, k + 1);
                zc sm = zmul(tau, zfma(u2, b, a));
                Hs(j, k) = zsub(a, sm);
                Hs(j, k + 1) = zsub(b, zmul(sm, zconj(u2)));
              }
            }
          }
          __syncthreads();
        }
      }
      if (st) break;
      if (tid == 0) ev[i] = Hs(i, i);
      i = l - 1;
      __syncthreads();
    }
    if (st) {
      for (int q = tid; q <= i; q += HQ_T) ev[q] = zmk(nan(""), nan(""));
    }
    if (tid == 0) {
      status[inst] = st;
      if (flops_out) flops_out[inst] = flops;
    }
    __syncthreads();
  }
}

size_t eig_plain_smem(int mmax) {
  return ((2 * (size_t)mmax * sizeof(int) + 15) / 16) * 16 + 3 * (size_t)mmax * sizeof(zc);
}

cudaError_t launch_eig_plain(int count, int mmax, const int32_t* msz, zc* A, const int64_t* a_off, zc* H,
                             const int64_t* h_off, zc* eig, const int64_t* eig_off, int32_t* status,
                             int32_t* work_counter, const int32_t* order, double* flops, int grid,
                             cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  size_t sm = eig_plain_smem(mmax);
  cudaError_t e = cudaFuncSetAttribute(k_eig_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(work_counter, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  k_eig_plain<<<grid, HQ_T, sm, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter, order,
                                     flops);
  return cudaGetLastError();
}

}  // namespace stab
