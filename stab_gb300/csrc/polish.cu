// Mixed-precision polish of one eigenpair per instance (no reference
// function: the reference leaves mode selection to a human with
// getevec -v, getevec.f90:161-172, and polishing to an external shooting
// code).  The eigenproblem is written as Q(t) x = 0 with
//   temporal:  Q(w) = A0 - w B0                 (t = omega)
//   spatial:   Q(l) = l^2 C0 + l C1 + C2        (t = lambda = 1/alpha)
// Steps (host side in capi.cu):
//   a. complex64 LU of Q(s) at the seed s; two inverse-iteration steps
//      x <- Q(s)^-1 Q'(s) x give the eigenvector direction;
//   b. complex64 LU of the bordered Jacobian J = [Q(s) with column p
//      replaced by Q'(s) x], p = arg max |x_p| (x_p = 1 fixes the scale);
//   c. Newton-chord steps: r = Q(t) x in FP64 (k_qmv, O(N^2) from the
//      per-node blocks), d = J^-1 r in complex64, x_j -= d_j (j != p),
//      t -= d_p.  The FP64 residual makes the fixed point FP64-accurate; the
//      complex64 factor only sets the contraction rate.
#include "common.cuh"
#include "kernels.cuh"
#include "polish.cuh"

namespace stab {

__device__ __forceinline__ int64_t pnode_index(const InstDesc& d) { return d.off_blk / BLK_STRIDE; }

// (P1, P2, P3)[e][v] of Q(t) (deriv = 0) or Q'(t) (deriv = 1) for node block b
__device__ __forceinline__ void qblock(const InstDesc& d, const zc* b, zc t, int deriv, int q, zc& p1, zc& p2,
                                       zc& p3) {
  const zc z0 = zmk(0.0, 0.0);
  if (d.itype == 1) {
    if (!deriv) { p1 = b[q]; p2 = b[25 + q]; p3 = zsub(b[50 + q], zmul(t, b[75 + q])); }
    else { p1 = z0; p2 = z0; p3 = zmk(-b[75 + q].x, -b[75 + q].y); }
  } else {
    if (!deriv) {
      const zc t2 = zmul(t, t);
      p1 = zadd(zmul(t2, b[q]), zmul(t, b[75 + q]));
      p2 = zmul(t2, b[25 + q]);
      p3 = zadd(zadd(zmul(t2, b[50 + q]), zmul(t, b[100 + q])), b[125 + q]);
    } else {
      const zc tt = zscale(t, 2.0);
      p1 = zadd(zmul(tt, b[q]), b[75 + q]);
      p2 = zmul(tt, b[25 + q]);
      p3 = zadd(zmul(tt, b[50 + q]), b[100 + q]);
    }
  }
}

// y = Q(t) x or Q'(t) x, FP64, one CTA per instance
__global__ void k_qmv(int count, const InstDesc* __restrict__ desc, const double* const* __restrict__ dtab,
                      const zc* __restrict__ blk, const zc* __restrict__ theta, int deriv, zc* __restrict__ vec,
                      int xslot, int yslot, const int32_t* __restrict__ skip) {
  extern __shared__ zc qsm[];
  const int k = blockIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int n = d.n, ny = d.ny;
  const double* D1 = dtab[2 * d.dmat];
  const double* D2 = dtab[2 * d.dmat + 1];
  const zc* bb = blk + d.off_blk;
  const zc* xv = vec + d.off_vec + (int64_t)xslot * n;
  zc* yv = vec + d.off_vec + (int64_t)yslot * n;
  const zc t = theta[k];
  zc* xs = qsm;
  zc* w1 = qsm + n;
  zc* w2 = qsm + 2 * n;
  for (int q = threadIdx.x; q < n; q += blockDim.x) xs[q] = xv[q];
  __syncthreads();
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int i = q / 5, v = q % 5;
    zc s1 = zmk(0.0, 0.0), s2 = zmk(0.0, 0.0);
    const double* r1 = D1 + (size_t)i * ny;
    const double* r2 = D2 + (size_t)i * ny;
    for (int j = 0; j < ny; ++j) {
      const zc xj = xs[j * 5 + v];
      const double a = r1[j], b = r2[j];
      s1.x = fma(a, xj.x, s1.x); s1.y = fma(a, xj.y, s1.y);
      s2.x = fma(b, xj.x, s2.x); s2.y = fma(b, xj.y, s2.y);
    }
    w1[q] = s1;
    w2[q] = s2;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int i = q / 5, e = q % 5;
    const zc* b = bb + (size_t)BLK_STRIDE * i;
    zc acc = zmk(0.0, 0.0);
    for (int v = 0; v < 5; ++v) {
      zc p1, p2, p3;
      qblock(d, b, t, deriv, e * 5 + v, p1, p2, p3);
      acc = zfma(p1, w1[i * 5 + v], acc);
      acc = zsub(acc, zmul(p2, w2[i * 5 + v]));
      acc = zfma(p3, xs[i * 5 + v], acc);
    }
    yv[q] = acc;
  }
}

// deterministic start vector (hash of the index), so it is not orthogonal to
// the wanted eigenvector by accident
__global__ void k_vec_init(int count, const InstDesc* __restrict__ desc, zc* __restrict__ vec, int slot,
                           const int32_t* __restrict__ skip) {
  const int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.n) return;
  uint32_t h = (uint32_t)q * 2654435761u + 0x9e3779b9u;
  h ^= h >> 15; h *= 0x85ebca6bu; h ^= h >> 13;
  const double a = (double)(h & 0xffff) / 65536.0, b = (double)((h >> 16) & 0xffff) / 65536.0;
  vec[d.off_vec + (int64_t)slot * d.n + q] = zmk(1.0 + a, b - 0.5);
}

// Start vector from Chebyshev coefficients of the five fields (a surrogate's
// prediction): x(node i, field e) = sum_{q < ncheb} c[e][q] T_q(eta_i) with
// eta_i = cos(pi i / (ny - 1)), so T_q(eta_i) = cos(q pi i / (ny - 1)).
// coef: ncheb * 5 complex values per instance (field-major), internal order.
__global__ void k_cheb_start(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ coef, int ncheb,
                             zc* __restrict__ vec, int slot, const int32_t* __restrict__ skip) {
  const int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.n) return;
  const int i = q / 5, e = q % 5;
  const zc* c = coef + ((int64_t)k * 5 + e) * ncheb;
  const double th = 3.14159265358979323846 * (double)i / (double)(d.ny - 1);
  zc s = zmk(0.0, 0.0);
  for (int t = 0; t < ncheb; ++t) {
    const double w = cos((double)t * th);
    s = zmk(s.x + w * c[t].x, s.y + w * c[t].y);
  }
  vec[d.off_vec + (int64_t)slot * d.n + q] = s;
}

// Chebyshev coefficients of vector slot 0 of a batch whose instances all
// have ny = M (the coarse level's eigenvectors): per instance and field
// c_q = 2/(M-1) w_q sum_i w_i x(i) cos(pi q i/(M-1)), w_0 = w_{M-1} = 1/2,
// so that sum_q c_q cos(q theta) interpolates x at the Gauss-Lobatto points
// and k_cheb_start evaluates it at the nodes of another N.
__global__ void k_cheb_coeffs(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ vec,
                              zc* __restrict__ coef, int M) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const InstDesc d = desc[k];
  const zc* x = vec + d.off_vec;
  const double pi = 3.14159265358979323846;
  for (int t = threadIdx.x; t < 5 * M; t += blockDim.x) {
    const int e = t / M, q = t % M;
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < M; ++i) {
      const double w = ((i == 0 || i == M - 1) ? 0.5 : 1.0) * cos(pi * (double)q * (double)i / (double)(M - 1));
      const zc v = x[5 * i + e];
      sr = fma(w, v.x, sr);
      si = fma(w, v.y, si);
    }
    const double f = (2.0 / (double)(M - 1)) * ((q == 0 || q == M - 1) ? 0.5 : 1.0);
    coef[((int64_t)k * 5 + e) * M + q] = zmk(f * sr, f * si);
  }
}

cudaError_t launch_cheb_coeffs(int count, const InstDesc* desc, const zc* vec, zc* coef, int M, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_cheb_coeffs<<<count, 128, 0, s>>>(count, desc, vec, coef, M);
  return cudaGetLastError();
}

// x <- x / x_p with p = first index of max |x|; writes p to piv_out when non-null
__global__ void k_normalize(int count, const InstDesc* __restrict__ desc, zc* __restrict__ vec, int slot,
                            int32_t* __restrict__ piv_out, const int32_t* __restrict__ skip) {
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ int s_p;
  const int k = blockIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  zc* x = vec + d.off_vec + (int64_t)slot * d.n;
  double best = -1.0;
  int idx = 0x7fffffff;
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) {
    double a = zabs(x[q]);
    if (a > best || (a == best && q < idx)) { best = a; idx = q; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ob = __shfl_down_sync(0xffffffffu, best, o);
    int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { bv[warp] = best; bi[warp] = idx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (bv[w] > best || (bv[w] == best && bi[w] < idx)) { best = bv[w]; idx = bi[w]; }
    if (idx < 0 || idx >= d.n) idx = 0;   // no finite entry
    s_p = idx;
    if (piv_out) piv_out[k] = idx;
  }
  __syncthreads();
  const zc sc = x[s_p];
  __syncthreads();
  if (sc.x == 0.0 && sc.y == 0.0) return;
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) x[q] = zdiv(x[q], sc);
}

// column p of the factor matrix <- vector slot (the bordered Jacobian)
template <typename T>
__global__ void k_set_column(int count, const InstDesc* __restrict__ desc, T* __restrict__ M,
                             const int64_t* __restrict__ m_off, const int32_t* __restrict__ pcol,
                             const zc* __restrict__ vec, int slot, const int32_t* __restrict__ skip) {
  const int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.n) return;
  const zc a = vec[d.off_vec + (int64_t)slot * d.n + q];
  M[m_off[k] + (int64_t)pcol[k] * d.n + q] = cx<T>::from(a);
}

// copy slot a -> slot b
__global__ void k_vec_copy(int count, const InstDesc* __restrict__ desc, zc* __restrict__ vec, int a, int b,
                           const int32_t* __restrict__ skip) {
  const int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.n) return;
  vec[d.off_vec + (int64_t)b * d.n + q] = vec[d.off_vec + (int64_t)a * d.n + q];
}

// Newton-chord update from the correction d (slot dslot):
// x_j -= d_j (j != p), t -= d_p; converged when |d_p| <= tol |t| and
// max_j |d_j| <= tol_vec max_j |x_j|.
__global__ void k_newton_update(int count, const InstDesc* __restrict__ desc, zc* __restrict__ vec, int xslot,
                                int dslot, const int32_t* __restrict__ pcol, zc* __restrict__ theta,
                                int32_t* __restrict__ done, double* __restrict__ err, int32_t* __restrict__ iters,
                                double tol, double tol_vec, const int32_t* __restrict__ skip) {
  __shared__ double red[64];
  const int k = blockIdx.x;
  if (k >= count) return;
  if (done[k] || (skip && skip[k])) return;
  const InstDesc d = desc[k];
  zc* x = vec + d.off_vec + (int64_t)xslot * d.n;
  const zc* dd = vec + d.off_vec + (int64_t)dslot * d.n;
  const int p = pcol[k];
  double dmax = 0.0, xmax = 0.0;
  bool bad = false;
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) {
    if (q == p) continue;
    zc a = dd[q];
    if (!isfinite(a.x) || !isfinite(a.y)) bad = true;
    zc nx = zsub(x[q], a);
    x[q] = nx;
    dmax = fmax(dmax, zabs(a));
    xmax = fmax(xmax, zabs(nx));
  }
  for (int o = 16; o > 0; o >>= 1) {
    dmax = fmax(dmax, __shfl_down_sync(0xffffffffu, dmax, o));
    xmax = fmax(xmax, __shfl_down_sync(0xffffffffu, xmax, o));
  }
  const int anybad = __syncthreads_or(bad);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { red[warp] = dmax; red[32 + warp] = xmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { dmax = fmax(dmax, red[w]); xmax = fmax(xmax, red[32 + w]); }
    xmax = fmax(xmax, 1.0);   // x_p = 1
    const zc dp = dd[p];
    const zc t = zsub(theta[k], dp);
    theta[k] = t;
    const double rel = zabs(dp) / fmax(zabs(t), 1e-300);
    err[k] = rel;
    iters[k] += 1;
    if (anybad || !isfinite(t.x) || !isfinite(t.y)) done[k] = 3;           // NaN
    else if (rel <= tol && dmax <= tol_vec * xmax) done[k] = 1;             // converged
  }
}

// theta <- sigma for the instances that run
__global__ void k_start_shift(int count, const zc* __restrict__ sigma, zc* __restrict__ theta,
                              const int32_t* __restrict__ skip) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  theta[k] = sigma[k];
}

// start of a polish round: done = iters = 0 for the instances that run and
// done = 4 for the skipped ones; counts the factorisations per instance when
// `lus` is non-null
__global__ void k_reset_polish(int count, int32_t* __restrict__ done, int32_t* __restrict__ iters,
                               const int32_t* __restrict__ skip, int32_t* __restrict__ lus, int nlu) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) {
    done[k] = 4;   // not run in this candidate round: its later steps pass over it
    return;
  }
  done[k] = 0;
  iters[k] = 0;
  if (lus) lus[k] += nlu;
}

// One step of fixed-shift inverse iteration for the complex128 retry: with
// x_p = 1 and y = Q(s)^-1 Q'(s) x, the eigenvalue nearest s is
// t = s - x_p / y_p (exact for the linear temporal pencil, to O((s - t)^2)
// for the quadratic spatial one); x <- y / y_q with q = arg max |y_q|.
// Converged when successive t agree to tol (relative).
__global__ void k_ii_update(int count, const InstDesc* __restrict__ desc, zc* __restrict__ vec, int xslot, int yslot,
                            int32_t* __restrict__ pcol, const zc* __restrict__ sigma, zc* __restrict__ theta,
                            int32_t* __restrict__ done, double* __restrict__ err, int32_t* __restrict__ iters,
                            double tol, const int32_t* __restrict__ skip) {
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ int s_q;
  __shared__ zc s_yq;
  const int k = blockIdx.x;
  if (k >= count) return;
  if (done[k] || (skip && skip[k])) return;
  const InstDesc d = desc[k];
  zc* x = vec + d.off_vec + (int64_t)xslot * d.n;
  const zc* y = vec + d.off_vec + (int64_t)yslot * d.n;
  double best = -1.0;
  int idx = 0x7fffffff;
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) {
    const double a = zabs(y[q]);
    if (a > best || (a == best && q < idx)) { best = a; idx = q; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_down_sync(0xffffffffu, best, o);
    const int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { bv[warp] = best; bi[warp] = idx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (bv[w] > best || (bv[w] == best && bi[w] < idx)) { best = bv[w]; idx = bi[w]; }
    if (idx < 0 || idx >= d.n) idx = 0;
    const int p = pcol[k];
    const zc yp = y[p];
    const zc told = theta[k];
    const zc t = zsub(sigma[k], zdiv(x[p], yp));
    theta[k] = t;
    const double rel = zabs(zsub(t, told)) / fmax(zabs(t), 1e-300);
    err[k] = rel;
    iters[k] += 1;
    if (!isfinite(t.x) || !isfinite(t.y)) done[k] = 3;
    else if (iters[k] >= 2 && rel <= tol) done[k] = 1;
    pcol[k] = idx;
    s_q = idx;
    s_yq = y[idx];
  }
  __syncthreads();
  const zc yq = s_yq;
  if (yq.x == 0.0 && yq.y == 0.0) return;
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) x[q] = zdiv(y[q], yq);
}

// ---- host launchers --------------------------------------------------------
cudaError_t launch_qmv(int count, int nmax, const InstDesc* desc, const double* const* dtab, const zc* blk,
                       const zc* theta, int deriv, zc* vec, int xslot, int yslot, const int32_t* skip,
                       cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  size_t sm = 3 * (size_t)nmax * sizeof(zc);
  cudaError_t e = cudaFuncSetAttribute(k_qmv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_qmv<<<count, 256, sm, s>>>(count, desc, dtab, blk, theta, deriv, vec, xslot, yslot, skip);
  return cudaGetLastError();
}

cudaError_t launch_vec_init(int count, int nmax, const InstDesc* desc, zc* vec, int slot, cudaStream_t s,
                            const int32_t* skip) {
  if (count <= 0) return cudaSuccess;
  dim3 g((nmax + 255) / 256, count);
  k_vec_init<<<g, 256, 0, s>>>(count, desc, vec, slot, skip);
  return cudaGetLastError();
}

cudaError_t launch_normalize(int count, const InstDesc* desc, zc* vec, int slot, int32_t* piv_out,
                             const int32_t* skip, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_normalize<<<count, 256, 0, s>>>(count, desc, vec, slot, piv_out, skip);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_set_column(int count, int nmax, const InstDesc* desc, T* M, const int64_t* m_off,
                              const int32_t* pcol, const zc* vec, int slot, cudaStream_t s, const int32_t* skip) {
  if (count <= 0) return cudaSuccess;
  dim3 g((nmax + 255) / 256, count);
  k_set_column<T><<<g, 256, 0, s>>>(count, desc, M, m_off, pcol, vec, slot, skip);
  return cudaGetLastError();
}
template cudaError_t launch_set_column<cc>(int, int, const InstDesc*, cc*, const int64_t*, const int32_t*, const zc*,
                                           int, cudaStream_t, const int32_t*);
template cudaError_t launch_set_column<zc>(int, int, const InstDesc*, zc*, const int64_t*, const int32_t*, const zc*,
                                           int, cudaStream_t, const int32_t*);

cudaError_t launch_vec_copy(int count, int nmax, const InstDesc* desc, zc* vec, int a, int b, const int32_t* skip,
                            cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  dim3 g((nmax + 255) / 256, count);
  k_vec_copy<<<g, 256, 0, s>>>(count, desc, vec, a, b, skip);
  return cudaGetLastError();
}

cudaError_t launch_newton_update(int count, const InstDesc* desc, zc* vec, int xslot, int dslot, const int32_t* pcol,
                                 zc* theta, int32_t* done, double* err, int32_t* iters, double tol, double tol_vec,
                                 cudaStream_t s, const int32_t* skip) {
  if (count <= 0) return cudaSuccess;
  k_newton_update<<<count, 256, 0, s>>>(count, desc, vec, xslot, dslot, pcol, theta, done, err, iters, tol, tol_vec,
                                        skip);
  return cudaGetLastError();
}

cudaError_t launch_start_shift(int count, const zc* sigma, zc* theta, const int32_t* skip, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_start_shift<<<(count + 255) / 256, 256, 0, s>>>(count, sigma, theta, skip);
  return cudaGetLastError();
}

cudaError_t launch_reset_polish(int count, int32_t* done, int32_t* iters, const int32_t* skip, cudaStream_t s,
                                int32_t* lus, int nlu) {
  if (count <= 0) return cudaSuccess;
  k_reset_polish<<<(count + 255) / 256, 256, 0, s>>>(count, done, iters, skip, lus, nlu);
  return cudaGetLastError();
}

cudaError_t launch_cheb_start(int count, int nmax, const InstDesc* desc, const zc* coef, int ncheb, zc* vec,
                              int slot, const int32_t* skip, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  dim3 g((nmax + 127) / 128, count);
  k_cheb_start<<<g, 128, 0, s>>>(count, desc, coef, ncheb, vec, slot, skip);
  return cudaGetLastError();
}

cudaError_t launch_ii_update(int count, const InstDesc* desc, zc* vec, int xslot, int yslot, int32_t* pcol,
                             const zc* sigma, zc* theta, int32_t* done, double* err, int32_t* iters, double tol,
                             const int32_t* skip, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_ii_update<<<count, 256, 0, s>>>(count, desc, vec, xslot, yslot, pcol, sigma, theta, done, err, iters, tol, skip);
  return cudaGetLastError();
}

}  // namespace stab
