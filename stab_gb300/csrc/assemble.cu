// Operator combination, dense assembly and the structured operator product.
//
// Every operator of the path has row block i equal to
//   P1 (x) D1(i,:) - P2 (x) D2(i,:) + delta_ij P3
// (temporal.f90:664-752 for A0, :622-662 for B0; spatial.f90:687-959 for
// C0, C1, C2).  k_node_ops forms (P1, P2, P3) of the operator a step needs
// (A0 - s B0, B0^-1 A0, s^2 C0 + s C1 + C2, ...), k_dense writes the dense
// column-major matrix in complex128 or complex64, and k_opmv applies the
// operator in O(N^2) without forming it (used for the FP64 residuals).
#include <algorithm>

#include "common.cuh"
#include "dw.cuh"
#include "kernels.cuh"

namespace stab {

__device__ __forceinline__ int64_t node_index(const InstDesc& d) { return d.off_blk / BLK_STRIDE; }

__global__ void k_node_ops(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ blk, int kind_t,
                           int kind_s, const zc* __restrict__ sigma, zc* __restrict__ ops, cc* __restrict__ ops32,
                           const int32_t* __restrict__ skip) {
  int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int kind = (d.itype == 1) ? kind_t : kind_s;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ny) return;
  const zc* b = blk + d.off_blk + (size_t)BLK_STRIDE * i;
  zc* o = ops + (node_index(d) + i) * 75;
  const zc z0 = zmk(0.0, 0.0);
  const zc s = sigma ? sigma[k] : z0;
  const zc s2 = zmul(s, s);
  const zc two_s = zscale(s, 2.0);
  for (int q = 0; q < 25; ++q) {
    zc p1 = z0, p2 = z0, p3 = z0;
    switch (kind) {
      case OP_T_A0: p1 = b[q]; p2 = b[25 + q]; p3 = b[50 + q]; break;
      case OP_T_B0: p3 = b[75 + q]; break;
      case OP_T_C: {
        const int e = q / 5, v = q % 5;
        for (int t = 0; t < 5; ++t) {
          const zc bi = b[100 + e * 5 + t];
          p1 = zfma(bi, b[t * 5 + v], p1);
          p2 = zfma(bi, b[25 + t * 5 + v], p2);
          p3 = zfma(bi, b[50 + t * 5 + v], p3);
        }
        break;
      }
      case OP_T_Q: p1 = b[q]; p2 = b[25 + q]; p3 = zsub(b[50 + q], zmul(s, b[75 + q])); break;
      case OP_T_DQ: p3 = zmk(-b[75 + q].x, -b[75 + q].y); break;
      case OP_S_C0: p1 = b[q]; p2 = b[25 + q]; p3 = b[50 + q]; break;
      case OP_S_C1: p1 = b[75 + q]; p3 = b[100 + q]; break;
      case OP_S_C2: p3 = b[125 + q]; break;
      case OP_S_Q:
        p1 = zadd(zmul(s2, b[q]), zmul(s, b[75 + q]));
        p2 = zmul(s2, b[25 + q]);
        p3 = zadd(zadd(zmul(s2, b[50 + q]), zmul(s, b[100 + q])), b[125 + q]);
        break;
      case OP_S_DQ:
        p1 = zadd(zmul(two_s, b[q]), b[75 + q]);
        p2 = zmul(two_s, b[25 + q]);
        p3 = zadd(zmul(two_s, b[50 + q]), b[100 + q]);
        break;
      default: break;
    }
    o[q] = p1;
    o[25 + q] = p2;
    o[50 + q] = p3;
    if (ops32) {   // rounded copy for the complex64 assembly
      cc* o32 = ops32 + (node_index(d) + i) * 75;
      o32[q] = cmk((float)p1.x, (float)p1.y);
      o32[25 + q] = cmk((float)p2.x, (float)p2.y);
      o32[50 + q] = cmk((float)p3.x, (float)p3.y);
    }
  }
}

template <typename T> __device__ __forceinline__ T store_cast(zc v);
template <> __device__ __forceinline__ zc store_cast<zc>(zc v) { return v; }
template <> __device__ __forceinline__ cc store_cast<cc>(zc v) { return cmk((float)v.x, (float)v.y); }
template <> __device__ __forceinline__ dz store_cast<dz>(zc v) { return dz_from64(v); }

// Dense column-major n x n.  Grid (ceil(n / 8), count); 256 threads walk the
// rows of 8 consecutive columns, so each warp writes contiguous addresses.
template <typename T>
__global__ void k_dense(int count, const InstDesc* __restrict__ desc, const double* const* __restrict__ dtab,
                        const zc* __restrict__ ops, T* __restrict__ out, const int64_t* __restrict__ out_off,
                        int ldmul, double scale, const int32_t* __restrict__ skip) {
  int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int n = d.n, ny = d.ny;
  const int c0 = blockIdx.x * 8;
  if (c0 >= n) return;
  const double* D1 = dtab[2 * d.dmat];
  const double* D2 = dtab[2 * d.dmat + 1];
  const zc* o = ops + node_index(d) * 75;
  T* M = out + out_off[k];
  const int64_t ld = (int64_t)ldmul * n;
  for (int cc_ = 0; cc_ < 8; ++cc_) {
    const int c = c0 + cc_;
    if (c >= n) break;
    const int j = c / 5, v = c % 5;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
      const int i = r / 5, e = r % 5;
      const zc* oi = o + (size_t)i * 75;
      const double d1 = D1[(size_t)i * ny + j], d2 = D2[(size_t)i * ny + j];
      const zc p1 = oi[e * 5 + v], p2 = oi[25 + e * 5 + v];
      zc val = zmk(p1.x * d1 - p2.x * d2, p1.y * d1 - p2.y * d2);
      if (i == j) val = zadd(val, oi[50 + e * 5 + v]);
      M[(size_t)c * ld + r] = store_cast<T>(zscale(val, scale));
    }
  }
}

// The complex64 assembly in FP32 arithmetic, from the rounded node blocks
// and D tables: each entry is fl32(p1 d1 - p2 d2 (+ p3)) * scale, within a
// few float roundings of the FP64 expression rounded to float.  The matrix
// only feeds a complex64 factorisation whose Newton-chord steps form their
// residuals in FP64, and FP64 arithmetic here (1/64 of the FP32 rate on this
// GPU) made the assembly bound by the FP64 pipe.  Same grid and write order
// as k_dense.
__global__ void k_dense32(int count, const InstDesc* __restrict__ desc, const float* const* __restrict__ dtab32,
                          const cc* __restrict__ ops32, cc* __restrict__ out, const int64_t* __restrict__ out_off,
                          int ldmul, float scale, const int32_t* __restrict__ skip) {
  int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  const int n = d.n, ny = d.ny;
  const int c0 = blockIdx.x * 8;
  if (c0 >= n) return;
  const float* D1 = dtab32[2 * d.dmat];
  const float* D2 = dtab32[2 * d.dmat + 1];
  const cc* o = ops32 + node_index(d) * 75;
  cc* M = out + out_off[k];
  const int64_t ld = (int64_t)ldmul * n;
  for (int cc_ = 0; cc_ < 8; ++cc_) {
    const int c = c0 + cc_;
    if (c >= n) break;
    const int j = c / 5, v = c % 5;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
      const int i = r / 5, e = r % 5;
      const cc* oi = o + (size_t)i * 75;
      const float d1 = D1[(size_t)i * ny + j], d2 = D2[(size_t)i * ny + j];
      const cc p1 = oi[e * 5 + v], p2 = oi[25 + e * 5 + v];
      float vr = fmaf(p1.x, d1, -p2.x * d2), vi = fmaf(p1.y, d1, -p2.y * d2);
      if (i == j) {
        const cc p3 = oi[50 + e * 5 + v];
        vr += p3.x;
        vi += p3.y;
      }
      M[(size_t)c * ld + r] = cmk(vr * scale, vi * scale);
    }
  }
}

cudaError_t launch_dense32(int count, int nmax, const InstDesc* desc, const float* const* dtab32, const cc* ops32,
                           cc* out, const int64_t* out_off, int ldmul, float scale, cudaStream_t s,
                           const int32_t* skip) {
  if (count <= 0) return cudaSuccess;
  dim3 g((nmax + 7) / 8, count);
  k_dense32<<<g, 256, 0, s>>>(count, desc, dtab32, ops32, out, out_off, ldmul, scale, skip);
  return cudaGetLastError();
}

__global__ void k_round_f32(int64_t count, const double* __restrict__ x, float* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

cudaError_t launch_round_f32(int64_t count, const double* x, float* y, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_round_f32<<<(unsigned)std::min<int64_t>(1024, (count + 255) / 256), 256, 0, s>>>(count, x, y);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_dense(int count, int nmax, const InstDesc* desc, const double* const* dtab, const zc* ops, T* out,
                         const int64_t* out_off, int ldmul, double scale, cudaStream_t s, const int32_t* skip) {
  if (count <= 0) return cudaSuccess;
  dim3 g((nmax + 7) / 8, count);
  k_dense<T><<<g, 256, 0, s>>>(count, desc, dtab, ops, out, out_off, ldmul, scale, skip);
  return cudaGetLastError();
}
template cudaError_t launch_dense<zc>(int, int, const InstDesc*, const double* const*, const zc*, zc*,
                                      const int64_t*, int, double, cudaStream_t, const int32_t*);
template cudaError_t launch_dense<cc>(int, int, const InstDesc*, const double* const*, const zc*, cc*,
                                      const int64_t*, int, double, cudaStream_t, const int32_t*);
template cudaError_t launch_dense<dz>(int, int, const InstDesc*, const double* const*, const zc*, dz*,
                                      const int64_t*, int, double, cudaStream_t, const int32_t*);

// Structured product y = M x (FP64).  One CTA per instance: x staged in
// shared memory, W1 = D1 X and W2 = D2 X formed per (node, variable), then
// the 5x5 blocks applied per (node, equation).  O(10 N^2) complex-real FMAs
// instead of the 25 N^2 complex FMAs of a dense product.
__global__ void k_opmv(int count, const InstDesc* __restrict__ desc, const double* const* __restrict__ dtab,
                       const zc* __restrict__ ops, const zc* __restrict__ x, int xslot, zc* __restrict__ y,
                       int yslot) {
  extern __shared__ zc sm[];
  int k = blockIdx.x;
  if (k >= count) return;
  const InstDesc d = desc[k];
  const int n = d.n, ny = d.ny;
  const double* D1 = dtab[2 * d.dmat];
  const double* D2 = dtab[2 * d.dmat + 1];
  const zc* o = ops + node_index(d) * 75;
  const zc* xv = x + d.off_vec + (int64_t)xslot * n;
  zc* yv = y + d.off_vec + (int64_t)yslot * n;
  zc* xs = sm;           // n
  zc* w1 = sm + n;       // n
  zc* w2 = sm + 2 * n;   // n
  for (int t = threadIdx.x; t < n; t += blockDim.x) xs[t] = xv[t];
  __syncthreads();
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = t / 5, v = t % 5;
    zc s1 = zmk(0.0, 0.0), s2 = zmk(0.0, 0.0);
    for (int j = 0; j < ny; ++j) {
      const double a = D1[(size_t)i * ny + j], b = D2[(size_t)i * ny + j];
      const zc xj = xs[j * 5 + v];
      s1.x = fma(a, xj.x, s1.x); s1.y = fma(a, xj.y, s1.y);
      s2.x = fma(b, xj.x, s2.x); s2.y = fma(b, xj.y, s2.y);
    }
    w1[t] = s1;
    w2[t] = s2;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = t / 5, e = t % 5;
    const zc* oi = o + (size_t)i * 75;
    zc acc = zmk(0.0, 0.0);
    for (int v = 0; v < 5; ++v) {
      acc = zfma(oi[e * 5 + v], w1[i * 5 + v], acc);
      const zc p2 = oi[25 + e * 5 + v];
      acc = zsub(acc, zmul(p2, w2[i * 5 + v]));
      acc = zfma(oi[50 + e * 5 + v], xs[i * 5 + v], acc);
    }
    yv[t] = acc;
  }
}

}  // namespace stab
