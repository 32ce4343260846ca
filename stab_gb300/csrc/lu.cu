// Batched dense complex LU with partial pivoting and triangular solves.
//
// Replaces ZGETRF (spatial.f90:978), ZGETRS (spatial.f90:996,1002) and the
// factorisation inside ZGESV (temporal.f90:774); complex64 and double-word
// (dw.cuh) instances of the same kernels factor A - s B for the
// mixed-precision polish.
//
// Layout: column-major n x n per instance at pool offset mat_off[k].  One
// CTA per instance (n <= 960 here).  Blocked right-looking algorithm:
//   1. the panel A[k0:n, k0:k0+w] is copied to shared memory and factored
//      there (pivot search = block arg-max of |re|+|im|, first index wins,
//      as IZAMAX);
//   2. the panel's row swaps are applied to the other columns;
//   3. U12 = L11^-1 A12 (forward substitution, one thread per column);
//   4. A22 -= L21 U12 as a 64x64-tiled GEMM with L21 read from shared memory
//      and each thread holding a 4x4 block of complex accumulators.
#include <cooperative_groups.h>

#include "common.cuh"
#include "dw.cuh"
#include "kernels.cuh"
#include "lu.cuh"

namespace cg = cooperative_groups;

namespace stab {

#include "lu_body.cuh"

template <typename T, int NB, int CL>
__global__ void __launch_bounds__(256) k_lu(int count, const InstDesc* __restrict__ desc, const int32_t* __restrict__ nsz,
                                            T* __restrict__ A, const int64_t* __restrict__ mat_off,
                                            int32_t* __restrict__ piv, const int64_t* __restrict__ piv_off,
                                            int32_t* __restrict__ info, const int32_t* __restrict__ skip,
                                            const int32_t* __restrict__ order) {
  typedef typename cx<T>::real R;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ R red_v[256 / 32];
  __shared__ int red_i[256 / 32];
  __shared__ int s_piv;
  const int rank = (CL > 1) ? (int)(cg::this_cluster().block_rank()) : 0;
  // CTAs start in block order: with `order` largest first, the last wave
  // holds the small factorisations
  const int slot = (int)blockIdx.x / CL;
  const int k = order ? order[slot] : slot;
  if (k >= count) return;
  if (skip && skip[k]) return;
  lu_body<T, NB, CL>(k, rank, nsz, A, mat_off, piv, piv_off, info, smraw, red_v, red_i, s_piv);
}

// Power-of-two row and column equilibration of complex64 matrices before the
// LU: M <- R M C with R, C diagonal powers of two (exact in floating point),
// chosen so every row and then every column has max |re|+|im| in [0.5, 1).
// This keeps pivoting and the complex64 rounding meaningful when the
// operator's rows differ by many orders of magnitude (e.g. the 1/(gamma M^2)
// pressure terms at low Mach number).  R and C are stored per instance.
__global__ void __launch_bounds__(256) k_equilibrate(int count, const int32_t* __restrict__ nsz, cc* __restrict__ A,
                                                     const int64_t* __restrict__ mat_off, float* __restrict__ rs,
                                                     float* __restrict__ cs, const int64_t* __restrict__ sc_off,
                                                     const int32_t* __restrict__ skip) {
  const int k = blockIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const int n = nsz[k];
  cc* M = A + mat_off[k];
  float* R = rs + sc_off[k];
  float* C = cs + sc_off[k];
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    float mx = 0.f;
    for (int c = 0; c < n; ++c) mx = fmaxf(mx, cabs1f(M[(size_t)c * n + r]));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    R[r] = ldexpf(1.f, -e);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = warp; c < n; c += nw) {
    float mx = 0.f;
    cc* col = M + (size_t)c * n;
    for (int r = lane; r < n; r += 32) {
      cc v = col[r];
      const float f = R[r];
      v.x *= f; v.y *= f;
      col[r] = v;
      mx = fmaxf(mx, cabs1f(v));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    const float g = ldexpf(1.f, -e);
    for (int r = lane; r < n; r += 32) {
      cc v = col[r];
      v.x *= g; v.y *= g;
      col[r] = v;
    }
    if (lane == 0) C[c] = g;
  }
}

cudaError_t launch_equilibrate(int count, const int32_t* nsz, cc* A, const int64_t* mat_off, float* rs, float* cs,
                               const int64_t* sc_off, cudaStream_t s, const int32_t* skip) {
  if (count <= 0) return cudaSuccess;
  k_equilibrate<<<count, 256, 0, s>>>(count, nsz, A, mat_off, rs, cs, sc_off, skip);
  return cudaGetLastError();
}

// Triangular solves with the factors of k_lu: X <- U^-1 L^-1 P X for nrhs
// columns per instance.  One warp per right-hand side, the column held in
// shared memory; the factor columns are read coalesced from global memory.
// Right-hand sides are complex128 in memory and solved in the factor's type.
template <typename T>
__global__ void __launch_bounds__(256) k_getrs(int count, const int32_t* __restrict__ nsz, const T* __restrict__ LU,
                                               const int64_t* __restrict__ mat_off, const int32_t* __restrict__ piv,
                                               const int64_t* __restrict__ piv_off, zc* __restrict__ X,
                                               const int64_t* __restrict__ x_off, int nrhs_fixed, int nrhs_mul,
                                               int ldmul, const int32_t* __restrict__ skip, const float* __restrict__ rs,
                                               const float* __restrict__ cs) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const int n = nsz[k];
  const int nrhs = nrhs_fixed > 0 ? nrhs_fixed : nrhs_mul * n;
  const int64_t ldx = (int64_t)ldmul * n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = blockIdx.x * (blockDim.x >> 5) + warp;
  if (col >= nrhs) return;
  T* xs = reinterpret_cast<T*>(smraw) + (size_t)warp * n;
  const T* M = LU + mat_off[k];
  const int32_t* ip = piv + piv_off[k];
  zc* xg = X + x_off[k] + (size_t)col * ldx;
  const float* R = rs ? rs + piv_off[k] : nullptr;   // equilibration (k_equilibrate), same offsets as pivots
  const float* C = cs ? cs + piv_off[k] : nullptr;
  for (int r = lane; r < n; r += 32) {
    zc b = xg[r];
    if (R) b = zscale(b, (double)R[r]);
    xs[r] = cx<T>::from(b);
  }
  __syncwarp();
  if (lane == 0)
    for (int j = 0; j < n; ++j) {
      const int p = ip[j];
      if (p != j) { T t = xs[j]; xs[j] = xs[p]; xs[p] = t; }
    }
  __syncwarp();
  for (int j = 0; j < n; ++j) {       // L y = b (unit diagonal)
    const T xj = xs[j];
    for (int r = j + 1 + lane; r < n; r += 32) xs[r] = cx<T>::fnma(M[(size_t)j * n + r], xj, xs[r]);
    __syncwarp();
  }
  for (int j = n - 1; j >= 0; --j) {  // U x = y
    T d = M[(size_t)j * n + j];
    T xj = xs[j];
    if (cx<T>::abs1(d) != 0) xj = cx<T>::div(xj, d);
    __syncwarp();
    if (lane == 0) xs[j] = xj;
    for (int r = lane; r < j; r += 32) xs[r] = cx<T>::fnma(M[(size_t)j * n + r], xj, xs[r]);
    __syncwarp();
  }
  for (int r = lane; r < n; r += 32) {
    zc y = cx<T>::to64(xs[r]);
    xg[r] = C ? zscale(y, (double)C[r]) : y;
  }
}

__device__ __forceinline__ zc shfl_cx(zc v, int src) {
  return zmk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ cc shfl_cx(cc v, int src) {
  return cmk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ dz shfl_cx(dz v, int src) {
  return make_float4(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                     __shfl_sync(0xffffffffu, v.z, src), __shfl_sync(0xffffffffu, v.w, src));
}

// The same solve for few right-hand sides: one CTA per (instance, column),
// blocked by 32 columns.  Warp 0 solves each 32 x 32 diagonal block from
// shared memory (one row per lane, shuffles broadcast the solved entry) and
// then all warps update the remaining rows with the block's 32 columns, so
// the O(n^2) work runs on every SM sub-partition instead of one warp's.
template <typename T>
__global__ void __launch_bounds__(256) k_getrs_blk(int count, const int32_t* __restrict__ nsz,
                                                   const T* __restrict__ LU, const int64_t* __restrict__ mat_off,
                                                   const int32_t* __restrict__ piv, const int64_t* __restrict__ piv_off,
                                                   zc* __restrict__ X, const int64_t* __restrict__ x_off,
                                                   int nrhs_fixed, int nrhs_mul, int ldmul,
                                                   const int32_t* __restrict__ skip, const float* __restrict__ rs,
                                                   const float* __restrict__ cs) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int k = blockIdx.y;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const int n = nsz[k];
  const int nrhs = nrhs_fixed > 0 ? nrhs_fixed : nrhs_mul * n;
  const int col = blockIdx.x;
  if (col >= nrhs) return;
  const int64_t ldx = (int64_t)ldmul * n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* xs = reinterpret_cast<T*>(smraw);
  T* tile = xs + n;                                  // 32 x 32 block, column-major, ld 33
  const T* M = LU + mat_off[k];
  const int32_t* ip = piv + piv_off[k];
  zc* xg = X + x_off[k] + (size_t)col * ldx;
  const float* R = rs ? rs + piv_off[k] : nullptr;
  const float* C = cs ? cs + piv_off[k] : nullptr;
  const T zero = cx<T>::make(0, 0);
  for (int r = tid; r < n; r += blockDim.x) {
    zc b = xg[r];
    if (R) b = zscale(b, (double)R[r]);
    xs[r] = cx<T>::from(b);
  }
  __syncthreads();
  if (tid == 0)
    for (int j = 0; j < n; ++j) {
      const int p = ip[j];
      if (p != j) { T t = xs[j]; xs[j] = xs[p]; xs[p] = t; }
    }
  __syncthreads();
  // L y = b, unit diagonal
  for (int jb = 0; jb < n; jb += 32) {
    const int bs = min(32, n - jb);
    for (int e = tid; e < bs * bs; e += blockDim.x) {
      const int c = e / bs, r = e % bs;
      tile[c * 33 + r] = M[(size_t)(jb + c) * n + jb + r];
    }
    __syncthreads();
    if (warp == 0) {
      T x = lane < bs ? xs[jb + lane] : zero;
      for (int j = 0; j < bs; ++j) {
        const T xj = shfl_cx(x, j);
        if (lane > j && lane < bs) x = cx<T>::fnma(tile[j * 33 + lane], xj, x);
      }
      if (lane < bs) xs[jb + lane] = x;
    }
    __syncthreads();
    for (int r = jb + bs + tid; r < n; r += blockDim.x) {
      T acc = xs[r];
      for (int j = 0; j < bs; ++j) acc = cx<T>::fnma(M[(size_t)(jb + j) * n + r], xs[jb + j], acc);
      xs[r] = acc;
    }
    __syncthreads();
  }
  // U x = y, blocks from the bottom; a zero diagonal entry is skipped
  for (int jb = ((n - 1) / 32) * 32; jb >= 0; jb -= 32) {
    const int bs = min(32, n - jb);
    for (int e = tid; e < bs * bs; e += blockDim.x) {
      const int c = e / bs, r = e % bs;
      tile[c * 33 + r] = M[(size_t)(jb + c) * n + jb + r];
    }
    __syncthreads();
    if (warp == 0) {
      T x = lane < bs ? xs[jb + lane] : zero;
      for (int j = bs - 1; j >= 0; --j) {
        const T d = tile[j * 33 + j];
        if (lane == j && cx<T>::abs1(d) != 0) x = cx<T>::div(x, d);
        const T xj = shfl_cx(x, j);
        if (lane < j) x = cx<T>::fnma(tile[j * 33 + lane], xj, x);
      }
      if (lane < bs) xs[jb + lane] = x;
    }
    __syncthreads();
    for (int r = tid; r < jb; r += blockDim.x) {
      T acc = xs[r];
      for (int j = 0; j < bs; ++j) acc = cx<T>::fnma(M[(size_t)(jb + j) * n + r], xs[jb + j], acc);
      xs[r] = acc;
    }
    __syncthreads();
  }
  for (int r = tid; r < n; r += blockDim.x) {
    zc y = cx<T>::to64(xs[r]);
    xg[r] = C ? zscale(y, (double)C[r]) : y;
  }
}

// ---- host launchers ------------------------------------------------------
template <typename T>
int lu_nb_for(int n) {
  // panel width such that the panel (n x NB) plus the U tile fit in shared memory
  const size_t lim = 200 * 1024;
  if ((size_t)n * 32 * sizeof(T) + 32 * 65 * sizeof(T) <= lim) return 32;
  if ((size_t)n * 16 * sizeof(T) + 16 * 65 * sizeof(T) <= lim) return 16;
  return 8;
}

template <typename T, int NB>
static cudaError_t launch_lu_nb(int count, const InstDesc* desc, const int32_t* nsz, int nmax, T* A,
                                const int64_t* mat_off, int32_t* piv, const int64_t* piv_off, int32_t* info,
                                cudaStream_t s, const int32_t* skip, const int32_t* order, int cluster) {
  size_t sm = (size_t)nmax * NB * sizeof(T) + (size_t)NB * 65 * sizeof(T);
  if (cluster == 4) {
    cudaError_t e = cudaFuncSetAttribute(k_lu<T, NB, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(4 * count);
      cfg.blockDim = dim3(256);
      cfg.dynamicSmemBytes = sm;
      cfg.stream = s;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 4;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, k_lu<T, NB, 4>, &cfg) == cudaSuccess && nclusters > 0)
        return cudaLaunchKernelEx(&cfg, k_lu<T, NB, 4>, count, desc, nsz, A, mat_off, piv, piv_off, info, skip,
                                  order);
    }
    cudaGetLastError();   // no cluster of this size fits: one CTA per matrix
  }
  cudaError_t e = cudaFuncSetAttribute(k_lu<T, NB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_lu<T, NB, 1><<<count, 256, sm, s>>>(count, desc, nsz, A, mat_off, piv, piv_off, info, skip, order);
  return cudaGetLastError();
}

template <typename T>
int lu_nb_max(int n) {
  return lu_nb_for<T>(n);
}

template <typename T>
cudaError_t launch_lu(int count, const InstDesc* desc, const int32_t* nsz, int nmax, T* A, const int64_t* mat_off,
                      int32_t* piv, const int64_t* piv_off, int32_t* info, cudaStream_t s, const int32_t* skip,
                      int nb_hint, const int32_t* order, int cluster) {
  if (count <= 0) return cudaSuccess;
  int nb = lu_nb_for<T>(nmax);
  // a tuned panel width no wider than shared memory allows
  if ((nb_hint == 8 || nb_hint == 16 || nb_hint == 32) && nb_hint <= nb) nb = nb_hint;
  if (nb == 32)
    return launch_lu_nb<T, 32>(count, desc, nsz, nmax, A, mat_off, piv, piv_off, info, s, skip, order, cluster);
  if (nb == 16)
    return launch_lu_nb<T, 16>(count, desc, nsz, nmax, A, mat_off, piv, piv_off, info, s, skip, order, cluster);
  return launch_lu_nb<T, 8>(count, desc, nsz, nmax, A, mat_off, piv, piv_off, info, s, skip, order, cluster);
}

template <typename T>
cudaError_t launch_getrs(int count, const int32_t* nsz, int nmax, const T* LU, const int64_t* mat_off,
                         const int32_t* piv, const int64_t* piv_off, zc* X, const int64_t* x_off, int nrhs_fixed,
                         int nrhs_mul, int ldmul, const int32_t* skip, cudaStream_t s, const float* rs,
                         const float* cs) {
  const int nrhs_max = nrhs_fixed > 0 ? nrhs_fixed : nrhs_mul * nmax;
  if (count <= 0 || nrhs_max <= 0) return cudaSuccess;
  if (nrhs_max < 8) {   // few right-hand sides: a whole CTA per column
    size_t sm = (size_t)nmax * sizeof(T) + 32 * 33 * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(k_getrs_blk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 g(nrhs_max, count);
    k_getrs_blk<T><<<g, 256, sm, s>>>(count, nsz, LU, mat_off, piv, piv_off, X, x_off, nrhs_fixed, nrhs_mul, ldmul,
                                      skip, rs, cs);
    return cudaGetLastError();
  }
  const int warps = 8;
  size_t sm = (size_t)warps * nmax * sizeof(T);
  cudaError_t e = cudaFuncSetAttribute(k_getrs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  dim3 g((nrhs_max + warps - 1) / warps, count);
  k_getrs<T><<<g, warps * 32, sm, s>>>(count, nsz, LU, mat_off, piv, piv_off, X, x_off, nrhs_fixed, nrhs_mul, ldmul,
                                        skip, rs, cs);
  return cudaGetLastError();
}

template cudaError_t launch_lu<zc>(int, const InstDesc*, const int32_t*, int, zc*, const int64_t*, int32_t*,
                                   const int64_t*, int32_t*, cudaStream_t, const int32_t*, int, const int32_t*, int);
template cudaError_t launch_lu<cc>(int, const InstDesc*, const int32_t*, int, cc*, const int64_t*, int32_t*,
                                   const int64_t*, int32_t*, cudaStream_t, const int32_t*, int, const int32_t*, int);
template cudaError_t launch_lu<dz>(int, const InstDesc*, const int32_t*, int, dz*, const int64_t*, int32_t*,
                                   const int64_t*, int32_t*, cudaStream_t, const int32_t*, int, const int32_t*, int);
template int lu_nb_max<zc>(int);
template int lu_nb_max<cc>(int);
template int lu_nb_max<dz>(int);

// Autotuning input: count dense n x n matrices with hashed entries in
// [-1, 1) + i[-1, 1) and the diagonal raised by n, so that every panel width
// factors the same well-conditioned problem.
template <typename T>
__global__ void k_tune_matrix(int count, int n, T* A) {
  const int64_t total = (int64_t)count * n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)(e * 2654435761u) ^ (uint32_t)(e >> 32) ^ 0x9e3779b9u;
    h ^= h >> 15; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    double re = (double)(h & 0xffff) / 32768.0 - 1.0, im = (double)(h >> 16) / 32768.0 - 1.0;
    const int64_t rc = e % ((int64_t)n * n);
    if (rc / n == rc % n) re += n;
    A[e] = cx<T>::from(zmk(re, im));
  }
}

template <typename T>
cudaError_t launch_tune_matrix(int count, int n, T* A, cudaStream_t s) {
  k_tune_matrix<T><<<1024, 256, 0, s>>>(count, n, A);
  return cudaGetLastError();
}
template cudaError_t launch_tune_matrix<zc>(int, int, zc*, cudaStream_t);
template cudaError_t launch_tune_matrix<cc>(int, int, cc*, cudaStream_t);
template cudaError_t launch_tune_matrix<dz>(int, int, dz*, cudaStream_t);
template cudaError_t launch_getrs<zc>(int, const int32_t*, int, const zc*, const int64_t*, const int32_t*,
                                      const int64_t*, zc*, const int64_t*, int, int, int, const int32_t*,
                                      cudaStream_t, const float*, const float*);
template cudaError_t launch_getrs<cc>(int, const int32_t*, int, const cc*, const int64_t*, const int32_t*,
                                      const int64_t*, zc*, const int64_t*, int, int, int, const int32_t*,
                                      cudaStream_t, const float*, const float*);
template cudaError_t launch_getrs<dz>(int, const int32_t*, int, const dz*, const int64_t*, const int32_t*,
                                      const int64_t*, zc*, const int64_t*, int, int, int, const int32_t*,
                                      cudaStream_t, const float*, const float*);

}  // namespace stab
