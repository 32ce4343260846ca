// The blocked LU of one matrix (k_lu's body), shared by lu.cu and the CPU
// test that builds it on the host.  lu.cu includes it inside namespace stab.
#pragma once

template <typename T>
struct Piv {
  typename cx<T>::real v;
  int i;
};

template <typename T>
__device__ __forceinline__ void argmax_merge(typename cx<T>::real& bv, int& bi, typename cx<T>::real v, int i) {
  if (v > bv || (v == bv && i < bi)) { bv = v; bi = i; }
}

// CL > 1: a thread-block cluster of CL CTAs factors one matrix.  Rank 0
// factors each panel and writes it (and its pivots) to global memory; after
// a cluster barrier every rank loads the panel and applies the swaps, the
// U12 solve and the trailing update to its own 64-column tiles of the
// trailing matrix (tile t of the columns right of the panel belongs to rank
// t mod CL); a second cluster barrier closes the step.  The barriers are
// cluster-scope release/acquire, which orders the global-memory writes.
//
// lu_panel: steps 1-3 of the panel that starts at column k0 of the n x n
// matrix M (pivots to ip, first exactly-zero pivot to first_zero on thread
// 0): factor the panel in shared memory P (n x NB, column-major, ld = n) and
// write it back, swap the rows of the other columns, U12 = L11^-1 A12.
// Returns false when the panel was the last one.  Ends with a barrier; P
// still holds the factored panel (L11 and L21).
template <typename T, int NB, int CL>
__device__ __forceinline__ bool lu_panel(int k0, int rank, int n, T* __restrict__ M, int32_t* __restrict__ ip, T* P,
                                         typename cx<T>::real* red_v, int* red_i, int& s_piv, int& first_zero) {
  typedef typename cx<T>::real R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int w = min(NB, n - k0);
  const int rows = n - k0;
  if (rank == 0) {
    // 1. load panel
    for (int c = 0; c < w; ++c)
      for (int r = tid; r < rows; r += blockDim.x) P[(size_t)c * n + r] = M[(size_t)(k0 + c) * n + k0 + r];
    __syncthreads();
    for (int j = 0; j < w; ++j) {
      // pivot search over panel rows j..rows-1 of column j
      R bv = (R)-1;
      int bi = 0x7fffffff;
      for (int r = j + tid; r < rows; r += blockDim.x) argmax_merge<T>(bv, bi, cx<T>::abs1(P[(size_t)j * n + r]), r);
      for (int o = 16; o > 0; o >>= 1) {
        R ov = __shfl_down_sync(0xffffffffu, bv, o);
        int oi = __shfl_down_sync(0xffffffffu, bi, o);
        argmax_merge<T>(bv, bi, ov, oi);
      }
      if (lane == 0) { red_v[warp] = bv; red_i[warp] = bi; }
      __syncthreads();
      if (tid == 0) {
        R v = red_v[0];
        int ii = red_i[0];
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) argmax_merge<T>(v, ii, red_v[q], red_i[q]);
        if (ii < j || ii >= rows) ii = j;   // no finite entry (NaN input): keep the diagonal
        s_piv = ii;
        ip[k0 + j] = k0 + ii;
        if (v == (R)0 && first_zero == 0) first_zero = k0 + j + 1;
      }
      __syncthreads();
      const int p = s_piv;
      if (p != j && tid < w) {
        T t = P[(size_t)tid * n + j];
        P[(size_t)tid * n + j] = P[(size_t)tid * n + p];
        P[(size_t)tid * n + p] = t;
      }
      __syncthreads();
      const T d = P[(size_t)j * n + j];
      const bool nz = (cx<T>::abs1(d) != (R)0);
      // scale the column below the pivot and update the rest of the panel
      for (int r = j + 1 + tid; r < rows; r += blockDim.x) {
        T l = P[(size_t)j * n + r];
        if (nz) l = cx<T>::div(l, d);
        P[(size_t)j * n + r] = l;
        for (int c = j + 1; c < w; ++c) {
          T u = P[(size_t)c * n + j];
          P[(size_t)c * n + r] = cx<T>::fnma(l, u, P[(size_t)c * n + r]);
        }
      }
      __syncthreads();
    }
    // write the factored panel back
    for (int c = 0; c < w; ++c)
      for (int r = tid; r < rows; r += blockDim.x) M[(size_t)(k0 + c) * n + k0 + r] = P[(size_t)c * n + r];
  }   // rank 0
  if constexpr (CL > 1) {
    cg::this_cluster().sync();
    if (rank != 0)
      for (int c = 0; c < w; ++c)
        for (int r = tid; r < rows; r += blockDim.x) P[(size_t)c * n + r] = M[(size_t)(k0 + c) * n + k0 + r];
    __syncthreads();
  }
  const int c1 = k0 + w;
  // owner of column c: left of the panel by 64-column tiles, right of it by
  // 64-column tiles counted from c1 (the tiles of the trailing update)
  auto mine = [&](int c) {
    if (CL == 1) return true;
    return ((c < k0 ? c : c - c1) >> 6) % CL == rank;
  };
  // 2. row swaps on the columns outside the panel (one thread per column)
  for (int c = tid; c < n; c += blockDim.x) {
    if (c >= k0 && c < k0 + w) continue;
    if (!mine(c)) continue;
    for (int j = 0; j < w; ++j) {
      const int p = ip[k0 + j];
      if (p != k0 + j) {
        T t = M[(size_t)c * n + k0 + j];
        M[(size_t)c * n + k0 + j] = M[(size_t)c * n + p];
        M[(size_t)c * n + p] = t;
      }
    }
  }
  __syncthreads();
  if (c1 >= n) return false;
  // 3. U12 = L11^-1 A12 (unit lower), one thread per column
  for (int c = c1 + tid; c < n; c += blockDim.x) {
    if (!mine(c)) continue;
    T x[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) x[j] = (j < w) ? M[(size_t)c * n + k0 + j] : cx<T>::make(0, 0);
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      if (j >= w) break;
#pragma unroll
      for (int r = j + 1; r < NB; ++r)
        if (r < w) x[r] = cx<T>::fnma(P[(size_t)j * n + r], x[j], x[r]);
    }
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < w) M[(size_t)c * n + k0 + j] = x[j];
  }
  __syncthreads();
  return true;
}

// Step 4 on the CUDA cores: A22 -= L21 U12 for the panel at k0 (width
// w = NB), 64x64 tiles with 4x4 complex accumulators per thread (16x16
// threads), L21 read from the shared panel P and the U12 tile staged in Ub.
template <typename T, int NB, int CL>
__device__ __forceinline__ void lu_update_simt(int k0, int rank, int n, T* __restrict__ M, const T* P, T* Ub) {
  const int tid = threadIdx.x;
  const int w = NB;
  const int c1 = k0 + w;
  const int m2 = n - c1;
  const int tr = tid & 15, tc = tid >> 4;
  for (int tc0 = 64 * rank; tc0 < m2; tc0 += 64 * CL) {
    // stage U12 tile (w x 64) in shared memory
    for (int q = tid; q < NB * 64; q += blockDim.x) {
      const int j = q % NB, cc_ = q / NB;   // coalesced along the column
      const int c = c1 + tc0 + cc_;
      Ub[j * 65 + cc_] = (j < w && c < n) ? M[(size_t)c * n + k0 + j] : cx<T>::make(0, 0);
    }
    __syncthreads();
    for (int tr0 = 0; tr0 < m2; tr0 += 64) {
      T acc[4][4], cur[4][4];
      // the A22 tile is loaded before the rank-w product so that its
      // global-memory latency overlaps the shared-memory FMAs
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int c = c1 + tc0 + tc + 16 * b;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int r = c1 + tr0 + tr + 16 * a;
          acc[a][b] = cx<T>::make(0, 0);
          cur[a][b] = (c < n && r < n) ? M[(size_t)c * n + r] : cx<T>::make(0, 0);
        }
      }
      for (int j = 0; j < w; ++j) {
        T lv[4], uv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int r = tr0 + tr + 16 * a;          // row within A22
          lv[a] = (r < m2) ? P[(size_t)j * n + w + r] : cx<T>::make(0, 0);
        }
#pragma unroll
        for (int b = 0; b < 4; ++b) uv[b] = Ub[j * 65 + tc + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = cx<T>::fma_(lv[a], uv[b], acc[a][b]);
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int c = c1 + tc0 + tc + 16 * b;
        if (c >= n) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int r = c1 + tr0 + tr + 16 * a;
          if (r >= n) continue;
          M[(size_t)c * n + r] = cx<T>::sub(cur[a][b], acc[a][b]);
        }
      }
    }
    __syncthreads();
  }
}

// k: the matrix; rank: this CTA's rank in its cluster (0 for CL = 1);
// smraw: the dynamic shared memory (panel, U tile); red_v, red_i, s_piv:
// static shared scratch of the pivot search.
template <typename T, int NB, int CL>
__device__ __forceinline__ void lu_body(int k, int rank, const int32_t* __restrict__ nsz, T* __restrict__ A,
                                        const int64_t* __restrict__ mat_off, int32_t* __restrict__ piv,
                                        const int64_t* __restrict__ piv_off, int32_t* __restrict__ info,
                                        unsigned char* smraw, typename cx<T>::real* red_v, int* red_i, int& s_piv) {
  const int n = nsz[k];
  T* M = A + mat_off[k];
  int32_t* ip = piv + piv_off[k];
  T* P = reinterpret_cast<T*>(smraw);                  // panel: n x NB, column-major, ld = n
  T* Ub = P + (size_t)n * NB;                          // U12 tile: NB rows x 64 (+1 pad)
  int first_zero = 0;
  for (int k0 = 0; k0 < n; k0 += NB) {
    if (!lu_panel<T, NB, CL>(k0, rank, n, M, ip, P, red_v, red_i, s_piv, first_zero)) break;
    lu_update_simt<T, NB, CL>(k0, rank, n, M, P, Ub);
    if constexpr (CL > 1) cg::this_cluster().sync();   // the next panel reads other ranks' tiles
  }
  if (threadIdx.x == 0 && rank == 0) info[k] = first_zero;
}
