// Surrogate network kernels: a BF16 multilayer perceptron trained and run on
// the GPU (no counterpart in the reference, which has no learned part).
//
//   k_gemm_tc<TA, TB, EPI>    C = op(A) op(B) on the fifth-generation tensor
//                             cores (tcgen05.mma kind::f16, bf16 operands
//                             staged in shared memory, f32 accumulator in
//                             TMEM), the default;
//   k_gemm_bf16<TA, TB, EPI>  the same on mma.sync m16n8k16 (bf16 operands,
//                             f32 accumulators in registers), kept as the
//                             comparison form;
//                             both with the layer epilogues fused:
//                               EPI_HIDDEN   Z = acc + b; H = bf16(gelu(Z))
//                               EPI_OUT      Y = acc + b
//                               EPI_DHIDDEN  dZ = acc * gelu'(Z); bf16 copy
//                               EPI_WGRAD    G += acc (split over the batch)
//   k_loss_grad      dY = 2 w (Y - T) / B and the loss
//   k_bias_grad      db = column sums of dZ
//   k_adam           Adam on float32 master weights + their bf16 copy
//   k_cast_bf16      float32 -> bf16
//
// Per-layer work is tiny next to the eigen-solves (a 8192 x 256 x 256 layer
// is 1 GFLOP), so the GEMM is a plain 64 x 64 x 32 tile kernel without TMA
// staging.  The arithmetic each kernel performs is restated in numpy in
// oracle/mlp_oracle.py.
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.cuh"
#include "mlp.cuh"
#include "tc.cuh"

namespace stab {

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad_f(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * z * z);
  return cdf + z * pdf;
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int GM = 64, GN = 64, GK = 32;
constexpr int AS_LD = GK + 8;   // bf16 elements per row of the A tile (80 B rows)
constexpr int BS_LD = GN + 8;

// C[M x N] = sum_k A(m, k) B(k, n); A(m, k) = A[m*lda + k] (TA = 0) or
// A[k*lda + m] (TA = 1); B(k, n) = B[k*ldb + n] (TB = 0) or B[n*ldb + k]
// (TB = 1).  blockIdx.z splits K (EPI_WGRAD only, which accumulates).
template <int TA, int TB, int EPI>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                                   const __nv_bfloat16* __restrict__ B, int ldb,
                                                   const float* __restrict__ bias, const float* __restrict__ zin,
                                                   float* __restrict__ c32, __nv_bfloat16* __restrict__ c16, int ldc,
                                                   int kchunk) {
  __shared__ __align__(16) __nv_bfloat16 As[GM * AS_LD];
  __shared__ __align__(16) __nv_bfloat16 Bs[GK * BS_LD];
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const int wm = warp >> 1, wn = warp & 1;
  const int m0 = blockIdx.y * GM, n0 = blockIdx.x * GN;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;
  const __nv_bfloat16 zero = __float2bfloat16(0.0f);
  for (int k0 = kbeg; k0 < kend; k0 += GK) {
    // A tile (GM x GK), read along the contiguous index of its layout
    for (int e = tid; e < GM * GK; e += 128) {
      int m, k;
      if (TA == 0) { m = e / GK; k = e % GK; } else { k = e / GM; m = e % GM; }
      const int gm = m0 + m, gk = k0 + k;
      __nv_bfloat16 v = zero;
      if (gm < M && gk < kend) v = TA == 0 ? A[(int64_t)gm * lda + gk] : A[(int64_t)gk * lda + gm];
      As[m * AS_LD + k] = v;
    }
    for (int e = tid; e < GK * GN; e += 128) {
      int k, n;
      if (TB == 0) { k = e / GN; n = e % GN; } else { n = e / GK; k = e % GK; }
      const int gk = k0 + k, gn = n0 + n;
      __nv_bfloat16 v = zero;
      if (gk < kend && gn < N) v = TB == 0 ? B[(int64_t)gk * ldb + gn] : B[(int64_t)gn * ldb + gk];
      Bs[k * BS_LD + n] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int r0 = wm * 32 + mt * 16 + g;
        const int c0 = kk + 2 * t;
        af[mt][0] = *reinterpret_cast<const uint32_t*>(&As[r0 * AS_LD + c0]);
        af[mt][1] = *reinterpret_cast<const uint32_t*>(&As[(r0 + 8) * AS_LD + c0]);
        af[mt][2] = *reinterpret_cast<const uint32_t*>(&As[r0 * AS_LD + c0 + 8]);
        af[mt][3] = *reinterpret_cast<const uint32_t*>(&As[(r0 + 8) * AS_LD + c0 + 8]);
      }
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int n = wn * 32 + nt * 8 + g;
        const int kb = kk + 2 * t;
        bf[nt][0] = pack_bf16(Bs[kb * BS_LD + n], Bs[(kb + 1) * BS_LD + n]);
        bf[nt][1] = pack_bf16(Bs[(kb + 8) * BS_LD + n], Bs[(kb + 9) * BS_LD + n]);
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bf[nt]);
    }
    __syncthreads();
  }
  // epilogue: fragment element q sits at row g (+8 for q >= 2), col 2t + (q & 1)
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = m0 + wm * 32 + mt * 16 + g + (q >= 2 ? 8 : 0);
        const int col = n0 + wn * 32 + nt * 8 + 2 * t + (q & 1);
        if (row >= M || col >= N) continue;
        const int64_t o = (int64_t)row * ldc + col;
        const float v = acc[mt][nt][q];
        if (EPI == EPI_HIDDEN) {
          const float z = v + bias[col];
          c32[o] = z;
          c16[o] = __float2bfloat16(gelu_f(z));
        } else if (EPI == EPI_OUT) {
          c32[o] = v + bias[col];
        } else if (EPI == EPI_DHIDDEN) {
          const float dz = v * gelu_grad_f(zin[o]);
          c32[o] = dz;
          c16[o] = __float2bfloat16(dz);
        } else {
          atomicAdd(&c32[o], v);
        }
      }
}

// ---- tcgen05 form ------------------------------------------------------------
// One CTA of 128 threads computes a 128 x 128 tile of C.  K runs in chunks
// of 64: the threads copy the op(A) rows (128 x 64) and the op(B) columns
// (128 x 64, as the K-major rows of the MMA's B operand) into shared memory
// in the canonical K-major layout without swizzle (core matrices of 8 rows x
// 8 bf16 = 128 bytes, K-adjacent ones 128 bytes apart, 8-row groups 1 KB
// apart), zero outside the matrices; thread 0 issues the chunk's four MMAs
// of 128 x 128 x 16 into the TMEM accumulator and commits them to an
// mbarrier, which every thread waits on (bounded) before the next chunk
// overwrites the operands.  The epilogue: warp w reads TMEM lanes 32 w ..
// 32 w + 31 (the tile's rows) and applies the layer's epilogue.
namespace {
constexpr int TC_M = 128, TC_N = 128, TC_KC = 64;
constexpr uint32_t TC_SBO = (TC_KC / 8) * 128;      // 8-row groups
constexpr uint32_t TC_LBO = 128;                    // K-adjacent core matrices
constexpr uint32_t TC_PLANE = TC_M * TC_KC * 2;     // bytes of one operand tile
constexpr uint32_t TC_WAIT = 1u << 22;              // polls of the MMA mbarrier before giving up

__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                       // D format: F32
         | (1u << 7)                     // A format: BF16 (kind::f16)
         | (1u << 10)                    // B format: BF16
         | ((uint32_t)(N >> 3) << 17)    // N / 8
         | ((uint32_t)(M >> 4) << 24);   // M / 16
}
__device__ __forceinline__ uint32_t bf16_off(int r, int k) {
  return (uint32_t)((r >> 3) * TC_SBO + (k >> 3) * TC_LBO + (r & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ void mma_bf16_tc(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
}  // namespace

// set by a tile whose MMA completion was not seen within the wait limit
__device__ int g_mlp_tc_timeout;

template <int TA, int TB, int EPI>
__global__ void __launch_bounds__(128, 4) k_gemm_tc(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                                    const __nv_bfloat16* __restrict__ B, int ldb,
                                                    const float* __restrict__ bias, const float* __restrict__ zin,
                                                    float* __restrict__ c32, __nv_bfloat16* __restrict__ c16, int ldc,
                                                    int kchunk) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  unsigned char* As = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_smem) + 1023) & ~(uintptr_t)1023);
  unsigned char* Bs = As + TC_PLANE;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * TC_N;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  if (warp == 0) {
    tc::tmem_alloc(&tmem_slot, TC_N);
    tc::tmem_relinquish();
  }
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_slot;
  const uint32_t idesc = idesc_bf16(TC_M, TC_N);
  const uint32_t a_s = tc::smem_u32(As), b_s = tc::smem_u32(Bs);
  const __nv_bfloat16 zero = __float2bfloat16(0.0f);
  uint32_t phase = 0;
  bool ok = true;
  bool any = false;
  // 16-byte loads (8 bf16) where the matrix and its leading dimension allow
  const bool a_vec = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && (lda % 8 == 0);
  const bool b_vec = ((reinterpret_cast<uintptr_t>(B) & 15) == 0) && (ldb % 8 == 0);
  for (int k0 = kbeg; k0 < kend; k0 += TC_KC) {
    // op(A)(m, k) rows and op(B)(k, n) columns, read along the contiguous
    // index of each layout, 8 values per thread and step: an 8-run along k
    // is one 16-byte row of a core matrix; an 8-run along m (n) goes to 8
    // rows.  Runs that leave the matrix, or matrices without 16-byte rows,
    // take element loads with zero fill.
    for (int e = tid; e < TC_M * TC_KC / 8; e += 128) {
      int m, k;
      if (TA == 0) { m = e / (TC_KC / 8); k = (e % (TC_KC / 8)) * 8; } else { k = e / (TC_M / 8); m = (e % (TC_M / 8)) * 8; }
      const int gm = m0 + m, gk = k0 + k;
      if (TA == 0) {
        if (a_vec && gm < M && gk + 8 <= kend) {
          *reinterpret_cast<uint4*>(As + bf16_off(m, k)) = *reinterpret_cast<const uint4*>(A + (int64_t)gm * lda + gk);
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i)
            *reinterpret_cast<__nv_bfloat16*>(As + bf16_off(m, k + i)) =
                (gm < M && gk + i < kend) ? A[(int64_t)gm * lda + gk + i] : zero;
        }
      } else {
        if (a_vec && gk < kend && gm + 8 <= M) {
          const uint4 v = *reinterpret_cast<const uint4*>(A + (int64_t)gk * lda + gm);
          const __nv_bfloat16* pv = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
          for (int i = 0; i < 8; ++i) *reinterpret_cast<__nv_bfloat16*>(As + bf16_off(m + i, k)) = pv[i];
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i)
            *reinterpret_cast<__nv_bfloat16*>(As + bf16_off(m + i, k)) =
                (gm + i < M && gk < kend) ? A[(int64_t)gk * lda + gm + i] : zero;
        }
      }
    }
    for (int e = tid; e < TC_N * TC_KC / 8; e += 128) {
      int k, n;
      if (TB == 0) { k = e / (TC_N / 8); n = (e % (TC_N / 8)) * 8; } else { n = e / (TC_KC / 8); k = (e % (TC_KC / 8)) * 8; }
      const int gk = k0 + k, gn = n0 + n;
      if (TB == 1) {
        if (b_vec && gn < N && gk + 8 <= kend) {
          *reinterpret_cast<uint4*>(Bs + bf16_off(n, k)) = *reinterpret_cast<const uint4*>(B + (int64_t)gn * ldb + gk);
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i)
            *reinterpret_cast<__nv_bfloat16*>(Bs + bf16_off(n, k + i)) =
                (gn < N && gk + i < kend) ? B[(int64_t)gn * ldb + gk + i] : zero;
        }
      } else {
        if (b_vec && gk < kend && gn + 8 <= N) {
          const uint4 v = *reinterpret_cast<const uint4*>(B + (int64_t)gk * ldb + gn);
          const __nv_bfloat16* pv = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
          for (int i = 0; i < 8; ++i) *reinterpret_cast<__nv_bfloat16*>(Bs + bf16_off(n + i, k)) = pv[i];
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i)
            *reinterpret_cast<__nv_bfloat16*>(Bs + bf16_off(n + i, k)) =
                (gn + i < N && gk < kend) ? B[(int64_t)gk * ldb + gn + i] : zero;
        }
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int ks = 0; ks < TC_KC / 16; ++ks) {
        const uint64_t ad = tc::sdesc(a_s + ks * 2 * TC_LBO, TC_LBO, TC_SBO);
        const uint64_t bd = tc::sdesc(b_s + ks * 2 * TC_LBO, TC_LBO, TC_SBO);
        mma_bf16_tc(tm, ad, bd, idesc, (any || ks > 0) ? 1u : 0u);
      }
      tc::mma_commit(&mbar);
    }
    __syncwarp();
    const bool got = tc::mbar_wait(&mbar, phase, TC_WAIT);
    phase ^= 1u;
    tc::fence_after_sync();
    any = true;
    if (!__syncthreads_and(got)) {
      ok = false;
      break;
    }
  }
  if (ok && any) {
    const int row = m0 + 32 * warp + lane;
    const uint32_t trow = tm + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < TC_N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(trow + (uint32_t)c0, v);
      tc::tmem_wait_ld();
      if (row >= M) continue;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int col = n0 + c0 + i;
        if (col >= N) continue;
        const int64_t o = (int64_t)row * ldc + col;
        if (EPI == EPI_HIDDEN) {
          const float z = v[i] + bias[col];
          c32[o] = z;
          c16[o] = __float2bfloat16(gelu_f(z));
        } else if (EPI == EPI_OUT) {
          c32[o] = v[i] + bias[col];
        } else if (EPI == EPI_DHIDDEN) {
          const float dz = v[i] * gelu_grad_f(zin[o]);
          c32[o] = dz;
          c16[o] = __float2bfloat16(dz);
        } else {
          atomicAdd(&c32[o], v[i]);
        }
      }
    }
  }
  if (!ok && tid == 0) {
    atomicExch(&g_mlp_tc_timeout, 1);
    (void)tc::mbar_wait(&mbar, phase ^ 1u, TC_WAIT);   // the MMAs in flight (bounded)
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, TC_N);
  if (tid == 0) tc::mbar_inval(&mbar);
}

__global__ void k_loss_grad(int B, int N, const float* __restrict__ Y, int ldy, const float* __restrict__ T,
                            const float* __restrict__ w, float* __restrict__ dy32, __nv_bfloat16* __restrict__ dy16,
                            double* __restrict__ loss) {
  __shared__ double red[8];
  const int64_t total = (int64_t)B * N;
  double part = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / N), c = (int)(e % N);
    const float d = Y[(int64_t)r * ldy + c] - T[e];
    part += (double)w[c] * (double)d * (double)d;
    const float g = 2.0f * w[c] * d / (float)B;
    dy32[e] = g;
    dy16[e] = __float2bfloat16(g);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    atomicAdd(loss, s / (double)B);
  }
}

// db[c] = sum_r dZ[r, c]; one block per column group of 32, rows split over warps
__global__ void k_bias_grad(int B, int N, const float* __restrict__ dz, int ld, float* __restrict__ db) {
  __shared__ float red[8][33];
  const int c = blockIdx.x * 32 + (threadIdx.x & 31);
  const int w = threadIdx.x >> 5;
  float s = 0.0f;
  if (c < N)
    for (int r = w; r < B; r += 8) s += dz[(int64_t)r * ld + c];
  red[w][threadIdx.x & 31] = s;
  __syncthreads();
  if (w == 0 && c < N) {
    float tot = 0.0f;
    for (int i = 0; i < 8; ++i) tot += red[i][threadIdx.x & 31];
    db[c] = tot;
  }
}

__global__ void k_adam(int64_t count, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ p16, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (p16) p16[i] = __float2bfloat16(pi);
  }
}

__global__ void k_cast_bf16(int64_t count, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

template <int TA, int TB, int EPI>
static cudaError_t gemm_t(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb,
                          const float* bias, const float* zin, float* c32, __nv_bfloat16* c16, int ldc, int splits,
                          cudaStream_t s, bool tc5) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  splits = std::max(1, splits);
  const int kq = tc5 ? TC_KC : GK;
  int kchunk = (K + splits - 1) / splits;
  kchunk = ((kchunk + kq - 1) / kq) * kq;
  splits = (K + kchunk - 1) / kchunk;
  if (tc5) {
    const size_t sm = 2 * (size_t)TC_PLANE + 1024;
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<TA, TB, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 grid((N + TC_N - 1) / TC_N, (M + TC_M - 1) / TC_M, splits);
    k_gemm_tc<TA, TB, EPI><<<grid, 128, sm, s>>>(M, N, K, A, lda, B, ldb, bias, zin, c32, c16, ldc, kchunk);
    return cudaGetLastError();
  }
  dim3 grid((N + GN - 1) / GN, (M + GM - 1) / GM, splits);
  k_gemm_bf16<TA, TB, EPI><<<grid, 128, 0, s>>>(M, N, K, A, lda, B, ldb, bias, zin, c32, c16, ldc, kchunk);
  return cudaGetLastError();
}

cudaError_t mlp_tc_timeouts(int* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_mlp_tc_timeout, sizeof(int));
  if (e != cudaSuccess || !reset) return e;
  const int zero = 0;
  return cudaMemcpyToSymbol(g_mlp_tc_timeout, &zero, sizeof(int));
}

cudaError_t mlp_gemm_hidden(int M, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* W, const float* b,
                            float* Z, __nv_bfloat16* H, cudaStream_t s, bool tc5) {
  return gemm_t<0, 0, EPI_HIDDEN>(M, N, K, X, K, W, N, b, nullptr, Z, H, N, 1, s, tc5);
}

cudaError_t mlp_gemm_out(int M, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* W, const float* b,
                         float* Y, cudaStream_t s, bool tc5) {
  return gemm_t<0, 0, EPI_OUT>(M, N, K, X, K, W, N, b, nullptr, Y, nullptr, N, 1, s, tc5);
}

// dZprev[M x K] = (dZ[M x N] W^T) * gelu'(Zprev), W stored K x N
cudaError_t mlp_gemm_dhidden(int M, int N, int K, const __nv_bfloat16* dZ, const __nv_bfloat16* W, const float* Zprev,
                             float* dZprev, __nv_bfloat16* dZprev16, cudaStream_t s, bool tc5) {
  return gemm_t<0, 1, EPI_DHIDDEN>(M, K, N, dZ, N, W, N, nullptr, Zprev, dZprev, dZprev16, K, 1, s, tc5);
}

// G[K x N] += X[B x K]^T dZ[B x N] (G zeroed by the caller)
cudaError_t mlp_gemm_wgrad(int Bsz, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* dZ, float* G,
                           cudaStream_t s, bool tc5) {
  const int splits = std::min(64, std::max(1, Bsz / 256));
  return gemm_t<1, 0, EPI_WGRAD>(K, N, Bsz, X, K, dZ, N, nullptr, nullptr, G, nullptr, N, splits, s, tc5);
}

cudaError_t mlp_loss_grad(int B, int N, const float* Y, int ldy, const float* T, const float* w, float* dy32,
                          __nv_bfloat16* dy16, double* loss, cudaStream_t s) {
  const int64_t total = (int64_t)B * N;
  const int grid = (int)std::min<int64_t>(1024, (total + 255) / 256);
  k_loss_grad<<<std::max(grid, 1), 256, 0, s>>>(B, N, Y, ldy, T, w, dy32, dy16, loss);
  return cudaGetLastError();
}

cudaError_t mlp_bias_grad(int B, int N, const float* dz, float* db, cudaStream_t s) {
  k_bias_grad<<<(N + 31) / 32, 256, 0, s>>>(B, N, dz, N, db);
  return cudaGetLastError();
}

cudaError_t mlp_adam(int64_t count, float* p, const float* g, float* m, float* v, __nv_bfloat16* p16, float lr,
                     float b1, float b2, float eps, int step, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  const int grid = (int)std::min<int64_t>(2048, (count + 255) / 256);
  k_adam<<<std::max(grid, 1), 256, 0, s>>>(count, p, g, m, v, p16, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t mlp_cast_bf16(int64_t count, const float* x, __nv_bfloat16* y, cudaStream_t s) {
  const int grid = (int)std::min<int64_t>(2048, (count + 255) / 256);
  k_cast_bf16<<<std::max(grid, 1), 256, 0, s>>>(count, x, y);
  return cudaGetLastError();
}

}  // namespace stab
