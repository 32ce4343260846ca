// Complex64 batched LU with the trailing-matrix update on the tensor cores
// (tcgen05, kind::tf32): the factorisation of A - s B in the mixed-precision
// polish (the LU of ZGESV, temporal.f90:774, and of ZGETRF,
// spatial.f90:978, in the precision of the shift-invert polish).
//
// One CTA of 256 threads per matrix, as k_lu: the panel (n x 16) is factored
// in shared memory by the CUDA cores (lu_panel of lu_body.cuh: pivot search,
// row swaps, U12 = L11^-1 A12).  The update A22 -= L21 U12 runs per tile of
// 128 rows x 64 complex columns:
//   - the panel rows of the tile (L21) and the U12 columns are split into
//     TF32 parts (tc.cuh) and written to shared memory (over the panel's,
//     L21 re-read from global memory / L2) in the canonical
//     K-major layout: A planes -Lr and Li (3 parts each, 128 x 16),
//     B planes [Ur | Ui] and [Ui | -Ur] (3 parts each, 128 x 16), so one
//     MMA of N = 128 produces the real part in TMEM columns 0-63 and the
//     imaginary part in columns 64-127;
//   - thread 0 issues 2 K-steps x 6 part products x 2 operand pairs = 24
//     MMAs of 128 x 128 x 8 into one float32 TMEM accumulator and commits
//     them to an mbarrier;
//   - all eight warps read the accumulator back (tcgen05.ld, warp w owns
//     TMEM lanes 32 (w mod 4) and half of the columns) and add it to the
//     tile of A22 in global memory, coalesced along the column.
// Six part products keep about 2^-33 relative error per product, so the
// factors carry complex64 (FP32) accuracy; the polish's Newton-chord steps
// form their residuals in FP64 (polish.cu).
//
// Every wait on the MMA mbarrier is bounded; a wait that gives up marks the
// instance (info = -1), waits once more (bounded) for the MMAs in flight,
// frees the TMEM and ends the factorisation.
#include <algorithm>
#include <vector>
#include <cooperative_groups.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "dw.cuh"
#include "lu.cuh"
#include "tc.cuh"

namespace cg = cooperative_groups;

namespace stab {

#include "lu_body.cuh"

namespace {
constexpr int kTcNB = 16;                       // panel width = MMA K extent per tile
constexpr int kTcRows = 128;                    // tile rows (MMA M)
constexpr int kTcCols = 64;                     // tile complex columns (MMA N = 128 reals)
constexpr uint32_t kPlane = kTcRows * kTcNB * 4;   // bytes of one TF32 plane (128 x 16)
constexpr uint32_t kSbo = kTcNB * 32;           // 8-row group stride of a plane
constexpr uint32_t kLbo = 128;                  // K-adjacent core matrices
constexpr uint32_t kWaitLimit = 1u << 22;       // polls of the MMA mbarrier before giving up
constexpr uint32_t kTmemCols = 128;

__device__ __forceinline__ void put_split(unsigned char* base, uint32_t off, float v) {
  float p0, p1, p2;
  tc::tf32_split3(v, p0, p1, p2);
  *reinterpret_cast<float*>(base + off) = p0;
  *reinterpret_cast<float*>(base + kPlane + off) = p1;
  *reinterpret_cast<float*>(base + 2 * kPlane + off) = p2;
}
}  // namespace

// The panel (steps 1-3) and the TF32 planes (step 4) are never live at the
// same time: the planes reuse the panel's shared memory, and the update
// reads L21 from global memory, where lu_panel has just written it back (L2).
// For n <= 640 that is 97 KB, so two CTAs share an SM and one's panel
// factorisation overlaps the other's update.
__host__ __device__ __forceinline__ size_t lu_tc_region(int nmax) {
  const size_t panel = ((size_t)nmax * kTcNB * sizeof(cc) + 1023) & ~(size_t)1023;
  const size_t planes = 12 * (size_t)kPlane;
  return panel > planes ? panel : planes;   // panel, or 6 A + 6 B planes
}
// With TMA the A22 tile buffer (64 KB) follows, and one CTA fits per SM.
size_t lu_tc_smem(int nmax, bool tma) {
  return 1024 + lu_tc_region(nmax) + (tma ? (size_t)kTcRows * kTcCols * sizeof(cc) : 0);
}

// A22 -= L21 U12 for the panel at k0 on the tensor cores.  Returns false if
// an MMA (or tile-load) completion was not seen within the wait limit.
// TMA: the A22 tile goes through shared memory (Cs, 128 x 64 complex,
// column-major): thread 0 starts its tensor load before the B planes are
// staged, so the load overlaps the staging and the MMAs; the epilogue adds
// the accumulator to the tile in shared memory and thread 0 stores it back
// with a tensor store that overlaps the next tile's staging.  Without TMA the
// epilogue reads and writes A22 in global memory from the registers.
template <bool TMA>
__device__ __forceinline__ bool lu_update_tc(int k0, int n, cc* __restrict__ M, unsigned char* Apl,
                                             unsigned char* Bpl, cc* Cs, const void* tmap, uint32_t tm,
                                             uint64_t* mbar, uint32_t& phase, uint64_t* tbar, uint32_t& tphase) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c1 = k0 + kTcNB;
  const int m2 = n - c1;
  const uint32_t idesc = tc::idesc_tf32(128, 128, false);
  const uint32_t a_s = tc::smem_u32(Apl), b_s = tc::smem_u32(Bpl);
  bool ok = true;
  for (int rb0 = 0; rb0 < m2; rb0 += kTcRows) {
    const int nrow = min(kTcRows, m2 - rb0);
    // A planes: -Lr (parts 0..2) then Li (parts 0..2); row r of the tile is
    // row c1 + rb0 + r of L21 (panel column k0 + j, in global memory)
    for (int q = tid; q < kTcRows * kTcNB; q += blockDim.x) {
      const int r = q & (kTcRows - 1), j = q >> 7;
      const cc v = (r < nrow) ? M[(size_t)(k0 + j) * n + c1 + rb0 + r] : cmk(0.f, 0.f);
      const uint32_t off = tc::plane_off(r, j, kTcNB);
      put_split(Apl, off, -v.x);
      put_split(Apl + 3 * kPlane, off, v.y);
    }
    for (int cb0 = 0; cb0 < m2; cb0 += kTcCols) {
      const int ncol = min(kTcCols, m2 - cb0);
      if constexpr (TMA) {
        // the tile's rows start at c1 + rb0, a multiple of 16 (16-byte aligned
        // for 8-byte elements); the previous tile's store has read Cs
        if (tid == 0) {
          tc::bulk_wait_read();
          tc::mbar_arrive_expect_tx(tbar, kTcRows * kTcCols * (uint32_t)sizeof(cc));
          tc::tma_load_2d(Cs, tmap, c1 + rb0, c1 + cb0, tbar);
        }
      }
      // B planes: [Ur | Ui] (parts 0..2) then [Ui | -Ur]; B row c is U12
      // column c1 + cb0 + c, K index j its row k0 + j
      for (int q = tid; q < kTcCols * kTcNB; q += blockDim.x) {
        const int j = q & (kTcNB - 1), c = q >> 4;
        const cc u = (c < ncol) ? M[(size_t)(c1 + cb0 + c) * n + k0 + j] : cmk(0.f, 0.f);
        const uint32_t o_lo = tc::plane_off(c, j, kTcNB), o_hi = tc::plane_off(kTcCols + c, j, kTcNB);
        put_split(Bpl, o_lo, u.x);
        put_split(Bpl, o_hi, u.y);
        put_split(Bpl + 3 * kPlane, o_lo, u.y);
        put_split(Bpl + 3 * kPlane, o_hi, -u.x);
      }
      tc::fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        // part pairs (a, b) with a + b <= 2
        const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
        uint32_t acc = 0;
#pragma unroll
        for (int ks = 0; ks < kTcNB / 8; ++ks) {
#pragma unroll
          for (int t = 0; t < 6; ++t) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {   // h = 0: (-Lr, [Ur | Ui]); h = 1: (Li, [Ui | -Ur])
              const uint64_t ad = tc::sdesc(a_s + (3 * h + pa[t]) * kPlane + ks * 256, kLbo, kSbo);
              const uint64_t bd = tc::sdesc(b_s + (3 * h + pb[t]) * kPlane + ks * 256, kLbo, kSbo);
              tc::mma_tf32(tm, ad, bd, idesc, acc);
              acc = 1;
            }
          }
        }
        tc::mma_commit(mbar);
      }
      __syncwarp();
      bool got = tc::mbar_wait(mbar, phase, kWaitLimit);
      phase ^= 1u;
      if constexpr (TMA) {
        got = tc::mbar_wait(tbar, tphase, kWaitLimit) && got;
        tphase ^= 1u;
      }
      tc::fence_after_sync();
      if (!got) {
        ok = false;
      } else {
        // epilogue: warp w reads TMEM lanes 32 (w mod 4) + lane = tile rows,
        // complex columns [32 (w / 4), +32)
        const int r = 32 * (warp & 3) + lane;
        const int ch = 32 * (warp >> 2);
        const uint32_t trow = tm + ((uint32_t)(32 * (warp & 3)) << 16);
        if constexpr (TMA) {
#pragma unroll 1
          for (int c0 = 0; c0 < 32; c0 += 8) {
            float re[8], im[8];
            tc::tmem_ld8(trow + (uint32_t)(ch + c0), re);
            tc::tmem_ld8(trow + (uint32_t)(kTcCols + ch + c0), im);
            tc::tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              cc* e = Cs + (size_t)(ch + c0 + i) * kTcRows + r;   // rows and columns outside A22 are not stored
              *e = cmk(e->x + re[i], e->y + im[i]);
            }
          }
        } else {
#pragma unroll 1
          for (int c0 = 0; c0 < 32; c0 += 8) {
            // the 8 A22 entries are loaded before any store, so their global
            // latencies overlap each other and the TMEM reads
            cc a[8];
            cc* col = M + (size_t)(c1 + cb0 + ch + c0) * n + c1 + rb0 + r;
            const bool row_ok = r < nrow;
#pragma unroll
            for (int i = 0; i < 8; ++i)
              a[i] = (row_ok && ch + c0 + i < ncol) ? col[(size_t)i * n] : cmk(0.f, 0.f);
            float re[8], im[8];
            tc::tmem_ld8(trow + (uint32_t)(ch + c0), re);             // real parts
            tc::tmem_ld8(trow + (uint32_t)(kTcCols + ch + c0), im);   // imaginary parts
            tc::tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 8; ++i)
              if (row_ok && ch + c0 + i < ncol) col[(size_t)i * n] = cmk(a[i].x + re[i], a[i].y + im[i]);
          }
        }
      }
      if constexpr (TMA) tc::fence_async_smem();   // Cs writes visible to the tensor store
      tc::fence_before_sync();
      __syncthreads();
      if (!__syncthreads_and(ok)) return false;
      if constexpr (TMA) {
        if (tid == 0) {
          tc::tma_store_2d(tmap, c1 + rb0, c1 + cb0, Cs);
          tc::bulk_commit();
        }
      }
    }
  }
  if constexpr (TMA) {
    // the next panel reads A22 with ordinary loads
    if (tid == 0) {
      tc::bulk_wait_all();
      tc::fence_async_global();
    }
    __syncthreads();
  }
  return ok;
}

template <bool TMA>
__global__ void __launch_bounds__(256, TMA ? 1 : 2) k_lu_tc(int count, const int32_t* __restrict__ nsz,
                                                            cc* __restrict__ A, const int64_t* __restrict__ mat_off,
                                                            int32_t* __restrict__ piv,
                                                            const int64_t* __restrict__ piv_off,
                                                            int32_t* __restrict__ info,
                                                            const int32_t* __restrict__ skip,
                                                            const int32_t* __restrict__ order, int nmax,
                                                            const CUtensorMap* __restrict__ tmaps) {
  extern __shared__ unsigned char smraw_tc[];
  __shared__ float red_v[256 / 32];
  __shared__ int red_i[256 / 32];
  __shared__ int s_piv;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t tbar;
  __shared__ uint32_t tmem_slot;
  const int k = order ? order[blockIdx.x] : (int)blockIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  // 1024-aligned panel, then (TMA) the A22 tile buffer
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smraw_tc) + 1023) & ~(uintptr_t)1023);
  cc* P = reinterpret_cast<cc*>(base);           // steps 1-3
  unsigned char* Apl = base;                      // step 4, over the panel
  unsigned char* Bpl = Apl + 6 * kPlane;
  cc* Cs = reinterpret_cast<cc*>(base + lu_tc_region(nmax));
  const void* tmap = TMA ? (const void*)(tmaps + k) : nullptr;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    if (TMA) {
      tc::mbar_init(&tbar, 1);
      tc::tmap_acquire(tmap);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tmem_slot;
  const int n = nsz[k];
  cc* Mk = A + mat_off[k];
  int32_t* ip = piv + piv_off[k];
  int first_zero = 0;
  uint32_t phase = 0, tphase = 0;
  bool ok = true;
  for (int k0 = 0; k0 < n; k0 += kTcNB) {
    if (!lu_panel<cc, kTcNB, 1>(k0, 0, n, Mk, ip, P, red_v, red_i, s_piv, first_zero)) break;
    if (!lu_update_tc<TMA>(k0, n, Mk, Apl, Bpl, Cs, tmap, tm, &mbar, phase, &tbar, tphase)) {
      ok = false;
      break;
    }
  }
  if (!ok && tid == 0) {   // drain what may still be in flight
    (void)tc::mbar_wait(&mbar, phase, kWaitLimit);
    if (TMA) {
      (void)tc::mbar_wait(&tbar, tphase, kWaitLimit);
      tc::bulk_wait_all();
    }
  }
  if (tid == 0) info[k] = ok ? first_zero : -1;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, kTmemCols);
  if (tid == 0) {
    tc::mbar_inval(&mbar);
    if (TMA) tc::mbar_inval(&tbar);
  }
}

cudaError_t launch_lu_tc(int count, const int32_t* nsz, int nmax, cc* A, const int64_t* mat_off, int32_t* piv,
                         const int64_t* piv_off, int32_t* info, cudaStream_t s, const int32_t* skip,
                         const int32_t* order, const CUtensorMap* tmaps) {
  if (count <= 0) return cudaSuccess;
  const bool tma = tmaps != nullptr;
  const size_t sm = lu_tc_smem(nmax, tma);
  if (tma) {
    cudaError_t e = cudaFuncSetAttribute(k_lu_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_lu_tc<true><<<count, 256, sm, s>>>(count, nsz, A, mat_off, piv, piv_off, info, skip, order, nmax, tmaps);
  } else {
    cudaError_t e = cudaFuncSetAttribute(k_lu_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_lu_tc<false><<<count, 256, sm, s>>>(count, nsz, A, mat_off, piv, piv_off, info, skip, order, nmax, nullptr);
  }
  return cudaGetLastError();
}

bool lu_tc_fits(int nmax, bool tma) { return nmax >= 2 && lu_tc_smem(nmax, tma) <= 227 * 1024; }

// Tensor maps of the complex64 matrices for the tile loads and stores: per
// instance a 2D tensor of 8-byte elements, n rows (contiguous) x n columns,
// boxes of 128 x 64.  Needs 16-byte aligned bases and strides, so every
// order n must be even and every offset even; returns false (nothing
// encoded) otherwise or when the driver entry point is missing.
bool lu_tc_tensor_maps(int count, const int32_t* n, const int64_t* off, cc* base, std::vector<CUtensorMap>& out) {
  // looked up once per process (thread-safe static initialisation: contexts
  // may build batches from several host threads)
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return false;
  out.assign(count, CUtensorMap{});
  for (int k = 0; k < count; ++k) {
    if ((n[k] & 1) || (off[k] & 1)) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)n[k], (cuuint64_t)n[k]};
    const cuuint64_t strides[1] = {(cuuint64_t)n[k] * sizeof(cc)};
    const cuuint32_t box[2] = {(cuuint32_t)kTcRows, (cuuint32_t)kTcCols};
    const cuuint32_t estr[2] = {1, 1};
    if (encode(&out[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, base + off[k], dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

}  // namespace stab
