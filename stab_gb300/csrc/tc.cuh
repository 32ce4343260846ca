// Fifth-generation tensor cores (tcgen05) for the complex trailing updates:
// inline-PTX wrappers for TMEM allocation, the kind::tf32 MMA with shared
// memory operands, its completion mbarrier, and the TMEM -> register loads of
// the epilogue; plus the split of complex64 operands into the TF32 planes the
// MMA reads.
//
// Complex product on real tensor cores (real split).  With L = Lr + i Li and
// U = Ur + i Ui, the update C -= L U is
//   Cr -= Lr Ur - Li Ui,   Ci -= Lr Ui + Li Ur,
// four real products accumulated in two TMEM regions, the signs carried by
// the operand planes (-Lr, and a B plane [Ui | -Ur] next to [Ur | Ui]).  Each real operand x is split into three TF32
// parts x = x0 + x1 + x2 (x0 = tf32(x), x1 = tf32(x - x0), x2 = tf32(x - x0 -
// x1)); a product keeps the six terms whose part indices sum to at most 2,
// x0y0 + x0y1 + x1y0 + x0y2 + x1y1 + x2y0, which leaves a relative error of
// about 2^-33 per product before the FP32 accumulation, so the update is as
// accurate as an FP32 FMA update.
//
// Operand layout in shared memory (the canonical K-major layout without
// swizzle): a plane holds `rows` x K values; core matrices of 8 rows x 4
// values (16 bytes per row, 128 bytes) are stored contiguously; the core
// matrices of one 8-row group follow each other along K (leading byte offset
// 128), and 8-row groups are K*32 bytes apart (stride byte offset).
#pragma once
#include <cstdint>

namespace stab {
namespace tc {

// ---- descriptors ---------------------------------------------------------
// Instruction descriptor of tcgen05.mma kind::tf32: D float32, A and B TF32,
// both K-major, M rows, N columns; neg_a negates A (D += -A B).
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N, bool neg_a) {
  return (1u << 4)                        // D format: F32
         | (2u << 7)                      // A format: TF32
         | (2u << 10)                     // B format: TF32
         | ((neg_a ? 1u : 0u) << 13)      // negate A
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// Shared-memory matrix descriptor, no swizzle, for a K-major plane at shared
// address `saddr` (16-byte aligned) with leading byte offset lbo (between
// core matrices adjacent in K) and stride byte offset sbo (between 8-row
// groups).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of tcgen05
  return d;                 // base offset 0, layout type 0 (no swizzle)
}

// byte offset of value (r, k) of a K-major plane with K values per row
__host__ __device__ __forceinline__ uint32_t plane_off(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K * 32)) + ((k >> 2) * 128) + ((r & 7) * 16) + ((k & 3) * 4));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ---- TMEM ------------------------------------------------------------------
// One warp allocates `ncols` (power of two >= 32) columns; the base address is
// written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// generic-proxy shared-memory writes visible to the tensor core's reads
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// ---- MMA -------------------------------------------------------------------
// D[tmem] (+)= A[adesc] * B[bdesc]; accumulate = 0 overwrites D.  Issued by
// one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on the mbarrier once every MMA issued so far by this thread is done
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

// ---- mbarrier ----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* mbar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smem_u32(mbar)) : "memory");
}
// Wait for the phase with parity `parity` to complete; gives up after
// `limit` polls and returns false (the caller records the error).
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- TMEM -> registers ---------------------------------------------------------
// 16 consecutive float32 columns of this thread's TMEM lane (the warp reads
// lanes 32*(warp%4) .. +31 starting at column taddr & 0xffff).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// 8 consecutive float32 columns, as tmem_ld16
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// ---- TMA (tensor copies between global and shared memory) --------------------
// The tensor map sits in global memory (written by the host before the
// launch); the acquire fence orders the tensor-map proxy's view of it.
__device__ __forceinline__ void tmap_acquire(const void* tmap) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(tmap) : "memory");
}
// Expect `bytes` of asynchronous transfers on the mbarrier and arrive once.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(bytes)
               : "memory");
}
// 2D tile load global -> shared: box at (x, y) of the tensor (x the
// contiguous dimension, in elements; x * element size must be a multiple of
// 16 bytes), completion counted on the mbarrier.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(mbar))
      : "memory");
}
// 2D tile store shared -> global (elements outside the tensor are not
// written), tracked by the issuing thread's bulk async-group.
__device__ __forceinline__ void tma_store_2d(const void* tmap, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(tmap), "r"(x),
               "r"(y), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// the source shared memory of every committed store has been read
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// every committed store is complete in global memory
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
// async-proxy global writes ordered before later generic-proxy accesses
__device__ __forceinline__ void fence_async_global() {
  asm volatile("fence.proxy.async.global;\n" ::: "memory");
}

// ---- TF32 split --------------------------------------------------------------
// Round to TF32 (10 explicit mantissa bits, nearest, ties away from zero on
// the magnitude), returned as a float whose low 13 bits are zero, so the MMA
// reads it exactly.
__host__ __device__ __forceinline__ float tf32_round(float x) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(x);
#else
  uint32_t u;
  __builtin_memcpy(&u, &x, 4);
#endif
  if ((u & 0x7f800000u) != 0x7f800000u) {   // finite: add half an ulp of TF32, then truncate
    u += 0x1000u;
    u &= 0xffffe000u;
  }
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float y;
  __builtin_memcpy(&y, &u, 4);
  return y;
#endif
}
// x = p0 + p1 + p2 with each part a TF32 value
__host__ __device__ __forceinline__ void tf32_split3(float x, float& p0, float& p1, float& p2) {
  p0 = tf32_round(x);
  const float r1 = x - p0;   // exact
  p1 = tf32_round(r1);
  p2 = tf32_round(r1 - p1);  // exact difference, rounded
}

}  // namespace tc
}  // namespace stab
