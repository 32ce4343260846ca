// Full-spectrum eigensolver: the GPU replacement of ZGEEV (temporal.f90:803,
// spatial.f90:1043) for all eigenvalues.
//
// Per instance (one CTA, instances taken from a work counter):
//   1. isolation: rows (columns) whose off-diagonal entries are exactly zero
//      within the active set give eigenvalue a_ii and are removed, repeated
//      until none is found (the permutation step of ZGEBAL).  The temporal
//      Dirichlet rows and the zero columns of the spatial companion matrix
//      leave this way, so they come out as exact zeros like in ZGEEV.
//   2. compaction of the active submatrix into H;
//   3. diagonal balancing by powers of two (the scaling step of ZGEBAL);
//   4. Householder reduction to upper Hessenberg form (as ZGEHD2);
//   5. complex QR (the algorithm of ZLAHQR, eigenvalues only): multi-bulge
//      sweeps with shifts from the trailing block, single-shift steps with
//      Wilkinson shifts on small windows, exceptional shifts every 10th
//      iteration and the deflation test of Ahues and Tisseur.  The
//      2-element reflectors are general complex ones, so the subdiagonal need
//      not be kept real.
//
// Steps 2-5 run in the working precision C: complex128 for the answer, or
// double-word complex (dw.cuh) for spectra that only seed a polish.  GB300
// issues FP64 at 1/59 of the FP32 rate, so the FP64 form is bound by the
// FP64 pipe; the double-word form runs the same algorithm on the FP32 pipe,
// with no FP64 instruction on the serial path of a QR step.
//
// GB300 shape of step 5: the serial work of a bulge step (the next
// reflector) runs on lanes of warp 0 while all threads do the row and column
// updates, with a barrier per phase.  The serial chains of different
// instances overlap because the kernel runs small CTAs, several per SM; the
// Hessenberg matrix is repacked in place into a column-packed layout with two
// subdiagonals (room for the bulge), which keeps the working set of the
// resident instances in L2.
//
// Every loop has an iteration cap; an instance that hits it gets status
// STAB_ST_NOCONV and NaN for the missing values.
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "dw.cuh"
#include "kernels.cuh"
#include "hqr.cuh"

namespace stab {

#include "qr.cuh"

// SM cycles spent per phase of k_eig_plain, summed over instances (thread 0
// of each CTA adds clock64 differences): isolation, compaction, balancing,
// Hessenberg reduction, repacking, QR iteration.  Read by stab_eig_phases.
__device__ unsigned long long g_eig_phase_cycles[6];

#include "eig_body.cuh"

#define EIG_PLAIN_ARGS                                                                                       \
  int count, const int32_t *__restrict__ msz, zc *__restrict__ A, const int64_t *__restrict__ a_off,         \
      zc *__restrict__ Hp, const int64_t *__restrict__ h_off, zc *__restrict__ eig,                          \
      const int64_t *__restrict__ eig_off, int32_t *__restrict__ status, int32_t *__restrict__ work_counter, \
      const int32_t *__restrict__ order, double *__restrict__ flops_out

template <class C>
__global__ void __launch_bounds__(HQ_T, 4) k_eig_plain(EIG_PLAIN_ARGS) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem<C> s;
  __shared__ int s_inst;
  eig_plain_body<C>(count, msz, A, a_off, Hp, h_off, eig, eig_off, status, work_counter, order, flops_out, smraw, s,
                    s_inst);
}

// mid-size batches (at most two instances per SM): 256-thread CTAs, two per SM
template <class C>
__global__ void __launch_bounds__(2 * HQ_T, 2) k_eig_plain_mid(EIG_PLAIN_ARGS) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem<C> s;
  __shared__ int s_inst;
  eig_plain_body<C>(count, msz, A, a_off, Hp, h_off, eig, eig_off, status, work_counter, order, flops_out, smraw, s,
                    s_inst);
}

// the batch kernel with 64-thread CTAs, eight per SM (more instances in flight)
template <class C>
__global__ void __launch_bounds__(HQ_T / 2, 8) k_eig_plain_half(EIG_PLAIN_ARGS) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem<C> s;
  __shared__ int s_inst;
  eig_plain_body<C>(count, msz, A, a_off, Hp, h_off, eig, eig_off, status, work_counter, order, flops_out, smraw, s,
                    s_inst);
}

template <class C>
__global__ void __launch_bounds__(HQ_WIDE, 1) k_eig_plain_wide(EIG_PLAIN_ARGS) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem<C> s;
  __shared__ int s_inst;
  eig_plain_body<C>(count, msz, A, a_off, Hp, h_off, eig, eig_off, status, work_counter, order, flops_out, smraw, s,
                    s_inst);
}


// The seed batches (order m <= 160 at N = 32): one 512-thread CTA per SM,
// the QR phase on the packed Hessenberg matrix in shared memory.  With one
// instance per SM the working matrices of the reduction (152 x 410 KB in
// double-word form) stay in L2, and the QR's bulge steps read and write
// shared memory instead of L2 / HBM.
template <class C>
__global__ void __launch_bounds__(HQ_WIDE, 1) k_eig_plain_sq(EIG_PLAIN_ARGS) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem<C> s;
  __shared__ int s_inst;
  eig_plain_body<C, true>(count, msz, A, a_off, Hp, h_off, eig, eig_off, status, work_counter, order, flops_out, smraw,
                          s, s_inst);
}

cudaError_t eig_phase_cycles(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_eig_phase_cycles, sizeof(unsigned long long) * 6);
  if (e != cudaSuccess || !reset) return e;
  static const unsigned long long zero[6] = {0, 0, 0, 0, 0, 0};
  return cudaMemcpyToSymbol(g_eig_phase_cycles, zero, sizeof(zero));
}

size_t eig_plain_smem(int mmax) { return eig_plain_smem_bytes(mmax); }

template <class C>
static cudaError_t launch_eig_t(int count, int mmax, const int32_t* msz, zc* A, const int64_t* a_off, zc* H,
                                const int64_t* h_off, zc* eig, const int64_t* eig_off, int32_t* status,
                                int32_t* work_counter, const int32_t* order, double* flops, int grid,
                                cudaStream_t s, bool qr_smem, int threads) {
  size_t sm = eig_plain_smem(mmax);
  cudaError_t e = cudaFuncSetAttribute(k_eig_plain<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(work_counter, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t sm_q = eig_plain_smem_bytes(mmax, true) + sizeof(HqrSmem<C>) + 64;
  if (qr_smem && count * 2 > sms && sm_q <= 227 * 1024) {
    const size_t dyn = eig_plain_smem_bytes(mmax, true);
    e = cudaFuncSetAttribute(k_eig_plain_sq<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    const int g = std::min(count, sms);
    k_eig_plain_sq<C><<<g, HQ_WIDE, dyn, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter,
                                              order, flops);
    return cudaGetLastError();
  }
  if (count * 2 <= sms) {
    // a few instances: one wide CTA each, so every phase spreads over 16 warps
    e = cudaFuncSetAttribute(k_eig_plain_wide<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_eig_plain_wide<C><<<count, HQ_WIDE, sm, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status,
                                                   work_counter, order, flops);
    return cudaGetLastError();
  }
  if (threads == 2 * HQ_T && count <= 2 * sms) {
    // one 256-thread CTA per instance, all resident at once
    e = cudaFuncSetAttribute(k_eig_plain_mid<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_eig_plain_mid<C><<<count, 2 * HQ_T, sm, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status,
                                                  work_counter, order, flops);
    return cudaGetLastError();
  }
  if (threads == HQ_T / 2) {
    // persistent grid of 64-thread CTAs
    e = cudaFuncSetAttribute(k_eig_plain_half<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eig_plain_half<C>, HQ_T / 2, sm) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    const int resident = sms * per_sm;
    if (grid <= 0 || grid > resident) grid = resident;
    if (grid > count) grid = count;
    k_eig_plain_half<C><<<grid, HQ_T / 2, sm, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status,
                                                  work_counter, order, flops);
    return cudaGetLastError();
  }
  // persistent grid: as many CTAs as can be resident at once
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eig_plain<C>, HQ_T, sm) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int resident = sms * per_sm;
  if (grid <= 0 || grid > resident) grid = resident;
  if (grid > count) grid = count;
  k_eig_plain<C><<<grid, HQ_T, sm, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter, order,
                                        flops);
  return cudaGetLastError();
}

cudaError_t launch_eig_plain(int count, int mmax, const int32_t* msz, zc* A, const int64_t* a_off, zc* H,
                             const int64_t* h_off, zc* eig, const int64_t* eig_off, int32_t* status,
                             int32_t* work_counter, const int32_t* order, double* flops, int grid,
                             cudaStream_t s, bool double_word, bool qr_smem, int threads) {
  if (count <= 0) return cudaSuccess;
  return double_word ? launch_eig_t<dz>(count, mmax, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter,
                                        order, flops, grid, s, qr_smem, threads)
                     : launch_eig_t<zc>(count, mmax, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter,
                                        order, flops, grid, s, qr_smem, threads);
}

}  // namespace stab

// ---------------------------------------------------------------------------
// Allocation-free entry point (stab_eigvals_noalloc).
//
// Some callers cannot allocate device memory at call time: codes whose device
// memory is entirely owned by another allocator (a framework's caching pool,
// a simulation that reserves a fixed budget at start-up) and latency-critical
// loops where the device-wide synchronisation of cudaFree is not acceptable.
// For them the full-spectrum kernel above runs with its working matrix in a
// fixed array of this translation unit instead of a pool allocation.  The
// CUDA driver creates the array when it loads this module on a device: at
// library load with CUDA_MODULE_LOADING=EAGER, otherwise (lazy loading, the
// default) at the first call on that device, which therefore should be made
// at start-up.  The array then stays resident on that GPU until the process
// exits.  Calls also add to the eigensolver's phase counters
// (g_eig_phase_cycles, read by stab_eig_phases), like every other solve.
// ---------------------------------------------------------------------------
namespace stab {

#define STAB_NOALLOC_HEADER_BYTES 256
static __device__ __align__(256) unsigned char g_noalloc_scratch[STAB_NOALLOC_HEADER_BYTES +
                                                                 (size_t)STAB_NOALLOC_MAX_M * STAB_NOALLOC_MAX_M *
                                                                     sizeof(zc)];

// header of the scratch array: the per-instance tables k_eig_plain reads
struct NoallocHeader {
  int32_t counter;   // work counter of the persistent loop, must start at 0
  int32_t m;
  int64_t a_off, h_off, eig_off;
};

__global__ void k_noalloc_header(NoallocHeader* h, int m) {
  h->counter = 0;
  h->m = m;
  h->a_off = 0;
  h->h_off = 0;
  h->eig_off = 0;
}

}  // namespace stab

namespace {
// device address of g_noalloc_scratch per device, looked up once
struct NoallocSetup {
  bool done = false;
  cudaError_t err = cudaSuccess;
  unsigned char* ptr = nullptr;
};
NoallocSetup g_noalloc_setup[64];
std::mutex g_noalloc_mutex;
}  // namespace

extern "C" int stab_eigvals_noalloc(const double* a_dev, int32_t m, double* eig_dev, int32_t* status_dev,
                                    void* stream) {
  using namespace stab;
  if (!a_dev || !eig_dev || !status_dev) return STAB_ERR_ARG;
  if (m < 1 || m > STAB_NOALLOC_MAX_M) return STAB_ERR_ARG;   // the fixed array holds m <= STAB_NOALLOC_MAX_M
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return STAB_ERR_CUDA;
  NoallocSetup& su = g_noalloc_setup[dev];
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!su.done) {   // first call on this device: resolve the array's device address with the device current
      void* p = nullptr;
      su.err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (su.err == cudaSuccess && p) {
        su.ptr = reinterpret_cast<unsigned char*>(p);
        su.done = true;   // a failed lookup (e.g. inside a stream capture) is retried by the next call
      } else {
        cudaGetLastError();
      }
    }
  }
  if (!su.done || !su.ptr) return STAB_ERR_CUDA;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  NoallocHeader* hdr = reinterpret_cast<NoallocHeader*>(su.ptr);
  zc* H = reinterpret_cast<zc*>(su.ptr + STAB_NOALLOC_HEADER_BYTES);
  k_noalloc_header<<<1, 1, 0, s>>>(hdr, m);   // resets the work counter left by the previous call
  if (cudaGetLastError() != cudaSuccess) return STAB_ERR_CUDA;
  const size_t sm = eig_plain_smem(m);
  // one instance: the 512-thread variant, as the batched launcher picks for
  // a few instances (lower latency than the 128-thread batch kernel)
  if (cudaFuncSetAttribute(k_eig_plain_wide<zc>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
      cudaSuccess)
    return STAB_ERR_CUDA;
  k_eig_plain_wide<zc><<<1, HQ_WIDE, sm, s>>>(1, &hdr->m, const_cast<zc*>(reinterpret_cast<const zc*>(a_dev)),
                                              &hdr->a_off, H, &hdr->h_off, reinterpret_cast<zc*>(eig_dev),
                                              &hdr->eig_off, status_dev, &hdr->counter, nullptr, nullptr);
  return cudaGetLastError() == cudaSuccess ? STAB_OK : STAB_ERR_CUDA;
}
