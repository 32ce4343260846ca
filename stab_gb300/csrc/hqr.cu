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

// The eigensolver of one CTA over a persistent queue of instances; it runs
// with either block size (HQ_T for the batch, HQ_WIDE for a few instances).
// C is the working precision from the compaction on: complex128, or
// double-word complex.  In double-word form the compacted matrix is scaled
// by a power of two that brings its largest entry near 1 (the float exponent
// range is narrow) and the QR eigenvalues are scaled back; the isolated
// eigenvalues come straight from the FP64 input.
template <class C>
__device__ __forceinline__ void eig_plain_body(int count, const int32_t* __restrict__ msz, zc* __restrict__ A,
                                               const int64_t* __restrict__ a_off, zc* __restrict__ Hp,
                                               const int64_t* __restrict__ h_off, zc* __restrict__ eig,
                                               const int64_t* __restrict__ eig_off, int32_t* __restrict__ status,
                                               int32_t* __restrict__ work_counter, const int32_t* __restrict__ order,
                                               double* __restrict__ flops_out, unsigned char* smraw, HqrSmem<C>& s,
                                               int& s_inst) {
  typedef typename ew<C>::real R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (;;) {
    if (tid == 0) s_inst = atomicAdd(work_counter, 1);
    __syncthreads();
    const int slot = s_inst;
    if (slot >= count) return;
    const int inst = order ? order[slot] : slot;
    const int m = msz[inst];
    zc* M = A + a_off[inst];
    C* Hg = reinterpret_cast<C*>(Hp + h_off[inst]);
    zc* ev = eig + eig_off[inst];
    // shared scratch: active flags and act list (m ints each), then v, w, z
    int* active = reinterpret_cast<int*>(smraw);
    int* act = active + m;
    C* zs = reinterpret_cast<C*>(smraw + ((2 * (size_t)m * sizeof(int) + 15) / 16) * 16);
    C* v = zs;
    C* w = v + m;
    C* z = w + m;
    C* vn = z + m;            // next step's reflector vector (Hessenberg reduction)
    for (int i = tid; i < m; i += NTH) active[i] = 1;
    if (tid == 0) { s.mp = 0; s.emax = 0; }
    __syncthreads();
    long long t_ph = clock64();
    auto phase = [&](int q) {
      if (tid == 0) {
        const long long t = clock64();
        atomicAdd(&g_eig_phase_cycles[q], (unsigned long long)(t - t_ph));
        t_ph = t;
      }
    };
    // ---- 1. isolation -----------------------------------------------------
    int n_iso = 0;           // isolated eigenvalues are written from the top: ev[m-1-q]
    for (int pass = 0; pass < m; ++pass) {
      if (tid == 0) s.found = 0;
      __syncthreads();
      for (int r = tid; r < m; r += NTH) {           // rows: thread per row
        if (!active[r]) continue;
        bool zero = true;
        for (int c = 0; c < m && zero; ++c) {
          if (c == r || !active[c]) continue;
          const zc a = M[(size_t)c * m + r];
          zero = (a.x == 0.0 && a.y == 0.0);
        }
        if (zero) { active[r] = 2; atomicAdd(&s.found, 1); }
      }
      for (int c = warp; c < m; c += NWA) {          // columns: warp per column
        if (active[c] != 1) continue;
        bool zero = true;
        for (int r = lane; r < m; r += 32) {
          if (r == c || active[r] == 0) continue;
          const zc a = M[(size_t)c * m + r];
          if (a.x != 0.0 || a.y != 0.0) zero = false;
        }
        zero = __all_sync(0xffffffffu, zero);
        if (zero && lane == 0) { active[c] = 3; atomicAdd(&s.found, 1); }
      }
      __syncthreads();
      if (s.found == 0) break;
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
    phase(0);
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
    double unscale = 1.0;
    if constexpr (std::is_same<C, zc>::value) {
      for (int c = warp; c < mp; c += NWA) {
        const int sc = act[c];
        for (int r = lane; r < mp; r += 32) Hg[(size_t)c * ld + r] = M[(size_t)sc * m + act[r]];
      }
    } else {
      // largest binary exponent of the active entries (integer work), then
      // the scaled copy in double-word form
      int emax = 0;
      for (int c = warp; c < mp; c += NWA) {
        const int sc = act[c];
        for (int r = lane; r < mp; r += 32) {
          const zc a = M[(size_t)sc * m + act[r]];
          emax = max(emax, max((__double2hiint(a.x) >> 20) & 0x7ff, (__double2hiint(a.y) >> 20) & 0x7ff));
        }
      }
      atomicMax(&s.emax, emax);
      __syncthreads();
      // 2^-e with e the unbiased exponent (0 for an all-zero matrix)
      const int e = (s.emax == 0 || s.emax == 0x7ff) ? 0 : s.emax - 1023;
      const double scale = ldexp(1.0, -e);
      unscale = ldexp(1.0, e);
      for (int c = warp; c < mp; c += NWA) {
        const int sc = act[c];
        for (int r = lane; r < mp; r += 32) Hg[(size_t)c * ld + r] = ew<C>::from64(zscale(M[(size_t)sc * m + act[r]], scale));
      }
    }
    __syncthreads();
    phase(1);
    // ---- 3. balancing -------------------------------------------------------
    // (powers of two only, so the norms need little precision: in the
    // double-word form they are taken from the high words in FP32)
    for (int sweep = 0; sweep < 64; ++sweep) {
      if (tid == 0) s.flag = 0;
      __syncthreads();
      for (int i = 0; i < mp; ++i) {
        R cs = 0, rs = 0;
        for (int r = tid; r < mp; r += NTH) {
          if (r == i) continue;
          cs += ew<C>::mag2(Hg[(size_t)i * ld + r]);
          rs += ew<C>::mag2(Hg[(size_t)r * ld + i]);
        }
        block_sum2(s, cs, rs);
        if (tid == 0) {
          R c = sqrt(cs), r = sqrt(rs), f = 1;
          if (c != (R)0 && r != (R)0) {
            R g = r / (R)2;
            const R sum = c + r;
            int guard = 0;
            while (c < g && guard++ < 2000) { f *= (R)2; c *= (R)2; r /= (R)2; g /= (R)2; }
            g = c / (R)2;
            while (g >= r && guard++ < 4000) { f /= (R)2; c /= (R)2; g /= (R)2; r *= (R)2; }
            if (c + r >= (R)0.95 * sum) f = 1;
          }
          s.sc[0] = (double)f;
          if (f != (R)1) s.flag = 1;
        }
        __syncthreads();
        const R f = (R)s.sc[0];
        if (f != (R)1) {
          const R gi = (R)1 / f;
          for (int q = tid; q < mp; q += NTH) {
            C* a = &Hg[(size_t)q * ld + i];    // row i
            *a = zscale(*a, gi);
          }
          __syncthreads();
          for (int q = tid; q < mp; q += NTH) {
            C* a = &Hg[(size_t)i * ld + q];    // column i
            *a = zscale(*a, f);
          }
        }
        __syncthreads();
      }
      if (!s.flag) break;
      __syncthreads();
    }
    phase(2);
    // ---- 4. Hessenberg reduction -----------------------------------------
    // The left update of step k leaves column k+1 final, so the warp that
    // updates it also copies it into the next step's reflector vector and
    // sums its squared tail: step k+1 starts without a pass or a block
    // reduction of its own.
    double flops = 0.0;   // counted work of the reduction and the sweeps (thread 0)
    bool have_next = false;
    for (int k = 0; k + 2 < mp; ++k) {
      const int L = mp - k - 1;
      if (tid == 0) flops += 16.0 * (double)mp * L + 16.0 * (double)L * L;
      double ss = 0.0;
      if (have_next) {
        C* t = v;                        // the vector gathered by the last step
        v = vn;
        vn = t;
        ss = s.sc[5];
      } else {
        typename ew<C>::sq acc = ew<C>::sq_zero();
        for (int r = tid; r < L; r += NTH) {
          const C x = Hg[(size_t)k * ld + k + 1 + r];
          v[r] = x;
          if (r >= 1) ew<C>::sq_add(acc, x);
        }
        ss = block_sum_sq<C>(s, acc);
      }
      have_next = false;
      if (tid == 0) {
        const zc alpha = ew<C>::to64(v[0]);
        if (ss == 0.0 && alpha.y == 0.0) {
          s.flag = 0;                                      // H(k) = I
        } else {
          s.flag = 1;
          const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + ss), alpha.x);
          const zc scal = zdiv(zmk(1.0, 0.0), zmk(alpha.x - beta, alpha.y));
          s.hc[0] = ew<C>::from64(zmk((beta - alpha.x) / beta, -alpha.y / beta));   // tau
          s.hc[1] = ew<C>::from64(scal);
          s.hc[2] = ew<C>::from64(zmk(beta, 0.0));
        }
      }
      __syncthreads();
      if (!s.flag) continue;
      const C tau = s.hc[0];
      const C scal = s.hc[1];
      for (int r = tid; r < L; r += NTH) v[r] = (r == 0) ? ew<C>::one() : zmul(v[r], scal);
      if (tid == 0) Hg[(size_t)k * ld + k + 1] = s.hc[2];
      for (int r = 2 + tid; r <= L; r += NTH) Hg[(size_t)k * ld + k + r] = ew<C>::zero();
      __syncthreads();
      // right: w = tau H(:, k+1:) v
      for (int r = tid; r < mp; r += NTH) {
        C acc = ew<C>::zero();
        for (int c = 0; c < L; ++c) acc = zfma(Hg[(size_t)(k + 1 + c) * ld + r], v[c], acc);
        w[r] = zmul(tau, acc);
      }
      __syncthreads();
      // right update fused with the left product z = conj(tau) v^H H(k+1:, k+1:), warp per column
      for (int c = warp; c < L; c += NWA) {
        const C vc = zconj(v[c]);
        C* col = Hg + (size_t)(k + 1 + c) * ld;
        C acc = ew<C>::zero();
        for (int r = lane; r < mp; r += 32) {
          const C h = zfnma(w[r], vc, col[r]);
          col[r] = h;
          if (r >= k + 1) acc = zcfma(v[r - k - 1], h, acc);
        }
        acc = ew<C>::warp_sum_c(acc);
        if (lane == 0) z[c] = zmul(zconj(tau), acc);
      }
      __syncthreads();
      // left update: H(k+1:, k+1:) -= v z; column k+1 (c = 0, warp 0) also
      // feeds the next step: vn = H(k+2:, k+1), s.sc[5] = sum |vn[1:]|^2
      for (int c = warp; c < L; c += NWA) {
        const C zc_ = z[c];
        C* col = Hg + (size_t)(k + 1 + c) * ld + k + 1;
        if (c == 0) {
          typename ew<C>::sq sn = ew<C>::sq_zero();
          for (int r = lane; r < L; r += 32) {
            const C h = zfnma(v[r], zc_, col[r]);
            col[r] = h;
            if (r >= 1) vn[r - 1] = h;
            if (r >= 2) ew<C>::sq_add(sn, h);
          }
          sn = warp_sum(sn);
          if (lane == 0) s.sc[5] = ew<C>::sq_64(sn);
        } else {
          for (int r = lane; r < L; r += 32) col[r] = zfnma(v[r], zc_, col[r]);
        }
      }
      have_next = true;
      __syncthreads();
    }
    phase(3);
    // ---- 5. QR iteration on the packed matrix ---------------------------------
    // in-place repack of H (ld = mp) to the column-packed layout: a packed
    // offset never exceeds the unpacked one, so moving column by column in
    // increasing order through shared memory is safe
    for (int c = 0; c < mp; ++c) {
      const int rmax = (c + 2 < mp - 1) ? c + 2 : mp - 1;
      for (int r = tid; r <= rmax; r += NTH) v[r] = (r <= c + 1) ? Hg[(size_t)c * ld + r] : ew<C>::zero();
      __syncthreads();
      const int64_t o = hess_coff(c, mp);
      for (int r = tid; r <= rmax; r += NTH) Hg[o + r] = v[r];
      __syncthreads();
    }
    phase(4);
    long long upd = 0;   // 2-element reflector applications (24 flops each), thread 0
    int st = qr_eigs<C, true>(SAcc<C>{Hg, mp}, mp, ev, s, s.refl, upd);
    flops += 24.0 * (double)upd;
    if (unscale != 1.0)
      for (int q = tid; q < mp; q += NTH) ev[q] = zscale(ev[q], unscale);
    phase(5);
    if (tid == 0) {
      status[inst] = st;
      if (flops_out) flops_out[inst] = flops;
    }
    __syncthreads();
  }
}

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

template <class C>
__global__ void __launch_bounds__(HQ_WIDE, 1) k_eig_plain_wide(EIG_PLAIN_ARGS) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ HqrSmem<C> s;
  __shared__ int s_inst;
  eig_plain_body<C>(count, msz, A, a_off, Hp, h_off, eig, eig_off, status, work_counter, order, flops_out, smraw, s,
                    s_inst);
}


cudaError_t eig_phase_cycles(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_eig_phase_cycles, sizeof(unsigned long long) * 6);
  if (e != cudaSuccess || !reset) return e;
  static const unsigned long long zero[6] = {0, 0, 0, 0, 0, 0};
  return cudaMemcpyToSymbol(g_eig_phase_cycles, zero, sizeof(zero));
}

size_t eig_plain_smem(int mmax) {
  const size_t head = ((2 * (size_t)mmax * sizeof(int) + 15) / 16) * 16;
  return head + 4 * (size_t)mmax * sizeof(zc);
}

template <class C>
static cudaError_t launch_eig_t(int count, int mmax, const int32_t* msz, zc* A, const int64_t* a_off, zc* H,
                                const int64_t* h_off, zc* eig, const int64_t* eig_off, int32_t* status,
                                int32_t* work_counter, const int32_t* order, double* flops, int grid,
                                cudaStream_t s) {
  size_t sm = eig_plain_smem(mmax);
  cudaError_t e = cudaFuncSetAttribute(k_eig_plain<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(work_counter, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (count * 2 <= sms) {
    // a few instances: one wide CTA each, so every phase spreads over 16 warps
    e = cudaFuncSetAttribute(k_eig_plain_wide<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_eig_plain_wide<C><<<count, HQ_WIDE, sm, s>>>(count, msz, A, a_off, H, h_off, eig, eig_off, status,
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
                             cudaStream_t s, bool double_word) {
  if (count <= 0) return cudaSuccess;
  return double_word ? launch_eig_t<dz>(count, mmax, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter,
                                        order, flops, grid, s)
                     : launch_eig_t<zc>(count, mmax, msz, A, a_off, H, h_off, eig, eig_off, status, work_counter,
                                        order, flops, grid, s);
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
// array is created when the library is loaded and stays resident on every
// GPU that loads it until the process exits.
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
      su.ptr = reinterpret_cast<unsigned char*>(p);
      su.done = true;
    }
  }
  if (su.err != cudaSuccess || !su.ptr) return STAB_ERR_CUDA;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  NoallocHeader* hdr = reinterpret_cast<NoallocHeader*>(su.ptr);
  zc* H = reinterpret_cast<zc*>(su.ptr + STAB_NOALLOC_HEADER_BYTES);
  k_noalloc_header<<<1, 1, 0, s>>>(hdr, m);   // resets the work counter left by the previous call
  if (cudaGetLastError() != cudaSuccess) return STAB_ERR_CUDA;
  const size_t sm = eig_plain_smem(m);
  if (cudaFuncSetAttribute(k_eig_plain<zc>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
    return STAB_ERR_CUDA;
  k_eig_plain<zc><<<1, HQ_T, sm, s>>>(1, &hdr->m, const_cast<zc*>(reinterpret_cast<const zc*>(a_dev)), &hdr->a_off, H,
                                  &hdr->h_off, reinterpret_cast<zc*>(eig_dev), &hdr->eig_off, status_dev,
                                  &hdr->counter, nullptr, nullptr);
  return cudaGetLastError() == cudaSuccess ? STAB_OK : STAB_ERR_CUDA;
}
