// Host stand-ins for the CUDA thread model and intrinsics used by the
// eigensolver headers, for the CPU tests in tests/host.  A block of
// g_block_threads std::threads (up to 256, eight warps) runs the
// device code: a spinning barrier over the block serves __syncthreads, one
// per warp serves __syncwarp, warp shuffles and votes go through per-warp
// exchange buffers between two warp barriers, and the rounding intrinsics
// map to IEEE float / double operations (the tests compile without FMA
// contraction).
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>

#include <cuda_runtime.h>

#define HOST_MAX_WARPS 8

namespace {
// generation-counting barrier; waiting threads yield (the block's threads
// share the host's cores)
struct SpinBarrier {
  std::atomic<int> count{0}, gen{0};
  int n = 32;
  void wait() {
    const int g = gen.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) == n - 1) {
      count.store(0, std::memory_order_relaxed);
      gen.fetch_add(1, std::memory_order_acq_rel);
    } else {
      while (gen.load(std::memory_order_acquire) == g) std::this_thread::yield();
    }
  }
};
thread_local int g_tid = 0;
int g_block_threads = 32;
SpinBarrier g_bar;                       // the block
SpinBarrier g_wbar[HOST_MAX_WARPS];      // one per warp
std::mutex g_mu;
alignas(16) unsigned char g_xch[32 * HOST_MAX_WARPS][16];
bool g_pred[32 * HOST_MAX_WARPS];
struct TIdx {
  unsigned x;
};
// set the block size before starting its threads
inline void host_block(int threads) {
  g_block_threads = threads;
  g_bar.n = threads;
}
}  // namespace
#define threadIdx (TIdx{(unsigned)g_tid})
#define blockDim (TIdx{(unsigned)g_block_threads})
inline void __syncthreads() { g_bar.wait(); }
inline void __syncwarp() { g_wbar[g_tid >> 5].wait(); }
inline int atomicMax(int* p, int v) {
  std::lock_guard<std::mutex> l(g_mu);
  const int o = *p;
  if (v > o) *p = v;
  return o;
}
inline int atomicAdd(int* p, int v) {
  std::lock_guard<std::mutex> l(g_mu);
  const int o = *p;
  *p = o + v;
  return o;
}
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
  std::lock_guard<std::mutex> l(g_mu);
  const unsigned long long o = *p;
  *p = o + v;
  return o;
}
template <class T>
T __shfl_down_sync(unsigned, T v, int o) {
  static_assert(sizeof(T) <= 16, "exchange slot");
  const int lane = g_tid & 31, base = g_tid - lane;
  std::memcpy(g_xch[g_tid], &v, sizeof(T));
  __syncwarp();
  T r = v;
  if (lane + o < 32) std::memcpy(&r, g_xch[base + lane + o], sizeof(T));
  __syncwarp();
  return r;
}
inline bool __all_sync(unsigned, bool p) {
  const int base = g_tid & ~31;
  g_pred[g_tid] = p;
  __syncwarp();
  bool a = true;
  for (int q = 0; q < 32; ++q) a = a && g_pred[base + q];
  __syncwarp();
  return a;
}
inline long long clock64() { return 0; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __double2float_rn(double x) { return (float)x; }
inline float __frcp_rn(float x) { return 1.0f / x; }
inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline double __drcp_rn(double x) { return 1.0 / x; }
inline int __double2hiint(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return (int)(b >> 32);
}
inline int __float_as_int(float x) {
  int b;
  std::memcpy(&b, &x, 4);
  return b;
}
using std::max;
using std::min;

