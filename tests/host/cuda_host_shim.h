// Host stand-ins for the CUDA thread model and intrinsics used by the
// eigensolver headers, for the CPU tests in tests/host: 32 std::threads run
// as the 32 threads of one warp, a spinning barrier serves __syncthreads /
// __syncwarp, warp shuffles and votes go through a shared exchange buffer
// between two barriers, and the rounding intrinsics map to IEEE float /
// double operations (the tests compile without FMA contraction).
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>

#include <cuda_runtime.h>

namespace {
// generation-counting barrier; waiting threads yield (32 threads share the
// host's cores)
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
SpinBarrier g_bar;
std::mutex g_mu;
alignas(16) unsigned char g_xch[32][16];
bool g_pred[32];
struct TIdx {
  unsigned x;
};
}  // namespace
#define threadIdx (TIdx{(unsigned)g_tid})
#define blockDim (TIdx{32u})
inline void __syncthreads() { g_bar.wait(); }
inline void __syncwarp() { g_bar.wait(); }
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
  std::memcpy(g_xch[g_tid], &v, sizeof(T));
  g_bar.wait();
  T r = v;
  if (g_tid + o < 32) std::memcpy(&r, g_xch[g_tid + o], sizeof(T));
  g_bar.wait();
  return r;
}
inline bool __all_sync(unsigned, bool p) {
  g_pred[g_tid] = p;
  g_bar.wait();
  bool a = true;
  for (int q = 0; q < 32; ++q) a = a && g_pred[q];
  g_bar.wait();
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

