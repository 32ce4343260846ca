// CPU build of the eigensolver's QR iteration (stab_gb300/csrc/qr.cuh) for
// the host tests: 32 std::threads stand in for the 32 threads of one warp,
// with a barrier for __syncthreads / __syncwarp, and the CUDA rounding
// intrinsics map to IEEE float / double operations (compiled without FMA
// contraction).  It reads a packed-or-dense Hessenberg matrix, runs the QR in
// complex128 and in double-word arithmetic, and writes both spectra.
//
// input  (argv[1]): int32 mp, then mp*mp complex128, column-major
// output (argv[2]): int32 status fp64, int32 status double-word,
//                   int64 updates fp64, int64 updates double-word,
//                   mp complex128 eigenvalues (fp64), mp (double-word)
#include <algorithm>
#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

namespace {
thread_local int g_tid = 0;
std::barrier<>* g_bar = nullptr;
std::mutex g_mu;
struct TIdx {
  unsigned x;
};
}  // namespace
#define threadIdx (TIdx{(unsigned)g_tid})
#define blockDim (TIdx{32u})
inline void __syncthreads() { g_bar->arrive_and_wait(); }
inline void __syncwarp() { g_bar->arrive_and_wait(); }
inline int atomicMax(int* p, int v) {
  std::lock_guard<std::mutex> l(g_mu);
  const int o = *p;
  if (v > o) *p = v;
  return o;
}
template <class T>
T __shfl_down_sync(unsigned, T v, int) {   // only reached through unused block reductions
  return v;
}
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __double2float_rn(double x) { return (float)x; }
inline float __frcp_rn(float x) { return 1.0f / x; }
inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline double __drcp_rn(double x) { return 1.0 / x; }
using std::max;
using std::min;

#include "../../stab_gb300/csrc/common.cuh"
#include "../../stab_gb300/csrc/dw.cuh"
namespace stab {
#include "../../stab_gb300/csrc/qr.cuh"
}

using namespace stab;

template <class E>
static std::vector<zc> run(const std::vector<zc>& Hd, int mp, int& st, long long& upd) {
  std::vector<E> P(hess_packed_size(mp) + 4);
  for (int c = 0; c < mp; ++c)
    for (int r = 0; r <= std::min(c + 2, mp - 1); ++r) {
      const zc v = (r <= c + 1) ? Hd[(size_t)c * mp + r] : zmk(0.0, 0.0);
      if constexpr (std::is_same<E, zc>::value) {
        P[hess_coff(c, mp) + r] = v;
      } else {
        const float hr = (float)v.x, hi = (float)v.y;
        P[hess_coff(c, mp) + r] = make_float4(hr, (float)(v.x - hr), hi, (float)(v.y - hi));
      }
    }
  std::vector<zc> ev(mp);
  static HqrSmem<E> s;
  std::barrier<> bar(32);
  g_bar = &bar;
  long long u0 = 0;
  int st0 = 0;
  std::vector<std::thread> th;
  for (int t = 0; t < 32; ++t)
    th.emplace_back([&, t] {
      g_tid = t;
      long long u = 0;
      const int r = qr_eigs<E, true>(SAcc<E>{P.data(), mp}, mp, ev.data(), s, s.refl, u);
      if (t == 0) {
        u0 = u;
        st0 = r;
      }
    });
  for (auto& x : th) x.join();
  st = st0;
  upd = u0;
  return ev;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int mp = 0;
  if (std::fread(&mp, 4, 1, f) != 1 || mp < 1 || mp > 4096) return 2;
  std::vector<zc> H((size_t)mp * mp);
  if (std::fread(H.data(), sizeof(zc), H.size(), f) != H.size()) return 2;
  std::fclose(f);
  int st1 = 0, st2 = 0;
  long long u1 = 0, u2 = 0;
  const std::vector<zc> e1 = run<zc>(H, mp, st1, u1);
  const std::vector<zc> e2 = run<dz>(H, mp, st2, u2);
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 2;
  std::fwrite(&st1, 4, 1, g);
  std::fwrite(&st2, 4, 1, g);
  std::fwrite(&u1, 8, 1, g);
  std::fwrite(&u2, 8, 1, g);
  std::fwrite(e1.data(), sizeof(zc), mp, g);
  std::fwrite(e2.data(), sizeof(zc), mp, g);
  std::fclose(g);
  return 0;
}
