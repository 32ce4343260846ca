// CPU build of the per-instance eigensolver (stab_gb300/csrc/qr.cuh and
// eig_body.cuh) for the host tests, with the CUDA thread model of
// cuda_host_shim.h.  The block has 32 threads (one warp), or 128 (four
// warps, the batch kernel's shape) when the environment variable
// HOST_BLOCK_THREADS is 128.
//
//   dw_qr_host qr   IN OUT [dw]   IN: int32 mp, mp*mp complex128 column-major
//                                 upper Hessenberg; runs the QR only
//   dw_qr_host body IN OUT        IN: int32 m, m*m complex128 column-major
//                                 standard-form matrix; runs isolation,
//                                 balancing, Hessenberg reduction and QR
// OUT: int32 status fp64, int32 status double-word, int64 reflector
// applications fp64, int64 double-word, then the eigenvalues (complex128) of
// the fp64 run and of the double-word run.  "dw" skips the fp64 run.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <type_traits>
#include <vector>

#include "cuda_host_shim.h"

#include "../../stab_gb300/csrc/common.cuh"
#include "../../stab_gb300/csrc/dw.cuh"
namespace stab {
unsigned long long g_eig_phase_cycles[6];
#include "../../stab_gb300/csrc/qr.cuh"
#include "../../stab_gb300/csrc/eig_body.cuh"
}  // namespace stab

using namespace stab;

template <class F>
static void run_block(F f) {
  std::vector<std::thread> th;
  for (int t = 0; t < g_block_threads; ++t)
    th.emplace_back([&, t] {
      g_tid = t;
      f(t);
    });
  for (auto& x : th) x.join();
}

template <class E>
static std::vector<zc> run_qr(const std::vector<zc>& Hd, int mp, int& st, long long& upd) {
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
  run_block([&](int t) {
    long long u = 0;
    const int r = qr_eigs<E, true>(SAcc<E>{P.data(), mp}, mp, ev.data(), s, s.refl, u);
    if (t == 0) {
      upd = u;
      st = r;
    }
  });
  return ev;
}

template <class C, bool QS = false>
static std::vector<zc> run_body(const std::vector<zc>& A, int m, int& st, long long& upd) {
  std::vector<zc> M(A), Hw((size_t)m * m), ev(m);
  std::vector<unsigned char> smraw(eig_plain_smem_bytes(m, QS));
  const int32_t msz = m;
  const int64_t off = 0;
  int32_t status = -1, counter = 0;
  double flops = 0.0;
  static HqrSmem<C> s;
  static int s_inst;
  run_block([&](int) {
    eig_plain_body<C, QS>(1, &msz, M.data(), &off, Hw.data(), &off, ev.data(), &off, &status, &counter, nullptr,
                          &flops, smraw.data(), s, s_inst);
  });
  st = status;
  upd = (long long)flops;
  return ev;
}

int main(int argc, char** argv) {
  if (argc != 4 && argc != 5) return 2;
  const char* bt = std::getenv("HOST_BLOCK_THREADS");
  host_block(bt && std::strcmp(bt, "128") == 0 ? 128 : 32);
  const std::string mode = argv[1];
  const bool dw_only = (argc == 5 && std::strcmp(argv[4], "dw") == 0);
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) return 2;
  int m = 0;
  if (std::fread(&m, 4, 1, f) != 1 || m < 1 || m > 4096) return 2;
  std::vector<zc> H((size_t)m * m);
  if (std::fread(H.data(), sizeof(zc), H.size(), f) != H.size()) return 2;
  std::fclose(f);
  int st1 = 0, st2 = 0;
  long long u1 = 0, u2 = 0;
  std::vector<zc> e1(m, zmk(0.0, 0.0)), e2;
  if (mode == "qr") {
    if (!dw_only) e1 = run_qr<zc>(H, m, st1, u1);
    e2 = run_qr<dz>(H, m, st2, u2);
  } else if (mode == "body") {
    if (!dw_only) e1 = run_body<zc>(H, m, st1, u1);
    e2 = run_body<dz>(H, m, st2, u2);
  } else if (mode == "bodyq") {   // the QR phase on the packed copy in (shared) scratch memory
    if (!dw_only) e1 = run_body<zc, true>(H, m, st1, u1);
    e2 = run_body<dz, true>(H, m, st2, u2);
  } else {
    return 2;
  }
  FILE* g = std::fopen(argv[3], "wb");
  if (!g) return 2;
  std::fwrite(&st1, 4, 1, g);
  std::fwrite(&st2, 4, 1, g);
  std::fwrite(&u1, 8, 1, g);
  std::fwrite(&u2, 8, 1, g);
  std::fwrite(e1.data(), sizeof(zc), m, g);
  std::fwrite(e2.data(), sizeof(zc), m, g);
  std::fclose(g);
  return 0;
}
