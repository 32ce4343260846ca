// CPU build of the batched LU's body (stab_gb300/csrc/lu_body.cuh) for the
// host tests, with the CUDA thread model of cuda_host_shim.h: one 256-thread
// CTA (eight warps) factors one matrix, panel width 16, in complex64,
// double-word and complex128.
//
//   lu_host IN OUT   IN: int32 n, n*n complex128 column-major
// OUT, per type (complex64, double-word, complex128): int32 info, n int32
// pivots (0-based row swapped with row j at step j), n*n complex128 factors
// (L below the diagonal, unit diagonal implied; U on and above).
#include <cstdio>
#include <vector>

#include "cuda_host_shim.h"

#include "../../stab_gb300/csrc/common.cuh"
#include "../../stab_gb300/csrc/dw.cuh"

// the cluster calls sit in branches for clusters of more than one CTA, which
// this build does not instantiate
namespace cg {
struct host_cluster {
  unsigned block_rank() const { return 0; }
  void sync() const {}
};
inline host_cluster this_cluster() { return {}; }
}  // namespace cg

namespace stab {
#include "../../stab_gb300/csrc/lu_body.cuh"
}  // namespace stab

using namespace stab;

template <class T>
static void factor(const std::vector<zc>& A, int n, FILE* out) {
  constexpr int NB = 16;
  std::vector<T> M((size_t)n * n);
  for (size_t q = 0; q < M.size(); ++q) M[q] = cx<T>::from(A[q]);
  std::vector<int32_t> ip(n, -1);
  int32_t info = -1;
  const int32_t nsz = n;
  const int64_t off = 0;
  std::vector<unsigned char> smraw((size_t)n * NB * sizeof(T) + (size_t)NB * 65 * sizeof(T) + 16);
  static typename cx<T>::real red_v[256 / 32];
  static int red_i[256 / 32];
  static int s_piv;
  host_block(256);
  std::vector<std::thread> th;
  for (int t = 0; t < 256; ++t)
    th.emplace_back([&, t] {
      g_tid = t;
      lu_body<T, NB, 1>(0, 0, &nsz, M.data(), &off, ip.data(), &off, &info, smraw.data(), red_v, red_i, s_piv);
    });
  for (auto& x : th) x.join();
  std::fwrite(&info, 4, 1, out);
  std::fwrite(ip.data(), 4, n, out);
  for (size_t q = 0; q < M.size(); ++q) {
    const zc v = cx<T>::to64(M[q]);
    std::fwrite(&v, sizeof(zc), 1, out);
  }
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int n = 0;
  if (std::fread(&n, 4, 1, f) != 1 || n < 1 || n > 2048) return 2;
  std::vector<zc> A((size_t)n * n);
  if (std::fread(A.data(), sizeof(zc), A.size(), f) != A.size()) return 2;
  std::fclose(f);
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 2;
  factor<cc>(A, n, g);
  factor<dz>(A, n, g);
  factor<zc>(A, n, g);
  std::fclose(g);
  return 0;
}
