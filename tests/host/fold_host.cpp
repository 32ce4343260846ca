// CPU build of the second candidate level's fold decision (fold.cuh, the
// code k_fold_copies runs per instance) on crafted copies: the sequential
// fold order, ties, quick accepts, and every condition of the agreement of
// the two seed levels.  Prints one line per case and exits non-zero if any
// case disagrees with its expected (pick, dn).
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "../../stab_gb300/csrc/common.cuh"
#include "../../stab_gb300/csrc/fold.cuh"

namespace {
const int K = 4, UNV = 5;

struct Case {
  const char* name;
  int itype;
  int done[K];
  double key[K];
  bool lev1;        // first-level data present and converged
  double th1_rel;   // |th1 - th| / |th| of copy 0's pair
  double e1_rel;    // |lam1 - th| / |th|
  double e2_rel;    // |cand0 - th| / |th| (this level's top candidate)
  int n1, n2t, n2s;
  int want_pick, want_dn;
};

int run(const Case& q) {
  const zc th = zmk(0.3, -2e-4);
  const double at = zabs(th);
  std::vector<int32_t> done(q.done, q.done + K);
  std::vector<double> key(q.key, q.key + K);
  std::vector<zc> theta(K, th), cand(K, th);
  cand[0] = zmk(th.x + q.e2_rel * at, th.y);                       // this level's top candidate
  const zc lam1 = zmk(th.x, th.y + q.e1_rel * at);                 // first level's top candidate
  const zc th1 = zmk(th.x + q.th1_rel * at, th.y);                 // its polished pair
  const int32_t ok1 = q.lev1 ? 1 : 0;
  const FoldPick f = fold_copies_pick(0, K, q.itype, done.data(), key.data(), theta.data(), UNV,
                                      q.lev1 ? &lam1 : nullptr, &th1, &ok1, cand.data(), 0.25, q.n1, q.n2t, q.n2s);
  const bool ok = (f.pick == q.want_pick && f.dn == q.want_dn);
  std::printf("%-58s pick %2d dn %d  %s\n", q.name, f.pick, f.dn, ok ? "ok" : "MISMATCH");
  return ok ? 0 : 1;
}
}  // namespace

int main() {
  const Case cases[] = {
      // name                                               itype done            key              lev1 th1  e1    e2    n1 n2t n2s pick dn
      {"top candidate quick-accepted", 1, {1, UNV, UNV, 0}, {1, 5, 6, 0}, false, 0, 0, 0, 32, 48, 24, 0, 1},
      {"copy 1 accepted, copy 0 less stable: keep copy 0", 1, {UNV, 1, 0, 0}, {3, 2, 0, 0}, false, 0, 0, 0, 32, 48, 24, 0, UNV},
      {"copy 1 accepted and less stable: keep it, unverified", 1, {UNV, 1, UNV, 0}, {2, 3, 9, 0}, false, 0, 0, 0, 32, 48, 24, 1, UNV},
      {"no converged copy", 1, {0, 0, 0, 0}, {0, 0, 0, 0}, false, 0, 0, 0, 32, 48, 24, -1, 0},
      {"equal keys: the earlier copy", 1, {UNV, UNV, 0, 0}, {2, 2, 0, 0}, false, 0, 0, 0, 32, 48, 24, 0, UNV},
      {"agreement, N = 48 closer (temporal)", 1, {UNV, UNV, 0, 0}, {3, 1, 0, 0}, true, 1e-12, 1e-4, 1e-6, 32, 48, 24, 0, 1},
      {"agreement, but N = 48 not 4x closer", 1, {UNV, UNV, 0, 0}, {3, 1, 0, 0}, true, 1e-12, 1e-5, 5e-6, 32, 48, 24, 0, UNV},
      {"agreement, but another copy less stable", 1, {UNV, UNV, UNV, 0}, {3, 1, 4, 0}, true, 1e-12, 1e-4, 1e-6, 32, 48, 24, 2, UNV},
      {"first level polished elsewhere", 1, {UNV, 0, 0, 0}, {3, 0, 0, 0}, true, 1e-8, 1e-4, 1e-6, 32, 48, 24, 0, UNV},
      {"first level did not converge", 1, {UNV, 0, 0, 0}, {3, 0, 0, 0}, false, 1e-12, 1e-4, 1e-6, 32, 48, 24, 0, UNV},
      {"spatial: N = 24 level, N = 32 the finer and closer", 2, {UNV, 0, 0, 0}, {3, 0, 0, 0}, true, 1e-12, 1e-5, 1e-3, 32, 48, 24, 0, 1},
      {"spatial: the finer N = 32 level is the farther", 2, {UNV, 0, 0, 0}, {3, 0, 0, 0}, true, 1e-12, 1e-3, 1e-5, 32, 48, 24, 0, UNV},
      {"finer level above 1e-3 relative", 1, {UNV, 0, 0, 0}, {3, 0, 0, 0}, true, 1e-12, 1e-1, 2e-3, 32, 48, 24, 0, UNV},
      {"accepted at copy 2 after less stable copy 0", 1, {UNV, 0, 1, UNV}, {5, 0, 1, 9}, true, 1e-12, 1e-4, 1e-6, 32, 48, 24, 0, UNV},
  };
  int bad = 0;
  for (const Case& q : cases) bad += run(q);
  return bad ? 1 : 0;
}
