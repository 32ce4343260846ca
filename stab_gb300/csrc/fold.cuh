// The decision of k_fold_copies for one instance (post.cu), as a host and
// device function so that the CPU tests (tests/host/fold_host.cpp) run the
// code the kernel runs.
//
// The copies c = k * ncand + j (j = 0 .. ncand-1, candidate order) of
// instance k hold copy_done (1: quick-accepted, `unverified`: converged, 0:
// no pair), the selection key of their pair and its eigenvalue copy_theta.
// They fold as the sequential rounds fold an instance's candidates: the less
// stable converged pair wins (ties to the earlier copy), and the first copy
// whose pair was quick-accepted ends the fold.  The instance is trusted
// (dn = 1) when that copy is the top candidate's; any other kept pair is
// `unverified`.
//
// With lam1 (the first level's top candidate), th1 (its polished pair) and
// ok1 (that polish converged), an `unverified` instance is trusted when both
// levels identify the same mode: the top candidates of both seed spectra
// polished to the same pair (within 1e-10), that pair is the least stable
// of every converged copy, and the seed values converge to it: the finer
// level's top candidate (N = max(n1, n2), n1 the first level's N and n2
// this level's, n2t / n2s for temporal / spatial instances) errs by at most
// conv times the coarser one's and by at most 1e-3 relative.
#pragma once

struct FoldPick {
  int pick;   // copy index of the kept pair, -1 for none
  int dn;     // 1 trusted, `unverified`, 0 no pair
};

__host__ __device__ inline FoldPick fold_copies_pick(int k, int ncand, int itype, const int32_t* copy_done,
                                                     const double* copy_key, const zc* copy_theta, int unverified,
                                                     const zc* lam1, const zc* th1, const int32_t* ok1,
                                                     const zc* cand, double conv, int n1, int n2t, int n2s) {
  int pick = -1, dn = 0;
  double bk = 0.0;
  for (int j = 0; j < ncand; ++j) {
    const int c = k * ncand + j;
    const int d = copy_done[c];
    if (d != 1 && d != unverified) continue;
    if (pick < 0 || copy_key[c] > bk) {
      pick = c;
      bk = copy_key[c];
    }
    if (d == 1) {
      dn = (j == 0) ? 1 : unverified;
      break;
    }
  }
  if (pick >= 0 && dn == 0) dn = unverified;
  if (dn == unverified && lam1 && ok1[k]) {
    const int c0 = k * ncand;
    bool top = (copy_done[c0] == 1 || copy_done[c0] == unverified);
    for (int j = 1; j < ncand && top; ++j) {
      const int c = c0 + j;
      if ((copy_done[c] == 1 || copy_done[c] == unverified) && copy_key[c] > copy_key[c0]) top = false;
    }
    if (top) {
      const zc th = copy_theta[c0];
      const double at = zabs(th);
      const double e2 = zabs(zsub(cand[c0], th)), e1 = zabs(zsub(lam1[k], th));
      // the finer seed level must be the closer one
      const int n2 = (itype == 2 || itype == 4) ? n2s : n2t;
      const double ef = (n2 > n1) ? e2 : e1, ec = (n2 > n1) ? e1 : e2;
      if (zabs(zsub(th1[k], th)) <= 1e-10 * at && ef <= conv * ec && ef <= 1e-3 * at) {
        pick = c0;
        dn = 1;
      }
    }
  }
  return FoldPick{pick, dn};
}
