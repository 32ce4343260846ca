// Post-processing of the spectrum and of the selected eigenvector.
//
//   k_companion_fill   identity / zero lower blocks of the spatial companion
//                      matrix B0 = [[-C0^-1 C1, -C0^-1 C2], [I, 0]]
//                      (spatial.f90:1007-1016)
//   k_take_candidate,  seed rounds of the coarse-shift mode
//   k_fold_best,
//   k_take_best
//   k_converged_mask   complex128 retry of the seeded modes
//   k_post_spectrum    alpha = 1/lambda with lambda = 0 -> 0
//                      (spatial.f90:1065-1069), ascending stable sort on the
//                      imaginary part (the PIKSR2 call, temporal.f90:844-855,
//                      spatial.f90:1073-1084) and selection of the
//                      least-stable mode (rule below)
//   k_temporal_vec     evec column divided by its first max-modulus entry
//                      (temporal.f90:867-879)
//   k_spatial_vec      companion eigenvector [lambda phi; phi] scaled to unit
//                      2-norm with its first max-modulus entry real positive
//                      (the convention of the ZGEEV call, spatial.f90:1043)
//
// The least-stable selection rule is stated in select.cuh.
#include "common.cuh"
#include "kernels.cuh"
#include "fold.cuh"
#include "select.cuh"

namespace stab {

__global__ void k_companion_fill(int count, const InstDesc* __restrict__ desc, zc* __restrict__ A,
                                 const int64_t* __restrict__ a_off) {
  const int k = blockIdx.y;
  if (k >= count) return;
  const InstDesc d = desc[k];
  const int n = d.n, m = 2 * n;
  const int c = blockIdx.x;
  if (c >= m) return;
  zc* col = A + a_off[k] + (int64_t)c * m;
  for (int r = n + threadIdx.x; r < m; r += blockDim.x) col[r] = zmk((c < n && r - n == c) ? 1.0 : 0.0, 0.0);
}

__device__ __forceinline__ bool zfinite(zc a) { return isfinite(a.x) && isfinite(a.y); }

__global__ void k_post_spectrum(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ eig_raw,
                                const int64_t* __restrict__ eig_off, zc* __restrict__ eig_sorted,
                                int32_t* __restrict__ least_sorted, zc* __restrict__ least_raw,
                                zc* __restrict__ least_val, zc* __restrict__ cand, int ncand) {
  extern __shared__ zc ps[];
  __shared__ double bestv[32];
  __shared__ int besti[32];
  __shared__ double s_amax;
  const int k = blockIdx.x;
  if (k >= count) return;
  const InstDesc d = desc[k];
  const int m = d.m;
  const zc* raw = eig_raw + eig_off[k];
  zc* out = eig_sorted + eig_off[k];
  zc* val = ps;  // m
  const bool spatial = (d.itype == 2);
  double lmax = 0.0;   // largest finite |lambda| of a spatial spectrum
  for (int q = threadIdx.x; q < m; q += blockDim.x) {
    zc l = raw[q];
    if (spatial) {
      const double al = zabs(l);
      if (isfinite(al)) lmax = fmax(lmax, al);
      l = (l.x != 0.0 || l.y != 0.0) ? zdiv(zmk(1.0, 0.0), l) : zmk(0.0, 0.0);
    }
    val[q] = l;
  }
  for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_down_sync(0xffffffffu, lmax, o));
  if ((threadIdx.x & 31) == 0) bestv[threadIdx.x >> 5] = lmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) lmax = fmax(lmax, bestv[w]);
    s_amax = (spatial && lmax > 0.0) ? 1e6 / lmax : INFINITY;
  }
  __syncthreads();
  const double amax = s_amax;
  // stable ascending sort on Im: rank = #{j: key_j < key_q} + #{j < q: key_j == key_q}
  for (int q = threadIdx.x; q < m; q += blockDim.x) {
    const double kq = val[q].y;
    int r = 0;
    for (int j = 0; j < m; ++j) {
      const double kj = val[j].y;
      r += (kj < kq) || (kj == kq && j < q);
    }
    out[r] = val[q];
  }
  __syncthreads();
  // selection on the sorted list: the least-stable mode, then (for shift
  // candidates) the next best modes that differ from all earlier picks by
  // more than 1e-6 relative
  __shared__ int s_pick[8];
  const int npass = (cand && ncand > 1) ? (ncand < 8 ? ncand : 8) : 1;
  for (int pass = 0; pass < npass; ++pass) {
    double best = -INFINITY;
    int bi = 0x7fffffff;
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
      const zc x = out[q];
      double key;
      if (!least_key(d, x, key, amax)) continue;
      bool dup = false;
      for (int pp = 0; pp < pass; ++pp) dup |= zabs(zsub(x, out[s_pick[pp]])) <= 1e-6 * zabs(out[s_pick[pp]]);
      if (dup) continue;
      if (key > best || (key == best && q < bi)) { best = key; bi = q; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { bestv[warp] = best; besti[warp] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        if (bestv[w] > best || (bestv[w] == best && besti[w] < bi)) { best = bestv[w]; bi = besti[w]; }
      const bool none = (bi == 0x7fffffff);
      const zc v = none ? zmk(nan(""), nan("")) : out[bi];
      const zc raw = none ? v : (spatial ? zdiv(zmk(1.0, 0.0), v) : v);
      if (pass == 0) {
        least_sorted[k] = none ? -1 : bi;
        least_val[k] = v;
        least_raw[k] = raw;
      }
      if (cand) cand[(int64_t)k * ncand + pass] = raw;
      s_pick[pass] = none ? -1 : bi;
    }
    __syncthreads();
    if (s_pick[pass] < 0) {
      if (threadIdx.x == 0 && cand)
        for (int pp = pass + 1; pp < ncand; ++pp) cand[(int64_t)k * ncand + pp] = zmk(nan(""), nan(""));
      break;
    }
  }
}

// Retry bookkeeping of the seeded modes: mask[k] = (done[k] == 1) before the
// complex128 inverse iteration, which marks the instances it skips done = 4;
// with `restore` the converged instances get done = 1 back afterwards.
__global__ void k_converged_mask(int count, int32_t* __restrict__ done, int32_t* __restrict__ mask, int restore) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  if (!restore) mask[k] = (done[k] == 1) ? 1 : 0;
  else if (mask[k]) done[k] = 1;
}

// sigma[k] <- candidate j of instance k
__global__ void k_take_candidate(int count, const zc* __restrict__ cand, int ncand, int j, zc* __restrict__ sigma) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  sigma[k] = cand[(int64_t)k * ncand + j];
}

// Fold the result of a polish round into the per-instance best: a pair
// counts when it converged and passes the selection filter; the less stable
// one is kept (theta, err, iters and the output vector).  With `quick`, a
// pair within quick_tol of its shift is final: that coarse candidate is a
// resolved mode, the candidates after it are less stable at N = 32, and
// later rounds skip the instance.
__global__ void k_fold_best(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ sigma,
                            const zc* __restrict__ theta, const int32_t* __restrict__ done,
                            const double* __restrict__ err, const int32_t* __restrict__ iters,
                            const zc* __restrict__ out, const int64_t* __restrict__ out_off,
                            int32_t* __restrict__ final_, int32_t* __restrict__ have, double* __restrict__ best_key,
                            zc* __restrict__ best_theta, double* __restrict__ best_err, int32_t* __restrict__ best_iters,
                            zc* __restrict__ best_out, int quick, double quick_tol, int32_t* __restrict__ skip64,
                            int slow_iters, int src, int32_t* __restrict__ best_src) {
  __shared__ int s_take;
  const int k = blockIdx.x;
  if (k >= count) return;
  if (final_[k]) {
    if (skip64 && threadIdx.x == 0) skip64[k] = 1;   // accepted: no retry
    return;
  }
  const InstDesc d = desc[k];
  if (threadIdx.x == 0) {
    s_take = 0;
    // a complex128 retry only where the complex64 polish failed or
    // contracted slowly (the sign of a cluster it cannot resolve)
    if (skip64) skip64[k] = (done[k] == 1 && iters[k] < slow_iters) ? 1 : 0;   // complex64 round: set retries
    const zc t = theta[k];
    const zc v = (d.itype == 2) ? ((t.x != 0.0 || t.y != 0.0) ? zdiv(zmk(1.0, 0.0), t) : t) : t;
    double key;
    if (done[k] == 1 && least_key(d, v, key)) {
      if (!have[k] || key > best_key[k]) {
        have[k] = 1;
        best_key[k] = key;
        best_theta[k] = t;
        best_err[k] = err[k];
        best_iters[k] = iters[k];
        if (best_src) best_src[k] = src;
        s_take = 1;
      }
      // quick accept: final_ = 1 + the candidate's index (1: the top candidate)
      if (quick && zabs(zsub(t, sigma[k])) <= quick_tol * zabs(sigma[k])) final_[k] = 1 + src;
    }
    if (skip64 && final_[k]) skip64[k] = 1;
  }
  __syncthreads();
  if (!s_take) return;
  const int64_t o = out_off[k];
  for (int q = threadIdx.x; q < d.m; q += blockDim.x) best_out[o + q] = out[o + q];
}

// After the rounds: the best pair becomes the result.  It is trusted
// (done = 1) only where the top candidate of the seed spectrum (the most
// unstable one after the selection filter) polished to within the quick-
// accept distance of itself (final_[k] == 1): the seed spectrum resolved its
// most unstable mode and the polish landed on it.  Otherwise a mode the seed
// spectrum did not resolve may be more unstable than the kept pair: the
// instance gets done = 0 and goes to the fallback chain, unless
// keep_unverified is set (the last seed level) or the pair came from the
// caller's seed round (best_src == seed_src), which keep it with done =
// unverified.  Instances without any converged pair get done = 0.
__global__ void k_take_best(int count, const InstDesc* __restrict__ desc, const int32_t* __restrict__ have,
                            const zc* __restrict__ best_theta, const double* __restrict__ best_err,
                            const int32_t* __restrict__ best_iters, const zc* __restrict__ best_out,
                            const int64_t* __restrict__ out_off, zc* __restrict__ theta, int32_t* __restrict__ done,
                            double* __restrict__ err, int32_t* __restrict__ iters, zc* __restrict__ out,
                            const int32_t* __restrict__ final_, const int32_t* __restrict__ best_src, int seed_src,
                            int unverified, int keep_unverified) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const InstDesc d = desc[k];
  int dn = have[k] ? 1 : 0;
  if (dn && final_[k] != 1) dn = (best_src[k] == seed_src || keep_unverified) ? unverified : 0;
  if (!dn) {
    if (threadIdx.x == 0) done[k] = 0;
    return;
  }
  if (threadIdx.x == 0) {
    theta[k] = best_theta[k];
    done[k] = dn;
    err[k] = best_err[k];
    iters[k] = best_iters[k];
  }
  const int64_t o = out_off[k];
  for (int q = threadIdx.x; q < d.m; q += blockDim.x) out[o + q] = best_out[o + q];
}

// Candidate copies (one instance per shift candidate, so that the candidates
// of a small batch are polished side by side rather than one round after
// another): copy c = k * ncand + j of instance k takes candidate j as its
// own top candidate; a missing candidate (NaN) marks the copy final with no
// pair (final = 2), so its rounds skip it.
__global__ void k_spread_candidates(int ncopy, const zc* __restrict__ cand, int ncand, zc* __restrict__ copy_cand) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncopy) return;
  copy_cand[(int64_t)c * ncand] = cand[c];
  for (int j = 1; j < ncand; ++j) copy_cand[(int64_t)c * ncand + j] = zmk(nan(""), nan(""));
}

// The first candidate level's view of the instances that reach the second:
// lam1 = top candidate of its seed spectrum, th1 = that candidate's polished
// pair and ok1 = it converged (have, and the kept pair came from the top
// candidate); idx maps second-level instances to first-level ones.
__global__ void k_gather_level(int count, const int32_t* __restrict__ idx, const zc* __restrict__ cand, int ncand,
                               const zc* __restrict__ best_theta, const int32_t* __restrict__ have,
                               const int32_t* __restrict__ best_src, zc* __restrict__ lam1, zc* __restrict__ th1,
                               int32_t* __restrict__ ok1) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= count) return;
  const int k = idx[q];
  lam1[q] = cand[(int64_t)k * ncand];
  th1[q] = best_theta[k];
  ok1[q] = (have[k] && best_src[k] == 0) ? 1 : 0;
}

__global__ void k_mark_missing(int count, const zc* __restrict__ cand, int ncand, int32_t* __restrict__ final_) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= count) return;
  const zc v = cand[(int64_t)c * ncand];
  if (!(isfinite(v.x) && isfinite(v.y))) final_[c] = 2;
}

// Fold the copies of each instance (k = blockIdx.x): thread 0 takes the
// decision of fold_copies_pick (fold.cuh: the sequential rounds' rule and
// the agreement of the two seed levels), then the block copies the kept
// pair's eigenvector.
__global__ void k_fold_copies(int count, int ncand, const InstDesc* __restrict__ desc,
                              const int32_t* __restrict__ copy_done, const double* __restrict__ copy_key,
                              const zc* __restrict__ copy_theta, const double* __restrict__ copy_err,
                              const int32_t* __restrict__ copy_iters, const zc* __restrict__ copy_out,
                              const int64_t* __restrict__ copy_out_off, zc* __restrict__ theta,
                              int32_t* __restrict__ done, double* __restrict__ err, int32_t* __restrict__ iters,
                              zc* __restrict__ out, const int64_t* __restrict__ out_off, int unverified,
                              const zc* __restrict__ lam1, const zc* __restrict__ th1, const int32_t* __restrict__ ok1,
                              const zc* __restrict__ cand, double conv, int n1, int n2t, int n2s) {
  __shared__ int s_pick;
  const int k = blockIdx.x;
  if (k >= count) return;
  if (threadIdx.x == 0) {
    const FoldPick f = fold_copies_pick(k, ncand, desc[k].itype, copy_done, copy_key, copy_theta, unverified, lam1,
                                        th1, ok1, cand, conv, n1, n2t, n2s);
    const int pick = f.pick, dn = f.dn;
    done[k] = dn;
    if (pick >= 0) {
      theta[k] = copy_theta[pick];
      err[k] = copy_err[pick];
      iters[k] = copy_iters[pick];
    }
    s_pick = pick;
  }
  __syncthreads();
  const int pick = s_pick;
  if (pick < 0) return;
  const int m = desc[k].m;
  const zc* src = copy_out + copy_out_off[pick];
  zc* dst = out + out_off[k];
  for (int q = threadIdx.x; q < m; q += blockDim.x) dst[q] = src[q];
}

__global__ void k_temporal_vec(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ vec, int slot,
                               zc* __restrict__ out, const int64_t* __restrict__ out_off,
                               const int32_t* __restrict__ skip) {
  const int k = blockIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  if (d.itype != 1) return;
  const zc* x = vec + d.off_vec + (int64_t)slot * d.n;
  zc* o = out + out_off[k];
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) o[q] = x[q];
}

__global__ void k_spatial_vec(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ theta,
                              const zc* __restrict__ vec, int slot, zc* __restrict__ out,
                              const int64_t* __restrict__ out_off, const int32_t* __restrict__ skip) {
  __shared__ double red[32];
  __shared__ int redi[32];
  __shared__ double s_norm;
  __shared__ int s_k;
  const int k = blockIdx.x;
  if (k >= count) return;
  if (skip && skip[k]) return;
  const InstDesc d = desc[k];
  if (d.itype != 2) return;
  const int n = d.n;
  const zc* x = vec + d.off_vec + (int64_t)slot * n;
  zc* o = out + out_off[k];
  const zc t = theta[k];
  double ss = 0.0;
  for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) {
    const zc v = (q < n) ? zmul(t, x[q]) : x[q - n];
    o[q] = v;
    ss += v.x * v.x + v.y * v.y;
  }
  for (int o2 = 16; o2 > 0; o2 >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, o2);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[w];
    s_norm = sqrt(a);
  }
  __syncthreads();
  const double inv = (s_norm > 0.0) ? 1.0 / s_norm : 1.0;
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) {
    zc v = zscale(o[q], inv);
    o[q] = v;
    const double a = v.x * v.x + v.y * v.y;
    if (a > best || (a == best && q < bi)) { best = a; bi = q; }
  }
  for (int o2 = 16; o2 > 0; o2 >>= 1) {
    const double ob = __shfl_down_sync(0xffffffffu, best, o2);
    const int oi = __shfl_down_sync(0xffffffffu, bi, o2);
    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
  }
  __syncthreads();
  if (lane == 0) { red[warp] = best; redi[warp] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (red[w] > best || (red[w] == best && redi[w] < bi)) { best = red[w]; bi = redi[w]; }
    if (bi < 0 || bi >= 2 * n) bi = 0;   // no finite entry
    s_k = bi;
  }
  __syncthreads();
  const zc vk = o[s_k];
  const double mk = zabs(vk);
  __syncthreads();
  if (mk == 0.0) return;
  const zc ph = zscale(zconj(vk), 1.0 / mk);
  for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) o[q] = (q == s_k) ? zmk(mk, 0.0) : zmul(o[q], ph);
}

}  // namespace stab
