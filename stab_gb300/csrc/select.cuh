// Least-stable selection rule shared by the spectrum post-processing and the
// choice between polished candidates.  The reference has no such rule (a user
// picks the mode with getevec -v, getevec.f90:161-172); this one is:
// with k = sqrt(alpha^2 + beta^2) and c_max = 10 (1 + 1/M),
//   temporal: finite omega, |omega| > 1e-12, |omega| <= c_max max(|k|, 1e-3);
//             key = Im(omega), larger is less stable.
//   spatial:  finite alpha != 0, Re(alpha) > 0, |Im(alpha)| <= Re(alpha),
//             |omega/alpha| <= c_max, and, in a full spectrum, lambda =
//             1/alpha not below 1e-6 max_j |lambda_j| (the companion's zero
//             eigenvalues come out of FP64 at rounding level, as large
//             alpha of arbitrary phase; a defective zero perturbs like
//             sqrt(eps)); key = -Im(alpha).
#pragma once
#include "common.cuh"

namespace stab {

// amax: the largest |alpha| a spatial full spectrum admits (1e6 / max |lambda|);
// infinite for single polished values
__device__ __forceinline__ bool least_key(const InstDesc& d, zc x, double& key, double amax = INFINITY) {
  if (!(isfinite(x.x) && isfinite(x.y))) return false;
  const double cmax = 10.0 * (1.0 + 1.0 / fmax(d.Ma, 1e-300));
  const double ax = zabs(x);
  if (d.itype == 1) {
    const zc al = zmk(d.ar, d.ai), be = zmk(d.br, d.bi);
    const double kabs = fmax(zabs(zsqrt(zadd(zmul(al, al), zmul(be, be)))), 1e-3);
    if (!(ax > 1e-12) || ax > cmax * kabs) return false;
    key = x.y;
    return true;
  }
  if (ax == 0.0 || !(x.x > 0.0) || fabs(x.y) > x.x || ax > amax) return false;
  if (zabs(zdiv(zmk(d.wr, d.wi), x)) > cmax) return false;
  key = -x.y;
  return true;
}

}  // namespace stab
