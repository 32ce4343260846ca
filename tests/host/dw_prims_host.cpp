// CPU build of the double-word primitives (stab_gb300/csrc/dw.cuh) for the
// host tests.  Random operands (fixed seed) over 40 binary orders of
// magnitude and both signs; each result is compared with the same operation
// in long double (at least 64 significant bits).  Prints one line per
// primitive: name, max error, and what the error is relative to.
#include <cstdio>
#include <random>
#include <vector>

#include "cuda_host_shim.h"

#include "../../stab_gb300/csrc/common.cuh"
#include "../../stab_gb300/csrc/dw.cuh"

typedef long double LD;

static LD val(dw x) { return (LD)x.x + (LD)x.y; }
static LD re(dz a) { return (LD)a.x + (LD)a.y; }
static LD im(dz a) { return (LD)a.z + (LD)a.w; }

int main() {
  std::mt19937_64 gen(20261204);
  std::uniform_real_distribution<double> u(-1.0, 1.0), ex(-20.0, 20.0);
  auto rnd = [&] {   // a double with a random sign and binary exponent in [-20, 20]
    return u(gen) * std::ldexp(1.0, (int)ex(gen));
  };
  auto to_dw = [](double v) { return dw_from64(v); };
  const int n = 200000;
  LD e_add = 0, e_mul = 0, e_fma = 0, e_rcp = 0, e_rsq = 0, e_zfma = 0, e_div = 0, e_norm = 0;
  for (int t = 0; t < n; ++t) {
    const dw x = to_dw(rnd()), y = to_dw(rnd()), c = to_dw(rnd());
    const LD X = val(x), Y = val(y), Cv = val(c);
    // sum: error relative to |x| + |y| (no relative bound under cancellation)
    const dw s = dw_add(x, y);
    e_add = std::max(e_add, std::fabs(val(s) - (X + Y)) / (std::fabs(X) + std::fabs(Y)));
    // a normalised result: |l| <= ulp(h)
    e_norm = std::max(e_norm, (LD)std::fabs(s.y) / ((LD)std::fabs(s.x) + 1e-300L) / (LD)std::ldexp(1.0, -23));
    const dw p = dw_mul(x, y);
    e_mul = std::max(e_mul, std::fabs(val(p) - X * Y) / std::fabs(X * Y));
    const dw f = dw_fma(x, y, c);
    e_fma = std::max(e_fma, std::fabs(val(f) - (X * Y + Cv)) / (std::fabs(X * Y) + std::fabs(Cv)));
    const dw r = dw_rcp(x);
    e_rcp = std::max(e_rcp, std::fabs(val(r) * X - 1));
    const dw ax = make_float2(std::fabs(x.x), x.x < 0 ? -x.y : x.y);   // |x|
    const dw q = dw_rsqrt(ax);
    e_rsq = std::max(e_rsq, std::fabs(val(q) * val(q) * val(ax) - 1));
    // complex multiply-add and division
    const dz a = dz_mk(x, y), b = dz_mk(c, to_dw(rnd())), d = dz_mk(to_dw(rnd()), to_dw(rnd()));
    const LD ar = re(a), ai = im(a), br = re(b), bi = im(b), dr = re(d), di = im(d);
    const dz g = zfma(a, b, d);
    const LD gr = ar * br - ai * bi + dr, gi = ar * bi + ai * br + di;
    const LD scale = std::hypot(ar, ai) * std::hypot(br, bi) + std::hypot(dr, di);
    e_zfma = std::max(e_zfma, std::hypot(re(g) - gr, im(g) - gi) / scale);
    const dz h = cx<dz>::div(a, b);
    const LD den = br * br + bi * bi;
    const LD hr = (ar * br + ai * bi) / den, hi = (ai * br - ar * bi) / den;
    e_div = std::max(e_div, std::hypot(re(h) - hr, im(h) - hi) / std::hypot(hr, hi));
  }
  std::printf("dw_add %.3Le of |x|+|y|\n", e_add);
  std::printf("dw_add_norm %.3Le of 2^-23 |h|\n", e_norm);
  std::printf("dw_mul %.3Le relative\n", e_mul);
  std::printf("dw_fma %.3Le of |xy|+|c|\n", e_fma);
  std::printf("dw_rcp %.3Le relative\n", e_rcp);
  std::printf("dw_rsqrt %.3Le relative (of r^2 s)\n", e_rsq);
  std::printf("zfma %.3Le of |a||b|+|c|\n", e_zfma);
  std::printf("zdiv %.3Le relative\n", e_div);
  return 0;
}
