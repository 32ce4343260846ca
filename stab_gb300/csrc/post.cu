// Post-processing of the spectrum and of the selected eigenvector.
//
//   k_companion_fill   identity / zero lower blocks of the spatial companion
//                      matrix B0 = [[-C0^-1 C1, -C0^-1 C2], [I, 0]]
//                      (spatial.f90:1007-1016)
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
// Least-stable selection (the reference has none; a user picks the mode with
// getevec -v).  With k = sqrt(alpha^2 + beta^2) and c_max = 10 (1 + 1/M):
//   temporal: finite omega, |omega| > 1e-12, |omega| <= c_max max(|k|, 1e-3);
//             largest Im(omega).
//   spatial:  finite alpha != 0, Re(alpha) > 0, |Im(alpha)| <= Re(alpha),
//             |omega/alpha| <= c_max; smallest Im(alpha).
// Ties go to the lower index of the sorted list.
#include "common.cuh"
#include "kernels.cuh"

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
                                zc* __restrict__ least_val) {
  extern __shared__ zc ps[];
  __shared__ double bestv[32];
  __shared__ int besti[32];
  const int k = blockIdx.x;
  if (k >= count) return;
  const InstDesc d = desc[k];
  const int m = d.m;
  const zc* raw = eig_raw + eig_off[k];
  zc* out = eig_sorted + eig_off[k];
  zc* val = ps;  // m
  const bool spatial = (d.itype == 2);
  for (int q = threadIdx.x; q < m; q += blockDim.x) {
    zc l = raw[q];
    if (spatial) l = (l.x != 0.0 || l.y != 0.0) ? zdiv(zmk(1.0, 0.0), l) : zmk(0.0, 0.0);
    val[q] = l;
  }
  __syncthreads();
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
  // selection on the sorted list
  const double M = d.Ma;
  const double cmax = 10.0 * (1.0 + 1.0 / fmax(M, 1e-300));
  const zc al = zmk(d.ar, d.ai), be = zmk(d.br, d.bi), om = zmk(d.wr, d.wi);
  const double kabs = fmax(zabs(zsqrt(zadd(zmul(al, al), zmul(be, be)))), 1e-3);
  double best = -INFINITY;
  int bi = 0x7fffffff;
  for (int q = threadIdx.x; q < m; q += blockDim.x) {
    const zc x = out[q];
    if (!zfinite(x)) continue;
    const double ax = zabs(x);
    double key;
    if (!spatial) {
      if (!(ax > 1e-12) || ax > cmax * kabs) continue;
      key = x.y;
    } else {
      if (ax == 0.0 || !(x.x > 0.0) || fabs(x.y) > x.x) continue;
      if (zabs(zdiv(om, x)) > cmax) continue;
      key = -x.y;
    }
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
    if (bi == 0x7fffffff) {
      least_sorted[k] = -1;
      least_raw[k] = zmk(nan(""), nan(""));
      least_val[k] = zmk(nan(""), nan(""));
    } else {
      least_sorted[k] = bi;
      const zc v = out[bi];
      least_val[k] = v;
      least_raw[k] = spatial ? zdiv(zmk(1.0, 0.0), v) : v;
    }
  }
}

__global__ void k_temporal_vec(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ vec, int slot,
                               zc* __restrict__ out, const int64_t* __restrict__ out_off) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const InstDesc d = desc[k];
  if (d.itype != 1) return;
  const zc* x = vec + d.off_vec + (int64_t)slot * d.n;
  zc* o = out + out_off[k];
  for (int q = threadIdx.x; q < d.n; q += blockDim.x) o[q] = x[q];
}

__global__ void k_spatial_vec(int count, const InstDesc* __restrict__ desc, const zc* __restrict__ theta,
                              const zc* __restrict__ vec, int slot, zc* __restrict__ out,
                              const int64_t* __restrict__ out_off) {
  __shared__ double red[32];
  __shared__ int redi[32];
  __shared__ double s_norm;
  __shared__ int s_k;
  const int k = blockIdx.x;
  if (k >= count) return;
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
