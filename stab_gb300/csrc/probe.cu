// FMA throughput probes: roofline denominators for the kernels bound by an
// arithmetic pipe that the copy-bandwidth and bf16-GEMM peaks do not cover:
// the FP32 CUDA cores (complex64 LU and solves), the FP64 pipe (operator
// products, plain spectra) and double-word complex arithmetic (seed spectra,
// retry LU), whose multiply-add is the zfma of dw.cuh.  Each thread runs
// independent chains of multiply-adds so the pipe, not the dependency
// latency, sets the rate; the chains' sum is stored only under a condition
// the compiler cannot decide, so no chain is removed.
#include "common.cuh"
#include "dw.cuh"
#include "kernels.cuh"

namespace stab {

constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) k_probe_f32(int iters, float m, float* out) {
  float a[8];
  for (int c = 0; c < 8; ++c) a[c] = 1.0f + 0.001f * (float)(threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = fmaf(a[c], m, 1e-7f);
  }
  float s = 0.f;
  for (int c = 0; c < 8; ++c) s += a[c];
  if (s == -1.0f) out[0] = s;
}

__global__ void __launch_bounds__(kProbeThreads) k_probe_f64(int iters, double m, float* out) {
  double a[8];
  for (int c = 0; c < 8; ++c) a[c] = 1.0 + 0.001 * (double)(threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = fma(a[c], m, 1e-15);
  }
  double s = 0.0;
  for (int c = 0; c < 8; ++c) s += a[c];
  if (s == -1.0) out[0] = (float)s;
}

__global__ void __launch_bounds__(kProbeThreads) k_probe_dz(int iters, float m, float* out) {
  dz a[4];
  for (int c = 0; c < 4; ++c) a[c] = make_float4(1.0f + 0.001f * (float)(threadIdx.x + c), 0.f, 0.5f, 0.f);
  const dz b = make_float4(m, 0.f, 1e-4f, 0.f), k = make_float4(1e-7f, 0.f, -1e-7f, 0.f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 4; ++c) a[c] = zfma(a[c], b, k);
  }
  float s = 0.f;
  for (int c = 0; c < 4; ++c) s += a[c].x + a[c].y + a[c].z + a[c].w;
  if (s == -1.0f) out[0] = s;
}

// kind 0: FP32 FMA, 1: FP64 FMA, 2: double-word complex multiply-add.
// Returns the flops of one launch (2 per real FMA, 8 per complex
// multiply-add, the count the kernels' own flop counters use).
double launch_probe(int kind, int blocks, int iters, float* out, cudaStream_t s) {
  const double threads = (double)blocks * kProbeThreads;
  if (kind == 0) {
    k_probe_f32<<<blocks, kProbeThreads, 0, s>>>(iters, 0.9999999f, out);
    return threads * iters * 8 * 2.0;
  }
  if (kind == 1) {
    k_probe_f64<<<blocks, kProbeThreads, 0, s>>>(iters, 0.9999999999, out);
    return threads * iters * 8 * 2.0;
  }
  k_probe_dz<<<blocks, kProbeThreads, 0, s>>>(iters, 0.9999999f, out);
  return threads * iters * 4 * 8.0;
}

}  // namespace stab
