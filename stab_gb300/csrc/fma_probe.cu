// Throughput probe for the FP64 and FP32 roofline denominators (the measured
// copy and bf16 GEMM peaks do not cover them): FMA issue rates with 8
// independent FMA chains per thread.
// Build and run: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fma_probe fma_probe.cu && ./fma_probe
#include <cstdio>
#include <cuda_runtime.h>
template <typename T>
__global__ void fma_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template <typename T>
void run(const char* name, int blocks, int threads, int iters) {
  T* out; cudaMalloc(&out, sizeof(T) * blocks * threads);
  fma_kernel<T><<<blocks, threads>>>(out, 10, (T)0.999, (T)0.001);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  cudaEventRecord(e0);
  fma_kernel<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1);
  double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  printf("%s blocks=%d threads=%d: %.3f ms  %.2f TFLOP/s\n", name, blocks, threads, ms, flops / ms / 1e9);
  cudaFree(out);
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  cudaDeviceProp pr; cudaGetDeviceProperties(&pr, 0);
  printf("device %s sms=%d cc=%d.%d smem/block optin=%zu l2=%d\n", pr.name, sms, pr.major, pr.minor, pr.sharedMemPerBlockOptin, pr.l2CacheSize);
  run<double>("fp64", sms * 4, 256, 4096);
  run<double>("fp64", sms * 8, 256, 4096);
  run<float>("fp32", sms * 8, 256, 65536);
  run<float>("fp32", sms * 16, 256, 65536);
  return 0;
}
