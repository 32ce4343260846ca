// Launchers of the surrogate network kernels (mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace stab {

enum MlpEpilogue { EPI_HIDDEN = 0, EPI_OUT = 1, EPI_DHIDDEN = 2, EPI_WGRAD = 3 };

// tc5: the tcgen05 form (default) or the mma.sync one
cudaError_t mlp_gemm_hidden(int M, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* W, const float* b,
                            float* Z, __nv_bfloat16* H, cudaStream_t s, bool tc5 = true);
cudaError_t mlp_gemm_out(int M, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* W, const float* b,
                         float* Y, cudaStream_t s, bool tc5 = true);
cudaError_t mlp_gemm_dhidden(int M, int N, int K, const __nv_bfloat16* dZ, const __nv_bfloat16* W, const float* Zprev,
                             float* dZprev, __nv_bfloat16* dZprev16, cudaStream_t s, bool tc5 = true);
cudaError_t mlp_gemm_wgrad(int Bsz, int N, int K, const __nv_bfloat16* X, const __nv_bfloat16* dZ, float* G,
                           cudaStream_t s, bool tc5 = true);
// tiles of the tcgen05 form that gave up waiting for their MMAs (sticky
// device flag; reset clears it)
cudaError_t mlp_tc_timeouts(int* out, bool reset);
cudaError_t mlp_loss_grad(int B, int N, const float* Y, int ldy, const float* T, const float* w, float* dy32,
                          __nv_bfloat16* dy16, double* loss, cudaStream_t s);
cudaError_t mlp_bias_grad(int B, int N, const float* dz, float* db, cudaStream_t s);
cudaError_t mlp_adam(int64_t count, float* p, const float* g, float* m, float* v, __nv_bfloat16* p16, float lr,
                     float b1, float b2, float eps, int step, cudaStream_t s);
cudaError_t mlp_cast_bf16(int64_t count, const float* x, __nv_bfloat16* y, cudaStream_t s);

}  // namespace stab
