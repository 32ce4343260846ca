// Host launchers of the batched LU / triangular-solve kernels (lu.cu).
#pragma once
#include <vector>
#include <cuda.h>
#include "common.cuh"

namespace stab {
// Factor count column-major matrices (n = nsz[k], nmax = max n) in place.
// piv receives 0-based absolute pivot rows; info[k] = 1-based index of the
// first exactly-zero pivot, 0 if none (ZGETRF's INFO convention).
template <typename T>
cudaError_t launch_lu(int count, const InstDesc* desc, const int32_t* nsz, int nmax, T* A, const int64_t* mat_off,
                      int32_t* piv, const int64_t* piv_off, int32_t* info, cudaStream_t s,
                      const int32_t* skip = nullptr, int nb_hint = 0, const int32_t* order = nullptr,
                      int cluster = 1);
// widest panel the shared memory admits for order n (8, 16 or 32)
template <typename T>
int lu_nb_max(int n);
// autotuning input: count well-conditioned n x n test matrices
template <typename T>
cudaError_t launch_tune_matrix(int count, int n, T* A, cudaStream_t s);
// Solve with the factors for complex128 right-hand sides at X + x_off[k]:
// nrhs = nrhs_fixed if > 0, else nrhs_mul * n; leading dimension ldmul * n.
// The solve runs in the factor's precision; instances with skip[k] != 0
// (skip may be null) are left alone.
template <typename T>
cudaError_t launch_getrs(int count, const int32_t* nsz, int nmax, const T* LU, const int64_t* mat_off,
                         const int32_t* piv, const int64_t* piv_off, zc* X, const int64_t* x_off, int nrhs_fixed,
                         int nrhs_mul, int ldmul, const int32_t* skip, cudaStream_t s, const float* rs = nullptr,
                         const float* cs = nullptr);
// Power-of-two row/column equilibration of complex64 matrices (scales stored
// at rs/cs + sc_off[k]); pass the same rs/cs to launch_getrs.
cudaError_t launch_equilibrate(int count, const int32_t* nsz, cc* A, const int64_t* mat_off, float* rs, float* cs,
                               const int64_t* sc_off, cudaStream_t s, const int32_t* skip = nullptr);
// Complex64 LU with the trailing update on the tensor cores (lu_tc.cu):
// same inputs, outputs and pivot order as launch_lu<cc> with panel width 16.
// info[k] = -1 marks an instance whose MMA completion was not seen.
// tmaps (device, one per instance, or null): tensor maps of the matrices
// (lu_tc_tensor_maps) for the TMA tile path.
cudaError_t launch_lu_tc(int count, const int32_t* nsz, int nmax, cc* A, const int64_t* mat_off, int32_t* piv,
                         const int64_t* piv_off, int32_t* info, cudaStream_t s, const int32_t* skip = nullptr,
                         const int32_t* order = nullptr, const CUtensorMap* tmaps = nullptr);
// dynamic shared memory of k_lu_tc for order nmax, and whether it fits
size_t lu_tc_smem(int nmax, bool tma = false);
bool lu_tc_fits(int nmax, bool tma = false);
// host: the tensor maps of count matrices at base + off[k] (orders n[k]);
// false if any order or offset is odd or the encoder is unavailable
bool lu_tc_tensor_maps(int count, const int32_t* n, const int64_t* off, cc* base, std::vector<CUtensorMap>& out);
}  // namespace stab
