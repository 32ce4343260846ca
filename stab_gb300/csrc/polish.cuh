// Host launchers of the mixed-precision polish kernels (polish.cu).
#pragma once
#include "common.cuh"

namespace stab {
cudaError_t launch_qmv(int count, int nmax, const InstDesc* desc, const double* const* dtab, const zc* blk,
                       const zc* theta, int deriv, zc* vec, int xslot, int yslot, const int32_t* skip,
                       cudaStream_t s);
cudaError_t launch_vec_init(int count, int nmax, const InstDesc* desc, zc* vec, int slot, cudaStream_t s,
                            const int32_t* skip = nullptr);
cudaError_t launch_normalize(int count, const InstDesc* desc, zc* vec, int slot, int32_t* piv_out,
                             const int32_t* skip, cudaStream_t s);
template <typename T>
cudaError_t launch_set_column(int count, int nmax, const InstDesc* desc, T* M, const int64_t* m_off,
                              const int32_t* pcol, const zc* vec, int slot, cudaStream_t s,
                              const int32_t* skip = nullptr);
cudaError_t launch_vec_copy(int count, int nmax, const InstDesc* desc, zc* vec, int a, int b, const int32_t* skip,
                            cudaStream_t s);
cudaError_t launch_newton_update(int count, const InstDesc* desc, zc* vec, int xslot, int dslot, const int32_t* pcol,
                                 zc* theta, int32_t* done, double* err, int32_t* iters, double tol, double tol_vec,
                                 cudaStream_t s, const int32_t* skip = nullptr);
cudaError_t launch_start_shift(int count, const zc* sigma, zc* theta, const int32_t* skip, cudaStream_t s);
cudaError_t launch_reset_polish(int count, int32_t* done, int32_t* iters, const int32_t* skip, cudaStream_t s,
                                int32_t* lus = nullptr, int nlu = 0);
// Chebyshev coefficients of vector slot 0 (instances with ny = M): count x 5 x M
cudaError_t launch_cheb_coeffs(int count, const InstDesc* desc, const zc* vec, zc* coef, int M, cudaStream_t s);
cudaError_t launch_cheb_start(int count, int nmax, const InstDesc* desc, const zc* coef, int ncheb, zc* vec,
                              int slot, const int32_t* skip, cudaStream_t s);
cudaError_t launch_ii_update(int count, const InstDesc* desc, zc* vec, int xslot, int yslot, int32_t* pcol,
                             const zc* sigma, zc* theta, int32_t* done, double* err, int32_t* iters, double tol,
                             const int32_t* skip, cudaStream_t s);
}  // namespace stab
