// Host launcher of the plain FP64 full-spectrum eigensolver (hqr.cu).
#pragma once
#include "common.cuh"

namespace stab {
// dynamic shared memory of k_eig_plain
size_t eig_plain_smem(int mmax);
// A: count column-major m x m matrices (destroyed); H: workspace of the same
// size; eig receives m eigenvalues per instance (QR eigenvalues first, then
// the isolated ones); status[k] = 0 or STAB_ST_NOCONV.  `order` (may be null)
// is the processing order (largest first balances the persistent grid).
// flops (may be null) receives the flops each instance executed in the
// Hessenberg reduction and the QR sweeps.  double_word runs the reduction
// and the QR iteration in double-word (float-float) arithmetic, for spectra
// that seed a polish.  qr_smem: where the packed Hessenberg matrix of order
// mmax fits in shared memory, run one 512-thread CTA per SM with the QR phase
// in shared memory (k_eig_plain_sq).
cudaError_t eig_phase_cycles(unsigned long long* out, bool reset);
cudaError_t launch_eig_plain(int count, int mmax, const int32_t* msz, zc* A, const int64_t* a_off, zc* H,
                             const int64_t* h_off, zc* eig, const int64_t* eig_off, int32_t* status,
                             int32_t* work_counter, const int32_t* order, double* flops, int grid,
                             cudaStream_t s, bool double_word = false, bool qr_smem = false, int threads = 0);
}  // namespace stab
