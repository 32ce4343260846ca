// Kernel declarations shared by the translation units of libstab_gb300.
#pragma once
#include "common.cuh"

namespace stab {

// operator kinds assembled from the per-node blocks (see k_blocks)
enum OpKind : int {
  OP_T_A0 = 0,   // temporal A0
  OP_T_B0 = 1,   // temporal B0 (block diagonal)
  OP_T_C = 2,    // B0^-1 A0 (the matrix ZGEEV sees after ZGESV)
  OP_T_Q = 3,    // A0 - s B0
  OP_T_DQ = 4,   // d/ds (A0 - s B0) = -B0
  OP_S_C0 = 5,
  OP_S_C1 = 6,
  OP_S_C2 = 7,
  OP_S_Q = 8,    // s^2 C0 + s C1 + C2   (lambda = 1/alpha form)
  OP_S_DQ = 9,   // 2 s C0 + C1
};

// prep.cu
__global__ void k_cheb_a(int ny, double* xa);
__global__ void k_cheb_d1(int ny, const double* xa, double* D1);
__global__ void k_cheb_d2(int ny, const double* D1, double* D2);
// bad[p] = 1 when profile p has non-finite values or non-ascending y
__global__ void k_spline(int nprof, const ProfDesc* pdesc, const double* prof, double* spl, int32_t* bad);
// flags[k] |= 2 when the instance's profile is bad
__global__ void k_nodes(int count, const InstDesc* desc, const double* prof, const double* spl, double* node,
                        const int32_t* bad, int32_t* flags);
__global__ void k_meanderiv(int count, const InstDesc* desc, const double* const* dtab, double* node);
__global__ void k_blocks(int count, const InstDesc* desc, const double* const* dtab, const double* node, zc* blk,
                         int* flags);

// assemble.cu
// per-node operator (P1, P2, P3): kind_t for temporal, kind_s for spatial
// instances, at shift sigma[k] (may be null)
// (ops32, if not null, receives the blocks rounded to complex64)
__global__ void k_node_ops(int count, const InstDesc* desc, const zc* blk, int kind_t, int kind_s, const zc* sigma,
                           zc* ops, cc* ops32, const int32_t* skip);
// dense column-major n x n operator (times `scale`) from ops into out +
// out_off[k] with leading dimension ldmul*n; element type T
template <typename T>
cudaError_t launch_dense(int count, int nmax, const InstDesc* desc, const double* const* dtab, const zc* ops, T* out,
                         const int64_t* out_off, int ldmul, double scale, cudaStream_t s,
                         const int32_t* skip = nullptr);
// the complex64 dense operator in FP32 arithmetic from the rounded blocks and
// tables (dtab32 pairs as dtab's)
cudaError_t launch_dense32(int count, int nmax, const InstDesc* desc, const float* const* dtab32, const cc* ops32,
                           cc* out, const int64_t* out_off, int ldmul, float scale, cudaStream_t s,
                           const int32_t* skip = nullptr);
// y[i] = (float) x[i]
cudaError_t launch_round_f32(int64_t count, const double* x, float* y, cudaStream_t s);
// structured y = M x for M given by ops (FP64):  y_i = P1 (D1 X)_i - P2 (D2 X)_i + P3 x_i
__global__ void k_opmv(int count, const InstDesc* desc, const double* const* dtab, const zc* ops, const zc* x,
                       int xslot, zc* y, int yslot);
// post.cu
__global__ void k_companion_fill(int count, const InstDesc* desc, zc* A, const int64_t* a_off);
__global__ void k_post_spectrum(int count, const InstDesc* desc, const zc* eig_raw, const int64_t* eig_off,
                                zc* eig_sorted, int32_t* least_sorted, zc* least_raw, zc* least_val, zc* cand,
                                int ncand);
__global__ void k_spatial_vec(int count, const InstDesc* desc, const zc* theta, const zc* vec, int slot,
                              zc* out, const int64_t* out_off, const int32_t* skip);
// seed rounds of the coarse mode: candidate j of k_post_spectrum -> sigma,
// folding of each round into the best pair, final pick
__global__ void k_take_candidate(int count, const zc* cand, int ncand, int j, zc* sigma);
__global__ void k_converged_mask(int count, int32_t* done, int32_t* mask, int restore);
// FMA throughput probes (probe.cu): kind 0 FP32, 1 FP64, 2 double-word
// complex; returns the flops of the launch
double launch_probe(int kind, int blocks, int iters, float* out, cudaStream_t s);
__global__ void k_fold_best(int count, const InstDesc* desc, const zc* sigma, const zc* theta, const int32_t* done,
                            const double* err, const int32_t* iters, const zc* out, const int64_t* out_off,
                            int32_t* final_, int32_t* have, double* best_key, zc* best_theta, double* best_err,
                            int32_t* best_iters, zc* best_out, int quick, double quick_tol, int32_t* skip64,
                            int slow_iters, int src, int32_t* best_src);
__global__ void k_take_best(int count, const InstDesc* desc, const int32_t* have, const zc* best_theta,
                            const double* best_err, const int32_t* best_iters, const zc* best_out,
                            const int64_t* out_off, zc* theta, int32_t* done, double* err, int32_t* iters, zc* out,
                            const int32_t* final_, const int32_t* best_src, int seed_src, int unverified,
                            int keep_unverified);
// candidate copies of a small batch (k_spread_candidates, k_mark_missing,
// k_fold_copies)
__global__ void k_spread_candidates(int ncopy, const zc* cand, int ncand, zc* copy_cand);
__global__ void k_mark_missing(int count, const zc* cand, int ncand, int32_t* final_);
__global__ void k_fold_copies(int count, int ncand, const InstDesc* desc, const int32_t* copy_done,
                              const double* copy_key, const zc* copy_theta, const double* copy_err,
                              const int32_t* copy_iters, const zc* copy_out, const int64_t* copy_out_off, zc* theta,
                              int32_t* done, double* err, int32_t* iters, zc* out, const int64_t* out_off,
                              int unverified, const zc* lam1, const zc* th1, const int32_t* ok1, const zc* cand,
                              double conv, int n1, int n2t, int n2s);
__global__ void k_gather_level(int count, const int32_t* idx, const zc* cand, int ncand, const zc* best_theta,
                               const int32_t* have, const int32_t* best_src, zc* lam1, zc* th1, int32_t* ok1);
__global__ void k_temporal_vec(int count, const InstDesc* desc, const zc* vec, int slot, zc* out,
                               const int64_t* out_off, const int32_t* skip);

}  // namespace stab
