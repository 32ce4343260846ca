/*
 * stab_gb300.h -- C ABI of the GB300 (sm_103a) compressible linear-stability
 * hot path: Chebyshev-collocation assembly of the temporal pencil and of the
 * alpha-linearised spatial operator, the full-spectrum FP64 eigensolve, and
 * the mixed-precision shift-invert polish of the least-stable mode.
 *
 * Conventions
 *   - Plain C types only; every array is caller-owned host memory unless a
 *     function says "device".  The library never frees caller memory.
 *   - A complex number is two doubles {re, im}; this is the layout of Fortran
 *     complex(8) and C99 double _Complex, so Fortran callers bind through
 *     iso_c_binding with complex(c_double_complex) arrays.
 *   - Matrices are column-major (Fortran order).  Unknown (i, dof) of node i
 *     (0-based, i = 0 is the free stream, i = ny-1 the wall) and field
 *     dof in {rho, u, v, w, T} sits at row 5*i + dof, as in the reference.
 *   - Functions return 0 on success and a negative STAB_ERR_* code on error;
 *     stab_last_error() gives a message.  Per-instance numerical outcomes are
 *     reported through status arrays (STAB_ST_*), never by aborting: the
 *     reference's `stop` paths (temporal.f90:776-785, :806-809) become codes.
 */
#ifndef STAB_GB300_H
#define STAB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STAB_GB300_ABI_VERSION 1

/* return codes */
#define STAB_OK 0
#define STAB_ERR_ARG (-1)     /* bad argument (size, flag, unsupported option)  */
#define STAB_ERR_CUDA (-2)    /* CUDA runtime error                              */
#define STAB_ERR_NOMEM (-3)   /* device allocation failed                        */
#define STAB_ERR_IO (-4)      /* file could not be read or written               */
#define STAB_ERR_STATE (-5)   /* object used in the wrong state                  */

/* per-instance status (LAPACK-like: 0 ok, >0 numerical) */
#define STAB_ST_OK 0
#define STAB_ST_SINGULAR 1    /* exactly singular factor (ZGESV/ZGETRF info>0)   */
#define STAB_ST_NOCONV 2      /* iteration cap reached (ZGEEV info>0 analogue)   */
#define STAB_ST_NAN 3         /* non-finite value in the inputs or results      */
#define STAB_ST_FELLBACK 4    /* polish did not converge; plain FP64 path used   */
#define STAB_ST_NOMODE 5      /* no eigenvalue passed the least-stable filter    */
#define STAB_ST_UNVERIFIED 6  /* a converged eigenpair that no resolved seed     *
                               * spectrum confirmed as the least-stable mode     *
                               * (STAB_MODE_COARSE / STAB_MODE_SURROGATE)        */

/* solve modes for stab_batch_run / stab_solve_batch */
#define STAB_MODE_PLAIN 0     /* FP64 full spectrum + least-stable eigenvector   */
#define STAB_MODE_SEEDED 1    /* mixed-precision polish from caller seeds; where *
                               * complex64 factors do not converge, complex128   *
                               * inverse iteration at the seed; where that fails *
                               * too, the FP64 spectrum's least-stable mode      *
                               * (STAB_ST_FELLBACK)                              */
#define STAB_MODE_COARSE 2    /* seeds from a full spectrum at N = 32, then the  *
                               * mixed-precision polish.  STAB_ST_OK only where  *
                               * the seed spectrum's most unstable candidate     *
                               * polished to within 1e-7 of itself (the seed     *
                               * spectrum resolved it).  Every other instance    *
                               * takes seeds from N = 48 under the same rule     *
                               * (STAB_ST_FELLBACK); where that does not settle  *
                               * it either, the least-stable converged pair is   *
                               * kept with STAB_ST_UNVERIFIED, and instances     *
                               * without one take the plain FP64 path            *
                               * (STAB_ST_FELLBACK).  A discrete mode that the   *
                               * seed spectrum misplaces below its top candidate *
                               * can still be missed: the check costs no fine    *
                               * spectrum, so it cannot rule that out            */
#define STAB_MODE_TRACK 4     /* polish from caller guesses (complex64, then     *
                               * complex128 inverse iteration); where both fail, *
                               * the FP64 spectrum's eigenvalue nearest the      *
                               * guess (the pick of getab.f90:185-192)           */
#define STAB_MODE_SURROGATE 3 /* STAB_MODE_COARSE plus the caller's predicted    *
                               * seed (and start vector, stab_batch_set_start)   *
                               * as one more candidate round                     */

/*
 * Run parameters of one solve: a mirror of module `stuff` (stuff.f90:11-55)
 * as input.f90:15-81 and stab.f90:46-55 fill it.  Te is derived as the
 * reference derives it (input.f90:25 evaluates te = t0/(1+0.2 Ma^2) before
 * Ma is read, so Te = T0 for Sutherland and Te = 0 for constant viscosity).
 */
typedef struct stab_params {
    int32_t mattyp;   /* 0 constant mu, 1 Sutherland                         */
    int32_t ny;       /* collocation points N (polynomial degree N-1)        */
    int32_t ievec;    /* 1: eigenvectors wanted                              */
    int32_t ider;     /* 1: mean derivatives by the collocation matrices;   *
                       * 0: from tables (getmean2.f90): profile rows then  *
                       * hold 18 values, the three tables side by side     */
    int32_t top;      /* spatial free-stream BC: 0 rho=0, 1 continuity       */
    int32_t wall;     /* carried through to evec.dat                         */
    int32_t wallt;    /* 0 isothermal, 2 adiabatic wall                      */
    int32_t curve;    /* spatial only: 0 flat; 1 parabolic cylinder       *
                       * y = sqrt(2x) at arc length x from its nose       *
                       * (calch.f90; STAB_ERR_ARG where its false-position *
                       * search stops without a root, e.g. x in (.02,.9)); *
                       * 2 circle of radius x (circh.f90; the x written to *
                       * evec.dat is 0, as circh leaves it); x = -1 keeps  *
                       * the wall flat in both                             */
    int32_t itype;    /* 1 temporal, 2 spatial, 3 temporal by finite         *
                       * differences (fd_temporal.f90: fourth-order        *
                       * stencils with Carpenter's closures on ogengrid's  *
                       * uniform eta, wall first; needs ymax > 2 yi and    *
                       * ny >= 10; evec.dat records itype 1)               */
    int32_t ind;      /* profile index (profile.<ind>)                       */
    double T0, Ma, Re, Pr, yi, ymax, x;
    double alpha[2];  /* temporal: streamwise wavenumber                     */
    double beta[2];   /* spanwise wavenumber                                 */
    double omega[2];  /* spatial: frequency                                  */
} stab_params;

typedef struct stab_ctx stab_ctx;
typedef struct stab_batch stab_batch;
typedef struct stab_mlp stab_mlp;

/* ---- context ---------------------------------------------------------- */
int stab_abi_version(void);
/* Create a context on CUDA device `device`; it owns a stream and device
 * memory pools.  Replaces nothing in the reference (which has no state
 * beyond module `stuff`). */
int stab_create(stab_ctx** ctx, int device);
int stab_destroy(stab_ctx* ctx);
const char* stab_last_error(const stab_ctx* ctx);
/* Launch on a caller stream (a cudaStream_t passed as void*); NULL restores
 * the context's own stream. */
int stab_set_stream(stab_ctx* ctx, void* stream);
int stab_sync(stab_ctx* ctx);
/* Per-kernel CUDA-event timing (0 off, 1 on) and its readout: for kernel
 * index k < *count, name, number of launches and total milliseconds. */
int stab_set_profiling(stab_ctx* ctx, int on);
int stab_kernel_stats(stab_ctx* ctx, int32_t k, const char** name, int64_t* launches, double* total_ms, int32_t* count);
int stab_reset_kernel_stats(stab_ctx* ctx);
/* Arithmetic of three stages (no reference counterpart):
 *   STAB_STAGE_SEED_EIG   Hessenberg reduction and QR of the spectra that
 *                         only seed the polish (STAB_MODE_COARSE /
 *                         STAB_MODE_SURROGATE and their second candidate
 *                         level: N = 48 temporal, N = 24 spatial);
 *                         default STAB_ARITH_DOUBLE_WORD;
 *   STAB_STAGE_PLAIN_EIG  the same for STAB_MODE_PLAIN, stab_full_spectrum
 *                         and the FP64 fallback (ZGEEV, temporal.f90:803);
 *                         default STAB_ARITH_FP64;
 *   STAB_STAGE_RETRY_LU   LU and solves of the complex128 inverse-iteration
 *                         retry of the polish (residuals and eigenvalue
 *                         updates stay FP64); default STAB_ARITH_DOUBLE_WORD.
 *   STAB_STAGE_POLISH_LU  the complex64 LUs of the polish (shift and bordered
 *                         Jacobian): STAB_ARITH_TF32_SPLIT (default) or
 *                         STAB_ARITH_FP32.
 * STAB_ARITH_DOUBLE_WORD is float-float pairs (about 48 significant bits)
 * run on the FP32 pipe. */
#define STAB_STAGE_SEED_EIG 0
#define STAB_STAGE_PLAIN_EIG 1
#define STAB_STAGE_RETRY_LU 2
#define STAB_STAGE_POLISH_LU 3
#define STAB_ARITH_FP64 0
#define STAB_ARITH_DOUBLE_WORD 1
#define STAB_ARITH_FP32 2          /* complex64 on the CUDA cores                   */
#define STAB_ARITH_TF32_SPLIT 3    /* complex64 with the trailing update on the     *
                                    * tensor cores: each FP32 operand split into     *
                                    * three TF32 parts, six part products, FP32      *
                                    * accumulation in TMEM                           */
int stab_set_arithmetic(stab_ctx* ctx, int32_t stage, int32_t arithmetic);
/* N of the seed spectrum that STAB_MODE_COARSE and STAB_MODE_SURROGATE
 * take their candidate shifts from (16 <= ny < 48; default 32).  Applies to
 * batches created afterwards.  A smaller N costs less (the eigensolve grows
 * as N^3) and resolves fewer least-stable modes.  No reference counterpart. */
int stab_set_seed_size(stab_ctx* ctx, int32_t ny);
/* Execution options (no reference counterpart):
 *   STAB_OPT_SEED_QR_SHARED  1: seed spectra whose packed Hessenberg matrix
 *     fits in shared memory (order <= 160, the N = 32 temporal seeds) run
 *     one 512-thread CTA per SM with the QR phase in shared memory; 0
 *     (default, measured faster on the 4096-instance sweep): the 128-thread
 *     batch kernel, four CTAs per SM, everything in global memory.  Same
 *     algorithm and arithmetic, bit-identical eigenvalues either way. */
#define STAB_OPT_SEED_QR_SHARED 1
/*   STAB_OPT_POLISH_LU_TMA  1 (default): the tensor-core LU moves each
 *     128 x 64 tile of the trailing matrix between global and shared memory
 *     with tensor (TMA) loads and stores, overlapped with the operand
 *     staging and the MMAs (batches larger than two instances per SM whose
 *     orders are all even; the others take the other form, two CTAs per
 *     SM); 0: the epilogue reads and writes the tile from the registers.
 *     Same arithmetic either way. */
#define STAB_OPT_POLISH_LU_TMA 2
/*   STAB_OPT_EIG_RESIDENT  k >= 1: the batch eigensolver (seed and plain
 *     spectra of batches larger than half the SM count) keeps at most k
 *     instances in flight per SM, so that their working matrices can stay
 *     in L2 (each CTA takes the next instance from a work counter when it
 *     finishes one); 0 (default): as many as the occupancy allows (four).
 *     Bit-identical eigenvalues for every value. */
#define STAB_OPT_EIG_RESIDENT 3
/*   STAB_OPT_EIG_THREADS  128 (default): the batch eigensolver runs 128-
 *     thread CTAs, four per SM; 64: 64-thread CTAs, eight per SM (twice the
 *     instances in flight).  The same algorithm; block sums run in another
 *     order, so eigenvalues agree to rounding, not bit for bit. */
#define STAB_OPT_EIG_THREADS 4
/*   STAB_OPT_EIG_MID  1 (default, measured 2.6 % faster on the 4096-instance
 *     sweep): batches of at most two instances per SM (the second candidate
 *     level of STAB_MODE_COARSE, small serving batches) run one 256-thread CTA per
 *     instance instead of the 128-thread persistent grid; 0: the persistent
 *     grid.  Same algorithm; block sums in another order. */
#define STAB_OPT_EIG_MID 5
/*   STAB_OPT_SEED_VECTORS  1 (default): STAB_MODE_COARSE starts the top
 *     candidate's polish from the seed level's eigenvector (inverse iteration
 *     on the N = 32 operator, interpolated through its Chebyshev
 *     coefficients) instead of factoring the full operator at the shift for
 *     two inverse-iteration steps (Chebyshev grids; batches with a finite-
 *     difference instance keep the steps); 0: the steps. */
#define STAB_OPT_SEED_VECTORS 6
/*   STAB_OPT_PARALLEL_CANDIDATES  1 (default): the second candidate level of
 *     STAB_MODE_COARSE polishes its instances' four shift candidates side by
 *     side (one sub-batch copy per candidate) instead of in four rounds one
 *     after another; the kept pair and status follow the sequential rule;
 *     0: sequential rounds. */
#define STAB_OPT_PARALLEL_CANDIDATES 7
/*   STAB_OPT_MEDIUM_NY  N of the second candidate level of STAB_MODE_COARSE
 *     for the temporal instances (the seed spectra of the instances whose
 *     first-level top candidate was not resolved): in [16, 64], not the seed
 *     size; default 48. */
#define STAB_OPT_MEDIUM_NY 8
/*   STAB_OPT_FIRST_RETRY  1 (default): at the first candidate level of
 *     STAB_MODE_COARSE, instances whose complex64 polish of the top candidate
 *     failed or contracted slowly take the double-word inverse-iteration
 *     retry before the second level; 0: they go to the second level
 *     directly. */
#define STAB_OPT_FIRST_RETRY 9
/*   STAB_OPT_LEVEL_CONSISTENCY  1 (default): at the second candidate level of
 *     STAB_MODE_COARSE (with STAB_OPT_PARALLEL_CANDIDATES), an instance whose
 *     second-level top candidate did not polish to within 1e-7 of itself is still
 *     trusted (STAB_ST_FELLBACK) when the top candidates of both seed levels
 *     polished to the same pair (within 1e-10), that pair is the least
 *     stable of the level's converged candidates, and the seed values
 *     converge to it (the finer level's error at most a quarter of the
 *     coarser one's and below 1e-3 relative); 0: such instances are
 *     STAB_ST_UNVERIFIED. */
#define STAB_OPT_LEVEL_CONSISTENCY 10
/*   STAB_OPT_MEDIUM_NY_SPATIAL  N of the second candidate level for the
 *     spatial instances (itypes 2 and 4), in [16, 64]: default 24.  Their
 *     least-stable alpha converges algebraically in N (about 1e-3 relative
 *     at N = 24, 1e-5 at N = 32 for crossflow profiles), so the agreement of
 *     a coarser second level with the first (STAB_OPT_LEVEL_CONSISTENCY:
 *     the finer level closer by a factor of four) certifies it at an eighth
 *     of the cost of an N = 48 companion spectrum. */
#define STAB_OPT_MEDIUM_NY_SPATIAL 11
/*   STAB_OPT_MLP_TCGEN05  1 (default): the surrogate network's GEMMs (forward
 *     and backward) run on the fifth-generation tensor cores (tcgen05.mma
 *     kind::f16, BF16 operands, FP32 accumulator in TMEM); 0: on mma.sync
 *     m16n8k16.  A tensor-core tile that does not see its MMAs complete
 *     within a bounded wait makes the next loss read (stab_mlp_gradients,
 *     stab_mlp_train_step) return STAB_ERR_CUDA. */
#define STAB_OPT_MLP_TCGEN05 12
int stab_set_option(stab_ctx* ctx, int32_t option, int32_t value);
/* SM cycles of the full-spectrum eigensolver per phase, summed over every
 * instance solved on this device since the last reset: [0] isolation,
 * [1] compaction, [2] balancing, [3] Hessenberg reduction, [4] repacking,
 * [5] QR iteration.  reset != 0 zeroes them after reading. */
int stab_eig_phases(stab_ctx* ctx, uint64_t* cycles_out, int32_t reset);

/* ---- operator assembly (parity / inspection) -------------------------- */
/*
 * Assemble the operator of one instance on the GPU and copy it back.
 *   itype 1: mats_out = [A0 | B0], two n x n complex matrices, n = 5*ny
 *            (temporal.f90:604-752; A0 x = omega B0 x).
 *   itype 2: mats_out = [C0 | C1 | C2], three n x n complex matrices
 *            (spatial.f90:677-959; (C0 + alpha C1 + alpha^2 C2) phi = 0).
 * profile: nym rows of (y, rho, u, v, w, T), row-major, as profile.<ind>
 * (getmean.f90:40-80; v is forced to zero).  With p->ider = 0 each row holds
 * 18 values: the profile row, then the row of the first y-derivative table
 * (first.<ind>) and of the second (second.<ind>), each "y f1..f5"
 * (getmean2.f90:99-175: the tables are splined on their own y and taken as
 * the mean derivatives without the map's chain rule).  The same holds for
 * every entry point that takes profiles.
 * Replaces the inline assembly of temporal.f90:95-752 / spatial.f90:96-959.
 */
int stab_assemble(stab_ctx* ctx, const stab_params* p, int32_t nym, const double* profile,
                  double* mats_out);

/* ---- autotuning --------------------------------------------------------- */
/*
 * Time the batched LU of both precisions at each order in orders[] with
 * every shared-memory-feasible panel width (8, 16, 32) on a full wave of
 * test matrices, and keep the fastest per size class in the context; later
 * factorisations of that class use it.  nb_out / ms_out (may be NULL):
 * 2 * norders entries, [2q] complex64 and [2q+1] complex128 choice and time.
 */
int stab_autotune(stab_ctx* ctx, const int32_t* orders, int32_t norders, int32_t* nb_out, float* ms_out);

/*
 * Self-check of the cluster path of the batched LU: count test matrices of
 * order n factored with one CTA each and with clusters of four CTAs (one
 * matrix per cluster).  max_diff: largest |difference| of the factors,
 * piv_diff: number of differing pivots; both 0 when the paths agree.
 */
int stab_lu_cluster_check(stab_ctx* ctx, int32_t n, int32_t count, int32_t complex128, double* max_diff,
                          int32_t* piv_diff);

/*
 * Self-check of the tensor-core LU: count test matrices of order n factored
 * in complex64 on the CUDA cores and with the tensor-core trailing update
 * (in the form STAB_OPT_POLISH_LU_TMA selects).
 * bwd_tc / bwd_simt: largest backward error max|P A - L U| / max|A| of
 * either path (computed on the host in FP64); piv_diff: number of differing
 * pivots.  No reference counterpart (the reference calls LAPACK's ZGETRF).
 */
int stab_lu_tc_check(stab_ctx* ctx, int32_t n, int32_t count, double* bwd_tc, double* bwd_simt, int32_t* piv_diff);

/*
 * Measured multiply-add throughput of this device, in TFLOP/s: out[0] FP32
 * FMA, out[1] FP64 FMA (2 flops each), out[2] double-word complex
 * multiply-add (8 flops each, the unit of stab_batch_work and the kernels'
 * flop counts).  Independent chains on every SM, timed with CUDA events
 * after a warm-up launch: the roofline denominators of the kernels bound by
 * these pipes.  No reference counterpart.
 */
int stab_peak_rates(stab_ctx* ctx, double* out);

/* ---- full spectrum (plain FP64 path) --------------------------------- */
/*
 * All eigenvalues of one instance, sorted ascending by imaginary part with
 * the stable order of PIKSR2: omega (itype 1, n = 5*ny values) or alpha
 * (itype 2, n = 10*ny values, alpha = 1/lambda and lambda = 0 -> 0).
 * vec_out (may be NULL): the least-stable eigenvector, n complex values,
 * normalised as the reference normalises evec.dat columns (temporal: divided
 * by its max-modulus entry, temporal.f90:867-879; spatial: unit 2-norm with
 * its max-modulus entry real and positive, the ZGEEV convention).
 * least_index_out (may be NULL): index in the sorted list of the selected
 * least-stable mode, -1 when none passed the filter.
 * Replaces ZGESV+ZGEEV+PIKSR2 (temporal.f90:771-855) and
 * ZGETRF+ZGETRS+ZGEEV+PIKSR2 (spatial.f90:972-1084).
 */
int stab_full_spectrum(stab_ctx* ctx, const stab_params* p, int32_t nym, const double* profile,
                       double* eig_out, double* vec_out, int32_t* least_index_out,
                       int32_t* status_out);

/*
 * Eigenvectors of one instance at `count` of its eigenvalues (omega for
 * itype 1, alpha for itype 2, as stab_full_spectrum returns them), by FP64
 * inverse iteration on an LU of Q(shift), instances run as one batch.
 * vec_out: count columns of n (temporal, 5*ny) or m (spatial, 10*ny) complex
 * values, column-major, normalised as in stab_full_spectrum.  status_out
 * (may be NULL): count STAB_ST_* values.  With every eigenvalue of the
 * spectrum this is the eigenvector matrix that ZGEEV('N','V') hands to the
 * evec.dat writer (temporal.f90:803, spatial.f90:1043); vectors of
 * repeated eigenvalues (the zero eigenvalues of the boundary rows) are some
 * vector of their eigenspace, as in LAPACK.
 */
int stab_eigenvectors(stab_ctx* ctx, const stab_params* p, int32_t nym, const double* profile,
                      int32_t count, const double* eig, double* vec_out, int32_t* status_out);

/* ---- the reference's file interface (host only, no GPU) --------------- */
/*
 * Parse the stdin protocol of `stab < input.dat`: input.f90:15-123 followed
 * by the index (and, for itype 2, x) reads of stab.f90:46-55.  Fortran
 * list-directed semantics: each read starts on a new record, takes blank- or
 * comma-separated values across records and drops the rest of its last
 * record.  Out-of-range mattyp and itype are read again as the reference
 * does; itype 3..9 (finite-difference, Stokes, bump and multi-point drivers)
 * return STAB_ERR_ARG.  msg (may be NULL) receives the reason.
 */
int stab_parse_input(const char* text, stab_params* p, char* msg, size_t msg_cap);
/* "profile.<ind>" (makename, getmean.f90:27-28). */
int stab_profile_name(int32_t ind, char* out, size_t cap);

/*
 * The multi-point drivers of `stab < input.dat` (stab.f90:85-90): itype 7
 * (mtemporal, an alpha x beta sweep on profile.0) and itype 8 (mspatial,
 * stations of delta.dat x omega x beta, each station on its own
 * profile.<ind>).  Every point's eigensystem goes to eig.<iver>, iver = 1, 2,
 * ... in loop order.
 */
typedef struct stab_sweep {
  int32_t itype;                   /* 7 or 8 (0 after a single-point input)       */
  int32_t dtype;                   /* itype 8: 0 Chebyshev collocation            */
  int32_t ind1, ind2, ind_inc;     /* itype 8: 1-based rows of delta.dat          */
  double p_min, p_max, p_inc;      /* alpha (itype 7) or omega (itype 8) range    */
  double b_min, b_max, b_inc;      /* beta range                                  */
} stab_sweep;
/* stab_parse_input that also takes itypes 7 and 8: after the common input it
 * reads the driver's ranges (mtemporal.f90:20-23; mspatial.f90:20-27, where
 * dtype 1, the finite-difference solver, returns STAB_ERR_ARG).  p->itype is
 * set to the solver's itype (1 or 2) and sw->itype to 7 or 8; for itypes 1
 * and 2, sw->itype is 0 and the result equals stab_parse_input's. */
int stab_parse_sweep_input(const char* text, stab_params* p, stab_sweep* sw, char* msg, size_t msg_cap);
/* delta.dat (mspatial.f90:29-63): records not starting with '#' hold
 * "xb delta".  xb, delta may be NULL (count only). */
int stab_read_delta(const char* path, int32_t cap, double* xb, double* delta, int32_t* nbody);
/* body.dat of the post-processors (getab.f90:73-86): "index xb" records. */
int stab_read_body(const char* path, int32_t cap, double* xb, int32_t* nbody);
/* "eig.<iver>" (makename, mtemporal.f90:53-76). */
int stab_eig_name(int32_t iver, char* out, size_t cap);
/* One line of the post-processors' output (no newline): "p Re Im" in
 * 3(1x,1pe20.13) (stab.out of getab, getab.f90:211) or, with with_ind,
 * "ind p Re Im" in i4,3(1x,1pe20.13) (stab.out of getax, getax.f90:214;
 * parm.new of getalpha, getalpha.f90:167).  Returns the length. */
int stab_stab_out_line(int32_t with_ind, int32_t ind, double p, double vr, double vi, char* out, size_t cap);
/*
 * The solves of a sweep in the reference's loop order, each a copy of base
 * with the swept values set: itype 7 (mtemporal.f90:25-39) alpha outer, beta
 * inner, na = max(nint((amax - amin) / ainc), 1) points in alpha (amax is not
 * reached); itype 8 (mspatial.f90:65-96) station outer, then omega, then beta,
 * zero increments replaced by one, nint(range / inc) + 1 points each, with
 * x = xb(ind), Yi = 2 delta(ind) and ind the station (profile.<ind>).
 * points may be NULL (count only); xb / delta (nbody rows) only for itype 8.
 */
int stab_sweep_points(const stab_params* base, const stab_sweep* sw, int32_t nbody, const double* xb,
                      const double* delta, int32_t cap, stab_params* points, int32_t* count);
/*
 * Read profile.<ind> (getmean.f90:27-80): rows "y rho u v w T", records that
 * start with '#' skipped.  rows == NULL counts only; else up to cap_rows rows
 * of 6 doubles are stored row-major.  *nym receives the row count.
 */
int stab_read_profile(const char* path, int32_t cap_rows, double* rows, int32_t* nym);
/* Collocation grid y, eta, d eta/dy, d2 eta/dy2 (sgengrid.f90:18-45). */
int stab_grid(int32_t ny, double yi, double ymax, double* y, double* eta, double* deta, double* d2eta);
/* Grid of the finite-difference solver (ogengrid.f90:20-44): uniform eta on
 * [0, 1] from the wall, y = a eta / (b - eta); needs ymax > 2 yi. */
int stab_fd_grid(int32_t ny, double yi, double ymax, double* y, double* eta, double* deta, double* d2eta);
/*
 * Write evec.dat as gfortran writes it (temporal.f90:883-890,
 * spatial.f90:1120-1126): sequential unformatted records with 4-byte
 * little-endian lengths; R1 10 x int32 (ind ny ndof itype ievec curve top
 * wall wallt ider), R2 omega alpha beta Re Ma Pr, R3 x y eta deta d2eta yi
 * ymax, R4 the nmax eigenvalues, R5 the nmax x nmax eigenvectors (always for
 * itype 1, only with ievec = 1 for itype 2; vec may be NULL otherwise).
 */
int stab_write_evec(const char* path, const stab_params* p, const double* eig, const double* vec);

/* evec.dat records R1-R3 as getevec.f90:77-91 reads them. */
typedef struct {
  int32_t ind, ny, ndof, itype, ievec, curve, top, wall, wallt, ider;
  int32_t nmax;         /* ndof*ny (itype 1) or 2*ndof*ny (itype 2)  */
  int32_t has_vectors;  /* R5 present                                 */
  double omega[2], alpha[2], beta[2];
  double Re, Ma, Pr, x, yi, ymax;
} stab_evec_header;
/* Read evec.dat; y (ny), eig (nmax complex) and vec (nmax x nmax complex)
 * may each be NULL (call once with NULLs to learn the sizes). */
int stab_read_evec(const char* path, stab_evec_header* h, double* y, double* eig, double* vec);
/* getevec -v (getevec.f90:161-172): 0-based index of the nearest
 * eigenvalue, the first minimum winning. */
int32_t stab_getevec_select(const double* eig, int32_t nmax, double vr, double vi);
/*
 * The time.N / space.N text for one eigenpair (getevec.f90:176-227): four
 * header lines, then rows wall to free stream "y Re/Im(rho u v w T)" in
 * 1P E21.13E3 with the scale quirk of getevec.f90:179-189 (the vector is
 * divided by the real part of its running max-modulus pick).  Returns the
 * text length; the text (NUL-terminated) is stored when cap > length.
 */
int64_t stab_eigfunction_text(const stab_evec_header* h, const double* y, const double* eig_j,
                              const double* vec_j, char* buf, int64_t cap);

/* ---- batched least-stable mode ---------------------------------------- */
/*
 * Upload `count` instances (parameters + profiles) to device memory.
 * profiles[k] points at nym[k] x 6 doubles; identical pointers are uploaded
 * once.  The instances may have different ny and itype.  The call copies
 * everything it needs and synchronises before it returns: the caller may
 * free or reuse p, nym and the profile buffers at once.  Each batch keeps
 * its own state; batches of different contexts may be used from different
 * host threads.
 */
int stab_batch_create(stab_ctx* ctx, int32_t count, const stab_params* p, const int32_t* nym,
                      const double* const* profiles, stab_batch** out);
/* Seeds for STAB_MODE_SEEDED: count complex values (omega for temporal,
 * alpha for spatial), copied to the device. */
int stab_batch_set_seeds(stab_batch* b, const double* seeds);
/*
 * Start vectors for STAB_MODE_SURROGATE and STAB_MODE_TRACK (ncheb <= 256):
 * per instance 5 x ncheb complex
 * Chebyshev coefficients (field-major: rho, u, v, w, T), evaluated at the
 * instance's collocation points, x(i, e) = sum_q c[e][q] cos(q pi i/(ny-1)).
 * ncheb = 0 clears them (the generic start vector is used).
 */
int stab_batch_set_start(stab_batch* b, const double* coef, int32_t ncheb);
/*
 * Run the whole path on the device.  STAB_MODE_SURROGATE polishes the coarse
 * candidates and then, for the instances that no resolved candidate settled,
 * the caller's seed (a surrogate's prediction).  Where the seed's converged
 * pair is the least stable of the converged pairs it is kept with
 * STAB_ST_UNVERIFIED (nothing but the seed supports it); the other
 * unsettled instances take the fallback chain of STAB_MODE_COARSE.  The
 * seed adds what the N = 32 spectrum cannot give: discrete modes that
 * N = 32 does not resolve (supersonic second modes), whose coarse candidates
 * are spurious.
 */
int stab_batch_run(stab_batch* b, int32_t mode);
/* After a STAB_MODE_PLAIN run: every instance's full spectrum, sorted as
 * stab_full_spectrum sorts it; eig_out[k] (caller order, NULL skips) receives
 * n_k complex values.  The eigenvalue record of a sweep point's evec.dat
 * (the eig.N files of mtemporal.f90:29-39 and mspatial.f90:77-96). */
int stab_batch_spectra(stab_batch* b, double* const* eig_out);
/* After a run: counts_out[0] instances resolved by the first stage (the
 * seeds, the coarse candidates, or the plain path), [1] whose kept pair came
 * from the caller's seed in STAB_MODE_SURROGATE (STAB_ST_UNVERIFIED), [2]
 * sent to the fallback chain (N = 48 seeds, then the plain FP64 path). */
int stab_batch_counts(stab_batch* b, int32_t* counts_out);
/*
 * Copy results back (synchronises): eig_out[2*k] least-stable eigenvalue,
 * err_out[k] relative FP64 residual estimate |r|/(|M||x|) of the final pair,
 * iters_out[k] refinement steps used, status_out[k] STAB_ST_*.  vec_out
 * (may be NULL) receives count pointers, each to n_k complex values.
 * Any output pointer may be NULL.
 */
int stab_batch_results(stab_batch* b, double* eig_out, double* err_out, int32_t* iters_out,
                       int32_t* status_out, double* const* vec_out);
/*
 * Algorithmic work of the last stab_batch_run, for roofline accounting:
 * work_out[0] FP64 flops executed by the full-spectrum eigensolver (plain
 * mode: every instance; seeded and coarse modes: the fallback instances),
 * [1] the same for the N = 32 seed batch (coarse mode), [2] complex64 LU
 * flops of the polish and [3] complex128 LU flops (8/3 n^3 real flops per
 * factorisation, counted per instance as run, fallback included).
 */
int stab_batch_work(stab_batch* b, double* work_out);
int stab_batch_destroy(stab_batch* b);

/* One-shot: create + run + results + destroy (the end-to-end call). */
int stab_solve_batch(stab_ctx* ctx, int32_t count, const stab_params* p, const int32_t* nym,
                     const double* const* profiles, int32_t mode, const double* seeds,
                     double* eig_out, double* err_out, int32_t* status_out, double* const* vec_out);

/* ---- surrogate network (no counterpart in the reference) -------------- */
/*
 * A multilayer perceptron run and trained on the GPU by the library's own
 * BF16 kernels (tensor-core GEMMs with bf16 operands and float32
 * accumulation, fused bias + GELU epilogues, Adam on float32 master weights).
 * sizes[0..nlayers]: layer widths; hidden layers use GELU (erf form), the
 * last layer is linear.  Parameters pack as [W_0, b_0, W_1, b_1, ...] with
 * W_l of shape sizes[l] x sizes[l+1], row-major.  x, t, y are row-major
 * float32 device arrays (batch x width); w holds one loss weight per output:
 * loss = sum_ij w_j (y_ij - t_ij)^2 / batch.  Runs on the context stream;
 * destroying the context first releases the network's device memory.
 */
int stab_mlp_create(stab_ctx* ctx, int32_t nlayers, const int32_t* sizes, int32_t max_batch, stab_mlp** out);
int64_t stab_mlp_param_count(const stab_mlp* m);
/* host float32 parameters in; resets the Adam moments and step */
int stab_mlp_set_params(stab_mlp* m, const float* params);
/* float32 parameters and the gradients of the last backward pass out (either may be NULL) */
int stab_mlp_get_params(stab_mlp* m, float* params_out, float* grads_out);
int stab_mlp_forward(stab_mlp* m, int32_t batch, const float* x_dev, float* y_dev);
/* forward + backward; loss_out (host, may be NULL: no synchronisation) */
int stab_mlp_gradients(stab_mlp* m, int32_t batch, const float* x_dev, const float* t_dev, const float* w_dev,
                       double* loss_out);
/* forward + backward + one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) */
int stab_mlp_train_step(stab_mlp* m, int32_t batch, const float* x_dev, const float* t_dev, const float* w_dev,
                        float lr, double* loss_out);
int stab_mlp_destroy(stab_mlp* m);

/* ---- allocation-free eigenvalues -------------------------------------- */
#define STAB_NOALLOC_MAX_M 256
/*
 * All eigenvalues of one dense m x m complex128 matrix (column-major, device
 * memory, read only) with the FP64 eigensolver of stab_full_spectrum, without
 * allocating any device memory.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory when they call, because
 * another allocator owns the GPU's memory (a framework's caching pool, a
 * simulation with a fixed budget) or because the device-wide synchronisation
 * of cudaFree is not acceptable on their path.
 *   a_dev       m x m input on the device (not modified)
 *   eig_dev     m complex128 outputs on the device, unsorted: the QR
 *               eigenvalues first, then those split off by isolation
 *   status_dev  one int32 on the device: STAB_ST_OK or STAB_ST_NOCONV
 *   stream      cudaStream_t to launch on (NULL: the legacy default stream)
 * Limits and sharing: m must be 1..STAB_NOALLOC_MAX_M (larger m returns
 * STAB_ERR_ARG).  The working matrix lives in one fixed 1 MiB array of the
 * library on each device (held until the process exits), shared by every
 * call: calls that overlap on the GPU (different streams, or different host
 * threads) race and must be serialised by the caller.  The first call on a
 * device looks up that array's device address, so make it before any stream
 * capture; a lookup that fails returns STAB_ERR_CUDA and is tried again by
 * the next call.  Under CUDA's lazy module loading (the default) that first
 * call also makes the driver load this part of the library on the device
 * and allocate the array then: make it at start-up, or set
 * CUDA_MODULE_LOADING=EAGER to have the array created when the library
 * loads.  Later calls allocate nothing.  Each call adds its cycles to the
 * counters stab_eig_phases reads.  Needs no stab_ctx.
 */
int stab_eigvals_noalloc(const double* a_dev, int32_t m, double* eig_dev, int32_t* status_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* STAB_GB300_H */
