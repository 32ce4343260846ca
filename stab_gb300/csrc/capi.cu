// C ABI of libstab_gb300: context, batches and the orchestration of the
// kernels of prep.cu, assemble.cu, lu.cu, hqr.cu, polish.cu and post.cu.
//
// Batch order: instances are kept internally with all temporal instances
// first and all spatial ones after (stable), so each phase launches on
// contiguous ranges; results are mapped back to the caller's order.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/stab_gb300.h"
#include "common.cuh"
#include "dw.cuh"
#include "hqr.cuh"
#include "kernels.cuh"
#include "lu.cuh"
#include "mlp.cuh"
#include "polish.cuh"

using namespace stab;

// shift candidates per instance taken from the coarse spectrum
static const int kShiftCandidates = 4;
// a polished eigenvalue within this relative distance of the top coarse
// candidate is final after the first round (the coarse mode is resolved)
static const double kQuickAcceptTol = 1e-7;
// a complex64 polish that needed this many Newton-chord steps or more is
// retried with complex128 factors (slow contraction: an unresolved cluster)
static const int kSlowNewton = 14;
// `done` value of an instance whose kept pair came from the caller's seed in
// STAB_MODE_SURROGATE without a resolved coarse candidate: a converged
// eigenpair that nothing verified as the least-stable (STAB_ST_UNVERIFIED)
static const int kDoneUnverified = 5;

namespace {

struct KStat {
  std::string name;
  int64_t launches = 0;
  double ms = 0.0;
};
struct PendingEv {
  int idx;
  cudaEvent_t a, b;
};

}  // namespace

struct stab_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  std::map<int, std::pair<double*, double*>> dtabs;  // table key -> (D1, D2) on the device
  std::map<int, std::pair<float*, float*>> dtabs32;  // the same tables rounded to float (complex64 assembly)
  int profiling = 0;
  std::vector<KStat> stats;
  std::vector<PendingEv> pending;
  std::vector<cudaEvent_t> evpool;
  int sms = 152;
  std::vector<stab_batch*> live;   // caller-visible batches, released by stab_destroy
  std::vector<stab_mlp*> nets;     // networks, released by stab_destroy
  std::map<std::pair<int, int>, int> lu_nb;   // (complex128?, size class) -> tuned LU panel width
  // arithmetic per stage (STAB_STAGE_*)
  int arith[4] = {STAB_ARITH_DOUBLE_WORD, STAB_ARITH_FP64, STAB_ARITH_DOUBLE_WORD, STAB_ARITH_TF32_SPLIT};
  int seed_ny = 32;        // N of the seed spectrum of STAB_MODE_COARSE / SURROGATE
  int seed_qr_shared = 0;  // STAB_OPT_SEED_QR_SHARED
  int lu_tma = 1;          // STAB_OPT_POLISH_LU_TMA
  int eig_resident = 0;    // STAB_OPT_EIG_RESIDENT
  int eig_threads = 128;   // STAB_OPT_EIG_THREADS
  int eig_mid = 1;         // STAB_OPT_EIG_MID
  int seed_vectors = 1;    // STAB_OPT_SEED_VECTORS
  int par_cand = 1;        // STAB_OPT_PARALLEL_CANDIDATES
  int medium_ny = 48;      // STAB_OPT_MEDIUM_NY: N of the second candidate level
  int first_retry = 1;     // STAB_OPT_FIRST_RETRY
  int level_trust = 1;     // STAB_OPT_LEVEL_CONSISTENCY
  int medium_ny_sp = 24;   // STAB_OPT_MEDIUM_NY_SPATIAL: N of the spatial instances' second level
  int mlp_tc = 1;          // STAB_OPT_MLP_TCGEN05: surrogate GEMMs on tcgen05 (0: mma.sync)
  int epoch = 0;           // bumped by every setting that changes the launched kernels
};

// size class of an LU order for the tuned panel-width table
static int lu_class(int n) {
  static const int cls[] = {160, 240, 320, 480, 640, 960, 1280, 1920};
  for (int q : cls)
    if (n <= q) return q;
  return 1 << 30;
}
static int tuned_nb(stab_ctx* c, bool z, int n) {
  auto it = c->lu_nb.find({z ? 1 : 0, lu_class(n)});
  return it == c->lu_nb.end() ? 0 : it->second;
}
static void release_net(stab_mlp* m);

static int set_err(stab_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
static int cuda_fail(stab_ctx* c, cudaError_t e, const char* what) {
  return set_err(c, STAB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(ctx, expr)                                  \
  do {                                                 \
    cudaError_t e_ = (expr);                           \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr); \
  } while (0)

static cudaEvent_t get_ev(stab_ctx* c) {
  if (!c->evpool.empty()) {
    cudaEvent_t e = c->evpool.back();
    c->evpool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
static int stat_index(stab_ctx* c, const char* name) {
  for (size_t i = 0; i < c->stats.size(); ++i)
    if (c->stats[i].name == name) return (int)i;
  c->stats.push_back(KStat{name, 0, 0.0});
  return (int)c->stats.size() - 1;
}
// Launch through f(); with profiling on, bracket it with events on the
// context stream and account the time to `name`.
template <typename F>
static cudaError_t timed(stab_ctx* c, const char* name, F&& f) {
  if (!c->profiling) return f();
  cudaEvent_t a = get_ev(c), b = get_ev(c);
  cudaEventRecord(a, c->stream);
  cudaError_t e = f();
  cudaEventRecord(b, c->stream);
  c->pending.push_back(PendingEv{stat_index(c, name), a, b});
  return e;
}
static void drain_stats(stab_ctx* c) {
  if (c->pending.empty()) return;
  cudaStreamSynchronize(c->stream);
  for (auto& p : c->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    c->stats[p.idx].launches += 1;
    c->stats[p.idx].ms += ms;
    c->evpool.push_back(p.a);
    c->evpool.push_back(p.b);
  }
  c->pending.clear();
}

// itype 2 (Chebyshev) and 4 (finite differences) are spatial
static inline bool is_spatial(int itype) { return itype == 2 || itype == 4; }

// Derivative tables, built once per context, by key: ny for the Chebyshev
// D1 and D1 D1; kFdOpKey + ny for the finite-difference operator's stencil
// matrices (temporal), kFdSpKey + ny for the spatial ones; kFdMeanKey + ny
// for grad.f90's matrix G and G G.
static const int kFdOpKey = 1 << 20, kFdMeanKey = 2 << 20, kFdSpKey = 3 << 20;

// stencils.f90:9-120, the reference's coefficient table (values as written there)
static const double kGa[4] = {8.333333333333333333333E-02, -6.666666666666666666667E-01, 6.666666666666666666667E-01,
                              -8.333333333333333333333E-02};
static const double kGg[6] = {-1.87603205562073772290017534999, 3.18538322557789286703668141674,
                              -1.81454567943752757247830550034, 0.59165824105260274421658150053,
                              -0.101052068000505624644095417028, 0.0145883364282753087693133500917};
static const double kGh[6] = {-0.384254232677925402043233692192, -0.290638947767348681070279077173,
                              0.67176478451531541138011989728, 0.071081659837399872713651693126,
                              -0.073630718761724245070378308432, 0.0056774548542830440901194873933};
static const double kGi[6] = {0.182885278686826206583549109115, -1.08001475417455516433881053795,
                              0.65787289649662525818641772732, 0.1776170486891931456381189546,
                              0.076779836395827558602005515075, -0.0151403060939170046712807681567};
static const double kGj[6] = {-0.0341837103365291857798396404953, 0.224829025740103121729831613399,
                              -0.89081233292845396245426338198, 0.165299947710035014782196870489,
                              0.61343955208752529977826815383, -0.078572482272680288056193615249};
static const double kDa[5] = {-8.333333333333333333333E-02, 1.333333333333333333333E+00, -2.500000000000000000000E+00,
                              1.333333333333333333333E+00, -8.333333333333333333333E-02};
static const double kDb[5] = {9.166666666666666666667E-01, -1.666666666666666666667E+00, 5.000000000000000000000E-01,
                              3.333333333333333333333E-01, -8.333333333333333333333E-02};
static const double kDd[5] = {2.916666666666666666667E+00, -8.666666666666666666667E+00, 9.500000000000000000000E+00,
                              -4.666666666666666666667E+00, 9.166666666666666666667E-01};

// Row-major ny x ny stencil matrices of the finite-difference solver, node 0
// at the wall (fd_temporal.f90:636-895): F1 multiplies Bh, F2 multiplies
// Vyy.  Rows 0-3 the one-sided and biased closures, central rows, the
// mirrored closures with the signs the reference writes (+da4 and +da5 on
// row ny-4, +da4 on row ny-3), and a zero free-stream row.
static void fd_operator_tables(int ny, std::vector<double>& F1, std::vector<double>& F2) {
  const double dy = 1.0 / (double)(ny - 1);
  F1.assign((size_t)ny * ny, 0.0);
  F2.assign((size_t)ny * ny, 0.0);
  auto f1 = [&](int i, int j, double v) { F1[(size_t)i * ny + j] = v / dy; };
  auto f2 = [&](int i, int j, double v) { F2[(size_t)i * ny + j] = v / (dy * dy); };
  for (int t = 0; t < 6; ++t) { f1(0, t, kGg[t]); f1(1, t, kGh[t]); f1(2, t, kGi[t]); f1(3, t, kGj[t]); }
  for (int t = 0; t < 5; ++t) { f2(0, t, kDd[t]); f2(1, t, kDb[t]); f2(2, t, kDa[t]); f2(3, 1 + t, kDa[t]); }
  for (int i = 4; i < ny - 4; ++i) {
    f1(i, i - 2, kGa[0]); f1(i, i - 1, kGa[1]); f1(i, i + 1, kGa[2]); f1(i, i + 2, kGa[3]);
    for (int t = 0; t < 5; ++t) f2(i, i - 2 + t, kDa[t]);
  }
  int i = ny - 4;
  for (int t = 0; t < 6; ++t) f1(i, i - 2 + t, -kGj[5 - t]);
  for (int t = 0; t < 5; ++t) f2(i, i - 2 + t, t < 3 ? kDa[t] : -kDa[t]);
  i = ny - 3;
  for (int t = 0; t < 6; ++t) f1(i, i - 3 + t, -kGi[5 - t]);
  for (int t = 0; t < 5; ++t) f2(i, i - 2 + t, t == 3 ? -kDa[t] : kDa[t]);
  i = ny - 2;
  for (int t = 0; t < 6; ++t) f1(i, i - 4 + t, -kGh[5 - t]);
  for (int t = 0; t < 5; ++t) f2(i, i - 3 + t, kDb[4 - t]);
}

// The spatial solver's stencil matrices (fd_spatial.f90:668-1160): rows
// 0-3 and the central rows as above, the central rows running to ny-3, row
// ny-2 the biased (-1, 6, -18, 10, 3)/12 with the mirrored db, row ny-1 the
// one-sided (3, -16, 36, -48, 25)/12 of the top = 1 continuity rows.
static void fd_spatial_tables(int ny, std::vector<double>& F1, std::vector<double>& F2) {
  const double dy = 1.0 / (double)(ny - 1);
  F1.assign((size_t)ny * ny, 0.0);
  F2.assign((size_t)ny * ny, 0.0);
  auto f1 = [&](int i, int j, double v) { F1[(size_t)i * ny + j] = v / dy; };
  auto f2 = [&](int i, int j, double v) { F2[(size_t)i * ny + j] = v / (dy * dy); };
  for (int t = 0; t < 6; ++t) { f1(0, t, kGg[t]); f1(1, t, kGh[t]); f1(2, t, kGi[t]); f1(3, t, kGj[t]); }
  for (int t = 0; t < 5; ++t) { f2(0, t, kDd[t]); f2(1, t, kDb[t]); f2(2, t, kDa[t]); f2(3, 1 + t, kDa[t]); }
  for (int i = 4; i < ny - 2; ++i) {
    f1(i, i - 2, kGa[0]); f1(i, i - 1, kGa[1]); f1(i, i + 1, kGa[2]); f1(i, i + 2, kGa[3]);
    for (int t = 0; t < 5; ++t) f2(i, i - 2 + t, kDa[t]);
  }
  const double b5[5] = {-1.0, 6.0, -18.0, 10.0, 3.0}, t5[5] = {3.0, -16.0, 36.0, -48.0, 25.0};
  int i = ny - 2;
  for (int t = 0; t < 5; ++t) { f1(i, i - 3 + t, b5[t] / 12.0); f2(i, i - 3 + t, kDb[4 - t]); }
  i = ny - 1;
  for (int t = 0; t < 5; ++t) f1(i, i - 4 + t, t5[t] / 12.0);
}

// grad.f90:62-86 as a matrix G (fourth-order five-point stencils, one-sided
// and biased at both ends, over 12 deta), and G G.
static void fd_mean_tables(int ny, std::vector<double>& G, std::vector<double>& GG) {
  const double dy = 1.0 / (double)(ny - 1);
  G.assign((size_t)ny * ny, 0.0);
  auto g = [&](int i, int j, double v) { G[(size_t)i * ny + j] = v / (12.0 * dy); };
  const double r0[5] = {-25.0, 48.0, -36.0, 16.0, -3.0}, r1[5] = {-3.0, -10.0, 18.0, -6.0, 1.0};
  for (int t = 0; t < 5; ++t) { g(0, t, r0[t]); g(1, t, r1[t]); }
  const double c[5] = {1.0, -8.0, 0.0, 8.0, -1.0};
  for (int i = 2; i < ny - 2; ++i)
    for (int t = 0; t < 5; ++t) if (c[t] != 0.0) g(i, i - 2 + t, c[t]);
  for (int t = 0; t < 5; ++t) { g(ny - 2, ny - 1 - t, -r1[t]); g(ny - 1, ny - 1 - t, -r0[t]); }
  GG.assign((size_t)ny * ny, 0.0);
  for (int i = 0; i < ny; ++i)
    for (int k = 0; k < ny; ++k) {
      const double a = G[(size_t)i * ny + k];
      if (a == 0.0) continue;
      for (int j = 0; j < ny; ++j) GG[(size_t)i * ny + j] += a * G[(size_t)k * ny + j];
    }
}

// float copies of a table pair (the complex64 assembly computes in FP32)
static int ensure_dtab32(stab_ctx* c, int key, int ny) {
  float *F1 = nullptr, *F2 = nullptr;
  CK(c, cudaMalloc(&F1, sizeof(float) * ny * ny));
  if (cudaMalloc(&F2, sizeof(float) * ny * ny) != cudaSuccess) {
    cudaFree(F1);
    return cuda_fail(c, cudaGetLastError(), "cudaMalloc of a float D table");
  }
  CK(c, launch_round_f32((int64_t)ny * ny, c->dtabs[key].first, F1, c->stream));
  CK(c, launch_round_f32((int64_t)ny * ny, c->dtabs[key].second, F2, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->dtabs32[key] = {F1, F2};
  return 0;
}

static int ensure_dtab(stab_ctx* c, int key) {
  if (c->dtabs.count(key)) {
    if (c->dtabs32.count(key)) return 0;
    // the float copies failed earlier (allocation): build them now
    const int ny = key >= kFdOpKey ? (key & (kFdOpKey - 1)) : key;
    return ensure_dtab32(c, key, ny);
  }
  if (key >= kFdOpKey) {
    const int ny = key & (kFdOpKey - 1);
    std::vector<double> T1, T2;
    if (key >= kFdSpKey) fd_spatial_tables(ny, T1, T2);
    else if (key >= kFdMeanKey) fd_mean_tables(ny, T1, T2);
    else fd_operator_tables(ny, T1, T2);
    double *D1 = nullptr, *D2 = nullptr;
    CK(c, cudaMalloc(&D1, sizeof(double) * ny * ny));
    CK(c, cudaMalloc(&D2, sizeof(double) * ny * ny));
    CK(c, cudaMemcpy(D1, T1.data(), sizeof(double) * ny * ny, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(D2, T2.data(), sizeof(double) * ny * ny, cudaMemcpyHostToDevice));
    c->dtabs[key] = {D1, D2};
    return ensure_dtab32(c, key, ny);
  }
  const int ny = key;
  double *D1 = nullptr, *D2 = nullptr, *xa = nullptr;
  CK(c, cudaMalloc(&D1, sizeof(double) * ny * ny));
  CK(c, cudaMalloc(&D2, sizeof(double) * ny * ny));
  CK(c, cudaMalloc(&xa, sizeof(double) * 2 * ny));
  k_cheb_a<<<(ny + 127) / 128, 128, 0, c->stream>>>(ny, xa);
  CK(c, cudaGetLastError());
  dim3 g((ny + 127) / 128, ny);
  k_cheb_d1<<<g, 128, 0, c->stream>>>(ny, xa, D1);
  CK(c, cudaGetLastError());
  k_cheb_d2<<<g, 128, 0, c->stream>>>(ny, D1, D2);
  CK(c, cudaGetLastError());
  CK(c, cudaStreamSynchronize(c->stream));
  cudaFree(xa);
  c->dtabs[key] = {D1, D2};
  return ensure_dtab32(c, key, ny);
}

// ---------------------------------------------------------------------------
// device buffer helpers
// ---------------------------------------------------------------------------
namespace {
// Device buffer from the stream-ordered allocator: the context keeps the
// device's default pool from releasing memory, so batches created per call
// reuse it instead of paying cudaMalloc each time.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, st);
  }
  cudaError_t ensure(size_t b, cudaStream_t s) {
    if (b <= bytes && p) return cudaSuccess;
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    bytes = 0;
    if (b == 0) b = 16;
    st = s;
    cudaError_t e = cudaMallocAsync(&p, b, s);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};
template <typename T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
  cudaError_t e = b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1), s);
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  return cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
}
}  // namespace

// ---------------------------------------------------------------------------
// batch
// ---------------------------------------------------------------------------
struct stab_batch {
  stab_ctx* ctx = nullptr;
  int count = 0, tcount = 0;             // tcount temporal instances first
  std::vector<stab_params> P;            // internal order (ny of the solve)
  std::vector<stab_params> Pin;          // internal order, the caller's parameters unchanged
  std::vector<int> perm;                 // internal k -> caller index
  std::vector<InstDesc> hd;
  std::vector<int32_t> hn, hm;
  std::vector<int64_t> h_n2, h_m2, h_m2c2, h_nof, h_mof, h_vec;
  int nmax = 0, mmax = 0;
  size_t sum_n2 = 0, sum_m2 = 0, sum_n = 0, sum_m = 0;
  // device
  DevBuf desc, dtab, dtab32, pdesc, prof, spl, node, blk, ops, ops32, vec;
  DevBuf nsz, msz, off_n2, off_m2, off_m2c2, off_nof, off_mof, xoff[VEC_SLOTS], order;
  DevBuf M32, Z64, Abig, Hbig, eigraw, eigsorted, outvec;
  DevBuf bad, flops, rsc, csc, cand, accepted, skip64, lus32, lus64, have, best_key, best_theta, best_err, best_iters, best_out;
  DevBuf piv, info, flags, theta, sigma, least_raw, least_val, least_idx, pcol, done, err, iters, status, counter;
  int nprof = 0;
  // profile pools in use: this batch's own (prof, spl, bad, pdesc), or its
  // parent's for a sub-batch (shared_prof), whose prep skips k_spline
  bool shared_prof = false;
  const double* prof_p = nullptr;
  double* spl_p = nullptr;
  int32_t* bad_p = nullptr;
  const ProfDesc* pdesc_p = nullptr;
  bool have_seeds = false;
  std::vector<double> seeds;             // caller order, 2 per instance
  int last_mode = -1;
  bool ran = false;
  // instances re-solved by the plain FP64 path after a failed polish
  std::vector<int> fell_back;                 // internal indices
  double fb_work[4] = {0.0, 0.0, 0.0, 0.0};   // sub-batch work, indexed as stab_batch_work's output
  std::vector<double> fb_err;
  std::vector<int32_t> fb_iters;
  int32_t counts[3] = {0, 0, 0};              // from seeds, from the coarse sub-batch, plain fallback
  std::vector<double> start_coef;             // caller order: count x 5 x ncheb complex
  int ncheb = 0;
  bool use_start = false;
  DevBuf startc;
  DevBuf seedc;               // coarse-level eigenvectors as Chebyshev coefficients (count x 5 x seedc_n)
  int seedc_n = 0;
  bool has_fd = false;        // a finite-difference instance (no Chebyshev grid)
  DevBuf seed_raw, best_src;                  // STAB_MODE_SURROGATE: the extra candidate, winner per instance
  DevBuf tmaps;                               // tensor maps of the complex64 matrices (TMA tiles of the LU)
  int tmaps_state = 0;                        // 0 not built, 1 built, -1 not possible (odd order)
  int graph_mode = -1;                        // mode of the captured graph
  int graph_epoch = -1;                       // context settings the graph was captured under
  int coarse_ny = 32;                         // N of the seed spectrum of STAB_MODE_COARSE
  int coarse_ny_sp = 32;                      // the same for the spatial instances
  int level = 1;                              // candidate level: 1 first (seed size), 2 the second
  std::vector<zc> fb_val;
  std::vector<int32_t> fb_status;
  std::vector<std::vector<zc>> fb_vec;
  stab_batch* coarse = nullptr;               // N = 32 batch of STAB_MODE_COARSE, built on first use
  stab_batch* copies = nullptr;               // one instance per shift candidate (the N = 48 level's rounds)
  // second-level batches: the first level's top candidate, its polished
  // pair and whether that converged, per instance (STAB_OPT_LEVEL_CONSISTENCY)
  DevBuf lev1_idx, lev1_lam, lev1_th, lev1_ok;
  bool has_lev1 = false;
  int lev1_n = 32;                            // N of the first level's seed spectra
  // the device work of a STAB_MODE_COARSE pass (prep, N = 32 eigensolve,
  // candidate rounds) captured once as a CUDA graph and replayed
  cudaGraphExec_t coarse_graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  int coarse_runs = 0;
  ~stab_batch();
  // free every device buffer now (used when the owning context goes away first)
  void release() {
    DevBuf* all[] = {&desc, &dtab, &dtab32, &pdesc, &prof, &spl, &node, &blk, &ops, &ops32, &vec, &nsz, &msz, &off_n2, &off_m2,
                     &off_m2c2, &off_nof, &off_mof, &order, &M32, &Z64, &Abig, &Hbig, &eigraw, &eigsorted, &outvec,
                     &bad, &flops, &rsc, &csc, &cand, &accepted, &skip64, &lus32, &lus64, &have, &best_key, &best_theta, &best_err,
                     &best_iters, &best_out, &piv, &info, &flags, &theta, &sigma, &least_raw, &least_val, &least_idx, &pcol,
                     &done, &err, &iters, &status, &counter, &startc, &seedc, &seed_raw, &best_src, &tmaps,
                     &lev1_idx, &lev1_lam, &lev1_th, &lev1_ok};
    for (DevBuf* d : all) {
      if (d->p) cudaFreeAsync(d->p, d->st);
      d->p = nullptr;
      d->bytes = 0;
    }
    for (auto& x : xoff) {
      if (x.p) cudaFreeAsync(x.p, x.st);
      x.p = nullptr;
      x.bytes = 0;
    }
    delete coarse;
    coarse = nullptr;
    delete copies;
    copies = nullptr;
    if (coarse_graph) cudaGraphExecDestroy(coarse_graph);
    coarse_graph = nullptr;
  }
};

stab_batch::~stab_batch() {
  delete coarse;
  delete copies;
}

// The station-independent scalars of circh (circh.f90:2-188, with xcloc and
// ycloc, :201-229): the wall of a circle of radius s at arc position 0.
// out = dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2; h(y) and
// its derivatives follow in k_blocks (circh.f90:190-199).
static void circh_scalars(double s, double out[8]) {
  const double infty = 1.0e30;
  const double radius = s;
  const double th1 = std::atan2(std::sqrt(radius * radius - 0.0), 0.0);   // xcloc(0, 0)
  const double xl = radius * std::cos(th1 - 0.0);
  const double yl = std::sqrt(radius * radius - xl * xl);                   // ycloc(xl)
  const double th = std::atan2(-xl, std::sqrt(radius * radius - xl * xl));
  const double bn1 = -std::sin(th), bn2 = std::cos(th);
  const double dydx = (xl == 0.0) ? -infty : (-xl) / yl;
  const double dxbds = 1.0 / std::sqrt(1.0 + dydx * dydx);
  const double dxdy = (xl == 0.0) ? -infty : yl / (-xl);
  const double dybds = (xl <= 0.0) ? 1.0 / std::sqrt(dxdy * dxdy + 1.0) : -1.0 / std::sqrt(dxdy * dxdy + 1.0);
  double dx, dy, ddxdx, ddydx, ddxdy, ddydy, d2dxdx2, d2dydx2, d2dxdy2, d2dydy2;
  if (yl == 0.0) {
    dx = 0.0; dy = -xl; ddxdx = -infty; ddydx = -1.0; ddxdy = 1.0; ddydy = 0.0;
    d2dxdx2 = -infty; d2dydx2 = 0.0; d2dxdy2 = 0.0; d2dydy2 = (xl * xl + yl * yl) / (xl * xl * xl);
  } else if (xl == 0.0) {
    dx = yl; dy = 0.0; ddxdx = 0.0; ddydx = -1.0; ddxdy = 1.0; ddydy = infty;
    d2dxdx2 = -(yl * yl + xl * xl) / (yl * yl * yl); d2dydx2 = 0.0; d2dxdy2 = 0.0; d2dydy2 = infty;
  } else {
    dx = yl; dy = -xl; ddxdx = -xl / yl; ddydx = -1.0; ddxdy = 1.0; ddydy = yl / xl;
    d2dxdx2 = -(yl * yl + xl * xl) / (yl * yl * yl); d2dydx2 = 0.0; d2dxdy2 = 0.0;
    d2dydy2 = (xl * xl + yl * yl) / (xl * xl * xl);
  }
  const double q = dx * dx + dy * dy;
  const double q05 = std::pow(q, 0.5), q15 = std::pow(q, 1.5), q25 = std::pow(q, 2.5);
  const bool nflat = std::fabs(bn1) > std::fabs(bn2);
  // derivatives along the arc through y (nflat) or through x
  const double ddx = nflat ? ddxdy : ddxdx, ddy = nflat ? ddydy : ddydx;
  const double d2dx = nflat ? d2dxdy2 : d2dxdx2, d2dy = nflat ? d2dydy2 : d2dydx2;
  const double dsd = nflat ? dybds : dxbds;
  const double dbn1 = (-ddy / q05 + 0.5 * dy * (2.0 * dx * ddx + 2.0 * dy * ddy) / q15) * dsd;
  const double dbn2 = (ddx / q05 - 0.5 * dx * (2.0 * dx * ddx + 2.0 * dy * ddy) / q15) * dsd;
  double d2xbds2, d2ybds2;
  if (nflat) {
    const double d2xdy2 = -(xl * xl + yl * yl) / (xl * xl * xl);
    d2ybds2 = (xl <= 0 ? -1.0 : 1.0) * std::pow(1.0 + dxdy * dxdy, -1.5) * dxdy * d2xdy2 * dybds;
    d2xbds2 = d2xdy2 * dybds * dybds + dxdy * d2ybds2;
  } else {
    const double d2ydx2 = -(xl * xl + yl * yl) / (yl * yl * yl);
    d2xbds2 = -std::pow(1.0 + dydx * dydx, -1.5) * dydx * d2ydx2 * dxbds;
    d2ybds2 = d2ydx2 * dxbds * dxbds + dydx * d2xbds2;
  }
  const double d2s = nflat ? d2ybds2 : d2xbds2;
  const double t1 = dy * ddx - dx * ddy, t2 = dx * ddx + dy * ddy;
  double d2bn1 = ((ddx * t1 + dx * (dy * d2dx - dx * d2dy)) / q15 - (3.0 * dx * t1 * t2) / q25) * dsd * dsd +
                 (-ddy / q05 + 0.5 * dy * (2.0 * dx * ddx + 2.0 * dy * ddy) / q15) * d2s;
  const double d2bn2 = ((ddy * t1 + dy * (dy * d2dx - dx * d2dy)) / q15 - (3.0 * dy * t1 * t2) / q25) * dsd * dsd +
                       (ddx / q05 - 0.5 * dx * (2.0 * dx * ddx + 2.0 * dy * ddy) / q15) * d2s;
  if (xl == 0.0) d2bn1 = 0.0;
  const double v[8] = {dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2};
  for (int i = 0; i < 8; ++i) out[i] = v[i];
}

// Arc length of the parabolic cylinder y = sqrt(2 x) from x1 to x2
// (calch.f90, function arc).
static double parabola_arc(double x1, double x2) {
  auto f = [](double x) {
    const double xi = std::sqrt(x), t = std::sqrt(1.0 + 2.0 * xi * xi);
    return std::sqrt(2.0) * 0.5 * xi * t + 0.5 * std::log(std::sqrt(2.0) * xi + t);
  };
  return f(x2) - f(x1);
}

// The method of false position as published in Numerical Recipes (Press,
// Teukolsky, Vetterling, Flannery, 2nd ed. 1992, section 9.2, routine
// rtflsp), which calch.f90's xloc calls and the reference does not ship:
// the endpoints with f < 0 and f >= 0 are kept, the one on the side of the
// secant root is replaced, and the search ends when the replaced endpoint
// moved less than xacc or f is exactly zero; 30 secant steps at most.
// Returns false where that routine stops the program (no bracket, no
// convergence).
template <class F>
static bool false_position(F f, double x1, double x2, double xacc, double& root) {
  double fl = f(x1), fh = f(x2);
  if (fl * fh > 0.0) return false;
  double lo = x1, hi = x2;
  if (!(fl < 0.0)) {
    std::swap(lo, hi);
    std::swap(fl, fh);
  }
  for (int it = 0; it < 30; ++it) {
    if (fl == fh) return false;
    const double x = lo + (hi - lo) * fl / (fl - fh);
    const double fx = f(x);
    double moved;
    if (fx < 0.0) {
      moved = lo - x;
      lo = x;
      fl = fx;
    } else {
      moved = hi - x;
      hi = x;
      fh = fx;
    }
    if (std::fabs(moved) < xacc || fx == 0.0) {
      root = x;
      return true;
    }
  }
  return false;
}

// The station-independent scalars of calch (calch.f90:31-148): the wall of
// the parabolic cylinder y = sqrt(2 x) at arc length s from its nose, the
// point located by xloc (calch.f90:170-184): false position on [0, 2 s] to
// 1e-12.  Same outputs as circh_scalars; h(y) and its derivatives follow in
// k_blocks with the closing formulas both routines share (calch.f90:152-167).
static bool calch_scalars(double s, double out[8]) {
  const double infty = 1.0e30;
  double xl = 0.0;
  if (!false_position([s](double x) { return s - parabola_arc(0.0, x); }, 0.0, 0.0 + 2.0 * s, 1.0e-12, xl))
    return false;
  const double yl = std::sqrt(2.0 * xl);
  const double th = std::atan2(1.0, yl);
  const double bn1 = -std::sin(th), bn2 = std::cos(th);
  const double dydx = (xl == 0.0) ? infty : 1.0 / std::sqrt(2.0 * xl);
  const double dxbds = 1.0 / std::sqrt(1.0 + dydx * dydx);
  const double dxdy = (xl == 0.0) ? 0.0 : std::sqrt(2.0 * xl);
  const double dybds = 1.0 / std::sqrt(dxdy * dxdy + 1.0);
  const double dx = (xl == 0.0) ? 0.0 : yl, dy = 1.0;
  const double ddxdx = (xl == 0.0) ? infty : 1.0 / yl, ddydx = 0.0, ddxdy = 1.0, ddydy = 0.0;
  const double d2dxdx2 = (xl == 0.0) ? infty : -std::sqrt(2.0) / (4.0 * std::pow(xl, 1.5));
  const double d2dydx2 = 0.0, d2dxdy2 = 0.0, d2dydy2 = 0.0;
  const double q = dx * dx + dy * dy, q05 = std::sqrt(q), q15 = std::pow(q, 1.5), q25 = std::pow(q, 2.5);
  double dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2;
  if (std::fabs(bn1) > std::fabs(bn2)) {   // the wall leans toward the y axis: derivatives through y
    dbn1 = (-ddydy / q05 + 0.5 * dy * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q15) * dybds;
    dbn2 = (ddxdy / q05 - 0.5 * dx * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q15) * dybds;
    const double d2xdy2 = 1.0;
    d2ybds2 = -std::pow(1.0 + dxdy * dxdy, -1.5) * dxdy * d2xdy2 * dybds;
    d2xbds2 = d2xdy2 * (dybds * dybds) + dxdy * d2ybds2;
    const double t1 = dy * ddxdy - dx * ddydy, t2 = dx * ddxdy + dy * ddydy;
    d2bn1 = ((ddxdy * t1 + dx * (dy * d2dxdy2 - dx * d2dydy2)) / q15 - (3.0 * dx * t1 * t2) / q25) * (dybds * dybds) +
            (-ddydy / q05 + 0.5 * dy * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q15) * d2ybds2;
    d2bn2 = ((ddydy * t1 + dy * (dy * d2dxdy2 - dx * d2dydy2)) / q15 - (3.0 * dy * t1 * t2) / q25) * (dybds * dybds) +
            (ddxdy / q05 - 0.5 * dx * (2.0 * dx * ddxdy + 2.0 * dy * ddydy) / q15) * d2ybds2;
  } else {                                  // through x
    dbn1 = (-ddydx / q05 + 0.5 * dy * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q15) * dxbds;
    dbn2 = (ddxdx / q05 - 0.5 * dx * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q15) * dxbds;
    const double d2ydx2 = -1.0 / (2.0 * std::sqrt(2.0) * std::pow(xl, 1.5));
    d2xbds2 = -std::pow(1.0 + dydx * dydx, -1.5) * dydx * d2ydx2 * dxbds;
    d2ybds2 = d2ydx2 * (dxbds * dxbds) + dydx * d2xbds2;
    const double t1 = dy * ddxdx - dx * ddydx, t2 = dx * ddxdx + dy * ddydx;
    d2bn1 = ((ddxdx * t1 + dx * (dy * d2dxdx2 - dx * d2dydx2)) / q15 - (3.0 * dx * t1 * t2) / q25) * (dxbds * dxbds) +
            (-ddydx / q05 + 0.5 * dy * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q15) * d2xbds2;
    d2bn2 = ((ddydx * t1 + dy * (dy * d2dxdx2 - dx * d2dydx2)) / q15 - (3.0 * dy * t1 * t2) / q25) * (dxbds * dxbds) +
            (ddxdx / q05 - 0.5 * dx * (2.0 * dx * ddxdx + 2.0 * dy * ddydx) / q15) * d2xbds2;
  }
  const double v[8] = {dxbds, dybds, dbn1, dbn2, d2xbds2, d2ybds2, d2bn1, d2bn2};
  for (int i = 0; i < 8; ++i) out[i] = v[i];
  return true;
}

// Descriptor of one instance from its run parameters (validated) and the
// entry of its mean profile in the profile pools.
static int make_desc(stab_ctx* c, const stab_params& q, int iprof, const ProfDesc& pd, InstDesc& d) {
  if (q.itype < 1 || q.itype > 4)
    return set_err(c, STAB_ERR_ARG, "itype must be 1 (temporal), 2 (spatial), 3 or 4 (the same by finite differences)");
  const bool fd = (q.itype == 3 || q.itype == 4);
  const bool spat = (q.itype == 2 || q.itype == 4);
  if (fd && q.ny < 10) return set_err(c, STAB_ERR_ARG, "the finite-difference solvers need ny >= 10");
  if (fd && !(q.yi != 0.0 && q.ymax > 2.0 * q.yi))
    return set_err(c, STAB_ERR_ARG, "the finite-difference grid (ogengrid) needs Yi != 0 and Ymax > 2 Yi");
  if (q.ny < 4 || q.ny > 400) return set_err(c, STAB_ERR_ARG, "ny out of range [4, 400]");
  if (spat && q.curve != 0 && q.curve != 1 && q.curve != 2)
    return set_err(c, STAB_ERR_ARG, "curve must be 0, 1 or 2");
  if (spat && q.curve == 1 && q.x != -1.0 && !(q.x > 0.0))
    return set_err(c, STAB_ERR_ARG, "curve = 1 needs an arc length x > 0 (or -1, no curvature)");
  if (q.ider != 0 && q.ider != 1) return set_err(c, STAB_ERR_ARG, "ider must be 0 or 1");
  if (q.wallt != 0 && q.wallt != 2) return set_err(c, STAB_ERR_ARG, "Illegal value of wallt");
  if (q.yi == 0.0) return set_err(c, STAB_ERR_ARG, "Yi = 0 (tanh map) is not supported");
  if (q.mattyp != 0 && q.mattyp != 1) return set_err(c, STAB_ERR_ARG, "mattyp must be 0 or 1");
  if (!(q.Ma > 0.0)) return set_err(c, STAB_ERR_ARG, "Ma must be > 0");
  d = InstDesc{};
  d.ny = q.ny;
  d.n = 5 * q.ny;
  d.itype = spat ? 2 : 1;
  d.fd = fd ? 1 : 0;
  d.m = (d.itype == 1) ? d.n : 2 * d.n;
  d.wallt = q.wallt;
  d.top = q.top;
  d.mattyp = q.mattyp;
  d.navier = !(q.Re >= 1.0e98 || q.Re == 0.0);
  d.Ma = q.Ma;
  d.Re = q.Re;
  d.Pr = q.Pr;
  d.Te = (q.mattyp == 1) ? q.T0 : 0.0;   // input.f90:25 runs before Ma is read
  d.yi = q.yi;
  d.ymax = q.ymax;
  d.ar = q.alpha[0]; d.ai = q.alpha[1];
  d.br = q.beta[0]; d.bi = q.beta[1];
  d.wr = q.omega[0]; d.wi = q.omega[1];
  d.iprof = iprof;
  d.nym = pd.nym;
  d.off_prof = pd.off_prof;
  d.off_spl = pd.off_spl;
  d.ider = q.ider;
  // spatial.f90:110-125: the temporal solver has no wall metric; x = -1
  // turns curvature off (calch.f90:31-39, circh.f90:46-53)
  // the finite-difference spatial solver has calch's metric only
  // (fd_spatial.f90:108-116): curve = 2 is a flat wall there
  d.curved = (spat && (q.curve == 1 || (q.curve == 2 && !fd)) && q.x != -1.0) ? 1 : 0;
  if (d.curved && q.curve == 2) circh_scalars(q.x, d.cw);
  if (d.curved && q.curve == 1 && !calch_scalars(q.x, d.cw))
    return set_err(c, STAB_ERR_ARG, "curve = 1: false position found no wall point in 30 steps (the reference's "
                                    "xloc stops there too)");
  return 0;
}

// Tables, offsets and pools of a batch whose P / Pin / perm / hd (profile
// fields filled) are set: node, block and vector offsets, derivative
// tables, per-instance offset arrays and the fixed-size device buffers.
static int batch_finish(stab_ctx* c, stab_batch* b) {
  const int count = b->count;
  std::vector<int> tab_ny;
  int64_t node_off = 0, blk_off = 0, vec_off = 0;
  b->tcount = 0;
  for (auto& d : b->hd) {
    const int kop = d.fd ? (d.itype == 2 ? kFdSpKey : kFdOpKey) + d.ny : d.ny;
    const int kmean = d.fd ? kFdMeanKey + d.ny : d.ny;
    for (int key : {kop, kmean})
      if (std::find(tab_ny.begin(), tab_ny.end(), key) == tab_ny.end()) tab_ny.push_back(key);
    d.off_node = node_off;
    d.off_blk = blk_off;
    d.off_vec = vec_off;
    node_off += (int64_t)NODE_STRIDE * d.ny;
    blk_off += (int64_t)BLK_STRIDE * d.ny;
    vec_off += (int64_t)VEC_SLOTS * d.n;
    if (d.itype == 1) b->tcount++;
    if (d.fd) b->has_fd = true;
  }
  for (int ny : tab_ny) {
    int r = ensure_dtab(c, ny);
    if (r) return r;
  }
  std::vector<double*> hdt;
  std::vector<float*> hdt32;
  std::map<int, int> tab_index;
  for (auto& kv : c->dtabs) {
    tab_index[kv.first] = (int)hdt.size() / 2;
    hdt.push_back(kv.second.first);
    hdt.push_back(kv.second.second);
    hdt32.push_back(c->dtabs32[kv.first].first);
    hdt32.push_back(c->dtabs32[kv.first].second);
  }
  for (auto& d : b->hd) {
    d.dmat = tab_index[d.fd ? (d.itype == 2 ? kFdSpKey : kFdOpKey) + d.ny : d.ny];
    d.dmean = tab_index[d.fd ? kFdMeanKey + d.ny : d.ny];
  }
  // offsets
  for (auto& d : b->hd) {
    b->hn.push_back(d.n);
    b->hm.push_back(d.m);
    b->h_n2.push_back((int64_t)b->sum_n2);
    b->h_m2.push_back((int64_t)b->sum_m2);
    b->h_m2c2.push_back((int64_t)b->sum_m2 + (int64_t)d.m * d.n);   // column n of the companion
    b->h_nof.push_back((int64_t)b->sum_n);
    b->h_mof.push_back((int64_t)b->sum_m);
    b->h_vec.push_back(d.off_vec);
    b->sum_n2 += (size_t)d.n * d.n;
    b->sum_m2 += (size_t)d.m * d.m;
    b->sum_n += d.n;
    b->sum_m += d.m;
    b->nmax = std::max(b->nmax, d.n);
    b->mmax = std::max(b->mmax, d.m);
  }
  cudaStream_t s = c->stream;
  CK(c, upload(b->desc, b->hd, s));
  CK(c, upload(b->dtab, hdt, s));
  CK(c, upload(b->dtab32, hdt32, s));
  CK(c, b->node.ensure(sizeof(double) * node_off, c->stream));
  CK(c, b->blk.ensure(sizeof(zc) * blk_off, c->stream));
  CK(c, b->ops.ensure(sizeof(zc) * (blk_off / BLK_STRIDE) * 75, c->stream));
  CK(c, b->ops32.ensure(sizeof(cc) * (blk_off / BLK_STRIDE) * 75, c->stream));
  CK(c, b->vec.ensure(sizeof(zc) * vec_off, c->stream));
  CK(c, upload(b->nsz, b->hn, s));
  CK(c, upload(b->msz, b->hm, s));
  CK(c, upload(b->off_n2, b->h_n2, s));
  CK(c, upload(b->off_m2, b->h_m2, s));
  CK(c, upload(b->off_m2c2, b->h_m2c2, s));
  CK(c, upload(b->off_nof, b->h_nof, s));
  CK(c, upload(b->off_mof, b->h_mof, s));
  for (int sl = 0; sl < VEC_SLOTS; ++sl) {
    std::vector<int64_t> xo(count);
    for (int k = 0; k < count; ++k) xo[k] = b->h_vec[k] + (int64_t)sl * b->hn[k];
    CK(c, upload(b->xoff[sl], xo, s));
  }
  // processing order of the persistent eigensolver: largest first
  std::vector<int32_t> ord(count);
  for (int k = 0; k < count; ++k) ord[k] = k;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int bb) { return b->hm[a] > b->hm[bb]; });
  CK(c, upload(b->order, ord, s));
  CK(c, b->M32.ensure(sizeof(cc) * b->sum_n2, c->stream));
  CK(c, b->piv.ensure(sizeof(int32_t) * b->sum_n, c->stream));
  CK(c, b->eigraw.ensure(sizeof(zc) * b->sum_m, c->stream));
  CK(c, b->eigsorted.ensure(sizeof(zc) * b->sum_m, c->stream));
  CK(c, b->outvec.ensure(sizeof(zc) * b->sum_m, c->stream));
  const size_t I4 = sizeof(int32_t) * count, Z = sizeof(zc) * count;
  CK(c, b->info.ensure(I4, c->stream));
  CK(c, b->flags.ensure(I4, c->stream));
  CK(c, b->theta.ensure(Z, c->stream));
  CK(c, b->sigma.ensure(Z, c->stream));
  CK(c, b->least_raw.ensure(Z, c->stream));
  CK(c, b->least_val.ensure(Z, c->stream));
  CK(c, b->least_idx.ensure(I4, c->stream));
  CK(c, b->pcol.ensure(I4, c->stream));
  CK(c, b->done.ensure(I4, c->stream));
  CK(c, b->iters.ensure(I4, c->stream));
  CK(c, b->status.ensure(I4, c->stream));
  CK(c, b->err.ensure(sizeof(double) * count, c->stream));
  CK(c, b->flops.ensure(sizeof(double) * count, c->stream));
  CK(c, b->lus32.ensure(I4, c->stream));
  CK(c, b->lus64.ensure(I4, c->stream));
  CK(c, b->rsc.ensure(sizeof(float) * b->sum_n, c->stream));
  CK(c, b->csc.ensure(sizeof(float) * b->sum_n, c->stream));
  CK(c, b->cand.ensure(Z * kShiftCandidates, c->stream));
  CK(c, b->accepted.ensure(I4, c->stream));
  CK(c, b->counter.ensure(sizeof(int32_t) * 4, c->stream));
  CK(c, cudaStreamSynchronize(s));
  return 0;
}

// A batch from caller memory.  The profiles are copied to the device here
// (deduplicated by pointer, in contiguous runs) and the call synchronises
// before it returns, so the caller may free or reuse its buffers at once.
static int batch_build(stab_ctx* c, int32_t count, const stab_params* p, const int32_t* nym,
                       const double* const* profiles, stab_batch** out) {
  if (!c || count <= 0 || !p || !nym || !profiles || !out) return set_err(c, STAB_ERR_ARG, "null argument or count <= 0");
  std::unique_ptr<stab_batch> b(new stab_batch());
  b->ctx = c;
  b->count = count;
  b->coarse_ny = c->seed_ny;
  b->coarse_ny_sp = c->seed_ny;
  std::vector<int> idx(count);
  for (int i = 0; i < count; ++i) idx[i] = i;
  // temporal (itype 1 and 3) before spatial (2 and 4)
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int bb) { return is_spatial(p[a].itype) < is_spatial(p[bb].itype); });
  b->perm = idx;
  // profiles: dedupe by pointer; copied straight from caller memory in
  // contiguous runs (validated on the device by k_spline).  With ider = 0 a
  // row holds three tables side by side (mean, first and second
  // y-derivatives, 6 values each): they become three consecutive profile
  // entries, separated on the host.
  std::map<const double*, int> pidx;
  std::vector<ProfDesc> pds;
  std::vector<std::pair<const double*, int64_t>> runs;   // (source, doubles)
  std::vector<std::vector<double>> staged;                // de-interleaved ider = 0 tables
  int64_t prof_off = 0, spl_off = 0;
  for (int i = 0; i < count; ++i) {
    const double* pp = profiles[i];
    if (!pp) return set_err(c, STAB_ERR_ARG, "null profile pointer");
    if (nym[i] < 4) return set_err(c, STAB_ERR_ARG, "profile needs at least 4 rows");
    const int ntab = (p[i].ider == 0) ? 3 : 1;
    auto it = pidx.find(pp);
    if (it != pidx.end()) {
      if (pds[it->second].nym != nym[i]) return set_err(c, STAB_ERR_ARG, "same profile pointer with different nym");
      if ((pds[it->second].three != 0) != (ntab == 3))
        return set_err(c, STAB_ERR_ARG, "same profile pointer with different ider");
      continue;
    }
    pidx[pp] = (int)pds.size();
    const int64_t len = (int64_t)nym[i] * 6;
    for (int t = 0; t < ntab; ++t) {
      ProfDesc pd{};
      pd.off_prof = prof_off;
      pd.off_spl = spl_off;
      pd.nym = nym[i];
      pd.three = (ntab == 3) ? 1 : 0;
      const double* src = pp;
      if (ntab == 3) {
        std::vector<double> tab((size_t)len);
        for (int64_t r = 0; r < nym[i]; ++r)
          for (int f = 0; f < 6; ++f) tab[(size_t)(6 * r + f)] = pp[18 * r + 6 * t + f];
        staged.push_back(std::move(tab));
        src = staged.back().data();
        runs.push_back({src, len});
      } else if (!runs.empty() && runs.back().first + runs.back().second == pp) {
        runs.back().second += len;
      } else {
        runs.push_back({pp, len});
      }
      prof_off += len;
      spl_off += len;
      pds.push_back(pd);
    }
  }
  b->nprof = (int)pds.size();
  for (int k = 0; k < count; ++k) {
    const int u = idx[k];
    const int ip = pidx[profiles[u]];
    InstDesc d;
    int rc = make_desc(c, p[u], ip, pds[ip], d);
    if (rc) return rc;
    if (d.ider == 0) {
      d.iprof_d1 = ip + 1;
      d.iprof_d2 = ip + 2;
      d.off_prof_d1 = pds[ip + 1].off_prof;
      d.off_spl_d1 = pds[ip + 1].off_spl;
      d.off_prof_d2 = pds[ip + 2].off_prof;
      d.off_spl_d2 = pds[ip + 2].off_spl;
    }
    b->P.push_back(p[u]);
    b->Pin.push_back(p[u]);
    b->hd.push_back(d);
  }
  cudaStream_t s = c->stream;
  CK(c, upload(b->pdesc, pds, s));
  CK(c, b->prof.ensure(sizeof(double) * std::max<int64_t>(prof_off, 1), c->stream));
  {
    int64_t o = 0;
    for (auto& r : runs) {
      CK(c, cudaMemcpyAsync(b->prof.as<double>() + o, r.first, sizeof(double) * r.second, cudaMemcpyHostToDevice, s));
      o += r.second;
    }
  }
  CK(c, b->spl.ensure(sizeof(double) * std::max<int64_t>(spl_off, 1), c->stream));
  CK(c, b->bad.ensure(sizeof(int32_t) * std::max(b->nprof, 1), c->stream));
  b->prof_p = b->prof.as<double>();
  b->spl_p = b->spl.as<double>();
  b->bad_p = b->bad.as<int32_t>();
  b->pdesc_p = b->pdesc.as<ProfDesc>();
  int rc = batch_finish(c, b.get());
  if (rc) return rc;
  *out = b.release();
  return 0;
}

// A batch of instances ks (internal indices, ascending) of `parent`, with
// ny forced to force_ny when > 0 (the seed spectra) and the caller's ny
// otherwise (the fallback).  It reads the parent's device-resident profiles
// and their spline tables, so its prep skips k_spline: the parent must have
// run its prep in the same pass, and must outlive the child.  Internal order
// is the parent's order restricted to ks (still temporal first), perm[q] = q.
// force_ny > 0: every temporal instance takes that N (force_ny_sp the
// spatial ones; 0 keeps the parent's N).
static int batch_build_child(stab_batch* parent, const std::vector<int>& ks, int force_ny, stab_batch** out,
                             int force_ny_sp = -1) {
  if (force_ny_sp < 0) force_ny_sp = force_ny;
  stab_ctx* c = parent->ctx;
  if (ks.empty()) return set_err(c, STAB_ERR_ARG, "empty sub-batch");
  std::unique_ptr<stab_batch> b(new stab_batch());
  b->ctx = c;
  b->count = (int)ks.size();
  b->coarse_ny = parent->coarse_ny;
  b->coarse_ny_sp = parent->coarse_ny_sp;
  b->level = parent->level;
  b->shared_prof = true;
  b->nprof = parent->nprof;
  b->prof_p = parent->prof_p;
  b->spl_p = parent->spl_p;
  b->bad_p = parent->bad_p;
  b->pdesc_p = parent->pdesc_p;
  for (int q = 0; q < b->count; ++q) {
    const int k = ks[q];
    stab_params pq = parent->Pin[k];
    const int fny = is_spatial(pq.itype) ? force_ny_sp : force_ny;
    if (fny > 0) pq.ny = fny;
    const InstDesc& pd0 = parent->hd[k];
    ProfDesc pd{};
    pd.off_prof = pd0.off_prof;
    pd.off_spl = pd0.off_spl;
    pd.nym = pd0.nym;
    InstDesc d;
    int rc = make_desc(c, pq, pd0.iprof, pd, d);
    if (rc) return rc;
    d.iprof_d1 = pd0.iprof_d1;
    d.iprof_d2 = pd0.iprof_d2;
    d.off_prof_d1 = pd0.off_prof_d1;
    d.off_spl_d1 = pd0.off_spl_d1;
    d.off_prof_d2 = pd0.off_prof_d2;
    d.off_spl_d2 = pd0.off_spl_d2;
    b->perm.push_back(q);
    b->P.push_back(pq);
    b->Pin.push_back(parent->Pin[k]);
    b->hd.push_back(d);
  }
  int rc = batch_finish(c, b.get());
  if (rc) return rc;
  *out = b.release();
  return 0;
}

// grid / index helpers over a contiguous internal range [k0, k0 + cnt)
struct Range {
  int k0, cnt;
};

static int run_prep(stab_batch* b) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const InstDesc* D = b->desc.as<InstDesc>();
  const double* const* T = b->dtab.as<const double*>();
  if (!b->shared_prof) {
    CK(c, timed(c, "k_spline", [&] {
      k_spline<<<(b->nprof + 63) / 64, 64, 0, s>>>(b->nprof, b->pdesc_p, b->prof_p, b->spl_p, b->bad_p);
      return cudaGetLastError();
    }));
  }
  const int nymax = b->nmax / 5;
  CK(c, cudaMemsetAsync(b->flags.p, 0, sizeof(int32_t) * b->count, s));
  CK(c, timed(c, "k_nodes", [&] {
    dim3 g((nymax + 127) / 128, b->count);
    k_nodes<<<g, 128, 0, s>>>(b->count, D, b->prof_p, b->spl_p, b->node.as<double>(), b->bad_p,
                              b->flags.as<int32_t>());
    return cudaGetLastError();
  }));
  CK(c, timed(c, "k_meanderiv", [&] {
    dim3 g((5 * nymax + 127) / 128, b->count);
    k_meanderiv<<<g, 128, 0, s>>>(b->count, D, T, b->node.as<double>());
    return cudaGetLastError();
  }));
  CK(c, timed(c, "k_blocks", [&] {
    dim3 g((nymax + 63) / 64, b->count);
    k_blocks<<<g, 64, 0, s>>>(b->count, D, T, b->node.as<double>(), b->blk.as<zc>(), b->flags.as<int>());
    return cudaGetLastError();
  }));
  return 0;
}

static int node_ops(stab_batch* b, Range r, int kind_t, int kind_s, const zc* sigma,
                    const int32_t* skip = nullptr) {
  stab_ctx* c = b->ctx;
  const int nymax = b->nmax / 5;
  return timed(c, "k_node_ops", [&] {
           dim3 g((nymax + 63) / 64, r.cnt);
           k_node_ops<<<g, 64, 0, c->stream>>>(r.cnt, b->desc.as<InstDesc>() + r.k0, b->blk.as<zc>(), kind_t, kind_s,
                                                sigma ? sigma + r.k0 : nullptr, b->ops.as<zc>(), b->ops32.as<cc>(),
                                                skip ? skip + r.k0 : nullptr);
           return cudaGetLastError();
         }) == cudaSuccess
             ? 0
             : set_err(c, STAB_ERR_CUDA, "k_node_ops launch failed");
}

template <typename T>
static int dense(stab_batch* b, Range r, T* out, const int64_t* off, int ldmul, double scale, const char* name,
                 const int32_t* skip = nullptr) {
  stab_ctx* c = b->ctx;
  cudaError_t e = timed(c, name, [&] {
    if constexpr (std::is_same<T, cc>::value)   // complex64 output: FP32 arithmetic on FP32 copies
      return launch_dense32(r.cnt, b->nmax, b->desc.as<InstDesc>() + r.k0, b->dtab32.as<const float*>(),
                            b->ops32.as<cc>(), out, off + r.k0, ldmul, (float)scale, c->stream,
                            skip ? skip + r.k0 : nullptr);
    else
      return launch_dense<T>(r.cnt, b->nmax, b->desc.as<InstDesc>() + r.k0, b->dtab.as<const double*>(),
                             b->ops.as<zc>(), out, off + r.k0, ldmul, scale, c->stream, skip ? skip + r.k0 : nullptr);
  });
  return e == cudaSuccess ? 0 : cuda_fail(c, e, name);
}

static int ensure_plain_pools(stab_batch* b) {
  stab_ctx* c = b->ctx;
  CK(c, b->Z64.ensure(sizeof(zc) * b->sum_n2, c->stream));
  CK(c, b->Abig.ensure(sizeof(zc) * b->sum_m2, c->stream));
  CK(c, b->Hbig.ensure(sizeof(zc) * b->sum_m2, c->stream));
  return 0;
}

// inverse iteration for the eigenvector of the pair (least_raw, .) with an
// LU of Q(theta) in precision T (complex128 for the plain path)
static int eigvec_inverse_iteration(stab_batch* b, Range r, const zc* theta_dev) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const InstDesc* D = b->desc.as<InstDesc>() + r.k0;
  int rc = node_ops(b, r, OP_T_Q, OP_S_Q, theta_dev);
  if (rc) return rc;
  rc = dense<zc>(b, r, b->Z64.as<zc>(), b->off_n2.as<int64_t>(), 1, 1.0, "k_dense_z");
  if (rc) return rc;
  CK(c, timed(c, "k_lu_z", [&] {
    return launch_lu<zc>(r.cnt, D, b->nsz.as<int32_t>() + r.k0, b->nmax, b->Z64.as<zc>(),
                         b->off_n2.as<int64_t>() + r.k0, b->piv.as<int32_t>(), b->off_nof.as<int64_t>() + r.k0,
                         b->info.as<int32_t>() + r.k0, s, nullptr, tuned_nb(c, true, b->nmax));
  }));
  CK(c, timed(c, "k_vec_init", [&] { return launch_vec_init(r.cnt, b->nmax, D, b->vec.as<zc>(), 0, s); }));
  for (int it = 0; it < 3; ++it) {
    CK(c, timed(c, "k_qmv", [&] {
      return launch_qmv(r.cnt, b->nmax, D, b->dtab.as<const double*>(), b->blk.as<zc>(), theta_dev + r.k0, 1,
                        b->vec.as<zc>(), 0, 1, nullptr, s);
    }));
    CK(c, timed(c, "k_getrs_z", [&] {
      return launch_getrs<zc>(r.cnt, b->nsz.as<int32_t>() + r.k0, b->nmax, b->Z64.as<zc>(),
                              b->off_n2.as<int64_t>() + r.k0, b->piv.as<int32_t>(), b->off_nof.as<int64_t>() + r.k0,
                              b->vec.as<zc>(), b->xoff[1].as<int64_t>() + r.k0, 1, 0, 1, nullptr, s);
    }));
    CK(c, timed(c, "k_normalize", [&] { return launch_normalize(r.cnt, D, b->vec.as<zc>(), 1, b->pcol.as<int32_t>() + r.k0, nullptr, s); }));
    CK(c, timed(c, "k_vec_copy", [&] { return launch_vec_copy(r.cnt, b->nmax, D, b->vec.as<zc>(), 1, 0, nullptr, s); }));
  }
  return 0;
}

static int write_vectors(stab_batch* b, Range r, const zc* theta_dev, const int32_t* skip = nullptr) {
  stab_ctx* c = b->ctx;
  const InstDesc* D = b->desc.as<InstDesc>() + r.k0;
  CK(c, timed(c, "k_temporal_vec", [&] {
    k_temporal_vec<<<r.cnt, 256, 0, c->stream>>>(r.cnt, D, b->vec.as<zc>(), 0, b->outvec.as<zc>(),
                                                  b->off_mof.as<int64_t>() + r.k0, skip ? skip + r.k0 : nullptr);
    return cudaGetLastError();
  }));
  CK(c, timed(c, "k_spatial_vec", [&] {
    k_spatial_vec<<<r.cnt, 256, 0, c->stream>>>(r.cnt, D, theta_dev + r.k0, b->vec.as<zc>(), 0,
                                                 b->outvec.as<zc>(), b->off_mof.as<int64_t>() + r.k0,
                                                 skip ? skip + r.k0 : nullptr);
    return cudaGetLastError();
  }));
  return 0;
}

// plain path on all instances: standard-form matrices, full spectrum, sort +
// select, optional eigenvector of the selected mode.  `seed` marks a spectrum
// that only seeds a polish (the seed arithmetic applies).
static int run_plain(stab_batch* b, bool want_vec, const char* eig_name = "k_eig_plain", bool seed = false) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  int rc = ensure_plain_pools(b);
  if (rc) return rc;
  const Range all{0, b->count};
  const Range tr{0, b->tcount};
  const Range sr{b->tcount, b->count - b->tcount};
  if (tr.cnt > 0) {
    rc = node_ops(b, tr, OP_T_C, OP_T_C, nullptr);
    if (rc) return rc;
    rc = dense<zc>(b, tr, b->Abig.as<zc>(), b->off_m2.as<int64_t>(), 1, 1.0, "k_dense_z");
    if (rc) return rc;
  }
  // seed spectra in double-word arithmetic also form their spatial companion
  // matrices in it (ZGETRF/ZGETRS of spatial.f90:978-1002 on the FP32 pipe;
  // the companion matrix only feeds the double-word eigensolve); spectra
  // that are answers keep FP64
  const bool seed_dw = seed && c->arith[STAB_STAGE_SEED_EIG] == STAB_ARITH_DOUBLE_WORD;
  if (sr.cnt > 0) {
    const InstDesc* D = b->desc.as<InstDesc>() + sr.k0;
    rc = node_ops(b, sr, OP_S_C0, OP_S_C0, nullptr);
    if (rc) return rc;
    if (seed_dw) {
      rc = dense<dz>(b, sr, b->Z64.as<dz>(), b->off_n2.as<int64_t>(), 1, 1.0, "k_dense_dz");
      if (rc) return rc;
      CK(c, timed(c, "k_lu_dz_seed", [&] {
        return launch_lu<dz>(sr.cnt, D, b->nsz.as<int32_t>() + sr.k0, b->nmax, b->Z64.as<dz>(),
                             b->off_n2.as<int64_t>() + sr.k0, b->piv.as<int32_t>(), b->off_nof.as<int64_t>() + sr.k0,
                             b->info.as<int32_t>() + sr.k0, s, nullptr, tuned_nb(c, true, b->nmax));
      }));
    } else {
      rc = dense<zc>(b, sr, b->Z64.as<zc>(), b->off_n2.as<int64_t>(), 1, 1.0, "k_dense_z");
      if (rc) return rc;
      CK(c, timed(c, "k_lu_z", [&] {
        return launch_lu<zc>(sr.cnt, D, b->nsz.as<int32_t>() + sr.k0, b->nmax, b->Z64.as<zc>(),
                             b->off_n2.as<int64_t>() + sr.k0, b->piv.as<int32_t>(), b->off_nof.as<int64_t>() + sr.k0,
                             b->info.as<int32_t>() + sr.k0, s, nullptr, tuned_nb(c, true, b->nmax));
      }));
    }
    rc = node_ops(b, sr, OP_S_C1, OP_S_C1, nullptr);
    if (rc) return rc;
    rc = dense<zc>(b, sr, b->Abig.as<zc>(), b->off_m2.as<int64_t>(), 2, -1.0, "k_dense_z");
    if (rc) return rc;
    rc = node_ops(b, sr, OP_S_C2, OP_S_C2, nullptr);
    if (rc) return rc;
    rc = dense<zc>(b, sr, b->Abig.as<zc>(), b->off_m2c2.as<int64_t>(), 2, -1.0, "k_dense_z");
    if (rc) return rc;
    CK(c, timed(c, seed_dw ? "k_getrs_dz_seed" : "k_getrs_z", [&] {
      return seed_dw ? launch_getrs<dz>(sr.cnt, b->nsz.as<int32_t>() + sr.k0, b->nmax, b->Z64.as<dz>(),
                                        b->off_n2.as<int64_t>() + sr.k0, b->piv.as<int32_t>(),
                                        b->off_nof.as<int64_t>() + sr.k0, b->Abig.as<zc>(),
                                        b->off_m2.as<int64_t>() + sr.k0, 0, 2, 2, nullptr, s)
                     : launch_getrs<zc>(sr.cnt, b->nsz.as<int32_t>() + sr.k0, b->nmax, b->Z64.as<zc>(),
                                        b->off_n2.as<int64_t>() + sr.k0, b->piv.as<int32_t>(),
                                        b->off_nof.as<int64_t>() + sr.k0, b->Abig.as<zc>(),
                                        b->off_m2.as<int64_t>() + sr.k0, 0, 2, 2, nullptr, s);
    }));
    CK(c, timed(c, "k_companion_fill", [&] {
      dim3 g(2 * (b->nmax), sr.cnt);
      k_companion_fill<<<g, 128, 0, s>>>(sr.cnt, D, b->Abig.as<zc>(), b->off_m2.as<int64_t>() + sr.k0);
      return cudaGetLastError();
    }));
  }
  CK(c, timed(c, eig_name, [&] {
    int grid = 0;   // sized by occupancy in the launcher, or capped per SM
    if (c->eig_resident > 0) {
      int dev = 0, sms = 1;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      grid = sms * c->eig_resident * (c->eig_threads == 64 ? 2 : 1);
    }
    return launch_eig_plain(b->count, b->mmax, b->msz.as<int32_t>(), b->Abig.as<zc>(), b->off_m2.as<int64_t>(),
                            b->Hbig.as<zc>(), b->off_m2.as<int64_t>(), b->eigraw.as<zc>(), b->off_mof.as<int64_t>(),
                            b->status.as<int32_t>(), b->counter.as<int32_t>(), b->order.as<int32_t>(),
                            b->flops.as<double>(), grid, s,
                            c->arith[seed ? STAB_STAGE_SEED_EIG : STAB_STAGE_PLAIN_EIG] == STAB_ARITH_DOUBLE_WORD,
                            seed && c->seed_qr_shared, c->eig_mid ? 256 : c->eig_threads);
  }));
  CK(c, timed(c, "k_post_spectrum", [&] {
    size_t sm = sizeof(zc) * b->mmax;
    cudaFuncSetAttribute(k_post_spectrum, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_post_spectrum<<<b->count, 256, sm, s>>>(b->count, b->desc.as<InstDesc>(), b->eigraw.as<zc>(),
                                              b->off_mof.as<int64_t>(), b->eigsorted.as<zc>(),
                                              b->least_idx.as<int32_t>(), b->least_raw.as<zc>(),
                                              b->least_val.as<zc>(), b->cand.as<zc>(), kShiftCandidates);
    return cudaGetLastError();
  }));
  CK(c, cudaMemsetAsync(b->err.p, 0, sizeof(double) * b->count, s));
  CK(c, cudaMemsetAsync(b->iters.p, 0, sizeof(int32_t) * b->count, s));
  if (want_vec) {
    CK(c, cudaMemcpyAsync(b->theta.p, b->least_raw.p, sizeof(zc) * b->count, cudaMemcpyDeviceToDevice, s));
    rc = eigvec_inverse_iteration(b, all, b->theta.as<zc>());
    if (rc) return rc;
    rc = write_vectors(b, all, b->theta.as<zc>());
    if (rc) return rc;
  }
  return 0;
}

// mixed-precision polish from sigma (device, internal order)
static const int kNewtonSteps = 20;
static const double kNewtonTol = 1e-13;      // |d theta| / |theta| of the last Newton-chord step
static const double kNewtonTolVec = 1e-11;   // max |d x| / max |x|

// The polish with factors in precision T: complex64 (the fast path) or
// complex128 (separates eigenvalue clusters closer than complex64 resolves).
template <typename T>
static T* polish_pool(stab_batch* b);
template <>
cc* polish_pool<cc>(stab_batch* b) { return b->M32.as<cc>(); }
template <>
zc* polish_pool<zc>(stab_batch* b) { return b->Z64.as<zc>(); }

// stage 0: the whole polish; 1: only the factorisation at the shift and the
// two inverse-iteration steps (x in vector slot 0, normalised at pcol);
// 2: start from the coarse level's eigenvector (Chebyshev coefficients in
// b->seedc, b->seedc_n of them per field) instead of those steps, so the
// factorisation at the shift is skipped.
template <typename T>
static int run_polish_t(stab_batch* b, bool want_vec, const int32_t* skip, int stage) {
  const bool c64 = std::is_same<T, cc>::value;
  const char* n_dense = c64 ? "k_dense_c" : "k_dense_z";
  const char* n_lu = c64 ? "k_lu_c" : "k_lu_z";
  const char* n_getrs = c64 ? "k_getrs_c" : "k_getrs_z";
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const Range all{0, b->count};
  const InstDesc* D = b->desc.as<InstDesc>();
  const double* const* DT = b->dtab.as<const double*>();
  zc* V = b->vec.as<zc>();
  int32_t* done = b->done.as<int32_t>();
  CK(c, timed(c, "k_start_shift", [&] {
    return launch_start_shift(b->count, b->sigma.as<zc>(), b->theta.as<zc>(), skip, s);
  }));
  int rc = node_ops(b, all, OP_T_Q, OP_S_Q, b->theta.as<zc>(), skip);
  if (rc) return rc;
  if (!c64) CK(c, b->Z64.ensure(sizeof(zc) * b->sum_n2, s));
  T* MP = polish_pool<T>(b);
  if (stage != 2) {
    rc = dense<T>(b, all, MP, b->off_n2.as<int64_t>(), 1, 1.0, n_dense, skip);
    if (rc) return rc;
  }
  const float* rs = c64 ? b->rsc.as<float>() : nullptr;
  const float* cs = c64 ? b->csc.as<float>() : nullptr;
  auto lu32 = [&]() {
    if (c64) {
      cudaError_t e = timed(c, "k_equilibrate", [&] {
        return launch_equilibrate(b->count, b->nsz.as<int32_t>(), b->M32.as<cc>(), b->off_n2.as<int64_t>(),
                                  b->rsc.as<float>(), b->csc.as<float>(), b->off_nof.as<int64_t>(), s, skip);
      });
      if (e != cudaSuccess) return e;
    }
    if (c64 && c->arith[STAB_STAGE_POLISH_LU] == STAB_ARITH_TF32_SPLIT && lu_tc_fits(b->nmax)) {
      const CUtensorMap* tm = nullptr;
      // TMA tiles hold one CTA per SM; a batch that two CTAs per SM take in
      // one wave (the N = 48 level) runs the form without them
      if (c->lu_tma && lu_tc_fits(b->nmax, true) && b->count > 2 * c->sms) {
        if (b->tmaps_state == 0) {
          std::vector<CUtensorMap> maps;
          if (lu_tc_tensor_maps(b->count, b->hn.data(), b->h_n2.data(), b->M32.as<cc>(), maps)) {
            cudaError_t e = upload(b->tmaps, maps, s);
            if (e != cudaSuccess) return e;
            b->tmaps_state = 1;
          } else {
            b->tmaps_state = -1;
          }
        }
        if (b->tmaps_state == 1) tm = b->tmaps.as<CUtensorMap>();
      }
      return timed(c, tm ? "k_lu_tc_tma" : "k_lu_tc", [&] {
        return launch_lu_tc(b->count, b->nsz.as<int32_t>(), b->nmax, b->M32.as<cc>(), b->off_n2.as<int64_t>(),
                            b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), b->info.as<int32_t>(), s, skip,
                            b->order.as<int32_t>(), tm);
      });
    }
    return timed(c, n_lu, [&] {
      return launch_lu<T>(b->count, D, b->nsz.as<int32_t>(), b->nmax, MP, b->off_n2.as<int64_t>(),
                          b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), b->info.as<int32_t>(), s, skip,
                          tuned_nb(c, !c64, b->nmax), b->order.as<int32_t>());
    });
  };
  auto solve32 = [&](int slot, const int32_t* sk) {
    return timed(c, n_getrs, [&] {
      return launch_getrs<T>(b->count, b->nsz.as<int32_t>(), b->nmax, MP, b->off_n2.as<int64_t>(),
                             b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), V, b->xoff[slot].as<int64_t>(), 1, 0, 1,
                             sk, s, rs, cs);
    });
  };
  auto qmv = [&](int deriv, int xs, int ys, const int32_t* sk) {
    return timed(c, "k_qmv", [&] {
      return launch_qmv(b->count, b->nmax, D, DT, b->blk.as<zc>(), b->theta.as<zc>(), deriv, V, xs, ys, sk, s);
    });
  };
  if (stage == 2) {
    CK(c, timed(c, "k_cheb_start", [&] {
      return launch_cheb_start(b->count, b->nmax, D, b->seedc.as<zc>(), b->seedc_n, V, 0, skip, s);
    }));
    CK(c, timed(c, "k_normalize", [&] { return launch_normalize(b->count, D, V, 0, b->pcol.as<int32_t>(), skip, s); }));
  } else {
    CK(c, lu32());
    if (b->use_start) {
      CK(c, timed(c, "k_cheb_start", [&] {
        return launch_cheb_start(b->count, b->nmax, D, b->startc.as<zc>(), b->ncheb, V, 0, skip, s);
      }));
    } else {
      CK(c, timed(c, "k_vec_init", [&] { return launch_vec_init(b->count, b->nmax, D, V, 0, s, skip); }));
    }
    for (int it = 0; it < 2; ++it) {   // inverse iteration at the shift
      CK(c, qmv(1, 0, 1, skip));
      CK(c, solve32(1, skip));
      CK(c, timed(c, "k_normalize",
                  [&] { return launch_normalize(b->count, D, V, 1, b->pcol.as<int32_t>(), skip, s); }));
      CK(c, timed(c, "k_vec_copy", [&] { return launch_vec_copy(b->count, b->nmax, D, V, 1, 0, skip, s); }));
    }
    if (stage == 1) return 0;
  }
  // bordered Jacobian at (sigma, x): Q(sigma) with column p <- Q'(sigma) x
  CK(c, qmv(1, 0, 2, skip));
  rc = dense<T>(b, all, MP, b->off_n2.as<int64_t>(), 1, 1.0, n_dense, skip);
  if (rc) return rc;
  CK(c, timed(c, "k_set_column", [&] {
    return launch_set_column<T>(b->count, b->nmax, D, MP, b->off_n2.as<int64_t>(), b->pcol.as<int32_t>(), V, 2, s,
                                skip);
  }));
  CK(c, lu32());
  CK(c, timed(c, "k_reset_polish", [&] {
    return launch_reset_polish(b->count, done, b->iters.as<int32_t>(), skip, s,
                               c64 ? b->lus32.as<int32_t>() : b->lus64.as<int32_t>(), 2);
  }));
  // Newton-chord steps; converged instances (done != 0) drop out
  for (int it = 0; it < kNewtonSteps; ++it) {
    CK(c, qmv(0, 0, 3, done));
    CK(c, solve32(3, done));
    CK(c, timed(c, "k_newton_update", [&] {
      return launch_newton_update(b->count, D, V, 0, 3, b->pcol.as<int32_t>(), b->theta.as<zc>(), done,
                                  b->err.as<double>(), b->iters.as<int32_t>(), kNewtonTol, kNewtonTolVec, s, skip);
    }));
  }
  CK(c, timed(c, "k_normalize", [&] { return launch_normalize(b->count, D, V, 0, nullptr, skip, s); }));
  // least_raw: omega (temporal) or lambda = 1/alpha (spatial)
  CK(c, cudaMemcpyAsync(b->least_raw.p, b->theta.p, sizeof(zc) * b->count, cudaMemcpyDeviceToDevice, s));
  if (want_vec) {
    rc = write_vectors(b, all, b->theta.as<zc>(), skip);
    if (rc) return rc;
  }
  return 0;
}

// Complex128 retry: fixed-shift inverse iteration on one complex128 LU of
// Q(sigma).  The eigenvalue estimate sigma - x_p / y_p converges with the
// ratio |sigma - lambda_1| / |sigma - lambda_2| per step, which separates
// mode clusters that complex64 factors cannot resolve.
static const int kInverseSteps = 8;
// N of the second candidate level of the fallback (the default of
// STAB_OPT_MEDIUM_NY); seed sizes stay below it
static const int kMediumNy = 48;
static const double kInverseTol = 1e-13;

static int run_polish64_ii(stab_batch* b, bool want_vec, const int32_t* skip) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const Range all{0, b->count};
  const InstDesc* D = b->desc.as<InstDesc>();
  zc* V = b->vec.as<zc>();
  int32_t* done = b->done.as<int32_t>();
  CK(c, b->Z64.ensure(sizeof(zc) * b->sum_n2, s));
  CK(c, timed(c, "k_start_shift", [&] {
    return launch_start_shift(b->count, b->sigma.as<zc>(), b->theta.as<zc>(), skip, s);
  }));
  int rc = node_ops(b, all, OP_T_Q, OP_S_Q, b->sigma.as<zc>(), skip);
  if (rc) return rc;
  // the factorisation in double-word form (same bytes per entry) or FP64;
  // the retried instances are few and their factorisations long: a cluster
  // of four SMs shares each large one
  const bool dwlu = c->arith[STAB_STAGE_RETRY_LU] == STAB_ARITH_DOUBLE_WORD;
  const int lu_cluster = b->nmax >= 240 ? 4 : 1;
  if (dwlu) {
    rc = dense<dz>(b, all, b->Z64.as<dz>(), b->off_n2.as<int64_t>(), 1, 1.0, "k_dense_dz", skip);
    if (rc) return rc;
    CK(c, timed(c, "k_lu_dz", [&] {
      return launch_lu<dz>(b->count, D, b->nsz.as<int32_t>(), b->nmax, b->Z64.as<dz>(), b->off_n2.as<int64_t>(),
                           b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), b->info.as<int32_t>(), s, skip,
                           tuned_nb(c, true, b->nmax), b->order.as<int32_t>(), lu_cluster);
    }));
  } else {
    rc = dense<zc>(b, all, b->Z64.as<zc>(), b->off_n2.as<int64_t>(), 1, 1.0, "k_dense_z", skip);
    if (rc) return rc;
    CK(c, timed(c, "k_lu_z", [&] {
      return launch_lu<zc>(b->count, D, b->nsz.as<int32_t>(), b->nmax, b->Z64.as<zc>(), b->off_n2.as<int64_t>(),
                           b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), b->info.as<int32_t>(), s, skip,
                           tuned_nb(c, true, b->nmax), b->order.as<int32_t>(), lu_cluster);
    }));
  }
  CK(c, timed(c, "k_vec_init", [&] { return launch_vec_init(b->count, b->nmax, D, V, 0, s, skip); }));
  CK(c, timed(c, "k_normalize", [&] { return launch_normalize(b->count, D, V, 0, b->pcol.as<int32_t>(), skip, s); }));
  CK(c, timed(c, "k_reset_polish", [&] {
    return launch_reset_polish(b->count, done, b->iters.as<int32_t>(), skip, s, b->lus64.as<int32_t>(), 1);
  }));
  for (int it = 0; it < kInverseSteps; ++it) {
    CK(c, timed(c, "k_qmv", [&] {
      return launch_qmv(b->count, b->nmax, D, b->dtab.as<const double*>(), b->blk.as<zc>(), b->sigma.as<zc>(), 1, V,
                        0, 1, done, s);
    }));
    CK(c, timed(c, dwlu ? "k_getrs_dz" : "k_getrs_z", [&] {
      return dwlu ? launch_getrs<dz>(b->count, b->nsz.as<int32_t>(), b->nmax, b->Z64.as<dz>(),
                                     b->off_n2.as<int64_t>(), b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), V,
                                     b->xoff[1].as<int64_t>(), 1, 0, 1, done, s)
                  : launch_getrs<zc>(b->count, b->nsz.as<int32_t>(), b->nmax, b->Z64.as<zc>(),
                                     b->off_n2.as<int64_t>(), b->piv.as<int32_t>(), b->off_nof.as<int64_t>(), V,
                                     b->xoff[1].as<int64_t>(), 1, 0, 1, done, s);
    }));
    CK(c, timed(c, "k_ii_update", [&] {
      return launch_ii_update(b->count, D, V, 0, 1, b->pcol.as<int32_t>(), b->sigma.as<zc>(), b->theta.as<zc>(), done,
                              b->err.as<double>(), b->iters.as<int32_t>(), kInverseTol, skip, s);
    }));
  }
  CK(c, timed(c, "k_normalize", [&] { return launch_normalize(b->count, D, V, 0, nullptr, skip, s); }));
  CK(c, cudaMemcpyAsync(b->least_raw.p, b->theta.p, sizeof(zc) * b->count, cudaMemcpyDeviceToDevice, s));
  if (want_vec) {
    rc = write_vectors(b, all, b->theta.as<zc>(), skip);
    if (rc) return rc;
  }
  return 0;
}

static int run_polish(stab_batch* b, bool want_vec, const int32_t* skip = nullptr) {
  return run_polish_t<cc>(b, want_vec, skip, 0);
}

// host-side: status from `done` and NaN checks; theta -> eigenvalue
static void finalize_polish_host(std::vector<zc>& val, std::vector<int32_t>& st, const std::vector<int32_t>& dn,
                                 const std::vector<stab_params>& P) {
  for (size_t k = 0; k < val.size(); ++k) {
    if (P[k].itype == 2 || P[k].itype == 4) {
      zc l = val[k];
      double d = l.x * l.x + l.y * l.y;
      val[k] = d > 0 ? zmk(l.x / d, -l.y / d) : zmk(0.0, 0.0);
    }
    st[k] = (dn[k] == 1) ? STAB_ST_OK
            : (dn[k] == 3 ? STAB_ST_NAN : (dn[k] == kDoneUnverified ? STAB_ST_UNVERIFIED : STAB_ST_NOCONV));
  }
}

// caller start-vector coefficients -> device, internal order
static int upload_start(stab_batch* b) {
  stab_ctx* c = b->ctx;
  const size_t per = (size_t)5 * b->ncheb;
  std::vector<zc> co(per * b->count);
  for (int k = 0; k < b->count; ++k) {
    const double* src = b->start_coef.data() + 2 * per * b->perm[k];
    for (size_t q = 0; q < per; ++q) co[per * k + q] = zmk(src[2 * q], src[2 * q + 1]);
  }
  CK(c, upload(b->startc, co, c->stream));
  return 0;
}

static int batch_run(stab_batch* b, int32_t mode) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  // other modes may grow pools the captured coarse pass points into
  if (b->coarse_graph) {
    cudaGraphExecDestroy(b->coarse_graph);
    b->coarse_graph = nullptr;
  }
  b->fell_back.clear();
  for (double& w : b->fb_work) w = 0.0;
  b->last_mode = mode;
  int rc = run_prep(b);
  if (mode != STAB_MODE_PLAIN) {
    CK(c, cudaMemsetAsync(b->lus32.p, 0, sizeof(int32_t) * b->count, s));
    CK(c, cudaMemsetAsync(b->lus64.p, 0, sizeof(int32_t) * b->count, s));
  }
  if (rc) return rc;
  if (mode == STAB_MODE_PLAIN) {
    rc = run_plain(b, true);
    if (rc) return rc;
    b->ran = true;
    return 0;
  }
  if (mode == STAB_MODE_SEEDED || mode == STAB_MODE_TRACK) {
    if (!b->have_seeds) return set_err(c, STAB_ERR_STATE, "seeded modes need stab_batch_set_seeds first");
    std::vector<zc> sg(b->count);
    for (int k = 0; k < b->count; ++k) {
      const int u = b->perm[k];
      zc a = zmk(b->seeds[2 * u], b->seeds[2 * u + 1]);
      if (b->P[k].itype == 2 || b->P[k].itype == 4) {
        double d = a.x * a.x + a.y * a.y;
        a = d > 0 ? zmk(a.x / d, -a.y / d) : zmk(0.0, 0.0);
      }
      sg[k] = a;
    }
    CK(c, cudaMemcpyAsync(b->sigma.p, sg.data(), sizeof(zc) * b->count, cudaMemcpyHostToDevice, s));
    b->use_start = false;
    if (mode == STAB_MODE_TRACK && b->ncheb > 0) {
      int rc2 = upload_start(b);
      if (rc2) return rc2;
      b->use_start = true;
    }
    CK(c, cudaStreamSynchronize(s));
  } else {
    return set_err(c, STAB_ERR_ARG, "unknown mode");
  }
  rc = run_polish(b, true);
  b->use_start = false;
  if (rc) return rc;
  b->ran = true;
  return 0;
}

extern "C" {

int stab_abi_version(void) { return STAB_GB300_ABI_VERSION; }

int stab_create(stab_ctx** out, int device) {
  if (!out) return STAB_ERR_ARG;
  std::unique_ptr<stab_ctx> c(new stab_ctx());
  c->device = device;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    *out = nullptr;
    return STAB_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return STAB_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return STAB_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) return STAB_ERR_CUDA;
  {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;   // keep freed blocks for reuse by later batches of this process
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  c->stream = c->own;
  cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
  *out = c.release();
  return STAB_OK;
}

int stab_destroy(stab_ctx* c) {
  if (!c) return STAB_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  // batches the caller has not destroyed lose their device memory and their
  // context; a later stab_batch_destroy only frees the host side
  for (stab_batch* b : c->live) {
    b->release();
    b->ctx = nullptr;
  }
  c->live.clear();
  for (stab_mlp* m : c->nets) release_net(m);
  c->nets.clear();
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->dtabs) {
    cudaFree(kv.second.first);
    cudaFree(kv.second.second);
  }
  for (auto& kv : c->dtabs32) {
    cudaFree(kv.second.first);
    cudaFree(kv.second.second);
  }
  for (auto& p : c->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : c->evpool) cudaEventDestroy(e);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return STAB_OK;
}

const char* stab_last_error(const stab_ctx* c) { return c ? c->err.c_str() : "null context"; }

int stab_set_stream(stab_ctx* c, void* stream) {
  if (!c) return STAB_ERR_ARG;
  c->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : c->own;
  return STAB_OK;
}

int stab_sync(stab_ctx* c) {
  if (!c) return STAB_ERR_ARG;
  CK(c, cudaStreamSynchronize(c->stream));
  return STAB_OK;
}

int stab_set_profiling(stab_ctx* c, int on) {
  if (!c) return STAB_ERR_ARG;
  drain_stats(c);
  c->profiling = on ? 1 : 0;
  return STAB_OK;
}

int stab_kernel_stats(stab_ctx* c, int32_t k, const char** name, int64_t* launches, double* total_ms,
                      int32_t* count) {
  if (!c) return STAB_ERR_ARG;
  drain_stats(c);
  if (count) *count = (int32_t)c->stats.size();
  if (k < 0 || k >= (int32_t)c->stats.size()) return (name || launches || total_ms) ? STAB_ERR_ARG : STAB_OK;
  if (name) *name = c->stats[k].name.c_str();
  if (launches) *launches = c->stats[k].launches;
  if (total_ms) *total_ms = c->stats[k].ms;
  return STAB_OK;
}

int stab_reset_kernel_stats(stab_ctx* c) {
  if (!c) return STAB_ERR_ARG;
  drain_stats(c);
  c->stats.clear();
  return STAB_OK;
}

int stab_batch_create(stab_ctx* c, int32_t count, const stab_params* p, const int32_t* nym,
                      const double* const* profiles, stab_batch** out) {
  if (!c) return STAB_ERR_ARG;
  cudaSetDevice(c->device);
  int rc = batch_build(c, count, p, nym, profiles, out);
  if (rc) return rc;
  c->live.push_back(*out);
  return STAB_OK;
}

int stab_batch_set_seeds(stab_batch* b, const double* seeds) {
  if (!b || !seeds) return STAB_ERR_ARG;
  if (!b->ctx) return STAB_ERR_STATE;
  b->seeds.assign(seeds, seeds + 2 * (size_t)b->count);
  b->have_seeds = true;
  return STAB_OK;
}

static int coarse_seeds(stab_batch* b) {
  stab_ctx* c = b->ctx;
  if (!b->coarse) {
    std::vector<int> all(b->count);
    for (int k = 0; k < b->count; ++k) all[k] = k;
    stab_batch* cb = nullptr;
    int rc = batch_build_child(b, all, b->coarse_ny, &cb, b->coarse_ny_sp);
    if (rc) return rc;
    b->coarse = cb;
  }
  stab_batch* cb = b->coarse;
  int rc = run_prep(cb);
  if (rc) return rc;
  rc = run_plain(cb, false, "k_eig_plain_coarse", true);
  if (rc) return rc;
  // same internal order in both batches (same stable itype sort)
  CK(c, cudaMemcpyAsync(b->cand.p, cb->cand.p, sizeof(zc) * b->count * kShiftCandidates, cudaMemcpyDeviceToDevice,
                        c->stream));
  return 0;
}

// Coarse-shift rounds.  Each polished pair is an eigenpair of the fine
// problem, so the least-stable of the converged pairs over the top coarse
// candidates is the answer whenever one candidate sits near the fine
// least-stable mode.  N = 32 carries unresolved modes above it at M > 1.4
// and spurious acoustic ones at M < 0.03, and resolves the right one only
// to ~1e-2.  Each candidate gets a complex64 round, and a complex128 retry
// where that failed or contracted slowly (a mode cluster closer than
// complex64 factors resolve).  Candidates go in selection order, and the
// first one whose polish lands within kQuickAcceptTol of its shift (a mode
// the N = 32 spectrum resolved) makes the instance final; otherwise the next
// candidates are polished too.  Instances with no converged pair go to the
// FP64 fallback.
// With `single` every instance is one candidate copy of a parent instance
// (polish_candidates_parallel): only its top candidate's two rounds run, and
// copies without a candidate are skipped.
static int polish_candidate_rounds(stab_batch* b, bool extra, bool single = false) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const int n = b->count;
  CK(c, b->have.ensure(sizeof(int32_t) * n, s));
  CK(c, b->skip64.ensure(sizeof(int32_t) * n, s));
  CK(c, b->best_key.ensure(sizeof(double) * n, s));
  CK(c, b->best_theta.ensure(sizeof(zc) * n, s));
  CK(c, b->best_err.ensure(sizeof(double) * n, s));
  CK(c, b->best_iters.ensure(sizeof(int32_t) * n, s));
  CK(c, b->best_out.ensure(sizeof(zc) * b->sum_m, s));
  int32_t* fin = b->accepted.as<int32_t>();
  CK(c, cudaMemsetAsync(fin, 0, sizeof(int32_t) * n, s));
  CK(c, cudaMemsetAsync(b->lus32.p, 0, sizeof(int32_t) * n, s));
  CK(c, cudaMemsetAsync(b->lus64.p, 0, sizeof(int32_t) * n, s));
  CK(c, cudaMemsetAsync(b->have.p, 0, sizeof(int32_t) * n, s));
  if (single) {
    CK(c, timed(c, "k_mark_missing", [&] {
      k_mark_missing<<<(n + 255) / 256, 256, 0, s>>>(n, b->cand.as<zc>(), kShiftCandidates, fin);
      return cudaGetLastError();
    }));
  }
  // per candidate: a complex64 round, then a complex128 retry for the
  // instances where it failed or contracted slowly
  CK(c, b->best_src.ensure(sizeof(int32_t) * n, s));
  CK(c, cudaMemsetAsync(b->best_src.p, 0xff, sizeof(int32_t) * n, s));
  // At the first candidate level without the surrogate's round, only the
  // top candidate (its complex64 round and complex128 retry) can make an
  // instance final: a pair from candidates 1-3 is not trusted there
  // (k_take_best) and the instance goes to the N = 48 level whatever it
  // holds, so those rounds are skipped.  The N = 48 level runs them all: its
  // best pair is kept as STAB_ST_UNVERIFIED.
  const bool first_level = (b->level == 1) && !extra && !single;
  const int rounds = first_level ? (c->first_retry ? 2 : 1) : single ? 2 : 2 * kShiftCandidates + (extra ? 2 : 0);
  // STAB_OPT_SEED_VECTORS: the top candidate's round starts from the coarse
  // level's eigenvector (inverse iteration on the N = 32 operator at the
  // candidate, interpolated through its Chebyshev coefficients) instead of
  // a factorisation of the full operator at the shift and two inverse-
  // iteration steps (Chebyshev grids only)
  const bool seedvec = first_level && c->seed_vectors && b->coarse && !b->has_fd;
  if (seedvec) {
    stab_batch* cb = b->coarse;
    CK(c, timed(c, "k_take_candidate", [&] {
      k_take_candidate<<<(cb->count + 255) / 256, 256, 0, s>>>(cb->count, cb->cand.as<zc>(), kShiftCandidates, 0,
                                                             cb->sigma.as<zc>());
      return cudaGetLastError();
    }));
    int rc = run_polish_t<cc>(cb, false, nullptr, 1);
    if (rc) return rc;
    b->seedc_n = b->coarse_ny;
    CK(c, b->seedc.ensure(sizeof(zc) * (size_t)n * 5 * b->seedc_n, s));
    CK(c, timed(c, "k_cheb_coeffs", [&] {
      return launch_cheb_coeffs(n, cb->desc.as<InstDesc>(), cb->vec.as<zc>(), b->seedc.as<zc>(), b->seedc_n, s);
    }));
  }
  for (int r = 0; r < rounds; ++r) {
    const int j = r / 2;
    const bool fp64 = (r & 1) != 0;
    const bool surrogate = (j == kShiftCandidates);   // the caller's predicted seed
    if (!fp64 && !surrogate) {
      CK(c, timed(c, "k_take_candidate", [&] {
        k_take_candidate<<<(n + 255) / 256, 256, 0, s>>>(n, b->cand.as<zc>(), kShiftCandidates, j, b->sigma.as<zc>());
        return cudaGetLastError();
      }));
    } else if (!fp64) {
      CK(c, cudaMemcpyAsync(b->sigma.p, b->seed_raw.p, sizeof(zc) * n, cudaMemcpyDeviceToDevice, s));
    }
    b->use_start = surrogate && !fp64 && b->ncheb > 0;
    // per-round wall time in profiling mode ("stage:" entries wrap launches)
    cudaEvent_t ra = nullptr, rb = nullptr;
    if (c->profiling) {
      ra = get_ev(c);
      rb = get_ev(c);
      cudaEventRecord(ra, s);
    }
    int rc = fp64 ? run_polish64_ii(b, true, b->skip64.as<int32_t>())
                  : run_polish_t<cc>(b, true, fin, (r == 0 && seedvec) ? 2 : 0);
    b->use_start = false;
    if (c->profiling) {
      cudaEventRecord(rb, s);
      char nm[32];
      std::snprintf(nm, sizeof(nm), "stage:round%d_%s", j, fp64 ? "c128" : "c64");
      c->pending.push_back(PendingEv{stat_index(c, nm), ra, rb});
    }
    if (rc) return rc;
    CK(c, timed(c, "k_fold_best", [&] {
      k_fold_best<<<n, 128, 0, s>>>(n, b->desc.as<InstDesc>(), b->sigma.as<zc>(), b->theta.as<zc>(),
                                    b->done.as<int32_t>(), b->err.as<double>(), b->iters.as<int32_t>(),
                                    b->outvec.as<zc>(), b->off_mof.as<int64_t>(), fin, b->have.as<int32_t>(),
                                    b->best_key.as<double>(), b->best_theta.as<zc>(), b->best_err.as<double>(),
                                    b->best_iters.as<int32_t>(), b->best_out.as<zc>(), surrogate ? 0 : 1,
                                    kQuickAcceptTol, fp64 ? nullptr : b->skip64.as<int32_t>(), kSlowNewton, j,
                                    b->best_src.as<int32_t>());
      return cudaGetLastError();
    }));
  }
  CK(c, timed(c, "k_take_best", [&] {
    k_take_best<<<n, 128, 0, s>>>(n, b->desc.as<InstDesc>(), b->have.as<int32_t>(), b->best_theta.as<zc>(),
                                  b->best_err.as<double>(), b->best_iters.as<int32_t>(), b->best_out.as<zc>(),
                                  b->off_mof.as<int64_t>(), b->theta.as<zc>(), b->done.as<int32_t>(),
                                  b->err.as<double>(), b->iters.as<int32_t>(), b->outvec.as<zc>(), fin,
                                  b->best_src.as<int32_t>(), kShiftCandidates, kDoneUnverified,
                                  b->level >= 2 ? 1 : 0);
    return cudaGetLastError();
  }));
  CK(c, cudaMemcpyAsync(b->least_raw.p, b->theta.p, sizeof(zc) * n, cudaMemcpyDeviceToDevice, s));
  return 0;
}

// The candidate rounds of a small batch (the N = 48 level: a few hundred
// instances, which leave most of the GPU idle in each round) run side by
// side: a sub-batch holds one copy of each instance per shift candidate,
// every copy takes its candidate's two rounds (complex64, then the
// double-word retry where that failed or contracted slowly), and
// k_fold_copies folds the copies in candidate order with the rules of the
// sequential rounds (the same kept pair and status; candidates after a
// quick-accepted one are computed but not folded).
// second-level trust (STAB_OPT_LEVEL_CONSISTENCY): the N = 48 top
// candidate's error against the polished pair is at most this fraction of
// the N = 32 top candidate's
static const double kLevelConvergence = 0.25;
static int polish_candidates_parallel(stab_batch* b) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const int n = b->count, K = kShiftCandidates;
  if (!b->copies) {
    std::vector<int> ks((size_t)n * K);
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < K; ++j) ks[(size_t)k * K + j] = k;
    stab_batch* cb = nullptr;
    int rc = batch_build_child(b, ks, 0, &cb);
    if (rc) return rc;
    b->copies = cb;
  }
  stab_batch* x = b->copies;
  int rc = run_prep(x);
  if (rc) return rc;
  // copy c = k * K + j of instance k: its top candidate is b's candidate j
  CK(c, timed(c, "k_spread_candidates", [&] {
    k_spread_candidates<<<(n * K + 255) / 256, 256, 0, s>>>(n * K, b->cand.as<zc>(), K, x->cand.as<zc>());
    return cudaGetLastError();
  }));
  rc = polish_candidate_rounds(x, false, true);
  if (rc) return rc;
  x->ran = true;
  x->last_mode = STAB_MODE_COARSE;
  CK(c, timed(c, "k_fold_copies", [&] {
    k_fold_copies<<<n, 128, 0, s>>>(n, K, b->desc.as<InstDesc>(), x->done.as<int32_t>(), x->best_key.as<double>(),
                                    x->theta.as<zc>(), x->err.as<double>(), x->iters.as<int32_t>(),
                                    x->outvec.as<zc>(), x->off_mof.as<int64_t>(), b->theta.as<zc>(),
                                    b->done.as<int32_t>(), b->err.as<double>(), b->iters.as<int32_t>(),
                                    b->outvec.as<zc>(), b->off_mof.as<int64_t>(), kDoneUnverified,
                                    b->has_lev1 ? b->lev1_lam.as<zc>() : nullptr, b->lev1_th.as<zc>(),
                                    b->lev1_ok.as<int32_t>(), b->cand.as<zc>(), kLevelConvergence, b->lev1_n,
                                    b->coarse_ny, b->coarse_ny_sp);
    return cudaGetLastError();
  }));
  CK(c, cudaMemcpyAsync(b->least_raw.p, b->theta.p, sizeof(zc) * n, cudaMemcpyDeviceToDevice, s));
  return 0;
}

// Seeded modes: the instances whose complex64 Newton-chord did not converge
// (operators whose scales complex64 factors do not resolve, such as the
// 1/(gamma M^2) pressure terms at M = 0.001) take the complex128 inverse
// iteration at their seed before the full-spectrum fallback.
static int retry_seeded(stab_batch* b) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const int n = b->count;
  std::vector<int32_t> dn(n);
  CK(c, cudaMemcpyAsync(dn.data(), b->done.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaStreamSynchronize(s));
  if (std::all_of(dn.begin(), dn.end(), [](int32_t d) { return d == 1; })) return 0;
  CK(c, b->skip64.ensure(sizeof(int32_t) * n, s));
  int32_t* mask = b->skip64.as<int32_t>();
  CK(c, timed(c, "k_converged_mask", [&] {
    k_converged_mask<<<(n + 255) / 256, 256, 0, s>>>(n, b->done.as<int32_t>(), mask, 0);
    return cudaGetLastError();
  }));
  int rc = run_polish64_ii(b, true, mask);
  if (rc) return rc;
  CK(c, timed(c, "k_converged_mask", [&] {
    k_converged_mask<<<(n + 255) / 256, 256, 0, s>>>(n, b->done.as<int32_t>(), mask, 1);
    return cudaGetLastError();
  }));
  return 0;
}

// Re-solve, with the plain FP64 path, every instance whose polish did not
// converge (or had no accepted shift); results are kept on the host for
// stab_batch_results.
// FP64 fallback on the instances whose polish did not converge.  With
// `track` (STAB_MODE_TRACK) the kept eigenvalue is the one nearest the
// instance's seed, as the reference's post-processors pick a mode from a
// guess (getevec.f90:161-172, getab.f90:185-192), instead of the least-stable.
static int run_fallback(stab_batch* b, bool track = false) {
  stab_ctx* c = b->ctx;
  const int n = b->count;
  std::vector<int32_t> dn(n);
  CK(c, cudaMemcpyAsync(dn.data(), b->done.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  b->fell_back.clear();
  for (double& w : b->fb_work) w = 0.0;
  b->fb_val.clear();
  b->fb_status.clear();
  b->fb_vec.clear();
  b->fb_err.clear();
  b->fb_iters.clear();
  b->counts[0] = b->counts[1] = 0;
  for (int k = 0; k < n; ++k) {
    if (dn[k] == 1) b->counts[0] += 1;
    else if (dn[k] == kDoneUnverified) b->counts[1] += 1;
    else b->fell_back.push_back(k);
  }
  b->counts[2] = (int)b->fell_back.size();
  if (b->fell_back.empty()) return 0;
  stab_batch* fb = nullptr;
  int rc = batch_build_child(b, b->fell_back, 0, &fb);
  if (rc) return rc;
  std::unique_ptr<stab_batch> guard(fb);
  if (!track && b->level == 1) {
    // A second candidate level first: seeds from the spectrum at N = 48,
    // which resolves what N = 32 did not, at a fraction of the full
    // eigensolve's cost for the large instances; its own failures take the
    // plain path.  Results keep the fallback status.
    fb->level = 2;
    fb->coarse_ny = c->medium_ny;
    fb->coarse_ny_sp = (c->medium_ny_sp != b->coarse_ny_sp) ? c->medium_ny_sp : c->medium_ny;
    if (c->level_trust && (b->last_mode == STAB_MODE_COARSE || b->last_mode == STAB_MODE_SURROGATE) &&
        b->best_theta.p && b->have.p && b->best_src.p) {
      const int nf = fb->count;
      std::vector<int32_t> idx(b->fell_back.begin(), b->fell_back.end());
      CK(c, upload(fb->lev1_idx, idx, c->stream));
      CK(c, fb->lev1_lam.ensure(sizeof(zc) * nf, c->stream));
      CK(c, fb->lev1_th.ensure(sizeof(zc) * nf, c->stream));
      CK(c, fb->lev1_ok.ensure(sizeof(int32_t) * nf, c->stream));
      CK(c, timed(c, "k_gather_level", [&] {
        k_gather_level<<<(nf + 255) / 256, 256, 0, c->stream>>>(
            nf, fb->lev1_idx.as<int32_t>(), b->cand.as<zc>(), kShiftCandidates, b->best_theta.as<zc>(),
            b->have.as<int32_t>(), b->best_src.as<int32_t>(), fb->lev1_lam.as<zc>(), fb->lev1_th.as<zc>(),
            fb->lev1_ok.as<int32_t>());
        return cudaGetLastError();
      }));
      fb->has_lev1 = true;
      fb->lev1_n = b->coarse_ny;
    }
    rc = stab_batch_run(fb, STAB_MODE_COARSE);
    const int nf = fb->count;
    std::vector<double> eig(2 * (size_t)nf), er(nf), w(4, 0.0);
    std::vector<int32_t> itv(nf), st(nf);
    std::vector<std::vector<zc>> vecs(nf);
    std::vector<double*> vp(nf);
    for (int q = 0; q < nf; ++q) {
      vecs[q].resize(b->hm[b->fell_back[q]]);
      vp[q] = reinterpret_cast<double*>(vecs[q].data());
    }
    if (rc == 0) rc = stab_batch_results(fb, eig.data(), er.data(), itv.data(), st.data(), vp.data());
    if (rc == 0) rc = stab_batch_work(fb, w.data());
    if (rc) return rc;
    for (int i = 0; i < 4; ++i) b->fb_work[i] += w[i];
    b->fb_val.assign(nf, zmk(0, 0));
    b->fb_status.assign(nf, 0);
    b->fb_err = er;
    b->fb_iters = itv;
    b->fb_vec = std::move(vecs);
    for (int q = 0; q < nf; ++q) {
      b->fb_val[q] = zmk(eig[2 * q], eig[2 * q + 1]);
      b->fb_status[q] = (st[q] == STAB_ST_OK) ? STAB_ST_FELLBACK : st[q];   // UNVERIFIED stays
    }
    return 0;
  }
  rc = run_prep(fb);
  if (rc) return rc;
  rc = run_plain(fb, !track, "k_eig_plain_fallback");
  if (rc) return rc;
  const int nf = fb->count;
  if (track) {
    // nearest eigenvalue (user variable: omega or alpha) to the seed; then
    // its eigenvector by the same FP64 inverse iteration
    std::vector<zc> spec(fb->sum_m), pick_raw(nf), pick_val(nf);
    std::vector<int32_t> pidx(nf, -1);
    CK(c, cudaMemcpyAsync(spec.data(), fb->eigsorted.p, sizeof(zc) * fb->sum_m, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    for (int q = 0; q < nf; ++q) {
      const int u = b->perm[b->fell_back[fb->perm[q]]];   // caller index of sub-batch entry q
      const zc sd = zmk(b->seeds[2 * u], b->seeds[2 * u + 1]);
      const zc* e = spec.data() + fb->h_mof[q];
      double best = INFINITY;
      int j = 0;
      for (int t = 0; t < fb->hm[q]; ++t) {
        const double d = std::hypot(e[t].x - sd.x, e[t].y - sd.y);
        if (d < best) { best = d; j = t; }
      }
      pidx[q] = j;
      pick_val[q] = e[j];
      zc r = e[j];
      if (fb->P[q].itype == 2 || fb->P[q].itype == 4) {
        const double dd = r.x * r.x + r.y * r.y;
        r = dd > 0 ? zmk(r.x / dd, -r.y / dd) : zmk(0.0, 0.0);
      }
      pick_raw[q] = r;
    }
    CK(c, cudaMemcpyAsync(fb->least_val.p, pick_val.data(), sizeof(zc) * nf, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(fb->least_raw.p, pick_raw.data(), sizeof(zc) * nf, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(fb->least_idx.p, pidx.data(), sizeof(int32_t) * nf, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(fb->theta.p, fb->least_raw.p, sizeof(zc) * nf, cudaMemcpyDeviceToDevice, c->stream));
    const Range fall{0, nf};
    rc = eigvec_inverse_iteration(fb, fall, fb->theta.as<zc>());
    if (rc) return rc;
    rc = write_vectors(fb, fall, fb->theta.as<zc>());
    if (rc) return rc;
  }
  std::vector<zc> val(nf);
  std::vector<int32_t> st(nf), li(nf);
  CK(c, cudaMemcpyAsync(val.data(), fb->least_val.p, sizeof(zc) * nf, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(st.data(), fb->status.p, sizeof(int32_t) * nf, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(li.data(), fb->least_idx.p, sizeof(int32_t) * nf, cudaMemcpyDeviceToHost, c->stream));
  std::vector<std::vector<zc>> vecs(nf);
  for (int q = 0; q < nf; ++q) {
    vecs[q].resize(fb->hm[q]);
    CK(c, cudaMemcpyAsync(vecs[q].data(), fb->outvec.as<zc>() + fb->h_mof[q], sizeof(zc) * fb->hm[q],
                          cudaMemcpyDeviceToHost, c->stream));
  }
  CK(c, cudaStreamSynchronize(c->stream));
  {
    std::vector<double> f(nf);
    CK(c, cudaMemcpy(f.data(), fb->flops.p, sizeof(double) * nf, cudaMemcpyDeviceToHost));
    for (int q = 0; q < nf; ++q) {
      b->fb_work[0] += f[q];
      b->fb_work[3] += (8.0 / 3.0) * (double)fb->hn[q] * fb->hn[q] * fb->hn[q];
    }
  }
  // the sub-batch orders its instances temporal-first internally; map back
  b->fb_val.assign(b->fell_back.size(), zmk(0, 0));
  b->fb_status.assign(b->fell_back.size(), 0);
  b->fb_vec.assign(b->fell_back.size(), {});
  b->fb_err.assign(b->fell_back.size(), 0.0);
  b->fb_iters.assign(b->fell_back.size(), 0);
  for (int q = 0; q < nf; ++q) {
    const int j = fb->perm[q];            // index into fell_back
    b->fb_val[j] = val[q];
    b->fb_status[j] = (st[q] == 0 && li[q] >= 0) ? STAB_ST_FELLBACK : (st[q] ? st[q] : STAB_ST_NOMODE);
    b->fb_vec[j] = std::move(vecs[q]);
  }
  return 0;
}

static int coarse_sequence(stab_batch* b, bool extra) {
  int rc = run_prep(b);
  if (rc) return rc;
  rc = coarse_seeds(b);
  if (rc) return rc;
  if (!extra && b->level >= 2 && b->ctx->par_cand) return polish_candidates_parallel(b);
  return polish_candidate_rounds(b, extra);
}

// The device part of a STAB_MODE_COARSE pass is a fixed sequence of ~400
// launches whose per-instance choices live in device masks, so after a first
// eager pass (which sizes every pool) it is captured into a CUDA graph and
// replayed.  Per-kernel profiling and the legacy stream run eagerly.
static int run_coarse_device(stab_batch* b, bool extra) {
  stab_ctx* c = b->ctx;
  cudaStream_t s = c->stream;
  const int gmode = extra ? STAB_MODE_SURROGATE : STAB_MODE_COARSE;
  if (b->graph_epoch != c->epoch) b->coarse_runs = 0;   // new settings: one eager pass first
  const bool graphable = !c->profiling && s != nullptr && b->coarse_runs > 0 && b->graph_mode == gmode;
  if (b->coarse_graph && (b->graph_stream != s || b->graph_mode != gmode || b->graph_epoch != c->epoch)) {
    cudaGraphExecDestroy(b->coarse_graph);
    b->coarse_graph = nullptr;
  }
  if (graphable && !b->coarse_graph) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int rc = coarse_sequence(b, extra);
      const cudaError_t e = cudaStreamEndCapture(s, &g);
      if (rc == 0 && e == cudaSuccess && g) {
        if (cudaGraphInstantiate(&b->coarse_graph, g, 0) != cudaSuccess) b->coarse_graph = nullptr;
        b->graph_stream = s;
        b->graph_epoch = c->epoch;
      }
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();   // a failed capture leaves no sticky error: run eagerly below
    }
  }
  b->coarse_runs = (b->graph_mode == gmode) ? b->coarse_runs + 1 : 1;
  b->graph_mode = gmode;
  b->graph_epoch = c->epoch;
  if (graphable && b->coarse_graph) {
    CK(c, cudaGraphLaunch(b->coarse_graph, s));
    return 0;
  }
  return coarse_sequence(b, extra);
}

int stab_batch_run(stab_batch* b, int32_t mode) {
  if (!b) return STAB_ERR_ARG;
  if (!b->ctx) return STAB_ERR_STATE;
  stab_ctx* c = b->ctx;
  cudaSetDevice(c->device);
  if (mode == STAB_MODE_COARSE || mode == STAB_MODE_SURROGATE) {
    const bool extra = (mode == STAB_MODE_SURROGATE);
    if (extra) {
      if (!b->have_seeds) return set_err(c, STAB_ERR_STATE, "STAB_MODE_SURROGATE needs stab_batch_set_seeds first");
      std::vector<zc> sg(b->count);
      for (int k = 0; k < b->count; ++k) {
        const int u = b->perm[k];
        zc a = zmk(b->seeds[2 * u], b->seeds[2 * u + 1]);
        if (b->P[k].itype == 2 || b->P[k].itype == 4) {
          const double d = a.x * a.x + a.y * a.y;
          a = d > 0 ? zmk(a.x / d, -a.y / d) : zmk(0.0, 0.0);
        }
        sg[k] = a;
      }
      CK(c, upload(b->seed_raw, sg, c->stream));
      if (b->ncheb > 0) {
        int rc0 = upload_start(b);
        if (rc0) return rc0;
      }
    }
    b->fell_back.clear();
    b->last_mode = mode;
    int rc = run_coarse_device(b, extra);
    if (rc) return rc;
    rc = run_fallback(b);
    if (rc) return rc;
    b->ran = true;
    return STAB_OK;
  }
  int rc = batch_run(b, mode);
  if (rc) return rc;
  if (mode == STAB_MODE_SEEDED || mode == STAB_MODE_TRACK) {
    rc = retry_seeded(b);
    if (rc) return rc;
    return run_fallback(b, mode == STAB_MODE_TRACK);
  }
  b->counts[0] = b->count;
  b->counts[1] = b->counts[2] = 0;
  return STAB_OK;
}

int stab_batch_set_start(stab_batch* b, const double* coef, int32_t ncheb) {
  if (!b) return STAB_ERR_ARG;
  if (!b->ctx) return STAB_ERR_STATE;
  if (ncheb < 0 || ncheb > 256 || (ncheb > 0 && !coef)) return set_err(b->ctx, STAB_ERR_ARG, "ncheb must be 0..256");
  b->ncheb = ncheb;
  b->start_coef.assign(coef ? coef : nullptr, coef ? coef + 2 * (size_t)5 * ncheb * b->count : nullptr);
  return STAB_OK;
}

}  // extern "C"

// Autotuner of the LU panel width: for each requested order and both
// precisions, time every panel width shared memory admits (8, 16, 32) on a
// full wave of well-conditioned test matrices (CUDA events on the context
// stream, best of two) and keep the fastest for that size class.
template <typename T>
static int tune_lu_one(stab_ctx* c, int n, int reps, int* best_nb, float* best_ms) {
  cudaStream_t s = c->stream;
  const int count = std::max(1, c->sms * reps);
  DevBuf A, piv, info, nsz, moff, poff;
  CK(c, A.ensure(sizeof(T) * (size_t)count * n * n, s));
  CK(c, piv.ensure(sizeof(int32_t) * (size_t)count * n, s));
  CK(c, info.ensure(sizeof(int32_t) * count, s));
  std::vector<int32_t> ns(count, n);
  std::vector<int64_t> mo(count), po(count);
  for (int k = 0; k < count; ++k) {
    mo[k] = (int64_t)k * n * n;
    po[k] = (int64_t)k * n;
  }
  CK(c, upload(nsz, ns, s));
  CK(c, upload(moff, mo, s));
  CK(c, upload(poff, po, s));
  cudaEvent_t e0 = get_ev(c), e1 = get_ev(c);
  *best_nb = 0;
  *best_ms = 1e30f;
  for (int nb : {8, 16, 32}) {
    if (nb > lu_nb_max<T>(n)) continue;
    float t = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      CK(c, launch_tune_matrix<T>(count, n, A.as<T>(), s));
      CK(c, cudaEventRecord(e0, s));
      CK(c, launch_lu<T>(count, nullptr, nsz.as<int32_t>(), n, A.as<T>(), moff.as<int64_t>(), piv.as<int32_t>(),
                         poff.as<int64_t>(), info.as<int32_t>(), s, nullptr, nb));
      CK(c, cudaEventRecord(e1, s));
      CK(c, cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(c, cudaEventElapsedTime(&ms, e0, e1));
      t = std::min(t, ms);
    }
    if (t < *best_ms) {
      *best_ms = t;
      *best_nb = nb;
    }
  }
  c->evpool.push_back(e0);
  c->evpool.push_back(e1);
  CK(c, cudaStreamSynchronize(s));
  return 0;
}

// Factor the same test matrices with one CTA per matrix and with clusters of
// four CTAs; the factors and pivots must agree bit for bit.
template <typename T>
static int lu_cluster_check(stab_ctx* c, int n, int count, double* max_diff, int32_t* piv_diff) {
  cudaStream_t s = c->stream;
  DevBuf A1, A4, piv1, piv4, info, nsz, moff, poff;
  const size_t elems = (size_t)count * n * n;
  CK(c, A1.ensure(sizeof(T) * elems, s));
  CK(c, A4.ensure(sizeof(T) * elems, s));
  CK(c, piv1.ensure(sizeof(int32_t) * (size_t)count * n, s));
  CK(c, piv4.ensure(sizeof(int32_t) * (size_t)count * n, s));
  CK(c, info.ensure(sizeof(int32_t) * count, s));
  std::vector<int32_t> ns(count, n);
  std::vector<int64_t> mo(count), po(count);
  for (int k = 0; k < count; ++k) {
    mo[k] = (int64_t)k * n * n;
    po[k] = (int64_t)k * n;
  }
  CK(c, upload(nsz, ns, s));
  CK(c, upload(moff, mo, s));
  CK(c, upload(poff, po, s));
  CK(c, launch_tune_matrix<T>(count, n, A1.as<T>(), s));
  CK(c, launch_tune_matrix<T>(count, n, A4.as<T>(), s));
  CK(c, launch_lu<T>(count, nullptr, nsz.as<int32_t>(), n, A1.as<T>(), moff.as<int64_t>(), piv1.as<int32_t>(),
                     poff.as<int64_t>(), info.as<int32_t>(), s, nullptr, 0, nullptr, 1));
  CK(c, launch_lu<T>(count, nullptr, nsz.as<int32_t>(), n, A4.as<T>(), moff.as<int64_t>(), piv4.as<int32_t>(),
                     poff.as<int64_t>(), info.as<int32_t>(), s, nullptr, 0, nullptr, 4));
  std::vector<T> h1(elems), h4(elems);
  std::vector<int32_t> p1((size_t)count * n), p4((size_t)count * n);
  CK(c, cudaMemcpyAsync(h1.data(), A1.p, sizeof(T) * elems, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(h4.data(), A4.p, sizeof(T) * elems, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(p1.data(), piv1.p, sizeof(int32_t) * p1.size(), cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(p4.data(), piv4.p, sizeof(int32_t) * p4.size(), cudaMemcpyDeviceToHost, s));
  CK(c, cudaStreamSynchronize(s));
  double md = 0.0;
  for (size_t q = 0; q < elems; ++q)
    md = std::max(md, std::max(std::fabs((double)h1[q].x - (double)h4[q].x), std::fabs((double)h1[q].y - (double)h4[q].y)));
  int32_t pd = 0;
  for (size_t q = 0; q < p1.size(); ++q) pd += (p1[q] != p4[q]) ? 1 : 0;
  *max_diff = md;
  *piv_diff = pd;
  return 0;
}

// Factor the same complex64 test matrices on the CUDA cores and with the
// tensor-core update; backward errors of both on the host in FP64.
static int lu_tc_check(stab_ctx* c, int n, int count, double* bwd_tc, double* bwd_simt, int32_t* piv_diff) {
  cudaStream_t s = c->stream;
  DevBuf A1, A2, piv1, piv2, info, nsz, moff, poff;
  const size_t elems = (size_t)count * n * n;
  CK(c, A1.ensure(sizeof(cc) * elems, s));
  CK(c, A2.ensure(sizeof(cc) * elems, s));
  CK(c, piv1.ensure(sizeof(int32_t) * (size_t)count * n, s));
  CK(c, piv2.ensure(sizeof(int32_t) * (size_t)count * n, s));
  CK(c, info.ensure(sizeof(int32_t) * count, s));
  std::vector<int32_t> ns(count, n);
  std::vector<int64_t> mo(count), po(count);
  for (int k = 0; k < count; ++k) {
    mo[k] = (int64_t)k * n * n;
    po[k] = (int64_t)k * n;
  }
  CK(c, upload(nsz, ns, s));
  CK(c, upload(moff, mo, s));
  CK(c, upload(poff, po, s));
  CK(c, launch_tune_matrix<cc>(count, n, A1.as<cc>(), s));
  std::vector<cc> h0(elems), h1(elems), h2(elems);
  CK(c, cudaMemcpyAsync(h0.data(), A1.p, sizeof(cc) * elems, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(A2.p, A1.p, sizeof(cc) * elems, cudaMemcpyDeviceToDevice, s));
  CK(c, launch_lu<cc>(count, nullptr, nsz.as<int32_t>(), n, A1.as<cc>(), moff.as<int64_t>(), piv1.as<int32_t>(),
                      poff.as<int64_t>(), info.as<int32_t>(), s, nullptr, 16, nullptr, 1));
  DevBuf tmaps;
  const CUtensorMap* tm = nullptr;
  if (c->lu_tma && lu_tc_fits(n, true)) {
    std::vector<CUtensorMap> maps;
    std::vector<int32_t> ns2(count, n);
    if (lu_tc_tensor_maps(count, ns2.data(), mo.data(), A2.as<cc>(), maps)) {
      CK(c, upload(tmaps, maps, s));
      tm = tmaps.as<CUtensorMap>();
    }
  }
  CK(c, launch_lu_tc(count, nsz.as<int32_t>(), n, A2.as<cc>(), moff.as<int64_t>(), piv2.as<int32_t>(),
                     poff.as<int64_t>(), info.as<int32_t>(), s, nullptr, nullptr, tm));
  std::vector<int32_t> p1((size_t)count * n), p2((size_t)count * n), inf(count);
  CK(c, cudaMemcpyAsync(h1.data(), A1.p, sizeof(cc) * elems, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(h2.data(), A2.p, sizeof(cc) * elems, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(p1.data(), piv1.p, sizeof(int32_t) * p1.size(), cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(p2.data(), piv2.p, sizeof(int32_t) * p2.size(), cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(inf.data(), info.p, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, s));
  CK(c, cudaStreamSynchronize(s));
  // max |P A - L U| / max |A| per matrix, P A formed by applying the swaps
  auto bwd = [&](const std::vector<cc>& F, const std::vector<int32_t>& pv, int k) {
    const cc* a = h0.data() + (size_t)k * n * n;
    const cc* f = F.data() + (size_t)k * n * n;
    std::vector<zc> pa((size_t)n * n);
    double amax = 0.0;
    for (size_t q = 0; q < pa.size(); ++q) {
      pa[q] = zmk(a[q].x, a[q].y);
      amax = std::max(amax, std::fabs((double)a[q].x) + std::fabs((double)a[q].y));
    }
    for (int j = 0; j < n; ++j) {
      const int p = pv[(size_t)k * n + j];
      if (p != j)
        for (int col = 0; col < n; ++col) std::swap(pa[(size_t)col * n + j], pa[(size_t)col * n + p]);
    }
    double emax = 0.0;
    for (int col = 0; col < n; ++col)
      for (int r = 0; r < n; ++r) {
        zc acc = zmk(0.0, 0.0);
        const int lim = std::min(r, col);
        for (int t = 0; t <= lim; ++t) {
          const cc l = (t == r) ? cmk(1.f, 0.f) : f[(size_t)t * n + r];
          const cc u = f[(size_t)col * n + t];
          acc = zfma(zmk(l.x, l.y), zmk(u.x, u.y), acc);
        }
        const zc d = zsub(pa[(size_t)col * n + r], acc);
        emax = std::max(emax, std::fabs(d.x) + std::fabs(d.y));
      }
    return amax > 0 ? emax / amax : emax;
  };
  double e1 = 0.0, e2 = 0.0;
  int32_t pd = 0;
  for (int k = 0; k < count; ++k) {
    e1 = std::max(e1, bwd(h1, p1, k));
    e2 = std::max(e2, inf[k] < 0 ? INFINITY : bwd(h2, p2, k));
    for (int j = 0; j < n; ++j) pd += (p1[(size_t)k * n + j] != p2[(size_t)k * n + j]) ? 1 : 0;
  }
  *bwd_simt = e1;
  *bwd_tc = e2;
  *piv_diff = pd;
  return 0;
}

extern "C" {

int stab_lu_tc_check(stab_ctx* c, int32_t n, int32_t count, double* bwd_tc, double* bwd_simt, int32_t* piv_diff) {
  if (!c || !bwd_tc || !bwd_simt || !piv_diff || n < 2 || count < 1 || count > 64) return STAB_ERR_ARG;
  if (!lu_tc_fits(n)) return set_err(c, STAB_ERR_ARG, "order too large for the tensor-core LU's shared memory");
  cudaSetDevice(c->device);
  return lu_tc_check(c, n, count, bwd_tc, bwd_simt, piv_diff);
}

int stab_peak_rates(stab_ctx* c, double* out) {
  if (!c || !out) return STAB_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  float* sink = nullptr;
  CK(c, cudaMallocAsync(reinterpret_cast<void**>(&sink), sizeof(float), s));
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int iters[3] = {65536, 2048, 4096};   // a few milliseconds per launch
  int rc = STAB_OK;
  for (int kind = 0; kind < 3 && rc == STAB_OK; ++kind) {
    launch_probe(kind, 4 * sms, iters[kind] / 8, sink, s);   // warm-up
    cudaEventRecord(a, s);
    const double flops = launch_probe(kind, 4 * sms, iters[kind], sink, s);
    cudaEventRecord(b, s);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e != cudaSuccess) {
      rc = set_err(c, STAB_ERR_CUDA, cudaGetErrorString(e));
      break;
    }
    out[kind] = flops / (ms * 1e-3) / 1e12;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFreeAsync(sink, s);
  cudaStreamSynchronize(s);
  return rc;
}

int stab_lu_cluster_check(stab_ctx* c, int32_t n, int32_t count, int32_t complex128, double* max_diff,
                          int32_t* piv_diff) {
  if (!c || !max_diff || !piv_diff || n < 2 || n > 1024 || count < 1) return STAB_ERR_ARG;
  cudaSetDevice(c->device);
  return complex128 ? lu_cluster_check<zc>(c, n, count, max_diff, piv_diff)
                    : lu_cluster_check<cc>(c, n, count, max_diff, piv_diff);
}

int stab_autotune(stab_ctx* c, const int32_t* orders, int32_t norders, int32_t* nb_out, float* ms_out) {
  if (!c || !orders || norders < 1) return set_err(c, STAB_ERR_ARG, "no orders to tune");
  cudaSetDevice(c->device);
  for (int q = 0; q < norders; ++q) {
    const int n = orders[q];
    if (n < 2 || n > 2048) return set_err(c, STAB_ERR_ARG, "order must be 2..2048");
    for (int z = 0; z < 2; ++z) {
      int nb = 0;
      float ms = 0.f;
      const int reps = n <= 480 ? 2 : 1;
      const int rc = z ? tune_lu_one<zc>(c, n, reps, &nb, &ms) : tune_lu_one<cc>(c, n, reps, &nb, &ms);
      if (rc) return rc;
      c->lu_nb[{z, lu_class(n)}] = nb;
      c->epoch += 1;
      if (nb_out) nb_out[2 * q + z] = nb;
      if (ms_out) ms_out[2 * q + z] = ms;
    }
  }
  return STAB_OK;
}

int stab_set_arithmetic(stab_ctx* c, int32_t stage, int32_t arithmetic) {
  if (!c) return STAB_ERR_ARG;
  if (stage < STAB_STAGE_SEED_EIG || stage > STAB_STAGE_POLISH_LU)
    return set_err(c, STAB_ERR_ARG, "stage must be one of STAB_STAGE_*");
  if (stage == STAB_STAGE_POLISH_LU) {
    if (arithmetic != STAB_ARITH_FP32 && arithmetic != STAB_ARITH_TF32_SPLIT)
      return set_err(c, STAB_ERR_ARG, "the polish LU takes STAB_ARITH_FP32 or STAB_ARITH_TF32_SPLIT");
  } else if (arithmetic != STAB_ARITH_FP64 && arithmetic != STAB_ARITH_DOUBLE_WORD) {
    return set_err(c, STAB_ERR_ARG, "arithmetic must be STAB_ARITH_FP64 or STAB_ARITH_DOUBLE_WORD");
  }
  c->arith[stage] = arithmetic;
  c->epoch += 1;
  return STAB_OK;
}

int stab_set_option(stab_ctx* c, int32_t option, int32_t value) {
  if (!c) return STAB_ERR_ARG;
  if (option == STAB_OPT_SEED_QR_SHARED) {
    c->seed_qr_shared = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_POLISH_LU_TMA) {
    c->lu_tma = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_SEED_VECTORS) {
    c->seed_vectors = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_PARALLEL_CANDIDATES) {
    c->par_cand = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_LEVEL_CONSISTENCY) {
    c->level_trust = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_FIRST_RETRY) {
    c->first_retry = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_MLP_TCGEN05) {
    c->mlp_tc = value ? 1 : 0;
    return STAB_OK;
  }
  if (option == STAB_OPT_MEDIUM_NY_SPATIAL) {
    if (value < 16 || value > 64 || value == c->seed_ny)
      return set_err(c, STAB_ERR_ARG, "the spatial second level's N must be in [16, 64] and differ from the seed size");
    c->medium_ny_sp = value;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_MEDIUM_NY) {
    if (value < 16 || value > 64 || value == c->seed_ny)
      return set_err(c, STAB_ERR_ARG, "the second level's N must be in [16, 64] and differ from the seed size");
    c->medium_ny = value;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_EIG_MID) {
    c->eig_mid = value ? 1 : 0;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_EIG_THREADS) {
    if (value != 64 && value != 128) return set_err(c, STAB_ERR_ARG, "eigensolver CTA size must be 64 or 128");
    c->eig_threads = value;
    c->epoch += 1;
    return STAB_OK;
  }
  if (option == STAB_OPT_EIG_RESIDENT) {
    if (value < 0 || value > 64) return set_err(c, STAB_ERR_ARG, "resident instances per SM must be in [0, 64]");
    c->eig_resident = value;
    c->epoch += 1;
    return STAB_OK;
  }
  return set_err(c, STAB_ERR_ARG, "unknown option");
}

int stab_set_seed_size(stab_ctx* c, int32_t ny) {
  if (!c) return STAB_ERR_ARG;
  if (ny < 16 || ny >= kMediumNy || ny == c->medium_ny || ny == c->medium_ny_sp)
    return set_err(c, STAB_ERR_ARG, "seed size must be in [16, 48) and differ from the second levels' N");
  c->seed_ny = ny;
  return STAB_OK;
}

int stab_eig_phases(stab_ctx* c, uint64_t* cycles_out, int32_t reset) {
  if (!c || !cycles_out) return STAB_ERR_ARG;
  cudaSetDevice(c->device);
  CK(c, cudaStreamSynchronize(c->stream));
  unsigned long long v[6];
  CK(c, eig_phase_cycles(v, reset != 0));
  for (int i = 0; i < 6; ++i) cycles_out[i] = v[i];
  return STAB_OK;
}

int stab_batch_spectra(stab_batch* b, double* const* eig_out) {
  if (!b || !eig_out) return STAB_ERR_ARG;
  if (!b->ctx) return STAB_ERR_STATE;
  stab_ctx* c = b->ctx;
  if (!b->ran || b->last_mode != STAB_MODE_PLAIN) return set_err(c, STAB_ERR_STATE, "needs a STAB_MODE_PLAIN run");
  for (int k = 0; k < b->count; ++k) {
    double* dst = eig_out[b->perm[k]];
    if (dst)
      CK(c, cudaMemcpyAsync(dst, b->eigsorted.as<zc>() + b->h_mof[k], sizeof(zc) * b->hm[k], cudaMemcpyDeviceToHost,
                            c->stream));
  }
  CK(c, cudaStreamSynchronize(c->stream));
  return STAB_OK;
}

int stab_batch_counts(stab_batch* b, int32_t* counts_out) {
  if (!b || !counts_out) return STAB_ERR_ARG;
  if (!b->ran) return STAB_ERR_STATE;
  for (int i = 0; i < 3; ++i) counts_out[i] = b->counts[i];
  return STAB_OK;
}

int stab_batch_results(stab_batch* b, double* eig_out, double* err_out, int32_t* iters_out, int32_t* status_out,
                       double* const* vec_out) {
  if (!b) return STAB_ERR_ARG;
  if (!b->ctx) return STAB_ERR_STATE;
  stab_ctx* c = b->ctx;
  if (!b->ran) return set_err(c, STAB_ERR_STATE, "stab_batch_run has not run");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int n = b->count;
  std::vector<zc> val(n), raw(n);
  std::vector<double> er(n);
  std::vector<int32_t> it(n), st(n), dn(n), li(n), fl(n);
  CK(c, cudaMemcpyAsync(raw.data(), b->least_raw.p, sizeof(zc) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(val.data(), b->least_val.p, sizeof(zc) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(er.data(), b->err.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(it.data(), b->iters.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(st.data(), b->status.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(dn.data(), b->done.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(li.data(), b->least_idx.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaMemcpyAsync(fl.data(), b->flags.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  CK(c, cudaStreamSynchronize(s));
  if (b->last_mode == STAB_MODE_PLAIN) {
    for (int k = 0; k < n; ++k)
      if (st[k] == 0 && li[k] < 0) st[k] = STAB_ST_NOMODE;
  } else {
    val = raw;
    finalize_polish_host(val, st, dn, b->P);
  }
  std::vector<int> fbpos(n, -1);
  for (size_t j = 0; j < b->fell_back.size(); ++j) {
    const int k = b->fell_back[j];
    fbpos[k] = (int)j;
    val[k] = b->fb_val[j];
    st[k] = b->fb_status[j];
    if (j < b->fb_err.size()) er[k] = b->fb_err[j];
    if (j < b->fb_iters.size()) it[k] = b->fb_iters[j];
  }
  for (int k = 0; k < n; ++k) {
    if (fl[k] & 2) { st[k] = STAB_ST_NAN; val[k] = zmk(NAN, NAN); }
    else if (fl[k] & 1) st[k] = STAB_ST_SINGULAR;
  }
  for (int k = 0; k < n; ++k) {
    const int u = b->perm[k];
    if (eig_out) { eig_out[2 * u] = val[k].x; eig_out[2 * u + 1] = val[k].y; }
    if (err_out) err_out[u] = er[k];
    if (iters_out) iters_out[u] = it[k];
    if (status_out) status_out[u] = st[k];
    if (vec_out && vec_out[u]) {
      if (fbpos[k] >= 0) {
        std::memcpy(vec_out[u], b->fb_vec[fbpos[k]].data(), sizeof(zc) * b->hm[k]);
      } else {
        CK(c, cudaMemcpyAsync(vec_out[u], b->outvec.as<zc>() + b->h_mof[k], sizeof(zc) * b->hm[k],
                              cudaMemcpyDeviceToHost, s));
      }
    }
  }
  CK(c, cudaStreamSynchronize(s));
  return STAB_OK;
}

int stab_batch_work(stab_batch* b, double* work_out) {
  if (!b || !work_out) return STAB_ERR_ARG;
  if (!b->ctx) return STAB_ERR_STATE;
  stab_ctx* c = b->ctx;
  if (!b->ran) return set_err(c, STAB_ERR_STATE, "stab_batch_run has not run");
  CK(c, cudaStreamSynchronize(c->stream));
  auto eig_flops = [&](stab_batch* x) -> double {
    std::vector<double> f(x->count);
    if (cudaMemcpy(f.data(), x->flops.p, sizeof(double) * x->count, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    double t = 0;
    for (double v : f) t += v;
    return t;
  };
  const bool plain = (b->last_mode == STAB_MODE_PLAIN);
  std::vector<int32_t> l32(b->count, 0), l64(b->count, 0);
  if (!plain) {
    cudaMemcpy(l32.data(), b->lus32.p, sizeof(int32_t) * b->count, cudaMemcpyDeviceToHost);
    cudaMemcpy(l64.data(), b->lus64.p, sizeof(int32_t) * b->count, cudaMemcpyDeviceToHost);
  }
  double lu_c = 0.0, lu_z = 0.0;
  for (int k = 0; k < b->count; ++k) {
    const double n3 = (double)b->hn[k] * b->hn[k] * b->hn[k];
    lu_c += l32[k] * (8.0 / 3.0) * n3;
    lu_z += (plain ? 1 : l64[k]) * (8.0 / 3.0) * n3;
  }
  work_out[0] = (plain ? eig_flops(b) : 0.0) + b->fb_work[0];
  work_out[1] = ((b->last_mode == STAB_MODE_COARSE && b->coarse) ? eig_flops(b->coarse) : 0.0) + b->fb_work[1];
  work_out[2] = lu_c + b->fb_work[2];
  work_out[3] = lu_z + b->fb_work[3];
  if (b->copies && b->copies->ran && !plain) {   // the candidate copies' factorisations
    double wx[4] = {0.0, 0.0, 0.0, 0.0};
    int rc = stab_batch_work(b->copies, wx);
    if (rc) return rc;
    work_out[2] += wx[2];
    work_out[3] += wx[3];
  }
  return STAB_OK;
}

int stab_batch_destroy(stab_batch* b) {
  if (!b) return STAB_ERR_ARG;
  if (!b->ctx) {            // context already destroyed: device memory is gone
    delete b;
    return STAB_OK;
  }
  stab_ctx* c = b->ctx;
  cudaSetDevice(c->device);
  c->live.erase(std::remove(c->live.begin(), c->live.end(), b), c->live.end());
  delete b;
  return STAB_OK;
}

int stab_solve_batch(stab_ctx* c, int32_t count, const stab_params* p, const int32_t* nym,
                     const double* const* profiles, int32_t mode, const double* seeds, double* eig_out,
                     double* err_out, int32_t* status_out, double* const* vec_out) {
  stab_batch* b = nullptr;
  int rc = stab_batch_create(c, count, p, nym, profiles, &b);
  if (rc) return rc;
  std::unique_ptr<stab_batch, int (*)(stab_batch*)> guard(b, stab_batch_destroy);
  if (seeds) {
    rc = stab_batch_set_seeds(b, seeds);
    if (rc) return rc;
  }
  rc = stab_batch_run(b, mode);
  if (rc) return rc;
  return stab_batch_results(b, eig_out, err_out, nullptr, status_out, vec_out);
}

int stab_assemble(stab_ctx* c, const stab_params* p, int32_t nym, const double* profile, double* mats_out) {
  if (!c || !p || !profile || !mats_out) return set_err(c, STAB_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  stab_batch* b = nullptr;
  const double* pr[1] = {profile};
  int rc = batch_build(c, 1, p, &nym, pr, &b);
  if (rc) return rc;
  std::unique_ptr<stab_batch> guard(b);
  rc = run_prep(b);
  if (rc) return rc;
  rc = ensure_plain_pools(b);
  if (rc) return rc;
  const int n = b->hn[0];
  const Range r{0, 1};
  const int kinds_t[2] = {OP_T_A0, OP_T_B0};
  const int kinds_s[3] = {OP_S_C0, OP_S_C1, OP_S_C2};
  const int nk = is_spatial(p->itype) ? 3 : 2;
  for (int q = 0; q < nk; ++q) {
    const int kd = is_spatial(p->itype) ? kinds_s[q] : kinds_t[q];
    rc = node_ops(b, r, kd, kd, nullptr);
    if (rc) return rc;
    rc = dense<zc>(b, r, b->Z64.as<zc>(), b->off_n2.as<int64_t>(), 1, 1.0, "k_dense_z");
    if (rc) return rc;
    CK(c, cudaMemcpyAsync(mats_out + 2 * (size_t)q * n * n, b->Z64.p, sizeof(zc) * n * n, cudaMemcpyDeviceToHost,
                          c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  return STAB_OK;
}

int stab_eigenvectors(stab_ctx* c, const stab_params* p, int32_t nym, const double* profile, int32_t count,
                      const double* eig, double* vec_out, int32_t* status_out) {
  if (!c || !p || !profile || !eig || !vec_out || count < 0) return set_err(c, STAB_ERR_ARG, "null argument");
  if (count == 0) return STAB_OK;
  if (p->itype < 1 || p->itype > 4) return set_err(c, STAB_ERR_ARG, "itype must be 1, 2, 3 or 4");
  cudaSetDevice(c->device);
  const bool spatial = is_spatial(p->itype);
  const int64_t mlen = (int64_t)(spatial ? 10 : 5) * p->ny;
  const zc* ev = reinterpret_cast<const zc*>(eig);
  // copies of the instance, one per eigenvalue, in chunks that bound memory
  const int chunk = 256;
  for (int k0 = 0; k0 < count; k0 += chunk) {
    const int cnt = std::min(chunk, count - k0);
    std::vector<stab_params> ps(cnt, *p);
    std::vector<int32_t> ns(cnt, nym);
    std::vector<const double*> pr(cnt, profile);
    stab_batch* b = nullptr;
    int rc = batch_build(c, cnt, ps.data(), ns.data(), pr.data(), &b);
    if (rc) return rc;
    std::unique_ptr<stab_batch> guard(b);
    rc = run_prep(b);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    CK(c, b->Z64.ensure(sizeof(zc) * b->sum_n2, s));
    // theta: the eigenvalue in the solver's variable (omega, or lambda =
    // 1/alpha with alpha = 0 -> lambda = 0); shift: theta moved by a few
    // ulps so that Q(shift) is not exactly singular
    std::vector<zc> th(cnt), sh(cnt);
    for (int k = 0; k < cnt; ++k) {
      const zc w = ev[k0 + b->perm[k]];
      zc t = w;
      if (spatial) t = (w.x != 0.0 || w.y != 0.0) ? zdiv(zmk(1.0, 0.0), w) : zmk(0.0, 0.0);
      const double d = 1e-14 * (std::hypot(t.x, t.y) + 1.0);
      th[k] = t;
      sh[k] = zmk(t.x + d, t.y + d);
    }
    CK(c, upload(b->theta, th, s));
    CK(c, upload(b->sigma, sh, s));
    rc = eigvec_inverse_iteration(b, Range{0, cnt}, b->sigma.as<zc>());
    if (rc) return rc;
    rc = write_vectors(b, Range{0, cnt}, b->theta.as<zc>());
    if (rc) return rc;
    std::vector<int32_t> info(cnt);
    CK(c, cudaMemcpyAsync(info.data(), b->info.p, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, s));
    for (int k = 0; k < cnt; ++k) {
      const int u = k0 + b->perm[k];
      CK(c, cudaMemcpyAsync(vec_out + 2 * (int64_t)u * mlen, b->outvec.as<zc>() + b->h_mof[k], sizeof(zc) * mlen,
                            cudaMemcpyDeviceToHost, s));
    }
    CK(c, cudaStreamSynchronize(s));
    if (status_out) {
      for (int k = 0; k < cnt; ++k) {
        const int u = k0 + b->perm[k];
        const double* v = vec_out + 2 * (int64_t)u * mlen;
        bool finite = true;
        for (int64_t q = 0; q < 2 * mlen; ++q) finite = finite && std::isfinite(v[q]);
        status_out[u] = !finite ? STAB_ST_NAN : (info[k] ? STAB_ST_SINGULAR : STAB_ST_OK);
      }
    }
  }
  return STAB_OK;
}

int stab_full_spectrum(stab_ctx* c, const stab_params* p, int32_t nym, const double* profile, double* eig_out,
                       double* vec_out, int32_t* least_index_out, int32_t* status_out) {
  if (!c || !p || !profile || !eig_out) return set_err(c, STAB_ERR_ARG, "null argument");
  cudaSetDevice(c->device);
  stab_batch* b = nullptr;
  const double* pr[1] = {profile};
  int rc = batch_build(c, 1, p, &nym, pr, &b);
  if (rc) return rc;
  std::unique_ptr<stab_batch> guard(b);
  rc = run_prep(b);
  if (rc) return rc;
  rc = run_plain(b, vec_out != nullptr);
  if (rc) return rc;
  const int m = b->hm[0];
  int32_t st = 0, li = -1, fl = 0;
  CK(c, cudaMemcpyAsync(eig_out, b->eigsorted.p, sizeof(zc) * m, cudaMemcpyDeviceToHost, c->stream));
  if (vec_out) CK(c, cudaMemcpyAsync(vec_out, b->outvec.p, sizeof(zc) * m, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(&st, b->status.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(&li, b->least_idx.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaMemcpyAsync(&fl, b->flags.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (fl & 2) st = STAB_ST_NAN;
  else if (fl & 1) st = STAB_ST_SINGULAR;
  if (st == 0 && li < 0) st = STAB_ST_NOMODE;
  if (least_index_out) *least_index_out = li;
  if (status_out) *status_out = st;
  return STAB_OK;
}


// ---- surrogate network -----------------------------------------------------
// A BF16 MLP with float32 master weights, trained and run by the kernels of
// mlp.cu on the context stream.  Layer l has sizes[l] inputs and
// sizes[l+1] outputs; W_l is stored sizes[l] x sizes[l+1] row-major, and the
// packed parameter vector is [W_0, b_0, W_1, b_1, ...].
}  // extern "C"

struct stab_mlp {
  stab_ctx* ctx = nullptr;
  std::vector<int> sz;
  int L = 0, maxb = 0;
  std::vector<int64_t> woff, boff;
  int64_t nparam = 0;
  DevBuf p32, g32, m32, v32, p16, loss;
  std::vector<DevBuf> hin16, z32;   // per layer: bf16 input, f32 pre-activation / output
  DevBuf dz32[2], dz16[2];
  int batch = 0;                      // batch of the last forward
  int step = 0;
};

// free the device memory of a network whose context goes away first
static void release_net(stab_mlp* m) {
  std::vector<DevBuf*> all = {&m->p32, &m->g32, &m->m32, &m->v32, &m->p16, &m->loss, &m->dz32[0], &m->dz32[1],
                              &m->dz16[0], &m->dz16[1]};
  for (auto& d : m->hin16) all.push_back(&d);
  for (auto& d : m->z32) all.push_back(&d);
  for (DevBuf* d : all) {
    if (d->p) cudaFreeAsync(d->p, d->st);
    d->p = nullptr;
    d->bytes = 0;
  }
  m->ctx = nullptr;
}

static int mlp_layers(stab_mlp* m, int b, const float* x) {
  stab_ctx* c = m->ctx;
  cudaStream_t s = c->stream;
  const __nv_bfloat16* P16 = m->p16.as<__nv_bfloat16>();
  const float* P = m->p32.as<float>();
  CK(c, timed(c, "k_cast_bf16", [&] {
    return stab::mlp_cast_bf16((int64_t)b * m->sz[0], x, m->hin16[0].as<__nv_bfloat16>(), s);
  }));
  for (int l = 0; l < m->L; ++l) {
    const int K = m->sz[l], N = m->sz[l + 1];
    const __nv_bfloat16* W = P16 + m->woff[l];
    const float* bias = P + m->boff[l];
    if (l + 1 < m->L) {
      CK(c, timed(c, "k_gemm_bf16_hidden", [&] {
        return stab::mlp_gemm_hidden(b, N, K, m->hin16[l].as<__nv_bfloat16>(), W, bias, m->z32[l].as<float>(),
                                     m->hin16[l + 1].as<__nv_bfloat16>(), s, c->mlp_tc != 0);
      }));
    } else {
      CK(c, timed(c, "k_gemm_bf16_out", [&] {
        return stab::mlp_gemm_out(b, N, K, m->hin16[l].as<__nv_bfloat16>(), W, bias, m->z32[l].as<float>(), s,
                                  c->mlp_tc != 0);
      }));
    }
  }
  m->batch = b;
  return 0;
}

static int mlp_backward(stab_mlp* m, const float* t, const float* w, double* loss_out) {
  stab_ctx* c = m->ctx;
  cudaStream_t s = c->stream;
  const int b = m->batch;
  const __nv_bfloat16* P16 = m->p16.as<__nv_bfloat16>();
  float* G = m->g32.as<float>();
  CK(c, cudaMemsetAsync(m->g32.p, 0, sizeof(float) * m->nparam, s));
  CK(c, cudaMemsetAsync(m->loss.p, 0, sizeof(double), s));
  const int Lo = m->L - 1;
  CK(c, timed(c, "k_loss_grad", [&] {
    return stab::mlp_loss_grad(b, m->sz[m->L], m->z32[Lo].as<float>(), m->sz[m->L], t, w, m->dz32[0].as<float>(),
                               m->dz16[0].as<__nv_bfloat16>(), m->loss.as<double>(), s);
  }));
  int cur = 0;
  for (int l = Lo; l >= 0; --l) {
    const int K = m->sz[l], N = m->sz[l + 1];
    CK(c, timed(c, "k_gemm_bf16_wgrad", [&] {
      return stab::mlp_gemm_wgrad(b, N, K, m->hin16[l].as<__nv_bfloat16>(), m->dz16[cur].as<__nv_bfloat16>(),
                                  G + m->woff[l], s, c->mlp_tc != 0);
    }));
    CK(c, timed(c, "k_bias_grad", [&] {
      return stab::mlp_bias_grad(b, N, m->dz32[cur].as<float>(), G + m->boff[l], s);
    }));
    if (l > 0) {
      CK(c, timed(c, "k_gemm_bf16_dhidden", [&] {
        return stab::mlp_gemm_dhidden(b, N, K, m->dz16[cur].as<__nv_bfloat16>(), P16 + m->woff[l],
                                      m->z32[l - 1].as<float>(), m->dz32[1 - cur].as<float>(),
                                      m->dz16[1 - cur].as<__nv_bfloat16>(), s, c->mlp_tc != 0);
      }));
      cur = 1 - cur;
    }
  }
  if (loss_out) {
    CK(c, cudaMemcpyAsync(loss_out, m->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(c, cudaStreamSynchronize(s));
    if (c->mlp_tc) {   // a tensor-core tile that gave up waiting leaves its outputs unwritten
      int to = 0;
      CK(c, stab::mlp_tc_timeouts(&to, true));
      if (to) return set_err(c, STAB_ERR_CUDA, "tcgen05 GEMM of the network: MMA completion not seen");
    }
  }
  return 0;
}

extern "C" {

int stab_mlp_create(stab_ctx* c, int32_t nlayers, const int32_t* sizes, int32_t max_batch, stab_mlp** out) {
  if (!c || !sizes || !out || nlayers < 1 || nlayers > 16 || max_batch < 1)
    return set_err(c, STAB_ERR_ARG, "bad network shape");
  for (int l = 0; l <= nlayers; ++l)
    if (sizes[l] < 1 || sizes[l] > 4096) return set_err(c, STAB_ERR_ARG, "layer width must be 1..4096");
  cudaSetDevice(c->device);
  std::unique_ptr<stab_mlp> m(new stab_mlp());
  m->ctx = c;
  m->L = nlayers;
  m->maxb = max_batch;
  m->sz.assign(sizes, sizes + nlayers + 1);
  int64_t off = 0;
  int maxw = 0;
  for (int l = 0; l < nlayers; ++l) {
    m->woff.push_back(off);
    off += (int64_t)sizes[l] * sizes[l + 1];
    m->boff.push_back(off);
    off += sizes[l + 1];
    maxw = std::max(maxw, std::max(sizes[l], sizes[l + 1]));
  }
  m->nparam = off;
  cudaStream_t s = c->stream;
  CK(c, m->p32.ensure(sizeof(float) * off, s));
  CK(c, m->g32.ensure(sizeof(float) * off, s));
  CK(c, m->m32.ensure(sizeof(float) * off, s));
  CK(c, m->v32.ensure(sizeof(float) * off, s));
  CK(c, m->p16.ensure(sizeof(__nv_bfloat16) * off, s));
  CK(c, m->loss.ensure(sizeof(double), s));
  CK(c, cudaMemsetAsync(m->p32.p, 0, sizeof(float) * off, s));
  CK(c, cudaMemsetAsync(m->p16.p, 0, sizeof(__nv_bfloat16) * off, s));
  m->hin16.resize(nlayers);
  m->z32.resize(nlayers);
  for (int l = 0; l < nlayers; ++l) {
    CK(c, m->hin16[l].ensure(sizeof(__nv_bfloat16) * (size_t)max_batch * sizes[l], s));
    CK(c, m->z32[l].ensure(sizeof(float) * (size_t)max_batch * sizes[l + 1], s));
  }
  for (int q = 0; q < 2; ++q) {
    CK(c, m->dz32[q].ensure(sizeof(float) * (size_t)max_batch * maxw, s));
    CK(c, m->dz16[q].ensure(sizeof(__nv_bfloat16) * (size_t)max_batch * maxw, s));
  }
  CK(c, cudaStreamSynchronize(s));
  c->nets.push_back(m.get());
  *out = m.release();
  return STAB_OK;
}

int64_t stab_mlp_param_count(const stab_mlp* m) { return m ? m->nparam : STAB_ERR_ARG; }

int stab_mlp_set_params(stab_mlp* m, const float* params) {
  if (!m || !params) return STAB_ERR_ARG;
  if (!m->ctx) return STAB_ERR_STATE;
  stab_ctx* c = m->ctx;
  cudaStream_t s = c->stream;
  CK(c, cudaMemcpyAsync(m->p32.p, params, sizeof(float) * m->nparam, cudaMemcpyHostToDevice, s));
  CK(c, cudaMemsetAsync(m->m32.p, 0, sizeof(float) * m->nparam, s));
  CK(c, cudaMemsetAsync(m->v32.p, 0, sizeof(float) * m->nparam, s));
  CK(c, stab::mlp_cast_bf16(m->nparam, m->p32.as<float>(), m->p16.as<__nv_bfloat16>(), s));
  CK(c, cudaStreamSynchronize(s));
  m->step = 0;
  return STAB_OK;
}

int stab_mlp_get_params(stab_mlp* m, float* params_out, float* grads_out) {
  if (!m) return STAB_ERR_ARG;
  if (!m->ctx) return STAB_ERR_STATE;
  stab_ctx* c = m->ctx;
  cudaStream_t s = c->stream;
  if (params_out)
    CK(c, cudaMemcpyAsync(params_out, m->p32.p, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost, s));
  if (grads_out)
    CK(c, cudaMemcpyAsync(grads_out, m->g32.p, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost, s));
  CK(c, cudaStreamSynchronize(s));
  return STAB_OK;
}

int stab_mlp_forward(stab_mlp* m, int32_t batch, const float* x_dev, float* y_dev) {
  if (m && !m->ctx) return STAB_ERR_STATE;
  if (!m || !x_dev || batch < 1 || batch > m->maxb) return set_err(m ? m->ctx : nullptr, STAB_ERR_ARG, "bad batch");
  int rc = mlp_layers(m, batch, x_dev);
  if (rc) return rc;
  if (y_dev)
    CK(m->ctx, cudaMemcpyAsync(y_dev, m->z32[m->L - 1].p, sizeof(float) * (size_t)batch * m->sz[m->L],
                               cudaMemcpyDeviceToDevice, m->ctx->stream));
  return STAB_OK;
}

int stab_mlp_gradients(stab_mlp* m, int32_t batch, const float* x_dev, const float* t_dev, const float* w_dev,
                       double* loss_out) {
  if (m && !m->ctx) return STAB_ERR_STATE;
  if (!m || !x_dev || !t_dev || !w_dev || batch < 1 || batch > m->maxb)
    return set_err(m ? m->ctx : nullptr, STAB_ERR_ARG, "bad batch");
  int rc = mlp_layers(m, batch, x_dev);
  if (rc) return rc;
  return mlp_backward(m, t_dev, w_dev, loss_out);
}

int stab_mlp_train_step(stab_mlp* m, int32_t batch, const float* x_dev, const float* t_dev, const float* w_dev,
                        float lr, double* loss_out) {
  int rc = stab_mlp_gradients(m, batch, x_dev, t_dev, w_dev, loss_out);
  if (rc) return rc;
  stab_ctx* c = m->ctx;
  m->step += 1;
  CK(c, timed(c, "k_adam", [&] {
    return stab::mlp_adam(m->nparam, m->p32.as<float>(), m->g32.as<float>(), m->m32.as<float>(), m->v32.as<float>(),
                          m->p16.as<__nv_bfloat16>(), lr, 0.9f, 0.999f, 1e-8f, m->step, c->stream);
  }));
  return STAB_OK;
}

int stab_mlp_destroy(stab_mlp* m) {
  if (!m) return STAB_ERR_ARG;
  if (m->ctx) {
    stab_ctx* c = m->ctx;
    cudaSetDevice(c->device);
    c->nets.erase(std::remove(c->nets.begin(), c->nets.end(), m), c->nets.end());
    release_net(m);
    cudaStreamSynchronize(c->stream);
  }
  delete m;
  return STAB_OK;
}

}  // extern "C"
