// Per-instance preparation on the GPU: Chebyshev derivative tables, mean-
// profile spline fit and evaluation, mapped mean derivatives, and the
// per-node 5x5 operator blocks of the temporal pencil / spatial operator.
//
// Reference map (sscollis/stab):
//   chebyd.f90:2-60        k_cheb_a, k_cheb_d1, k_cheb_d2 (D2 = D1 D1, temporal.f90:136)
//   spline.f90:2-49        k_spline (SPLINE, cantilever end condition, lambda = 1)
//   sgengrid.f90:2-45      node_grid (algebraic maps)
//   spline.f90:52-75 +     k_nodes (SPEVAL; getmean clamps above the last row,
//   getmean.f90:95-112               getmean.f90:103-108; with ider = 0 the
//   getmean2.f90:99-175              derivative tables too)
//   temporal.f90:148-179   k_meanderiv (D1 v, D2 v and the map chain rule)
//   temporal.f90:206-598   k_blocks (materials, coefficient blocks), and
//   spatial.f90:138-673    the spatial variant: h = 1 (node_blocks), or the
//                          circular wall of circh.f90 (node_blocks_curved)
//   temporal.f90:604-662   temporal operator blocks (Dh, Bh, mapping, B0)
//   spatial.f90:677-959    spatial operator blocks (C0, C1, C2)
#include "common.cuh"
#include "kernels.cuh"

namespace stab {

// ---------------------------------------------------------------------------
// Chebyshev derivative matrix on Gauss-Lobatto points (CHEBYD): D1(j,k) =
// a_j / (a_k (x_j - x_k)), D1(j,j) = sum_{k != j} 1/(x_j - x_k),
// a_j = prod_{k != j} (x_j - x_k).  Tables are row-major N x N.
// ---------------------------------------------------------------------------
__global__ void k_cheb_a(int ny, double* xa /* [2*ny]: x then a */) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ny) return;
  const int N = ny - 1;
  const double pi = acos(-1.0);
  double xj = cos(pi * (double)j / (double)N);
  double a = 1.0;
  for (int k = 0; k <= N; ++k) {
    if (k == j) continue;
    double xk = cos(pi * (double)k / (double)N);
    a *= (xj - xk);
  }
  xa[j] = xj;
  xa[ny + j] = a;
}

__global__ void k_cheb_d1(int ny, const double* xa, double* D1) {
  int j = blockIdx.y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ny || k >= ny) return;
  double xj = xa[j];
  if (k == j) {
    double s = 0.0;
    for (int q = 0; q < ny; ++q)
      if (q != j) s += 1.0 / (xj - xa[q]);
    D1[(size_t)j * ny + k] = s;
  } else {
    D1[(size_t)j * ny + k] = xa[ny + j] / (xa[ny + k] * (xj - xa[k]));
  }
}

__global__ void k_cheb_d2(int ny, const double* D1, double* D2) {
  int j = blockIdx.y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ny || k >= ny) return;
  double s = 0.0;
  for (int q = 0; q < ny; ++q) s = fma(D1[(size_t)j * ny + q], D1[(size_t)q * ny + k], s);
  D2[(size_t)j * ny + k] = s;
}

// ---------------------------------------------------------------------------
// SPLINE: second derivatives of the interpolating cubic spline of each of the
// five profile fields, with the cantilever end condition.  One thread per
// instance; the five fields share the modified diagonal and run as five
// independent recurrences (instruction-level parallelism).
// Spline pool layout per instance: nym rows x 6 (fdp[5], modified diag).
// ---------------------------------------------------------------------------
__global__ void k_spline(int nprof, const ProfDesc* __restrict__ pdesc, const double* __restrict__ prof,
                         double* __restrict__ spl, int32_t* __restrict__ bad) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nprof) return;
  const ProfDesc d = pdesc[k];
  const int n = d.nym;
  const double* P = prof + d.off_prof;   // row i: y rho u v w T
  double* S = spl + d.off_spl;           // row i: five second derivatives, then 1/b(i) (scratch)
  // the interval search of SPEVAL needs strictly ascending, finite abscissae
  int ok = 1;
  for (int i = 0; i < n; ++i) {
    for (int f = 0; f < 6; ++f) ok &= isfinite(P[6 * i + f]) ? 1 : 0;
    if (i > 0) ok &= (P[6 * i] > P[6 * (i - 1)]) ? 1 : 0;
  }
  bad[k] = ok ? 0 : 1;
  auto X = [&](int i) { return P[6 * i]; };
  auto Y = [&](int i, int f) { return f == 2 ? 0.0 : P[6 * i + 1 + f]; };  // v forced to 0
  // assemble c(i), a(i), b(i), r(i) and eliminate forward in one pass.
  // One thread runs the whole recurrence, and on GB300 each FP64 division is
  // a multi-instruction sequence at 1/64 rate.  So every row takes one
  // reciprocal of its interval and one of the pivot, shared by the five
  // fields; the pivot's reciprocal is stored in place of b(i) for the back
  // substitution.
  double c_prev = X(1) - X(0);           // C(1)
  double ic_prev = 1.0 / c_prev;
  double ib_prev = 0.0, r_prev[5] = {0, 0, 0, 0, 0};
  for (int i = 1; i <= n - 2; ++i) {
    const double ci = X(i + 1) - X(i);
    const double ici = 1.0 / ci;
    const double ai = c_prev;
    double bi = 2.0 * (ai + ci);
    double ri[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) ri[f] = 6.0 * ((Y(i + 1, f) - Y(i, f)) * ici - (Y(i, f) - Y(i - 1, f)) * ic_prev);
    if (i == 1) bi += 1.0 * (X(1) - X(0));          // B(2) += lambda*C(1)
    if (i == n - 2) bi += 1.0 * ci;                  // B(NM1) += lambda*C(NM1)
    if (i >= 2) {
      const double t = ai * ib_prev;
      bi = bi - t * c_prev;
#pragma unroll
      for (int f = 0; f < 5; ++f) ri[f] = ri[f] - t * r_prev[f];
    }
    const double ibi = 1.0 / bi;
#pragma unroll
    for (int f = 0; f < 5; ++f) { S[6 * i + f] = ri[f]; r_prev[f] = ri[f]; }
    S[6 * i + 5] = ibi;
    ib_prev = ibi;
    c_prev = ci;
    ic_prev = ici;
  }
  // back substitution, FDP(NM1) = R(NM1)/B(NM1); FDP(k) = (R(k) - C(k) FDP(k+1))/B(k)
  double nxt[5];
  {
    int i = n - 2;
    const double ibi = S[6 * i + 5];
#pragma unroll
    for (int f = 0; f < 5; ++f) { nxt[f] = S[6 * i + f] * ibi; S[6 * i + f] = nxt[f]; }
  }
  for (int i = n - 3; i >= 1; --i) {
    const double ci = X(i + 1) - X(i);
    const double ibi = S[6 * i + 5];
#pragma unroll
    for (int f = 0; f < 5; ++f) { nxt[f] = (S[6 * i + f] - ci * nxt[f]) * ibi; S[6 * i + f] = nxt[f]; }
  }
#pragma unroll
  for (int f = 0; f < 5; ++f) {
    S[f] = 1.0 * S[6 * 1 + f];
    S[6 * (n - 1) + f] = 1.0 * S[6 * (n - 2) + f];
  }
}

// grid of sgengrid (algebraic maps): eta = cos(pi (i-1)/(ny-1))
__device__ __forceinline__ void node_grid(const InstDesc& d, int i, double& y, double& eta, double& deta,
                                          double& d2eta) {
  if (d.fd) {
    // ogengrid.f90:20-44: eta = i / (ny - 1) on [0, 1], wall first,
    // y = a eta / (b - eta), a = ymax yi / (ymax - 2 yi), b = 1 + a / ymax
    const double dy = 1.0 / (double)(d.ny - 1);
    const double aa = d.ymax * d.yi / (d.ymax - 2.0 * d.yi);
    const double bb = 1.0 + aa / d.ymax;
    eta = (double)i * dy;
    y = aa * eta / (bb - eta);
    const double q = bb - eta;
    deta = q * q / (aa * bb);
    d2eta = -2.0 * q * q * q / ((aa * bb) * (aa * bb));
    return;
  }
  const double pi = 3.1415926535897932385;
  double dth = pi / (double)(d.ny - 1);
  eta = cos((double)i * dth);
  const double yi = d.yi, ymax = d.ymax;
  if (ymax == 0.0) {  // infinite domain
    deta = (eta - 1.0) * (eta - 1.0) / (2.0 * yi);
    d2eta = (eta - 1.0) * (eta - 1.0) * (eta - 1.0) / (2.0 * yi * yi);
    y = (eta != 1.0) ? yi * (1.0 + eta) / (1.0 - eta) : 1.0e99;
  } else {            // Streett's map
    double q = 2.0 * yi + 1.0 - eta;
    y = ymax * yi * (1.0 + eta) / (1.0 + 2.0 * yi - eta);
    deta = q * q / (2.0 * ymax * yi * (yi + 1.0));
    double r = ymax * yi * (yi + 1.0);
    d2eta = -0.5 * q * q * q / (r * r);
  }
}

// Grid + SPEVAL of the five fields at every node; one thread per node.
// The interval search returns the first I with y <= X(I+1) like SPEVAL's
// linear scan; the profile abscissae are strictly ascending, so a binary
// search gives the same interval.
// SPEVAL (spline.f90:52-75) of the five fields of a table (rows y f1..f5,
// v = 0) at y; above ymaxm the table's last row.
__device__ __forceinline__ void table_eval(const double* __restrict__ P, const double* __restrict__ S, int n,
                                           double y, double ymaxm, double* __restrict__ out) {
  if (y <= ymaxm) {
    int lo = 0, hi = n - 2;  // find first I in [0, n-2] with y <= X(I+1)
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (y <= P[6 * (mid + 1)]) hi = mid; else lo = mid + 1;
    }
    int I = lo;
    double x0 = P[6 * I], x1 = P[6 * (I + 1)];
    double dxm = y - x0, dxp = x1 - y, del = x1 - x0;
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      double y0 = (f == 2) ? 0.0 : P[6 * I + 1 + f];
      double y1 = (f == 2) ? 0.0 : P[6 * (I + 1) + 1 + f];
      double f0 = S[6 * I + f], f1 = S[6 * (I + 1) + f];
      out[f] = f0 * dxp * (dxp * dxp / del - del) / 6.0 + f1 * dxm * (dxm * dxm / del - del) / 6.0 +
               y0 * dxp / del + y1 * dxm / del;
    }
  } else {
#pragma unroll
    for (int f = 0; f < 5; ++f) out[f] = (f == 2) ? 0.0 : P[6 * (n - 1) + 1 + f];
  }
}

__global__ void k_nodes(int count, const InstDesc* __restrict__ desc, const double* __restrict__ prof,
                        const double* __restrict__ spl, double* __restrict__ node, const int32_t* __restrict__ bad,
                        int32_t* __restrict__ flags) {
  int k = blockIdx.y;
  if (k >= count) return;
  const InstDesc d = desc[k];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ny) return;
  if (i == 0 && (bad[d.iprof] || (d.ider == 0 && (bad[d.iprof_d1] || bad[d.iprof_d2])))) atomicOr(flags + k, 2);
  double y, eta, deta, d2eta;
  node_grid(d, i, y, eta, deta, d2eta);
  const double* P = prof + d.off_prof;
  const int n = d.nym;
  double* out = node + d.off_node + (size_t)NODE_STRIDE * i;
  out[NODE_Y] = y;
  out[NODE_ETA] = eta;
  out[NODE_DETA] = deta;
  out[NODE_D2ETA] = d2eta;
  // nodes above the mean profile's last row take each table's last row
  // (getmean.f90:103-108, getmean2.f90:84-97, 127-140, 163-176)
  const double ymaxm = P[6 * (n - 1)];
  table_eval(P, spl + d.off_spl, n, y, ymaxm, out + NODE_VM);
  if (d.ider == 0) {
    table_eval(prof + d.off_prof_d1, spl + d.off_spl_d1, n, y, ymaxm, out + NODE_G2);
    table_eval(prof + d.off_prof_d2, spl + d.off_spl_d2, n, y, ymaxm, out + NODE_G22);
  }
}

// g2 = deta * D1 v,  g22 = deta^2 * D2 v + d2eta * D1 v; one thread per (node, field).
// D1, D2: the Chebyshev matrices, or for the finite-difference solver
// grad.f90's fourth-order matrix G and G G (fd_temporal.f90:135-152)
__global__ void k_meanderiv(int count, const InstDesc* __restrict__ desc, const double* const* __restrict__ dtab,
                            double* __restrict__ node) {
  int k = blockIdx.y;
  if (k >= count) return;
  const InstDesc d = desc[k];
  if (d.ider == 0) return;   // derivatives from the tables (temporal.f90:149-179 skip with ider false)
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.ny * 5) return;
  int i = t / 5, f = t % 5;
  const int ny = d.ny;
  const double* D1 = dtab[2 * d.dmean];
  const double* D2 = dtab[2 * d.dmean + 1];
  double* nb = node + d.off_node;
  double s1 = 0.0, s2 = 0.0;
  for (int j = 0; j < ny; ++j) {
    double v = nb[(size_t)NODE_STRIDE * j + NODE_VM + f];
    s1 = fma(D1[(size_t)i * ny + j], v, s1);
    s2 = fma(D2[(size_t)i * ny + j], v, s2);
  }
  double deta = nb[(size_t)NODE_STRIDE * i + NODE_DETA];
  double d2eta = nb[(size_t)NODE_STRIDE * i + NODE_D2ETA];
  nb[(size_t)NODE_STRIDE * i + NODE_G22 + f] = s2 * deta * deta + s1 * d2eta;
  nb[(size_t)NODE_STRIDE * i + NODE_G2 + f] = s1 * deta;
}

// ---------------------------------------------------------------------------
// Physics: the eleven real 5x5 coefficient blocks of one node.
// ---------------------------------------------------------------------------
struct Blocks {
  double G[5][5], A[5][5], B[5][5], C[5][5], D[5][5];
  double Vxx[5][5], Vxy[5][5], Vyy[5][5], Vxz[5][5], Vyz[5][5], Vzz[5][5];
};

// Material law (getmat.f90:2-37) at temperature t: mu, mu', mu''.
__device__ __forceinline__ void material(int mattyp, double t, double& mu, double& dmu, double& d2mu) {
  if (mattyp == 0) {
    mu = 1.0; dmu = 0.0; d2mu = 0.0;
  } else {
    const double c0 = 1.715336725523065e-05, c1 = 273.0, c2 = 110.4;
    double s = sqrt(t / c1);
    mu = c0 * t / c1 * s * (c1 + c2) / (t + c2);
    dmu = (c0 * (3.0 * c2 + t) * (c2 + c1) * s) / (2.0 * (c2 + t) * (c2 + t) * c1);
    d2mu = (c0 * (3.0 * c2 * c2 - 6.0 * c2 * t - t * t) * (c2 + c1)) / (4.0 * (c2 + t) * (c2 + t) * (c2 + t) * s * c1 * c1);
  }
}

// Coefficient blocks of the linearised compressible Navier-Stokes equations
// for a parallel mean flow (U(y), 0, W(y)) with rho(y), T(y).  `spatial`
// selects the gamma-multiplied energy equation of the spatial solver.
// Mean gradients are wall-normal only: x and z derivatives vanish.
__device__ void node_blocks(const InstDesc& d, const double* nd, bool spatial, Blocks& b) {
  const double gamma = 1.4, gamma1 = 0.4, cp = 1003.1, pt66 = 6.6666666666666666666e-1;
  const double Ma = d.Ma, Re = d.Re, Pr = d.Pr, Te = d.Te;
  const double rho = nd[NODE_VM + 0], U = nd[NODE_VM + 1], W = nd[NODE_VM + 3], T = nd[NODE_VM + 4];
  const double V = spatial ? 0.0 : nd[NODE_VM + 2];  // spatial.f90:147 sets u2m = 0
  // wall-normal gradients of the mean (g2) and second derivatives (g22)
  const double drho = nd[NODE_G2 + 0], dU = nd[NODE_G2 + 1], dV = nd[NODE_G2 + 2], dW = nd[NODE_G2 + 3],
               dT = nd[NODE_G2 + 4];
  const double d2U = nd[NODE_G22 + 1], d2V = nd[NODE_G22 + 2], d2W = nd[NODE_G22 + 3], d2T = nd[NODE_G22 + 4];
  // grad u (velocity i, direction j); only j = y survives
  double gu[3][3] = {{0.0, dU, 0.0}, {0.0, dV, 0.0}, {0.0, dW, 0.0}};
  const double divu = gu[0][0] + gu[1][1] + gu[2][2];
  const double grho[3] = {0.0, drho, 0.0}, gT[3] = {0.0, dT, 0.0};
  const double ig = 1.0 / (gamma * Ma * Ma);
  double gp[3];
  for (int c = 0; c < 3; ++c) gp[c] = ig * (grho[c] * T + rho * gT[c]);
  const double gdiv[3] = {0.0, d2V, 0.0};  // gradient of div u: y-part is d2V
  double S[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) S[i][j] = 0.5 * (gu[i][j] + gu[j][i]);
  // div of the strain-rate tensor per component (the S_ijj terms)
  const double Sjj[3] = {0.5 * d2U, d2V, 0.5 * d2W};
  const double LapT = d2T;
  // material properties, nondimensionalised by their values at Te
  double mue, dmue, d2mue;
  material(d.mattyp, Te, mue, dmue, d2mue);
  const double rmue = mue, cone = mue * cp / Pr, rlme = -pt66 * mue;
  double mu, dmu, d2mu;
  material(d.mattyp, T * Te, mu, dmu, d2mu);
  const double con_d = mu * cp / Pr, dcon_d = dmu * cp / Pr, d2con_d = d2mu * cp / Pr;
  const double rlm_d = -pt66 * mu, dlm_d = -pt66 * dmu, d2lm_d = -pt66 * d2mu;
  const double rmu = mu / rmue, dmun = dmu * Te / rmue, d2mun = d2mu * Te * Te / rmue;
  const double con = con_d / cone, dcon = dcon_d * Te / cone, d2con = d2con_d * Te * Te / cone;
  const double rlm = rlm_d / rlme, dlm = dlm_d * Te / rlme, d2lm = d2lm_d * Te * Te / rlme;
  double gmu[3], gdmu[3], gcon[3], gdcon[3], glm[3], gdlm[3];
  for (int c = 0; c < 3; ++c) {
    gmu[c] = dmun * gT[c]; gdmu[c] = d2mun * gT[c];
    gcon[c] = dcon * gT[c]; gdcon[c] = d2con * gT[c];
    glm[c] = dlm * gT[c]; gdlm[c] = d2lm * gT[c];
  }
  double* all = &b.G[0][0];
  for (int q = 0; q < 11 * 25; ++q) all[q] = 0.0;
  double(*P[3])[5] = {b.A, b.B, b.C};    // convective operators along x, y, z
  const double uvw[3] = {U, V, W};
  const bool nav = !(Re >= 1.0e98 || Re == 0.0);

  // continuity
  b.G[0][0] = 1.0;
  for (int c = 0; c < 3; ++c) { P[c][0][0] = uvw[c]; P[c][0][1 + c] = rho; }
  b.D[0][0] = divu;
  for (int c = 0; c < 3; ++c) b.D[0][1 + c] = grho[c];

  // momentum: equation e = 1 + c carries the pressure gradient along c
  for (int c = 0; c < 3; ++c) {
    const int e = 1 + c;
    b.G[e][e] = rho;
    for (int q = 0; q < 3; ++q) P[q][e][e] = rho * uvw[q];
    P[c][e][0] = T * ig;
    P[c][e][4] = rho * ig;
    b.D[e][0] = U * gu[c][0] + V * gu[c][1] + W * gu[c][2] + gT[c] * ig;
    for (int q = 0; q < 3; ++q) b.D[e][1 + q] = rho * gu[c][q];
    b.D[e][4] = grho[c] * ig;
  }
  if (nav) {
    double(*Vx[3])[5] = {b.Vxx, b.Vxy, b.Vxz};   // second derivatives d/dx d/dc
    double(*Vy[3])[5] = {b.Vxy, b.Vyy, b.Vyz};
    double(*Vz[3])[5] = {b.Vxz, b.Vyz, b.Vzz};
    for (int c = 0; c < 3; ++c) {
      const int e = 1 + c;
      // bulk (lambda) viscosity: d/dc of lambda div u
      const double fl = rlme / (rmue * Re);
      for (int q = 0; q < 3; ++q) P[q][e][1 + q] -= fl * glm[c];
      P[c][e][4] -= fl * dlm * divu;
      b.D[e][4] -= fl * (gdlm[c] * divu + dlm * gdiv[c]);
      // lambda d2/(dc dq) u_q
      double(*Vrow[3])[5] = {Vx[c], Vy[c], Vz[c]};
      for (int q = 0; q < 3; ++q) Vrow[q][e][1 + q] = fl * rlm;
      // shear (mu) viscosity
      const double fm = 1.0 / Re;
      for (int q = 0; q < 3; ++q) {
        // d/dq of mu (du_c/dq + du_q/dc): first-derivative coefficients
        P[q][e][1 + c] -= fm * gmu[q];
        P[c][e][1 + q] -= fm * gmu[q];
        P[q][e][4] -= fm * dmun * 2.0 * S[c][q];
      }
      b.D[e][4] -= fm * 2.0 * (gdmu[0] * S[c][0] + gdmu[1] * S[c][1] + gdmu[2] * S[c][2] + dmun * Sjj[c]);
      // mu (d2 u_c/dq dq + d2 u_q/dc dq)
      b.Vxx[e][e] += fm * rmu; b.Vyy[e][e] += fm * rmu; b.Vzz[e][e] += fm * rmu;
      for (int q = 0; q < 3; ++q) Vrow[q][e][1 + q] += fm * rmu;
    }
  }
  // energy
  if (!spatial) {
    b.G[4][0] = -gamma1 * T / gamma;
    b.G[4][4] = rho / gamma;
    for (int c = 0; c < 3; ++c) { P[c][4][0] = -gamma1 * uvw[c] * T / gamma; P[c][4][4] = rho * uvw[c] / gamma; }
    b.D[4][0] = 1.0 / gamma * (U * gT[0] + V * gT[1] + W * gT[2]);
    for (int c = 0; c < 3; ++c) b.D[4][1 + c] = rho * gT[c] - gamma1 * Ma * Ma * gp[c];
    b.D[4][4] = -gamma1 / gamma * (U * grho[0] + V * grho[1] + W * grho[2]);
    if (nav) {
      double f = 1.0 / (Pr * Re);
      for (int c = 0; c < 3; ++c) P[c][4][4] -= f * (gcon[c] + dcon * gT[c]);
      b.D[4][4] -= f * (gdcon[0] * gT[0] + gdcon[1] * gT[1] + gdcon[2] * gT[2] + dcon * LapT);
      b.Vxx[4][4] = f * con; b.Vyy[4][4] = f * con; b.Vzz[4][4] = f * con;
      f = gamma1 * Ma * Ma * rlme / (Re * rmue);
      for (int c = 0; c < 3; ++c) P[c][4][1 + c] -= f * 2.0 * rlm * divu;
      b.D[4][4] -= f * dlm * divu * divu;
      f = 2.0 * gamma1 * Ma * Ma / Re;
      double ss = 0.0;
      for (int c = 0; c < 3; ++c)
        for (int q = 0; q < 3; ++q) { P[q][4][1 + c] -= f * 2.0 * rmu * S[c][q]; ss += S[c][q] * S[c][q]; }
      b.D[4][4] -= f * dmun * ss;
    }
  } else {
    b.G[4][4] = rho;
    for (int c = 0; c < 3; ++c) { P[c][4][1 + c] = rho * gamma1 * T; P[c][4][4] = rho * uvw[c]; }
    b.D[4][0] = U * gT[0] + V * gT[1] + W * gT[2] + gamma1 * T * divu;
    for (int c = 0; c < 3; ++c) b.D[4][1 + c] = rho * gT[c];
    b.D[4][4] = rho * gamma1 * divu;
    if (nav) {
      double f = gamma / (Pr * Re);
      for (int c = 0; c < 3; ++c) P[c][4][4] -= f * (gcon[c] + dcon * gT[c]);
      b.D[4][4] -= f * (gdcon[0] * gT[0] + gdcon[1] * gT[1] + gdcon[2] * gT[2] + dcon * LapT);
      b.Vxx[4][4] = f * con; b.Vyy[4][4] = f * con; b.Vzz[4][4] = f * con;
      f = gamma * gamma1 * Ma * Ma * rlme / (Re * rmue);
      for (int c = 0; c < 3; ++c) P[c][4][1 + c] -= f * 2.0 * rlm * divu;
      b.D[4][4] -= f * dlm * divu * divu;
      f = gamma * gamma1 * Ma * Ma / Re;
      double ss = 0.0;
      for (int c = 0; c < 3; ++c)
        for (int q = 0; q < 3; ++q) { P[q][4][1 + c] -= f * 4.0 * rmu * S[c][q]; ss += S[c][q] * S[c][q]; }
      b.D[4][4] -= f * 2.0 * dmun * ss;
    }
  }
}

// The spatial blocks on a curved wall, spatial.f90:230-673 term by term,
// with the metric h of the wall at this node and its derivatives
// (dh/ds, dh/dr, d2h/dsdr, d2h/dr2).  The parallel mean has u2m = 0 and no
// streamwise or spanwise gradients (spatial.f90:147, 167-185), so of the
// reference's mean-gradient arrays only the y derivatives survive.
__device__ void node_blocks_curved(const InstDesc& d, const double* nd, double h, double dhds, double dhdr,
                                   double dhdsr, double dhdrr, Blocks& b) {
  const double gamma = 1.4, gamma1 = 0.4, cp = 1003.1, pt66 = 6.6666666666666666666e-1;
  const double Ma = d.Ma, Re = d.Re, Pr = d.Pr, Te = d.Te;
  const double rhom = nd[NODE_VM + 0], u1m = nd[NODE_VM + 1], u3m = nd[NODE_VM + 3], tm = nd[NODE_VM + 4];
  const double u2m = 0.0;
  // gum[i][j] = d u_i / d x_j: only j = y (index 1) of u and w
  double gum[3][3] = {{0.0, nd[NODE_G2 + 1], 0.0}, {0.0, nd[NODE_G2 + 2], 0.0}, {0.0, nd[NODE_G2 + 3], 0.0}};
  const double g22u = nd[NODE_G22 + 1], g22v = nd[NODE_G22 + 2], g22w = nd[NODE_G22 + 3], g22t = nd[NODE_G22 + 4];
  const double grhom[3] = {0.0, nd[NODE_G2 + 0], 0.0}, gtm[3] = {0.0, nd[NODE_G2 + 4], 0.0};
  const double h2 = h * h, h3 = h2 * h;
  const double divum = (gum[0][0] + u2m * dhdr) / h + gum[1][1] + gum[2][2];
  const double g1divum = -dhds / h3 * (gum[0][0] + u2m * dhdr) + 1.0 / h2 * (gum[1][0] * dhdr + u2m * dhdsr);
  const double g2divum = -dhdr / h2 * (gum[0][0] + u2m * dhdr) + 1.0 / h * (gum[1][1] * dhdr + u2m * dhdrr) + g22v;
  const double g3divum = 1.0 / h * (gum[1][2] * dhdr);
  double S[3][3];
  S[0][0] = (gum[0][0] + u2m * dhdr) / h;
  S[0][1] = 0.5 * ((gum[1][0] - u1m * dhdr) / h + gum[0][1]);
  S[0][2] = 0.5 * (gum[2][0] / h + gum[0][2]);
  S[1][0] = S[0][1];
  S[1][1] = gum[1][1];
  S[1][2] = 0.5 * (gum[2][1] + gum[1][2]);
  S[2][0] = S[0][2];
  S[2][1] = S[1][2];
  S[2][2] = gum[2][2];
  const double S1jj = -0.5 * (dhdr * dhdr + dhdrr * h) / h2 * u1m + 0.5 * dhdr * gum[0][1] / h + 0.5 * g22u -
                      dhds * gum[0][0] / h3 + (h * dhdsr - dhdr * dhds) / h3 * u2m +
                      3.0 * dhdr * gum[1][0] / (2.0 * h2);
  const double S2jj = 0.5 * (dhdr * dhds - h * dhdsr) / h3 * u1m - 3.0 * dhdr * gum[0][0] / (2.0 * h2) -
                      dhdr * dhdr * u2m / h2 + dhdr * gum[1][1] / h + g22v - 0.5 * dhds * gum[1][0] / h3;
  const double S3jj = 0.5 * dhdr * gum[1][2] / h + 0.5 * dhdr * gum[2][1] / h + 0.5 * g22w -
                      0.5 * dhds * gum[2][0] / h3;
  const double LapT = 1.0 / h * (-dhds / h2 * gtm[0] + h * g22t + gtm[1] * dhdr);
  double mue, dmue, d2mue;
  material(d.mattyp, Te, mue, dmue, d2mue);
  const double rmue = mue, cone = mue * cp / Pr, rlme = -pt66 * mue;
  double mu, dmu0, d2mu0;
  material(d.mattyp, tm * Te, mu, dmu0, d2mu0);
  const double rmu = mu / rmue, dmu = dmu0 * Te / rmue, d2mu = d2mu0 * Te * Te / rmue;
  const double con = mu * cp / Pr / cone, dcon = dmu0 * cp / Pr * Te / cone, d2con = d2mu0 * cp / Pr * Te * Te / cone;
  const double rlm = -pt66 * mu / rlme, dlm = -pt66 * dmu0 * Te / rlme, d2lm = -pt66 * d2mu0 * Te * Te / rlme;
  double g1mu = dmu * gtm[0], g2mu = dmu * gtm[1], g3mu = dmu * gtm[2];
  double g1dmu = d2mu * gtm[0], g2dmu = d2mu * gtm[1], g3dmu = d2mu * gtm[2];
  double g1con = dcon * gtm[0], g2con = dcon * gtm[1], g3con = dcon * gtm[2];
  double g1dcon = d2con * gtm[0], g2dcon = d2con * gtm[1], g3dcon = d2con * gtm[2];
  double g1lm = dlm * gtm[0], g2lm = dlm * gtm[1], g3lm = dlm * gtm[2];
  double g1dlm = d2lm * gtm[0], g2dlm = d2lm * gtm[1], g3dlm = d2lm * gtm[2];
  const double gM2 = gamma * Ma * Ma;
  const bool nav = !(Re >= 1.0e98 || Re == 0.0);
  double* all = &b.G[0][0];
  for (int q = 0; q < 11 * 25; ++q) all[q] = 0.0;
  auto &G = b.G, &A = b.A, &B = b.B, &C = b.C, &D = b.D;
  auto &Vxx = b.Vxx, &Vxy = b.Vxy, &Vyy = b.Vyy, &Vxz = b.Vxz, &Vyz = b.Vyz, &Vzz = b.Vzz;
  // continuity (spatial.f90:356-371)
  G[0][0] = 1.0;
  A[0][0] = u1m / h; A[0][1] = rhom / h;
  B[0][0] = u2m; B[0][2] = rhom;
  C[0][0] = u3m; C[0][3] = rhom;
  D[0][0] = divum; D[0][1] = grhom[0] / h; D[0][2] = grhom[1] + rhom * dhdr / h; D[0][3] = grhom[2];
  // x_1 momentum (spatial.f90:375-455)
  G[1][1] = rhom;
  A[1][0] = tm / (h * gM2); A[1][1] = rhom * u1m / h; A[1][4] = rhom / (h * gM2);
  B[1][1] = rhom * u2m;
  C[1][1] = rhom * u3m;
  D[1][0] = u1m / h * (gum[0][0] + u2m * dhdr) + u2m * gum[0][1] + u3m * gum[0][2] + gtm[0] / (h * gM2);
  D[1][1] = rhom * (gum[0][0] + u2m * dhdr) / h;
  D[1][2] = rhom * (gum[0][1] + u1m * dhdr / h);
  D[1][3] = rhom * gum[0][2];
  D[1][4] = grhom[0] / (h * gM2);
  if (nav) {
    double f = rlme / (rmue * Re);
    A[1][1] -= f * (g1lm / h2 - rlm / h3 * dhds);
    A[1][2] -= f * rlm / h2 * dhdr;
    A[1][4] -= f * dlm * divum / h;
    B[1][2] -= f * (g1lm / h);
    C[1][3] -= f * (g1lm / h);
    D[1][2] -= f * (g1lm * dhdr / h2 - rlm / h3 * dhds * dhdr + rlm / h2 * dhdsr);
    D[1][4] -= f * (g1dlm * divum / h + dlm * g1divum);
    Vxx[1][1] = f * rlm / h2;
    Vxy[1][2] = f * rlm / h;
    Vxz[1][3] = f * rlm / h;
    f = 1.0 / Re;
    A[1][1] -= f * (2.0 * g1mu / h2 - 2.0 * rmu * dhds / h3);
    A[1][2] -= f * (g2mu / h + rmu * 3.0 * dhdr / h2);
    A[1][3] -= f * g3mu / h;
    A[1][4] -= f * dmu * 2.0 * S[0][0] / h;
    B[1][1] -= f * (g2mu + rmu * dhdr / h);
    B[1][4] -= f * dmu * 2.0 * S[0][1];
    C[1][1] -= f * g3mu;
    C[1][4] -= f * dmu * 2.0 * S[0][2];
    D[1][1] -= f * (g2mu / h * (-dhdr) - rmu * (dhdr * dhdr + dhdrr * h) / h2);
    D[1][2] -= f * (2.0 * g1mu / h2 * dhdr + 2.0 * rmu * (dhdsr * h - dhds * dhdr) / h3);
    D[1][4] -= f * 2.0 * (g1dmu / h * S[0][0] + g2dmu * S[0][1] + g3dmu * S[0][2] + dmu * S1jj);
    Vxx[1][1] += f * 2.0 * rmu / h2;
    Vxy[1][2] += f * rmu / h;
    Vyy[1][1] += f * rmu;
    Vxz[1][3] += f * rmu / h;
    Vzz[1][1] += f * rmu;
  }
  // x_2 momentum (spatial.f90:459-541)
  G[2][2] = rhom;
  A[2][2] = rhom * u1m / h;
  B[2][0] = tm / gM2; B[2][2] = rhom * u2m; B[2][4] = rhom / gM2;
  C[2][2] = rhom * u3m;
  D[2][0] = u1m / h * (gum[1][0] - u1m * dhdr) + u2m * gum[1][1] + u3m * gum[1][2] + gtm[1] / gM2;
  D[2][1] = rhom * (gum[1][0] - 2.0 * u1m * dhdr) / h;
  D[2][2] = rhom * gum[1][1];
  D[2][3] = rhom * gum[1][2];
  D[2][4] = grhom[1] / gM2;
  if (nav) {
    double f = rlme / (rmue * Re);
    A[2][1] -= f * (g2lm / h - rlm * dhdr / h2);
    B[2][2] -= f * (g2lm + rlm * dhdr / h);
    B[2][4] -= f * dlm * divum;
    C[2][3] -= f * g2lm;
    D[2][2] -= f * (g2lm / h * dhdr - rlm * dhdr / h2 * dhdr + rlm / h * dhdrr);
    D[2][4] -= f * (g2dlm * divum + dlm * g2divum);
    Vxy[2][1] = f * rlm / h;
    Vyy[2][2] = f * rlm;
    Vyz[2][3] = f * rlm;
    f = 1.0 / Re;
    A[2][1] += f * rmu * 3.0 * dhdr / h2;
    A[2][2] -= f * (g1mu / h2 - rmu * dhds / h3);
    A[2][4] -= f * dmu * 2.0 * S[1][0] / h;
    B[2][1] -= f * g1mu / h;
    B[2][2] -= f * (2.0 * g2mu + 2.0 * rmu * dhdr / h);
    B[2][3] -= f * g3mu;
    B[2][4] -= f * dmu * 2.0 * S[1][1];
    C[2][2] -= f * g3mu;
    C[2][4] -= f * dmu * 2.0 * S[1][2];
    D[2][1] -= f * (g1mu / h2 * (-dhdr) + rmu * (dhds * dhdr - h * dhdsr) / h3);
    D[2][2] += f * 2.0 * rmu * dhdr * dhdr / h2;
    D[2][4] -= f * 2.0 * (g1dmu / h * S[1][0] + g2dmu * S[1][1] + g3dmu * S[1][2] + dmu * S2jj);
    Vxx[2][2] += f * rmu / h2;
    Vxy[2][1] += f * rmu / h;
    Vyy[2][2] += f * 2.0 * rmu;
    Vyz[2][3] += f * rmu;
    Vzz[2][2] += f * rmu;
  }
  // x_3 momentum (spatial.f90:545-597)
  G[3][3] = rhom;
  A[3][3] = rhom * u1m / h;
  B[3][3] = rhom * u2m;
  C[3][0] = tm / gM2; C[3][3] = rhom * u3m; C[3][4] = rhom / gM2;
  D[3][0] = u1m * gum[2][0] / h + u2m * gum[2][1] + u3m * gum[2][2] + gtm[2] / gM2;
  D[3][1] = rhom * gum[2][0] / h;
  D[3][2] = rhom * gum[2][1];
  D[3][3] = rhom * gum[2][2];
  D[3][4] = grhom[2] / gM2;
  if (nav) {
    double f = rlme / (rmue * Re);
    A[3][1] -= f * g3lm / h;
    B[3][2] -= f * g3lm;
    C[3][3] -= f * g3lm;
    C[3][2] -= f * rlm / h * dhdr;
    C[3][4] -= f * dlm * divum;
    D[3][2] -= f * (g2lm / h * dhdr);
    D[3][4] -= f * (g3dlm * divum + dlm * g3divum);
    Vxz[3][1] = f * rlm / h;
    Vyz[3][2] = f * rlm;
    Vzz[3][3] = f * rlm;
    f = 1.0 / Re;
    A[3][3] -= f * (g1mu / h2 - rmu * dhds / h3);
    A[3][4] -= f * dmu * 2.0 * S[2][0] / h;
    B[3][3] -= f * (g2mu + rmu * dhdr / h);
    B[3][4] -= f * dmu * 2.0 * S[2][1];
    C[3][1] -= f * g1mu / h;
    C[3][2] -= f * (g2mu + rmu * dhdr / h);
    C[3][3] -= f * 2.0 * g3mu;
    C[3][4] -= f * dmu * 2.0 * S[2][2];
    D[3][4] -= f * 2.0 * (g1dmu / h * S[2][0] + g2dmu * S[2][1] + g3dmu * S[2][2] + dmu * S3jj);
    Vxx[3][3] += f * rmu / h2;
    Vyy[3][3] += f * rmu;
    Vxz[3][1] += f * rmu / h;
    Vyz[3][2] += f * rmu;
    Vzz[3][3] += f * 2.0 * rmu;
  }
  // energy (spatial.f90:601-673)
  G[4][4] = rhom;
  A[4][1] = rhom * gamma1 * tm / h; A[4][4] = rhom * u1m / h;
  B[4][2] = rhom * gamma1 * tm; B[4][4] = rhom * u2m;
  C[4][3] = rhom * gamma1 * tm; C[4][4] = rhom * u3m;
  D[4][0] = u1m / h * gtm[0] + u2m * gtm[1] + u3m * gtm[2] + gamma1 * tm * divum;
  D[4][1] = rhom * gtm[0] / h;
  D[4][2] = rhom * gtm[1] + rhom * gamma1 * tm * dhdr / h;
  D[4][3] = rhom * gtm[2];
  D[4][4] = rhom * gamma1 * divum;
  if (nav) {
    double f = gamma / (Pr * Re);
    A[4][4] -= f * (g1con / h2 + dcon * gtm[0] / h2 - con * dhds / h3);
    B[4][4] -= f * (g2con + dcon * gtm[1] + con * dhdr / h);
    C[4][4] -= f * (g3con + dcon * gtm[2]);
    D[4][4] -= f * (g1dcon * gtm[0] / h2 + g2dcon * gtm[1] + g3dcon * gtm[2] + dcon * LapT);
    Vxx[4][4] = f * con / h2;
    Vyy[4][4] = f * con;
    Vzz[4][4] = f * con;
    f = gamma * gamma1 * Ma * Ma * rlme / (Re * rmue);
    A[4][1] -= f * 2.0 * rlm * divum / h;
    B[4][2] -= f * 2.0 * rlm * divum;
    C[4][3] -= f * 2.0 * rlm * divum;
    D[4][2] -= f * 2.0 * rlm * divum * dhdr / h;
    D[4][4] -= f * dlm * divum * divum;
    f = gamma * gamma1 * Ma * Ma / Re;
    for (int c = 0; c < 3; ++c) {
      A[4][1 + c] -= f * 4.0 * rmu * S[c][0] / h;
      B[4][1 + c] -= f * 4.0 * rmu * S[c][1];
      C[4][1 + c] -= f * 4.0 * rmu * S[c][2];
    }
    D[4][1] += f * 4.0 * rmu * S[1][0] * dhdr / h;
    D[4][2] -= f * 4.0 * rmu * S[0][0] * dhdr / h;
    double ss = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) ss += S[i][j] * S[i][j];
    D[4][4] -= f * 2.0 * dmu * ss;
  }
}

// 5x5 complex inverse by Gauss-Jordan with partial pivoting (B0 blocks)
__device__ bool inv5(const zc in[5][5], zc out[5][5]) {
  zc a[5][10];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) { a[i][j] = in[i][j]; a[i][5 + j] = zmk(i == j ? 1.0 : 0.0, 0.0); }
  for (int c = 0; c < 5; ++c) {
    int p = c;
    double best = zabs1(a[c][c]);
    for (int r = c + 1; r < 5; ++r)
      if (zabs1(a[r][c]) > best) { best = zabs1(a[r][c]); p = r; }
    if (best == 0.0) return false;
    if (p != c)
      for (int j = 0; j < 10; ++j) { zc t = a[c][j]; a[c][j] = a[p][j]; a[p][j] = t; }
    zc piv = a[c][c];
    for (int j = 0; j < 10; ++j) a[c][j] = zdiv(a[c][j], piv);
    for (int r = 0; r < 5; ++r) {
      if (r == c) continue;
      zc f = a[r][c];
      if (f.x == 0.0 && f.y == 0.0) continue;
      for (int j = 0; j < 10; ++j) a[r][j] = zsub(a[r][j], zmul(f, a[c][j]));
    }
  }
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) out[i][j] = a[i][5 + j];
  return true;
}

// ---------------------------------------------------------------------------
// Operator blocks per node.  Row block i of each dense operator is
//   P1 (x) D1(i,:) - P2 (x) D2(i,:) + delta_ij P3
// with 5x5 complex P's.  Temporal (itype 1): blk = {P1, P2, P3} of A0, the
// B0 diagonal block, and B0^-1.  Spatial (itype 2): {P1, P2, P3} of C0,
// {P1, P3} of C1, and P3 of C2.  One thread per node.
// ---------------------------------------------------------------------------
__global__ void k_blocks(int count, const InstDesc* __restrict__ desc, const double* const* __restrict__ dtab,
                         const double* __restrict__ node, zc* __restrict__ blk, int* __restrict__ flags) {
  int k = blockIdx.y;
  if (k >= count) return;
  const InstDesc d = desc[k];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.ny) return;
  const int ny = d.ny;
  const bool spatial = (d.itype == 2);
  const double* nd = node + d.off_node + (size_t)NODE_STRIDE * i;
  const double deta = nd[NODE_DETA], d2eta = nd[NODE_D2ETA];
  const double* D1 = dtab[2 * d.dmat];
  const double dww = D1[(size_t)(ny - 1) * ny + (ny - 1)];   // D1(wall, wall), for the adiabatic row
  Blocks b;
  if (spatial && d.curved) {
    // the circle's metric at this node's distance r = y from the wall
    // (circh.f90:190-199)
    const double r = nd[NODE_Y];
    const double* w = d.cw;
    const double a = w[0] + r * w[2], bb = w[1] + r * w[3];
    const double h = sqrt(a * a + bb * bb);
    const double dads = w[4] + r * w[6], dbds = w[5] + r * w[7];
    const double dhds = (a * dads + bb * dbds) / h;
    const double dhdr = (a * w[2] + bb * w[3]) / h;
    const double dhdrr = (-dhdr * dhdr + w[2] * w[2] + w[3] * w[3]) / h;
    const double dhdsr = -dhds / (h * h) * (a * w[2] + bb * w[3]) + (dads * w[2] + a * w[6] + dbds * w[3] + bb * w[7]) / h;
    node_blocks_curved(d, nd, h, dhds, dhdr, dhdsr, dhdrr, b);
  } else {
    node_blocks(d, nd, spatial, b);
  }
  const zc I = zmk(0.0, 1.0);
  // Chebyshev nodes run from the free stream to the wall, the
  // finite-difference ones from the wall
  const bool top_node = d.fd ? (i == ny - 1) : (i == 0), wall_node = d.fd ? (i == 0) : (i == ny - 1);
  zc* out = blk + d.off_blk + (size_t)BLK_STRIDE * i;
  zc P1[5][5], P2[5][5], P3[5][5];
  const zc z0 = zmk(0.0, 0.0);
  for (int e = 0; e < 5; ++e)
    for (int v = 0; v < 5; ++v) { P1[e][v] = z0; P2[e][v] = z0; P3[e][v] = z0; }
  if (!spatial) {
    const zc al = zmk(d.ar, d.ai), be = zmk(d.br, d.bi);
    const zc ia = zmul(I, al), ib = zmul(I, be);
    const zc a2 = zmul(al, al), ab = zmul(al, be), b2 = zmul(be, be);
    zc Dh[5][5], Bh[5][5];
    double Vy[5][5];
    for (int e = 0; e < 5; ++e)
      for (int v = 0; v < 5; ++v) {
        zc t = zmk(b.D[e][v], 0.0);
        t = zadd(t, zscale(ia, b.A[e][v]));
        t = zadd(t, zscale(ib, b.C[e][v]));
        t = zadd(t, zscale(a2, b.Vxx[e][v]));
        t = zadd(t, zscale(ab, b.Vxz[e][v]));
        t = zadd(t, zscale(b2, b.Vzz[e][v]));
        Dh[e][v] = t;
        zc bh = zmk(b.B[e][v], 0.0);
        bh = zsub(bh, zscale(ia, b.Vxy[e][v]));
        bh = zsub(bh, zscale(ib, b.Vyz[e][v]));
        Bh[e][v] = zsub(zscale(bh, deta), zmk(b.Vyy[e][v] * d2eta, 0.0));
        Vy[e][v] = b.Vyy[e][v] * deta * deta;
      }
    zc B0[5][5];
    for (int e = 0; e < 5; ++e)
      for (int v = 0; v < 5; ++v) B0[e][v] = z0;
    if (d.fd && (top_node || wall_node)) {
      // fd_temporal.f90:601-708: free stream B0 = i I, A0 = 0; wall
      // continuity row Dh + F1 Bh, momentum rows B0 = i, A0 = 0, energy row
      // Dh + F1 Bh - F2 Vyy without the temperature column's Bh term, with
      // B0's energy row i G (the wall temperature option is not read)
      for (int e = 0; e < 5; ++e) B0[e][e] = I;
      if (wall_node) {
        for (int v = 0; v < 5; ++v) {
          P1[0][v] = Bh[0][v];
          P3[0][v] = Dh[0][v];
          P1[4][v] = (v < 4) ? Bh[4][v] : z0;
          P2[4][v] = zmk(Vy[4][v], 0.0);
          P3[4][v] = Dh[4][v];
          B0[4][v] = zscale(I, b.G[4][v]);
        }
      }
    } else if (top_node || wall_node) {
      // continuity row only, no Vyy D2 term (temporal.f90:664-681, :706-722)
      for (int v = 0; v < 5; ++v) { P1[0][v] = Bh[0][v]; P3[0][v] = Dh[0][v]; }
      for (int e = 0; e < 5; ++e) B0[e][e] = I;
      if (wall_node && d.wallt == 2) {
        // adiabatic wall energy row (temporal.f90:724-752): the reference pairs
        // Vyy with D1 for the first four variables; temperature uses Dt1, Dt2
        // with Dt1(wall,:) = 0 and Dt2(wall,:) = D2(wall,:) - D1(wall,wall) D1(wall,:).
        for (int v = 0; v < 4; ++v) { P1[4][v] = zsub(Bh[4][v], zmk(Vy[4][v], 0.0)); P3[4][v] = Dh[4][v]; }
        P1[4][4] = zmk(Vy[4][4] * dww, 0.0);
        P2[4][4] = zmk(Vy[4][4], 0.0);
        P3[4][4] = Dh[4][4];
        for (int v = 0; v < 5; ++v) B0[4][v] = zscale(I, b.G[4][v]);
      }
    } else {
      for (int e = 0; e < 5; ++e)
        for (int v = 0; v < 5; ++v) {
          P1[e][v] = Bh[e][v];
          P2[e][v] = zmk(Vy[e][v], 0.0);
          P3[e][v] = Dh[e][v];
          B0[e][v] = zscale(I, b.G[e][v]);
        }
    }
    zc Bi[5][5];
    if (!inv5(B0, Bi)) {
      atomicOr(flags + k, 1);
      for (int e = 0; e < 5; ++e)
        for (int v = 0; v < 5; ++v) Bi[e][v] = z0;
    }
    for (int e = 0; e < 5; ++e)
      for (int v = 0; v < 5; ++v) {
        out[0 * 25 + e * 5 + v] = P1[e][v];
        out[1 * 25 + e * 5 + v] = P2[e][v];
        out[2 * 25 + e * 5 + v] = P3[e][v];
        out[3 * 25 + e * 5 + v] = B0[e][v];
        out[4 * 25 + e * 5 + v] = Bi[e][v];
        out[5 * 25 + e * 5 + v] = z0;
      }
  } else {
    const zc om = zmk(d.wr, d.wi), be = zmk(d.br, d.bi);
    const zc ib = zmul(I, be), b2 = zmul(be, be), iom = zmul(I, om);
    zc Dh0[5][5], Bh0[5][5], Dh1[5][5], Bh1[5][5];
    double Vy[5][5];
    for (int e = 0; e < 5; ++e)
      for (int v = 0; v < 5; ++v) {
        zc t = zmk(b.D[e][v], 0.0);
        t = zadd(t, zscale(ib, b.C[e][v]));
        t = zadd(t, zscale(b2, b.Vzz[e][v]));
        Dh0[e][v] = t;
        zc bh = zsub(zmk(b.B[e][v], 0.0), zscale(ib, b.Vyz[e][v]));
        Bh0[e][v] = zsub(zscale(bh, deta), zmk(b.Vyy[e][v] * d2eta, 0.0));
        Vy[e][v] = b.Vyy[e][v] * deta * deta;
        Dh1[e][v] = zadd(zscale(I, b.A[e][v]), zscale(be, b.Vxz[e][v]));
        Bh1[e][v] = zscale(zmk(0.0, -b.Vxy[e][v]), deta);
      }
    zc Q1[5][5], Q3[5][5], R3[5][5];  // C1 (P1, P3) and C2 (P3)
    for (int e = 0; e < 5; ++e)
      for (int v = 0; v < 5; ++v) { Q1[e][v] = z0; Q3[e][v] = z0; R3[e][v] = z0; }
    if (top_node) {
      if (d.top == 1) {
        for (int v = 0; v < 5; ++v) { P1[0][v] = Bh0[0][v]; P3[0][v] = Dh0[0][v]; Q1[0][v] = Bh1[0][v]; Q3[0][v] = Dh1[0][v]; }
        P3[0][0] = zsub(P3[0][0], iom);
      } else {
        P3[0][0] = zmk(-1.0, 0.0);   // zero density at infinity (spatial.f90:797)
      }
      for (int e = 1; e < 5; ++e) P3[e][e] = zmk(-1.0, 0.0);
    } else if (wall_node) {
      for (int v = 0; v < 5; ++v) { P1[0][v] = Bh0[0][v]; P3[0][v] = Dh0[0][v]; Q1[0][v] = Bh1[0][v]; Q3[0][v] = Dh1[0][v]; }
      P3[0][0] = zsub(P3[0][0], iom);
      for (int e = 1; e < 4; ++e) P3[e][e] = zmk(-1.0, 0.0);
      if (d.fd && d.wallt == 2) {
        // fd_spatial.f90:697-750, 994-1025, 1164-1171: the wall energy row,
        // its temperature column without the first-derivative term, and
        // the -i omega G term taken from the G of the node the assembly
        // loops leave behind (ny-1 with top = 1, else ny-2, 0-based here)
        Blocks bq;
        const int gq = (d.top == 1) ? ny - 1 : ny - 2;
        node_blocks(d, node + d.off_node + (size_t)NODE_STRIDE * gq, true, bq);
        for (int v = 0; v < 5; ++v) {
          P1[4][v] = (v < 4) ? Bh0[4][v] : z0;
          P2[4][v] = zmk(Vy[4][v], 0.0);
          P3[4][v] = zsub(Dh0[4][v], zscale(iom, bq.G[4][v]));
          Q1[4][v] = (v < 4) ? Bh1[4][v] : z0;
          Q3[4][v] = Dh1[4][v];
          R3[4][v] = zmk(b.Vxx[4][v], 0.0);
        }
      } else if (d.wallt == 2) {
        for (int v = 0; v < 4; ++v) {
          P1[4][v] = Bh0[4][v]; P2[4][v] = zmk(Vy[4][v], 0.0); P3[4][v] = Dh0[4][v];
          Q1[4][v] = Bh1[4][v]; Q3[4][v] = Dh1[4][v];
        }
        P1[4][4] = zmk(Vy[4][4] * dww, 0.0);
        P2[4][4] = zmk(Vy[4][4], 0.0);
        P3[4][4] = Dh0[4][4];
        Q3[4][4] = Dh1[4][4];
        for (int v = 0; v < 5; ++v) { P3[4][v] = zsub(P3[4][v], zscale(iom, b.G[4][v])); R3[4][v] = zmk(b.Vxx[4][v], 0.0); }
      } else {
        P3[4][4] = zmk(-1.0, 0.0);
      }
    } else {
      for (int e = 0; e < 5; ++e)
        for (int v = 0; v < 5; ++v) {
          P1[e][v] = Bh0[e][v];
          P2[e][v] = zmk(Vy[e][v], 0.0);
          P3[e][v] = zsub(Dh0[e][v], zscale(iom, b.G[e][v]));
          Q1[e][v] = Bh1[e][v];
          Q3[e][v] = Dh1[e][v];
          R3[e][v] = zmk(b.Vxx[e][v], 0.0);
        }
    }
    for (int e = 0; e < 5; ++e)
      for (int v = 0; v < 5; ++v) {
        out[0 * 25 + e * 5 + v] = P1[e][v];
        out[1 * 25 + e * 5 + v] = P2[e][v];
        out[2 * 25 + e * 5 + v] = P3[e][v];
        out[3 * 25 + e * 5 + v] = Q1[e][v];
        out[4 * 25 + e * 5 + v] = Q3[e][v];
        out[5 * 25 + e * 5 + v] = R3[e][v];
      }
  }
}

}  // namespace stab
