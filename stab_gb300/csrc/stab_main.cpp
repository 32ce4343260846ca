// `stab` drop-in for the Chebyshev temporal and spatial paths: reads the
// reference's stdin protocol (input.f90:15-123, stab.f90:46-55), the mean
// flow from profile.<ind> in the working directory, solves on the GPU and
// writes evec.dat as temporal.f90:883-890 / spatial.f90:1120-1126 do.
// The multi-point drivers (itype 7, mtemporal.f90; itype 8, mspatial.f90
// with delta.dat) solve every sweep point in one batch and write each
// point's eigensystem to eig.<iver>, as the drivers' temporal('eig.<iver>')
// / spatial('eig.<iver>') calls do.
//
//   stab_gpu [-d device] [-o evec.dat] < input.dat
//
// The eigenvalues are written sorted by imaginary part (the PIKSR2 order);
// R5 holds every eigenvector (temporal always, spatial with ievec = 1).
// Prints the least-stable eigenvalue; exits non-zero on any error.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iterator>
#include <string>
#include <vector>
#include <iostream>

#include "stab_gb300.h"

static int fail(const char* what, int rc, stab_ctx* ctx) {
  std::fprintf(stderr, "stab_gpu: %s failed (%d)%s%s\n", what, rc, ctx ? ": " : "", ctx ? stab_last_error(ctx) : "");
  if (ctx) stab_destroy(ctx);
  return 1;
}

static bool read_table(const std::string& name, std::vector<double>& rows, int32_t& nym) {
  nym = 0;
  if (stab_read_profile(name.c_str(), 0, nullptr, &nym)) {
    std::fprintf(stderr, "stab_gpu: cannot read %s\n", name.c_str());
    return false;
  }
  rows.assign(6 * (size_t)nym, 0.0);
  if (stab_read_profile(name.c_str(), nym, rows.data(), &nym)) {
    std::fprintf(stderr, "stab_gpu: cannot read %s\n", name.c_str());
    return false;
  }
  return true;
}

// profile.<ind>; with ider = 0 also first.<ind> and second.<ind>
// (getmean2.f90:27, 103, 146: nym rows each, the profile's count), packed
// as rows of 18 values
static bool load_profile(int32_t ind, int32_t ider, std::vector<double>& prof, int32_t& nym) {
  char pname[64];
  stab_profile_name(ind, pname, sizeof(pname));
  if (!read_table(pname, prof, nym)) return false;
  if (ider != 0) return true;
  std::vector<double> t[2];
  for (int q = 0; q < 2; ++q) {
    int32_t n2 = 0;
    const std::string name = std::string(q == 0 ? "first." : "second.") + std::to_string(ind);
    if (!read_table(name, t[q], n2)) return false;
    if (n2 < nym) {
      std::fprintf(stderr, "stab_gpu: %s has %d rows, the profile %d\n", name.c_str(), n2, nym);
      return false;
    }
  }
  std::vector<double> rows(18 * (size_t)nym);
  for (int32_t r = 0; r < nym; ++r)
    for (int f = 0; f < 6; ++f) {
      rows[18 * (size_t)r + f] = prof[6 * (size_t)r + f];
      rows[18 * (size_t)r + 6 + f] = t[0][6 * (size_t)r + f];
      rows[18 * (size_t)r + 12 + f] = t[1][6 * (size_t)r + f];
    }
  prof.swap(rows);
  return true;
}

// itype 7 / 8: every point of the sweep in one batch of the plain FP64
// path, then each point's eigensystem to eig.<iver>
static int run_sweep(const stab_params& base, const stab_sweep& sw, int device) {
  std::vector<double> xb, delta;
  int32_t nbody = 0;
  if (sw.itype == 8) {
    if (stab_read_delta("delta.dat", 0, nullptr, nullptr, &nbody) || nbody < 1) {
      std::fprintf(stderr, "stab_gpu: cannot read delta.dat\n");
      return 1;
    }
    xb.resize(nbody);
    delta.resize(nbody);
    stab_read_delta("delta.dat", nbody, xb.data(), delta.data(), &nbody);
    if (sw.ind1 < 1 || sw.ind2 > nbody) {
      std::fprintf(stderr, "ERROR: illegal index...check delta.dat\n");   // mspatial.f90:45-49
      return 1;
    }
  }
  int32_t np = 0;
  if (stab_sweep_points(&base, &sw, nbody, xb.data(), delta.data(), 0, nullptr, &np) || np < 1) {
    std::fprintf(stderr, "stab_gpu: empty or invalid sweep\n");
    return 1;
  }
  std::vector<stab_params> pts(np);
  stab_sweep_points(&base, &sw, nbody, xb.data(), delta.data(), np, pts.data(), &np);
  // one profile per distinct index
  std::vector<std::vector<double>> profs;
  std::vector<int32_t> pind, pnym;
  std::vector<const double*> pp(np);
  std::vector<int32_t> nyms(np);
  for (int k = 0; k < np; ++k) {
    int slot = -1;
    for (size_t q = 0; q < pind.size(); ++q)
      if (pind[q] == pts[k].ind) slot = (int)q;
    if (slot < 0) {
      std::vector<double> pr;
      int32_t nym = 0;
      if (!load_profile(pts[k].ind, pts[k].ider, pr, nym)) return 1;
      profs.push_back(std::move(pr));
      pind.push_back(pts[k].ind);
      pnym.push_back(nym);
      slot = (int)profs.size() - 1;
    }
    nyms[k] = pnym[slot];
  }
  for (int k = 0; k < np; ++k)
    for (size_t q = 0; q < pind.size(); ++q)
      if (pind[q] == pts[k].ind) pp[k] = profs[q].data();
  stab_ctx* ctx = nullptr;
  int rc = stab_create(&ctx, device);
  if (rc) return fail("stab_create", rc, nullptr);
  stab_batch* b = nullptr;
  rc = stab_batch_create(ctx, np, pts.data(), nyms.data(), pp.data(), &b);
  if (rc) return fail("stab_batch_create", rc, ctx);
  rc = stab_batch_run(b, STAB_MODE_PLAIN);
  if (rc) return fail("stab_batch_run", rc, ctx);
  std::vector<std::vector<double>> eig(np);
  std::vector<double*> ep(np);
  for (int k = 0; k < np; ++k) {
    eig[k].assign(2 * (size_t)(pts[k].itype == 1 ? 5 : 10) * pts[k].ny, 0.0);
    ep[k] = eig[k].data();
  }
  rc = stab_batch_spectra(b, ep.data());
  if (rc) return fail("stab_batch_spectra", rc, ctx);
  std::vector<double> least(2 * (size_t)np);
  std::vector<int32_t> st(np);
  rc = stab_batch_results(b, least.data(), nullptr, nullptr, st.data(), nullptr);
  if (rc) return fail("stab_batch_results", rc, ctx);
  stab_batch_destroy(b);
  for (int k = 0; k < np; ++k) {
    const stab_params& q = pts[k];
    const int64_t m = (int64_t)(q.itype == 1 ? 5 : 10) * q.ny;
    std::vector<double> vec;
    const bool want_vec = (q.itype == 1 || q.ievec == 1);
    if (want_vec) {
      vec.resize(2 * m * m);
      std::vector<int32_t> vs(m);
      rc = stab_eigenvectors(ctx, &q, nyms[k], pp[k], (int32_t)m, eig[k].data(), vec.data(), vs.data());
      if (rc) return fail("stab_eigenvectors", rc, ctx);
    }
    char name[64];
    stab_eig_name(k + 1, name, sizeof(name));
    stab_params qw = q;
    if (qw.itype == 2 && qw.curve == 2 && qw.x != -1.0) qw.x = 0.0;   // circh.f90:60
    rc = stab_write_evec(name, &qw, eig[k].data(), want_vec ? vec.data() : nullptr);
    if (rc) return fail("stab_write_evec", rc, ctx);
    if (q.itype == 1)
      std::printf("%4d  alpha = (%.6e, %.6e)  beta = (%.6e, %.6e)  least-stable omega = (%.15e, %.15e)  status %d  "
                  "-> %s\n", k + 1, q.alpha[0], q.alpha[1], q.beta[0], q.beta[1], least[2 * k], least[2 * k + 1],
                  st[k], name);
    else
      std::printf("%4d  ind %d  x = %.6e  Yi = %.6e  omega = (%.6e, %.6e)  beta = (%.6e, %.6e)  least-stable alpha = "
                  "(%.15e, %.15e)  status %d  -> %s\n", k + 1, q.ind, q.x, q.yi, q.omega[0], q.omega[1], q.beta[0],
                  q.beta[1], least[2 * k], least[2 * k + 1], st[k], name);
  }
  stab_destroy(ctx);
  return 0;
}

int main(int argc, char** argv) {
  int device = 0;
  std::string out = "evec.dat";
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "-d") && i + 1 < argc) {
      device = std::atoi(argv[++i]);
    } else if (!std::strcmp(argv[i], "-o") && i + 1 < argc) {
      out = argv[++i];
    } else {
      std::fprintf(stderr, "usage: stab_gpu [-d device] [-o evec.dat] < input.dat\n");
      return 2;
    }
  }
  std::string text((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
  stab_params p;
  stab_sweep sw;
  char msg[256] = {0};
  int rc = stab_parse_sweep_input(text.c_str(), &p, &sw, msg, sizeof(msg));
  if (rc) {
    std::fprintf(stderr, "stab_gpu: input: %s\n", msg);
    return 1;
  }
  if (sw.itype == 7 || sw.itype == 8) return run_sweep(p, sw, device);
  int32_t nym = 0;
  std::vector<double> prof;
  if (!load_profile(p.ind, p.ider, prof, nym)) return 1;
  stab_ctx* ctx = nullptr;
  rc = stab_create(&ctx, device);
  if (rc) return fail("stab_create", rc, nullptr);
  const bool spatial = (p.itype == 2 || p.itype == 4);
  const int64_t m = (int64_t)(spatial ? 10 : 5) * p.ny;
  std::vector<double> eig(2 * m);
  int32_t least = -1, status = 0;
  rc = stab_full_spectrum(ctx, &p, nym, prof.data(), eig.data(), nullptr, &least, &status);
  if (rc) return fail("stab_full_spectrum", rc, ctx);
  std::vector<double> vec;
  const bool want_vec = (!spatial || p.ievec == 1);
  if (want_vec) {
    vec.resize(2 * m * m);
    std::vector<int32_t> st(m);
    rc = stab_eigenvectors(ctx, &p, nym, prof.data(), (int32_t)m, eig.data(), vec.data(), st.data());
    if (rc) return fail("stab_eigenvectors", rc, ctx);
  }
  if (p.itype == 2 && p.curve == 2 && p.x != -1.0) p.x = 0.0;   // circh zeroes the module's x (circh.f90:60)
  rc = stab_write_evec(out.c_str(), &p, eig.data(), want_vec ? vec.data() : nullptr);
  if (rc) return fail("stab_write_evec", rc, ctx);
  if (least >= 0)
    std::printf("least-stable %s = (%.15e, %.15e)  index %d of %lld  status %d\n", spatial ? "alpha" : "omega",
                eig[2 * least], eig[2 * least + 1], least + 1, (long long)m, status);
  else
    std::printf("no eigenvalue passed the least-stable filter (status %d)\n", status);
  std::printf("Eigensystem written to %s\n", out.c_str());
  stab_destroy(ctx);
  return 0;
}
