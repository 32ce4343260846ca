// `stab` drop-in for the Chebyshev temporal and spatial paths: reads the
// reference's stdin protocol (input.f90:15-123, stab.f90:46-55), the mean
// flow from profile.<ind> in the working directory, solves on the GPU and
// writes evec.dat as temporal.f90:883-890 / spatial.f90:1120-1126 do.
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
  char msg[256] = {0};
  int rc = stab_parse_input(text.c_str(), &p, msg, sizeof(msg));
  if (rc) {
    std::fprintf(stderr, "stab_gpu: input: %s\n", msg);
    return 1;
  }
  char pname[64];
  stab_profile_name(p.ind, pname, sizeof(pname));
  int32_t nym = 0;
  rc = stab_read_profile(pname, 0, nullptr, &nym);
  if (rc) {
    std::fprintf(stderr, "stab_gpu: cannot read %s\n", pname);
    return 1;
  }
  std::vector<double> prof(6 * (size_t)nym);
  rc = stab_read_profile(pname, nym, prof.data(), &nym);
  if (rc) {
    std::fprintf(stderr, "stab_gpu: cannot read %s\n", pname);
    return 1;
  }
  stab_ctx* ctx = nullptr;
  rc = stab_create(&ctx, device);
  if (rc) return fail("stab_create", rc, nullptr);
  const int64_t m = (int64_t)(p.itype == 1 ? 5 : 10) * p.ny;
  std::vector<double> eig(2 * m);
  int32_t least = -1, status = 0;
  rc = stab_full_spectrum(ctx, &p, nym, prof.data(), eig.data(), nullptr, &least, &status);
  if (rc) return fail("stab_full_spectrum", rc, ctx);
  std::vector<double> vec;
  const bool want_vec = (p.itype == 1 || p.ievec == 1);
  if (want_vec) {
    vec.resize(2 * m * m);
    std::vector<int32_t> st(m);
    rc = stab_eigenvectors(ctx, &p, nym, prof.data(), (int32_t)m, eig.data(), vec.data(), st.data());
    if (rc) return fail("stab_eigenvectors", rc, ctx);
  }
  rc = stab_write_evec(out.c_str(), &p, eig.data(), want_vec ? vec.data() : nullptr);
  if (rc) return fail("stab_write_evec", rc, ctx);
  if (least >= 0)
    std::printf("least-stable %s = (%.15e, %.15e)  index %d of %lld  status %d\n", p.itype == 1 ? "omega" : "alpha",
                eig[2 * least], eig[2 * least + 1], least + 1, (long long)m, status);
  else
    std::printf("no eigenvalue passed the least-stable filter (status %d)\n", status);
  std::printf("Eigensystem written to %s\n", out.c_str());
  stab_destroy(ctx);
  return 0;
}
