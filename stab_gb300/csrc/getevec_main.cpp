// `getevec` drop-in (getevec.f90:2-233) over the library's evec.dat reader:
//
//   getevec_gpu [-i | -v] [evec file]
//
// -i (default) reads eigenvalue indices (1-based) from stdin, -v reads
// approximate eigenvalues "re im" and picks the nearest (first minimum
// wins).  Each pick writes time.<k> / space.<k>, k = 1, 2, ... with the
// reference's header, row order and format.  Index 0, a value of 0 or the
// end of stdin stops; index -1 prints the eigenvalue table again.
// Host only: no GPU is used.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "stab_gb300.h"

static void table(const stab_evec_header& h, const std::vector<double>& eig) {
  const bool temporal = h.itype == 1;
  std::printf("\n%s Eigensystem:\n\n", temporal ? "Temporal" : "Spatial");
  std::printf("s = %13.6E Yi = %20.13E, Ymax = %13.6E\n", h.x, h.yi, h.ymax);
  if (temporal)
    std::printf("Alpha = (%13.6E,%13.6E)\n", h.alpha[0], h.alpha[1]);
  else
    std::printf("Omega = (%13.6E,%13.6E)\n", h.omega[0], h.omega[1]);
  std::printf("Beta  = (%13.6E,%13.6E)\n", h.beta[0], h.beta[1]);
  std::printf("Re = %13.6E, Ma = %13.6E, Pr = %13.6E\n", h.Re, h.Ma, h.Pr);
  std::printf("%s\n", std::string(100, '=').c_str());
  std::printf("  Index         %s_r                %s_i                  c_r                    c_i\n",
              temporal ? "omega" : "alpha", temporal ? "omega" : "alpha");
  std::printf("%s\n", std::string(100, '=').c_str());
  // phase speed: omega / k with k = sqrt(alpha^2 + beta^2) (temporal), omega / alpha (spatial)
  for (int j = 0; j < h.nmax; ++j) {
    const double er = eig[2 * j], ei = eig[2 * j + 1];
    double cr = 0.0, ci = 0.0;
    if (temporal) {
      // k^2 = alpha^2 + beta^2 (complex), k = principal sqrt
      const double ar = h.alpha[0], ai = h.alpha[1], br = h.beta[0], bi = h.beta[1];
      const double k2r = ar * ar - ai * ai + br * br - bi * bi, k2i = 2.0 * (ar * ai + br * bi);
      const double mod = std::hypot(k2r, k2i);
      double kr = std::sqrt(0.5 * (mod + k2r)), ki = std::sqrt(0.5 * (mod - k2r));
      if (k2i < 0) ki = -ki;
      const double d = kr * kr + ki * ki;
      if (d > 0) {
        cr = (er * kr + ei * ki) / d;
        ci = (ei * kr - er * ki) / d;
      }
    } else if (er != 0.0 || ei != 0.0) {
      const double d = er * er + ei * ei;
      cr = (h.omega[0] * er + h.omega[1] * ei) / d;
      ci = (h.omega[1] * er - h.omega[0] * ei) / d;
    }
    std::printf("%5d    %21.13E  %21.13E  %21.13E  %21.13E\n", j + 1, er, ei, cr, ci);
  }
  std::printf("%s\n\n", std::string(100, '=').c_str());
}

int main(int argc, char** argv) {
  bool use_index = true;
  std::string fname;
  for (int i = 1; i < argc; ++i) {
    if (argv[i][0] != '-') {
      if (!fname.empty()) {
        std::printf("Only one filename argument allowed\n");
        return 1;
      }
      fname = argv[i];
    } else if (!std::strncmp(argv[i], "-i", 2)) {
      use_index = true;
    } else if (!std::strncmp(argv[i], "-v", 2)) {
      use_index = false;
    } else if (!std::strncmp(argv[i], "-h", 2)) {
      std::printf("Usage:  getevec_gpu [-i | -v] [evec file]\n");
      return 0;
    } else {
      std::printf("Argument %2d ignored.\n", i);
    }
  }
  if (fname.empty()) {
    std::printf("Enter the Eigensystem filename ==> ");
    if (!std::getline(std::cin, fname)) return 1;
  }
  stab_evec_header h;
  if (stab_read_evec(fname.c_str(), &h, nullptr, nullptr, nullptr) != STAB_OK) {
    std::printf("Error opening file...\n");
    return 1;
  }
  std::vector<double> y(h.ny), eig(2 * (size_t)h.nmax), vec;
  if (h.has_vectors) vec.resize(2 * (size_t)h.nmax * h.nmax);
  if (stab_read_evec(fname.c_str(), &h, y.data(), eig.data(), h.has_vectors ? vec.data() : nullptr) != STAB_OK) {
    std::printf("Error opening file...\n");
    return 1;
  }
  table(h, eig);
  const char* base = h.itype == 1 ? "time" : "space";
  int iver = 0;
  for (;;) {
    int j = -1;
    if (use_index) {
      std::printf("Which eigenfunction ==> ");
      long v;
      if (!(std::cin >> v)) break;
      if (v == 0) break;
      if (v == -1) {
        table(h, eig);
        continue;
      }
      if (v < -1 || v > h.nmax) continue;
      j = (int)v - 1;
    } else {
      std::printf("Approximate eigenvalue: real, imag  ==> ");
      double vr, vi;
      if (!(std::cin >> vr)) break;
      if (std::cin.peek() == ',') std::cin.get();
      if (!(std::cin >> vi)) break;
      j = stab_getevec_select(eig.data(), h.nmax, vr, vi);
      if (vr == 0.0 && vi == 0.0) break;
    }
    if (!h.has_vectors) {
      std::printf("evec file holds no eigenvectors (ievec = 0)\n");
      return 1;
    }
    const double* vj = vec.data() + 2 * (size_t)j * h.nmax;
    const int64_t len = stab_eigfunction_text(&h, y.data(), eig.data() + 2 * j, vj, nullptr, 0);
    std::string text((size_t)len + 1, '\0');
    stab_eigfunction_text(&h, y.data(), eig.data() + 2 * j, vj, &text[0], len + 1);
    text.resize((size_t)len);
    ++iver;
    const std::string out = std::string(base) + "." + std::to_string(iver);
    std::FILE* f = std::fopen(out.c_str(), "w");
    if (!f) {
      std::printf("cannot write %s\n", out.c_str());
      return 1;
    }
    std::fwrite(text.data(), 1, text.size(), f);
    std::fclose(f);
    std::printf("  Eigenfunction saved in: %s\n", out.c_str());
  }
  return 0;
}
