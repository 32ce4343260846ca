// Drop-ins for the reference's sweep post-processors, which follow one mode
// through the eig.<iver> files that the multi-point drivers write:
//
//   getab_gpu    [-i | -v]  getab.f90: beta sweep; stdin "iver1 iver2
//                           iver_inc", then for the first two files the
//                           mode's index (-i, default) or an approximate
//                           value (-v); later files take the eigenvalue
//                           nearest the linear extrapolation through the two
//                           previous picks (getab.f90:188-201); stab.out
//                           lines "beta Re Im" (format 3(1x,1pe20.13))
//   getax_gpu    [-i | -v]  getax.f90: the same over x (the stations of a
//                           spatial sweep); stab.out lines "ind x Re Im"
//                           (format i4,3(1x,1pe20.13))
//   getalpha_gpu            getalpha.f90: stdin "ind1 ind2 ind_inc", the
//                           first file's mode by index, then the eigenvalue
//                           nearest the previous pick; parm.new lines
//                           "ind xb(ind) Re Im" with xb from body.dat
//
// The program is chosen by the executable's name (or a first argument
// getab / getax / getalpha).  Every run reads body.dat, as the reference
// does.  Host only: the eig.<iver> files come from stab_gpu.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "stab_gb300.h"

typedef std::complex<double> cd;

namespace {

struct EigFile {
  stab_evec_header h;
  std::vector<cd> eval;
};

bool read_eig(int iver, EigFile& f) {
  char name[64];
  stab_eig_name(iver, name, sizeof(name));
  if (stab_read_evec(name, &f.h, nullptr, nullptr, nullptr)) {
    std::fprintf(stderr, "cannot read %s\n", name);
    return false;
  }
  f.eval.assign(f.h.nmax, cd(0, 0));
  if (stab_read_evec(name, &f.h, nullptr, reinterpret_cast<double*>(f.eval.data()), nullptr)) {
    std::fprintf(stderr, "cannot read %s\n", name);
    return false;
  }
  return true;
}

// list-directed reads of the interactive prompts: whitespace/comma tokens
struct Input {
  std::vector<std::string> tok;
  size_t at = 0;
  explicit Input(const std::string& text) {
    std::string s = text;
    for (char& c : s)
      if (c == ',') c = ' ';
    std::istringstream is(s);
    std::string t;
    while (is >> t) tok.push_back(t);
  }
  bool num(double& v) {
    if (at >= tok.size()) return false;
    std::string t = tok[at++];
    for (char& c : t)
      if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && *end == 0;
  }
  bool integer(int& v) {
    double d;
    if (!num(d)) return false;
    v = (int)d;
    return true;
  }
};

// the eigenvalue table of the first files (getab.f90:114-151)
void print_table(const EigFile& f) {
  const cd alpha(f.h.alpha[0], f.h.alpha[1]), beta(f.h.beta[0], f.h.beta[1]), omega(f.h.omega[0], f.h.omega[1]);
  const cd k = std::sqrt(alpha * alpha + beta * beta);
  if (f.h.itype == 1) {
    std::printf("\nTemporal Eigensystem:\n\nAlpha = (%13.6E,%13.6E)\nBeta  = (%13.6E,%13.6E)\n", alpha.real(),
                alpha.imag(), beta.real(), beta.imag());
  } else {
    std::printf("\nSpatial Eigensystem:\n\nOmega = (%13.6E,%13.6E)\nBeta  = (%13.6E,%13.6E)\n", omega.real(),
                omega.imag(), beta.real(), beta.imag());
  }
  std::printf("Re = %13.6E, Ma = %13.6E, Pr = %13.6E\n", f.h.Re, f.h.Ma, f.h.Pr);
  for (int j = 0; j < f.h.nmax; ++j) {
    const cd e = f.eval[j];
    cd c;
    if (f.h.itype == 1) c = e / k;
    else c = (e != cd(0, 0)) ? omega / e : cd(0, 0);
    std::printf("%5d    %21.13E  %21.13E  %21.13E  %21.13E\n", j + 1, e.real(), e.imag(), c.real(), c.imag());
  }
  std::printf("\n");
}

// nearest eigenvalue, strict '<' scan from the first (getab.f90:192-198)
int nearest(const EigFile& f, cd g) {
  return stab_getevec_select(reinterpret_cast<const double*>(f.eval.data()), f.h.nmax, g.real(), g.imag());
}

std::string line(bool with_ind, int ind, double p, cd v) {
  char buf[160];
  stab_stab_out_line(with_ind ? 1 : 0, ind, p, v.real(), v.imag(), buf, sizeof(buf));
  return buf;
}

int run_ab(bool over_x, bool use_index, Input& in) {
  int iver1, iver2, inc;
  if (!in.integer(iver1) || !in.integer(iver2) || !in.integer(inc) || inc == 0) {
    std::fprintf(stderr, "need iver1, iver2, iver_inc\n");
    return 1;
  }
  int32_t nbody = 0;
  if (stab_read_body("body.dat", 0, nullptr, &nbody)) {
    std::fprintf(stderr, "cannot read body.dat\n");
    return 1;
  }
  std::FILE* out = nullptr;
  cd eval1, eval2, parm1, parm2;
  int icount = 0;
  for (int iver = iver1; inc > 0 ? iver <= iver2 : iver >= iver2; iver += inc) {
    ++icount;
    EigFile f;
    if (!read_eig(iver, f)) return 1;
    const cd parm = over_x ? cd(f.h.x, 0.0) : cd(f.h.beta[0], f.h.beta[1]);
    int j = 0;
    if (icount <= 2) {
      print_table(f);
      if (use_index) {
        std::printf("Which eigenvalue ==> ");
        if (!in.integer(j) || j < 1 || j > f.h.nmax) {
          std::fprintf(stderr, "bad eigenvalue index\n");
          return 1;
        }
        j -= 1;
      } else {
        std::printf("Approximate eigenvalue: real, imag ==> ");
        double vr, vi;
        if (!in.num(vr) || !in.num(vi)) {
          std::fprintf(stderr, "need real, imag\n");
          return 1;
        }
        j = nearest(f, cd(vr, vi));
      }
      std::printf("\n");
      if (icount == 2) {
        eval2 = eval1;
        parm2 = parm1;
      }
      eval1 = f.eval[j];
      parm1 = parm;
      if (!out) out = std::fopen("stab.out", "w");
      if (!out) return 1;
    } else {
      const cd g = eval1 + (eval2 - eval1) / (parm2 - parm1) * (parm - parm1);
      j = nearest(f, g);
      eval2 = eval1;
      parm2 = parm1;
      eval1 = f.eval[j];
      parm1 = parm;
    }
    const std::string s = over_x ? line(true, f.h.ind, f.h.x, f.eval[j]) : line(false, 0, parm.real(), f.eval[j]);
    std::fputs(s.c_str(), out);
    std::fputc('\n', out);
  }
  if (out) std::fclose(out);
  return 0;
}

int run_alpha(Input& in) {
  int ind1, ind2, inc;
  if (!in.integer(ind1) || !in.integer(ind2) || !in.integer(inc) || inc == 0) {
    std::fprintf(stderr, "need ind1, ind2, ind_inc\n");
    return 1;
  }
  int32_t nbody = 0;
  if (stab_read_body("body.dat", 0, nullptr, &nbody)) {
    std::fprintf(stderr, "cannot read body.dat\n");
    return 1;
  }
  std::vector<double> xb(nbody);
  stab_read_body("body.dat", nbody, xb.data(), &nbody);
  if (ind1 < 1 || ind2 > nbody) {
    std::printf("ERROR: illegal index...check body.dat\n");   // getalpha.f90:45-48
    return 1;
  }
  std::FILE* out = nullptr;
  cd eval1;
  int iver = 0;
  for (int ind = ind1; inc > 0 ? ind <= ind2 : ind >= ind2; ind += inc) {
    ++iver;
    EigFile f;
    if (!read_eig(iver, f)) return 1;
    int j = 0;
    if (iver == 1) {
      print_table(f);
      std::printf("Which eigenvalue ==> ");
      if (!in.integer(j) || j < 1 || j > f.h.nmax) {
        std::fprintf(stderr, "bad eigenvalue index\n");
        return 1;
      }
      j -= 1;
      std::printf("\n");
      out = std::fopen("parm.new", "w");
      if (!out) return 1;
    } else {
      j = nearest(f, eval1);
    }
    eval1 = f.eval[j];
    const std::string s = line(true, ind, xb[ind - 1], eval1);
    std::fputs(s.c_str(), out);
    std::fputc('\n', out);
  }
  if (out) std::fclose(out);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::string prog = argv[0];
  const size_t sl = prog.find_last_of('/');
  if (sl != std::string::npos) prog = prog.substr(sl + 1);
  int a = 1;
  if (argc > 1 && (!std::strcmp(argv[1], "getab") || !std::strcmp(argv[1], "getax") || !std::strcmp(argv[1], "getalpha"))) {
    prog = argv[1];
    a = 2;
  }
  bool use_index = true;
  for (; a < argc; ++a) {
    if (!std::strncmp(argv[a], "-i", 2)) use_index = true;
    else if (!std::strncmp(argv[a], "-v", 2)) use_index = false;
    else if (!std::strncmp(argv[a], "-h", 2)) {
      std::printf("Usage:  %s [-i | -v]\n   -i:  locate based on index (default)\n   -v:  locate based on eigenvalue\n",
                  prog.c_str());
      return 0;
    } else {
      std::printf("Argument %2d ignored.\n", a);
    }
  }
  std::string text((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
  Input in(text);
  if (prog.rfind("getalpha", 0) == 0) return run_alpha(in);
  if (prog.rfind("getax", 0) == 0) return run_ab(true, use_index, in);
  if (prog.rfind("getab", 0) == 0) return run_ab(false, use_index, in);
  std::fprintf(stderr, "run as getab_gpu, getax_gpu or getalpha_gpu\n");
  return 2;
}
