// The reference's file interface for the Chebyshev path, on the host.
//
//   stab_parse_input       stdin of `stab < input.dat`: input.f90:15-123 and the
//                          index / x reads of stab.f90:46-55
//   stab_parse_sweep_input the same with the multi-point drivers (itype 7,
//                          mtemporal.f90:20-23; itype 8, mspatial.f90:20-27)
//   stab_sweep_points      the drivers' loops (mtemporal.f90:25-39,
//                          mspatial.f90:65-96) as a list of solves
//   stab_read_delta        delta.dat (mspatial.f90:29-63)
//   stab_read_body         body.dat (getab.f90:73-86, getalpha.f90:36-53)
//   stab_eig_name          eig.<iver> (makename, mtemporal.f90:53-76)
//   stab_read_profile      profile.<ind>: rows "y rho u v w T", records that
//                          start with '#' skipped (getmean.f90:27-80)
//   stab_grid              Gauss-Lobatto points and the algebraic maps
//                          (sgengrid.f90:18-45)
//   stab_write_evec        evec.dat, gfortran sequential unformatted: 4-byte
//                          little-endian record lengths around each record
//                          (temporal.f90:883-890, spatial.f90:1120-1126)
//   stab_read_evec         the reader side (getevec.f90:77-91)
//   stab_getevec_select    getevec -v: nearest eigenvalue, first minimum wins
//                          (getevec.f90:161-172)
//   stab_eigfunction_text  the time.N / space.N file, including the scale
//                          quirk of getevec.f90:179-189 (`scale` is REAL, so
//                          only the real part of the running pick is kept)
//
// Nothing here touches the GPU; these run wherever the library loads.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "stab_gb300.h"

namespace {

const int kNdof = 5;

// Fortran list-directed input over the records of a text.  Each read
// statement starts at the next record, takes values separated by blanks or
// commas from as many records as it needs, and drops the rest of its last
// record; a '/' ends the statement early.
struct ListReader {
  std::vector<std::string> recs;
  size_t next = 0;
  bool slash = false;   // the last read ended at a '/'

  explicit ListReader(const char* text) {
    std::string cur;
    for (const char* q = text; *q; ++q) {
      if (*q == '\n') {
        recs.push_back(cur);
        cur.clear();
      } else if (*q != '\r') {
        cur.push_back(*q);
      }
    }
    if (!cur.empty()) recs.push_back(cur);
  }

  int read(int k, std::vector<std::string>& out) {
    out.clear();
    slash = false;
    while (next < recs.size() && (int)out.size() < k) {
      const std::string& r = recs[next++];
      size_t i = 0;
      while (i < r.size() && (int)out.size() < k) {
        while (i < r.size() && (r[i] == ' ' || r[i] == '\t' || r[i] == ',')) ++i;
        if (i >= r.size()) break;
        size_t j = i;
        while (j < r.size() && r[j] != ' ' && r[j] != '\t' && r[j] != ',') ++j;
        std::string tok = r.substr(i, j - i);
        i = j;
        if (tok == "/") {
          slash = true;
          return (int)out.size();
        }
        out.push_back(tok);
      }
    }
    return (int)out.size();
  }
};

bool to_int(const std::string& s, int32_t& v) {
  char* end = nullptr;
  errno = 0;
  long x = std::strtol(s.c_str(), &end, 10);
  if (errno || end == s.c_str() || *end) return false;
  v = (int32_t)x;
  return true;
}

bool to_real(std::string s, double& v) {
  for (char& ch : s)
    if (ch == 'd' || ch == 'D') ch = 'e';
  char* end = nullptr;
  errno = 0;
  double x = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end) return false;
  v = x;
  return true;
}

void set_msg(char* msg, size_t cap, const std::string& s) {
  if (msg && cap) std::snprintf(msg, cap, "%s", s.c_str());
}

// Fortran 1P Ew.d[Ee] edit: one digit before the point, d after; without Ee
// the exponent is E+dd up to 99 and +ddd beyond; right-justified in w.
std::string fortran_e(double x, int w, int d, int e) {
  std::string out;
  if (std::isnan(x)) {
    out = "NaN";
  } else if (std::isinf(x)) {
    out = x > 0 ? "Infinity" : "-Infinity";
  } else {
    char buf[64];
    int ex = 0;
    std::string mant;
    if (x == 0.0) {
      mant = "0." + std::string(d, '0');
    } else {
      std::snprintf(buf, sizeof(buf), "%.*E", d, std::fabs(x));
      const char* ep = std::strchr(buf, 'E');
      mant.assign(buf, ep - buf);
      ex = std::atoi(ep + 1);
    }
    const bool neg = std::signbit(x);
    char es[16];
    const int ax = ex < 0 ? -ex : ex;
    if (e > 0)
      std::snprintf(es, sizeof(es), "E%c%0*d", ex < 0 ? '-' : '+', e, ax);
    else if (ax <= 99)
      std::snprintf(es, sizeof(es), "E%c%02d", ex < 0 ? '-' : '+', ax);
    else
      std::snprintf(es, sizeof(es), "%c%03d", ex < 0 ? '-' : '+', ax);
    out = (neg ? "-" : "") + mant + es;
  }
  if ((int)out.size() < w) out = std::string(w - out.size(), ' ') + out;
  return out;
}

std::string e2113(double x) { return fortran_e(x, 21, 13, 3); }
std::string e136(double x) { return fortran_e(x, 13, 6, 0); }

// gfortran sequential unformatted record
void put_record(std::FILE* f, const void* data, size_t bytes) {
  const uint32_t n = (uint32_t)bytes;
  unsigned char len[4] = {(unsigned char)(n & 0xff), (unsigned char)((n >> 8) & 0xff),
                          (unsigned char)((n >> 16) & 0xff), (unsigned char)((n >> 24) & 0xff)};
  std::fwrite(len, 1, 4, f);
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fwrite(len, 1, 4, f);
}

uint32_t le32(const unsigned char* b) {
  return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}

bool get_record(std::FILE* f, std::vector<unsigned char>& rec) {
  unsigned char len[4], tail[4];
  if (std::fread(len, 1, 4, f) != 4) return false;
  const uint32_t n = le32(len);
  rec.resize(n);
  if (n && std::fread(rec.data(), 1, n, f) != n) return false;
  if (std::fread(tail, 1, 4, f) != 4) return false;
  return le32(tail) == n;
}

}  // namespace

// The stdin protocol shared by stab_parse_input (itypes 1 and 2) and
// stab_parse_sweep_input (also the multi-point drivers, itypes 7 and 8).
static int parse_protocol(const char* text, stab_params* p, stab_sweep* sw, char* msg, size_t msg_cap) {
  if (!text || !p) return STAB_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  if (sw) std::memset(sw, 0, sizeof(*sw));
  ListReader rd(text);
  std::vector<std::string> v;
  // a read cut short by '/' leaves the remaining items as they were
  auto need = [&](int k, const char* what) -> bool {
    if (rd.read(k, v) < k && !rd.slash) {
      set_msg(msg, msg_cap, std::string("input ended before ") + what);
      return false;
    }
    return true;
  };
  auto ints = [&](int k, int32_t* dst, const char* what) -> bool {
    if (!need(k, what)) return false;
    for (int i = 0; i < (int)v.size(); ++i)
      if (!to_int(v[i], dst[i])) {
        set_msg(msg, msg_cap, std::string("bad integer '") + v[i] + "' for " + what);
        return false;
      }
    return true;
  };
  auto reals = [&](int k, double* dst, const char* what) -> bool {
    if (!need(k, what)) return false;
    for (int i = 0; i < (int)v.size(); ++i)
      if (!to_real(v[i], dst[i])) {
        set_msg(msg, msg_cap, std::string("bad real '") + v[i] + "' for " + what);
        return false;
      }
    return true;
  };
  // the reference asks again until it gets 0 or 1 (input.f90:15-17)
  do {
    if (!ints(1, &p->mattyp, "mattyp")) return STAB_ERR_ARG;
  } while (p->mattyp != 0 && p->mattyp != 1);
  if (p->mattyp == 1 && !reals(1, &p->T0, "T0")) return STAB_ERR_ARG;
  double mrp[3] = {0.0, 0.0, 0.0};
  if (!reals(3, mrp, "Ma, Re, Pr")) return STAB_ERR_ARG;
  p->Ma = mrp[0];
  p->Re = mrp[1];
  p->Pr = mrp[2];
  if (!need(3, "ny, Yi, Ymax")) return STAB_ERR_ARG;
  if (v.size() < 3 || !to_int(v[0], p->ny) || !to_real(v[1], p->yi) || !to_real(v[2], p->ymax)) {
    set_msg(msg, msg_cap, "bad ny, Yi, Ymax");
    return STAB_ERR_ARG;
  }
  if (!ints(1, &p->ievec, "ievec")) return STAB_ERR_ARG;
  int32_t itmp = 0;
  if (!ints(1, &itmp, "ider")) return STAB_ERR_ARG;
  p->ider = itmp != 0 ? 1 : 0;
  int32_t bc[4] = {0, 0, 0, 0};
  if (!ints(4, bc, "top, wall, wallt, curve")) return STAB_ERR_ARG;
  p->top = bc[0];
  p->wall = bc[1];
  p->wallt = bc[2];
  p->curve = bc[3];
  // itype outside 1..9 is asked again (input.f90:53,120-121)
  do {
    if (!ints(1, &p->itype, "itype")) return STAB_ERR_ARG;
  } while (p->itype < 1 || p->itype > 9);
  if (sw && (p->itype == 7 || p->itype == 8)) {
    // stab.f90:85-90: the drivers run with ind = 0 and itype 1 / 2; input.f90
    // reads no wavenumbers for them (input.f90:104-115)
    sw->itype = p->itype;
    p->itype = (sw->itype == 7) ? 1 : 2;
    double r[3];
    // mtemporal.f90:20-23 / mspatial.f90:20-23
    if (!reals(3, r, sw->itype == 7 ? "alpha_min, alpha_max, alpha_inc" : "omega_min, omega_max, omega_inc"))
      return STAB_ERR_ARG;
    sw->p_min = r[0]; sw->p_max = r[1]; sw->p_inc = r[2];
    if (!reals(3, r, "beta_min, beta_max, beta_inc")) return STAB_ERR_ARG;
    sw->b_min = r[0]; sw->b_max = r[1]; sw->b_inc = r[2];
    if (sw->itype == 8) {
      int32_t ii[3];
      if (!ints(3, ii, "ind1, ind2, ind_inc")) return STAB_ERR_ARG;   // mspatial.f90:24-25
      sw->ind1 = ii[0]; sw->ind2 = ii[1]; sw->ind_inc = ii[2];
      if (!ints(1, &sw->dtype, "dtype")) return STAB_ERR_ARG;         // mspatial.f90:26-27
      if (sw->dtype != 0) {
        set_msg(msg, msg_cap, "dtype 1 (finite-difference spatial solver) is outside the Chebyshev path");
        return STAB_ERR_ARG;
      }
    }
    if (p->ny < 2) {
      set_msg(msg, msg_cap, "ny < 2");
      return STAB_ERR_ARG;
    }
    return STAB_OK;
  }
  if (p->itype < 1 || p->itype > 4) {
    set_msg(msg, msg_cap, "itype " + std::to_string(p->itype) +
                              (sw ? " (Stokes or bump solver)" : " (Stokes, bump or multi-point driver)") +
                              " is outside the temporal/spatial path");
    return STAB_ERR_ARG;
  }
  // itypes 3 and 4: the finite-difference solvers, with the questions of
  // the Chebyshev ones (stab.f90:56-67)
  if (p->itype == 1 || p->itype == 3) {
    if (!reals(2, p->alpha, "alphar, alphai")) return STAB_ERR_ARG;
  } else {
    if (!reals(2, p->omega, "omegar, omegai")) return STAB_ERR_ARG;
  }
  if (!reals(2, p->beta, "betar, betai")) return STAB_ERR_ARG;
  if (!ints(1, &p->ind, "index")) return STAB_ERR_ARG;
  if ((p->itype == 2 || p->itype == 4) && !reals(1, &p->x, "x")) return STAB_ERR_ARG;
  if (p->ny < 2) {
    set_msg(msg, msg_cap, "ny < 2");
    return STAB_ERR_ARG;
  }
  return STAB_OK;
}

extern "C" {

int stab_parse_input(const char* text, stab_params* p, char* msg, size_t msg_cap) {
  return parse_protocol(text, p, nullptr, msg, msg_cap);
}

int stab_parse_sweep_input(const char* text, stab_params* p, stab_sweep* sw, char* msg, size_t msg_cap) {
  if (!sw) return STAB_ERR_ARG;
  return parse_protocol(text, p, sw, msg, msg_cap);
}

int stab_read_delta(const char* path, int32_t cap, double* xb, double* delta, int32_t* nbody) {
  // mspatial.f90:29-63: every record that does not start with '#' holds
  // "xb delta" (list-directed; further items ignored)
  if (!path || !nbody) return STAB_ERR_ARG;
  std::FILE* f = std::fopen(path, "r");
  if (!f) return STAB_ERR_IO;
  int32_t n = 0;
  char line[4096];
  int rc = STAB_OK;
  while (std::fgets(line, sizeof(line), f)) {
    if (line[0] == '#') continue;
    ListReader rd(line);
    std::vector<std::string> v;
    double a = 0.0, b = 0.0;
    if (rd.read(2, v) < 2 || !to_real(v[0], a) || !to_real(v[1], b)) {
      rc = STAB_ERR_IO;
      break;
    }
    if (xb && delta) {
      if (n >= cap) { rc = STAB_ERR_ARG; break; }
      xb[n] = a;
      delta[n] = b;
    }
    ++n;
  }
  std::fclose(f);
  *nbody = n;
  return rc;
}

int stab_read_body(const char* path, int32_t cap, double* xb, int32_t* nbody) {
  // getab.f90:73-86, getalpha.f90:36-53: one record per station, "index xb"
  if (!path || !nbody) return STAB_ERR_ARG;
  std::FILE* f = std::fopen(path, "r");
  if (!f) return STAB_ERR_IO;
  int32_t n = 0;
  char line[4096];
  int rc = STAB_OK;
  while (std::fgets(line, sizeof(line), f)) {
    ListReader rd(line);
    std::vector<std::string> v;
    if (rd.read(2, v) == 0) break;   // the reference's counting read stops at the end of the data
    int32_t it = 0;
    double a = 0.0;
    if (v.size() < 2 || !to_int(v[0], it) || !to_real(v[1], a)) {
      rc = STAB_ERR_IO;
      break;
    }
    if (xb) {
      if (n >= cap) { rc = STAB_ERR_ARG; break; }
      xb[n] = a;
    }
    ++n;
  }
  std::fclose(f);
  *nbody = n;
  return rc;
}

int stab_stab_out_line(int32_t with_ind, int32_t ind, double p, double vr, double vi, char* out, size_t cap) {
  // getab.f90:211 format 60: 3(1x,1pe20.13); getax.f90:214 / getalpha.f90:167
  // format 50: i4,3(1x,1pe20.13)
  if (!out || cap == 0) return STAB_ERR_ARG;
  std::string s;
  if (with_ind) {
    char b[32];
    std::snprintf(b, sizeof(b), "%4d", (int)ind);
    s = (std::strlen(b) > 4) ? std::string(4, '*') : std::string(b);
  }
  for (double x : {p, vr, vi}) s += " " + fortran_e(x, 20, 13, 0);
  if (s.size() + 1 > cap) return STAB_ERR_ARG;
  std::memcpy(out, s.c_str(), s.size() + 1);
  return (int)s.size();
}

int stab_eig_name(int32_t iver, char* out, size_t cap) {
  // makename (mtemporal.f90:53-76): "eig." + iver in I1..I4
  if (!out || iver < 0 || iver > 9999) return STAB_ERR_ARG;
  std::snprintf(out, cap, "eig.%d", (int)iver);
  return STAB_OK;
}

int stab_sweep_points(const stab_params* base, const stab_sweep* sw, int32_t nbody, const double* xb,
                      const double* delta, int32_t cap, stab_params* points, int32_t* count) {
  if (!base || !sw || !count) return STAB_ERR_ARG;
  std::vector<stab_params> pts;
  if (sw->itype == 7) {
    // mtemporal.f90:25-39: na = max(nint((amax-amin)/ainc), 1) (amax itself
    // is not reached), beta innermost, profile.0
    if (sw->p_inc == 0.0 || sw->b_inc == 0.0) return STAB_ERR_ARG;
    const int na = std::max((int)std::lround((sw->p_max - sw->p_min) / sw->p_inc), 1);
    const int nb = std::max((int)std::lround((sw->b_max - sw->b_min) / sw->b_inc), 1);
    for (int ia = 1; ia <= na; ++ia)
      for (int ib = 1; ib <= nb; ++ib) {
        stab_params q = *base;
        q.itype = 1;
        q.ind = 0;
        q.alpha[0] = sw->p_min + (double)(ia - 1) * sw->p_inc;
        q.alpha[1] = 0.0;
        q.beta[0] = sw->b_min + (double)(ib - 1) * sw->b_inc;
        q.beta[1] = 0.0;
        pts.push_back(q);
      }
  } else if (sw->itype == 8) {
    // mspatial.f90:65-96: zero increments become one, no = nint(...) + 1,
    // stations ind1..ind2 step ind_inc with x = xb(ind), Yi = 2 delta(ind)
    if (!xb || !delta) return STAB_ERR_ARG;
    const int i1 = sw->ind1, i2 = sw->ind2;
    if (i1 < 1 || i2 > nbody) return STAB_ERR_ARG;
    const double oinc = (sw->p_inc == 0.0) ? 1.0 : sw->p_inc;
    const double binc = (sw->b_inc == 0.0) ? 1.0 : sw->b_inc;
    const int inc = (sw->ind_inc == 0) ? 1 : sw->ind_inc;
    const int no = (int)std::lround((sw->p_max - sw->p_min) / oinc) + 1;
    const int nb = (int)std::lround((sw->b_max - sw->b_min) / binc) + 1;
    for (int ind = i1; inc > 0 ? ind <= i2 : ind >= i2; ind += inc)
      for (int io = 1; io <= no; ++io)
        for (int ib = 1; ib <= nb; ++ib) {
          stab_params q = *base;
          q.itype = 2;
          q.ind = ind;
          q.x = xb[ind - 1];
          q.yi = 2.0 * delta[ind - 1];
          q.omega[0] = sw->p_min + (double)(io - 1) * oinc;
          q.omega[1] = 0.0;
          q.beta[0] = sw->b_min + (double)(ib - 1) * binc;
          q.beta[1] = 0.0;
          q.alpha[0] = q.alpha[1] = 0.0;
          pts.push_back(q);
        }
  } else {
    return STAB_ERR_ARG;
  }
  *count = (int32_t)pts.size();
  if (points) {
    if ((int32_t)pts.size() > cap) return STAB_ERR_ARG;
    std::memcpy(points, pts.data(), sizeof(stab_params) * pts.size());
  }
  return STAB_OK;
}

int stab_profile_name(int32_t ind, char* out, size_t cap) {
  // makename (getmean.f90:27-28): base + '.' + the index in I1/I2/I3
  if (!out || ind < 0 || ind > 999) return STAB_ERR_ARG;
  std::snprintf(out, cap, "profile.%d", (int)ind);
  return STAB_OK;
}

int stab_read_profile(const char* path, int32_t cap_rows, double* rows, int32_t* nym) {
  if (!path || !nym) return STAB_ERR_ARG;
  std::FILE* f = std::fopen(path, "r");
  if (!f) return STAB_ERR_IO;
  std::string line;
  int32_t n = 0;
  int rc = STAB_OK;
  char buf[4096];
  while (std::fgets(buf, sizeof(buf), f)) {
    line = buf;
    while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
    if (!line.empty() && line[0] == '#') continue;
    ListReader rd(line.c_str());
    std::vector<std::string> v;
    const int got = rd.read(6, v);
    if (got == 0) continue;   // blank record
    if (got < 6) {
      rc = STAB_ERR_IO;
      break;
    }
    if (rows) {
      if (n >= cap_rows) {
        rc = STAB_ERR_ARG;
        break;
      }
      for (int i = 0; i < 6; ++i)
        if (!to_real(v[i], rows[6 * (int64_t)n + i])) rc = STAB_ERR_IO;
      if (rc) break;
    }
    ++n;
  }
  std::fclose(f);
  *nym = n;
  if (rc == STAB_OK && n < 2) rc = STAB_ERR_IO;
  return rc;
}

int stab_fd_grid(int32_t ny, double yi, double ymax, double* y, double* eta, double* deta, double* d2eta) {
  if (ny < 2 || yi == 0.0 || !(ymax > 2.0 * yi) || !y || !eta || !deta || !d2eta) return STAB_ERR_ARG;
  const double dy = 1.0 / (double)(ny - 1);
  const double aa = ymax * yi / (ymax - 2.0 * yi);
  const double bb = 1.0 + aa / ymax;
  for (int i = 0; i < ny; ++i) {
    const double e = (double)i * dy, q = bb - e;
    eta[i] = e;
    y[i] = aa * e / q;
    deta[i] = q * q / (aa * bb);
    d2eta[i] = -2.0 * q * q * q / ((aa * bb) * (aa * bb));
  }
  return STAB_OK;
}

int stab_grid(int32_t ny, double yi, double ymax, double* y, double* eta, double* deta, double* d2eta) {
  if (ny < 2 || yi == 0.0 || !y || !eta || !deta || !d2eta) return STAB_ERR_ARG;
  const double pi = std::acos(-1.0);
  const double dth = pi / (double)(ny - 1);
  for (int i = 0; i < ny; ++i) {
    const double e = std::cos((double)i * dth);
    eta[i] = e;
    if (ymax == 0.0) {   // infinite domain, L = Yi
      const double L = yi;
      deta[i] = (e - 1.0) * (e - 1.0) / (2.0 * L);
      d2eta[i] = (e - 1.0) * (e - 1.0) * (e - 1.0) / (2.0 * L * L);
      y[i] = (e != 1.0) ? L * (1.0 + e) / (1.0 - e) : 1.0e99;
    } else {             // Streett's map on [0, ymax]
      const double g = 2.0 * yi + 1.0 - e;
      const double h = ymax * yi * (yi + 1.0);
      y[i] = ymax * yi * (1.0 + e) / (1.0 + 2.0 * yi - e);
      deta[i] = g * g / (2.0 * h);
      d2eta[i] = -0.5 * g * g * g / (h * h);
    }
  }
  return STAB_OK;
}

int stab_write_evec(const char* path, const stab_params* p, const double* eig, const double* vec) {
  if (!path || !p || !eig || p->ny < 2) return STAB_ERR_ARG;
  if (p->itype < 1 || p->itype > 4) return STAB_ERR_ARG;
  const int ny = p->ny;
  // itypes 3 and 4 (finite differences) are recorded as 1 and 2
  // (stab.f90:59, :66), with ogengrid's grid (fd_temporal.f90:1052-1055)
  const bool fd = (p->itype == 3 || p->itype == 4);
  const int32_t itype = (p->itype == 3) ? 1 : (p->itype == 4 ? 2 : p->itype);
  const int64_t nmax = (int64_t)(itype == 1 ? 1 : 2) * kNdof * ny;
  const bool want_vec = (itype == 1 || p->ievec == 1);
  if (want_vec && !vec) return STAB_ERR_ARG;
  std::vector<double> y(ny), eta(ny), deta(ny), d2eta(ny);
  int rc = fd ? stab_fd_grid(ny, p->yi, p->ymax, y.data(), eta.data(), deta.data(), d2eta.data())
              : stab_grid(ny, p->yi, p->ymax, y.data(), eta.data(), deta.data(), d2eta.data());
  if (rc) return rc;
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return STAB_ERR_IO;
  const int32_t r1[10] = {p->ind, p->ny, kNdof, itype, p->ievec, p->curve, p->top, p->wall, p->wallt,
                          p->ider ? 1 : 0};
  put_record(f, r1, sizeof(r1));
  const double r2[9] = {p->omega[0], p->omega[1], p->alpha[0], p->alpha[1], p->beta[0], p->beta[1],
                        p->Re, p->Ma, p->Pr};
  put_record(f, r2, sizeof(r2));
  std::vector<double> r3;
  r3.reserve(3 + 4 * (size_t)ny);
  r3.push_back(p->x);
  r3.insert(r3.end(), y.begin(), y.end());
  r3.insert(r3.end(), eta.begin(), eta.end());
  r3.insert(r3.end(), deta.begin(), deta.end());
  r3.insert(r3.end(), d2eta.begin(), d2eta.end());
  r3.push_back(p->yi);
  r3.push_back(p->ymax);
  put_record(f, r3.data(), sizeof(double) * r3.size());
  put_record(f, eig, sizeof(double) * 2 * nmax);
  if (want_vec) put_record(f, vec, sizeof(double) * 2 * nmax * nmax);
  rc = std::ferror(f) ? STAB_ERR_IO : STAB_OK;
  if (std::fclose(f) != 0) rc = STAB_ERR_IO;
  return rc;
}

int stab_read_evec(const char* path, stab_evec_header* h, double* y, double* eig, double* vec) {
  if (!path || !h) return STAB_ERR_ARG;
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return STAB_ERR_IO;
  std::vector<unsigned char> r;
  int rc = STAB_OK;
  std::memset(h, 0, sizeof(*h));
  do {
    // R1 holds 9 or 10 int32 (readers take the first 9; getevec.f90:79)
    if (!get_record(f, r) || r.size() < 9 * 4) { rc = STAB_ERR_IO; break; }
    int32_t i1[10] = {0};
    std::memcpy(i1, r.data(), r.size() >= 40 ? 40 : 36);
    h->ind = i1[0]; h->ny = i1[1]; h->ndof = i1[2]; h->itype = i1[3]; h->ievec = i1[4];
    h->curve = i1[5]; h->top = i1[6]; h->wall = i1[7]; h->wallt = i1[8]; h->ider = i1[9];
    if (h->ny < 2 || h->ndof != kNdof || (h->itype != 1 && h->itype != 2)) { rc = STAB_ERR_IO; break; }
    h->nmax = (h->itype == 1 ? 1 : 2) * h->ndof * h->ny;
    if (!get_record(f, r) || r.size() != 9 * 8) { rc = STAB_ERR_IO; break; }
    double r2[9];
    std::memcpy(r2, r.data(), sizeof(r2));
    h->omega[0] = r2[0]; h->omega[1] = r2[1]; h->alpha[0] = r2[2]; h->alpha[1] = r2[3];
    h->beta[0] = r2[4]; h->beta[1] = r2[5]; h->Re = r2[6]; h->Ma = r2[7]; h->Pr = r2[8];
    if (!get_record(f, r) || r.size() != (size_t)(3 + 4 * h->ny) * 8) { rc = STAB_ERR_IO; break; }
    std::vector<double> r3(3 + 4 * (size_t)h->ny);
    std::memcpy(r3.data(), r.data(), r.size());
    h->x = r3[0];
    h->yi = r3[1 + 4 * (size_t)h->ny];
    h->ymax = r3[2 + 4 * (size_t)h->ny];
    if (y) std::memcpy(y, r3.data() + 1, sizeof(double) * h->ny);
    if (!get_record(f, r) || r.size() != (size_t)h->nmax * 16) { rc = STAB_ERR_IO; break; }
    if (eig) std::memcpy(eig, r.data(), r.size());
    h->has_vectors = 0;
    if (get_record(f, r)) {
      if (r.size() != (size_t)h->nmax * h->nmax * 16) { rc = STAB_ERR_IO; break; }
      h->has_vectors = 1;
      if (vec) std::memcpy(vec, r.data(), r.size());
    }
  } while (false);
  std::fclose(f);
  return rc;
}

int32_t stab_getevec_select(const double* eig, int32_t nmax, double vr, double vi) {
  if (!eig || nmax <= 0) return -1;
  int32_t best = 0;
  double bd = std::hypot(vr - eig[0], vi - eig[1]);
  for (int32_t j = 1; j < nmax; ++j) {
    const double d = std::hypot(vr - eig[2 * j], vi - eig[2 * j + 1]);
    if (d < bd) {
      bd = d;
      best = j;
    }
  }
  return best;
}

int64_t stab_eigfunction_text(const stab_evec_header* h, const double* y, const double* eig_j, const double* vec_j,
                              char* buf, int64_t cap) {
  if (!h || !y || !eig_j || !vec_j || h->ny < 2) return STAB_ERR_ARG;
  const int ny = h->ny, nd = h->ndof;
  // getevec.f90:179-189: running pick by modulus, only its real part kept
  double scale = 0.0;
  for (int i = 0; i < ny * nd; ++i) {
    const double a = std::hypot(vec_j[2 * i], vec_j[2 * i + 1]);
    if (a > std::fabs(scale)) scale = vec_j[2 * i];
  }
  std::string s;
  s += "# Re = " + e136(h->Re) + ", Ma = " + e136(h->Ma) + ", Pr = " + e136(h->Pr) + "\n";
  auto cx = [&](double re, double im) { return "(" + e2113(re) + "," + e2113(im) + ")"; };
  if (h->itype == 1) {
    s += "# Omega = " + cx(eig_j[0], eig_j[1]) + "\n";
    s += "# Alpha = " + cx(h->alpha[0], h->alpha[1]) + "\n";
  } else {
    s += "# Omega = " + cx(h->omega[0], h->omega[1]) + "\n";
    s += "# Alpha = " + cx(eig_j[0], eig_j[1]) + "\n";
  }
  s += "# Beta  = " + cx(h->beta[0], h->beta[1]) + "\n";
  for (int i = ny - 1; i >= 0; --i) {
    s += e2113(y[i]);
    for (int e = 0; e < nd; ++e) {
      double re = vec_j[2 * (i * nd + e)], im = vec_j[2 * (i * nd + e) + 1];
      if (scale != 0.0) {
        re /= scale;
        im /= scale;
      }
      // the format's trailing 1X only positions: one blank between fields
      s += " " + e2113(re) + " " + e2113(im);
    }
    s += "\n";
  }
  const int64_t need = (int64_t)s.size();
  if (buf && cap > need) std::memcpy(buf, s.c_str(), (size_t)need + 1);
  return need;
}

}  // extern "C"
