// ocn_io.cpp -- the reference's text interface for this path: the bse.in
// solver settings (OCEAN2/OCEAN_driver.f90:66-70, OCEAN_haydock.f90:2109-2118,
// OCEAN_gmres.f90:84-124) and the abslanc / absspct / abs.gmres outputs
// (OCEAN_haydock.f90:1831-1892,1922-1985,2318-2358; OCEAN_gmres.f90:864-869),
// written byte for byte as the Fortran edit descriptors there produce them, so
// that existing post-processing reads the GPU results unchanged.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ocn_internal.h"

namespace ocn {
namespace {

// Fortran Iw: right-justified, asterisks when the value does not fit.
std::string fmt_i(long long v, int w) {
  char b[64];
  std::snprintf(b, sizeof b, "%*lld", w, v);
  std::string s(b);
  if ((int)s.size() > w) return std::string(w, '*');
  return s;
}

std::string right(const std::string& s, int w) {
  if ((int)s.size() >= w) return s.substr(0, w);
  return std::string(w - s.size(), ' ') + s;
}

// Non-finite values as gfortran writes them in a field of width w.
bool nonfinite(double x, int w, std::string* out) {
  if (std::isnan(x)) {
    *out = right("NaN", w);
    return true;
  }
  if (std::isinf(x)) {
    const std::string s = x < 0 ? (w >= 9 ? "-Infinity" : "-Inf") : (w >= 8 ? "Infinity" : "Inf");
    *out = right(s, w);
    return true;
  }
  return false;
}

// Correctly rounded significant digits and decimal exponent of |x|:
// |x| = 0.d1 d2 ... dn x 10^e10 (digits has n characters).
void sig_digits(double ax, int n, std::string* digits, int* e10) {
  if (ax == 0.0) {
    *digits = std::string(n, '0');
    *e10 = 0;
    return;
  }
  char b[64];
  std::snprintf(b, sizeof b, "%.*E", n - 1, ax);  // d.ddddE+xx
  std::string m;
  const char* p = b;
  for (; *p && *p != 'E'; ++p)
    if (*p != '.') m += *p;
  *digits = m;
  *e10 = std::atoi(p + 1) + 1;
}

// Exponent part of an E / ES field: E+dd, or +ddd without the letter when
// |exp| > 99 (the Fortran rule for Ew.d without Ee).
std::string exp_part(int e) {
  char b[16];
  if (std::abs(e) <= 99) std::snprintf(b, sizeof b, "E%c%02d", e < 0 ? '-' : '+', std::abs(e));
  else std::snprintf(b, sizeof b, "%c%03d", e < 0 ? '-' : '+', std::abs(e));
  return b;
}

// Fortran Ew.d with scale factor k = 0 (0.ddd form) or k = 1 (1P: d.ddd form).
std::string fmt_e(double x, int w, int d, int k = 0) {
  std::string out;
  if (nonfinite(x, w, &out)) return out;
  const bool neg = std::signbit(x);
  std::string dig;
  int e10;
  const int nsig = (k == 0) ? d : d + 1;
  sig_digits(std::fabs(x), nsig, &dig, &e10);
  std::string body;
  if (k == 0) {
    body = "0." + dig;
  } else {
    body = dig.substr(0, 1) + "." + dig.substr(1);
    if (x != 0.0) e10 -= 1;
  }
  std::string s = (neg ? "-" : "") + body + exp_part(x == 0.0 ? 0 : e10);
  if ((int)s.size() > w && k == 0 && s.compare(neg ? 1 : 0, 1, "0") == 0) s.erase(neg ? 1 : 0, 1);  // drop the optional 0
  if ((int)s.size() > w) return std::string(w, '*');
  return right(s, w);
}

// Fortran ESw.d: d.ddd...E+ee with d digits after the point.
std::string fmt_es(double x, int w, int d) { return fmt_e(x, w, d, 1); }

// Fortran Fw.d.
std::string fmt_f(double x, int w, int d) {
  std::string out;
  if (nonfinite(x, w, &out)) return out;
  char b[512];
  std::snprintf(b, sizeof b, "%.*f", d, x);
  std::string s(b);
  if ((int)s.size() > w) return std::string(w, '*');
  return right(s, w);
}

// ---- list-directed input (the subset bse.in uses)

// Splits a record into values: blanks and commas separate, quotes delimit
// character values, a slash ends the record, Fortran D exponents read as E.
std::vector<std::string> ld_values(const std::string& line) {
  std::vector<std::string> v;
  size_t i = 0;
  while (i < line.size()) {
    const char ch = line[i];
    if (ch == ' ' || ch == '\t' || ch == ',' || ch == '\r' || ch == '\n') {
      ++i;
      continue;
    }
    if (ch == '/') break;
    std::string tok;
    if (ch == '\'' || ch == '"') {
      const char q = ch;
      ++i;
      while (i < line.size() && line[i] != q) tok += line[i++];
      ++i;
    } else {
      while (i < line.size() && line[i] != ' ' && line[i] != '\t' && line[i] != ',' && line[i] != '/' &&
             line[i] != '\r' && line[i] != '\n')
        tok += line[i++];
    }
    v.push_back(tok);
  }
  return v;
}

bool ld_real(const std::string& t, double* out) {
  std::string s = t;
  for (char& c : s)
    if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'E';
  char* end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  if (s.empty() || (end && *end)) return false;
  *out = v;
  return true;
}

bool ld_int(const std::string& t, int* out) {
  char* end = nullptr;
  const long v = std::strtol(t.c_str(), &end, 10);
  if (t.empty() || (end && *end)) return false;
  *out = (int)v;
  return true;
}

// Reads records until n values are collected (list-directed input continues
// onto the next record when one runs short).
bool ld_read(FILE* f, size_t n, std::vector<std::string>* vals) {
  vals->clear();
  char buf[4096];
  while (vals->size() < n) {
    if (!std::fgets(buf, sizeof buf, f)) return false;
    std::string line(buf);
    const bool slash = line.find('/') != std::string::npos;
    for (auto& t : ld_values(line)) vals->push_back(t);
    if (slash) break;
  }
  return vals->size() >= n;
}

}  // namespace
}  // namespace ocn

using namespace ocn;

namespace {

constexpr double kEv2Ha = 0.036749322175666;   // OCEAN2/OCEAN_constants.f90
constexpr double kHa2Ev = 27.211386245980;

// Fortran A edit of a character(len=w) value written with An.
std::string fmt_a(const std::string& s, int w) { return right(s, w); }

int open_out(const char* path, FILE** f) {
  if (!path) return set_err(nullptr, OCN_ERR_ARG, "null path");
  *f = std::fopen(path, "w");
  if (!*f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  return OCN_OK;
}

int close_out(FILE* f, const char* path) {
  const bool bad = std::ferror(f) != 0;
  if (std::fclose(f) != 0 || bad) return set_err(nullptr, OCN_ERR_ARG, std::string("write failed: ") + path);
  return OCN_OK;
}

void put(FILE* f, const std::string& s) {
  std::fputs(s.c_str(), f);
  std::fputc('\n', f);
}

}  // namespace

extern "C" {

int ocn_read_bse_in(const char* path, ocn_bse_in* out, double* energies, int cap) {
  if (!path || !out) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_bse_in: null argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  ocn_bse_in b;
  std::memset(&b, 0, sizeof b);
  std::vector<std::string> v;
  auto fail = [&](const char* what) {
    std::fclose(f);
    return set_err(nullptr, OCN_ERR_ARG, std::string("bse.in: ") + what);
  };
  // records 1-3 (OCEAN_driver.f90:67-69): an integer, a real, the solver style
  if (!ld_read(f, 1, &v) || !ld_int(v[0], &b.dumi)) return fail("record 1 (integer)");
  if (!ld_read(f, 1, &v) || !ld_real(v[0], &b.dumf)) return fail("record 2 (real)");
  if (!ld_read(f, 1, &v)) return fail("record 3 (style)");
  std::snprintf(b.style, sizeof b.style, "%.4s", v[0].c_str());  // character(len=4)
  const std::string style(b.style);
  if (style == "hay") {
    // OCEAN_haydock.f90:2118: niter, ne, el, eh, gam0, ebase (eV)
    if (!ld_read(f, 6, &v) || !ld_int(v[0], &b.niter) || !ld_int(v[1], &b.ne) || !ld_real(v[2], &b.el) ||
        !ld_real(v[3], &b.eh) || !ld_real(v[4], &b.gam0) || !ld_real(v[5], &b.ebase))
      return fail("record 4 (niter, ne, el, eh, gam0, ebase)");
  } else if (style == "inv") {
    // OCEAN_gmres.f90:89-124: depth, resolution, preconditioner, convergence; list | loop
    if (!ld_read(f, 4, &v) || !ld_int(v[0], &b.depth) || !ld_real(v[1], &b.resolution) ||
        !ld_real(v[2], &b.preconditioner) || !ld_real(v[3], &b.convergence))
      return fail("record 4 (depth, resolution, preconditioner, convergence)");
    if (!ld_read(f, 1, &v)) return fail("record 5 (list | loop)");
    std::snprintf(b.inv_style, sizeof b.inv_style, "%.4s", v[0].c_str());
    const std::string is(b.inv_style);
    if (is == "list") {
      if (!ld_read(f, 1, &v) || !ld_int(v[0], &b.nomega) || b.nomega < 0) return fail("energy count");
      for (int i = 0; i < b.nomega; ++i) {
        double e;
        if (!ld_read(f, 1, &v) || !ld_real(v[0], &e)) return fail("energy list");
        if (energies && i < cap) energies[i] = e;
      }
    } else if (is == "loop") {
      double e0, e1, de;
      if (!ld_read(f, 3, &v) || !ld_real(v[0], &e0) || !ld_real(v[1], &e1) || !ld_real(v[2], &de) || de == 0.0)
        return fail("energy loop (start, stop, step)");
      b.nomega = 1 + (int)std::ceil((e1 - e0 - de * 0.0001) / de);
      if (b.nomega < 0) b.nomega = 0;
      for (int i = 0; i < b.nomega && energies && i < cap; ++i) energies[i] = e0 + (double)i * de;
    } else {
      return fail("unsupported energy point style");
    }
  } else if (style != "exa" && style != "dia") {
    return fail("unsupported style");
  }
  std::fclose(f);
  *out = b;
  if (energies && b.nomega > cap) return set_err(nullptr, OCN_ERR_ARG, "bse.in: energy buffer too small");
  return OCN_OK;
}

int ocn_write_abslanc(const char* path, int n, double kpref, const double* real_a, const double* imag_a,
                      const double* real_b, const double* imag_b, const double* real_c, const double* imag_c,
                      const double* eigs) {
  if (n < 0 || !real_a || !real_b) return set_err(nullptr, OCN_ERR_ARG, "ocn_write_abslanc: bad argument");
  FILE* f;
  int rc = open_out(path, &f);
  if (rc) return rc;
  auto im = [](const double* p, int i) { return p ? p[i] : 0.0; };
  // write_lanczos (OCEAN_haydock.f90:2335-2355)
  put(f, fmt_i(n, 8) + " " + fmt_es(kpref, 24, 17));
  if (imag_a) {  // complex_haydock
    put(f, "  " + fmt_es(real_a[0], 24, 17) + "  " + fmt_es(imag_a[0], 24, 17));
    for (int i = 1; i <= n; ++i) {
      const double rc_ = real_c ? real_c[i] : real_b[i];
      const double ic = imag_c ? imag_c[i] : im(imag_b, i);
      put(f, "  " + fmt_es(real_a[i], 24, 17) + fmt_es(imag_a[i], 24, 17) + fmt_es(real_b[i], 24, 17) +
                 fmt_es(im(imag_b, i), 24, 17) + fmt_es(rc_, 24, 17) + fmt_es(ic, 24, 17));
    }
  } else {
    put(f, "  " + fmt_es(real_a[0], 24, 17));
    for (int i = 1; i <= n; ++i) put(f, "  " + fmt_es(real_a[i], 24, 17) + "  " + fmt_es(real_b[i], 24, 17));
  }
  if (eigs)  // redtrid's eigenvalues, '(2x,2i5,1f20.10)'
    for (int i = 1; i <= n + 1; ++i) put(f, "  " + fmt_i(i, 5) + fmt_i(n + 1, 5) + fmt_f(eigs[i - 1], 20, 10));
  return close_out(f, path);
}

int ocn_write_absspct(const char* path, int iter, double gam0, double kpref, double ucvol, int ne,
                      const double* rows, int voigt) {
  if (ne < 0 || !rows) return set_err(nullptr, OCN_ERR_ARG, "ocn_write_absspct: bad argument");
  FILE* f;
  int rc = open_out(path, &f);
  if (rc) return rc;
  const int ncol = voigt ? 5 : 9;
  // write_core (OCEAN_haydock.f90:1831-1833,1890-1891), write_core_Voigt (:1922-1923,1985)
  std::string h = "#   iter=" + fmt_i(iter, 5) + "   gam=" + fmt_e(gam0, 15, 8) + "   kpref=" + fmt_e(kpref, 15, 8);
  if (!voigt) h += "vol=" + fmt_e(ucvol, 15, 8);
  put(f, h);
  static const char* names[9] = {"#   Energy",     "Spect",         "Spect(0)",        "SPKK",           "SPKK(0)",
                                 "sigma (a.u.^2)", "sigma( cm^2 )", "sig.^2 (a.u.^5)", "sig.^2 cm^4 sec"};
  std::string line;
  for (int j = 0; j < ncol; ++j) line += (j ? " " : "") + fmt_a(names[j], 15);
  put(f, line);  // the trailing 1x of the last item writes nothing
  for (int r = 0; r <= ne; ++r) {
    line.clear();
    for (int j = 0; j < ncol; ++j) line += (j ? " " : "") + fmt_e(rows[(size_t)r * 9 + j], 15, 8);
    put(f, line);
  }
  return close_out(f, path);
}

int ocn_write_abs_gmres(const char* path, int nomega, const double* energies_ev, const double* out_re,
                        const double* out_im, const double* rel_err, const int* iters) {
  if (nomega < 0 || !energies_ev || !out_re || !out_im || !rel_err || !iters)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_write_abs_gmres: bad argument");
  FILE* f;
  int rc = open_out(path, &f);
  if (rc) return rc;
  long long global_iter = 0;
  for (int i = 0; i < nomega; ++i) {
    global_iter += iters[i];
    // OCEAN_gmres.f90:866: '(1p,4(1e15.8,1x),1i6,1x,i10)', energy through Hartree and back
    const double ener = energies_ev[i] * kEv2Ha;
    put(f, fmt_e(ener * kHa2Ev, 15, 8, 1) + " " + fmt_e(out_re[i], 15, 8, 1) + " " + fmt_e(out_im[i], 15, 8, 1) +
               " " + fmt_e(rel_err[i], 15, 8, 1) + " " + fmt_i(iters[i], 6) + " " + fmt_i(global_iter, 10));
  }
  return close_out(f, path);
}

int ocn_output_filename(const char* kind, const char* calc_type, const char* elname, int indx,
                        const char* corelevel, int photon, char* buf, size_t len) {
  if (!kind || !calc_type || !elname || !corelevel || !buf || len == 0)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_output_filename: null argument");
  const std::string k(kind), ct(calc_type);
  if (k != "spct" && k != "lanc") return set_err(nullptr, OCN_ERR_ARG, "kind must be spct or lanc");
  if (ct == "RXS" || ct == "C2C" || ct == "VAL")
    return set_err(nullptr, OCN_ERR_UNSUPPORTED, "only core-level XAS / XES file names");
  // OCEAN_filenames.f90:21-107: '(A8,A2,A1,I4.4,A1,A2,A1,I2.2)'
  const std::string pre = std::string(ct == "XES" ? "xes" : "abs") + k + "_";
  char tail[64];
  if (indx < 0 || indx > 9999 || photon < 0 || photon > 99)
    return set_err(nullptr, OCN_ERR_ARG, "site index or photon out of the I4.4 / I2.2 range");
  std::snprintf(tail, sizeof tail, ".%04d_%s_%02d", indx, fmt_a(corelevel, 2).c_str(), photon);
  const std::string name = pre + fmt_a(elname, 2) + tail;
  if (name.size() + 1 > len) return set_err(nullptr, OCN_ERR_ARG, "buffer too small");
  std::memcpy(buf, name.c_str(), name.size() + 1);
  return OCN_OK;
}

}  // extern "C"
