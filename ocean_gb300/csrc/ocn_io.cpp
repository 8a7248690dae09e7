// ocn_io.cpp -- the reference's file interface for this path: the bse.in
// solver settings (OCEAN2/OCEAN_driver.f90:66-70, OCEAN_haydock.f90:2109-2118,
// OCEAN_gmres.f90:84-124) and the abslanc / absspct / abs.gmres outputs
// (OCEAN_haydock.f90:1831-1892,1922-1985,2318-2358; OCEAN_gmres.f90:864-869),
// written byte for byte as the Fortran edit descriptors there produce them, so
// that existing post-processing reads the GPU results unchanged; and the
// pipeline files the hot path's operator data come from: u2.dat
// (OCEAN_bloch.f90:515-575), rpottrim.z* (long_range.f90:1689-1698),
// wvfcninfo / wvfvainfo (OCEAN_energies.f90:629-689), cksc.* / parcksc.*
// (OCEAN_multiplet.f90:414-481) and cmel<l> (OCEAN_multiplet.f90:489-500).
#include <algorithm>
#include <cctype>
#include <cstdint>
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

// Fortran sequential unformatted file as gfortran and ifort write it: each
// record is framed by its payload length as a 4-byte little-endian integer,
// before and after.  Read through a large buffer (u2.dat holds one record per
// (band, k-point, x-point)).
class SeqFile {
 public:
  explicit SeqFile(const char* path) : f_(std::fopen(path, "rb")), buf_(1 << 22) {}
  ~SeqFile() {
    if (f_) std::fclose(f_);
  }
  bool ok() const { return f_ != nullptr; }
  // next record's payload: pointer valid until the next call; false at the end
  // of the file or on a broken frame
  bool next(const unsigned char** data, uint32_t* n) {
    uint32_t n1 = 0, n2 = 0;
    if (!take(&n1, 4)) return false;
    if (n1 > (1u << 31)) return false;  // not a record length
    const unsigned char* p = view(n1);
    if (!p) return false;
    if (!take(&n2, 4) || n1 != n2) return false;
    *data = p;
    *n = n1;
    return true;
  }
  bool skip() {
    const unsigned char* d;
    uint32_t n;
    return next(&d, &n);
  }

 private:
  bool fill(size_t need) {  // at least need bytes buffered
    if (end_ - pos_ >= need) return true;
    std::memmove(buf_.data(), buf_.data() + pos_, end_ - pos_);
    end_ -= pos_;
    pos_ = 0;
    if (need > buf_.size()) buf_.resize(need);
    while (end_ < need) {
      const size_t got = std::fread(buf_.data() + end_, 1, buf_.size() - end_, f_);
      if (got == 0) return false;
      end_ += got;
    }
    return true;
  }
  bool take(void* out, size_t n) {
    if (!fill(n)) return false;
    std::memcpy(out, buf_.data() + pos_, n);
    pos_ += n;
    return true;
  }
  const unsigned char* view(size_t n) {
    if (!fill(n)) return nullptr;
    const unsigned char* p = buf_.data() + pos_;
    pos_ += n;
    return p;
  }
  FILE* f_;
  std::vector<unsigned char> buf_;
  size_t pos_ = 0, end_ = 0;
};

template <typename T>
T load(const unsigned char* p) {
  T v;
  std::memcpy(&v, p, sizeof v);
  return v;
}

// Fortran A2 of a character(len=2) variable: short names padded on the right.
std::string a2(const char* s) {
  std::string t(s);
  t.resize(2, ' ');
  return t;
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

int ocn_read_haydockconv(const char* path, double* threshold, int* spacing) {
  if (!path || !threshold || !spacing) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_haydockconv: null argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  std::vector<std::string> v;
  // read(99, *) haydockConvergeThreshold, haydockConvergeSpacing (OCEAN_system.f90:455)
  const bool ok = ld_read(f, 2, &v) && ld_real(v[0], threshold) && ld_int(v[1], spacing);
  std::fclose(f);
  if (!ok) return set_err(nullptr, OCN_ERR_ARG, "haydockconv.ipt: expected a real and an integer");
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

int ocn_write_opcons(const char* path, int ne, const double* rows) {
  if (ne < 0 || (ne > 0 && !rows)) return set_err(nullptr, OCN_ERR_ARG, "ocn_write_opcons: bad argument");
  FILE* f;
  int rc = open_out(path, &f);
  if (rc) return rc;
  // write_val (OCEAN_haydock.f90:1717-1719,1797): "(a)" header, '(8(1E24.16,1X))' rows
  put(f, "#   omega (eV)      epsilon_1       epsilon_2       n               kappa           mu (cm^(-1))    R"
         "               epsinv");
  std::string line;
  for (int r = 0; r < ne; ++r) {
    line.clear();
    for (int j = 0; j < 8; ++j) line += (j ? " " : "") + fmt_e(rows[(size_t)r * 8 + j], 24, 16);
    put(f, line);  // the trailing 1x of the last item writes nothing
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

int ocn_read_u2dat(const char* path, int nx, int ny, int nz, int nkpts, int nspn, int nband_file,
                   const int* first, int nfirst, int nbd, double* re, double* im) {
  if (!path || !first || !re || !im) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_u2dat: null argument");
  if (nx < 1 || ny < 1 || nz < 1 || nkpts < 1 || nspn < 1 || nbd < 1 || nband_file < nbd ||
      (nfirst != 1 && nfirst != nkpts * nspn))
    return set_err(nullptr, OCN_ERR_ARG, "ocn_read_u2dat: bad dimensions");
  for (int i = 0; i < nfirst; ++i)
    if (first[i] < 0 || first[i] + nbd > nband_file)
      return set_err(nullptr, OCN_ERR_ARG, "ocn_read_u2dat: band window outside the file's bands");
  SeqFile f(path);
  if (!f.ok()) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  const size_t nxyz = (size_t)nx * ny * nz;
  // OCEAN_bloch.f90:534-575: per spin, per k-point (iq1, iq2, iq3 nested), the
  // skipped bands, then nbd bands of records (ix, iy, iz with iz fastest) each
  // holding three integers and the real and imaginary parts, then the rest
  for (int s = 0; s < nspn; ++s)
    for (int iq = 0; iq < nkpts; ++iq) {
      const int f0 = first[nfirst == 1 ? 0 : iq + nkpts * s];
      for (size_t r = 0; r < (size_t)f0 * nxyz; ++r)
        if (!f.skip()) return set_err(nullptr, OCN_ERR_ARG, "u2.dat ends early or a record frame is broken");
      for (int b = 0; b < nbd; ++b)
        for (int ix = 0; ix < nx; ++ix)
          for (int iy = 0; iy < ny; ++iy)
            for (int iz = 0; iz < nz; ++iz) {
              const unsigned char* d;
              uint32_t n;
              if (!f.next(&d, &n)) return set_err(nullptr, OCN_ERR_ARG, "u2.dat ends early or a record frame is broken");
              if (n < 28) return set_err(nullptr, OCN_ERR_ARG, "u2.dat record shorter than 3 integers + 2 reals");
              // re_bloch_state(band, k, x, spin), x = ix + nx*(iy + ny*iz) (the transpose loop, :577-587)
              const size_t x = (size_t)ix + (size_t)nx * ((size_t)iy + (size_t)ny * iz);
              const size_t o = (size_t)b + (size_t)nbd * ((size_t)iq + (size_t)nkpts * (x + nxyz * s));
              re[o] = load<double>(d + 12);
              im[o] = load<double>(d + 20);
            }
      for (size_t r = 0; r < (size_t)(nband_file - f0 - nbd) * nxyz; ++r)
        if (!f.skip()) return set_err(nullptr, OCN_ERR_ARG, "u2.dat ends early or a record frame is broken");
    }
  return OCN_OK;
}

int ocn_read_u2par(const char* path, const int xmesh[3], int nkpts, int nspn, int width3, const int* first,
                   int nfirst, int nbd, double* re, double* im) {
  if (!path || !xmesh || !first || !re || !im || nkpts < 1 || nspn < 1 || nbd < 1 || width3 < nbd ||
      (nfirst != 1 && nfirst != nkpts * nspn))
    return set_err(nullptr, OCN_ERR_ARG, "ocn_read_u2par: bad argument");
  const int n1 = xmesh[0], n2 = xmesh[1], n3 = xmesh[2];
  if (n1 < 1 || n2 < 1 || n3 < 1) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_u2par: bad mesh");
  const size_t nx = (size_t)n1 * n2 * n3;
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // load_new_u2 (OCEAN_bloch.f90:697-996): a raw array of complex(DP); the states
  // of (k-point iq, spin) start at element ((iq-1) + (ispn-1) nkpts) width(3) Nx,
  // the first ivh2 bands are skipped, and each band is u2_buf(iz, iy, ix) with iz
  // fastest; it lands in re_bloch_state(band, iq, x, spin), x = ix + nx(iy + ny iz)
  std::vector<double> buf(2 * nx * (size_t)nbd);
  int rc = OCN_OK;
  for (int sp = 0; sp < nspn && rc == OCN_OK; ++sp)
    for (int k = 0; k < nkpts && rc == OCN_OK; ++k) {
      const int f0 = first[nfirst == 1 ? 0 : k + nkpts * sp];
      if (f0 < 0 || f0 + nbd > width3) {
        rc = set_err(nullptr, OCN_ERR_ARG, "u2par.dat: band window outside width(3)");
        break;
      }
      const long long off = (((long long)k + (long long)sp * nkpts) * width3 + f0) * (long long)nx * 16;
      if (std::fseek(f, (long)off, SEEK_SET) != 0 || std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) {
        rc = set_err(nullptr, OCN_ERR_ARG, "u2par.dat: file ends early");
        break;
      }
      size_t ii = 0;
      for (int b = 0; b < nbd; ++b)
        for (int ix = 0; ix < n1; ++ix)
          for (int iy = 0; iy < n2; ++iy)
            for (int iz = 0; iz < n3; ++iz, ++ii) {
              const size_t x = (size_t)ix + (size_t)n1 * ((size_t)iy + (size_t)n2 * iz);
              const size_t o = (size_t)b + (size_t)nbd * ((size_t)k + (size_t)nkpts * (x + nx * sp));
              re[o] = buf[2 * ii];
              im[o] = buf[2 * ii + 1];
            }
    }
  std::fclose(f);
  return rc;
}

int ocn_read_con_u2(const char* path, int nxpts, int nkpts, int nspn, int bands_in_file, int nbd, double* re,
                    double* im) {
  if (!path || !re || !im || nxpts < 1 || nkpts < 1 || nspn < 1 || nbd < 1 || bands_in_file < nbd)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_read_con_u2: bad argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // single_load_prefixu2dat (OCEAN_bloch.f90:998-1115): stream access, for each
  // spin, k-point and file band one complex(DP) array over the x-mesh in the
  // order the states use; bands beyond num_bands are read and dropped
  const size_t nx = (size_t)nxpts;
  std::vector<double> buf(2 * nx);
  int rc = OCN_OK;
  for (int sp = 0; sp < nspn && rc == OCN_OK; ++sp)
    for (int k = 0; k < nkpts && rc == OCN_OK; ++k)
      for (int b = 0; b < bands_in_file; ++b) {
        if (std::fread(buf.data(), sizeof(double), 2 * nx, f) != 2 * nx) {
          rc = set_err(nullptr, OCN_ERR_ARG, "con.u2.dat: file ends early");
          break;
        }
        if (b >= nbd) continue;
        for (size_t x = 0; x < nx; ++x) {
          const size_t o = (size_t)b + (size_t)nbd * ((size_t)k + (size_t)nkpts * (x + nx * sp));
          re[o] = buf[2 * x];
          im[o] = buf[2 * x + 1];
        }
      }
  std::fclose(f);
  return rc;
}

int ocn_read_obf_control(const char* path, int width[3]) {
  if (!path || !width) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_obf_control: null argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  std::vector<std::string> v;
  bool ok = true;
  for (int i = 0; i < 3 && ok; ++i) ok = ld_read(f, 1, &v) && ld_int(v[0], &width[i]);  // three read(99,*)
  std::fclose(f);
  if (!ok) return set_err(nullptr, OCN_ERR_ARG, "obf_control: expected three integers");
  return OCN_OK;
}

int ocn_read_slater(const char* path, int np, double* f, double* scale) {
  if (!path || np < 1 || !f || !scale) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_slater: bad argument");
  FILE* fh = std::fopen(path, "r");
  if (!fh) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // read(99, *) fk(:, :, k), scfk(k) (OCEAN_multiplet.f90:2094-2097): np*np values
  // in column order, then the scale factor
  std::vector<std::string> v;
  const size_t n = (size_t)np * np;
  bool ok = ld_read(fh, n + 1, &v);
  for (size_t i = 0; ok && i < n; ++i) ok = ld_real(v[i], &f[i]);
  ok = ok && ld_real(v[n], scale);
  std::fclose(fh);
  if (!ok) return set_err(nullptr, OCN_ERR_ARG, std::string("Slater file ") + path + ": expected np*np values and a scale");
  return OCN_OK;
}

int ocn_read_rpottrim(const char* path, int* nptab, double* ptab, double* rtab, int cap) {
  if (!path || !nptab) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_rpottrim: null argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // long_range.f90:1694-1698: read(99,*) dumc, nptab; then nptab records ptab, rtab
  std::vector<std::string> v;
  int n = 0;
  int rc = OCN_OK;
  if (!ld_read(f, 2, &v) || !ld_int(v[1], &n) || n < 1) rc = set_err(nullptr, OCN_ERR_ARG, "rpottrim: bad header");
  if (rc == OCN_OK) {
    *nptab = n;
    if (ptab || rtab) {
      if (n > cap) rc = set_err(nullptr, OCN_ERR_ARG, "rpottrim: table longer than cap");
      for (int i = 0; i < n && rc == OCN_OK; ++i) {
        double p = 0.0, r = 0.0;
        if (!ld_read(f, 2, &v) || !ld_real(v[0], &p) || !ld_real(v[1], &r))
          rc = set_err(nullptr, OCN_ERR_ARG, "rpottrim: bad table record");
        if (ptab) ptab[i] = p;
        if (rtab) rtab[i] = r;
      }
    }
  }
  std::fclose(f);
  return rc;
}

int ocn_read_energies(const char* path, int nspn, int* nbd, int* nq, double* e, size_t cap) {
  if (!path || !nbd || !nq || (nspn != 1 && nspn != 2))
    return set_err(nullptr, OCN_ERR_ARG, "ocn_read_energies: bad argument");
  SeqFile f(path);
  if (!f.ok()) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // OCEAN_energies.f90:657-676: (nbd, nq) or, with two spins, (nbd, nq, nspn); then energies(nbd, nq, nspn)
  const unsigned char* d;
  uint32_t n;
  if (!f.next(&d, &n) || n < (nspn == 2 ? 12u : 8u)) return set_err(nullptr, OCN_ERR_ARG, "energy file: bad header");
  *nbd = load<int32_t>(d);
  *nq = load<int32_t>(d + 4);
  if (nspn == 2 && load<int32_t>(d + 8) != 2) return set_err(nullptr, OCN_ERR_ARG, "energy file: spin mismatch");
  if (*nbd < 1 || *nq < 1) return set_err(nullptr, OCN_ERR_ARG, "energy file: bad header");
  if (!e) return OCN_OK;
  const size_t cnt = (size_t)*nbd * *nq * nspn;
  if (cnt > cap) return set_err(nullptr, OCN_ERR_ARG, "energy file: more values than cap");
  if (!f.next(&d, &n) || n < cnt * sizeof(double)) return set_err(nullptr, OCN_ERR_ARG, "energy file: bad energy record");
  std::memcpy(e, d, cnt * sizeof(double));
  return OCN_OK;
}

int ocn_read_val_u2(const char* path, const int xmesh[3], int nkpts, int nspn, int file_b0, int file_b1,
                    int band_lo, int nb, double* re, double* im) {
  if (!path || !xmesh || !re || !im || nkpts < 1 || nspn < 1 || nb < 1 || file_b1 < file_b0 ||
      band_lo < file_b0 || band_lo + nb - 1 > file_b1)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_read_val_u2: bad argument");
  const int n1 = xmesh[0], n2 = xmesh[1], n3 = xmesh[2];
  if (n1 < 1 || n2 < 1 || n3 < 1) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_val_u2: bad mesh");
  const size_t nx = (size_t)n1 * n2 * n3;
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // load_single_prefixu2dat (OCEAN_val_states.f90:421-560): stream access, for
  // each spin, k-point and file band one complex(DP) array over the x-mesh with
  // x1 fastest; bands outside [band_lo, band_lo + nb) are skipped; the arrays
  // land in re_val / re_con(x, band, k, spin) with x3 fastest
  std::vector<double> buf(2 * nx);
  int rc = OCN_OK;
  for (int sp = 0; sp < nspn && rc == OCN_OK; ++sp)
    for (int k = 0; k < nkpts && rc == OCN_OK; ++k)
      for (int b = file_b0; b <= file_b1 && rc == OCN_OK; ++b) {
        if (std::fread(buf.data(), sizeof(double), 2 * nx, f) != 2 * nx) {
          rc = set_err(nullptr, OCN_ERR_ARG, "val/con u2: file ends early");
          break;
        }
        if (b < band_lo || b >= band_lo + nb) continue;
        const size_t base = nx * ((size_t)(b - band_lo) + (size_t)nb * ((size_t)k + (size_t)nkpts * sp));
        size_t ii = 0;
        for (int iz = 0; iz < n3; ++iz)
          for (int iy = 0; iy < n2; ++iy)
            for (int ix = 0; ix < n1; ++ix, ++ii) {
              const size_t x = (size_t)iz + (size_t)n3 * ((size_t)iy + (size_t)n2 * ix);
              re[base + x] = buf[2 * ii];
              im[base + x] = buf[2 * ii + 1];
            }
      }
  std::fclose(f);
  return rc;
}

int ocn_val_pair_energies(int nc, int nv, int nkpts, int nspn, int vspin, const double* con_e, int ncon_file,
                          int con_lo, const double* val_e, int nval_file, int val_lo, double* out) {
  if (nc < 1 || nv < 1 || nkpts < 1 || (nspn != 1 && nspn != 2) || (vspin != 1 && vspin != 2) || !con_e ||
      !val_e || !out || con_lo < 1 || val_lo < 1 || con_lo + nc - 1 > ncon_file || val_lo + nv - 1 > nval_file)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_val_pair_energies: bad argument");
  // OCEAN_read_energies (OCEAN_val_energy.f90:266-296, nbw = 1): block ibeta
  // pairs valence spin i with conduction spin j, E = e_c - e_v
  size_t o = 0;
  for (int i = 0; i < vspin; ++i) {
    const int is = std::min(i, nspn - 1);
    for (int j = 0; j < vspin; ++j) {
      const int js = std::min(j, nspn - 1);
      for (int k = 0; k < nkpts; ++k)
        for (int v = 0; v < nv; ++v)
          for (int c = 0; c < nc; ++c, ++o)
            out[o] = con_e[(size_t)(c + con_lo - 1) + (size_t)ncon_file * ((size_t)k + (size_t)nkpts * js)] -
                     val_e[(size_t)(v + val_lo - 1) + (size_t)nval_file * ((size_t)k + (size_t)nkpts * is)];
    }
  }
  return OCN_OK;
}

int ocn_read_cks(const char* path, int stream, int nptot, int nb, int nkpts, int nspn, double* pcr, double* pci) {
  if (!path || !pcr || !pci || nptot < 1 || nb < 1 || nkpts < 1 || nspn < 1)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_read_cks: bad argument");
  const size_t per_b = (size_t)nptot;
  if (stream) {
    // parcksc.*: stream access, three integers (the second nbd*nkpts) then
    // complex(DP) pcTemp(nptot, nbd, nkpts, nspn) (OCEAN_multiplet.f90:430-452)
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
    int32_t h[3];
    int rc = OCN_OK;
    if (std::fread(h, 4, 3, f) != 3) rc = set_err(nullptr, OCN_ERR_ARG, "cks: short header");
    const int nbd = rc == OCN_OK ? h[1] / nkpts : 0;
    if (rc == OCN_OK && (h[1] != nbd * nkpts || nbd < nb)) rc = set_err(nullptr, OCN_ERR_ARG, "Badly formed cks");
    std::vector<double> band(2 * per_b);
    for (int s = 0; s < nspn && rc == OCN_OK; ++s)
      for (int k = 0; k < nkpts && rc == OCN_OK; ++k)
        for (int b = 0; b < nbd && rc == OCN_OK; ++b) {
          if (std::fread(band.data(), sizeof(double), 2 * per_b, f) != 2 * per_b) {
            rc = set_err(nullptr, OCN_ERR_ARG, "cks: file ends early");
            break;
          }
          if (b >= nb) continue;  // only the first num_bands are used (:444-450)
          const size_t o = per_b * ((size_t)b + (size_t)nb * ((size_t)k + (size_t)nkpts * s));
          for (size_t p = 0; p < per_b; ++p) {
            pcr[o + p] = band[2 * p];
            pci[o + p] = band[2 * p + 1];
          }
        }
    std::fclose(f);
    return rc;
  }
  // cksc.*: two records skipped, then pcr and pci (nptot, nb, nkpts, nspn) (:456-461)
  SeqFile f(path);
  if (!f.ok()) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  const size_t cnt = per_b * nb * nkpts * nspn;
  if (!f.skip() || !f.skip()) return set_err(nullptr, OCN_ERR_ARG, "cks: missing header records");
  const unsigned char* d;
  uint32_t n;
  for (double* out : {pcr, pci}) {
    if (!f.next(&d, &n) || n < cnt * sizeof(double)) return set_err(nullptr, OCN_ERR_ARG, "cks: bad coefficient record");
    std::memcpy(out, d, cnt * sizeof(double));
  }
  return OCN_OK;
}

int ocn_cks_to_mpc(int lmin, int lmax, const int* nproj, int nb, int nkpts, int nspn, const double* pcr,
                   const double* pci, double* mpcr, double* mpci) {
  if (!nproj || !pcr || !pci || !mpcr || !mpci || lmin < 0 || lmax < lmin)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_cks_to_mpc: bad argument");
  int npmax = 0, nptot = 0;
  for (int l = lmin; l <= lmax; ++l) {
    if (nproj[l - lmin] < 0) return set_err(nullptr, OCN_ERR_ARG, "ocn_cks_to_mpc: negative projector count");
    npmax = std::max(npmax, nproj[l - lmin]);
    nptot += (2 * l + 1) * nproj[l - lmin];
  }
  const int nm = 2 * lmax + 1, nl = lmax - lmin + 1;
  const size_t total = (size_t)nb * nkpts * npmax * nm * nl * nspn;
  std::fill(mpcr, mpcr + total, 0.0);
  std::fill(mpci, mpci + total, 0.0);
  // OCEAN_multiplet.f90:466-481: ip runs over l, m = -l..l, nu
  for (int s = 0; s < nspn; ++s)
    for (int k = 0; k < nkpts; ++k)
      for (int b = 0; b < nb; ++b) {
        int ip = 0;
        const size_t src = (size_t)nptot * ((size_t)b + (size_t)nb * ((size_t)k + (size_t)nkpts * s));
        for (int l = lmin; l <= lmax; ++l)
          for (int m = -l; m <= l; ++m)
            for (int nu = 0; nu < nproj[l - lmin]; ++nu, ++ip) {
              const size_t dst = (size_t)b + (size_t)nb * ((size_t)k + (size_t)nkpts * ((size_t)nu + (size_t)npmax *
                                 ((size_t)(m + lmax) + (size_t)nm * ((size_t)(l - lmin) + (size_t)nl * s))));
              mpcr[dst] = pcr[src + ip];
              mpci[dst] = pci[src + ip];
            }
      }
  return OCN_OK;
}

int ocn_read_cmel(const char* path, int nproj, double* mpm) {
  if (!path || !mpm || nproj < 1) return set_err(nullptr, OCN_ERR_ARG, "ocn_read_cmel: bad argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_err(nullptr, OCN_ERR_ARG, std::string("cannot open ") + path);
  // OCEAN_multiplet.f90:493-499: list-directed nproj*nproj values; column nu of
  // mpm(:, :, l) takes values nu*nproj .. nu*nproj + nproj - 1
  std::vector<std::string> v;
  int rc = OCN_OK;
  if (!ld_read(f, (size_t)nproj * nproj, &v)) rc = set_err(nullptr, OCN_ERR_ARG, "cmel: too few values");
  for (int i = 0; i < nproj * nproj && rc == OCN_OK; ++i)
    if (!ld_real(v[i], &mpm[i])) rc = set_err(nullptr, OCN_ERR_ARG, "cmel: bad value");
  std::fclose(f);
  return rc;
}

int ocn_input_filename(const char* kind, const char* calc_type, const char* elname, int indx, int n, int l,
                       char* buf, size_t len) {
  if (!kind || !elname || !buf || len == 0) return set_err(nullptr, OCN_ERR_ARG, "ocn_input_filename: null argument");
  if (indx < 0 || indx > 9999 || n < 0 || n > 99 || l < 0 || l > 99)
    return set_err(nullptr, OCN_ERR_ARG, "index outside the I4.4 / I2.2 range");
  const std::string k(kind), ct(calc_type ? calc_type : "XAS");
  char tail[32];
  std::string name;
  if (k == "rpottrim") {
    // long_range.f90:1689-1690: '(A10,A2,I4.4,A2,I2.2,A1,I2.2)'
    std::snprintf(tail, sizeof tail, "%04d_n%02dl%02d", indx, n, l);
    name = "rpottrim.z" + a2(elname) + tail;
  } else if (k == "cks" || k == "parcks") {
    // OCEAN_multiplet.f90:417-428,454: 'cksc.' (cksv. for XES) + '(A2,I4.4)', 'par' in front for the stream file
    std::snprintf(tail, sizeof tail, "%04d", indx);
    name = std::string(k == "parcks" ? "par" : "") + (ct == "XES" ? "cksv." : "cksc.") + a2(elname) + tail;
  } else if (k == "cmel") {
    if (l > 9) return set_err(nullptr, OCN_ERR_ARG, "l exceeds 9 in multip");  // :491
    std::snprintf(tail, sizeof tail, "cmel%d", l);
    name = tail;
  } else if (k == "energies") {
    name = ct == "VAL" ? "wvfvainfo" : "wvfcninfo";  // OCEAN_energies.f90:650-654 (conduct)
  } else {
    return set_err(nullptr, OCN_ERR_ARG, "kind must be rpottrim, cks, parcks, cmel or energies");
  }
  if (name.size() + 1 > len) return set_err(nullptr, OCN_ERR_ARG, "buffer too small");
  std::memcpy(buf, name.c_str(), name.size() + 1);
  return OCN_OK;
}

}  // extern "C"
