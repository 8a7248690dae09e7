// ocean_oracle.cpp -- CPU ORACLE (test infrastructure only; never linked into the
// product library).  A plain FP64 restatement of the reference Fortran for the
// OCEAN core-level BSE hot path.  Every routine cites the reference file:line it
// follows.  Build: oracle/Makefile (g++ -O3 -fopenmp -ffp-contract=off).
//
// Parity status: write_core/redtrid pinned against EXAMPLE/Cu_TwoPhoton golden
// files; the action, Lanczos and GMRES follow the cited source and are pinned by
// structural checks only (the reference ships no u2/W/projector inputs).

#include "ocean_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <functional>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cd;

// OCEAN2/OCEAN_constants.f90:15-30
const double kEV2Ha = 0.036749322175666;
const double kHa2eV = 27.211386245980;
const double kAlpha = 0.0072973525643;
const double kBohr = 0.529177210544;
const double kAu2sec = 2.4188843265864e-17;
const double kPi = 3.1415926535897932384626433832795028841971693993751;

inline int nk_of(const or_dims* d) { return d->kmesh[0] * d->kmesh[1] * d->kmesh[2]; }
inline int nx_of(const or_dims* d) { return d->xmesh[0] * d->xmesh[1] * d->xmesh[2]; }

// Smith's complex division; the product library's continued-fraction kernel uses
// the same formula so the two agree to the last bit.
inline cd cdiv(cd n, cd d) {
  double dr = d.real(), di = d.imag();
  if (std::fabs(dr) >= std::fabs(di)) {
    double r = di / dr;
    double t = 1.0 / (dr + di * r);
    return cd((n.real() + n.imag() * r) * t, (n.imag() - n.real() * r) * t);
  }
  double r = dr / di;
  double t = 1.0 / (dr * r + di);
  return cd((n.real() * r + n.imag()) * t, (n.imag() * r - n.real()) * t);
}

// Principal complex square root, same formula as the product library.
inline cd csqrt_p(cd z) {
  double x = z.real(), y = z.imag();
  if (x == 0.0 && y == 0.0) return cd(0.0, y);
  double t = std::sqrt((std::fabs(x) + std::sqrt(x * x + y * y)) * 0.5);
  if (x >= 0.0) return cd(t, y / (2.0 * t));
  return cd(std::fabs(y) / (2.0 * t), std::copysign(t, y));
}

inline cd cmul(cd a, cd b) {
  return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}

// Fortran cmplx(x, y) without KIND returns default (single precision) complex;
// OCEAN_haydock.f90:1837,1868-1869 rely on that, so restate it.
inline cd cmplx_sp(double x, double y) { return cd((double)(float)x, (double)(float)y); }
inline cd cmul_sp(double ar, double ai, double br, double bi) {
  float a = (float)ar, b = (float)ai, c = (float)br, e = (float)bi;
  float re = a * c - b * e;
  float im = a * e + b * c;
  return cd((double)re, (double)im);
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------ setup

// OCEAN_bloch_lrLOAD, OCEAN2/OCEAN_bloch.f90:54-219.
int or_lrload(const or_dims* d, double tau[3], const int ovr[3], int xshift[3], double* ur,
              double* ui) {
  const int nb = d->nb, nk = nk_of(d), nx = nx_of(d);
  const double pi = 4.0 * std::atan(1.0);
  for (int i = 0; i < 3; ++i) {
    if (d->kmesh[i] % 2 == 0)
      xshift[i] = (int)std::floor((double)d->xmesh[i] * tau[i]);
    else
      xshift[i] = (int)std::floor((double)d->xmesh[i] * (tau[i] - 0.5));
    xshift[i] *= (ovr ? ovr[i] : 1);
  }
  for (int i = 0; i < 3; ++i) tau[i] = tau[i] - (double)xshift[i] / (double)d->xmesh[i];
  if (!ur) return 0;
  for (int s = 0; s < d->nspn; ++s) {
    int xiter = 0;
    for (int iz = 1; iz <= d->xmesh[2]; ++iz) {
      int ztarg = iz - xshift[2], zph = 0;
      if (ztarg > d->xmesh[2]) zph = -d->xmesh[2];
      else if (ztarg < 1) zph = d->xmesh[2];
      for (int iy = 1; iy <= d->xmesh[1]; ++iy) {
        int ytarg = iy - xshift[1], yph = 0;
        if (ytarg > d->xmesh[1]) yph = -d->xmesh[1];
        else if (ytarg < 1) yph = d->xmesh[1];
        for (int ix = 1; ix <= d->xmesh[0]; ++ix) {
          int xtarg = ix - xshift[0], xph = 0;
          if (xtarg > d->xmesh[0]) xph = -d->xmesh[0];
          else if (xtarg < 1) xph = d->xmesh[0];
          int iq = 0;
          for (int iq1 = 1; iq1 <= d->kmesh[0]; ++iq1)
            for (int iq2 = 1; iq2 <= d->kmesh[1]; ++iq2)
              for (int iq3 = 1; iq3 <= d->kmesh[2]; ++iq3) {
                double phsx = 2.0 * pi * (double)((xph + ix - 1) * (iq1 - 1)) /
                              (double)(d->xmesh[0] * d->kmesh[0]);
                double phsy = 2.0 * pi * (double)((yph + iy - 1) * (iq2 - 1)) /
                              (double)(d->xmesh[1] * d->kmesh[1]);
                double phsz = 2.0 * pi * (double)((zph + iz - 1) * (iq3 - 1)) /
                              (double)(d->xmesh[2] * d->kmesh[2]);
                double c = std::cos(phsx + phsy + phsz);
                double sn = std::sin(phsx + phsy + phsz);
                size_t base = (size_t)nb * ((size_t)iq + (size_t)nk * ((size_t)xiter + (size_t)nx * s));
                for (int n = 0; n < nb; ++n) {
                  double r = ur[base + n], im = ui[base + n];
                  ur[base + n] = c * r - sn * im;
                  ui[base + n] = c * im + sn * r;
                }
                ++iq;
              }
          ++xiter;
        }
      }
    }
  }
  return 0;
}

// intval(..., 'cap', 'cap'), CNBSE/zcmsnmult/zf90/intval.f90:8-60.
double or_intval(int n, const double* xtab, const double* ytab, double x) {
  if (x < xtab[0]) return ytab[0];
  if (x > xtab[n - 1]) return ytab[n - 1];
  int ii = 0;
  while (xtab[ii + 1] < x) ++ii;
  double rat = (x - xtab[ii]) / (xtab[ii + 1] - xtab[ii]);
  return ytab[ii] + rat * (ytab[ii + 1] - ytab[ii]);
}

// lr_populate_W2, OCEAN2/long_range.f90:1659-1853 (single rank: my_start_nx = 1).
int or_populate_w2(const or_dims* d, const or_lr_in* p, const double tau[3], const int xshift[3],
                   double* W) {
  const int nk = nk_of(d);
  double epsi = 1.0 / p->epsilon0;
  double amet[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int c = 0; c < 3; ++c) s += p->avec[c + 3 * i] * p->avec[c + 3 * j];
      amet[i][j] = s;
    }
  int pbc[3];
  bool have_pbc = (p->pbc[0] | p->pbc[1] | p->pbc[2]) != 0;
  for (int i = 0; i < 3; ++i) {
    if (have_pbc) pbc[i] = p->pbc[i] != 0 ? d->kmesh[i] : 0;
    else pbc[i] = d->kmesh[i];
  }
  const double rmax = p->rtab[p->nptab - 1];
  int xiter = 0;
  double fr[3], xk[3], alf[3], pref[3];
  for (int iz = 1; iz <= d->xmesh[2]; ++iz) {
    int zt = iz - xshift[2];
    if (zt > d->xmesh[2]) zt -= d->xmesh[2];
    else if (zt < 1) zt += d->xmesh[2];
    fr[2] = (double)(zt - 1) / (double)d->xmesh[2];
    for (int iy = 1; iy <= d->xmesh[1]; ++iy) {
      int yt = iy - xshift[1];
      if (yt > d->xmesh[1]) yt -= d->xmesh[1];
      else if (yt < 1) yt += d->xmesh[1];
      fr[1] = (double)(yt - 1) / (double)d->xmesh[1];
      for (int ix = 1; ix <= d->xmesh[0]; ++ix) {
        int xt = ix - xshift[0];
        if (xt > d->xmesh[0]) xt -= d->xmesh[0];
        else if (xt < 1) xt += d->xmesh[0];
        fr[0] = (double)(xt - 1) / (double)d->xmesh[0];
        int kiter = 0;
        for (int k1 = 1; k1 <= d->kmesh[0]; ++k1) {
          int kk1 = k1 - 1;
          if (kk1 >= (d->kmesh[0] + 1) / 2) kk1 -= d->kmesh[0];
          if (d->kmesh[0] == 1) kk1 = 0;
          xk[0] = kk1;
          pref[0] = (kk1 > pbc[0]) ? 0.0 : 1.0;
          for (int k2 = 1; k2 <= d->kmesh[1]; ++k2) {
            int kk2 = k2 - 1;
            if (kk2 >= (d->kmesh[1] + 1) / 2) kk2 -= d->kmesh[1];
            if (d->kmesh[1] == 1) kk2 = 0;
            xk[1] = kk2;
            pref[1] = (kk2 > pbc[1]) ? 0.0 : pref[0];
            for (int k3 = 1; k3 <= d->kmesh[2]; ++k3) {
              int kk3 = k3 - 1;
              if (kk3 >= (d->kmesh[2] + 1) / 2) kk3 -= d->kmesh[2];
              if (d->kmesh[2] == 1) kk3 = 0;
              xk[2] = kk3;
              pref[2] = (kk3 > pbc[2]) ? 0.0 : pref[1];
              for (int i = 0; i < 3; ++i) alf[i] = xk[i] + fr[i] - tau[i];
              double r2 = 0.0;
              for (int i = 0; i < 3; ++i) {
                double m = 0.0;
                for (int j = 0; j < 3; ++j) m += amet[i][j] * alf[j];
                r2 += alf[i] * m;
              }
              double r = std::sqrt(r2);
              double potn;
              if (p->isolated && r > p->iso_cut) {
                potn = 0.0;
              } else if (r > rmax) {
                if (p->have_eps3d) {
                  double dir[3];
                  for (int c = 0; c < 3; ++c) {
                    double s = 0.0;
                    for (int j = 0; j < 3; ++j) s += p->avec[c + 3 * j] * alf[j];
                    dir[c] = s / r;
                  }
                  potn = (dir[0] * dir[0] / p->epsilon3d[0] + dir[1] * dir[1] / p->epsilon3d[1] +
                          dir[2] * dir[2] / p->epsilon3d[2]) / r;
                  if (r < rmax + 5.0)
                    potn = potn * (r - rmax) / 5.0 + (rmax + 5.0 - r) * epsi / (5.0 * r);
                } else {
                  potn = epsi / r;
                }
              } else {
                potn = or_intval(p->nptab, p->rtab, p->ptab, r);
              }
              W[(size_t)kiter + (size_t)nk * xiter] = potn * pref[2] * p->interaction_scale;
              ++kiter;
            }
          }
        }
        ++xiter;
      }
    }
  }
  return 0;
}

// ------------------------------------------------------------------- FFT

// Multi-dimensional DFT with FFTW's sign convention (Modules/FFT_wrapper.f90:24-25):
// X(m) = sum_j x(j) exp(sign * 2 pi i j.m / n), no normalisation.  The transform is
// separable, so it is applied along each k-mesh axis with exact root tables.
void or_fft3d(const int kmesh[3], double* re, double* im, int sign) {
  const int n1 = kmesh[0], n2 = kmesh[1], n3 = kmesh[2];
  const int dims[3] = {n1, n2, n3};
  const int strides[3] = {n2 * n3, n3, 1};
  const int nk = n1 * n2 * n3;
  std::vector<double> tr, ti, cr, ci, wr, wi;
  for (int ax = 0; ax < 3; ++ax) {
    int n = dims[ax];
    if (n == 1) continue;
    int st = strides[ax];
    wr.assign(n, 0.0);
    wi.assign(n, 0.0);
    for (int j = 0; j < n; ++j) {
      double ang = 2.0 * kPi * (double)j / (double)n;
      wr[j] = std::cos(ang);
      wi[j] = (double)sign * std::sin(ang);
    }
    tr.assign(n, 0.0);
    ti.assign(n, 0.0);
    cr.assign(n, 0.0);
    ci.assign(n, 0.0);
    for (int base = 0; base < nk; ++base) {
      // base must be the first element of a line along ax
      if ((base / st) % n != 0) continue;
      for (int j = 0; j < n; ++j) {
        cr[j] = re[base + j * st];
        ci[j] = im[base + j * st];
      }
      for (int m = 0; m < n; ++m) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < n; ++j) {
          int t = (j * m) % n;
          sr += cr[j] * wr[t] - ci[j] * wi[t];
          si += cr[j] * wi[t] + ci[j] * wr[t];
        }
        tr[m] = sr;
        ti[m] = si;
      }
      for (int m = 0; m < n; ++m) {
        re[base + m * st] = tr[m];
        im[base + m * st] = ti[m];
      }
    }
  }
}

// ------------------------------------------------------------------ action

namespace {

// lr_act_traditional_x + lr_kernel, OCEAN2/long_range.f90:758-963.  The
// reference parallelises over alpha; here x-points are split over threads with
// private accumulators summed in thread order (deterministic).
void lr_act(const or_dims* d, const or_ops* o, const double* pr, const double* pi, double* hr,
            double* hi) {
  const int nb = d->nb, nk = nk_of(d), nx = nx_of(d), na = d->na;
  const size_t npsi = (size_t)nb * nk * na;
  int nt = 1;
#ifdef _OPENMP
  nt = o->nthreads > 0 ? o->nthreads : omp_get_max_threads();
#endif
  std::vector<std::vector<double>> accr(nt), acci(nt);
  const double norm = 1.0 / (double)nk;  // fo%norm, FFT_wrapper.f90:60
#pragma omp parallel num_threads(nt)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<double>& ar = accr[tid];
    std::vector<double>& ai = acci[tid];
    ar.assign(npsi, 0.0);
    ai.assign(npsi, 0.0);
    std::vector<double> fr(nk), fi(nk);
#pragma omp for schedule(static)
    for (int x = 0; x < nx; ++x) {
      for (int a = 0; a < na; ++a) {
        int s = (d->nspn == 1) ? 0 : (a % 2);  // val_spin, long_range.f90:788-801
        const double* Ur = o->ur + (size_t)nb * nk * ((size_t)x + (size_t)nx * s);
        const double* Ui = o->ui + (size_t)nb * nk * ((size_t)x + (size_t)nx * s);
        const double* Pr = pr + (size_t)nb * nk * a;
        const double* Pi = pi + (size_t)nb * nk * a;
        for (int k = 0; k < nk; ++k) {  // :897-906 (no conjugate on u)
          double sr = 0.0, si = 0.0;
          const double* ur = Ur + (size_t)nb * k;
          const double* ui = Ui + (size_t)nb * k;
          const double* qr = Pr + (size_t)nb * k;
          const double* qi = Pi + (size_t)nb * k;
          for (int n = 0; n < nb; ++n) {
            sr += qr[n] * ur[n] - qi[n] * ui[n];
            si += qr[n] * ui[n] + qi[n] * ur[n];
          }
          fr[k] = sr;
          fi[k] = si;
        }
        or_fft3d(d->kmesh, fr.data(), fi.data(), +1);  // OCEAN_BACKWARD, :928
        const double* Wx = o->W + (size_t)nk * x;
        for (int k = 0; k < nk; ++k) {
          fr[k] *= Wx[k];
          fi[k] *= Wx[k];
        }
        or_fft3d(d->kmesh, fr.data(), fi.data(), -1);  // OCEAN_FORWARD, :932
        double* Ar = ar.data() + (size_t)nb * nk * a;
        double* Ai = ai.data() + (size_t)nb * nk * a;
        for (int k = 0; k < nk; ++k) {  // :943-961
          double xr = fr[k] * norm, xi = fi[k] * norm;
          const double* ur = Ur + (size_t)nb * k;
          const double* ui = Ui + (size_t)nb * k;
          double* hr_ = Ar + (size_t)nb * k;
          double* hi_ = Ai + (size_t)nb * k;
          for (int n = 0; n < nb; ++n) {
            hr_[n] = hr_[n] - ur[n] * xr - ui[n] * xi;
            hi_[n] = hi_[n] - ur[n] * xi + ui[n] * xr;
          }
        }
      }
    }
  }
  for (int t = 0; t < nt; ++t)
    for (size_t i = 0; i < npsi; ++i) {
      hr[i] += accr[t][i];
      hi[i] += acci[t][i];
    }
}

inline size_t mpc_idx(const or_dims* d, const or_ops* o, int n, int k, int nu, int m, int l,
                      int s) {
  const int nk = nk_of(d), nl = o->lmax - o->lmin + 1, nm = 2 * o->lmax + 1;
  return (size_t)n +
         (size_t)d->nb *
             ((size_t)k + (size_t)nk * ((size_t)nu + (size_t)o->npmax *
                                                         ((size_t)(m + o->lmax) +
                                                          (size_t)nm * ((size_t)(l - o->lmin) +
                                                                        (size_t)nl * s))));
}

// OCEAN_fg_combo, OCEAN2/OCEAN_multiplet.f90:1617-2005 (lmin = lvl, lmax = lvh).
void fg_combo(const or_dims* d, const or_ops* o, double inter, const double* pr, const double* pi,
              double* hr, double* hi) {
  const int nb = d->nb, nk = nk_of(d), na = d->na;
  const int lmin = o->lmin, lmax = o->lmax, npmax = o->npmax;
  const double mul = inter / ((double)nk * o->celvol);  // :1641
  const int landm = (lmax + 1) * (lmax + 1) - lmin * lmin;
  std::vector<double> ampr((size_t)npmax * landm * na, 0.0), ampi(ampr.size(), 0.0);
  std::vector<double> hampr(ampr.size(), 0.0), hampi(ampr.size(), 0.0);
  auto aidx = [&](int nu, int l, int m, int a) {
    return (size_t)nu + (size_t)npmax * ((size_t)(l * l + l + m - lmin * lmin) + (size_t)landm * a);
  };
  // amplitudes, :1730-1783
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads > 0 ? o->nthreads : 1)
  for (int a = 0; a < na; ++a)
    for (int l = lmin; l <= lmax; ++l) {
      int s = (d->nspn == 1) ? 0 : (1 - ((a + 1) % 2));  // ispn = 2 - mod(ialpha,2)
      for (int m = -l; m <= l; ++m)
        for (int nu = 0; nu < o->nproj[l - lmin]; ++nu) {
          double sr = 0.0, si = 0.0;
          for (int k = 0; k < nk; ++k) {
            size_t pb = (size_t)nb * ((size_t)k + (size_t)nk * a);
            size_t mb = mpc_idx(d, o, 0, k, nu, m, l, s);
            for (int n = 0; n < nb; ++n) {
              double qr = pr[pb + n], qi = pi[pb + n];
              double cr = o->mpcr[mb + n], ci = o->mpci[mb + n];
              sr = sr + qr * cr - qi * ci;
              si = si + qr * ci + qi * cr;
            }
          }
          ampr[aidx(nu, l, m, a)] = sr;
          ampi[aidx(nu, l, m, a)] = si;
        }
    }
  // direct term, :1819-1856
  for (int a = 0; a < na; ++a)
    for (int l = lmin; l <= lmax; ++l)
      for (int m = -l; m <= l; ++m) {
        int np = o->nproj[l - lmin];
        for (int nup = 0; nup < npmax; ++nup) {
          hampr[aidx(nup, l, m, a)] = 0.0;
          hampi[aidx(nup, l, m, a)] = 0.0;
        }
        for (int nu = 0; nu < np; ++nu)
          for (int nup = 0; nup < np; ++nup) {
            double mm = o->mpm[(size_t)nup + (size_t)npmax * ((size_t)nu + (size_t)npmax * (l - lmin))];
            hampr[aidx(nup, l, m, a)] -= mm * ampr[aidx(nu, l, m, a)];
            hampi[aidx(nup, l, m, a)] -= mm * ampi[aidx(nu, l, m, a)];
          }
        for (int nup = 0; nup < npmax; ++nup) {
          hampr[aidx(nup, l, m, a)] *= mul;
          hampi[aidx(nup, l, m, a)] *= mul;
        }
      }
  // exchange term, :1868-1936
  size_t jbeg = 0;
  for (int l = lmin; l <= lmax; ++l) {
    int np = o->nproj[l - lmin];
    int mham = na * (2 * l + 1) * np;
    std::vector<double> pwr(mham), pwi(mham);
    for (int a = 0; a < na; ++a)
      for (int m = -l; m <= l; ++m)
        for (int nu = 0; nu < np; ++nu) {
          int ii = nu + (m + l) * np + a * (2 * l + 1) * np;
          pwr[ii] = ampr[aidx(nu, l, m, a)];
          pwi[ii] = ampi[aidx(nu, l, m, a)];
        }
    for (int a = 0; a < na; ++a)
      for (int m = -l; m <= l; ++m)
        for (int nu = 0; nu < np; ++nu) {
          int ii = nu + (m + l) * np + a * (2 * l + 1) * np;
          double sr = 0.0, si = 0.0;
          for (int jj = 0; jj < mham; ++jj) {
            size_t j1 = jbeg + (size_t)jj + (size_t)ii * mham;
            sr = sr + o->mhr[j1] * pwr[jj] - o->mhi[j1] * pwi[jj];
            si = si + o->mhr[j1] * pwi[jj] + o->mhi[j1] * pwr[jj];
          }
          hampr[aidx(nu, l, m, a)] += sr * mul;
          hampi[aidx(nu, l, m, a)] += si * mul;
        }
    jbeg += (size_t)mham * mham;
  }
  // back projection, :1943-1998: out += conj(mpc) * hamp
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->nthreads > 0 ? o->nthreads : 1)
  for (int a = 0; a < na; ++a)
    for (int k = 0; k < nk; ++k) {
      int s = (d->nspn == 1) ? 0 : (1 - ((a + 1) % 2));
      size_t pb = (size_t)nb * ((size_t)k + (size_t)nk * a);
      for (int l = lmin; l <= lmax; ++l)
        for (int m = -l; m <= l; ++m)
          for (int nu = 0; nu < o->nproj[l - lmin]; ++nu) {
            double xr = hampr[aidx(nu, l, m, a)], xi = hampi[aidx(nu, l, m, a)];
            size_t mb = mpc_idx(d, o, 0, k, nu, m, l, s);
            for (int n = 0; n < nb; ++n) {
              double cr = o->mpcr[mb + n], ci = o->mpci[mb + n];
              hr[pb + n] = hr[pb + n] + cr * xr + ci * xi;
              hi[pb + n] = hi[pb + n] + cr * xi - ci * xr;
            }
          }
    }
}

// OCEAN_new_soact, OCEAN2/OCEAN_multiplet.f90:1543-1612.
void soact(const or_dims* d, const or_ops* o, const double* pr, const double* pi, double* hr,
           double* hi, int backwards) {
  const int nb = d->nb, nk = nk_of(d), na = d->na;
  for (int ic = 0; ic < na; ++ic)
    for (int k = 0; k < nk; ++k)
      for (int n = 0; n < nb; ++n) {
        size_t o_ = (size_t)n + (size_t)nb * ((size_t)k + (size_t)nk * ic);
        double r = hr[o_], im = hi[o_];
        for (int jc = 0; jc < na; ++jc) {
          size_t i_ = (size_t)n + (size_t)nb * ((size_t)k + (size_t)nk * jc);
          double sr = o->somelr[ic + na * jc], si = o->someli[ic + na * jc];
          if (backwards) {
            r = r + sr * pr[i_] + si * pi[i_];
            im = im + sr * pi[i_] - si * pr[i_];
          } else {
            r = r + sr * pr[i_] - si * pi[i_];
            im = im + sr * pi[i_] + si * pr[i_];
          }
        }
        hr[o_] = r;
        hi[o_] = im;
      }
}

}  // namespace

// OCEAN_xact core branch, OCEAN2/OCEAN_action.f90:286-618.
int or_xact(const or_dims* d, const or_ops* o, const double* pr, const double* pi, double* hr,
            double* hi, const int* hflag_in, int backwards) {
  const size_t npsi = (size_t)d->nb * nk_of(d) * d->na;
  int hflag[6];
  for (int i = 0; i < 6; ++i) hflag[i] = hflag_in ? hflag_in[i] : o->nhflag[i];
  std::vector<double> fr(npsi, 0.0), fi(npsi, 0.0);  // new_psi full (zero_full :325)
  std::vector<double> qr(npsi), qi(npsi);            // psi_o = allow o psi (:337-340)
  for (size_t i = 0; i < npsi; ++i) {
    qr[i] = pr[i] * o->allow[i];
    qi[i] = pi[i] * o->allow[i];
  }
  if (o->mult && hflag[4] == 1 && o->mpcr) fg_combo(d, o, o->interaction_scale, qr.data(), qi.data(), fr.data(), fi.data());
  if (o->long_range && hflag[0] == 1) lr_act(d, o, qr.data(), qi.data(), fr.data(), fi.data());
  for (size_t i = 0; i < npsi; ++i) {  // allow_full(new_psi), :361
    fr[i] *= o->allow[i];
    fi[i] *= o->allow[i];
  }
  if (hflag[5] == 1 && o->mult && o->somelr) soact(d, o, pr, pi, fr.data(), fi.data(), backwards);
  // energies_act into min (overwrite), then buffer2min (min += full), :596-608
  for (size_t i = 0; i < npsi; ++i) {
    double er = 0.0, ei = 0.0, mr = 0.0, mi = 0.0;
    if (o->e0) {
      er = o->er[i];
      ei = o->ei ? o->ei[i] : 0.0;
      if (backwards) {  // f2m_3element_mult is_conjugate, OCEAN_psi.f90:3262-3267
        mr = er * pr[i] + ei * pi[i];
        mi = er * pi[i] - ei * pr[i];
      } else {
        mr = er * pr[i] - ei * pi[i];
        mi = er * pi[i] + ei * pr[i];
      }
    }
    hr[i] = mr + fr[i];
    hi[i] = mi + fi[i];
  }
  return 0;
}

// ----------------------------------------------------------------- Haydock

// core_pnorm, OCEAN2/OCEAN_psi.f90:5589-5638 (single rank, full store).
double or_pnorm(int n, int nkpts, double celvol, double* pr, double* pi) {
  double val = 0.0;
  for (int i = 0; i < n; ++i) val += pr[i] * pr[i] + pi[i] * pi[i];
  val = std::sqrt(val);
  double kpref = 4.0 * kPi * val * val / ((double)nkpts * celvol * celvol);
  double inv = 1.0 / val;
  for (int i = 0; i < n; ++i) {
    pr[i] *= inv;
    pi[i] *= inv;
  }
  return kpref;
}

// OCEAN_haydock_Herm_do (OCEAN_haydock.f90:190-320) with
// ocean_hay_ab_twoterm (:824-938); psi_dot = sum conj(p) q (OCEAN_psi.f90:2029-2034).
int or_haydock(const or_dims* d, const or_ops* o, const double* p0r, const double* p0i, int niter,
               double* real_a, double* imag_a, double* real_b, int* niter_done) {
  const size_t n = (size_t)d->nb * nk_of(d) * d->na;
  std::vector<double> psr(p0r, p0r + n), psi_(p0i, p0i + n);
  std::vector<double> olr(n, 0.0), oli(n, 0.0), hr(n), hi(n);
  for (int i = 0; i <= niter; ++i) real_a[i] = imag_a[i] = real_b[i] = 0.0;
  int done = 0;
  for (int iter = 1; iter <= niter; ++iter) {
    or_xact(d, o, psr.data(), psi_.data(), hr.data(), hi.data(), nullptr, 0);
    double bm = -real_b[iter - 1];
    for (size_t i = 0; i < n; ++i) {  // axpy(-b, old, hpsi)
      hr[i] += bm * olr[i];
      hi[i] += bm * oli[i];
    }
    double ar = 0.0, ai = 0.0;  // dot(hpsi, psi)
    for (size_t i = 0; i < n; ++i) {
      ar += hr[i] * psr[i] + hi[i] * psi_[i];
      ai += hr[i] * psi_[i] - hi[i] * psr[i];
    }
    real_a[iter - 1] = ar;
    for (size_t i = 0; i < n; ++i) {  // axpy(-a, psi, hpsi)
      hr[i] += -ar * psr[i];
      hi[i] += -ar * psi_[i];
    }
    double bb = 0.0;
    for (size_t i = 0; i < n; ++i) bb += hr[i] * hr[i] + hi[i] * hi[i];
    olr = psr;
    oli = psi_;
    real_b[iter] = std::sqrt(bb);
    double inv = 1.0 / real_b[iter];
    for (size_t i = 0; i < n; ++i) {
      psr[i] = hr[i] * inv;
      psi_[i] = hi[i] * inv;
    }
    imag_a[iter - 1] = ai;
    done = iter;
    if (std::isnan(real_a[iter - 1])) {
      *niter_done = done;
      return -1;
    }
  }
  *niter_done = done;
  return 0;
}

// The two-sided Lanczos of OCEAN_haydock_nonHerm_do (OCEAN_haydock.f90:53-164)
// with the step of haydock_abc_1 (:1250-1433) written as the algorithm its
// comments cite (Saad, two-sided Lanczos; (x, y) = sum x conj(y) = <y|x>):
//   alpha_j = <w_j|A v_j>,  delta_{j+1} = sqrt(z) (principal, as :1373-1374),
//   beta_{j+1} = z / delta_{j+1},  z = <w^_{j+1}|v^_{j+1}>,
//   v^_{j+1} = A v_j - alpha_j v_j - beta_j v_{j-1},
//   w^_{j+1} = A^H w_j - conj(alpha_j) w_j - conj(delta_j) w_{j-1},
//   v_{j+1} = v^ / delta,  w_{j+1} = w^ / conj(beta).
// haydock_abc_1 itself subtracts conj(beta_j) v_{j-1} and divides w^ by beta,
// so its tridiagonal matches the moments <w_1|A^k v_1> only for k <= 2 (the
// routine is not called: complex_haydock is .false., :47,181).  Stored as
// write_core reads them (z - conj(a), products b*c, :1846-1870): a = alpha,
// b = conj(beta), c = conj(delta), so that the continued fraction is
// <psi|(z - A^H)^-1|psi>, the Hermitian run's convention.
int or_haydock_nonherm(const or_dims* d, const or_ops* o, const double* p0r, const double* p0i, int niter,
                       double* real_a, double* imag_a, double* real_b, double* imag_b, double* real_c,
                       double* imag_c, int* niter_done) {
  const size_t n = (size_t)d->nb * nk_of(d) * d->na;
  std::vector<double> vr(p0r, p0r + n), vi(p0i, p0i + n), wr(vr), wi(vi);
  std::vector<double> ovr(n, 0.0), ovi(n, 0.0), owr(n, 0.0), owi(n, 0.0);
  std::vector<double> hvr(n), hvi(n), hwr(n), hwi(n);
  for (int i = 0; i <= niter; ++i) real_a[i] = imag_a[i] = real_b[i] = imag_b[i] = real_c[i] = imag_c[i] = 0.0;
  auto allow = [&](std::vector<double>& r, std::vector<double>& im) {  // OCEAN_energies_allow
    for (size_t i = 0; i < n; ++i) {
      r[i] *= o->allow[i];
      im[i] *= o->allow[i];
    }
  };
  auto dot = [&](const std::vector<double>& pr, const std::vector<double>& pi, const std::vector<double>& qr,
                 const std::vector<double>& qi, double* rr, double* ii) {  // sum conj(p) q
    double a = 0.0, b = 0.0;
    for (size_t i = 0; i < n; ++i) {
      a += pr[i] * qr[i] + pi[i] * qi[i];
      b += pr[i] * qi[i] - pi[i] * qr[i];
    }
    *rr = a;
    *ii = b;
  };
  auto axpy = [&](double ar, double ai, const std::vector<double>& xr, const std::vector<double>& xi,
                  std::vector<double>& yr, std::vector<double>& yi) {  // y += (ar + i ai) x
    for (size_t i = 0; i < n; ++i) {
      yr[i] += ar * xr[i] - ai * xi[i];
      yi[i] += ar * xi[i] + ai * xr[i];
    }
  };
  auto divide = [&](std::vector<double>& xr, std::vector<double>& xi, double rv, double iv) {  // OCEAN_psi_divide
    const double denom = rv * rv + iv * iv, rn = rv / denom, in = iv / denom;
    for (size_t i = 0; i < n; ++i) {
      const double buf = -in * xr[i];
      xr[i] = rn * xr[i] + in * xi[i];
      xi[i] = buf + rn * xi[i];
    }
  };
  int done = 0;
  for (int iter = 1; iter <= niter; ++iter) {
    allow(vr, vi);
    allow(wr, wi);
    or_xact(d, o, vr.data(), vi.data(), hvr.data(), hvi.data(), nullptr, 0);
    or_xact(d, o, wr.data(), wi.data(), hwr.data(), hwi.data(), nullptr, 1);  // A^H
    allow(hvr, hvi);
    allow(hwr, hwi);
    double ar, ai;
    dot(wr, wi, hvr, hvi, &ar, &ai);  // alpha = <w|A v>
    // beta_j = conj(b_j), conj(delta_j) = c_j
    axpy(-real_b[iter - 1], imag_b[iter - 1], ovr, ovi, hvr, hvi);
    axpy(-real_c[iter - 1], -imag_c[iter - 1], owr, owi, hwr, hwi);
    axpy(-ar, -ai, vr, vi, hvr, hvi);
    axpy(-ar, ai, wr, wi, hwr, hwi);
    real_a[iter - 1] = ar;
    imag_a[iter - 1] = ai;
    allow(hvr, hvi);
    allow(hwr, hwi);
    double zr, zi;
    dot(hwr, hwi, hvr, hvi, &zr, &zi);
    ovr = vr;
    ovi = vi;
    owr = wr;
    owi = wi;
    const double az = std::sqrt(zr * zr + zi * zi);
    const double dr = std::sqrt((az + zr) / 2.0), di = std::copysign(std::sqrt((az - zr) / 2.0), zi);
    const cd beta = cdiv(cd(zr, zi), cd(dr, di));
    real_b[iter] = beta.real();
    imag_b[iter] = -beta.imag();
    real_c[iter] = dr;
    imag_c[iter] = -di;
    divide(hwr, hwi, beta.real(), -beta.imag());  // w^ / conj(beta)
    divide(hvr, hvi, dr, di);                      // v^ / delta
    vr = hvr;
    vi = hvi;
    wr = hwr;
    wi = hwi;
    done = iter;
    if (std::isnan(real_a[iter - 1])) {
      *niter_done = done;
      return -1;
    }
  }
  *niter_done = done;
  return 0;
}

// gamfcn, CNBSE/zcmsnmult/zf90/gamfcn.f90:8-42.
double or_gamfcn(double e, double n, double e0) {
  const double pi = 3.14159265358979;
  double kf = std::pow(3.0 * pi * pi * n, 1.0 / 3.0);
  double wp = std::sqrt(4.0 * pi * n);
  double k = kf * kf / 2.0 + e;
  double g = 0.0;
  if (k < kf * kf / 2.0) return 0.0;
  k = std::sqrt(2.0 * k);
  double wf = kf * kf / 2.0;
  double lam = std::sqrt(wp * wp / (wf * wf * (e0 - 1.0)));
  double dq = 0.005 * kf;
  double q = 0.5 * dq;
  bool test1 = true;
  double su = 0.0;
  int guard = 0;
  while (test1 && guard < 100000000) {
    ++guard;
    double qq = q / kf;
    double xp = qq * (2.0 + qq) / lam;
    double xm = qq * (2.0 - qq) / lam;
    double term1 = lam / (2.0 * qq * qq * qq) * (std::atan(xp) + std::atan(xm));
    double term2 = (0.125 * lam * lam / std::pow(qq, 5) + 0.5 / (qq * qq * qq) - 0.125 / qq) *
                   std::log((1.0 + xp * xp) / (1.0 + xm * xm));
    double epsq = 1.0 + 2.0 / (pi * kf) * (1.0 / (qq * qq) - term1 + term2);
    double wq = wp / std::sqrt(1.0 - 1.0 / epsq);
    test1 = (k * k - kf * kf - 2.0 * wq > 0.0);
    bool test2 = (k * q - wq - q * q / 2.0 > 0.0);
    if (test1 && test2) su = su + dq / (q * wq);
    q = q + dq;
  }
  g = g + wp * wp * su / (2.0 * k);
  return g;
}

namespace {
// Continued fraction at one energy, write_core inner loops
// (OCEAN_haydock.f90:1831-1873), single-precision cmplx() quirk included.
// b_j c_j: cmplx(real_b, imag_b) * cmplx(real_c, imag_c), binary32; without
// imag_b / real_c / imag_c the Hermitian run's c = b, imag parts zero
cd bc_sp(const double* rb, const double* ib, const double* rc, const double* ic, int j) {
  return cmul_sp(rb[j], ib ? ib[j] : 0.0, rc ? rc[j] : rb[j], ic ? ic[j] : 0.0);
}

cd cf_delta(const double* ra, const double* ia, const double* rb, const double* ib, const double* rc,
            const double* ic, int iter, double e, double gam) {
  double ia_last = ia ? ia[iter - 1] : 0.0;
  cd ctmp(e - ra[iter - 1], gam + ia_last);
  cd bc = bc_sp(rb, ib, rc, ic, iter);
  cd four_bc((double)(4.0f * (float)bc.real()), (double)(4.0f * (float)bc.imag()));
  cd disc = csqrt_p(cmul(ctmp, ctmp) - four_bc);
  cd delta = (disc.imag() > 0.0) ? (ctmp + disc) * 0.5 : (ctmp - disc) * 0.5;
  for (int jj = iter - 1; jj >= 0; --jj) {
    cd c2 = bc_sp(rb, ib, rc, ic, jj + 1);
    double iaj = ia ? ia[jj] : 0.0;
    delta = cmplx_sp(e - ra[jj], gam + iaj) - cdiv(c2, delta);
  }
  return delta;
}
}  // namespace

// write_core (OCEAN_haydock.f90:1801-1894) and write_core_Voigt (:1896-1989).
int or_write_core(const double* ra, const double* ia, const double* rb, int iter, double kpref,
                  double el, double eh, int ne, double gam0, double ebase, double gam_gauss,
                  double ucvol, int old_broaden, double nval, double eps, double* out) {
  if (gam_gauss > gam0 / 10.0) {
    // write_core_Voigt
    double de = (eh - el) / (double)ne;
    double estep = std::min(gam0, gam_gauss) / 2.0;
    int nratio = (int)((de - estep) / estep) + 1;
    estep = de / (double)nratio;
    int nstep = (int)((2.99999 * gam_gauss) / estep) + 1;
    double prefactor = estep / (gam_gauss * 2.506628274631);
    double inv2s2 = 1.0 / (2.0 * gam_gauss * gam_gauss);
    std::vector<double> sa(2 * nstep + 1), sb(2 * nstep + 1), ka(2 * nstep + 1), kb(2 * nstep + 1);
    int row = 0;
    double e = 0.0;
    for (int ie = 0; ie <= 2 * ne; ie += 2) {
      double ee = el + (eh - el) * (double)ie / (double)(2 * ne);
      int istart;
      if (ie == 0) {
        istart = -nstep;
      } else {
        istart = nstep - nratio;
        for (int ii = -nstep; ii <= nstep - nratio; ++ii) {
          sa[ii + nstep] = sa[ii + nratio + nstep];
          sb[ii + nstep] = sb[ii + nratio + nstep];
          ka[ii + nstep] = ka[ii + nratio + nstep];
          kb[ii + nstep] = kb[ii + nratio + nstep];
        }
      }
      for (int ii = istart; ii <= nstep; ++ii) {
        e = ee + (double)ii * estep;
        for (int jd = 0; jd <= 1; ++jd) {
          double gam = gam0 + (jd ? or_gamfcn(e, nval, eps) : 0.0);
          cd delta = cf_delta(ra, ia, rb, nullptr, nullptr, nullptr, iter, e, gam);
          double dr = delta.real(), di = std::fabs(delta.imag());
          double sp = prefactor * kpref * di / (dr * dr + di * di);
          double sk = prefactor * kpref * dr / (dr * dr + di * di);
          if (jd == 0) { sa[ii + nstep] = sp; ka[ii + nstep] = sk; }
          else { sb[ii + nstep] = sp; kb[ii + nstep] = sk; }
        }
      }
      double s0 = 0, s1 = 0, k0 = 0, k1 = 0;
      for (int ii = -nstep; ii <= nstep; ++ii) {
        double pref = std::exp(-(double)(ii * ii) * estep * estep * inv2s2);
        s0 += pref * sa[ii + nstep];
        s1 += pref * sb[ii + nstep];
        k0 += pref * ka[ii + nstep];
        k1 += pref * kb[ii + nstep];
      }
      double* r = out + 9 * (size_t)row;
      r[0] = ebase + kHa2eV * e;  // the reference prints the last fine-grid energy
      r[1] = s1; r[2] = s0; r[3] = k1; r[4] = k0;
      r[5] = r[6] = r[7] = r[8] = 0.0;
      ++row;
    }
    return 0;
  }
  const double alphaByVolumeHartree = kEV2Ha * kAlpha * ucvol;
  const double tpa = (kAlpha * kAlpha * 2.0 * kPi) * ucvol;
  const double bohrSq2CmSq = kBohr * kBohr * 1.0e-16;
  const double tpacm4 = tpa * bohrSq2CmSq * bohrSq2CmSq * kAu2sec;
  int jdstop = old_broaden ? 1 : 0;
  int row = 0;
  for (int ie = 0; ie <= 2 * ne; ie += 2) {
    double e = el + (eh - el) * (double)ie / (double)(2 * ne);
    double spct[2] = {0, 0}, spkk[2] = {0, 0};
    for (int jd = 0; jd <= jdstop; ++jd) {
      // gam0 + gamfcn(...)*dble(jdamp): the product is zero for jdamp = 0
      double gam = gam0 + (jd ? or_gamfcn(e, nval, eps) : 0.0);
      cd delta = cf_delta(ra, ia, rb, nullptr, nullptr, nullptr, iter, e, gam);
      double dr = delta.real(), di = std::fabs(delta.imag());
      spct[jd] = kpref * di / (dr * dr + di * di);
      spkk[jd] = kpref * dr / (dr * dr + di * di);
    }
    if (!old_broaden) {
      spct[1] = spct[0];
      spkk[1] = spkk[0];
    }
    double ener = ebase + kHa2eV * e;
    double sigma = alphaByVolumeHartree * ener * spct[0];
    double* r = out + 9 * (size_t)row;
    r[0] = ener; r[1] = spct[1]; r[2] = spct[0]; r[3] = spkk[1]; r[4] = spkk[0];
    r[5] = sigma; r[6] = sigma * bohrSq2CmSq; r[7] = spct[0] * tpa; r[8] = spct[0] * tpacm4;
    ++row;
  }
  return 0;
}

// write_core's rows for complex b and c (no Voigt, no second damping).
int or_write_core_bc(const double* ra, const double* ia, const double* rb, const double* ib,
                     const double* rc, const double* ic, int iter, double kpref, double el, double eh,
                     int ne, double gam0, double ebase, double ucvol, double* out) {
  const double alphaByVolumeHartree = kEV2Ha * kAlpha * ucvol;
  const double tpa = (kAlpha * kAlpha * 2.0 * kPi) * ucvol;
  const double bohrSq2CmSq = kBohr * kBohr * 1.0e-16;
  const double tpacm4 = tpa * bohrSq2CmSq * bohrSq2CmSq * kAu2sec;
  int row = 0;
  for (int ie = 0; ie <= 2 * ne; ie += 2) {
    double e = el + (eh - el) * (double)ie / (double)(2 * ne);
    cd delta = cf_delta(ra, ia, rb, ib, rc, ic, iter, e, gam0);
    double dr = delta.real(), di = std::fabs(delta.imag());
    double sp = kpref * di / (dr * dr + di * di), sk = kpref * dr / (dr * dr + di * di);
    double ener = ebase + kHa2eV * e;
    double sigma = alphaByVolumeHartree * ener * sp;
    double* r = out + 9 * (size_t)row;
    r[0] = ener; r[1] = sp; r[2] = sp; r[3] = sk; r[4] = sk;
    r[5] = sigma; r[6] = sigma * bohrSq2CmSq; r[7] = sp * tpa; r[8] = sp * tpacm4;
    ++row;
  }
  return 0;
}

// write_val, OCEAN_haydock.f90:1706-1799: the valence dielectric function and
// optical constants, ne rows of (omega eV, eps1, eps2, Re n - 1, Im n, mu, R,
// epsinv).  b_j c_j = cmplx(real_b, imag_b, DP) * cmplx(real_c, -imag_c, DP).
int or_write_val(const double* ra, const double* ia, const double* rb, const double* ib, const double* rc,
                 const double* ic, int iter, double kpref, double ucvol, int val_ham_spin, int semi_tda, int backf,
                 double el, double eh, int ne, double gam0, double* out) {
  if (iter < 1 || ne < 1 || (val_ham_spin != 1 && val_ham_spin != 2)) return -1;
  const double h2e = 27.211386245980, bohr = 0.529177210544, alphainv = 137.035999177;
  const double fact = kpref * (double)(2 / val_ham_spin) * ucvol;
  for (int r = 0; r < ne; ++r) {
    const int ie = 2 * r + 1;
    double ere = el + (eh - el) * (double)ie / (double)(2 * ne);
    cd ctmp(ere, gam0);
    if (backf) {
      ctmp = cmul(ctmp, ctmp);
      ere = ere * ere;
    }
    const double an = ra[iter - 1];
    const cd arg = csqrt_p(cd((ere - an) * (ere - an) - 4.0 * rb[iter] * rb[iter], 0.0));
    const cd rp = (cd(ere - an, 0.0) + arg) * 0.5;
    const cd rm = (cd(ere - an, 0.0) - arg) * 0.5;
    const cd rrr = rp.imag() < 0.0 ? rp : rm;
    cd al = ctmp - an - rrr;
    cd be = -ctmp - an - rrr;
    for (int i = iter - 1; i >= 0; --i) {
      const double a = rb[i + 1], b = ib ? ib[i + 1] : 0.0;
      const double c = rc ? rc[i + 1] : a, dd = ic ? -ic[i + 1] : 0.0;
      const cd bc(a * c - b * dd, a * dd + b * c);
      const cd ai(ra[i], ia ? ia[i] : 0.0);
      al = ctmp - ai - cdiv(bc, al);
      be = -ctmp - ai - cdiv(bc, be);
    }
    cd eps = cd(1.0, 0.0) - cdiv(cd(fact, 0.0), al);
    if (semi_tda) eps -= cdiv(cd(fact, 0.0), be);
    if (backf) ere = std::sqrt(ere);
    const double reeps = eps.real(), imeps = eps.imag();
    const double lossf = imeps / (reeps * reeps + imeps * imeps);
    const cd refrac = csqrt_p(eps);
    const double reflct = std::norm(cdiv(refrac - 1.0, refrac + 1.0));
    const double mu = 2.0 * ere * h2e * refrac.imag() / (bohr * alphainv * 1000.0);
    double* o = out + 8 * (size_t)r;
    o[0] = ere * h2e;
    o[1] = reeps;
    o[2] = imeps;
    o[3] = refrac.real() - 1.0;
    o[4] = refrac.imag();
    o[5] = mu;
    o[6] = reflct;
    o[7] = lossf;
  }
  return 0;
}

// calc_spect_core, OCEAN_haydock.f90:1991-2027.
int or_calc_spect_core(const double* ra, const double* ia, const double* rb, int iter, double kpref,
                       double el, double eh, int ne, double gam0, double ebase, double* out) {
  for (int ie = 1; ie <= ne; ++ie) {
    double e = el + (eh - el) * (double)(2 * (ie - 1) + 1) / (double)(2 * ne);
    cd delta = cf_delta(ra, ia, rb, nullptr, nullptr, nullptr, iter, e, gam0);
    double dr = delta.real(), di = std::fabs(delta.imag());
    out[3 * (ie - 1) + 0] = ebase + kHa2eV * e;
    out[3 * (ie - 1) + 1] = kpref * dr / (dr * dr + di * di);
    out[3 * (ie - 1) + 2] = kpref * di / (dr * dr + di * di);
  }
  return 0;
}

// check_convergence (OCEAN_haydock.f90:1608-1661), core branch: the calc_spect_core
// spectra of iter1 and iter2 steps on the ne midpoints; relArea =
// 2 sum|sp1 - sp2| / (sum|sp1| + sum|sp2|), maxDiff = max|sp1 - sp2| (column 3,
// sums in energy order).
int or_check_convergence(const double* ra, const double* ia, const double* rb, int iter1, int iter2, double kpref,
                         double el, double eh, int ne, double gam0, double* max_diff, double* rel_area) {
  std::vector<double> sp1(3 * (size_t)ne), sp2(3 * (size_t)ne);
  or_calc_spect_core(ra, ia, rb, iter1, kpref, el, eh, ne, gam0, 0.0, sp1.data());
  or_calc_spect_core(ra, ia, rb, iter2, kpref, el, eh, ne, gam0, 0.0, sp2.data());
  double md = 0.0, rel = 0.0, a1 = 0.0, a2 = 0.0;
  for (int i = 0; i < ne; ++i) {
    const double diff = std::fabs(sp1[3 * i + 2] - sp2[3 * i + 2]);
    if (diff > md) md = diff;
    rel += diff;
    a1 += std::fabs(sp1[3 * i + 2]);
    a2 += std::fabs(sp2[3 * i + 2]);
  }
  *max_diff = md;
  *rel_area = 2.0 * rel / (a1 + a2);
  return 0;
}

// Stopping iteration of the early exit of OCEAN_haydock_Herm_do
// (OCEAN_haydock.f90:268-292) from the relArea of each iteration
// (rel[iter], iter = spacing+1 .. niter): the first iter whose relArea and the
// previous iteration's are both below the threshold (prevConv), else niter.
int or_early_exit_iter(const double* rel, int niter, int spacing, double threshold) {
  bool prev = false;
  for (int iter = 1; iter <= niter; ++iter) {
    if (threshold > 0.0 && iter > spacing) {
      if (rel[iter] < threshold) {
        if (prev) return iter;
        prev = true;
      } else {
        prev = false;
      }
    }
  }
  return niter;
}

// OCEAN_haydock_Herm_do with haydockconv.ipt (earlyExit): the Lanczos run of
// or_haydock, with check_convergence after every step beyond the spacing;
// rel_out[iter] (may be NULL) receives each relArea (0 where not checked).
int or_haydock_conv(const or_dims* d, const or_ops* o, const double* p0r, const double* p0i, int niter,
                    double threshold, int spacing, double kpref, double el, double eh, int ne, double gam0,
                    double* real_a, double* imag_a, double* real_b, double* rel_out, int* niter_done) {
  const size_t n = (size_t)d->nb * nk_of(d) * d->na;
  std::vector<double> psr(p0r, p0r + n), psi_(p0i, p0i + n);
  std::vector<double> olr(n, 0.0), oli(n, 0.0), hr(n), hi(n);
  for (int i = 0; i <= niter; ++i) real_a[i] = imag_a[i] = real_b[i] = 0.0;
  if (rel_out)
    for (int i = 0; i <= niter; ++i) rel_out[i] = 0.0;
  bool prev = false;
  int done = 0;
  for (int iter = 1; iter <= niter; ++iter) {
    or_xact(d, o, psr.data(), psi_.data(), hr.data(), hi.data(), nullptr, 0);
    double bm = -real_b[iter - 1];
    for (size_t i = 0; i < n; ++i) {
      hr[i] += bm * olr[i];
      hi[i] += bm * oli[i];
    }
    double ar = 0.0, ai = 0.0;
    for (size_t i = 0; i < n; ++i) {
      ar += hr[i] * psr[i] + hi[i] * psi_[i];
      ai += hr[i] * psi_[i] - hi[i] * psr[i];
    }
    real_a[iter - 1] = ar;
    for (size_t i = 0; i < n; ++i) {
      hr[i] += -ar * psr[i];
      hi[i] += -ar * psi_[i];
    }
    double bb = 0.0;
    for (size_t i = 0; i < n; ++i) bb += hr[i] * hr[i] + hi[i] * hi[i];
    olr = psr;
    oli = psi_;
    real_b[iter] = std::sqrt(bb);
    double inv = 1.0 / real_b[iter];
    for (size_t i = 0; i < n; ++i) {
      psr[i] = hr[i] * inv;
      psi_[i] = hi[i] * inv;
    }
    imag_a[iter - 1] = ai;
    done = iter;
    if (std::isnan(real_a[iter - 1])) {
      *niter_done = done;
      return -1;
    }
    if (threshold > 0.0 && iter > spacing) {
      double md, rel;
      or_check_convergence(real_a, imag_a, real_b, iter, iter - spacing, kpref, el, eh, ne, gam0, &md, &rel);
      if (rel_out) rel_out[iter] = rel;
      if (rel < threshold) {
        if (prev) break;
        prev = true;
      } else {
        prev = false;
      }
    }
  }
  *niter_done = done;
  return 0;
}

// ---- nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181) with threey
// (CNBSE/zcmsnmult/zf90/newthreey.f90), newgetylm and newgetprefs.

}  // extern "C"

namespace {

// Gauss-Legendre nodes and weights on [-1, 1] (the role of the Pquadrature file;
// weights rescaled to sum to 2 as nbsemhsetup2 does).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int l = 2; l <= n; ++l) {
        const double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  double su = 0.0;
  for (double v : w) su += v;
  for (double& v : w) v = v * 2.0 / su;
}

// newgetylm at (x, y, z) on the unit sphere: prefs(l,|m|) f(l,|m|)(u) (x + i y)^m,
// m < 0: times (-(x - i y))^|m|; f = (-1)^m d^m P_l / du^m (the table of newgetylm),
// prefs = sqrt((2l+1)/(4 pi) (l-|m|)!/(l+|m|)!) (newgetprefs).
cd ylm_ref(int l, int m, double x, double y, double z) {
  const double pi = 3.14159265358979323846;
  const int am = std::abs(m);
  // m-th derivative of P_l at u = z: coefficients of P_l by the three-term recurrence
  std::vector<std::vector<double>> P(l + 1, std::vector<double>(l + 1, 0.0));
  P[0][0] = 1.0;
  if (l >= 1) P[1][1] = 1.0;
  for (int n = 2; n <= l; ++n)
    for (int k = 0; k <= n; ++k) {
      double v = 0.0;
      if (k >= 1) v += (2.0 * n - 1.0) * P[n - 1][k - 1];
      v -= (n - 1.0) * P[n - 2][k];
      P[n][k] = v / n;
    }
  double f = 0.0;
  for (int k = am; k <= l; ++k) {
    double c = P[l][k];
    for (int j = 0; j < am; ++j) c *= (double)(k - j);
    f += c * std::pow(z, k - am);
  }
  if (am & 1) f = -f;
  double pref = (2.0 * l + 1.0) / (4.0 * pi);
  for (int j = 1; j <= am; ++j) pref /= (double)((l - j + 1) * (l + j));
  cd y0(std::sqrt(pref) * f, 0.0);
  for (int j = 0; j < am; ++j) y0 *= (m > 0) ? cd(x, y) : -cd(x, -y);
  return y0;
}

cd threey_ref(int ll, int ml, int lmid, int mmid, int lr, int mr, bool conjug, const std::vector<double>& xq,
              const std::vector<double>& wq) {
  const double pi = 3.14159265358979323846;
  cd i0(0.0, 0.0);
  const bool mdo = conjug ? (ml == mr - mmid) : (ml == mr + mmid);
  bool ldo = false;
  for (int j = ll + lr; j >= std::max(std::abs(mmid), std::abs(ll - lr)); j -= 2)
    if (j == lmid) ldo = true;
  if (!(ldo && mdo)) return i0;
  for (size_t j = 0; j < xq.size(); ++j) {  // phi = 0
    const double ct = xq[j], st = std::sqrt(1.0 - ct * ct);
    const cd yl = ylm_ref(ll, ml, st, 0.0, ct);
    cd ym = ylm_ref(lmid, mmid, st, 0.0, ct);
    if (conjug) ym = std::conj(ym);
    const cd yr = ylm_ref(lr, mr, st, 0.0, ct);
    i0 += wq[j] * std::conj(yl) * ym * yr;
  }
  return i0 * (2.0 * pi);
}

}  // namespace

extern "C" {

double or_threey(int ll, int ml, int lm, int mm, int lr, int mr, int conjug, int npt) {
  std::vector<double> xq, wq;
  gauss_legendre(npt, xq, wq);
  return threey_ref(ll, ml, lm, mm, lr, mr, conjug != 0, xq, wq).real();
}

int or_nbsemhsetup2(int lc, int lv, int np, int kfl, int kfh, const double* fk, const double* scfk, int kgl,
                    int kgh, const double* gk, const double* scgk, double scfac, int npt, double* mhr_out,
                    double* mhi_out) {
  std::vector<double> xq, wq;
  gauss_legendre(npt, xq, wq);
  const int nalpha = 4 * (2 * lc + 1);
  const int mham = nalpha * (2 * lv + 1) * np;
  // hcms, hcml, hvms, hvml, hvnu of OCEAN_multiplet.f90:342-369
  std::vector<double> cms(mham), cml(mham), vms(mham), vml(mham);
  std::vector<int> vnu(mham);
  std::vector<double> acms, acml, avms;
  for (int icms = -1; icms <= 1; icms += 2)
    for (int icml = -lc; icml <= lc; ++icml)
      for (int ivms = -1; ivms <= 1; ivms += 2) {
        acms.push_back(0.5 * icms);
        acml.push_back(icml);
        avms.push_back(0.5 * ivms);
      }
  int ii = 0;
  for (int ic = 0; ic < nalpha; ++ic)
    for (int ivml = -lv; ivml <= lv; ++ivml)
      for (int nu = 1; nu <= np; ++nu, ++ii) {
        cms[ii] = acms[ic];
        cml[ii] = acml[ic];
        vms[ii] = avms[ic];
        vml[ii] = ivml;
        vnu[ii] = nu;
      }
  const double pi = 4.0 * std::atan(1.0);
  const size_t npp = (size_t)np * np;
  auto nint = [](double v) { return (int)std::lround(v); };
  for (int i1 = 0; i1 < mham; ++i1) {
    const int nu1 = vnu[i1] - 1;
    for (int i2 = 0; i2 < mham; ++i2) {
      const int nu2 = vnu[i2] - 1;
      double mr = 0.0, mi = 0.0;
      if (kfh >= kfl) {
        const int l1 = lc, m1 = nint(cml[i2]), s1 = nint(2 * cms[i2]);
        const int l2 = lv, m2 = nint(vml[i1]), s2 = nint(2 * vms[i1]);
        const int l3 = lc, m3 = nint(cml[i1]), s3 = nint(2 * cms[i1]);
        const int l4 = lv, m4 = nint(vml[i2]), s4 = nint(2 * vms[i2]);
        if (s1 == s3 && s2 == s4) {
          const int mk = m1 - m3;
          if (m1 + m2 == m3 + m4)
            for (int k = kfl; k <= kfh; k += 2)
              if (std::abs(mk) <= k) {
                const int ik = (k - kfl) / 2;
                const double ffk = scfk[ik] * fk[ik * npp + nu1 + (size_t)np * nu2] * scfac;
                const cd f1 = threey_ref(l1, m1, k, mk, l3, m3, false, xq, wq);
                const cd f2 = threey_ref(l2, m2, k, mk, l4, m4, true, xq, wq);
                const cd ct = -ffk * f1 * f2 * (4 * pi / (2 * k + 1));
                mr += ct.real();
                mi += ct.imag();
              }
        }
      }
      if (kgh >= kgl) {
        const int l1 = lc, m1 = nint(cml[i2]), s1 = nint(2 * cms[i2]);
        const int l2 = lv, m2 = nint(vml[i1]), s2 = nint(2 * vms[i1]);
        const int l3 = lv, m3 = nint(vml[i2]), s3 = nint(2 * vms[i2]);
        const int l4 = lc, m4 = nint(cml[i1]), s4 = nint(2 * cms[i1]);
        if (s1 == s3 && s2 == s4) {
          const int mk = m1 - m3;
          if (m1 + m2 == m3 + m4)
            for (int k = kgl; k <= kgh; k += 2)
              if (std::abs(mk) <= k) {
                const int ik = (k - kgl) / 2;
                const double ggk = scgk[ik] * gk[ik * npp + nu1 + (size_t)np * nu2] * scfac;
                const cd f1 = threey_ref(l1, m1, k, mk, l3, m3, false, xq, wq);
                const cd f2 = threey_ref(l2, m2, k, mk, l4, m4, true, xq, wq);
                const cd ct = ggk * f1 * f2 * (4 * pi / (2 * k + 1));
                mr += ct.real();
                mi += ct.imag();
              }
        }
      }
      // mhr_l(i1, i2) then the eV -> Hartree of OCEAN_create_central (:386-387)
      mhr_out[(size_t)i1 + (size_t)mham * i2] = mr * kEV2Ha;
      mhi_out[(size_t)i1 + (size_t)mham * i2] = mi * kEV2Ha;
    }
  }
  return mham;
}

// redtrid (OCEAN_haydock.f90:2273-2316): eigenvalues of the (n+1)x(n+1) Hermitian
// tridiagonal with diagonal real_a(0:n) and off-diagonal real_b(1:n).  elsch
// (EISPACK htridi + tqlrat) is restated as the equivalent symmetric tridiagonal
// implicit-QL eigenvalue iteration; the result is sorted ascending.
int or_redtrid(int n, const double* ra, const double* rb, double* w) {
  int nn = n + 1;
  std::vector<double> dd(nn), e(nn, 0.0);
  for (int i = 0; i < nn; ++i) dd[i] = ra[i];
  for (int i = 1; i < nn; ++i) e[i - 1] = std::fabs(rb[i]);
  for (int l = 0; l < nn; ++l) {
    int iter = 0;
    int m;
    do {
      for (m = l; m < nn - 1; ++m) {
        double dd2 = std::fabs(dd[m]) + std::fabs(dd[m + 1]);
        if (std::fabs(e[m]) <= 1e-16 * dd2) break;
      }
      if (m != l) {
        if (iter++ == 60) return 1;
        double g = (dd[l + 1] - dd[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = dd[m] - dd[l] + e[l] / (g + std::copysign(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; --i) {
          double f = s * e[i], b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) {
            dd[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = dd[i + 1] - p;
          r = (dd[i] - g) * s + 2.0 * c * b;
          p = s * r;
          dd[i + 1] = g + p;
          g = c * r - b;
        }
        if (r == 0.0 && i >= l) continue;
        dd[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  std::sort(dd.begin(), dd.end());
  for (int i = 0; i < nn; ++i) w[i] = dd[i];
  return 0;
}

// ------------------------------------------------------------ zhptrf/zhptrs

// LAPACK zhptrf, UPLO = 'U' (Bunch-Kaufman diagonal pivoting on packed Hermitian
// storage), as called at OCEAN_gmres.f90:309.  Restated from the published
// algorithm; 1-based index helpers keep the packed addressing readable.
int or_zhptrf_u(int n, double* ap_, int* ipiv) {
  cd* ap = reinterpret_cast<cd*>(ap_);
  auto P = [&](int i, int j) -> cd& { return ap[(i - 1) + (j - 1) * j / 2]; };  // i <= j
  auto cabs1 = [](cd z) { return std::fabs(z.real()) + std::fabs(z.imag()); };
  const double alpha = (1.0 + std::sqrt(17.0)) / 8.0;
  int info = 0;
  int k = n;
  while (k >= 1) {
    int kstep = 1;
    double absakk = std::fabs(P(k, k).real());
    int imax = 0;
    double colmax = 0.0;
    if (k > 1) {
      imax = 1;
      colmax = cabs1(P(1, k));
      for (int i = 2; i <= k - 1; ++i)
        if (cabs1(P(i, k)) > colmax) { colmax = cabs1(P(i, k)); imax = i; }
    }
    int kp;
    if (std::max(absakk, colmax) == 0.0 || std::isnan(absakk)) {
      if (info == 0) info = k;
      kp = k;
      P(k, k) = cd(P(k, k).real(), 0.0);
    } else {
      if (absakk >= alpha * colmax) {
        kp = k;
      } else {
        double rowmax = 0.0;
        for (int j = imax + 1; j <= k; ++j)
          if (cabs1(P(imax, j)) > rowmax) rowmax = cabs1(P(imax, j));
        if (imax > 1) {
          int jm = 1;
          double mx = cabs1(P(1, imax));
          for (int i = 2; i <= imax - 1; ++i)
            if (cabs1(P(i, imax)) > mx) { mx = cabs1(P(i, imax)); jm = i; }
          (void)jm;
          rowmax = std::max(rowmax, mx);
        }
        if (absakk >= alpha * colmax * (colmax / rowmax)) {
          kp = k;
        } else if (std::fabs(P(imax, imax).real()) >= alpha * rowmax) {
          kp = imax;
        } else {
          kp = imax;
          kstep = 2;
        }
      }
      int kk = k - kstep + 1;
      if (kp != kk) {
        for (int j = 1; j <= kp - 1; ++j) std::swap(P(j, kk), P(j, kp));
        for (int j = kp + 1; j <= kk - 1; ++j) {
          cd t = std::conj(P(j, kk));
          P(j, kk) = std::conj(P(kp, j));
          P(kp, j) = t;
        }
        P(kp, kk) = std::conj(P(kp, kk));
        double r1 = P(kk, kk).real();
        P(kk, kk) = cd(P(kp, kp).real(), 0.0);
        P(kp, kp) = cd(r1, 0.0);
        if (kstep == 2) {
          P(k, k) = cd(P(k, k).real(), 0.0);
          std::swap(P(k - 1, k), P(kp, k));
        }
      } else {
        P(k, k) = cd(P(k, k).real(), 0.0);
        if (kstep == 2) P(k - 1, k - 1) = cd(P(k - 1, k - 1).real(), 0.0);
      }
      if (kstep == 1) {
        double r1 = 1.0 / P(k, k).real();
        // ZHPR: A := A - r1 * x x^H on the leading (k-1) block, x = column k
        for (int j = 1; j <= k - 1; ++j) {
          cd xj = P(j, k);
          if (xj != cd(0.0, 0.0)) {
            cd temp = -r1 * std::conj(xj);
            for (int i = 1; i <= j - 1; ++i) P(i, j) += P(i, k) * temp;
            P(j, j) = cd(P(j, j).real() + (xj * temp).real(), 0.0);
          } else {
            P(j, j) = cd(P(j, j).real(), 0.0);
          }
        }
        for (int i = 1; i <= k - 1; ++i) P(i, k) *= r1;
      } else {
        if (k > 2) {
          cd a12 = P(k - 1, k);
          double dd = std::hypot(a12.real(), a12.imag());
          double d22 = P(k - 1, k - 1).real() / dd;
          double d11 = P(k, k).real() / dd;
          double tt = 1.0 / (d11 * d22 - 1.0);
          cd d12 = a12 / dd;
          dd = tt / dd;
          for (int j = k - 2; j >= 1; --j) {
            cd wkm1 = dd * (d11 * P(j, k - 1) - std::conj(d12) * P(j, k));
            cd wk = dd * (d22 * P(j, k) - d12 * P(j, k - 1));
            for (int i = j; i >= 1; --i)
              P(i, j) = P(i, j) - P(i, k) * std::conj(wk) - P(i, k - 1) * std::conj(wkm1);
            P(j, k) = wk;
            P(j, k - 1) = wkm1;
            P(j, j) = cd(P(j, j).real(), 0.0);
          }
        }
      }
    }
    if (kstep == 1) {
      ipiv[k - 1] = kp;
    } else {
      ipiv[k - 1] = -kp;
      ipiv[k - 2] = -kp;
    }
    k -= kstep;
  }
  return info;
}

// LAPACK zhptrs, UPLO = 'U', NRHS = 1 (OCEAN_gmres.f90:320).
int or_zhptrs_u(int n, const double* ap_, const int* ipiv, double* b_) {
  const cd* ap = reinterpret_cast<const cd*>(ap_);
  cd* b = reinterpret_cast<cd*>(b_);
  auto P = [&](int i, int j) -> cd { return ap[(i - 1) + (j - 1) * j / 2]; };
  auto B = [&](int i) -> cd& { return b[i - 1]; };
  int k = n;
  while (k >= 1) {
    if (ipiv[k - 1] > 0) {
      int kp = ipiv[k - 1];
      if (kp != k) std::swap(B(k), B(kp));
      for (int i = 1; i <= k - 1; ++i) B(i) -= P(i, k) * B(k);
      double s = 1.0 / P(k, k).real();
      B(k) *= s;
      k -= 1;
    } else {
      int kp = -ipiv[k - 1];
      if (kp != k - 1) std::swap(B(k - 1), B(kp));
      for (int i = 1; i <= k - 2; ++i) B(i) -= P(i, k) * B(k);
      for (int i = 1; i <= k - 2; ++i) B(i) -= P(i, k - 1) * B(k - 1);
      cd akm1k = P(k - 1, k);
      cd akm1 = P(k - 1, k - 1) / akm1k;
      cd ak = P(k, k) / std::conj(akm1k);
      cd denom = akm1 * ak - 1.0;
      cd bkm1 = B(k - 1) / akm1k;
      cd bk = B(k) / std::conj(akm1k);
      B(k - 1) = (ak * bkm1 - bk) / denom;
      B(k) = (akm1 * bk - bkm1) / denom;
      k -= 2;
    }
  }
  k = 1;
  while (k <= n) {
    if (ipiv[k - 1] > 0) {
      if (k > 1) {
        cd s = 0.0;
        for (int i = 1; i <= k - 1; ++i) s += std::conj(P(i, k)) * B(i);
        B(k) -= s;
      }
      int kp = ipiv[k - 1];
      if (kp != k) std::swap(B(k), B(kp));
      k += 1;
    } else {
      if (k > 1) {
        cd s = 0.0;
        for (int i = 1; i <= k - 1; ++i) s += std::conj(P(i, k)) * B(i);
        B(k) -= s;
        cd s2 = 0.0;
        for (int i = 1; i <= k - 1; ++i) s2 += std::conj(P(i, k + 1)) * B(i);
        B(k + 1) -= s2;
      }
      int kp = -ipiv[k - 1];
      if (kp != k) std::swap(B(k), B(kp));
      k += 2;
    }
  }
  return 0;
}

// ------------------------------------------------------------------- GMRES

namespace {

struct Vec {
  std::vector<double> r, i;
  explicit Vec(size_t n = 0) : r(n, 0.0), i(n, 0.0) {}
};

void dotc(const Vec& p, const Vec& q, double& rv, double& iv) {  // OCEAN_psi.f90:2029-2034
  double a = 0.0, b = 0.0;
  for (size_t j = 0; j < p.r.size(); ++j) {
    a += p.r[j] * q.r[j] + p.i[j] * q.i[j];
    b += p.r[j] * q.i[j] - p.i[j] * q.r[j];
  }
  rv = a;
  iv = b;
}
double nrm2(const Vec& x) {  // OCEAN_psi_nrm returns sum |x|^2, OCEAN_psi.f90:1704-1707
  double s = 0.0;
  for (size_t j = 0; j < x.r.size(); ++j) s += x.r[j] * x.r[j] + x.i[j] * x.i[j];
  return s;
}
// y = (rv + i iv) x - y, OCEAN_psi_axmy (OCEAN_psi.f90:1468-1562)
void axmy(const Vec& x, Vec& y, double rv, double iv) {
  for (size_t j = 0; j < x.r.size(); ++j) {
    double br = rv * x.r[j] - y.r[j];
    double bi = rv * x.i[j] - y.i[j];
    y.r[j] = br - iv * x.i[j];
    y.i[j] = bi + iv * x.r[j];
  }
}
// y = x - z, OCEAN_psi_axmz (OCEAN_psi.f90:1571-1661)
void axmz(const Vec& x, Vec& y, const Vec& z) {
  for (size_t j = 0; j < x.r.size(); ++j) {
    y.r[j] = x.r[j] - z.r[j];
    y.i[j] = x.i[j] - z.i[j];
  }
}
// y += (ar + i ai) x, OCEAN_psi_axpy (OCEAN_psi.f90:1386-1458)
void axpy(double ar, double ai, const Vec& x, Vec& y) {
  for (size_t j = 0; j < x.r.size(); ++j) {
    y.r[j] += ar * x.r[j] - ai * x.i[j];
    y.i[j] += ar * x.i[j] + ai * x.r[j];
  }
}
// OCEAN_psi_min_set_prec without prev_energy (OCEAN_psi.f90:2961-2965)
void set_prec(double energy, double gprc, const Vec& h, Vec& out) {
  double g2 = gprc * gprc;
  for (size_t j = 0; j < h.r.size(); ++j) {
    cd c(h.r[j], h.i[j]);
    cd e_minus = cd(energy, 0.0) - c;
    cd den = e_minus * e_minus + g2;
    cd num = cd(energy, 0.0) - cd(h.r[j], h.i[j] + gprc);
    cd q = num / den;
    out.r[j] = q.real();
    out.i[j] = q.imag();
  }
}

struct GmresState {
  std::function<void(const double*, const double*, double*, double*)> act;  // OCEAN_xact
  int depth;
  std::vector<Vec> u, au;
  std::vector<cd> cmat;  // packed upper, module-global c_matrix
  long long hpsi = 0;
  void H(const Vec& in, Vec& out) {
    act(in.r.data(), in.i.data(), out.r.data(), out.i.data());
    ++hpsi;
  }
  // update_gmres, OCEAN_gmres.f90:241-344
  int update(int cur, Vec& g, Vec& x, Vec& ax) {
    std::vector<double> rec(cur, 0.0), imc(cur, 0.0), rr(cur, 0.0), ri(cur, 0.0);
    for (int it = 1; it <= cur - 1; ++it) {
      dotc(au[cur - 1], au[it - 1], rec[it - 1], imc[it - 1]);
      dotc(au[it - 1], g, rr[it - 1], ri[it - 1]);
    }
    rec[cur - 1] = nrm2(au[cur - 1]);
    imc[cur - 1] = 0.0;
    dotc(au[cur - 1], g, rr[cur - 1], ri[cur - 1]);
    int start = cur * (cur - 1) / 2;
    for (int it = 1; it <= cur; ++it) cmat[it - 1 + start] = cd(rec[it - 1], -imc[it - 1]);
    int csize = cur * (cur + 1) / 2;
    std::vector<cd> ct(cmat.begin(), cmat.begin() + csize);
    std::vector<int> ipiv(cur);
    int info = or_zhptrf_u(cur, reinterpret_cast<double*>(ct.data()), ipiv.data());
    if (info != 0) return info;
    std::vector<cd> coeff(cur);
    for (int it = 0; it < cur; ++it) coeff[it] = -cd(rr[it], ri[it]);
    or_zhptrs_u(cur, reinterpret_cast<double*>(ct.data()), ipiv.data(),
                reinterpret_cast<double*>(coeff.data()));
    for (int it = 0; it < cur; ++it) {
      axpy(coeff[it].real(), coeff[it].imag(), u[it], x);
      axpy(coeff[it].real(), coeff[it].imag(), au[it], ax);
    }
    return 0;
  }
};

}  // namespace

// OCEAN_gmres_do_recycle, OCEAN_gmres.f90:508-908 (core, bwflg = F, loud = T,
// do_precondition = allow_reuse_x = force_reuse_x = allow_recycle = T per :24-27).
}  // extern "C"

namespace {

// OCEAN_gmres_do_recycle (OCEAN_gmres.f90:508-908) over an action on vectors of
// n complex values; allow: the sfact / allow mask (rhs = allow o hay, :586; with
// mask_ones the H*1 of the preconditioner is H(allow o 1), the valence branch
// :603-606); fact scales the output columns (kpref, or kpref 2 celvol for a
// valence run, :544-548).
int gmres_generic(size_t n, const double* allow, bool mask_ones,
                  const std::function<void(const double*, const double*, double*, double*)>& act,
                  const double* hay_r, const double* hay_i, double fact, const double* elist, int nomega, int depth,
                  double gres, double gprc, double ffff, int max_restarts, double* out_re, double* out_im,
                  double* rel_err, int* iters, int* total_hpsi) {
  GmresState st;
  st.act = act;
  st.depth = depth;
  st.u.assign(depth, Vec(n));
  st.au.assign(depth, Vec(n));
  st.cmat.assign((size_t)depth * (depth + 1) / 2, cd(0.0, 0.0));
  Vec x(n), ax(n), hpsi1(n), g(n), pcdiv(n), rhs(n);
  for (size_t j = 0; j < n; ++j) {  // sfact_copy: allow%i (= allow for core) o hay_vec
    rhs.r[j] = allow[j] * hay_r[j];
    rhs.i[j] = allow[j] * hay_i[j];
  }
  for (size_t j = 0; j < n; ++j) {  // psi_one_full (then allow_full for valence)
    x.r[j] = mask_ones ? allow[j] : 1.0;
    x.i[j] = 0.0;
  }
  st.H(x, hpsi1);
  int global_iter = 0, prev_iter = 0;
  double prev_energy = -1.0e308;
  double rval = 0, ival = 0, gval = 0;
  for (int step = 0; step < nomega; ++step) {
    int complete_iter = 0;
    double ener = elist[step] * kEV2Ha;
    bool converged = false;
    if (prev_iter == 0) {
      prev_energy = ener;
      set_prec(ener, gprc, hpsi1, pcdiv);
    }
    // set_initial_vector (OCEAN_gmres.f90:1213-1283): force_reuse_x keeps x for step > 0
    auto initial_vector = [&]() {
      if (step > 0) {
        st.H(x, ax);
        axmy(x, ax, ener, gres);
      } else {
        std::fill(x.r.begin(), x.r.end(), 0.0);
        std::fill(x.i.begin(), x.i.end(), 0.0);
        std::fill(ax.r.begin(), ax.r.end(), 0.0);
        std::fill(ax.i.begin(), ax.i.end(), 0.0);
      }
      axmz(ax, g, rhs);
    };
    if (prev_iter == 0) {
      initial_vector();
      gval = nrm2(g);
      dotc(rhs, x, rval, ival);
    } else {
      double delta = elist[step] * kEV2Ha - elist[step - 1] * kEV2Ha;  // make_recycle
      for (int i = 0; i < prev_iter; ++i) axpy(delta, 0.0, st.u[i], st.au[i]);
      initial_vector();
      for (int it = 1; it <= prev_iter; ++it) {
        int info = st.update(it, g, x, ax);
        if (info) return 7;
        axmz(ax, g, rhs);
      }
      gval = nrm2(g);
      dotc(rhs, x, rval, ival);
      if (gval < ffff) {
        dotc(rhs, x, rval, ival);
        double rel = -gval / ival;
        if (rel < 0.001 || gval < ffff / 10.0) converged = true;
      }
      if (!converged && std::fabs(prev_energy - ener) > gprc / 4.0) {
        prev_iter = 0;
        prev_energy = ener;
        set_prec(ener, gprc, hpsi1, pcdiv);
      }
    }
    int restarts = 0;
    while (!converged) {
      for (int iter = prev_iter + 1; iter <= depth; ++iter) {
        ++complete_iter;
        ++global_iter;
        Vec& pg = st.u[iter - 1];
        Vec& apg = st.au[iter - 1];
        for (size_t j = 0; j < n; ++j) {  // 3element_mult: pg = g o pcdiv
          pg.r[j] = g.r[j] * pcdiv.r[j] - g.i[j] * pcdiv.i[j];
          pg.i[j] = g.r[j] * pcdiv.i[j] + g.i[j] * pcdiv.r[j];
        }
        st.H(pg, apg);
        axmy(pg, apg, ener, gres);
        int info = st.update(iter, g, x, ax);
        if (info) return 7;
        if (iter == depth) {
          st.H(x, ax);
          axmy(x, ax, ener, gres);
          if (ener != prev_energy) {
            set_prec(ener, gprc, hpsi1, pcdiv);
            prev_energy = ener;
          }
          prev_iter = 0;
        }
        axmz(ax, g, rhs);
        gval = nrm2(g);
        dotc(rhs, x, rval, ival);
        if (gval < ffff) {
          dotc(rhs, x, rval, ival);
          double rel = -gval / ival;
          if (rel < 0.001 || gval < ffff / 10.0) {
            prev_iter = iter;
            if (iter == depth) prev_iter = 0;
            converged = true;
            break;
          }
        }
      }
      if (converged) break;
      if (++restarts > max_restarts) return 6;
    }
    if (out_re) out_re[step] = 1.0 - rval * fact;
    if (out_im) out_im[step] = -ival * fact;
    if (rel_err) rel_err[step] = -gval / ival;
    if (iters) iters[step] = complete_iter;
  }
  if (total_hpsi) *total_hpsi = (int)st.hpsi;
  return 0;
}

}  // namespace

extern "C" {

int or_gmres(const or_dims* d, const or_ops* o, const double* hay_r, const double* hay_i,
             double kpref, const double* elist, int nomega, int depth, double gres, double gprc,
             double ffff, int max_restarts, double* out_re, double* out_im, double* rel_err,
             int* iters, int* total_hpsi) {
  const size_t n = (size_t)d->nb * nk_of(d) * d->na;
  auto act = [&](const double* pr, const double* pi, double* hr, double* hi) {
    or_xact(d, o, pr, pi, hr, hi, nullptr, 0);
  };
  return gmres_generic(n, o->allow, false, act, hay_r, hay_i, kpref, elist, nomega, depth, gres, gprc, ffff,
                       max_restarts, out_re, out_im, rel_err, iters, total_hpsi);
}

// GMRES over a caller-supplied action (the valence action of ocean_oracle_val.cpp).
int or_gmres_with(size_t n, const double* allow, int mask_ones,
                  void (*act)(void* user, const double* pr, const double* pi, double* hr, double* hi), void* user,
                  const double* hay_r, const double* hay_i, double fact, const double* elist, int nomega, int depth,
                  double gres, double gprc, double ffff, int max_restarts, double* out_re, double* out_im,
                  double* rel_err, int* iters, int* total_hpsi) {
  auto f = [&](const double* pr, const double* pi, double* hr, double* hi) { act(user, pr, pi, hr, hi); };
  return gmres_generic(n, allow, mask_ones != 0, f, hay_r, hay_i, fact, elist, nomega, depth, gres, gprc, ffff,
                       max_restarts, out_re, out_im, rel_err, iters, total_hpsi);
}

// OCEAN_soprep without core_broaden.ipt (OCEAN_multiplet.f90:572-690), jimel
// from CNBSE/zcmsnmult/zf90/jimel.f90:10-39; channel order from :345-360.
int or_soprep(int lc, double xi, double* somelr, double* someli) {
  int na = 4 * (2 * lc + 1);
  std::vector<double> cms(na), cml(na), vms(na);
  int ic = 0;
  for (int icms = -1; icms <= 1; icms += 2)
    for (int icml = -lc; icml <= lc; ++icml)
      for (int ivms = -1; ivms <= 1; ivms += 2) {
        cms[ic] = 0.5 * icms;
        cml[ic] = icml;
        vms[ic] = 0.5 * ivms;
        ++ic;
      }
  auto jimel = [](double j, double m, double mp, int i) -> cd {
    double x = std::fabs(j * (j + 1.0) - m * mp);
    int mdiff = (int)std::lround(m - mp);
    cd rm1(0.0, 1.0);
    switch (i) {
      case 1:
        if (mdiff == 1 || mdiff == -1) return cd(0.5 * std::sqrt(x), 0.0);
        return cd(0.0, 0.0);
      case 2:
        if (mdiff == 1) return cd(0.5 * std::sqrt(x), 0.0) / rm1;
        if (mdiff == -1) return cd(-0.5 * std::sqrt(x), 0.0) / rm1;
        return cd(0.0, 0.0);
      default:
        if (mdiff == 0) return cd(m, 0.0);
        return cd(0.0, 0.0);
    }
  };
  for (int a = 0; a < na; ++a)
    for (int b = 0; b < na; ++b) {
      somelr[a + na * b] = 0.0;
      someli[a + na * b] = 0.0;
      if (vms[a] == vms[b]) {
        cd ctmp(0.0, 0.0);
        for (int i = 1; i <= 3; ++i)
          ctmp += jimel((double)lc, cml[b], cml[a], i) * jimel(0.5, cms[b], cms[a], i);
        somelr[a + na * b] = -xi * ctmp.real();
        someli[a + na * b] = -ctmp.real() * 0.0;
      }
    }
  return 0;
}

}  // extern "C"
