// ocn_setup.cpp -- host-side set-up of the long-range operator (index maps, the
// core-hole phase table, the W(R,x) table), the spin-orbit matrix and the
// tridiagonal eigen-solver.  Compiled with -ffp-contract=off so that every
// product and sum rounds exactly as written (the W table and phase table are
// compared bit for bit against an independent CPU restatement).
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "ocn_internal.h"

namespace ocn {

namespace {
inline int prod3(const int v[3]) { return v[0] * v[1] * v[2]; }

// Signed supercell index of k-mesh point k (0-based) along one axis: the upper
// half folds to negative values, with the extra cell of an even mesh on the
// negative side (long_range.f90:1777-1781).
inline int fold(int k0, int n) {
  if (n == 1) return 0;
  return (k0 >= (n + 1) / 2) ? k0 - n : k0;
}

// Wraps a shifted 1-based x-mesh index back into 1..n (long_range.f90:1749-1773).
inline int wrap1(int t, int n) {
  if (t > n) return t - n;
  if (t < 1) return t + n;
  return t;
}
}  // namespace

// xshift and the shifted core position of OCEAN_bloch_lrLOAD
// (OCEAN_bloch.f90:94-123): an even k-mesh centres the core hole near the origin
// of the x-mesh, an odd one near the middle.
void lrload_shift(const ocn_dims& d, double tau[3], const int ovr[3], int xshift[3]) {
  for (int i = 0; i < 3; ++i) {
    const double nxm = (double)d.xmesh[i];
    const double t = (d.kmesh[i] % 2 == 0) ? tau[i] : tau[i] - 0.5;
    xshift[i] = (int)std::floor(nxm * t) * (ovr ? ovr[i] : 1);
  }
  for (int i = 0; i < 3; ++i) tau[i] -= (double)xshift[i] / (double)d.xmesh[i];
}

// Phase e^{i phi(x,q)} that OCEAN_bloch_lrLOAD (OCEAN_bloch.f90:141-204) multiplies
// into u(n,q,x): phi = 2 pi sum_i (xph_i + x_i - 1)(q_i - 1) / (Nx_i Nk_i), where
// xph_i = -/+ Nx_i when the shifted point wrapped.  Stored as cos/sin at [x*Nk + q].
void lrload_phase_table(const ocn_dims& d, const int xshift[3], std::vector<double>& c,
                        std::vector<double>& s) {
  const int nk = prod3(d.kmesh), nx = prod3(d.xmesh);
  c.assign((size_t)nk * nx, 0.0);
  s.assign((size_t)nk * nx, 0.0);
  const double pi = 4.0 * std::atan(1.0);
  for (int xi = 0; xi < nx; ++xi) {
    const int ix = xi % d.xmesh[0] + 1;
    const int iy = (xi / d.xmesh[0]) % d.xmesh[1] + 1;
    const int iz = xi / (d.xmesh[0] * d.xmesh[1]) + 1;
    const int pos[3] = {ix, iy, iz};
    int ph[3];
    for (int a = 0; a < 3; ++a) {
      const int t = pos[a] - xshift[a];
      ph[a] = (t > d.xmesh[a]) ? -d.xmesh[a] : ((t < 1) ? d.xmesh[a] : 0);
    }
    for (int q = 0; q < nk; ++q) {
      const int q3 = q % d.kmesh[2] + 1;
      const int q2 = (q / d.kmesh[2]) % d.kmesh[1] + 1;
      const int q1 = q / (d.kmesh[2] * d.kmesh[1]) + 1;
      const int qq[3] = {q1, q2, q3};
      double angle[3];
      for (int a = 0; a < 3; ++a)
        angle[a] = 2.0 * pi * (double)((ph[a] + pos[a] - 1) * (qq[a] - 1)) /
                   (double)(d.xmesh[a] * d.kmesh[a]);
      const double total = angle[0] + angle[1] + angle[2];
      c[(size_t)xi * nk + q] = std::cos(total);
      s[(size_t)xi * nk + q] = std::sin(total);
    }
  }
}

namespace {

// Geometry of lr_populate_W2 (long_range.f90:1659-1853): for every supercell
// vector R (k-mesh index, k3 fastest) and x-mesh point x (x fastest, z slowest)
// calls f(index x*Nk + k, r, pbc prefactor, alf) with r = |R + x_frac - tau| in
// the metric of avec and alf the lattice coordinates of that separation.
template <class F>
void w2_visit(const ocn_dims& d, const ocn_lr_params& p, const double tau[3], const int xshift[3], F f) {
  const int nk = prod3(d.kmesh), nx = prod3(d.xmesh);
  double metric[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int c = 0; c < 3; ++c) acc += p.avec[c + 3 * i] * p.avec[c + 3 * j];
      metric[i][j] = acc;
    }
  const bool any_pbc = (p.pbc[0] | p.pbc[1] | p.pbc[2]) != 0;
  int pbc[3];
  for (int i = 0; i < 3; ++i) pbc[i] = any_pbc ? (p.pbc[i] != 0 ? d.kmesh[i] : 0) : d.kmesh[i];
  for (int xi = 0; xi < nx; ++xi) {
    const int pos[3] = {xi % d.xmesh[0] + 1, (xi / d.xmesh[0]) % d.xmesh[1] + 1,
                        xi / (d.xmesh[0] * d.xmesh[1]) + 1};
    double frac[3];
    for (int a = 0; a < 3; ++a)
      frac[a] = (double)(wrap1(pos[a] - xshift[a], d.xmesh[a]) - 1) / (double)d.xmesh[a];
    for (int k = 0; k < nk; ++k) {
      const int k3 = k % d.kmesh[2];
      const int k2 = (k / d.kmesh[2]) % d.kmesh[1];
      const int k1 = k / (d.kmesh[2] * d.kmesh[1]);
      const int R[3] = {fold(k1, d.kmesh[0]), fold(k2, d.kmesh[1]), fold(k3, d.kmesh[2])};
      // pbc_prefac chain of long_range.f90:1782-1812
      double pref = (R[0] > pbc[0]) ? 0.0 : 1.0;
      pref = (R[1] > pbc[1]) ? 0.0 : pref;
      pref = (R[2] > pbc[2]) ? 0.0 : pref;
      double alf[3];
      for (int a = 0; a < 3; ++a) alf[a] = (double)R[a] + frac[a] - tau[a];
      double r2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        double m = 0.0;
        for (int j = 0; j < 3; ++j) m += metric[i][j] * alf[j];
        r2 += alf[i] * m;
      }
      f((size_t)xi * nk + k, std::sqrt(r2), pref, alf);
    }
  }
}

// Table interval of r for the linear interpolation of intval ('cap', 'cap'):
// W = (1 - t) ptab[i] + t ptab[i+1]; below the first radius t = 0, i = 0.
inline void w2_interval(const ocn_lr_params& p, double r, int* i_out, double* t_out) {
  if (r < p.rtab[0]) {
    *i_out = 0;
    *t_out = 0.0;
    return;
  }
  int i = 0;
  while (p.rtab[i + 1] < r) ++i;
  *i_out = i;
  *t_out = (r - p.rtab[i]) / (p.rtab[i + 1] - p.rtab[i]);
}

}  // namespace

// W(R, x) of lr_populate_W2 (long_range.f90:1659-1853): the screened core-hole
// potential between supercell vector R and x-mesh point x relative to the
// shifted core site, times interactionScale.  Stored at [x*Nk + k] (the Fortran
// W(k, x)).
void populate_w2(const ocn_dims& d, const ocn_lr_params& p, const double tau[3], const int xshift[3],
                 std::vector<double>& W) {
  W.assign((size_t)prod3(d.kmesh) * prod3(d.xmesh), 0.0);
  const double epsi = 1.0 / p.epsilon0;
  const double rlast = p.rtab[p.nptab - 1];
  w2_visit(d, p, tau, xshift, [&](size_t idx, double r, double pref, const double alf[3]) {
    double v;
    if (p.isolated && r > p.iso_cut) {
      v = 0.0;
    } else if (r > rlast) {
      if (p.have_eps3d) {
        double dir[3];
        for (int c = 0; c < 3; ++c) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc += p.avec[c + 3 * j] * alf[j];
          dir[c] = acc / r;
        }
        v = (dir[0] * dir[0] / p.epsilon3d[0] + dir[1] * dir[1] / p.epsilon3d[1] +
             dir[2] * dir[2] / p.epsilon3d[2]) / r;
        if (r < rlast + 5.0) v = v * (r - rlast) / 5.0 + (rlast + 5.0 - r) * epsi / (5.0 * r);
      } else {
        v = epsi / r;
      }
    } else if (r < p.rtab[0]) {
      v = p.ptab[0];
    } else {
      int i;
      double t;
      w2_interval(p, r, &i, &t);
      v = p.ptab[i] + t * (p.ptab[i + 1] - p.ptab[i]);
    }
    W[idx] = v * pref * p.interaction_scale;
  });
}

// Vector-Jacobian product of populate_w2: given G = dL/dW (at [x*Nk + k]),
// g_ptab[m] = sum G dW/dptab_m (only entries with r inside the table depend on
// it) and g_scale = sum G dW/d(interactionScale) = sum G W / interactionScale.
void w2_vjp(const ocn_dims& d, const ocn_lr_params& p, const double tau[3], const int xshift[3],
            const double* G, double* g_ptab, double* g_scale) {
  std::vector<double> W;
  populate_w2(d, p, tau, xshift, W);
  const double rlast = p.rtab[p.nptab - 1];
  for (int m = 0; m < p.nptab; ++m) g_ptab[m] = 0.0;
  double gs = 0.0;
  w2_visit(d, p, tau, xshift, [&](size_t idx, double r, double pref, const double*) {
    const double gw = G[idx];
    gs += gw * W[idx];
    if ((p.isolated && r > p.iso_cut) || r > rlast) return;
    const double f = gw * pref * p.interaction_scale;
    if (r < p.rtab[0]) {
      g_ptab[0] += f;
      return;
    }
    int i;
    double t;
    w2_interval(p, r, &i, &t);
    g_ptab[i] += f * (1.0 - t);
    g_ptab[i + 1] += f * t;
  });
  *g_scale = (p.interaction_scale != 0.0) ? gs / p.interaction_scale : 0.0;
}

// Spin-orbit matrix of OCEAN_soprep (OCEAN_multiplet.f90:572-690) without the
// core_broaden.ipt lifetime terms: somelr(ic,jc) = -xi <l ml_i|l|l ml_j>.<s_i|s|s_j>
// for equal valence spins, channels ordered (core ms, core ml, valence ms) with
// valence ms fastest (:345-360).  Matrix elements of the angular-momentum
// components follow CNBSE/zcmsnmult/zf90/jimel.f90:10-39.
void soprep(int lc, double xi, std::vector<double>& re, std::vector<double>& im) {
  typedef std::complex<double> cd;
  const int na = 4 * (2 * lc + 1);
  std::vector<double> cms, cml, vms;
  for (int a = -1; a <= 1; a += 2)
    for (int m = -lc; m <= lc; ++m)
      for (int v = -1; v <= 1; v += 2) {
        cms.push_back(0.5 * a);
        cml.push_back((double)m);
        vms.push_back(0.5 * v);
      }
  // <j m | J_i | j mp>, i = x, y, z
  auto jmat = [](double j, double m, double mp, int i) -> cd {
    const double x = std::fabs(j * (j + 1.0) - m * mp);
    const long dm = std::lround(m - mp);
    if (i == 3) return dm == 0 ? cd(m, 0.0) : cd(0.0, 0.0);
    if (dm != 1 && dm != -1) return cd(0.0, 0.0);
    const double h = 0.5 * std::sqrt(x);
    if (i == 1) return cd(h, 0.0);
    // (+-0.5 sqrt(x)) / i
    return dm == 1 ? cd(h, 0.0) / cd(0.0, 1.0) : cd(-h, 0.0) / cd(0.0, 1.0);
  };
  re.assign((size_t)na * na, 0.0);
  im.assign((size_t)na * na, 0.0);
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < na; ++j) {
      if (vms[i] != vms[j]) continue;
      cd sum(0.0, 0.0);
      for (int comp = 1; comp <= 3; ++comp)
        sum += jmat((double)lc, cml[j], cml[i], comp) * jmat(0.5, cms[j], cms[i], comp);
      re[(size_t)i + (size_t)na * j] = -xi * sum.real();
      im[(size_t)i + (size_t)na * j] = 0.0;
    }
}

// Energy-dependent valence damping of the old XAS broadening model
// (CNBSE/zcmsnmult/zf90/gamfcn.f90:8-42): plasmon-pole integral over momentum
// transfer for an electron gas of density n with dielectric constant e0.
double gamfcn(double e, double n, double e0) {
  const double pi = 3.14159265358979;
  const double kf = std::pow(3.0 * pi * pi * n, 1.0 / 3.0);
  const double wp = std::sqrt(4.0 * pi * n);
  double k = kf * kf / 2.0 + e;
  if (k < kf * kf / 2.0) return 0.0;
  k = std::sqrt(2.0 * k);
  const double wf = kf * kf / 2.0;
  const double lam = std::sqrt(wp * wp / (wf * wf * (e0 - 1.0)));
  const double dq = 0.005 * kf;
  double q = 0.5 * dq, su = 0.0;
  for (long guard = 0; guard < 100000000L; ++guard) {
    const double qq = q / kf;
    const double xp = qq * (2.0 + qq) / lam;
    const double xm = qq * (2.0 - qq) / lam;
    const double term1 = lam / (2.0 * qq * qq * qq) * (std::atan(xp) + std::atan(xm));
    const double term2 = (0.125 * lam * lam / std::pow(qq, 5) + 0.5 / (qq * qq * qq) - 0.125 / qq) *
                         std::log((1.0 + xp * xp) / (1.0 + xm * xm));
    const double epsq = 1.0 + 2.0 / (pi * kf) * (1.0 / (qq * qq) - term1 + term2);
    const double wq = wp / std::sqrt(1.0 - 1.0 / epsq);
    const bool above = (k * k - kf * kf - 2.0 * wq > 0.0);
    const bool inside = (k * q - wq - q * q / 2.0 > 0.0);
    if (above && inside) su = su + dq / (q * wq);
    q = q + dq;
    if (!above) break;
  }
  return wp * wp * su / (2.0 * k);
}

// Eigenvalues of the symmetric tridiagonal Lanczos matrix (redtrid,
// OCEAN_haydock.f90:2273-2316): implicit-shift QL iteration, sorted ascending.
int redtrid_eigs(int n, const double* ra, const double* rb, double* w) {
  const int m = n + 1;
  std::vector<double> dg(ra, ra + m), off(m, 0.0);
  for (int i = 0; i < n; ++i) off[i] = std::fabs(rb[i + 1]);
  for (int l = 0; l < m; ++l) {
    for (int sweep = 0;; ++sweep) {
      int e = l;
      while (e < m - 1 && std::fabs(off[e]) > 1e-16 * (std::fabs(dg[e]) + std::fabs(dg[e + 1]))) ++e;
      if (e == l) break;
      if (sweep >= 60) return 1;
      double g = (dg[l + 1] - dg[l]) / (2.0 * off[l]);
      double r = std::hypot(g, 1.0);
      g = dg[e] - dg[l] + off[l] / (g + std::copysign(r, g));
      double sn = 1.0, cs = 1.0, p = 0.0;
      bool early = false;
      for (int i = e - 1; i >= l; --i) {
        const double f = sn * off[i], b = cs * off[i];
        r = std::hypot(f, g);
        off[i + 1] = r;
        if (r == 0.0) {
          dg[i + 1] -= p;
          off[e] = 0.0;
          early = true;
          break;
        }
        sn = f / r;
        cs = g / r;
        g = dg[i + 1] - p;
        r = (dg[i] - g) * sn + 2.0 * cs * b;
        p = sn * r;
        dg[i + 1] = g + p;
        g = cs * r - b;
      }
      if (early) continue;
      dg[l] -= p;
      off[l] = g;
      off[e] = 0.0;
    }
  }
  std::sort(dg.begin(), dg.end());
  std::copy(dg.begin(), dg.end(), w);
  return 0;
}

// ---- nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181): the exchange matrices of
// the multiplet term from Slater integrals and angular algebra.
namespace {

double lfact(int n) {  // log(n!)
  return std::lgamma((double)n + 1.0);
}

// Wigner 3j symbol (j1 j2 j3; m1 m2 m3) for integer arguments (Racah's formula).
double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
  const double tri = 0.5 * (lfact(j1 + j2 - j3) + lfact(j1 - j2 + j3) + lfact(-j1 + j2 + j3) - lfact(j1 + j2 + j3 + 1));
  const double pre = 0.5 * (lfact(j1 + m1) + lfact(j1 - m1) + lfact(j2 + m2) + lfact(j2 - m2) + lfact(j3 + m3) +
                            lfact(j3 - m3));
  const int t0 = std::max(std::max(0, j2 - j3 - m1), j1 - j3 + m2);
  const int t1 = std::min(std::min(j1 + j2 - j3, j1 - m1), j2 + m2);
  double sum = 0.0;
  for (int t = t0; t <= t1; ++t) {
    const double den = lfact(t) + lfact(j3 - j2 + t + m1) + lfact(j3 - j1 + t - m2) + lfact(j1 + j2 - j3 - t) +
                       lfact(j1 - t - m1) + lfact(j2 - t + m2);
    sum += ((t & 1) ? -1.0 : 1.0) * std::exp(tri + pre - den);
  }
  return ((j1 - j2 - m3) & 1) ? -sum : sum;
}

// threey (CNBSE/zcmsnmult/zf90/newthreey.f90): integral over the sphere of
// conj(Y_{ll,ml}) Y_{lm,mm} Y_{lr,mr} (Y_{lm,mm} conjugated when conjug), with
// the complex spherical harmonics of newgetylm (Condon-Shortley phase).  The
// reference integrates it by quadrature in cos(theta) at phi = 0 (times 2 pi,
// the phi integral of the m-selected integrand); here it is the closed form
// (-1)^ml sqrt((2ll+1)(2lm+1)(2lr+1)/4pi) (ll lm lr; 0 0 0)(ll lm lr; -ml mm mr),
// with conj(Y_{l,m}) = (-1)^m Y_{l,-m}.  The reference's selection rules
// (m balance, lm in ll+lr, ll+lr-2, ..., max(|mm|, |ll-lr|)) give the same zeros.
double threey(int ll, int ml, int lm, int mm, int lr, int mr, bool conjug) {
  double sign = 1.0;
  if (conjug) {
    if (mm & 1) sign = -1.0;
    mm = -mm;
  }
  if (ml != mm + mr) return 0.0;
  if (((ll + lm + lr) & 1) != 0) return 0.0;
  const double pi = 3.14159265358979323846;
  const double pre = std::sqrt((2.0 * ll + 1.0) * (2.0 * lm + 1.0) * (2.0 * lr + 1.0) / (4.0 * pi));
  const double s_ml = (ml & 1) ? -1.0 : 1.0;
  return sign * s_ml * pre * wigner3j(ll, lm, lr, 0, 0, 0) * wigner3j(ll, lm, lr, -ml, mm, mr);
}

}  // namespace

int mult_exchange_matrix(int lc, int lv, int np, int kfl, int kfh, const double* fk, const double* scfk, int kgl,
                         int kgh, const double* gk, const double* scgk, double scfac, double* mhr, double* mhi) {
  const int na = 4 * (2 * lc + 1);
  const int mham = na * (2 * lv + 1) * np;
  // the basis of OCEAN_multiplet.f90:342-369: alpha = (core spin, core m, valence
  // spin) with the valence spin fastest, then valence m, then the radial index nu
  // fastest of all
  std::vector<int> cms(mham), cml(mham), vms(mham), vml(mham), vnu(mham);
  {
    int ii = 0;
    for (int icms = -1; icms <= 1; icms += 2)
      for (int icml = -lc; icml <= lc; ++icml)
        for (int ivms = -1; ivms <= 1; ivms += 2)
          for (int ivml = -lv; ivml <= lv; ++ivml)
            for (int nu = 0; nu < np; ++nu, ++ii) {
              cms[ii] = icms;  // 2 * spin
              cml[ii] = icml;
              vms[ii] = ivms;
              vml[ii] = ivml;
              vnu[ii] = nu;
            }
  }
  const double pi = 3.14159265358979323846;
  const double ev2ha = 0.036749322175666;
  const size_t npp = (size_t)np * np;
  for (int i2 = 0; i2 < mham; ++i2)
    for (int i1 = 0; i1 < mham; ++i1) {
      const int nu1 = vnu[i1], nu2 = vnu[i2];
      double acc = 0.0;
      if (kfh >= kfl && fk) {  // direct Slater F^k part
        const int m1 = cml[i2], s1 = cms[i2], m2 = vml[i1], s2 = vms[i1];
        const int m3 = cml[i1], s3 = cms[i1], m4 = vml[i2], s4 = vms[i2];
        if (s1 == s3 && s2 == s4 && m1 + m2 == m3 + m4) {
          const int mk = m1 - m3;
          for (int k = kfl; k <= kfh; k += 2) {
            if (std::abs(mk) > k) continue;
            const int ik = (k - kfl) / 2;
            const double ffk = scfk[ik] * fk[ik * npp + nu1 + (size_t)np * nu2] * scfac;
            const double f1 = threey(lc, m1, k, mk, lc, m3, false);
            const double f2 = threey(lv, m2, k, mk, lv, m4, true);
            acc += -ffk * f1 * f2 * (4.0 * pi / (2.0 * k + 1.0));
          }
        }
      }
      if (kgh >= kgl && gk) {  // exchange Slater G^k part
        const int m1 = cml[i2], s1 = cms[i2], m2 = vml[i1], s2 = vms[i1];
        const int m3 = vml[i2], s3 = vms[i2], m4 = cml[i1], s4 = cms[i1];
        if (s1 == s3 && s2 == s4 && m1 + m2 == m3 + m4) {
          const int mk = m1 - m3;
          for (int k = kgl; k <= kgh; k += 2) {
            if (std::abs(mk) > k) continue;
            const int ik = (k - kgl) / 2;
            const double ggk = scgk[ik] * gk[ik * npp + nu1 + (size_t)np * nu2] * scfac;
            const double f1 = threey(lc, m1, k, mk, lv, m3, false);
            const double f2 = threey(lv, m2, k, mk, lc, m4, true);
            acc += ggk * f1 * f2 * (4.0 * pi / (2.0 * k + 1.0));
          }
        }
      }
      // mhr_l(i1, i2), i1 fastest; eV -> Hartree as OCEAN_create_central does (:386-387)
      mhr[(size_t)i1 + (size_t)mham * i2] = acc * ev2ha;
      mhi[(size_t)i1 + (size_t)mham * i2] = 0.0;
    }
  return mham;
}

double gaunt_threey(int ll, int ml, int lm, int mm, int lr, int mr, int conjug) {
  return threey(ll, ml, lm, mm, lr, mr, conjug != 0);
}

}  // namespace ocn
