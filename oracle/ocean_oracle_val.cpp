// ocean_oracle_val.cpp -- CPU ORACLE for the valence BSE action (test
// infrastructure only; never linked into the product library).  A plain FP64
// restatement of the reference Fortran for resonant pairs (nbw = 1), one or two
// valence-Hamiltonian spins (valence_ham_spin) and DFT spins (nspn):
//
//   H psi = E o psi + allow o [ 2 X(allow o psi) - D(allow o psi) ]
//
// with the exchange ("bubble") X of OCEAN2/OCEAN_bubble.f90:420-796 and the
// screened direct ("ladder") D of OCEAN2/OCEAN_ladder.f90:155-1004, in the
// order of OCEAN_xact's valence branch (OCEAN2/OCEAN_action.f90:521-575,
// 590-600).
//
// Layouts (Fortran order of the reference arrays, single rank):
//   psi, E, allow   (Nc, Nv, Nk, vs^2) psi%valr/vali(c, v, k, ibeta)
//   con             (Nx, Nc, Nk, nspn) re_con/im_con(x, c, k, spin)
//   val             (Nx, Nv, Nk, nspn) re_val/im_val(x, v, k, spin)
//   bubble          (Nx)              bubble(x) of AI_bubble_populate
//   ladder          (Nk, Nx, Nx)      ladder(k, x, y) after resort_ladder
// The flat k index runs k3 fastest and the flat x index x3 fastest, the FFT
// orders of OCEAN_ladder_init (OCEAN_ladder.f90:1599-1695) and
// AI_bubble_prep (OCEAN_bubble.f90:67-157).
//
// Parity status: unpinned by reference data (the reference ships no valence
// states, bubble or ladder files); pinned by Hermiticity, a dense-H check and
// agreement with the cited source.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "ocean_oracle.h"

namespace {

const double kPiV = 3.14159265358979323846;

inline int nk_of(const or_val_dims* d) { return d->kmesh[0] * d->kmesh[1] * d->kmesh[2]; }
inline int nx_of(const or_val_dims* d) { return d->xmesh[0] * d->xmesh[1] * d->xmesh[2]; }

// gvec_length, OCEAN_bubble.f90:38-47 (the squared length |B g|^2; bvec
// column j is the j-th reciprocal vector, b[i + 3 j] = bvec(i+1, j+1)).
double gvec_length(const int g[3], const double* b) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) {
    const double c = b[i] * g[0] + b[i + 3] * g[1] + b[i + 6] * g[2];
    s += c * c;
  }
  return s;
}

int ifloor_half(int n) { return (int)std::floor(-(double)n / 2.0); }
int iceil_half(int n) { return (int)std::ceil((double)n / 2.0); }

}  // namespace

extern "C" {

// wall_search_old_way, OCEAN_bubble.f90:238-297.
double or_val_wall_length(const int xmesh[3], const double bvec[9]) {
  double length = HUGE_VAL;
  int g[3];
  for (g[0] = ifloor_half(xmesh[0]); g[0] <= iceil_half(xmesh[0]); ++g[0])
    for (g[1] = ifloor_half(xmesh[1]); g[1] <= iceil_half(xmesh[1]); ++g[1])
      for (g[2] = ifloor_half(xmesh[2]); g[2] <= iceil_half(xmesh[2]); ++g[2])
        if (2 * std::abs(g[2]) >= xmesh[2] || 2 * std::abs(g[1]) >= xmesh[1] || 2 * std::abs(g[0]) >= xmesh[0]) {
          const double t = gvec_length(g, bvec);
          if (t < length) length = t;
        }
  double next = 0.0;
  for (g[0] = ifloor_half(xmesh[0]); g[0] <= iceil_half(xmesh[0]); ++g[0])
    for (g[1] = ifloor_half(xmesh[1]); g[1] <= iceil_half(xmesh[1]); ++g[1])
      for (g[2] = ifloor_half(xmesh[2]); g[2] <= iceil_half(xmesh[2]); ++g[2]) {
        const double t = gvec_length(g, bvec);
        if (t < length && t > next) next = t;
      }
  return 0.5 * (length + next);
}

// AI_bubble_populate, OCEAN_bubble.f90:300-407: bubble(x) on the x-mesh in
// the FFT order (x3 fastest), G = 0 removed.  Returns the number of retained
// G-vectors minus one, as the reference prints it.
int or_val_bubble_populate(const int xmesh[3], const double bvec[9], const double qinb[3], double celvol,
                           int nkpts, double length, double* bubble) {
  const int n1 = xmesh[0], n2 = xmesh[1], n3 = xmesh[2];
  const int nx = n1 * n2 * n3;
  double bmet[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int c = 0; c < 3; ++c) s += bvec[c + 3 * i] * bvec[c + 3 * j];
      bmet[i][j] = s;
    }
  const double floor_g2 = 8.0 * kPiV * kPiV * kPiV / (celvol * (double)nx);
  for (int i = 0; i < nx; ++i) bubble[i] = 0.0;
  int igvec = 0;
  int g[3];
  for (g[0] = (int)std::ceil(-(double)n1 / 2.0); g[0] <= (int)std::floor((double)n1 / 2.0); ++g[0])
    for (g[1] = (int)std::ceil(-(double)n2 / 2.0); g[1] <= (int)std::floor((double)n2 / 2.0); ++g[1])
      for (g[2] = (int)std::ceil(-(double)n3 / 2.0); g[2] <= (int)std::floor((double)n3 / 2.0); ++g[2]) {
        double qq[3];
        for (int i = 0; i < 3; ++i) qq[i] = qinb[i] + (double)g[i];
        double gsqd = 0.0;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) gsqd += qq[i] * qq[j] * bmet[i][j];
        if (gsqd < floor_g2) gsqd = floor_g2;  // vanishing q (:350-357, :364-372)
        int ixx = 1 + g[0], iyy = 1 + g[1], izz = 1 + g[2];
        if (ixx <= 0) ixx += n1;
        if (iyy <= 0) iyy += n2;
        if (izz <= 0) izz += n3;
        double mul = 0.0;
        if (gvec_length(g, bvec) < length) {
          mul = 4.0 * kPiV / (celvol * gsqd * (double)nkpts);
          ++igvec;
        }
        bubble[(izz - 1) + n3 * ((iyy - 1) + n2 * (ixx - 1))] = mul;  // later g overwrite (even meshes)
      }
  bubble[0] = 0.0;
  return igvec - 1;
}

// A(x, v, k) = sum_c con(x, c, k) psi(c, v, k): the first DGEMM group of both
// AI_bubble_act (OCEAN_bubble.f90:521-530) and OCEAN_ladder_act_single
// (OCEAN_ladder.f90:317-326).
static void val_amat(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi,
                     std::vector<double>& ar, std::vector<double>& ai) {
  const int nc = d->nc, nv = d->nv, nk = nk_of(d), nx = nx_of(d);
  ar.assign((size_t)nx * nv * nk, 0.0);
  ai.assign((size_t)nx * nv * nk, 0.0);
  for (int k = 0; k < nk; ++k)
    for (int v = 0; v < nv; ++v)
      for (int c = 0; c < nc; ++c) {
        const size_t ip = c + (size_t)nc * (v + (size_t)nv * k);
        const double qr = pr[ip], qi = pi[ip];
        const double* cr = o->conr + (size_t)nx * (c + (size_t)nc * k);
        const double* ci = o->coni + (size_t)nx * (c + (size_t)nc * k);
        double* a_r = ar.data() + (size_t)nx * (v + (size_t)nv * k);
        double* a_i = ai.data() + (size_t)nx * (v + (size_t)nv * k);
        for (int x = 0; x < nx; ++x) {
          a_r[x] += cr[x] * qr - ci[x] * qi;
          a_i[x] += ci[x] * qr + cr[x] * qi;
        }
      }
}

// out(c, v, k) += pref * sum_x conj(con(x, c, k)) M(x, v, k): the closing
// DGEMM group of both terms (OCEAN_bubble.f90:742-757, OCEAN_ladder.f90:900-911).
static void val_project(const or_val_dims* d, const or_val_ops* o, double pref, const std::vector<double>& mr,
                        const std::vector<double>& mi, double* outr, double* outi) {
  const int nc = d->nc, nv = d->nv, nk = nk_of(d), nx = nx_of(d);
  for (int k = 0; k < nk; ++k)
    for (int v = 0; v < nv; ++v)
      for (int c = 0; c < nc; ++c) {
        const double* cr = o->conr + (size_t)nx * (c + (size_t)nc * k);
        const double* ci = o->coni + (size_t)nx * (c + (size_t)nc * k);
        const double* m_r = mr.data() + (size_t)nx * (v + (size_t)nv * k);
        const double* m_i = mi.data() + (size_t)nx * (v + (size_t)nv * k);
        double sr = 0.0, si = 0.0;
        for (int x = 0; x < nx; ++x) {
          sr += cr[x] * m_r[x] + ci[x] * m_i[x];
          si += cr[x] * m_i[x] - ci[x] * m_r[x];
        }
        const size_t ip = c + (size_t)nc * (v + (size_t)nv * k);
        outr[ip] += pref * sr;
        outi[ip] += pref * si;
      }
}

// AI_bubble_act, OCEAN_bubble.f90:420-796 (nbw = 1), in two halves:
// l(x) += sum_{v,k} conj(val) A for one same-spin block (:509-580), and, after
// s = FFT_fwd[ bubble o FFT_bwd[l] ] (neither normalised, :663-665),
// out += pref sum_x conj(con) s val for one same-spin block (:687-760);
// pref = spin_prefac, 2 for valence_ham_spin = 1 and 1 for 2 (:465-470).
static void bubble_l(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi,
                     std::vector<double>& lr, std::vector<double>& li) {
  const int nv = d->nv, nk = nk_of(d), nx = nx_of(d);
  std::vector<double> ar, ai;
  val_amat(d, o, pr, pi, ar, ai);
  for (int k = 0; k < nk; ++k)
    for (int v = 0; v < nv; ++v) {
      const size_t b = (size_t)nx * (v + (size_t)nv * k);
      for (int x = 0; x < nx; ++x) {
        const double vr = o->valr[b + x], vi = o->vali[b + x];
        lr[x] += vr * ar[b + x] + vi * ai[b + x];
        li[x] += vr * ai[b + x] - vi * ar[b + x];
      }
    }
}

static void bubble_s(const or_val_dims* d, const or_val_ops* o, std::vector<double>& lr, std::vector<double>& li) {
  const int nx = nx_of(d);
  or_fft3d(d->xmesh, lr.data(), li.data(), +1);
  for (int x = 0; x < nx; ++x) {
    lr[x] *= o->bubble[x];
    li[x] *= o->bubble[x];
  }
  or_fft3d(d->xmesh, lr.data(), li.data(), -1);
}

static void bubble_project(const or_val_dims* d, const or_val_ops* o, double pref, const std::vector<double>& lr,
                           const std::vector<double>& li, double* outr, double* outi) {
  const int nv = d->nv, nk = nk_of(d), nx = nx_of(d);
  std::vector<double> mr((size_t)nx * nv * nk), mi((size_t)nx * nv * nk);
  for (int k = 0; k < nk; ++k)
    for (int v = 0; v < nv; ++v) {
      const size_t b = (size_t)nx * (v + (size_t)nv * k);
      for (int x = 0; x < nx; ++x) {
        const double vr = o->valr[b + x], vi = o->vali[b + x];
        mr[b + x] = lr[x] * vr - li[x] * vi;
        mi[b + x] = li[x] * vr + lr[x] * vi;
      }
    }
  val_project(d, o, pref, mr, mi, outr, outi);
}

// One spin channel (valence_ham_spin = 1): spin_prefac 2.
void or_val_bubble_act(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, double* outr,
                       double* outi) {
  std::vector<double> lr(nx_of(d), 0.0), li(nx_of(d), 0.0);
  bubble_l(d, o, pr, pi, lr, li);
  bubble_s(d, o, lr, li);
  bubble_project(d, o, 2.0, lr, li, outr, outi);
}

// OCEAN_ladder_act_single, OCEAN_ladder.f90:155-1004 (one rank, nbw = 1):
// T(x, y, k) = sum_v A(x, v, k) conj(val(y, v, k));
// T(x, y, .) = FFT_bwd[ ladder(., x, y) o FFT_fwd[ T(x, y, .) ] ] / Nk;
// B(x, v, k) = sum_y T(x, y, k) val(y, v, k);  out += -1 sum_x conj(con) B.
// The part of the direct term from y in [y0, y1); lad holds ladder(., ., y) for
// those y only (lad[nk (x + nx (y - y0)) + k]).  Summing the parts over a
// partition of the y-range gives or_val_ladder_act up to the order of the sums.
void or_val_ladder_slab(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, int y0, int y1,
                        const double* lad_slab, double* outr, double* outi);

void or_val_ladder_act(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, double* outr,
                       double* outi) {
  or_val_ladder_slab(d, o, pr, pi, 0, nx_of(d), o->ladder, outr, outi);
}

void or_val_ladder_slab(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, int y0, int y1,
                        const double* lad_slab, double* outr, double* outi) {
  const int nv = d->nv, nk = nk_of(d), nx = nx_of(d);
  std::vector<double> ar, ai;
  val_amat(d, o, pr, pi, ar, ai);
  std::vector<double> br((size_t)nx * nv * nk, 0.0), bi((size_t)nx * nv * nk, 0.0);
  const double inv_nk = 1.0 / (double)nk;
  // x-points split over threads (each thread owns B(x, ., .) of its x and adds
  // the y in order, so the sums do not depend on the thread count)
#pragma omp parallel for schedule(dynamic, 1)
  for (int x = 0; x < nx; ++x) {
    std::vector<double> tr(nk), ti(nk);
    for (int y = y0; y < y1; ++y) {
      for (int k = 0; k < nk; ++k) {
        double sr = 0.0, si = 0.0;
        for (int v = 0; v < nv; ++v) {
          const size_t b = (size_t)nx * (v + (size_t)nv * k);
          const double a_r = ar[b + x], a_i = ai[b + x];
          const double vr = o->valr[b + y], vi = o->vali[b + y];
          sr += a_r * vr + a_i * vi;
          si += a_i * vr - a_r * vi;
        }
        tr[k] = sr;
        ti[k] = si;
      }
      or_fft3d(d->kmesh, tr.data(), ti.data(), -1);
      const double* lad = lad_slab + (size_t)nk * (x + (size_t)nx * (y - y0));
      for (int k = 0; k < nk; ++k) {
        tr[k] *= lad[k];
        ti[k] *= lad[k];
      }
      or_fft3d(d->kmesh, tr.data(), ti.data(), +1);
      for (int k = 0; k < nk; ++k) {
        const double t_r = tr[k] * inv_nk, t_i = ti[k] * inv_nk;
        for (int v = 0; v < nv; ++v) {
          const size_t b = (size_t)nx * (v + (size_t)nv * k);
          const double vr = o->valr[b + y], vi = o->vali[b + y];
          br[b + x] += t_r * vr - t_i * vi;
          bi[b + x] += t_i * vr + t_r * vi;
        }
      }
    }
  }
  val_project(d, o, -1.0, br, bi, outr, outi);
}

// cacorr (OCEAN_fxc.f90:333-470) for the unpolarised, non-relativistic gas it
// is called with (xn1 = xn2 = n/2, rel = 0): Slater exchange per particle and
// the Ceperley-Alder correlation in the Perdew-Zunger parametrisation (Phys.
// Rev. B 23, 5048); zeta = 0 selects the unpolarised fit.
static void lda_ex_ec(double n, double* ex, double* ec) {
  const double pi = kPiV;
  if (n < 0.00000001) {
    *ex = 0.0;
    *ec = 0.0;
    return;
  }
  const double third = 1.0 / 3.0;
  const double rs = std::pow(3.0 / (4.0 * pi * n), third);
  const double half = n / 2.0;
  const double ex1 = -1.5 * std::pow(0.75 / pi, third) * std::pow(half, third);
  *ex = (half * ex1 + half * ex1) / n;
  if (rs >= 1.0) {
    const double rr = std::sqrt(rs);
    *ec = -0.1423 / (1.0 + 1.0529 * rr + 0.3334 * rs);
  } else {
    const double lr = std::log(rs);
    *ec = 0.0311 * lr + (-0.048) + 0.002 * (rs * lr) + (-0.0116) * rs;
  }
}

// OCEAN_fxc_prep (OCEAN_fxc.f90:35-123): f_xc(x) = d^2[n (ex + ec)]/dn^2 by the
// five-point rule with step dn = n/100, times Nx / (Nk V); rho in the x-mesh
// order (x3 fastest, the rho(iz, iy, ix) loop).
void or_val_fxc_from_rho(int nx, const double* rho, double celvol, int nkpts, double* fxc) {
  for (int i = 0; i < nx; ++i) {
    const double n = rho[i], dn = 0.01 * n;
    const double ns[5] = {n + 2 * dn, n + dn, n, n - dn, n - 2 * dn};
    double v[5];
    for (int j = 0; j < 5; ++j) {
      double ex, ec;
      lda_ex_ec(ns[j], &ex, &ec);
      v[j] = ns[j] * (ex + ec);
    }
    fxc[i] = (16.0 * (v[3] + v[1]) - (v[4] + v[0]) - 30.0 * v[2]) / (12.0 * dn * dn) * (double)nx /
             ((double)nkpts * celvol);
  }
}

// The operator data seen by one (valence spin, conduction spin) pair: con of
// the conduction spin, val of the valence spin (DFT spin index = min(spin,
// nspn), OCEAN_ladder.f90:118-133, OCEAN_bubble.f90:511-512).
static or_val_ops spin_view(const or_val_dims* d, const or_val_ops* o, int cs, int vs) {
  const size_t nxk = (size_t)nx_of(d) * nk_of(d);
  or_val_ops v = *o;
  v.conr = o->conr + (size_t)cs * nxk * d->nc;
  v.coni = o->coni + (size_t)cs * nxk * d->nc;
  v.valr = o->valr + (size_t)vs * nxk * d->nv;
  v.vali = o->vali + (size_t)vs * nxk * d->nv;
  return v;
}

static int vspin_of(const or_val_dims* d) { return d->vspin > 1 ? 2 : 1; }
static int nspn_of(const or_val_dims* d) { return d->nspn > 1 ? 2 : 1; }

// OCEAN_xact valence branch (OCEAN_action.f90:521-575) followed by
// OCEAN_energies_act (:590-600, OCEAN_energies.f90:890-906).  psi holds
// valence_ham_spin^2 blocks (Nc, Nv, Nk) in the order ibeta = (i - 1) vs + j
// of OCEAN_ladder_act (i the valence spin, j the conduction spin).  The
// exchange sums the same-spin blocks (ispn, ispn) into one l and feeds it back
// to each of them; the direct term acts on every block.
int or_val_act(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, double* hr,
               double* hi, int backwards) {
  const int vs = vspin_of(d), ns = nspn_of(d);
  const size_t nb1 = (size_t)d->nc * d->nv * nk_of(d), n = nb1 * vs * vs;
  std::vector<double> qr(n), qi(n), kr(n, 0.0), ki(n, 0.0);
  for (size_t i = 0; i < n; ++i) {
    qr[i] = pr[i] * o->allow[i];
    qi[i] = pi[i] * o->allow[i];
  }
  if (o->bflag) {
    std::vector<double> lr(nx_of(d), 0.0), li(nx_of(d), 0.0);
    for (int is = 0; is < vs; ++is) {
      const int ds = std::min(is, ns - 1);
      const or_val_ops v = spin_view(d, o, ds, ds);
      const size_t off = nb1 * (size_t)(is * vs + is);
      bubble_l(d, &v, qr.data() + off, qi.data() + off, lr, li);
    }
    bubble_s(d, o, lr, li);
    const double pref = vs == 1 ? 2.0 : 1.0;
    for (int js = 0; js < vs; ++js) {
      const int ds = std::min(js, ns - 1);
      const or_val_ops v = spin_view(d, o, ds, ds);
      const size_t off = nb1 * (size_t)(js * vs + js);
      bubble_project(d, &v, pref, lr, li, kr.data() + off, ki.data() + off);
    }
  }
  if (o->fxc && vs == 1) {  // OCEAN_fxc_act (OCEAN_fxc.f90:127-322): phi = fxc l, spin_prefac 2
    std::vector<double> lr(nx_of(d), 0.0), li(nx_of(d), 0.0);
    const or_val_ops v = spin_view(d, o, 0, 0);
    bubble_l(d, &v, qr.data(), qi.data(), lr, li);
    for (int x = 0; x < nx_of(d); ++x) {
      lr[x] *= o->fxc[x];
      li[x] *= o->fxc[x];
    }
    bubble_project(d, &v, 2.0, lr, li, kr.data(), ki.data());
  }
  if (o->lflag)
    for (int iv = 0; iv < vs; ++iv)
      for (int jc = 0; jc < vs; ++jc) {
        const or_val_ops v = spin_view(d, o, std::min(jc, ns - 1), std::min(iv, ns - 1));
        const size_t off = nb1 * (size_t)(iv * vs + jc);
        or_val_ladder_act(d, &v, qr.data() + off, qi.data() + off, kr.data() + off, ki.data() + off);
      }
  for (size_t i = 0; i < n; ++i) {
    double er = 0.0, ei = 0.0;
    if (o->bande) {
      const double a = o->er[i], b = o->ei ? o->ei[i] : 0.0;
      if (backwards) {
        er = a * pr[i] + b * pi[i];
        ei = a * pi[i] - b * pr[i];
      } else {
        er = a * pr[i] - b * pi[i];
        ei = a * pi[i] + b * pr[i];
      }
    }
    hr[i] = er + o->allow[i] * kr[i];
    hi[i] = ei + o->allow[i] * ki[i];
  }
  return 0;
}

// OCEAN_gmres_do_recycle over the valence action (the have_val branches of
// OCEAN_gmres.f90:544-548, 603-606): rhs = allow o hay, the preconditioner from
// H (allow o 1), and the output scaled by fact = kpref 2 celvol.
int or_val_gmres(const or_val_dims* d, const or_val_ops* o, const double* hay_r, const double* hay_i, double kpref,
                 double celvol, const double* elist, int nomega, int depth, double gres, double gprc, double ffff,
                 int max_restarts, double* out_re, double* out_im, double* rel_err, int* iters, int* total_hpsi) {
  const size_t n = (size_t)d->nc * d->nv * nk_of(d) * vspin_of(d) * vspin_of(d);
  struct U {
    const or_val_dims* d;
    const or_val_ops* o;
  } u{d, o};
  auto act = [](void* user, const double* pr, const double* pi, double* hr, double* hi) {
    const U* q = static_cast<const U*>(user);
    or_val_act(q->d, q->o, pr, pi, hr, hi, 0);
  };
  return or_gmres_with(n, o->allow, 1, act, &u, hay_r, hay_i, kpref * 2.0 * celvol, elist, nomega, depth, gres,
                       gprc, ffff, max_restarts, out_re, out_im, rel_err, iters, total_hpsi);
}

// The Hermitian Haydock recursion of OCEAN_haydock_Herm_do with
// ocean_hay_ab_twoterm (OCEAN_haydock.f90:190-320, 824-938) over the valence
// action, in the same arithmetic order as or_haydock.
int or_val_haydock(const or_val_dims* d, const or_val_ops* o, const double* p0r, const double* p0i, int niter,
                   double* real_a, double* imag_a, double* real_b, int* niter_done) {
  const size_t n = (size_t)d->nc * d->nv * nk_of(d) * vspin_of(d) * vspin_of(d);
  std::vector<double> psr(p0r, p0r + n), psi_(p0i, p0i + n);
  std::vector<double> olr(n, 0.0), oli(n, 0.0), hr(n), hi(n);
  for (int i = 0; i <= niter; ++i) real_a[i] = imag_a[i] = real_b[i] = 0.0;
  int done = 0;
  for (int iter = 1; iter <= niter; ++iter) {
    or_val_act(d, o, psr.data(), psi_.data(), hr.data(), hi.data(), 0);
    const double bm = -real_b[iter - 1];
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
    const double inv = 1.0 / real_b[iter];
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

}  // extern "C"
