// ocn_cf.cu -- Haydock continued fraction on the GPU (write_core,
// OCEAN_haydock.f90:1801-1894, and write_core_Voigt, :1896-1989).
//
// One thread per energy point, FP64.  The reference builds two of the complex
// numbers in its recurrence with cmplx(x, y) without a KIND, which Fortran
// evaluates in default (single) precision: b_j*c_j and (e - a_j) + i(gam + ia_j)
// are rounded to binary32 before entering the FP64 recurrence (:1837, :1868-1869).
// The golden spectra in EXAMPLE/Cu_TwoPhoton/Results carry that rounding, so it is
// restated here.  This file is compiled with -fmad=false so that every product
// and sum rounds exactly as written.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <string>
#include <vector>

#include "ocn_internal.h"

namespace ocn {

namespace {

// OCEAN2/OCEAN_constants.f90:15-30
constexpr double kEV2Ha = 0.036749322175666;
constexpr double kHa2eV = 27.211386245980;
constexpr double kAlpha = 0.0072973525643;
constexpr double kBohr = 0.529177210544;
constexpr double kAu2sec = 2.4188843265864e-17;
constexpr double kPi = 3.1415926535897932384626433832795028841971693993751;

struct cplx {
  double x, y;
};

__device__ __forceinline__ cplx cdiv_smith(cplx n, cplx d) {
  if (fabs(d.x) >= fabs(d.y)) {
    const double r = d.y / d.x;
    const double t = 1.0 / (d.x + d.y * r);
    return {(n.x + n.y * r) * t, (n.y - n.x * r) * t};
  }
  const double r = d.x / d.y;
  const double t = 1.0 / (d.x * r + d.y);
  return {(n.x * r + n.y) * t, (n.y * r - n.x) * t};
}

__device__ __forceinline__ cplx csqrt_principal(cplx z) {
  if (z.x == 0.0 && z.y == 0.0) return {0.0, z.y};
  const double t = sqrt((fabs(z.x) + sqrt(z.x * z.x + z.y * z.y)) * 0.5);
  if (z.x >= 0.0) return {t, z.y / (2.0 * t)};
  return {fabs(z.y) / (2.0 * t), copysign(t, z.y)};
}

// b_j c_j with c = b real (Hermitian Lanczos), as a binary32 product.
__device__ __forceinline__ double bsq_sp(double b) {
  const float f = __double2float_rn(b);
  return (double)__fmul_rn(f, f);
}

// Imaginary parts of b and the c coefficients of a non-Hermitian run (all NULL:
// the Hermitian run, c = b real).
struct BcArrays {
  const double *ib, *rc, *ic;
};

// b_j c_j as write_core forms it: cmplx(real_b, imag_b) * cmplx(real_c, imag_c)
// without a KIND, a binary32 complex product (OCEAN_haydock.f90:1847-1848,1868).
__device__ __forceinline__ cplx bc_sp(const double* __restrict__ rb, const BcArrays& q, int j) {
  if (!q.ib && !q.rc && !q.ic) return {bsq_sp(rb[j]), 0.0};
  const float a = __double2float_rn(rb[j]), b = q.ib ? __double2float_rn(q.ib[j]) : 0.0f;
  const float c = q.rc ? __double2float_rn(q.rc[j]) : a, d = q.ic ? __double2float_rn(q.ic[j]) : 0.0f;
  return {(double)__fsub_rn(__fmul_rn(a, c), __fmul_rn(b, d)), (double)__fadd_rn(__fmul_rn(a, d), __fmul_rn(b, c))};
}

__device__ cplx cf_delta(const double* __restrict__ ra, const double* __restrict__ ia,
                         const double* __restrict__ rb, const BcArrays& q, int iter, double e, double gam) {
  const double ial = ia ? ia[iter - 1] : 0.0;
  const cplx ct = {e - ra[iter - 1], gam + ial};
  const cplx bcl = bc_sp(rb, q, iter);
  const double bc4 = (double)__fmul_rn(4.0f, __double2float_rn(bcl.x));
  const double bc4i = (double)__fmul_rn(4.0f, __double2float_rn(bcl.y));
  const cplx sq = {ct.x * ct.x - ct.y * ct.y - bc4, ct.x * ct.y + ct.y * ct.x - bc4i};
  const cplx disc = csqrt_principal(sq);
  cplx delta;
  if (disc.y > 0.0)
    delta = {(ct.x + disc.x) * 0.5, (ct.y + disc.y) * 0.5};
  else
    delta = {(ct.x - disc.x) * 0.5, (ct.y - disc.y) * 0.5};
  for (int jj = iter - 1; jj >= 0; --jj) {
    const cplx c2 = bc_sp(rb, q, jj + 1);
    const double iaj = ia ? ia[jj] : 0.0;
    const cplx z = {(double)__double2float_rn(e - ra[jj]), (double)__double2float_rn(gam + iaj)};
    const cplx q = cdiv_smith(c2, delta);
    delta = {z.x - q.x, z.y - q.y};
  }
  return delta;
}

__global__ void k_write_core(const double* __restrict__ ra, const double* __restrict__ ia,
                             const double* __restrict__ rb, const BcArrays q, int iter, double kpref, double el,
                             double eh, int ne, double gam0, const double* __restrict__ gam1,
                             double ebase, double ucvol, double* __restrict__ out) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row > ne) return;
  const int ie = 2 * row;
  const double e = el + (eh - el) * (double)ie / (double)(2 * ne);
  const cplx d = cf_delta(ra, ia, rb, q, iter, e, gam0);
  const double dr = d.x, di = fabs(d.y);
  const double spct = kpref * di / (dr * dr + di * di);
  const double spkk = kpref * dr / (dr * dr + di * di);
  double spct1 = spct, spkk1 = spkk;
  if (gam1) {  // oldXASbroaden: second damping with gamfcn (OCEAN_haydock.f90:1839-1841)
    const cplx d1 = cf_delta(ra, ia, rb, q, iter, e, gam1[row]);
    const double dr1 = d1.x, di1 = fabs(d1.y);
    spct1 = kpref * di1 / (dr1 * dr1 + di1 * di1);
    spkk1 = kpref * dr1 / (dr1 * dr1 + di1 * di1);
  }
  const double alphaByVolumeHartree = kEV2Ha * kAlpha * ucvol;
  const double tpa = (kAlpha * kAlpha * 2.0 * kPi) * ucvol;
  const double bohrSq2CmSq = kBohr * kBohr * 1.0e-16;
  const double tpacm4 = tpa * bohrSq2CmSq * bohrSq2CmSq * kAu2sec;
  const double ener = ebase + kHa2eV * e;
  const double sigma = alphaByVolumeHartree * ener * spct;
  double* r = out + 9 * (size_t)row;
  r[0] = ener;
  r[1] = spct1;
  r[2] = spct;
  r[3] = spkk1;
  r[4] = spkk;
  r[5] = sigma;
  r[6] = sigma * bohrSq2CmSq;
  r[7] = spct * tpa;
  r[8] = spct * tpacm4;
}

// check_convergence (OCEAN_haydock.f90:1608-1661) after the Lanczos step that
// brought the device counter to it = *itp: calc_spect_core's column 3
// (:1991-2027) at it and at it - spacing steps on the ne midpoints
// el + (eh - el)(2i+1)/(2 ne), one thread per (spectrum, point).
__global__ void k_conv_spect(const double* __restrict__ ra, const double* __restrict__ ia,
                             const double* __restrict__ rb, const int* __restrict__ itp, int spacing, double kpref,
                             double el, double eh, int ne, double gam0, double* __restrict__ sp) {
  const int it = *itp;
  if (it <= spacing) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * ne) return;
  const int which = i / ne, ie = i - which * ne;
  const double e = el + (eh - el) * (double)(2 * ie + 1) / (double)(2 * ne);
  const cplx d = cf_delta(ra, ia, rb, BcArrays{nullptr, nullptr, nullptr}, which ? it - spacing : it, e, gam0);
  const double dr = d.x, di = fabs(d.y);
  sp[i] = kpref * di / (dr * dr + di * di);
}
// relArea = 2 sum|sp1 - sp2| / (sum|sp1| + sum|sp2|) summed in energy order by
// one thread, as the reference does (:1640-1652); rel[it] (0 when it <= spacing).
__global__ void k_conv_rel(const double* __restrict__ sp, int ne, const int* __restrict__ itp, int spacing,
                           double* __restrict__ rel) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int it = *itp;
  if (it <= spacing) {
    rel[it] = 0.0;
    return;
  }
  double d = 0.0, a1 = 0.0, a2 = 0.0;
  for (int i = 0; i < ne; ++i) {
    d += fabs(sp[i] - sp[ne + i]);
    a1 += fabs(sp[i]);
    a2 += fabs(sp[ne + i]);
  }
  rel[it] = 2.0 * d / (a1 + a2);
}

// Voigt variant: Lorentzian spectrum on the fine grid e_i = el + (i - nstep)*estep
// (each fine point of write_core_Voigt evaluated once), with damping gam[i].
__global__ void k_cf_points(const double* __restrict__ ra, const double* __restrict__ ia,
                            const double* __restrict__ rb, const BcArrays q, int iter, double kpref, double el,
                            int nstep, double estep, const double* __restrict__ gam,
                            double prefactor, double* __restrict__ sp, double* __restrict__ sk,
                            int npts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npts) return;
  const double e = el + (double)(i - nstep) * estep;
  const cplx d = cf_delta(ra, ia, rb, q, iter, e, gam[i]);
  const double dr = d.x, di = fabs(d.y);
  sp[i] = prefactor * kpref * di / (dr * dr + di * di);
  sk[i] = prefactor * kpref * dr / (dr * dr + di * di);
}

// ---- write_val (OCEAN_haydock.f90:1706-1799): the valence dielectric function

constexpr double kAlphaInv = 137.035999177;

__host__ __device__ inline void csqrt_hd(double x, double y, double* rx, double* ry) {
  if (x == 0.0 && y == 0.0) {
    *rx = 0.0;
    *ry = y;
    return;
  }
  const double t = sqrt((fabs(x) + sqrt(x * x + y * y)) * 0.5);
  if (x >= 0.0) {
    *rx = t;
    *ry = y / (2.0 * t);
  } else {
    *rx = fabs(y) / (2.0 * t);
    *ry = copysign(t, y);
  }
}

// The optical constants write_val prints for one energy (Hartree) and eps
// (:1778-1795): omega (eV), eps1, eps2, Re(n) - 1, Im(n), mu (1/cm), R, epsinv,
// n = sqrt(eps) (principal), R = |(n-1)/(n+1)|^2, mu = 2 omega Im(n) / (bohr
// alphainv 1000), epsinv = Im(eps) / |eps|^2.
__host__ __device__ inline void val_optical(double ere, double er, double ei, double* o) {
  const double lossf = ei / (er * er + ei * ei);
  double nr, ni;
  csqrt_hd(er, ei, &nr, &ni);
  const double ar = nr - 1.0, br = nr + 1.0;
  const double reflct = (ar * ar + ni * ni) / (br * br + ni * ni);
  const double mu = 2.0 * ere * kHa2eV * ni / (kBohr * kAlphaInv * 1000.0);
  o[0] = ere * kHa2eV;
  o[1] = er;
  o[2] = ei;
  o[3] = nr - 1.0;
  o[4] = ni;
  o[5] = mu;
  o[6] = reflct;
  o[7] = lossf;
}

// b_j c_j as write_val forms it: cmplx(real_b, imag_b, DP) * cmplx(real_c, -imag_c, DP),
// FP64 (c = b real in the Hermitian run).
__device__ __forceinline__ cplx bc_val(const double* __restrict__ rb, const BcArrays& q, int j) {
  const double a = rb[j], b = q.ib ? q.ib[j] : 0.0;
  const double c = q.rc ? q.rc[j] : a, d = q.ic ? -q.ic[j] : 0.0;
  return {a * c - b * d, a * d + b * c};
}

// One output row per thread: energies at the midpoints el + (eh - el)(2r+1)/(2 ne),
// the square-root terminator at the real energy, the resonant (al) and
// anti-resonant (be) fractions, eps = 1 - fact/al (- fact/be with semiTDA).
__global__ void k_write_val(const double* __restrict__ ra, const double* __restrict__ ia,
                            const double* __restrict__ rb, const BcArrays q, int iter, double fact, double el,
                            double eh, int ne, double gam0, int semi_tda, int backf, double* __restrict__ out) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= ne) return;
  const int ie = 2 * row + 1;
  double ere = el + (eh - el) * (double)ie / (double)(2 * ne);
  cplx ct = {ere, gam0};
  if (backf) {
    ct = {ct.x * ct.x - ct.y * ct.y, ct.x * ct.y + ct.y * ct.x};
    ere = ere * ere;
  }
  const double an = ra[iter - 1];
  double sx, sy;
  csqrt_hd((ere - an) * (ere - an) - 4.0 * rb[iter] * rb[iter], 0.0, &sx, &sy);
  const cplx rp = {0.5 * (ere - an + sx), 0.5 * sy};
  const cplx rm = {0.5 * (ere - an - sx), 0.5 * (-sy)};
  const cplx rrr = rp.y < 0.0 ? rp : rm;
  cplx al = {ct.x - an - rrr.x, ct.y - rrr.y};
  cplx be = {-ct.x - an - rrr.x, -ct.y - rrr.y};
  for (int i = iter - 1; i >= 0; --i) {
    const double ai = ia ? ia[i] : 0.0;
    const cplx bc = bc_val(rb, q, i + 1);
    const cplx qa = cdiv_smith(bc, al), qb = cdiv_smith(bc, be);
    al = {ct.x - ra[i] - qa.x, ct.y - ai - qa.y};
    be = {-ct.x - ra[i] - qb.x, -ct.y - ai - qb.y};
  }
  const cplx fa = cdiv_smith({fact, 0.0}, al);
  cplx eps = {1.0 - fa.x, -fa.y};
  if (semi_tda) {
    const cplx fb = cdiv_smith({fact, 0.0}, be);
    eps = {eps.x - fb.x, eps.y - fb.y};
  }
  if (backf) ere = sqrt(ere);
  val_optical(ere, eps.x, eps.y, out + 8 * (size_t)row);
}

}  // namespace

void val_optical_host(double ere, double er, double ei, double* o) { val_optical(ere, er, ei, o); }

int conv_check_launch(ocn_ctx* c, const double* ra, const double* ia, const double* rb, const int* itp) {
  const ocn_haydock_conv& p = c->conv;
  k_conv_spect<<<(2 * p.ne + 127) / 128, 128, 0, c->stream>>>(ra, ia, rb, itp, p.spacing, p.kpref, p.el, p.eh,
                                                               p.ne, p.gam0, c->d_conv_sp);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  k_conv_rel<<<1, 32, 0, c->stream>>>(c->d_conv_sp, p.ne, itp, p.spacing, c->d_conv_rel);
  ++c->launches;
  OCN_CUDA(c, cudaGetLastError());
  return OCN_OK;
}

int val_spectrum_eval(const double* ra, const double* ia, const double* rb, const double* ib, const double* rc,
                      const double* ic, int iter, const ocn_val_cf_params* p, double* out, std::string* err) {
  if (iter < 1 || p->ne < 1 || (p->val_ham_spin != 1 && p->val_ham_spin != 2)) {
    if (err) *err = "ocn_val_spectrum: iter and ne must be >= 1, val_ham_spin 1 or 2";
    return OCN_ERR_ARG;
  }
  const size_t nco = (size_t)iter + 1;
  std::vector<void*> owned;
  cudaError_t e = cudaSuccess;
  auto dup = [&](const double* h) -> double* {
    if (!h) return nullptr;
    void* q = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&q, nco * sizeof(double));
    if (e != cudaSuccess) return nullptr;
    owned.push_back(q);
    e = cudaMemcpy(q, h, nco * sizeof(double), cudaMemcpyHostToDevice);
    return static_cast<double*>(q);
  };
  double* d_ra = dup(ra);
  double* d_ia = dup(ia);
  double* d_rb = dup(rb);
  BcArrays dq{dup(ib), dup(rc), dup(ic)};
  double* d_out = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_out), (size_t)p->ne * 8 * sizeof(double));
  if (e == cudaSuccess) {
    owned.push_back(d_out);
    // fact = kpref * real(2 / val_ham_spin, DP) * ucvol (integer division, :1715)
    const double fact = p->kpref * (double)(2 / p->val_ham_spin) * p->ucvol;
    k_write_val<<<(p->ne + 63) / 64, 64>>>(d_ra, d_ia, d_rb, dq, iter, fact, p->el, p->eh, p->ne, p->gam0,
                                          p->semi_tda, p->backf, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d_out, (size_t)p->ne * 8 * sizeof(double), cudaMemcpyDeviceToHost);
  for (void* q : owned) cudaFree(q);
  if (e != cudaSuccess) {
    if (err) *err = std::string("ocn_val_spectrum: ") + cudaGetErrorString(e);
    return OCN_ERR_CUDA;
  }
  return OCN_OK;
}

int cf_eval(const double* ra, const double* ia, const double* rb, int iter, double kpref,
            const ocn_cf_params* p, double* out, std::string* err, const double* ib, const double* rc,
            const double* ic) {
  if (iter < 1 || p->ne < 1) {
    if (err) *err = "ocn_spectrum_cf: iter and ne must be >= 1";
    return OCN_ERR_ARG;
  }
  const size_t nco = (size_t)iter + 1;
  std::vector<void*> owned;
  cudaError_t e = cudaSuccess;
  auto cleanup = [&]() {
    for (void* q : owned) cudaFree(q);
    owned.clear();
  };
  auto dalloc = [&](size_t bytes) -> double* {
    void* q = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&q, bytes);
    if (e == cudaSuccess) owned.push_back(q);
    return static_cast<double*>(q);
  };
  auto h2d = [&](double* d, const double* h, size_t n) {
    if (e == cudaSuccess) e = cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice);
  };
  double* d_ra = dalloc(nco * sizeof(double));
  double* d_rb = dalloc(nco * sizeof(double));
  double* d_ia = ia ? dalloc(nco * sizeof(double)) : nullptr;
  h2d(d_ra, ra, nco);
  h2d(d_rb, rb, nco);
  if (ia) h2d(d_ia, ia, nco);
  BcArrays dq{nullptr, nullptr, nullptr};
  double* d_bc[3] = {nullptr, nullptr, nullptr};
  const double* h_bc[3] = {ib, rc, ic};
  for (int i = 0; i < 3; ++i)
    if (h_bc[i]) {
      d_bc[i] = dalloc(nco * sizeof(double));
      h2d(d_bc[i], h_bc[i], nco);
    }
  dq.ib = d_bc[0];
  dq.rc = d_bc[1];
  dq.ic = d_bc[2];
  const int ne = p->ne;
  if (e == cudaSuccess && p->gam_gauss > p->gam0 / 10.0) {
    // write_core_Voigt: fine grid shared between neighbouring output rows
    const double de = (p->eh - p->el) / (double)ne;
    double estep = fmin(p->gam0, p->gam_gauss) / 2.0;
    const int nratio = (int)((de - estep) / estep) + 1;
    estep = de / (double)nratio;
    const int nstep = (int)((2.99999 * p->gam_gauss) / estep) + 1;
    const double prefactor = estep / (p->gam_gauss * 2.506628274631);
    const double inv2s2 = 1.0 / (2.0 * p->gam_gauss * p->gam_gauss);
    const int npts = ne * nratio + 2 * nstep + 1;
    std::vector<double> g0(npts, p->gam0), g1(npts);
    for (int i = 0; i < npts; ++i)
      g1[i] = p->gam0 + gamfcn(p->el + (double)(i - nstep) * estep, p->nval, p->eps);
    double* d_g0 = dalloc(npts * sizeof(double));
    double* d_g1 = dalloc(npts * sizeof(double));
    double* d_sp = dalloc(2 * (size_t)npts * sizeof(double));
    double* d_sk = dalloc(2 * (size_t)npts * sizeof(double));
    h2d(d_g0, g0.data(), npts);
    h2d(d_g1, g1.data(), npts);
    if (e == cudaSuccess) {
      k_cf_points<<<(npts + 127) / 128, 128>>>(d_ra, d_ia, d_rb, dq, iter, kpref, p->el, nstep, estep,
                                              d_g0, prefactor, d_sp, d_sk, npts);
      k_cf_points<<<(npts + 127) / 128, 128>>>(d_ra, d_ia, d_rb, dq, iter, kpref, p->el, nstep, estep,
                                              d_g1, prefactor, d_sp + npts, d_sk + npts, npts);
      e = cudaGetLastError();
    }
    std::vector<double> sp(2 * (size_t)npts), sk(2 * (size_t)npts);
    if (e == cudaSuccess)
      e = cudaMemcpy(sp.data(), d_sp, sp.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      e = cudaMemcpy(sk.data(), d_sk, sk.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
      for (int row = 0; row <= ne; ++row) {
        double s0 = 0.0, s1 = 0.0, k0 = 0.0, k1 = 0.0;
        for (int ii = -nstep; ii <= nstep; ++ii) {
          const double pref = exp(-(double)(ii * ii) * estep * estep * inv2s2);
          const int idx = row * nratio + ii + nstep;
          s0 += pref * sp[idx];
          s1 += pref * sp[npts + idx];
          k0 += pref * sk[idx];
          k1 += pref * sk[npts + idx];
        }
        const double ee = p->el + (p->eh - p->el) * (double)(2 * row) / (double)(2 * ne);
        double* r = out + 9 * (size_t)row;
        r[0] = p->ebase + kHa2eV * (ee + (double)nstep * estep);
        r[1] = s1;
        r[2] = s0;
        r[3] = k1;
        r[4] = k0;
        r[5] = r[6] = r[7] = r[8] = 0.0;
      }
    }
  } else if (e == cudaSuccess) {
    double* d_g1 = nullptr;
    if (p->old_broaden) {
      std::vector<double> g1(ne + 1);
      for (int row = 0; row <= ne; ++row) {
        const double en = p->el + (p->eh - p->el) * (double)(2 * row) / (double)(2 * ne);
        g1[row] = p->gam0 + gamfcn(en, p->nval, p->eps);
      }
      d_g1 = dalloc((ne + 1) * sizeof(double));
      h2d(d_g1, g1.data(), ne + 1);
    }
    double* d_out = dalloc((size_t)(ne + 1) * 9 * sizeof(double));
    if (e == cudaSuccess) {
      k_write_core<<<(ne + 1 + 63) / 64, 64>>>(d_ra, d_ia, d_rb, dq, iter, kpref, p->el, p->eh, ne,
                                             p->gam0, d_g1, p->ebase, p->ucvol, d_out);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpy(out, d_out, (size_t)(ne + 1) * 9 * sizeof(double), cudaMemcpyDeviceToHost);
  }
  cleanup();
  if (e != cudaSuccess) {
    if (err) *err = std::string("ocn_spectrum_cf: ") + cudaGetErrorString(e);
    return OCN_ERR_CUDA;
  }
  return OCN_OK;
}

// ---- write_core without allocation (ocn_spectrum_cf_noalloc) ----------------
//
// Some callers cannot allocate device memory at the moment they want a spectrum:
// a run whose HBM is held by a caching allocator or by the Lanczos / Krylov
// buffers of a large problem (cudaMalloc then fails, or makes the pool hand
// memory back), and callers that must not stall the device, because cudaFree
// waits for all work on it, including other streams' Haydock chains.  For them
// this variant keeps every device buffer of k_write_core in one fixed array.
//
// Scratch layout, in doubles: real_a | imag_a | real_b (kNaCoef each) | damping
// column (kNaRows) | output rows (9 * kNaRows).  No part of it has to start at
// zero: each call uploads every coefficient and damping value that the kernel
// reads before it launches, and the kernel writes every output row that is
// copied back.  Calls that overlap on one device (two host threads of one
// process) share the array and race; a caller serialises them.  Each process
// and each device has its own copy.
namespace {

constexpr size_t kNaCoef = (size_t)OCN_CF_NOALLOC_MAX_ITER + 1;
constexpr size_t kNaRows = (size_t)OCN_CF_NOALLOC_MAX_NE + 1;
constexpr size_t kNaDoubles = 3 * kNaCoef + 10 * kNaRows;  // 94,221 doubles = 736 KiB

static __device__ __align__(256) double g_cf_scratch[kNaDoubles];

// Device address of g_cf_scratch per device, looked up once with that device
// current (the first call on a device does the set-up).  The cached address
// belongs to the device's primary context as it was at set-up; after
// cudaDeviceReset the module may load at another address, so the entry point
// is not to be used on a device after a reset (stated in the header).
constexpr int kNaMaxDevices = 64;
std::atomic<double*> g_cf_scratch_ptr[kNaMaxDevices] = {};

int noalloc_scratch(double** out, std::string* err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    if (err) *err = std::string("ocn_spectrum_cf_noalloc: cudaGetDevice: ") + cudaGetErrorString(e);
    return OCN_ERR_CUDA;
  }
  if (dev < 0 || dev >= kNaMaxDevices) {
    if (err) *err = "ocn_spectrum_cf_noalloc: device ordinal beyond the set-up table (64 devices)";
    return OCN_ERR_ARG;
  }
  double* p = g_cf_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    void* q = nullptr;
    e = cudaGetSymbolAddress(&q, g_cf_scratch);
    if (e != cudaSuccess || !q) {
      if (err)
        *err = std::string("ocn_spectrum_cf_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return OCN_ERR_CUDA;
    }
    p = static_cast<double*>(q);
    g_cf_scratch_ptr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return OCN_OK;
}

}  // namespace

int cf_eval_noalloc(const double* ra, const double* ia, const double* rb, int iter, double kpref,
                    const ocn_cf_params* p, double* out, std::string* err) {
  auto fail = [&](int code, const std::string& msg) {
    if (err) *err = "ocn_spectrum_cf_noalloc: " + msg;
    return code;
  };
  if (iter < 1 || p->ne < 1) return fail(OCN_ERR_ARG, "iter and ne must be >= 1");
  if (iter > OCN_CF_NOALLOC_MAX_ITER)
    return fail(OCN_ERR_ARG, "iter = " + std::to_string(iter) + " exceeds the static scratch limit of " +
                                 std::to_string(OCN_CF_NOALLOC_MAX_ITER) + "; use ocn_spectrum_cf");
  if (p->ne > OCN_CF_NOALLOC_MAX_NE)
    return fail(OCN_ERR_ARG, "ne = " + std::to_string(p->ne) + " exceeds the static scratch limit of " +
                                 std::to_string(OCN_CF_NOALLOC_MAX_NE) + "; use ocn_spectrum_cf");
  if (p->gam_gauss > p->gam0 / 10.0)
    return fail(OCN_ERR_ARG, "Voigt broadening (gam_gauss > gam0/10) is not available here; use ocn_spectrum_cf");
  double* s = nullptr;
  int rc = noalloc_scratch(&s, err);
  if (rc) return rc;
  double* d_ra = s;
  double* d_ia = s + kNaCoef;
  double* d_rb = s + 2 * kNaCoef;
  double* d_g1 = s + 3 * kNaCoef;
  double* d_out = d_g1 + kNaRows;
  const int ne = p->ne;
  const size_t nco = (size_t)iter + 1;
  cudaError_t e = cudaMemcpy(d_ra, ra, nco * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_rb, rb, nco * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ia) e = cudaMemcpy(d_ia, ia, nco * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && p->old_broaden) {
    // the damping column is staged in the caller's output array, overwritten below
    for (int row = 0; row <= ne; ++row) {
      const double en = p->el + (p->eh - p->el) * (double)(2 * row) / (double)(2 * ne);
      out[row] = p->gam0 + gamfcn(en, p->nval, p->eps);
    }
    e = cudaMemcpy(d_g1, out, (size_t)(ne + 1) * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {
    k_write_core<<<(ne + 1 + 63) / 64, 64>>>(d_ra, ia ? d_ia : nullptr, d_rb, BcArrays{nullptr, nullptr, nullptr},
                                             iter, kpref, p->el, p->eh, ne,
                                           p->gam0, p->old_broaden ? d_g1 : nullptr, p->ebase, p->ucvol,
                                           d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(out, d_out, (size_t)(ne + 1) * 9 * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(OCN_ERR_CUDA, cudaGetErrorString(e));
  return OCN_OK;
}

}  // namespace ocn
