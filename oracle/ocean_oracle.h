/*
 * ocean_oracle.h -- CPU ORACLE for the OCEAN core-level BSE hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain FP64 C++ restatement of the
 * reference's Fortran (the OCEAN2 Fortran sources) used as the checker for libocean_gpu.so and
 * as the timed CPU baseline.  The product library never links, loads or calls it.
 *
 * Parity pins: the continued-fraction writer and the tridiagonal eigenvalue
 * routine are pinned against the reference's own golden files
 * (EXAMPLE/Cu_TwoPhoton/Results/abslanc_* / absspct_*).  The H*psi action, the
 * Lanczos recurrence and the GMRES driver are restatements of the cited source
 * with no reference output to pin them (the reference ships none of u2.dat,
 * rpottrim, cks or the Slater files): their parity is pinned by structure
 * (Hermiticity, dense-H eigenvalues vs Lanczos Ritz values, FFT vs numpy) only.
 *
 * Array layouts are the reference's Fortran (column-major) layouts; see
 * include/ocean_gpu.h.
 */
#ifndef OCEAN_ORACLE_H
#define OCEAN_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nb;
  int kmesh[3];
  int xmesh[3];
  int na;
  int nspn;
  int core_l;
} or_dims;

typedef struct {
  const double* er;      /* energies (nb,nk,na) real          */
  const double* ei;      /* energies imaginary, may be NULL    */
  const double* allow;   /* (nb,nk,na)                         */
  const double* ur;      /* phased Bloch functions (nb,nk,nx,nspn) */
  const double* ui;
  const double* W;       /* (nk,nx)                            */
  const double* somelr;  /* (na,na) or NULL                    */
  const double* someli;
  int lmin, lmax, npmax;
  const int* nproj;      /* (lmax-lmin+1)                      */
  const double* mpcr;    /* (nb,nk,npmax,2lmax+1,lmax-lmin+1,nspn) */
  const double* mpci;
  const double* mpm;     /* (npmax,npmax,lmax-lmin+1)          */
  const double* mhr;     /* sum mham^2                         */
  const double* mhi;
  double celvol;
  double interaction_scale;
  int e0, long_range, mult;
  int nhflag[6];
  int nthreads;          /* OpenMP threads for the action (0 = default) */
} or_ops;

typedef struct {
  double avec[9];
  double tau[3];
  double epsilon0;
  double interaction_scale;
  int nptab;
  const double* rtab;
  const double* ptab;
  int isolated;
  double iso_cut;
  int pbc[3];
  int have_eps3d;
  double epsilon3d[3];
  int xshift_override[3];
} or_lr_in;

/* OCEAN_bloch_lrLOAD (OCEAN_bloch.f90:54-219). tau is updated in place. */
int or_lrload(const or_dims* d, double tau[3], const int xshift_override[3], int xshift[3],
              double* ur, double* ui);
/* lr_populate_W2 (long_range.f90:1659-1853). */
int or_populate_w2(const or_dims* d, const or_lr_in* p, const double tau[3], const int xshift[3],
                   double* W);
/* intval with 'cap','cap' (CNBSE/zcmsnmult/zf90/intval.f90:8-60). */
double or_intval(int n, const double* xtab, const double* ytab, double x);
/* 3-D DFT over the k-mesh in the FFTW convention used by FFT_wrapper
 * (Modules/FFT_wrapper.f90:46-87,185-228): sign +1 backward, -1 forward,
 * unnormalised.  Flat index k3 fastest, k1 slowest. */
void or_fft3d(const int kmesh[3], double* re, double* im, int sign);
/* OCEAN_xact core branch (OCEAN_action.f90:286-618). */
int or_xact(const or_dims* d, const or_ops* o, const double* pr, const double* pi,
            double* hr, double* hi, const int* hflag, int backwards);
/* OCEAN_haydock_Herm_do + ocean_hay_ab_twoterm (OCEAN_haydock.f90:190-320,824-938). */
int or_haydock(const or_dims* d, const or_ops* o, const double* p0r, const double* p0i, int niter,
               double* real_a, double* imag_a, double* real_b, int* niter_done);
/* OCEAN_haydock_nonHerm_do + haydock_abc_1 (OCEAN_haydock.f90:53-164,1250-1433):
 * two-sided Lanczos with H on the right vectors and H^dagger (xact backwards) on
 * the left ones; complex a (0:niter), b and c (1:niter). */
int or_haydock_nonherm(const or_dims* d, const or_ops* o, const double* p0r, const double* p0i, int niter,
                       double* real_a, double* imag_a, double* real_b, double* imag_b, double* real_c,
                       double* imag_c, int* niter_done);
/* core_pnorm (OCEAN_psi.f90:5589-5638). */
double or_pnorm(int n, int nkpts, double celvol, double* pr, double* pi);
/* write_core / write_core_Voigt (OCEAN_haydock.f90:1801-1989). out (ne+1)*9. */
int or_write_core(const double* real_a, const double* imag_a, const double* real_b, int iter,
                  double kpref, double el, double eh, int ne, double gam0, double ebase,
                  double gam_gauss, double ucvol, int old_broaden, double nval, double eps,
                  double* out);
/* write_core with complex b and c (OCEAN_haydock.f90:1846-1870, the products
 * cmplx(real_b, imag_b) * cmplx(real_c, imag_c) of the non-Hermitian run). */
int or_write_core_bc(const double* real_a, const double* imag_a, const double* real_b, const double* imag_b,
                     const double* real_c, const double* imag_c, int iter, double kpref, double el, double eh,
                     int ne, double gam0, double ebase, double ucvol, double* out);
/* write_val (OCEAN_haydock.f90:1706-1799). out ne*8. */
int or_write_val(const double* real_a, const double* imag_a, const double* real_b, const double* imag_b,
                 const double* real_c, const double* imag_c, int iter, double kpref, double ucvol, int val_ham_spin,
                 int semi_tda, int backf, double el, double eh, int ne, double gam0, double* out);
/* calc_spect_core (OCEAN_haydock.f90:1991-2027). out ne*3. */
int or_calc_spect_core(const double* real_a, const double* imag_a, const double* real_b, int iter,
                       double kpref, double el, double eh, int ne, double gam0, double ebase,
                       double* out);
/* check_convergence (OCEAN_haydock.f90:1608-1661), core branch. */
int or_check_convergence(const double* real_a, const double* imag_a, const double* real_b, int iter1, int iter2,
                         double kpref, double el, double eh, int ne, double gam0, double* max_diff,
                         double* rel_area);
/* The early-exit rule of OCEAN_haydock_Herm_do (OCEAN_haydock.f90:268-292) on
 * per-iteration relArea values rel[0..niter]. */
int or_early_exit_iter(const double* rel, int niter, int spacing, double threshold);
/* Hermitian Haydock with the haydockconv.ipt early exit. */
int or_haydock_conv(const or_dims* d, const or_ops* o, const double* p0r, const double* p0i, int niter,
                    double threshold, int spacing, double kpref, double el, double eh, int ne, double gam0,
                    double* real_a, double* imag_a, double* real_b, double* rel_out, int* niter_done);
/* nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181) with threey by npt-point
 * Gauss-Legendre quadrature; mhr/mhi(mham, mham), Hartree. */
int or_nbsemhsetup2(int lc, int lv, int np, int kfl, int kfh, const double* fk, const double* scfk, int kgl,
                    int kgh, const double* gk, const double* scgk, double scfac, int npt, double* mhr,
                    double* mhi);
double or_threey(int ll, int ml, int lm, int mm, int lr, int mr, int conjug, int npt);
/* gamfcn (CNBSE/zcmsnmult/zf90/gamfcn.f90:8-42). */
double or_gamfcn(double e, double n, double e0);
/* redtrid eigenvalues (OCEAN_haydock.f90:2273-2316). */
int or_redtrid(int n, const double* real_a, const double* real_b, double* w);
/* zhptrf / zhptrs, uplo = 'U' (LAPACK), as called by update_gmres
 * (OCEAN_gmres.f90:309,320).  ap: packed upper, interleaved complex (2*n(n+1)/2). */
int or_zhptrf_u(int n, double* ap, int* ipiv);
int or_zhptrs_u(int n, const double* ap, const int* ipiv, double* b);
/* OCEAN_gmres_do_recycle (OCEAN_gmres.f90:508-908). */
int or_gmres(const or_dims* d, const or_ops* o, const double* hay_r, const double* hay_i,
             double kpref, const double* energies_ev, int nomega, int depth, double gres,
             double gprc, double ffff, int max_restarts, double* out_re, double* out_im,
             double* rel_err, int* iters, int* total_hpsi);
/* OCEAN_soprep without core_broaden.ipt (OCEAN_multiplet.f90:572-690). */
int or_soprep(int core_l, double xi, double* somelr, double* someli);

/* ---- valence BSE (ocean_oracle_val.cpp): one spin channel, resonant pairs */
typedef struct {
  int nc, nv;    /* conduction / valence bands */
  int kmesh[3];  /* flat k index k3 fastest */
  int xmesh[3];  /* flat x index x3 fastest */
  int nspn;      /* DFT spins of con/val (0 or 1: one) */
  int vspin;     /* valence_ham_spin (0 or 1: one; 2: psi has 4 spin blocks) */
} or_val_dims;

typedef struct {
  const double *er, *ei;      /* (Nc, Nv, Nk) pair energies; ei may be NULL */
  const double* allow;        /* (Nc, Nv, Nk) */
  const double *conr, *coni;  /* (Nx, Nc, Nk) conduction states on the x-mesh */
  const double *valr, *vali;  /* (Nx, Nv, Nk) valence states on the x-mesh */
  const double* bubble;       /* (Nx) */
  const double* ladder;       /* (Nk, Nx, Nx) */
  int bande, bflag, lflag;    /* energies, exchange, screened direct */
  const double* fxc;          /* (Nx) ALDA kernel, NULL = off (aldaf) */
} or_val_ops;

/* OCEAN_fxc_prep (OCEAN_fxc.f90:35-123) with cacorr (:333-470). */
void or_val_fxc_from_rho(int nx, const double* rho, double celvol, int nkpts, double* fxc);

/* wall_search_old_way (OCEAN_bubble.f90:238-297). */
double or_val_wall_length(const int xmesh[3], const double bvec[9]);
/* AI_bubble_populate (OCEAN_bubble.f90:300-407). */
int or_val_bubble_populate(const int xmesh[3], const double bvec[9], const double qinb[3], double celvol,
                           int nkpts, double length, double* bubble);
/* AI_bubble_act / OCEAN_ladder_act_single, accumulating into out. */
void or_val_bubble_act(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi,
                       double* outr, double* outi);
void or_val_ladder_act(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi,
                       double* outr, double* outi);
/* The direct term's part from y in [y0, y1), lad_slab = ladder(., ., y0..y1-1). */
void or_val_ladder_slab(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, int y0,
                        int y1, const double* lad_slab, double* outr, double* outi);
/* OCEAN_xact valence branch + energies (OCEAN_action.f90:521-600). */
int or_val_act(const or_val_dims* d, const or_val_ops* o, const double* pr, const double* pi, double* hr,
               double* hi, int backwards);
/* GMRES (OCEAN_gmres_do_recycle) over a caller-supplied action on n complex values. */
int or_gmres_with(size_t n, const double* allow, int mask_ones,
                  void (*act)(void* user, const double* pr, const double* pi, double* hr, double* hi), void* user,
                  const double* hay_r, const double* hay_i, double fact, const double* elist, int nomega, int depth,
                  double gres, double gprc, double ffff, int max_restarts, double* out_re, double* out_im,
                  double* rel_err, int* iters, int* total_hpsi);
/* GMRES over the valence action (OCEAN_gmres.f90:508-908, have_val branches). */
int or_val_gmres(const or_val_dims* d, const or_val_ops* o, const double* hay_r, const double* hay_i, double kpref,
                 double celvol, const double* elist, int nomega, int depth, double gres, double gprc, double ffff,
                 int max_restarts, double* out_re, double* out_im, double* rel_err, int* iters, int* total_hpsi);
/* Hermitian Haydock over the valence action (OCEAN_haydock.f90:190-320, 824-938). */
int or_val_haydock(const or_val_dims* d, const or_val_ops* o, const double* p0r, const double* p0i, int niter,
                   double* real_a, double* imag_a, double* real_b, int* niter_done);

#ifdef __cplusplus
}
#endif
#endif
