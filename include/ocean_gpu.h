/*
 * ocean_gpu.h -- C ABI of libocean_gpu.so, the GB300 (sm_103a) implementation of
 * OCEAN's core-level BSE Hamiltonian action H*psi and the Haydock / GMRES solvers
 * that apply it.
 *
 * Conventions (mirroring the Fortran module procedures this library replaces):
 *   - Every entry point returns an int status; 0 = success.  Negative -1 is the
 *     reference's "NaN in the Lanczos a_n" code (OCEAN2/OCEAN_haydock.f90:913-920);
 *     positive codes are listed in ocn_status below.  Nothing aborts the process.
 *   - All arrays are borrowed for the duration of the call.  Arrays with a
 *     Fortran shape are passed in Fortran (column-major) order, exactly as the
 *     reference stores them, as separate real and imaginary FP64 planes:
 *       psi%r / psi%i                (Nb, Nk, Na)          OCEAN2/OCEAN_psi.f90:63-76,4272-4274
 *       re/im_bloch_state            (Nb, Nk, Nx, nspn)    OCEAN2/long_range.f90:168-179
 *       W                            (Nk, Nx)              OCEAN2/long_range.f90:1846
 *       mpcr / mpci                  (Nb, Nk, npmax, 2*lmax+1, lmax-lmin+1, nspn)
 *                                                          OCEAN2/OCEAN_multiplet.f90:401
 *       mpm                          (npmax, npmax, lmax-lmin+1)  OCEAN_multiplet.f90:534
 *       mhr / mhi                    packed blocks, row ii of block l contiguous,
 *                                    j1 = jbeg(l) + (jj-1) + (ii-1)*mham(l)
 *                                                          OCEAN_multiplet.f90:1906
 *       somelr / someli              (Na, Na)              OCEAN_multiplet.f90:666-671
 *     Energies are in Hartree, as inside ocean.x.
 *   - One context owns one CUDA stream and the device copies of the operator data
 *     (the module-global `save` state of the reference).  Calls on one context are
 *     not thread safe; calls on different contexts are.
 *   - Entry points ending in _dev take device pointers (FP64 planes laid out as
 *     above) and run on the context's stream; they do not synchronise unless
 *     stated.
 */
#ifndef OCEAN_GPU_H
#define OCEAN_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ocn_ctx ocn_ctx;

enum ocn_status {
  OCN_OK = 0,
  OCN_ERR_NAN = -1,          /* NaN in a Lanczos coefficient (OCEAN_haydock.f90:917-919) */
  OCN_ERR_ARG = 1,           /* bad argument / dimension */
  OCN_ERR_CUDA = 2,          /* CUDA runtime or driver error */
  OCN_ERR_ALLOC = 3,         /* device or host allocation failed */
  OCN_ERR_STATE = 4,         /* required operator data not set */
  OCN_ERR_TIMEOUT = 5,       /* a bounded device wait gave up */
  OCN_ERR_NOCONV = 6,        /* GMRES hit its restart cap before converging */
  OCN_ERR_SOLVE = 7,         /* Gram-matrix factorisation failed (LAPACK info analogue) */
  OCN_ERR_UNSUPPORTED = 9962 /* unsupported flag combination (OCEAN_gmres.f90:539-541) */
};

enum ocn_precision {
  OCN_PREC_FP64 = 0,   /* every product and sum in FP64 (reference numerics) */
  OCN_PREC_MIXED = 1   /* split-BF16 tcgen05 u2 contractions with FP32 accumulation,
                          FP32 k<->R FFT, FP64 vector/Lanczos/GMRES arithmetic */
};

/* Problem dimensions.  Replaces the sizes carried by o_system
 * (OCEAN2/OCEAN_system.f90:14-124) that the hot path reads. */
typedef struct {
  int num_bands;   /* Nb   = sys%num_bands                          */
  int kmesh[3];    /* sys%kmesh; Nk = kmesh[0]*kmesh[1]*kmesh[2]     */
  int xmesh[3];    /* sys%xmesh; Nx = xmesh[0]*xmesh[1]*xmesh[2]     */
  int nalpha;      /* Na   = 4*(2*l_c+1) = sys%nalpha                */
  int nspn;        /* valence spins, 1 or 2 = sys%nspn               */
  int core_l;      /* l_c  = sys%cur_run%ZNL(3)                      */
  int precision;   /* enum ocn_precision                             */
  int device;      /* CUDA device ordinal                            */
  int nvec;        /* largest block of psi vectors acted on together (0 or 1: single) */
} ocn_dims;

/* Scalars of o_system used by the action (OCEAN_system.f90). */
typedef struct {
  double celvol;            /* sys%celvol, Bohr^3                                  */
  double interaction_scale; /* sys%interactionScale (multiplet mul, OCEAN_multiplet.f90:1641) */
  int e0;                   /* sys%e0: one-electron energies on                    */
  int long_range;           /* sys%long_range                                      */
  int mult;                 /* sys%mult: multiplet (F/G) + spin-orbit terms         */
  int nhflag[6];            /* sys%nhflag: LR, ladder, bubble, ct, fg, SO switches   */
} ocn_system;

/* Inputs of lr_populate_W2 / OCEAN_bloch_lrLOAD (long_range.f90:1659-1853,
 * OCEAN_bloch.f90:54-219). */
typedef struct {
  double avec[9];           /* avec(3,3) Fortran order: column i = lattice vector i, Bohr */
  double tau[3];            /* core-site position, fractional                          */
  double epsilon0;          /* sys%epsilon0                                            */
  double interaction_scale; /* sys%interactionScale (W prefactor, long_range.f90:1846)  */
  int nptab;                /* rpottrim table length                                    */
  const double* rtab;       /* (nptab) radii, Bohr, ascending                           */
  const double* ptab;       /* (nptab) screened potential                               */
  int isolated;             /* isolated.inp present                                     */
  double iso_cut;           /* its cutoff, Bohr                                         */
  int pbc[3];               /* pbc.inp (nonzero = periodic); all zero = file absent     */
  int have_eps3d;           /* sys%have3dEpsilon                                        */
  double epsilon3d[3];      /* sys%epsilon3D                                            */
  int xshift_override[3];   /* xshift_override (OCEAN_bloch.f90:113); normally 1,1,1    */
} ocn_lr_params;

/* Multiplet data loaded by OCEAN_create_central (OCEAN_multiplet.f90:248-570). */
typedef struct {
  int lmin, lmax;           /* projector angular momenta                  */
  const int* nproj;         /* (lmax-lmin+1) radial projectors per l       */
  const double* mpcr;       /* see layout notes above                      */
  const double* mpci;
  const double* mpm;        /* direct (Slater F) matrix, Hartree           */
  const double* mhr;        /* exchange (G) matrices, Hartree, sum mham^2  */
  const double* mhi;
} ocn_mult_data;

/* ---------------------------------------------------------------- context */

/* Allocates device state for one problem.  Replaces the allocations done by
 * OCEAN_psi_init/new (OCEAN_psi.f90:3867-4060) and lr_init (long_range.f90:108-244). */
int ocn_ctx_create(const ocn_dims* dims, ocn_ctx** out);
int ocn_ctx_destroy(ocn_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own
 * work or timing events against the library's. */
void* ocn_stream(ocn_ctx* ctx);
/* Copies the last error message of ctx (or of the last failed create when ctx
 * is NULL) into buf. */
int ocn_last_error(const ocn_ctx* ctx, char* buf, size_t len);
/* Library version string and the compute capability it was built for. */
const char* ocn_version(void);

/* ---------------------------------------------------------- operator data */

/* o_system scalars and term switches (OCEAN_system.f90:149-614). */
int ocn_set_system(ocn_ctx* ctx, const ocn_system* sys);

/* p_energy%r/%i after stubby (OCEAN_energies.f90:829-888): complex band energies
 * epsilon + i Sigma'' on the (Nb,Nk,Na) grid.  im may be NULL (zero). */
int ocn_set_energies(ocn_ctx* ctx, const double* re, const double* im);

/* allow%r (OCEAN_energies.f90:371-417): real occupation mask on (Nb,Nk,Na). */
int ocn_set_allow(ocn_ctx* ctx, const double* allow);

/* Raw Bloch functions as read by OCEAN_bloch_load (OCEAN_bloch.f90:395-694),
 * before the core-hole phase.  (Nb,Nk,Nx,nspn). */
int ocn_set_bloch(ocn_ctx* ctx, const double* re, const double* im);

/* lr_init step (4): OCEAN_bloch_lrLOAD phase + xshift (OCEAN_bloch.f90:54-219)
 * applied to the stored Bloch functions, then lr_populate_W2
 * (long_range.f90:1659-1853).  Requires ocn_set_bloch first. */
int ocn_lr_init(ocn_ctx* ctx, const ocn_lr_params* p);

/* Direct replacement of W(Nk,Nx) (e.g. from a caller that built it itself). */
int ocn_set_W(ocn_ctx* ctx, const double* W);

/* Reads back W(Nk,Nx), the xshift and the shifted tau computed by ocn_lr_init.
 * Any output pointer may be NULL. */
int ocn_get_W(ocn_ctx* ctx, double* W, int xshift[3], double tau_shifted[3]);

/* Host-only pieces of ocn_lr_init, usable without a GPU or a context:
 * the xshift / shifted tau of OCEAN_bloch_lrLOAD (OCEAN_bloch.f90:94-123) and
 * the W(Nk,Nx) table of lr_populate_W2 (long_range.f90:1659-1853).  Only the
 * kmesh and xmesh fields of dims are read. */
int ocn_w2_host(const ocn_dims* dims, const ocn_lr_params* p, double* W, int xshift[3],
                double tau_shifted[3]);
/* The core-hole phase e^{i phi(x,k)} of OCEAN_bloch_lrLOAD (OCEAN_bloch.f90:141-204)
 * as cos/sin tables, index x*Nk + k, for the given xshift. */
int ocn_phase_table_host(const ocn_dims* dims, const int xshift[3], double* cos_tab, double* sin_tab);

/* Reads back the phased Bloch functions (Nb,Nk,Nx,nspn) produced by ocn_lr_init
 * (the re/im_bloch_state arrays after OCEAN_bloch_lrLOAD). */
int ocn_get_bloch(ocn_ctx* ctx, double* re, double* im);

/* Multiplet projector data (OCEAN_multiplet.f90:248-570). */
int ocn_set_mult(ocn_ctx* ctx, const ocn_mult_data* m);

/* nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181): the multiplet exchange
 * matrix of one valence angular momentum lv from Slater radial integrals, on
 * the host.  Basis (OCEAN_multiplet.f90:342-369), i = nu + np*((m_v + lv) +
 * (2lv+1)*alpha), alpha = (core spin, core m, valence spin) with the valence
 * spin fastest: mham = 4(2lc+1)(2lv+1)np.  F^k (k = kfl, kfl+2, .., kfh;
 * normally 2 .. min(2lc, 2lv), 0 .. 0 for tdlda's kk files) and G^k (k = kgl,
 * kgl+2, .., kgh; |lc-lv| .. lc+lv) are np x np column-major slices in eV with
 * scale factors scfk / scgk; scfac multiplies all.  Writes mhr/mhi(mham, mham)
 * in the layout ocn_mult_data.mhr takes for this l, in Hartree (the eV2Hartree
 * of OCEAN_multiplet.f90:386-387).  The angular integrals (threey,
 * CNBSE/zcmsnmult/zf90/newthreey.f90) are the closed-form Gaunt coefficients of
 * the complex spherical harmonics the reference evaluates by quadrature. */
int ocn_mult_exchange(int lc, int lv, int np, int kfl, int kfh, const double* fk, const double* scfk, int kgl,
                      int kgh, const double* gk, const double* scgk, double scfac, double* mhr, double* mhi);
/* threey: the integral of conj(Y_{ll,ml}) Y_{lm,mm} Y_{lr,mr} over the sphere
 * (Y_{lm,mm} conjugated when conjug != 0). */
double ocn_threey(int ll, int ml, int lm, int mm, int lr, int mr, int conjug);
/* A Slater-integral file fk<lc><lv><k><add10>, gk.., kk.. (OCEAN_multiplet.f90:
 * 2087-2120): np*np list-directed values (column order) and the scale factor. */
int ocn_read_slater(const char* path, int np, double* f, double* scale);

/* Spin-orbit matrix somelr + i someli, (Na,Na) (OCEAN_multiplet.f90:572-690). */
int ocn_set_spin_orbit(ocn_ctx* ctx, const double* somelr, const double* someli);

/* OCEAN_soprep (OCEAN_multiplet.f90:572-690) without core_broaden.ipt: builds
 * somelr/someli from xi (Hartree) for core angular momentum dims.core_l and
 * installs them. */
int ocn_soprep(ocn_ctx* ctx, double xi);

/* ------------------------------------------------------------------ action */

/* OCEAN_xact (OCEAN_action.f90:286-618), core branch:
 *   out = E o in + A o [H_fg + H_lr](A o in) + H_so in
 * hflag may be NULL (use the system's nhflag).  backwards conjugates E and the
 * spin-orbit matrix as the reference does.  Host buffers; synchronous. */
int ocn_apply_H(ocn_ctx* ctx, const double* in_r, const double* in_i,
                double* out_r, double* out_i, const int* hflag, int backwards);

/* Same on device buffers (each (Nb,Nk,Na) FP64), on the context stream. */
int ocn_apply_H_dev(ocn_ctx* ctx, const double* d_in_r, const double* d_in_i,
                    double* d_out_r, double* d_out_i, const int* hflag, int backwards);

/* H applied to nv vectors at once (host buffers: nv consecutive (Nb,Nk,Na) planes
 * each).  Mixed precision reads the Bloch functions once for the whole block. */
int ocn_apply_H_block(ocn_ctx* ctx, int nv, const double* in_r, const double* in_i,
                      double* out_r, double* out_i, const int* hflag, int backwards);

/* ----------------------------------------------------------------- Haydock */

/* OCEAN_haydock_do -> OCEAN_haydock_Herm_do (OCEAN_haydock.f90:167-320) with
 * ocean_hay_ab_twoterm (:824-938).  psi0 must already be normalised (core_pnorm,
 * OCEAN_psi.f90:5589-5638).  Writes real_a[0..niter], imag_a[0..niter],
 * real_b[0..niter] (index 0 of b unused = 0, a[niter] = 0 as in the reference's
 * zero-initialised arrays).  *niter_done = iterations completed.
 * Returns OCN_ERR_NAN if an a_n is NaN (checked after the loop).  Host buffers.
 * Mixed-precision contexts keep the Lanczos vectors in double-float (binary32
 * pairs, ~48 significant bits) on the device; a, b are formed and returned in FP64. */
int ocn_haydock(ocn_ctx* ctx, const double* psi0_r, const double* psi0_i, int niter,
                double* real_a, double* imag_a, double* real_b, int* niter_done);

/* Same with psi0 in device memory; coefficient outputs are host arrays. */
int ocn_haydock_dev(ocn_ctx* ctx, const double* d_psi0_r, const double* d_psi0_i, int niter,
                    double* real_a, double* imag_a, double* real_b, int* niter_done);

/* Block Haydock: nv independent Lanczos chains that share H (the polarisations
 * or photons of one core site, OCEAN.f90:51-83 runs them one after another),
 * advanced in lockstep so that every read of the Bloch functions serves all nv
 * vectors.  Each chain is exactly OCEAN_haydock_Herm_do on its own psi0.
 * psi0_r/psi0_i: nv consecutive (Nb,Nk,Na) planes (host); real_a, imag_a,
 * real_b: nv consecutive arrays of niter+1; niter_done: nv entries (may be NULL).
 * nv <= dims.nvec; the FP64 path runs the chains one after another.  Returns
 * OCN_ERR_NAN if any chain produced a NaN a_n (its niter_done entry stops there). */
int ocn_haydock_block(ocn_ctx* ctx, int nv, const double* psi0_r, const double* psi0_i, int niter,
                      double* real_a, double* imag_a, double* real_b, int* niter_done);

/* Same with the nv psi0 vectors in device memory: vector v at d_psi0 + 2*v*npsi
 * (real plane, then imaginary plane). */
int ocn_haydock_block_dev(ocn_ctx* ctx, int nv, const double* d_psi0, int niter, double* real_a,
                          double* imag_a, double* real_b, int* niter_done);

/* Non-Hermitian Haydock: the two-sided Lanczos of OCEAN_haydock_nonHerm_do
 * (OCEAN_haydock.f90:53-164, selected there by complex_haydock), for an H
 * made non-Hermitian by complex band energies or a broadened spin-orbit term.
 * Right vectors see H, left vectors H^dagger (the action with backwards set,
 * OCEAN_action.f90:286); both start from psi0 under the allow mask.  The step
 * follows the algorithm that haydock_abc_1 (:1250-1433) cites (Saad):
 * alpha_j = <w_j|H v_j>, z = <w^|v^>, delta = sqrt(z) (principal, as :1373-1374),
 * beta = z/delta, v_{j+1} = (H v_j - alpha_j v_j - beta_j v_{j-1}) / delta,
 * w_{j+1} = (H^dagger w_j - conj(alpha_j) w_j - conj(delta_j) w_{j-1}) / conj(beta).
 * (haydock_abc_1 itself, never called in the reference, subtracts conj(beta_j)
 * and divides by beta; its tridiagonal then fails the moment test beyond k = 2.)
 * Stored as write_core reads them (e - real_a, gam + imag_a, products b*c):
 * a = alpha, b = conj(beta), c = conj(delta), so ocn_spectrum_cf_bc gives
 * kpref |Im <psi0|(z - H^dagger)^-1|psi0>|, the Hermitian run's convention.
 * Arrays (0:niter); b and c from index 1.  Host planes in, FP64 recurrence in
 * both precisions (the action in the context's precision). */
int ocn_haydock_nonherm(ocn_ctx* ctx, const double* psi0_r, const double* psi0_i, int niter, double* real_a,
                        double* imag_a, double* real_b, double* imag_b, double* real_c, double* imag_c,
                        int* niter_done);

/* Batched Haydock over independent problems: context i runs nv[i] chains
 * (ocn_haydock_block_dev on d_psi0[i]) for niter iterations.  Three iterations
 * of every context are captured into one CUDA graph that is replayed niter/3
 * times, so one launch advances all problems.  Mixed-precision contexts with the
 * long-range term and without the multiplet term share grouped launches: each
 * stage of a step (the two tensor-core contractions, the k-mesh transforms, the
 * operand builders, the Lanczos kernels) is one persistent launch over the tiles
 * or vectors of all of them, each context keeping its own tiling, so its results
 * equal those of its own launches bit for bit.  Other contexts run as branches
 * of their own (also with the environment variable OCN_BATCH_BRANCHES=1).  The
 * reference runs such problems one after another (OCEAN.f90:51-83, one ocean.x
 * run per site and photon).  Contexts must share one device; outputs per
 * context as for ocn_haydock_block_dev (niter_done may be NULL).  Returns the
 * first hard error, else OCN_ERR_NAN if a chain hit a NaN. */
int ocn_haydock_batch(ocn_ctx* const* ctxs, int nctx, const int* nv, const double* const* d_psi0,
                      int niter, double* const* real_a, double* const* imag_a,
                      double* const* real_b, int* const* niter_done);

/* core_pnorm (OCEAN_psi.f90:5589-5638): normalises psi in place (host planes of
 * n = Nb*Nk*Na values) and returns kpref = 4 pi |psi|^2 / (Nk celvol^2). */
int ocn_psi_pnorm(int n, int nkpts, double celvol, double* psi_r, double* psi_i, double* kpref);

/* write_core (OCEAN_haydock.f90:1801-1894) or write_core_Voigt (:1896-1989)
 * when gam_gauss > gam0/10: the continued fraction with square-root terminator on
 * ne+1 energies e = el + (eh-el)*ie/(2ne), ie = 0,2,..,2ne, evaluated on the GPU
 * in FP64.  Output rows of 9 columns (Voigt: 5 columns, remaining zero):
 *   Energy(eV), Spect, Spect(0), SPKK, SPKK(0), sigma, sigma cm^2, sig^2, sig^2 cm^4 s.
 * imag_a may be NULL.  el, eh, gam0, gam_gauss in Hartree; ebase in eV.
 * old_broaden selects the gamfcn column (nval, eps as in OCEAN_haydock_setup). */
typedef struct {
  double el, eh, gam0, ebase, gam_gauss;
  int ne;
  double ucvol;
  int old_broaden;
  double nval, eps;
} ocn_cf_params;
int ocn_spectrum_cf(const double* real_a, const double* imag_a, const double* real_b,
                    int iter, double kpref, const ocn_cf_params* p, double* out /* (ne+1)*9 */);

/* ocn_spectrum_cf with the complex b and c of ocn_haydock_nonherm: write_core's
 * products cmplx(real_b, imag_b) * cmplx(real_c, imag_c) (binary32, as the
 * reference forms them, OCEAN_haydock.f90:1846-1870).  imag_b, real_c, imag_c
 * NULL: the Hermitian run (c = b real). */
int ocn_spectrum_cf_bc(const double* real_a, const double* imag_a, const double* real_b, const double* imag_b,
                       const double* real_c, const double* imag_c, int iter, double kpref,
                       const ocn_cf_params* p, double* out);

/* ocn_spectrum_cf (write_core path only) without any device allocation: no
 * counterpart in the reference, which evaluates the fraction on the host.  For
 * callers that cannot allocate device memory at that point (HBM held by a
 * caching allocator or by the vectors of a large run) or must not stall the
 * device with cudaFree.  Its buffers live in one static device array of
 * 3*(OCN_CF_NOALLOC_MAX_ITER+1) + 10*(OCN_CF_NOALLOC_MAX_NE+1) doubles (736 KiB).
 * Runs on the calling thread's current device; the first call on a device looks
 * up that array's address (set-up), so make it before any stream capture.
 * The address is kept for the life of the process: do not call this entry
 * point on a device after cudaDeviceReset (the module may be reloaded at
 * another address).
 * iter > OCN_CF_NOALLOC_MAX_ITER, ne > OCN_CF_NOALLOC_MAX_NE and Voigt broadening
 * (gam_gauss > gam0/10) return OCN_ERR_ARG.  Nothing must be zeroed first.  Calls
 * that overlap on one device share the array and race: serialise them.  Same
 * output as ocn_spectrum_cf; on error the contents of out are unspecified. */
#define OCN_CF_NOALLOC_MAX_ITER 4096
#define OCN_CF_NOALLOC_MAX_NE 8192
int ocn_spectrum_cf_noalloc(const double* real_a, const double* imag_a, const double* real_b,
                            int iter, double kpref, const ocn_cf_params* p, double* out);

/* Haydock early exit: the haydockconv.ipt test of OCEAN_haydock_Herm_do
 * (OCEAN_haydock.f90:268-292, check_convergence :1608-1661, calc_spect_core
 * :1991-2027; switched on by OCEAN_system.f90:452-462).  After every Lanczos
 * step it > spacing the run compares the spectra of it and it - spacing steps
 * on ne midpoints (column Spect(0)) by relArea = 2 sum|s1 - s2| / (sum|s1| +
 * sum|s2|); the run stops at the first step whose relArea and the previous
 * step's are both below the threshold (*niter_done = that step; coefficients
 * beyond it are returned as 0).  The test runs on the device inside the
 * captured Lanczos graph; the host reads the relArea of each step every 30
 * steps, so up to 30 steps beyond the stop are computed and discarded. */
typedef struct {
  double threshold;      /* haydockConvergeThreshold; <= 0 switches the test off */
  int spacing;           /* haydockConvergeSpacing (>= 1) */
  int ne;                /* energy points of the test spectra (bse.in ne) */
  double el, eh, gam0;   /* bse.in energy window and broadening, Hartree */
  double kpref;          /* hay_vec%kpref of the run */
} ocn_haydock_conv;
/* Sets (p != NULL, threshold > 0) or clears the test for this context's
 * single-chain Haydock runs (ocn_haydock, ocn_haydock_dev); block and batched
 * runs ignore it. */
int ocn_set_haydock_conv(ocn_ctx* ctx, const ocn_haydock_conv* p);
/* haydockconv.ipt: "threshold spacing", list-directed (OCEAN_system.f90:452-458). */
int ocn_read_haydockconv(const char* path, double* threshold, int* spacing);

/* redtrid (OCEAN_haydock.f90:2273-2316): eigenvalues (ascending) of the (n+1)x(n+1)
 * tridiagonal Lanczos matrix; host FP64. */
int ocn_redtrid(int n, const double* real_a, const double* real_b, double* w /* n+1 */);

/* ------------------------------------------------------------------- GMRES */

typedef struct {
  int depth;              /* gmres_depth (bse.in)                                */
  double resolution;      /* gmres_resolution = Gamma, Hartree                    */
  double preconditioner;  /* gmres_preconditioner (gprc), Hartree                 */
  double convergence;     /* gmres_convergence (ffff) on |g|^2                    */
  int max_restarts;       /* cap on restart cycles per energy (the reference loops forever) */
} ocn_gmres_params;

/* OCEAN_gmres_do_recycle (OCEAN_gmres.f90:508-908) with update_gmres (:241-344),
 * make_recycle (:207-239), set_initial_vector (:1213-1283) and
 * OCEAN_psi_min_set_prec (OCEAN_psi.f90:2907-2994).  hay_vec is the normalised
 * psi0 (host planes); energies[nomega] in eV as in bse.in.  The recycled P
 * updates at a new energy run as one P x P projection built from Gram matrices
 * of the basis kept across energies (equal in exact arithmetic).  Mixed-
 * precision contexts form the Gram dots and basis updates in double-float
 * (binary32 pairs, 48-bit significands); the solve stays FP64.  Writes, per energy,
 *   out_re[i] = 1 - Re<b|x>*kpref, out_im[i] = -Im<b|x>*kpref,
 *   rel_err[i] = -|g|^2/Im<b|x>, iters[i] = complete_iter
 * (the abs.gmres columns, OCEAN_gmres.f90:864-869).  Any output may be NULL. */
int ocn_gmres(ocn_ctx* ctx, const double* hay_r, const double* hay_i, double kpref,
              const double* energies_ev, int nomega, const ocn_gmres_params* p,
              double* out_re, double* out_im, double* rel_err, int* iters);

/* Energy lanes of the GMRES sweep of this context (no counterpart in the
 * reference; default 1 = its single sweep, OCEAN_gmres.f90:613-884).  With
 * nlanes > 1, ocn_gmres, ocn_gmres_dev and ocn_gmres_vjp split the energy list
 * into nlanes contiguous chunks; each chunk is the reference's recycled sweep
 * from x = 0 at its first energy, and the chunks advance together so that one
 * block action (ocn_apply_H_block; up to nvec vectors per launch set on
 * mixed-precision contexts) serves all of them.  Results agree with the single
 * sweep within the convergence tolerance; iteration counts differ.  nlanes in
 * 1..64, else OCN_ERR_ARG. */
int ocn_gmres_set_lanes(ocn_ctx* ctx, int nlanes);

/* Same with psi0 in device memory (d_hay: real plane then imaginary plane, npsi
 * each).  d_x (device, may be NULL) receives the solution x of every energy:
 * nomega consecutive blocks of 2*npsi doubles (the input of ocn_gmres_vjp). */
int ocn_gmres_dev(ocn_ctx* ctx, const double* d_hay, double kpref, const double* energies_ev,
                  int nomega, const ocn_gmres_params* p, double* out_re, double* out_im,
                  double* rel_err, int* iters, double* d_x);

/* Adjoint (reverse-mode) derivatives of the ocn_gmres spectrum; no counterpart
 * in the reference.  With F(w) = <b|x(w)>, x = (w + i Gamma - H)^-1 b, and the
 * adjoint y = (w - i Gamma - H)^-1 b (the same recycled GMRES at -Gamma), a
 * parameter t of H or of the resolvent gives dF/dt = <y| dH/dt |x>.  For the
 * loss L = sum_w grad_re[w]*out_re[w] + grad_im[w]*out_im[w] (either grad
 * array may be NULL = 0) this returns
 *   *g_gamma   = dL/dGamma            (dF/dGamma = -i <y|x>)
 *   *g_scissor = dL/ds for E -> E + s (dF/ds = <y|x>)
 *   d_gW       = dL/dW(R, x) on the device, Nk*Nx doubles at [x*Nk + k]
 *                (dF/dW = -(1/Nk) sum_alpha conj(A^y) A^x, A^v the band-to-x
 *                 transform of allow o v taken back over the k-mesh).
 * d_x: the forward solutions from ocn_gmres_dev.  Needs real energies, no
 * multiplet or spin-orbit term, and a cubic k-mesh of extent 2,3,4,5,6 or 8
 * (else OCN_ERR_UNSUPPORTED).  ocn_w2_vjp maps d_gW to the W(r) table. */
int ocn_gmres_vjp(ocn_ctx* ctx, const double* d_hay, double kpref, const double* energies_ev,
                  int nomega, const ocn_gmres_params* p, const double* d_x,
                  const double* grad_re, const double* grad_im, double* g_gamma,
                  double* g_scissor, double* d_gW);

/* Chain rule through lr_populate_W2 (long_range.f90:1659-1853) on the host:
 * from G = dL/dW (Nk*Nx, [x*Nk + k]) returns dL/dptab[nptab] (the radial table
 * samples, linear interpolation of intval) and dL/d(interaction_scale). */
int ocn_w2_vjp(const ocn_dims* dims, const ocn_lr_params* p, const double* G, double* g_ptab,
               double* g_scale);

/* ----------------------------------------------------- reference text files */

/* The solver settings of bse.in as ocean.x reads them (list-directed input):
 * record 1 an integer, record 2 a real (OCEAN_driver.f90:67-68), record 3 the
 * style; for 'hay' (OCEAN_haydock.f90:2118) niter ne el eh gam0 ebase; for 'inv'
 * (OCEAN_gmres.f90:89-124) depth resolution preconditioner convergence, then
 * 'list' (count, one energy per record) or 'loop' (start stop step, count
 * 1 + ceiling((stop - start - step*1e-4)/step)).  Energies stay in eV as written;
 * a non-positive gam0 / resolution means "core-hole lifetime" to the reference
 * and is returned unchanged. */
typedef struct {
  int dumi;
  double dumf;
  char style[8];        /* 'hay', 'inv', 'exa' or 'dia' */
  int niter, ne;        /* hay */
  double el, eh, gam0, ebase;
  int depth;            /* inv */
  double resolution, preconditioner, convergence;
  char inv_style[8];    /* 'list' or 'loop' */
  int nomega;
} ocn_bse_in;
/* energies (may be NULL): receives up to cap GMRES energies in eV; returns
 * OCN_ERR_ARG if the list is longer than cap (out->nomega is still set). */
int ocn_read_bse_in(const char* path, ocn_bse_in* out, double* energies, int cap);

/* write_lanczos (OCEAN_haydock.f90:2318-2358), byte for byte: '(1i8,1x,1ES24.17)'
 * n, kpref; the coefficients ('(2x,ES24.17)' / '(2(2x,ES24.17))', or six per
 * record when imag_a is given: the complex Haydock form with real_c/imag_c,
 * which default to the b arrays); then, when eigs (n+1 values) is given, the
 * redtrid eigenvalues '(2x,2i5,1f20.10)'.  Arrays are (0:n). */
int ocn_write_abslanc(const char* path, int n, double kpref, const double* real_a,
                      const double* imag_a, const double* real_b, const double* imag_b,
                      const double* real_c, const double* imag_c, const double* eigs);

/* write_core / write_core_Voigt output (OCEAN_haydock.f90:1831-1892,1922-1985),
 * byte for byte: header, column names, then ne+1 rows of the 9 (Voigt: first 5)
 * columns of ocn_spectrum_cf's output, '(9(1e15.8,1x))'.  gam0 in Hartree. */
int ocn_write_absspct(const char* path, int iter, double gam0, double kpref, double ucvol,
                      int ne, const double* rows /* (ne+1)*9 */, int voigt);

/* abs.gmres (OCEAN_gmres.f90:864-869): per energy '(1p,4(1e15.8,1x),1i6,1x,i10)'
 * energy (eV, through Hartree and back as the reference does), out_re, out_im,
 * rel_err, iterations, running total of iterations. */
int ocn_write_abs_gmres(const char* path, int nomega, const double* energies_ev,
                        const double* out_re, const double* out_im, const double* rel_err,
                        const int* iters);

/* OCEAN_filenames_spectrum / _lanc (OCEAN_filenames.f90:21-107) for XAS / XES
 * runs: kind "spct" or "lanc", e.g. absspct_Cu.0001_1s_01. */
int ocn_output_filename(const char* kind, const char* calc_type, const char* elname, int indx,
                        const char* corelevel, int photon, char* buf, size_t len);

/* ------------------------------------------------ pipeline input files */

/* Files written by the OCEAN pipeline for ocean.x, read as ocean.x reads them.
 * Sequential unformatted files are read with 4-byte record frames (gfortran,
 * ifort).  All return OCN_ERR_ARG on a missing, short or malformed file. */

/* u2.dat (OCEAN_bloch.f90:515-575, the 'old' Bloch-state format): per spin, per
 * k-point (kmesh loops iq1, iq2, iq3), nband_file bands of nx*ny*nz records
 * (ix, iy, iz with iz fastest), each three integers and the real and imaginary
 * part.  first[] is the first band read per (k-point, spin) (0-based: the
 * occupied bands the reference skips, ivh2 - ivl + 1 in its notation; nfirst = 1
 * for one value everywhere, else nkpts*nspn values, k fastest); nbd bands are
 * read from there.  re/im receive re_bloch_state(nbd, nkpts, nx*ny*nz, nspn)
 * with x = ix + nx*(iy + ny*iz), before the lrLOAD phase (ocn_set_bloch). */
int ocn_read_u2dat(const char* path, int nx, int ny, int nz, int nkpts, int nspn, int nband_file,
                   const int* first, int nfirst, int nbd, double* re, double* im);

/* u2par.dat, the 'new' Bloch-state format (load_new_u2, OCEAN_bloch.f90:697-996,
 * chosen by bloch_type = 'new'): a raw complex(DP) array without record frames;
 * the states of (k-point, spin) start at element (k + spin*nkpts)*width3*Nx
 * (width3 = the third line of obf_control), the first[] bands of each are
 * skipped (first as in ocn_read_u2dat) and nbd bands read, each band over the
 * x-mesh with iz fastest.  Output as ocn_read_u2dat: re_bloch_state(nbd,
 * nkpts, Nx, nspn), x = ix + nx*(iy + ny*iz). */
int ocn_read_u2par(const char* path, const int xmesh[3], int nkpts, int nspn, int width3, const int* first,
                   int nfirst, int nbd, double* re, double* im);
/* con.u2.dat of a core-level run, the 'par' route that ocean.x takes whenever
 * con.u2.dat exists (OCEAN_bloch.f90:481-482; single_load_prefixu2dat :998-1115;
 * val.u2.dat for XES): stream access, per spin, k-point and file band one
 * complex(DP) array over the Nx x-points in the states' order; bands_in_file
 * bands per k-point (brange(4) - brange(3) + 1), the first nbd kept.  Output as
 * ocn_read_u2dat. */
int ocn_read_con_u2(const char* path, int nxpts, int nkpts, int nspn, int bands_in_file, int nbd, double* re,
                    double* im);
/* obf_control: the three widths of the 'new' format (OCEAN_bloch.f90:722-727). */
int ocn_read_obf_control(const char* path, int width[3]);

/* rpottrim.z<El><idx>_n<nn>l<ll> (long_range.f90:1689-1698): a header record
 * (a word, nptab) then nptab records ptab rtab.  With ptab and rtab NULL only
 * *nptab is returned; otherwise up to cap samples (OCN_ERR_ARG if more). */
int ocn_read_rpottrim(const char* path, int* nptab, double* ptab, double* rtab, int cap);

/* val.u2.dat / con.u2.dat of a valence run (load_single_prefixu2dat,
 * OCEAN_val_states.f90:421-560): stream access (no record markers), for each
 * spin, k-point and file band [file_b0, file_b1] the complex(DP) state over
 * the x-mesh with x1 fastest.  Bands band_lo .. band_lo + nb - 1 land in
 * re / im(Nx, nb, nkpts, nspn) with x3 fastest: the layout ocn_val_set_states
 * takes (val: brange(1), nbv; con: brange(3), nbc). */
int ocn_read_val_u2(const char* path, const int xmesh[3], int nkpts, int nspn, int file_b0, int file_b1,
                    int band_lo, int nb, double* re, double* im);
/* Pair energies of a valence run (OCEAN_read_energies, OCEAN_val_energy.f90:
 * 266-296, nbw = 1): out(Nc, Nv, Nk, vspin^2) = e_con(c + con_lo - 1, k, j-spin)
 * - e_val(v + val_lo - 1, k, i-spin) from the wvfcninfo / wvfvainfo arrays
 * (ncon_file / nval_file bands each, ocn_read_energies), 1-based band offsets
 * (brange(3), brange(1)).  The Fermi-level, GW and allow steps of that routine
 * are set-up left to the caller. */
int ocn_val_pair_energies(int nc, int nv, int nkpts, int nspn, int vspin, const double* con_e, int ncon_file,
                          int con_lo, const double* val_e, int nval_file, int val_lo, double* out);

/* wvfcninfo / wvfvainfo (OCEAN_energies.f90:629-689): header (nbd, nq) or, with
 * two spins, (nbd, nq, nspn); then energies(nbd, nq, nspn) as written (the
 * pipeline's units; stubby, OCEAN_energies.f90:829-888, turns them into the
 * energies of ocn_set_energies).  e NULL: header only. */
int ocn_read_energies(const char* path, int nspn, int* nbd, int* nq, double* e, size_t cap);

/* Projector coefficients (OCEAN_multiplet.f90:414-463): stream = 1 for the
 * parallel file parcksc.* (three integers, the second nbd*nkpts, then complex
 * pcTemp(nptot, nbd, nkpts, nspn); bands beyond nb are dropped), stream = 0 for
 * the legacy cksc.* (two records skipped, then pcr and pci).  pcr/pci receive
 * (nptot, nb, nkpts, nspn). */
int ocn_read_cks(const char* path, int stream, int nptot, int nb, int nkpts, int nspn, double* pcr,
                 double* pci);
/* The reordering of OCEAN_multiplet.f90:466-481 into the mpcr/mpci layout of
 * ocn_mult_data (Nb, Nk, npmax, 2*lmax+1, lmax-lmin+1, nspn); projector ip runs
 * over l, m = -l..l, nu.  Unused (nu, m) slots are zero. */
int ocn_cks_to_mpc(int lmin, int lmax, const int* nproj, int nb, int nkpts, int nspn, const double* pcr,
                   const double* pci, double* mpcr, double* mpci);
/* cmel<l> (OCEAN_multiplet.f90:489-500): nproj*nproj list-directed values into
 * mpm(1:nproj, 1:nproj) of that l, column-major as the reference fills it. */
int ocn_read_cmel(const char* path, int nproj, double* mpm);

/* Input file names as ocean.x forms them: kind "rpottrim" (uses n, l),
 * "cks" / "parcks" (calc_type "XES" gives cksv.), "cmel" (uses l), "energies"
 * (calc_type "VAL" gives wvfvainfo). */
int ocn_input_filename(const char* kind, const char* calc_type, const char* elname, int indx, int n, int l,
                       char* buf, size_t len);

/* --------------------------------------------------------------- counters */

/* Number of kernels this context launched since creation (for accounting). */
long long ocn_kernel_launches(const ocn_ctx* ctx);

/* Tile configuration of the mixed-precision tensor-core contractions (no
 * counterpart in the reference, whose BLAS calls have none): tiles[7] =
 * {shared-memory pipeline stages, K splits of the x->band contraction,
 *  persistent grid cap of the band->x contraction, of the x->band one,
 *  k-mesh transforms per CTA (0 = all of an x-point), threads of a k-mesh
 *  transform CTA (128, 256 or 512; 0 = 128), band->x output staging (1: the
 *  contraction's outputs go through shared memory and are stored coalesced,
 *  when the pipeline leaves room; 0: stored directly)}.
 * ocn_autotune times the long-range term of an nv-vector block under each
 * candidate (reps launches each, CUDA events) and keeps the fastest; returns
 * its time in ms, the time of the tiling in force before the call, and the
 * chosen tiles (any output may be NULL).  Tilings change only the order of
 * FP32 partial sums.  Mixed precision only (else OCN_ERR_UNSUPPORTED). */
int ocn_autotune(ocn_ctx* ctx, int nv, int reps, double* best_ms, double* current_ms, int tiles[7]);
int ocn_set_tiles(ocn_ctx* ctx, const int tiles[7]);
int ocn_get_tiles(const ocn_ctx* ctx, int tiles[7]);

/* Test hook for the bounded waits of the tensor-core contractions (no
 * counterpart in the reference).  on = 1: the long-range contractions' load
 * warp issues no loads, so the MMA warp's first bounded wait (about 1 s) runs
 * out with no copy or MMA in flight; the kernel records it, frees its tensor
 * memory and returns, and the call reports OCN_ERR_TIMEOUT.  on = 0 restores
 * normal operation; the context stays usable.  Mixed precision only. */
int ocn_test_starve_tc(ocn_ctx* ctx, int on);

/* Per-kernel device timing with CUDA events recorded on the context stream
 * (replaces the wall-clock buckets of OCEAN_timekeeper, OCEAN_timekeeper.f90:13-168).
 * Classes: 0 LR band->x contraction, 1 LR k-mesh transform x W, 2 LR x->band
 * contraction, 3 LR operand preparation, 4 multiplet, 5 combine + Lanczos step.
 * ocn_timing_read synchronises the stream and returns, per class, the launch
 * count and the summed milliseconds since the last reset. */
int ocn_timing_enable(ocn_ctx* ctx, int on);
int ocn_timing_reset(ocn_ctx* ctx);
int ocn_timing_read(ocn_ctx* ctx, long long counts[6], double ms[6]);

/* ------------------------------------------------------- valence BSE
 * The valence branch of OCEAN_xact (OCEAN_action.f90:521-600) for resonant
 * pairs (nbw = 1), valence_ham_spin 1 or 2 and one or two DFT spins:
 *   H psi = E o psi + allow o [ 2 X(allow o psi) - D(allow o psi) (+ 2 F(allow o psi)) ]
 * X: AI_bubble_act (OCEAN_bubble.f90:420-796); F: OCEAN_fxc_act when a kernel
 * is set (OCEAN_fxc.f90:127-322); D: OCEAN_ladder_act_single
 * (OCEAN_ladder.f90:155-1004).  Replaces those routines and the module state
 * they read (re/im_con, re/im_val of OCEAN_val_states, p_energy and allow of
 * OCEAN_energies, bubble of OCEAN_bubble, ladder of OCEAN_ladder).
 * Layouts are the reference's Fortran orders:
 *   psi, energies, allow  (Nc, Nv, Nk, vspin^2)  psi%valr(c, v, k, ibeta)
 *   con                   (Nx, Nc, Nk, nspn)     re_con / im_con(x, c, k, spin)
 *   val                   (Nx, Nv, Nk, nspn)     re_val / im_val(x, v, k, spin)
 * ibeta = (i - 1) vspin + j pairs valence spin i with conduction spin j
 * (OCEAN_ladder.f90:118-133); the exchange couples the same-spin blocks
 * (OCEAN_bubble.f90:509-760, spin_prefac 2 for one spin, 1 for two).
 *   bubble                (Nx)
 *   ladder                (Nk, Nx, Nx)   ladder(k, x, y) after resort_ladder
 * with the flat k index k3 fastest and the flat x index x3 fastest (the FFT
 * orders of OCEAN_ladder_init, OCEAN_ladder.f90:1599-1695, and AI_bubble_prep,
 * OCEAN_bubble.f90:67-157).  OCN_PREC_MIXED computes the direct term's
 * O(Nx^2 Nk) part (A, val, ladder, k-mesh transforms, B) in FP32; the rest,
 * and all Lanczos vectors, stay FP64. */
typedef struct ocn_val_ctx ocn_val_ctx;

typedef struct {
  int nc, nv;     /* conduction / valence bands (1 <= nv <= 32) */
  int kmesh[3];   /* k-mesh (each 1..32) */
  int xmesh[3];   /* x-mesh of the states, bubble and ladder (each 1..32) */
  int precision;  /* OCN_PREC_FP64 or OCN_PREC_MIXED */
  int device;     /* CUDA device ordinal */
  int nspn;       /* DFT spins of con/val: 1 (0 reads as 1) or 2 */
  int vspin;      /* valence_ham_spin: 1 (0 reads as 1) or 2 */
} ocn_val_dims;

int ocn_val_create(const ocn_val_dims* dims, ocn_val_ctx** out);
int ocn_val_destroy(ocn_val_ctx* ctx);
int ocn_val_last_error(const ocn_val_ctx* ctx, char* buf, size_t len);
long long ocn_val_kernel_launches(const ocn_val_ctx* ctx);
void* ocn_val_stream(ocn_val_ctx* ctx);

/* Operator data (host buffers; the _dev variants take device pointers). */
int ocn_val_set_energies(ocn_val_ctx* ctx, const double* re, const double* im /* may be NULL */);
int ocn_val_set_allow(ocn_val_ctx* ctx, const double* allow);
int ocn_val_set_states(ocn_val_ctx* ctx, const double* con_r, const double* con_i, const double* val_r,
                       const double* val_i);
int ocn_val_set_states_dev(ocn_val_ctx* ctx, const double* con_r, const double* con_i, const double* val_r,
                           const double* val_i);
int ocn_val_set_bubble(ocn_val_ctx* ctx, const double* bubble);
int ocn_val_set_ladder(ocn_val_ctx* ctx, const double* ladder);
int ocn_val_set_ladder_dev(ocn_val_ctx* ctx, const double* d_ladder);

/* The ALDA f_xc term (OCEAN_fxc_act, OCEAN_fxc.f90:127-322; aldaf): on while a
 * kernel fxc(Nx) is set (NULL: off); valence_ham_spin = 1 only, as the
 * reference (else OCN_ERR_UNSUPPORTED).  ocn_val_fxc_from_rho builds it from
 * the density on the x-mesh (OCEAN_fxc_prep with cacorr, :35-123,333-470).
 * Host only; rho in the x-mesh order. */
int ocn_val_set_fxc(ocn_val_ctx* ctx, const double* fxc);
int ocn_val_fxc_from_rho(int nx, const double* rho, double celvol, int nkpts, double* fxc);

/* bubble(x) from the cell (AI_bubble_populate with wall_search_old_way,
 * OCEAN_bubble.f90:238-407): bvec column-major (bvec[i + 3 j] = bvec(i+1, j+1),
 * Bohr^-1), qinb = sys%qinunitsofbvectors, celvol in Bohr^3; *ngvec (may be
 * NULL) = retained G-vectors - 1 as the reference prints it.  Host only. */
int ocn_val_bubble_populate(const int xmesh[3], const double bvec[9], const double qinb[3], double celvol,
                            int nkpts, double* bubble, int* ngvec);

/* H psi.  flags[3] = {bande (energies), bflag & hflag(3) (exchange),
 * lflag & hflag(2) (direct)}; backwards conjugates E (OCEAN_energies.f90:890-906).
 * Host buffers (in/out planes of Nc*Nv*Nk); _dev: device vectors, real plane
 * then imaginary plane (2*Nc*Nv*Nk doubles), on the context stream. */
int ocn_val_apply_H(ocn_val_ctx* ctx, const double* in_r, const double* in_i, double* out_r, double* out_i,
                    const int flags[3], int backwards);
int ocn_val_apply_H_dev(ocn_val_ctx* ctx, const double* d_in, double* d_out, const int flags[3], int backwards);

/* OCEAN_haydock_Herm_do with ocean_hay_ab_twoterm over the valence action
 * (OCEAN_haydock.f90:190-320, 824-938): arrays of niter+1; OCN_ERR_NAN on a NaN
 * a_n.  psi0 is used as given (normalise it first, core_pnorm). */
/* OCEAN_gmres_do_recycle over the valence action (OCEAN_gmres.f90:508-908 with
 * the have_val branches :544-548, :603-606): rhs = allow o psi0, the
 * preconditioner from H (allow o 1), outputs as ocn_gmres with kpref replaced
 * by fact = kpref * 2 * celvol.  flags as ocn_val_apply_H (NULL: all terms).
 * The single recycled sweep; mixed-precision contexts form the Gram dots in
 * double-float as ocn_gmres does. */
int ocn_val_gmres(ocn_val_ctx* ctx, const double* hay_r, const double* hay_i, double kpref, double celvol,
                  const double* energies_ev, int nomega, const ocn_gmres_params* p, const int flags[3],
                  double* out_re, double* out_im, double* rel_err, int* iters);
int ocn_val_haydock(ocn_val_ctx* ctx, const double* psi0_r, const double* psi0_i, int niter, const int flags[3],
                    double* real_a, double* imag_a, double* real_b, int* niter_done);
int ocn_val_haydock_dev(ocn_val_ctx* ctx, const double* d_psi0, int niter, const int flags[3], double* real_a,
                        double* imag_a, double* real_b, int* niter_done);

/* write_val (OCEAN_haydock.f90:1706-1799), the spectrum of a valence run
 * (haydump's 'VAL'/'RXS' branch, file "opcons"): ne rows at the midpoints
 * el + (eh - el)(2r+1)/(2 ne) (Hartree), each 8 values
 *   omega (eV), eps1, eps2, Re(n) - 1, Im(n), mu (1/cm), R, epsinv
 * with eps = 1 - fact/al [- fact/be when semi_tda], fact = kpref (2/val_ham_spin)
 * ucvol (integer division), al/be the resonant / anti-resonant continued
 * fractions with the square-root terminator at the real energy, backf: z and
 * the energy squared (the backward-pair form).  imag_a/imag_b/real_c/imag_c may
 * be NULL (Hermitian run: c = b, imaginary parts 0).  Evaluated on the GPU,
 * FP64.  out: ne * 8. */
typedef struct {
  double kpref, ucvol;
  double el, eh, gam0;  /* Hartree */
  int ne, val_ham_spin, semi_tda, backf;
} ocn_val_cf_params;

int ocn_val_spectrum(const double* real_a, const double* imag_a, const double* real_b, const double* imag_b,
                     const double* real_c, const double* imag_c, int iter, const ocn_val_cf_params* p, double* out);
/* write_val's optical constants (:1778-1795) for given eps at energies omega
 * (Hartree); out: n * 8 in the column order above.  Host only. */
int ocn_val_optical_constants(int n, const double* omega, const double* eps_re, const double* eps_im, double* out);
/* The "opcons" file write_val writes: its header and '(8(1E24.16,1X))' rows. */
int ocn_write_opcons(const char* path, int ne, const double* rows);

#ifdef __cplusplus
}
#endif

#endif /* OCEAN_GPU_H */
