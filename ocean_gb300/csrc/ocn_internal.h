// ocn_internal.h -- shared definitions of libocean_gpu.so (not installed).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/ocean_gpu.h"

#define OCN_MAX_NA 12       // 4*(2*l_c+1) for l_c <= 1 (1s, 2p edges)
#define OCN_MAX_KDIM 32     // largest k-mesh extent along one axis handled by the FFT kernels
#define OCN_MAX_NK 4096     // largest k-mesh size (shared-memory FFT)
#define LZ_THREADS 256      // threads of the Lanczos-step kernels
#define LZ_DF_THREADS 512   // threads of the double-float (mixed-precision) Lanczos-step kernels

namespace ocn {

struct MixedLR;  // split-BF16 / tcgen05 state (ocn_mixed.cu)

// Strides between the vectors of a block of psi (chain v = blockIdx.y).
struct BlockStrides {
  size_t vec;   // between vectors: 2*npsi (real plane, imaginary plane)
  size_t part;  // between K-splits of the long-range partial sums
  size_t coef;  // between the coefficient arrays of two chains
  size_t red;   // between the reduction-partial arrays of two chains
};

// Argument records of the Lanczos-step kernels of one context, for launches
// that serve several contexts at once (batched Haydock).
struct CombineArgs {
  const double *pr, *pi, *er, *ei, *allow, *acc, *part;
  int nparts;
  const double2* so;
  double *outr, *outi;
  int nbk, na;
  size_t npsi;
  int use_e0, use_so, backwards;
  const double *oldr, *oldi, *rb_base;
  const int* itp;
  double* red;
  BlockStrides bs;
  const float2 *er_df, *ei_df;  // double-float loop (mixed precision): operator copies
  const float* allow_f;
  const float2* so_f;
  int nv;    // vectors of this context; blocks beyond it return at once
  int nblk;  // blocks per vector of this context (its own launches' grid); blocks beyond return
};

// Kernel classes timed with CUDA events on the context stream when timing is on.
enum TimedClass { T_LR_GEMM1 = 0, T_LR_FFT, T_LR_GEMM2, T_LR_PREP, T_MULT, T_LANCZOS, T_NCLASS };

struct Timing {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[T_NCLASS];
  double total_ms[T_NCLASS] = {0, 0, 0, 0, 0, 0};
  long long count[T_NCLASS] = {0, 0, 0, 0, 0, 0};
};

// Multiplet data packed for the device: valid projectors only.
struct MultDev {
  int np = 0;                  // number of valid (nu, m, l) projectors
  int lmin = 0, lmax = -1, npmax = 0;
  std::vector<int> nproj;
  double2* mpc = nullptr;      // [s][p][k][n] complex (conjugation applied in kernels)
  double* mpm = nullptr;       // packed per l blocks as given (npmax,npmax,nl)
  double2* mh = nullptr;       // concatenated blocks, row ii contiguous
  int* p_l = nullptr;          // per projector: l, m, nu  (device)
  int* p_m = nullptr;
  int* p_nu = nullptr;
  int* d_pfirst = nullptr;     // per l: first projector index of the block
  int* d_nproj = nullptr;      // per l: radial projectors
  long long* d_jbeg = nullptr; // per l: offset of the exchange block in mh
  double2* amp = nullptr;      // [p][a] amplitudes
  double2* amp_part = nullptr; // [chunk][p][a]
  double2* hamp = nullptr;     // [p][a]
  int nchunk = 0;
};

}  // namespace ocn

struct ocn_ctx {
  ocn_dims dims{};
  int nb = 0, nk = 0, nx = 0, na = 0, nspn = 1;
  size_t npsi = 0;           // Nb*Nk*Na
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long launches = 0;

  ocn_system sys{};
  bool have_energies = false, have_allow = false, have_bloch = false, have_W = false;
  bool ei_nonzero = false;   // any Sigma'' != 0 (else the imaginary energy plane is skipped)
  bool acc_valid = false;    // d_acc holds the multiplet term of the current action
  bool have_so = false, have_mult = false;

  // operator data (device)
  double* d_er = nullptr;    // energies (npsi)
  double* d_ei = nullptr;
  double* d_allow = nullptr;
  // operator copies of the mixed-precision (double-float) Haydock loop, rebuilt per run
  float2* d_er_df = nullptr;
  float2* d_ei_df = nullptr;
  float* d_allow_f = nullptr;
  float2* d_so_f = nullptr;
  double2* d_u = nullptr;    // phased Bloch functions, [s][x][k][n] complex (reference order)
  double* d_W = nullptr;     // (Nk, Nx): W[x*Nk + k]
  double2* d_tw = nullptr;   // k-mesh twiddles exp(+2 pi i t / n_axis), [axis][t] (3 x OCN_MAX_KDIM)
  double2* d_so = nullptr;   // (Na,Na) somelr + i someli, [jc*Na + ic]
  std::vector<double> h_so_r, h_so_i;

  // host copies of setup inputs / results
  std::vector<double> h_ur, h_ui;  // raw Bloch functions
  std::vector<double> h_W;
  int xshift[3] = {0, 0, 0};
  double tau_shifted[3] = {0, 0, 0};

  // work buffers
  double2* d_phi = nullptr;        // FP64 path: [k][x][a]
  double* d_acc = nullptr;         // full-store accumulator: re plane then im plane (npsi each)
  double* d_accpart = nullptr;     // long-range partials [split][vector][re|im][npsi]
  int lr_xsplit = 1;
  int mult_parts = 0;              // multiplet partial slices after the LR ones (mixed precision)
  size_t part_stride = 0;          // elements between two splits of d_accpart
  int nvec = 1;                    // largest psi block
  double* d_vec = nullptr;         // general vector pool (see ocn_solvers.cu)
  size_t vec_pool_n = 0;
  double* d_red = nullptr;         // reduction partials
  double* d_scal = nullptr;        // device scalars (a, b, ...)
  int red_blocks = 0;

  ocn::MultDev mult;
  ocn::MixedLR* mixed = nullptr;

  ocn::Timing timing;

  int gmres_lanes = 1;         // energy lanes of the GMRES sweep (ocn_gmres_set_lanes)

  // Haydock early exit (haydockconv.ipt): test parameters and device buffers
  bool conv_on = false;
  ocn_haydock_conv conv{};
  double* d_conv_sp = nullptr;   // 2*ne: the two test spectra
  double* d_conv_rel = nullptr;  // relArea per iteration (hay_cap + 1)
  int conv_cap_ne = 0, conv_cap_iter = 0;

  // Haydock loop: persistent buffers and the captured 3-iteration CUDA graph
  double* hay_vec = nullptr;   // old | psi | h, each 2*npsi
  double* hay_coef = nullptr;  // real_a | imag_a | real_b, each hay_cap+1
  int hay_cap = 0;
  int* d_iter = nullptr;       // device iteration counter
  cudaGraphExec_t hay_exec = nullptr;
  unsigned long long hay_key = 0;
  long long hay_graph_kernels = 0;
  bool use_graphs = true;
  bool capturing = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> graph_events;
};

namespace ocn {

int set_err(ocn_ctx* c, int code, const std::string& msg);
int cuda_fail(ocn_ctx* c, cudaError_t e, const char* what);

#define OCN_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return ocn::cuda_fail(ctx, _e, #call); \
  } while (0)

// Lets kernel f use up to the device's opt-in shared memory per block.  The
// attribute belongs to the function, process-wide: a context of one size must
// not lower it under a live context of another, so it is always set to the
// device maximum (the launch's own request still decides occupancy).
template <class F>
int allow_max_smem(ocn_ctx* c, F* f) {
  int optin = 0;
  cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  return e == cudaSuccess ? 0 : cuda_fail(c, e, "cudaFuncSetAttribute");
}

// Event bracket around one timed launch (no-op unless timing is on).
struct TimedScope {
  ocn_ctx* c;
  int cls;
  cudaEvent_t a = nullptr, b = nullptr;
  TimedScope(ocn_ctx* ctx, int k) : c(ctx), cls(k) {
    if (!c->timing.on) return;
    a = take();
    b = take();
    if (a && b) record(a);
  }
  // Inside stream capture only an "external" record becomes an event-record node.
  void record(cudaEvent_t e) {
    if (c->capturing) cudaEventRecordWithFlags(e, c->stream, cudaEventRecordExternal);
    else cudaEventRecord(e, c->stream);
  }
  ~TimedScope();
  cudaEvent_t take() {
    if (!c->timing.pool.empty()) {
      cudaEvent_t e = c->timing.pool.back();
      c->timing.pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
  }
};

}  // namespace ocn

// Closing event of a timed launch: kept for the next ocn_timing_read, or, while a
// graph is being captured, attached to that graph (read after each replay).
inline ocn::TimedScope::~TimedScope() {
  if (!a || !b) return;
  record(b);
  if (c->capturing) c->graph_events.push_back({cls, {a, b}});
  else c->timing.pending[cls].emplace_back(a, b);
}

namespace ocn {

// ---- host setup (ocn_setup.cpp)
void lrload_shift(const ocn_dims& d, double tau[3], const int ovr[3], int xshift[3]);
void lrload_phase_table(const ocn_dims& d, const int xshift[3], std::vector<double>& c,
                        std::vector<double>& s);  // (Nk, Nx) cos/sin, [x*Nk + k]
void populate_w2(const ocn_dims& d, const ocn_lr_params& p, const double tau[3], const int xshift[3],
                 std::vector<double>& W);
// dL/dptab and dL/d(interactionScale) from dL/dW (index x*Nk + k)
void w2_vjp(const ocn_dims& d, const ocn_lr_params& p, const double tau[3], const int xshift[3],
            const double* G, double* g_ptab, double* g_scale);
void soprep(int core_l, double xi, std::vector<double>& r, std::vector<double>& i);
int redtrid_eigs(int n, const double* ra, const double* rb, double* w);
double gamfcn(double e, double n, double e0);
// nbsemhsetup2 (OCEAN_multiplet.f90:2007-2181): mhr/mhi(mham, mham) of one
// valence l, reference layout, Hartree; returns mham
int mult_exchange_matrix(int lc, int lv, int np, int kfl, int kfh, const double* fk, const double* scfk, int kgl,
                         int kgh, const double* gk, const double* scgk, double scfac, double* mhr, double* mhi);
double gaunt_threey(int ll, int ml, int lm, int mm, int lr, int mr, int conjug);

// ---- FP64 kernels (ocn_kernels.cu)
int upload_twiddles(ocn_ctx* c);
int lr_apply_fp64(ocn_ctx* c, const double* d_pr, const double* d_pi);  // adds into d_acc
int mult_apply(ocn_ctx* c, const double* d_pr, const double* d_pi, double* acc);  // adds into acc
int mult_hamp(ocn_ctx* c, const double2* amp, double2* hamp);  // one vector, [p][a]
// base: binary32 partials on the mixed path, FP64 otherwise
void active_parts(const ocn_ctx* c, const int* hflag, const void** base, int* count);
int phase_bloch(ocn_ctx* c, const double* d_ur, const double* d_ui, const double* d_cos,
                const double* d_sin);
// out = E o in + A o acc + SO in   (acc already holds H_fg + H_lr of A o in), for nv
// vectors at stride vstride (vector v: planes at d_pr + v*vstride, d_pi + v*vstride)
// dL/dW accumulation for one (x, y) pair of GMRES solutions (FP64):
// gW[x*Nk + R] += a Re(D) + b Im(D), D = -(1/Nk) sum_alpha conj(A^y) A^x with
// A^v the band-to-x result of allow o v transformed back over the k-mesh.
// phi: scratch of 2*Nk*Nx*Na complex values.
int lr_wgrad_fp64(ocn_ctx* c, const double* x, const double* y, double2* phi, double a, double b, double* gW);
bool lr_wgrad_supported(const ocn_ctx* c);
int combine(ocn_ctx* c, int nv, const double* d_pr, const double* d_pi, double* d_or, double* d_oi,
            size_t vstride, const int* hflag, int backwards, int v0 = 0);
int zero_acc(ocn_ctx* c, int nv);

// Fused Lanczos step (combine + ocean_hay_ab_twoterm) of nv chains; coefficients stay
// on device, indexed by the device iteration counter *itp (advanced by advance_iter).
int lanczos_launch(ocn_ctx* c, int nv, const double* old, const double* psi, double* h, double* ra,
                   double* ia, double* rb, size_t cstride, const int* itp);
int advance_iter(ocn_ctx* c, int* itp);

// ---- batched Haydock with grouped launches (one launch per stage for all
// member contexts; ocn_kernels.cu / ocn_mixed.cu)
struct BatchMember {
  ocn_ctx* c;
  int nv;
  double* buf[3];  // Haydock vectors: iteration r uses old = buf[r], psi = buf[r+1], h = buf[r+2] (mod 3)
  double *ra, *ia, *rb;
  size_t cstride;
};
struct LzGroup;  // combine + Lanczos stage 2 + iteration counters
struct LrGroup;  // long-range term (tensor-core contractions, transforms, operands) + normalisation
// Why a context cannot join a grouped batch (empty: it can).
std::string batch_group_refusal(const ocn_ctx* c);
int lz_group_create(const std::vector<BatchMember>& mem, LzGroup** out);
int lz_group_advance(LzGroup* g, cudaStream_t s);
int lz_group_step(LzGroup* g, int rot, cudaStream_t s);
int lz_group_launches(const LzGroup* g);
void lz_group_destroy(LzGroup* g);
int lr_group_create(const std::vector<BatchMember>& mem, LrGroup** out);
int lr_group_apply(LrGroup* g, cudaStream_t s);
int lr_group_norm(LrGroup* g, int rot, cudaStream_t s);
int lr_group_launches(const LrGroup* g);
void lr_group_destroy(LrGroup* g);

// ---- the action and the GMRES sweep (ocn_capi.cu, ocn_gmres.cu)
// H*psi on device planes (OCEAN_xact); hflag NULL: the context's switches
int apply_H_impl(ocn_ctx* c, const double* ir, const double* ii, double* orr, double* oi, const int* hflag_in,
                 int backwards);
// H on a block of nv <= nvec vectors (vector v at in + 2 v npsi)
int apply_H_block_impl(ocn_ctx* c, int nv, const double* in, double* out, const int* hflag_in, int backwards,
                       const int* back_each = nullptr);
typedef std::function<int(int step, const double* x)> GmresHook;
// The action and context a GMRES sweep runs on (core or valence).
struct GmresOp {
  size_t n = 0;                  // complex values per vector (planes of n doubles)
  bool dfmt = false;             // double-float basis (mixed-precision contexts)
  int sm_count = 1;
  cudaStream_t stream = nullptr;
  long long* launches = nullptr;
  int nvec = 1;                  // vectors per block action
  const double* allow = nullptr; // device allow mask (n)
  bool mask_ones = false;        // preconditioner from H (allow o 1) (valence runs)
  std::function<int(const double*, double*)> H;             // device planes in, out
  std::function<int(int, const double*, double*)> Hblock;   // nv vectors at stride 2n (may be empty)
  std::function<int(int, const std::string&)> err;          // records an error, returns the code
  std::function<int()> finish;                              // after the sweep (may be empty)
};
int gmres_solve_op(const GmresOp& op, const double* d_rhs, double kpref, const double* elist, int nomega,
                   const ocn_gmres_params* p, int nlanes, double* out_re, double* out_im, double* rel_err,
                   int* iters, const GmresHook* on_x, bool adjoint);
// OCEAN_gmres_do_recycle over the energy list in nlanes lanes; d_rhs: device
// planes of the right-hand side before the allow mask.  on_x: called with each
// energy's solution (device planes) once it has converged.  adjoint: solve
// (w - i Gamma - H) y = b instead.
int gmres_solve(ocn_ctx* c, const double* d_rhs, double kpref, const double* elist, int nomega,
                const ocn_gmres_params* p, int nlanes, double* out_re, double* out_im, double* rel_err,
                int* iters, const GmresHook* on_x, bool adjoint);

// BLAS-1 helpers for GMRES (ocn_kernels.cu); vectors are [re plane | im plane]
int vec_dot_dev(ocn_ctx* c, const double* p, const double* q, double* d_out);
int vec_axmy(ocn_ctx* c, const double* x, double* y, double rv, double iv);
int vec_axmz(ocn_ctx* c, const double* x, double* y, const double* z);
int vec_axpy(ocn_ctx* c, double ar, double ai, const double* x, double* y);
int vec_mul(ocn_ctx* c, const double* x, const double* y, double* z);
int vec_mask_inplace(ocn_ctx* c, double* x);
int vec_divide(ocn_ctx* c, double* x, double rv, double iv);  // x /= rv + i iv
int vec_set_prec(ocn_ctx* c, double energy, double gprc, const double* h, double* out);
int vec_mask_copy(ocn_ctx* c, const double* in, double* out);
int vec_fill(ocn_ctx* c, double* x, double vr, double vi);

// ---- continued fraction (ocn_cf.cu)
int cf_eval(const double* ra, const double* ia, const double* rb, int iter, double kpref,
            const ocn_cf_params* p, double* out, std::string* err,
            const double* ib = nullptr, const double* rc = nullptr, const double* ic = nullptr);
int val_spectrum_eval(const double* ra, const double* ia, const double* rb, const double* ib, const double* rc,
                      const double* ic, int iter, const ocn_val_cf_params* p, double* out, std::string* err);
void val_optical_host(double ere, double er, double ei, double* o);
// check_convergence after the Lanczos step that set *itp (graph-capturable)
int conv_check_launch(ocn_ctx* c, const double* ra, const double* ia, const double* rb, const int* itp);
int cf_eval_noalloc(const double* ra, const double* ia, const double* rb, int iter, double kpref,
                    const ocn_cf_params* p, double* out, std::string* err);

// ---- mixed precision (ocn_mixed.cu)
int mixed_init(ocn_ctx* c);
int mixed_free(ocn_ctx* c);
int mixed_set_bloch(ocn_ctx* c);   // builds split-BF16 layouts from d_u
// Long-range term of nv vectors (vector v: planes d_pr + v*vstride, d_pi + v*vstride)
// into d_accpart; b1_ready: the psi operand was already built (fused Lanczos step)
int lr_apply_mixed(ocn_ctx* c, const double* d_pr, const double* d_pi, size_t vstride, int nv,
                   bool b1_ready = false);
int mixed_prep_b1(ocn_ctx* c, const double* d_pr, const double* d_pi, size_t vstride, int nv);
void mixed_defer_advance(ocn_ctx* c, int* itp);  // the next band -> x launch adds 1 to *itp
bool mixed_take_advance(ocn_ctx* c);             // true (and cleared) if no launch took the request
// b_i = sqrt(partials), psi = h / b_i, and the psi operand of the next action (nv chains)
// Tensor-core partials (binary32) and the double-float Haydock vectors: mixed precision.
inline bool mixed_parts(const ocn_ctx* c) { return c->dims.precision == OCN_PREC_MIXED && c->mixed != nullptr; }
int haydock_to_df(ocn_ctx* c, double* buf, int nv);
// Lanczos stage 2 and the normalisation of nv double-float chains from the combine
// partials: a_{i-1}, b_i, psi = (h - a psi) / b_i in place of h, and the next psi operand
int mixed_norm_prep(ocn_ctx* c, int nv, const double* psi, double* h, double* ra, double* ia, double* rb,
                    size_t cstride, const int* itp);
int mixed_check(ocn_ctx* c);       // reads and clears the device timeout flag
int mixed_set_starve(ocn_ctx* c, int on);  // test hook of ocn_test_starve_tc
// multiplet on the tensor cores: operands from c->mult (after ocn_set_mult), and
// the action's multiplet term of nv vectors into its d_accpart slices
int mixed_set_mult(ocn_ctx* c);
int mult_apply_mixed(ocn_ctx* c, const double* d_pr, const double* d_pi, size_t vstride, int nv,
                     bool b1_ready);
// tile configuration {stages, GEMM2 K splits, GEMM1 grid cap, GEMM2 grid cap,
// k-mesh transforms per CTA, k-mesh transform threads}
int mixed_configure(ocn_ctx* c, const int cfg[7]);
int mixed_config(const ocn_ctx* c, int cfg[7]);
int mixed_autotune(ocn_ctx* c, int nv, int reps, double* best_ms, double* current_ms, int best_cfg[7]);

}  // namespace ocn
