// ocn_capi.cu -- the extern "C" boundary of libocean_gpu.so: context and operator
// data management, the H*psi action, and the Haydock and GMRES drivers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <vector>

#include "ocn_internal.h"

namespace {
std::string g_create_err;
}

namespace ocn {

int set_err(ocn_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_err = msg;
  return code;
}

int cuda_fail(ocn_ctx* c, cudaError_t e, const char* what) {
  return set_err(c, OCN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int kernels_init(ocn_ctx* c);  // ocn_kernels.cu

namespace {

template <typename T>
int dev_alloc(ocn_ctx* c, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return OCN_OK;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) return set_err(c, OCN_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return OCN_OK;
}

int require(ocn_ctx* c) {
  if (!c->have_energies && c->sys.e0) return set_err(c, OCN_ERR_STATE, "energies not set");
  if (!c->have_allow) return set_err(c, OCN_ERR_STATE, "allow mask not set");
  if (c->sys.long_range && (!c->have_bloch || !c->have_W))
    return set_err(c, OCN_ERR_STATE, "long-range term on but Bloch functions / W not set");
  return OCN_OK;
}

}  // namespace

// H*psi on device vectors (OCEAN_xact, OCEAN_action.f90:286-618).
int apply_H_impl(ocn_ctx* c, const double* ir, const double* ii, double* orr, double* oi,
                 const int* hflag_in, int backwards) {
  int hflag[6];
  for (int i = 0; i < 6; ++i) hflag[i] = hflag_in ? hflag_in[i] : c->sys.nhflag[i];
  int rc = require(c);
  if (rc) return rc;
  c->acc_valid = false;
  const bool mult_on = c->sys.mult && hflag[4] == 1 && c->have_mult;
  const bool lr_on = c->sys.long_range && hflag[0] == 1;
  if (c->mult_parts > 0) {  // mixed precision with tensor-core multiplet: one psi operand for both
    if ((mult_on || lr_on) && (rc = mixed_prep_b1(c, ir, ii, 0, 1))) return rc;
    if (mult_on && (rc = mult_apply_mixed(c, ir, ii, 0, 1, true))) return rc;
    if (lr_on && (rc = lr_apply_mixed(c, ir, ii, 0, 1, true))) return rc;
    return combine(c, 1, ir, ii, orr, oi, 0, hflag, backwards);
  }
  if (mult_on) {
    if ((rc = zero_acc(c, 1))) return rc;
    if ((rc = mult_apply(c, ir, ii, c->d_acc))) return rc;
    c->acc_valid = true;
  }
  if (lr_on) {
    if (c->dims.precision == OCN_PREC_MIXED) rc = lr_apply_mixed(c, ir, ii, 0, 1);
    else rc = lr_apply_fp64(c, ir, ii);
    if (rc) return rc;
  }
  return combine(c, 1, ir, ii, orr, oi, 0, hflag, backwards);
}

// H on a block of nv vectors (vector v at in + 2*v*npsi) -- mixed precision reads
// the Bloch functions once for the block; the FP64 path acts vector by vector.
// back_each (may be NULL): the backwards switch of each vector (H or H^dagger).
int apply_H_block_impl(ocn_ctx* c, int nv, const double* in, double* out, const int* hflag_in,
                       int backwards, const int* back_each) {
  const size_t n = c->npsi;
  if (nv < 1 || nv > c->nvec) return set_err(c, OCN_ERR_ARG, "block size must be in 1..nvec");
  if (c->dims.precision != OCN_PREC_MIXED) {
    for (int v = 0; v < nv; ++v) {
      int rc = apply_H_impl(c, in + 2 * v * n, in + 2 * v * n + n, out + 2 * v * n, out + 2 * v * n + n,
                            hflag_in, back_each ? back_each[v] : backwards);
      if (rc) return rc;
    }
    return OCN_OK;
  }
  int hflag[6];
  for (int i = 0; i < 6; ++i) hflag[i] = hflag_in ? hflag_in[i] : c->sys.nhflag[i];
  int rc = require(c);
  if (rc) return rc;
  c->acc_valid = false;
  const bool mult_on = c->sys.mult && hflag[4] == 1 && c->have_mult;
  const bool lr_on = c->sys.long_range && hflag[0] == 1;
  bool b1_ready = false;
  if (c->mult_parts > 0 && mult_on) {
    if ((rc = mixed_prep_b1(c, in, in + n, 2 * n, nv)) || (rc = mult_apply_mixed(c, in, in + n, 2 * n, nv, true)))
      return rc;
    b1_ready = true;
  } else if (mult_on) {
    if ((rc = zero_acc(c, nv))) return rc;
    for (int v = 0; v < nv; ++v)
      if ((rc = mult_apply(c, in + 2 * v * n, in + 2 * v * n + n, c->d_acc + 2 * v * n))) return rc;
    c->acc_valid = true;
  }
  if (lr_on && (rc = lr_apply_mixed(c, in, in + n, 2 * n, nv, b1_ready))) return rc;
  if (!back_each) return combine(c, nv, in, in + n, out, out + n, 2 * n, hflag, backwards);
  for (int v = 0; v < nv && rc == OCN_OK; ++v)  // the shared terms are Hermitian; E and SO conjugate per vector
    rc = combine(c, 1, in + 2 * v * n, in + 2 * v * n + n, out + 2 * v * n, out + 2 * v * n + n, 2 * n, hflag,
                 back_each[v], v);
  return rc;
}

}  // namespace ocn

using namespace ocn;

extern "C" {

const char* ocn_version(void) { return "ocean_gb300 0.1 (sm_103a)"; }

int ocn_last_error(const ocn_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return OCN_ERR_ARG;
  const std::string& s = ctx ? ctx->err : g_create_err;
  std::snprintf(buf, len, "%s", s.c_str());
  return OCN_OK;
}

long long ocn_kernel_launches(const ocn_ctx* ctx) { return ctx ? ctx->launches : 0; }

void* ocn_stream(ocn_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

namespace {
void drop_haydock_graph(ocn_ctx* c);
}

int ocn_autotune(ocn_ctx* c, int nv, int reps, double* best_ms, double* current_ms, int tiles[7]) {
  if (!c) return OCN_ERR_ARG;
  if (c->dims.precision != OCN_PREC_MIXED || !c->mixed)
    return set_err(c, OCN_ERR_UNSUPPORTED, "ocn_autotune: tiles exist on the mixed-precision path only");
  cudaSetDevice(c->device);
  drop_haydock_graph(c);  // a captured graph holds the old tiling
  return mixed_autotune(c, nv, reps, best_ms, current_ms, tiles);
}

int ocn_set_tiles(ocn_ctx* c, const int tiles[7]) {
  if (!c || !tiles) return OCN_ERR_ARG;
  if (c->dims.precision != OCN_PREC_MIXED || !c->mixed)
    return set_err(c, OCN_ERR_UNSUPPORTED, "ocn_set_tiles: tiles exist on the mixed-precision path only");
  cudaSetDevice(c->device);
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  drop_haydock_graph(c);
  return mixed_configure(c, tiles);
}

int ocn_test_starve_tc(ocn_ctx* c, int on) {
  if (!c) return OCN_ERR_ARG;
  if (c->dims.precision != OCN_PREC_MIXED || !c->mixed)
    return set_err(c, OCN_ERR_UNSUPPORTED, "ocn_test_starve_tc: mixed-precision contexts only");
  cudaSetDevice(c->device);
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  drop_haydock_graph(c);  // a captured graph holds the launch parameters
  return mixed_set_starve(c, on);
}

int ocn_get_tiles(const ocn_ctx* c, int tiles[7]) {
  if (!c || !tiles) return OCN_ERR_ARG;
  return c->mixed ? mixed_config(c, tiles) : OCN_ERR_UNSUPPORTED;
}

int ocn_timing_enable(ocn_ctx* c, int on) {
  if (!c) return OCN_ERR_ARG;
  c->timing.on = on != 0;
  return OCN_OK;
}

int ocn_timing_read(ocn_ctx* c, long long counts[6], double ms[6]) {
  if (!c) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < T_NCLASS; ++k) {
    for (auto& pr : c->timing.pending[k]) {
      float t = 0.0f;
      if (cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess) {
        c->timing.total_ms[k] += t;
        c->timing.count[k] += 1;
      }
      c->timing.pool.push_back(pr.first);
      c->timing.pool.push_back(pr.second);
    }
    c->timing.pending[k].clear();
    if (counts) counts[k] = c->timing.count[k];
    if (ms) ms[k] = c->timing.total_ms[k];
  }
  return OCN_OK;
}

int ocn_timing_reset(ocn_ctx* c) {
  if (!c) return OCN_ERR_ARG;
  int rc = ocn_timing_read(c, nullptr, nullptr);
  for (int k = 0; k < T_NCLASS; ++k) {
    c->timing.total_ms[k] = 0.0;
    c->timing.count[k] = 0;
  }
  return rc;
}

int ocn_ctx_create(const ocn_dims* d, ocn_ctx** out) {
  if (!d || !out) return set_err(nullptr, OCN_ERR_ARG, "null argument");
  *out = nullptr;
  const int nk = d->kmesh[0] * d->kmesh[1] * d->kmesh[2];
  const int nx = d->xmesh[0] * d->xmesh[1] * d->xmesh[2];
  for (int i = 0; i < 3; ++i) {
    if (d->kmesh[i] < 1 || d->kmesh[i] > OCN_MAX_KDIM)
      return set_err(nullptr, OCN_ERR_ARG, "kmesh extent out of range 1..32");
    if (d->xmesh[i] < 1) return set_err(nullptr, OCN_ERR_ARG, "xmesh extent must be >= 1");
  }
  if (d->num_bands < 1 || d->num_bands > 1024)
    return set_err(nullptr, OCN_ERR_ARG, "num_bands must be in 1..1024");
  if (d->core_l < 0 || d->core_l > 1) return set_err(nullptr, OCN_ERR_ARG, "core_l must be 0 or 1");
  if (d->nalpha != 4 * (2 * d->core_l + 1))
    return set_err(nullptr, OCN_ERR_ARG, "nalpha must equal 4*(2*core_l+1)");
  if (d->nspn != 1 && d->nspn != 2) return set_err(nullptr, OCN_ERR_ARG, "nspn must be 1 or 2");
  if (nk > OCN_MAX_NK) return set_err(nullptr, OCN_ERR_ARG, "k-mesh larger than 4096 points");
  if (sizeof(double2) * (3 * OCN_MAX_KDIM + (size_t)d->nalpha * d->kmesh[0] * d->kmesh[1] * (d->kmesh[2] + 1)) >
      227u * 1024u)
    return set_err(nullptr, OCN_ERR_ARG, "nalpha*Nk too large for the shared-memory k-mesh transform");
  if (d->precision != OCN_PREC_FP64 && d->precision != OCN_PREC_MIXED)
    return set_err(nullptr, OCN_ERR_ARG, "unknown precision");
  if (d->precision == OCN_PREC_MIXED && d->num_bands > 256)
    return set_err(nullptr, OCN_ERR_ARG, "mixed precision supports at most 256 bands");
  if (d->nvec < 0 || d->nvec > 16) return set_err(nullptr, OCN_ERR_ARG, "nvec must be in 0..16");

  ocn_ctx* c = new (std::nothrow) ocn_ctx();
  if (!c) return set_err(nullptr, OCN_ERR_ALLOC, "host allocation failed");
  c->dims = *d;
  c->nvec = d->nvec > 1 ? d->nvec : 1;
  c->nb = d->num_bands;
  c->nk = nk;
  c->nx = nx;
  c->na = d->nalpha;
  c->nspn = d->nspn;
  c->npsi = (size_t)c->nb * nk * c->na;
  c->device = d->device;
  c->sys.celvol = 1.0;
  c->sys.interaction_scale = 1.0;
  c->sys.e0 = 1;
  c->sys.long_range = 1;
  c->sys.mult = 0;
  for (int i = 0; i < 6; ++i) c->sys.nhflag[i] = 1;

  auto fail = [&](int rc) {
    std::string m = c->err;
    ocn_ctx_destroy(c);
    set_err(nullptr, rc, m);
    return rc;
  };
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(cuda_fail(c, e, "cudaSetDevice"));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  c->sm_count = sms > 0 ? sms : 1;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_fail(c, e, "cudaStreamCreate"));

  // Blocks of the Lanczos-step and dot-product kernels: two per SM, or fewer for
  // small vectors (about two elements per thread); each block's partial is
  // re-reduced by every block of the next stage, so extra blocks cost.
  c->red_blocks = (int)std::min<size_t>(2 * (size_t)c->sm_count, std::max<size_t>(1, (c->npsi + 511) / 512));
  c->lr_xsplit = std::max(1, std::min((2 * c->sm_count + nk - 1) / nk, std::max(1, nx / 64)));
  int rc = OCN_OK;
  if ((rc = dev_alloc(c, &c->d_er, c->npsi)) || (rc = dev_alloc(c, &c->d_ei, c->npsi)) ||
      (rc = dev_alloc(c, &c->d_allow, c->npsi)) ||
      (rc = dev_alloc(c, &c->d_u, (size_t)c->nb * nk * nx * c->nspn)) ||
      (rc = dev_alloc(c, &c->d_W, (size_t)nk * nx)) ||
      (rc = dev_alloc(c, &c->d_so, (size_t)c->na * c->na)) ||
      (rc = dev_alloc(c, &c->d_acc, 2 * c->npsi * c->nvec)) ||
      (rc = dev_alloc(c, &c->d_red, (size_t)8 * c->red_blocks * c->nvec)) ||
      (rc = dev_alloc(c, &c->d_scal, 64)))
    return fail(rc);
  if (d->precision == OCN_PREC_FP64) {
    c->part_stride = 2 * c->npsi;  // the FP64 path acts on one vector at a time
    if ((rc = dev_alloc(c, &c->d_phi, (size_t)nk * nx * c->na)) ||
        (rc = dev_alloc(c, &c->d_accpart, (size_t)c->lr_xsplit * c->part_stride)))
      return fail(rc);
  }
  cudaMemsetAsync(c->d_ei, 0, sizeof(double) * c->npsi, c->stream);
  cudaMemsetAsync(c->d_so, 0, sizeof(double2) * c->na * c->na, c->stream);
  if ((rc = upload_twiddles(c)) || (rc = kernels_init(c))) return fail(rc);
  if (d->precision == OCN_PREC_MIXED && (rc = mixed_init(c))) return fail(rc);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(cuda_fail(c, e, "ocn_ctx_create"));
  *out = c;
  return OCN_OK;
}

int ocn_ctx_destroy(ocn_ctx* c) {
  if (!c) return OCN_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->mixed) mixed_free(c);
  void* bufs[] = {c->d_er, c->d_ei, c->d_allow, c->d_u, c->d_W, c->d_tw, c->d_so, c->d_phi, c->d_acc,
                  c->d_accpart, c->d_vec, c->d_red, c->d_scal, c->mult.mpc, c->mult.mpm, c->mult.mh,
                  c->mult.p_l, c->mult.p_m, c->mult.p_nu, c->mult.d_pfirst, c->mult.d_nproj,
                  c->mult.d_jbeg, c->mult.amp, c->mult.amp_part, c->mult.hamp, c->d_er_df, c->d_ei_df,
                  c->d_allow_f, c->d_so_f};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (c->hay_exec) cudaGraphExecDestroy(c->hay_exec);
  for (void* p : {(void*)c->hay_vec, (void*)c->hay_coef, (void*)c->d_iter, (void*)c->d_conv_sp,
                  (void*)c->d_conv_rel})
    if (p) cudaFree(p);
  for (auto& ge : c->graph_events) {
    cudaEventDestroy(ge.second.first);
    cudaEventDestroy(ge.second.second);
  }
  for (int k = 0; k < T_NCLASS; ++k)
    for (auto& pr : c->timing.pending[k]) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  for (cudaEvent_t e : c->timing.pool) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return OCN_OK;
}

int ocn_set_system(ocn_ctx* c, const ocn_system* s) {
  if (!c || !s) return OCN_ERR_ARG;
  if (s->celvol <= 0.0) return set_err(c, OCN_ERR_ARG, "celvol must be positive");
  c->sys = *s;
  return OCN_OK;
}

int ocn_set_energies(ocn_ctx* c, const double* re, const double* im) {
  if (!c || !re) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  OCN_CUDA(c, cudaMemcpyAsync(c->d_er, re, sizeof(double) * c->npsi, cudaMemcpyHostToDevice, c->stream));
  if (im)
    OCN_CUDA(c, cudaMemcpyAsync(c->d_ei, im, sizeof(double) * c->npsi, cudaMemcpyHostToDevice, c->stream));
  else
    OCN_CUDA(c, cudaMemsetAsync(c->d_ei, 0, sizeof(double) * c->npsi, c->stream));
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_energies = true;
  c->ei_nonzero = false;
  if (im)
    for (size_t i = 0; i < c->npsi; ++i)
      if (im[i] != 0.0) {
        c->ei_nonzero = true;
        break;
      }
  return OCN_OK;
}

int ocn_set_allow(ocn_ctx* c, const double* allow) {
  if (!c || !allow) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  OCN_CUDA(c, cudaMemcpyAsync(c->d_allow, allow, sizeof(double) * c->npsi, cudaMemcpyHostToDevice, c->stream));
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_allow = true;
  return OCN_OK;
}

int ocn_set_bloch(ocn_ctx* c, const double* re, const double* im) {
  if (!c || !re || !im) return OCN_ERR_ARG;
  const size_t n = (size_t)c->nb * c->nk * c->nx * c->nspn;
  try {
    c->h_ur.assign(re, re + n);
    c->h_ui.assign(im, im + n);
  } catch (...) {
    return set_err(c, OCN_ERR_ALLOC, "host copy of the Bloch functions failed");
  }
  c->have_bloch = false;  // phased copy produced by ocn_lr_init
  return OCN_OK;
}

int ocn_lr_init(ocn_ctx* c, const ocn_lr_params* p) {
  if (!c || !p || !p->rtab || !p->ptab || p->nptab < 2) return OCN_ERR_ARG;
  if (c->h_ur.empty()) return set_err(c, OCN_ERR_STATE, "ocn_set_bloch must precede ocn_lr_init");
  if (p->epsilon0 <= 0.0) return set_err(c, OCN_ERR_ARG, "epsilon0 must be positive");
  cudaSetDevice(c->device);
  double tau[3] = {p->tau[0], p->tau[1], p->tau[2]};
  int xs[3];
  const int ovr[3] = {p->xshift_override[0], p->xshift_override[1], p->xshift_override[2]};
  lrload_shift(c->dims, tau, ovr, xs);
  std::vector<double> pc, ps;
  lrload_phase_table(c->dims, xs, pc, ps);
  populate_w2(c->dims, *p, tau, xs, c->h_W);
  for (int i = 0; i < 3; ++i) {
    c->xshift[i] = xs[i];
    c->tau_shifted[i] = tau[i];
  }
  const size_t n = c->h_ur.size();
  double *d_raw = nullptr, *d_tab = nullptr;
  int rc = dev_alloc(c, &d_raw, 2 * n);
  if (rc) return rc;
  rc = dev_alloc(c, &d_tab, 2 * pc.size());
  if (rc) {
    cudaFree(d_raw);
    return rc;
  }
  cudaError_t e = cudaMemcpyAsync(d_raw, c->h_ur.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_raw + n, c->h_ui.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_tab, pc.data(), pc.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_tab + pc.size(), ps.data(), ps.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_W, c->h_W.data(), c->h_W.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) rc = phase_bloch(c, d_raw, d_raw + n, d_tab, d_tab + pc.size());
  if (e == cudaSuccess && rc == OCN_OK) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_raw);
  cudaFree(d_tab);
  if (e != cudaSuccess) return cuda_fail(c, e, "ocn_lr_init");
  if (rc) return rc;
  c->have_bloch = true;
  c->have_W = true;
  if (c->dims.precision == OCN_PREC_MIXED) return mixed_set_bloch(c);
  return OCN_OK;
}

int ocn_set_W(ocn_ctx* c, const double* W) {
  if (!c || !W) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  const size_t n = (size_t)c->nk * c->nx;
  c->h_W.assign(W, W + n);
  OCN_CUDA(c, cudaMemcpyAsync(c->d_W, W, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_W = true;
  if (c->dims.precision == OCN_PREC_MIXED && c->have_bloch) return mixed_set_bloch(c);
  return OCN_OK;
}

int ocn_get_W(ocn_ctx* c, double* W, int xshift[3], double tau_shifted[3]) {
  if (!c) return OCN_ERR_ARG;
  if (W) {
    if (c->h_W.empty()) return set_err(c, OCN_ERR_STATE, "W not set");
    std::memcpy(W, c->h_W.data(), c->h_W.size() * sizeof(double));
  }
  for (int i = 0; i < 3; ++i) {
    if (xshift) xshift[i] = c->xshift[i];
    if (tau_shifted) tau_shifted[i] = c->tau_shifted[i];
  }
  return OCN_OK;
}

int ocn_w2_host(const ocn_dims* d, const ocn_lr_params* p, double* W, int xshift[3],
                double tau_shifted[3]) {
  if (!d || !p || !p->rtab || !p->ptab || p->nptab < 2 || p->epsilon0 <= 0.0)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_w2_host: bad argument");
  for (int i = 0; i < 3; ++i)
    if (d->kmesh[i] < 1 || d->xmesh[i] < 1) return set_err(nullptr, OCN_ERR_ARG, "bad mesh");
  double tau[3] = {p->tau[0], p->tau[1], p->tau[2]};
  int xs[3];
  const int ovr[3] = {p->xshift_override[0], p->xshift_override[1], p->xshift_override[2]};
  lrload_shift(*d, tau, ovr, xs);
  std::vector<double> w;
  populate_w2(*d, *p, tau, xs, w);
  if (W) std::memcpy(W, w.data(), w.size() * sizeof(double));
  for (int i = 0; i < 3; ++i) {
    if (xshift) xshift[i] = xs[i];
    if (tau_shifted) tau_shifted[i] = tau[i];
  }
  return OCN_OK;
}

int ocn_phase_table_host(const ocn_dims* d, const int xshift[3], double* ct, double* st) {
  if (!d || !xshift || !ct || !st) return set_err(nullptr, OCN_ERR_ARG, "ocn_phase_table_host: null");
  std::vector<double> c, s;
  lrload_phase_table(*d, xshift, c, s);
  std::memcpy(ct, c.data(), c.size() * sizeof(double));
  std::memcpy(st, s.data(), s.size() * sizeof(double));
  return OCN_OK;
}

int ocn_get_bloch(ocn_ctx* c, double* re, double* im) {
  if (!c || !re || !im) return OCN_ERR_ARG;
  if (!c->have_bloch) return set_err(c, OCN_ERR_STATE, "Bloch functions not initialised");
  cudaSetDevice(c->device);
  const size_t n = (size_t)c->nb * c->nk * c->nx * c->nspn;
  std::vector<double2> tmp(n);
  OCN_CUDA(c, cudaMemcpy(tmp.data(), c->d_u, n * sizeof(double2), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < n; ++i) {
    re[i] = tmp[i].x;
    im[i] = tmp[i].y;
  }
  return OCN_OK;
}

int ocn_set_spin_orbit(ocn_ctx* c, const double* r, const double* im) {
  if (!c || !r || !im) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  const int na = c->na;
  std::vector<double2> so((size_t)na * na);
  for (int j = 0; j < na; ++j)
    for (int i = 0; i < na; ++i) so[(size_t)j * na + i] = make_double2(r[i + na * j], im[i + na * j]);
  c->h_so_r.assign(r, r + (size_t)na * na);
  c->h_so_i.assign(im, im + (size_t)na * na);
  OCN_CUDA(c, cudaMemcpyAsync(c->d_so, so.data(), so.size() * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_so = true;
  return OCN_OK;
}

int ocn_soprep(ocn_ctx* c, double xi) {
  if (!c) return OCN_ERR_ARG;
  std::vector<double> r, im;
  soprep(c->dims.core_l, xi, r, im);
  // have_spin_orbit = .false. when xi < 1e-12 (OCEAN_multiplet.f90:615)
  if (xi < 1.0e-12) {
    c->have_so = false;
    return OCN_OK;
  }
  return ocn_set_spin_orbit(c, r.data(), im.data());
}

int ocn_set_mult(ocn_ctx* c, const ocn_mult_data* m) {
  if (!c || !m || !m->nproj || !m->mpcr || !m->mpci || !m->mpm || !m->mhr || !m->mhi)
    return OCN_ERR_ARG;
  if (m->lmin < 0 || m->lmax < m->lmin) return set_err(c, OCN_ERR_ARG, "bad lmin/lmax");
  cudaSetDevice(c->device);
  MultDev& d = c->mult;
  const int nl = m->lmax - m->lmin + 1;
  int npmax = 0;
  for (int i = 0; i < nl; ++i) {
    if (m->nproj[i] < 0) return set_err(c, OCN_ERR_ARG, "negative nproj");
    npmax = std::max(npmax, m->nproj[i]);
  }
  // valid projector list in the reference's (l, m, nu) order
  std::vector<int> pl, pm, pnu, pfirst(nl), nproj(m->nproj, m->nproj + nl);
  std::vector<long long> jbeg(nl);
  long long jt = 0;
  for (int l = m->lmin; l <= m->lmax; ++l) {
    const int li = l - m->lmin;
    pfirst[li] = (int)pl.size();
    for (int mm = -l; mm <= l; ++mm)
      for (int nu = 0; nu < nproj[li]; ++nu) {
        pl.push_back(l);
        pm.push_back(mm);
        pnu.push_back(nu);
      }
    jbeg[li] = jt;
    const long long mham = (long long)c->na * (2 * l + 1) * nproj[li];
    jt += mham * mham;
  }
  const int np = (int)pl.size();
  const int nbk = c->nb * c->nk;
  const int nm = 2 * m->lmax + 1;
  // repack mpc(nb, nk, npmax, 2lmax+1, nl, nspn) -> [s][p][k*nb + n]
  std::vector<double2> mpc((size_t)c->nspn * np * nbk);
  for (int s = 0; s < c->nspn; ++s)
    for (int p = 0; p < np; ++p) {
      const size_t src = (size_t)nbk * ((size_t)pnu[p] + (size_t)npmax * ((size_t)(pm[p] + m->lmax) +
                                        (size_t)nm * ((size_t)(pl[p] - m->lmin) + (size_t)nl * s)));
      double2* dst = mpc.data() + ((size_t)s * np + p) * nbk;
      for (int e = 0; e < nbk; ++e) dst[e] = make_double2(m->mpcr[src + e], m->mpci[src + e]);
    }
  std::vector<double2> mh((size_t)jt);
  for (long long j = 0; j < jt; ++j) mh[j] = make_double2(m->mhr[j], m->mhi[j]);
  // free a previous set (a captured Haydock graph refers to the old buffers)
  if (c->hay_exec) {
    cudaGraphExecDestroy(c->hay_exec);
    c->hay_exec = nullptr;
  }
  void* old[] = {d.mpc, d.mpm, d.mh, d.p_l, d.p_m, d.p_nu, d.d_pfirst, d.d_nproj, d.d_jbeg,
                 d.amp, d.amp_part, d.hamp};
  for (void* p : old)
    if (p) cudaFree(p);
  d = MultDev();
  d.np = np;
  d.lmin = m->lmin;
  d.lmax = m->lmax;
  d.npmax = npmax;
  d.nproj = nproj;
  const int chunk = 256;
  d.nchunk = (nbk + chunk - 1) / chunk;
  int rc;
  if ((rc = dev_alloc(c, &d.mpc, mpc.size())) || (rc = dev_alloc(c, &d.mpm, (size_t)npmax * npmax * nl)) ||
      (rc = dev_alloc(c, &d.mh, mh.size())) || (rc = dev_alloc(c, &d.p_l, np)) ||
      (rc = dev_alloc(c, &d.p_m, np)) || (rc = dev_alloc(c, &d.p_nu, np)) ||
      (rc = dev_alloc(c, &d.d_pfirst, nl)) || (rc = dev_alloc(c, &d.d_nproj, nl)) ||
      (rc = dev_alloc(c, &d.d_jbeg, nl)) || (rc = dev_alloc(c, &d.amp, (size_t)np * c->na)) ||
      (rc = dev_alloc(c, &d.hamp, (size_t)np * c->na)) ||
      (rc = dev_alloc(c, &d.amp_part, (size_t)d.nchunk * np * c->na)))
    return rc;
  OCN_CUDA(c, cudaMemcpy(d.mpc, mpc.data(), mpc.size() * sizeof(double2), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.mpm, m->mpm, (size_t)npmax * npmax * nl * sizeof(double), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.mh, mh.data(), mh.size() * sizeof(double2), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.p_l, pl.data(), np * sizeof(int), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.p_m, pm.data(), np * sizeof(int), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.p_nu, pnu.data(), np * sizeof(int), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.d_pfirst, pfirst.data(), nl * sizeof(int), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.d_nproj, nproj.data(), nl * sizeof(int), cudaMemcpyHostToDevice));
  OCN_CUDA(c, cudaMemcpy(d.d_jbeg, jbeg.data(), nl * sizeof(long long), cudaMemcpyHostToDevice));
  c->have_mult = true;
  // mixed precision: the projector contractions run on the tensor cores
  if (c->mixed && (rc = mixed_set_mult(c))) return rc;
  return OCN_OK;
}

int ocn_apply_H_dev(ocn_ctx* c, const double* ir, const double* ii, double* orr, double* oi,
                    const int* hflag, int backwards) {
  if (!c || !ir || !ii || !orr || !oi) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  return apply_H_impl(c, ir, ii, orr, oi, hflag, backwards);
}

int ocn_apply_H(ocn_ctx* c, const double* ir, const double* ii, double* orr, double* oi,
                const int* hflag, int backwards) {
  if (!c || !ir || !ii || !orr || !oi) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  double* buf = nullptr;
  int rc = dev_alloc(c, &buf, 4 * n);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(buf, ir, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(buf + n, ii, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) rc = apply_H_impl(c, buf, buf + n, buf + 2 * n, buf + 3 * n, hflag, backwards);
  if (e == cudaSuccess && rc == OCN_OK)
    e = cudaMemcpyAsync(orr, buf + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && rc == OCN_OK)
    e = cudaMemcpyAsync(oi, buf + 3 * n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(c, e, "ocn_apply_H");
  if (rc == OCN_OK && c->mixed) rc = mixed_check(c);
  return rc;
}

// ----------------------------------------------------------------- Haydock

namespace {

// One Haydock iteration (OCEAN_haydock.f90:250-268) of nv chains in lockstep:
// H*psi then the fused two-term Lanczos update, for iteration index *d_iter
// (advanced first).  old/psi/h are block bases (vector v at +2*v*npsi).
int haydock_iteration(ocn_ctx* c, int nv, double* old, double* psi, double* h, double* ra, double* ia,
                      double* rb, size_t cstride) {
  const size_t n = c->npsi;
  int rc;
  // mixed precision: the step's first tensor-core launch advances the iteration counter
  if (mixed_parts(c)) mixed_defer_advance(c, c->d_iter);
  else if ((rc = advance_iter(c, c->d_iter))) return rc;
  c->acc_valid = false;
  if (c->sys.mult && c->sys.nhflag[4] == 1 && c->have_mult) {
    if (c->mult_parts > 0) {  // tensor cores; the psi operand was built with the last normalisation
      if ((rc = mult_apply_mixed(c, psi, psi + n, 2 * n, nv, true))) return rc;
    } else {
      if (mixed_parts(c))  // the FP64 multiplet kernels cannot read the double-float vectors
        return set_err(c, OCN_ERR_STATE, "mixed-precision multiplet operands not built");
      if ((rc = zero_acc(c, nv))) return rc;
      for (int v = 0; v < nv; ++v)
        if ((rc = mult_apply(c, psi + 2 * v * n, psi + 2 * v * n + n, c->d_acc + 2 * v * n))) return rc;
      c->acc_valid = true;
    }
  }
  if (c->sys.long_range && c->sys.nhflag[0] == 1) {
    // mixed: the psi operand was built by the previous normalisation (or before the loop)
    rc = (c->dims.precision == OCN_PREC_MIXED) ? lr_apply_mixed(c, psi, psi + n, 2 * n, nv, true)
                                               : lr_apply_fp64(c, psi, psi + n);
    if (rc) return rc;
  }
  if (mixed_take_advance(c) && (rc = advance_iter(c, c->d_iter))) return rc;  // no term ran a contraction
  rc = lanczos_launch(c, nv, old, psi, h, ra, ia, rb, cstride, c->d_iter);
  if (rc == OCN_OK && c->conv_on && nv == 1) rc = conv_check_launch(c, ra, ia, rb, c->d_iter);
  return rc;
}

void drop_haydock_graph(ocn_ctx* c) {
  if (c->hay_exec) cudaGraphExecDestroy(c->hay_exec);
  c->hay_exec = nullptr;
  for (auto& ge : c->graph_events) {
    c->timing.pool.push_back(ge.second.first);
    c->timing.pool.push_back(ge.second.second);
  }
  c->graph_events.clear();
}

unsigned long long haydock_key(const ocn_ctx* c, int nv) {
  unsigned long long k = reinterpret_cast<uintptr_t>(c->hay_vec) ^
                         (reinterpret_cast<uintptr_t>(c->hay_coef) << 1) ^ ((unsigned long long)c->hay_cap << 40);
  k ^= (unsigned long long)(c->sys.mult ? 1 : 0) << 1;
  k ^= (unsigned long long)(c->sys.long_range ? 1 : 0) << 2;
  k ^= (unsigned long long)(c->sys.e0 ? 1 : 0) << 3;
  k ^= (unsigned long long)(c->timing.on ? 1 : 0) << 4;
  k ^= (unsigned long long)(c->have_mult ? 1 : 0) << 5;
  k ^= (unsigned long long)(c->have_so ? 1 : 0) << 6;
  k ^= (unsigned long long)(c->ei_nonzero ? 1 : 0) << 7;
  for (int i = 0; i < 6; ++i) k ^= (unsigned long long)(c->sys.nhflag[i] & 1) << (8 + i);
  k ^= (unsigned long long)nv << 16;
  if (c->conv_on && nv == 1) {  // the convergence test's launch parameters are part of the graph
    const double v[5] = {c->conv.el, c->conv.eh, c->conv.gam0, c->conv.kpref, (double)c->conv.ne};
    for (int i = 0; i < 5; ++i) {
      unsigned long long b;
      std::memcpy(&b, &v[i], 8);
      k ^= (b * 0x9E3779B97F4A7C15ull) >> (i + 1);
    }
    k ^= ((unsigned long long)c->conv.spacing << 24) ^ (1ull << 23);
    k ^= reinterpret_cast<uintptr_t>(c->d_conv_sp) ^ (reinterpret_cast<uintptr_t>(c->d_conv_rel) << 3);
  }
  return k;
}

// Chains held at once by the Haydock buffers: a block in mixed precision, one
// chain in FP64 (the FP64 block driver runs its chains one after another).
int haydock_chains(const ocn_ctx* c) { return c->dims.precision == OCN_PREC_MIXED ? c->nvec : 1; }

// Buffers of one Haydock run of nv chains on a context (see haydock_prepare).
struct HayRun {
  int nv = 0, niter = 0, hv = 0;
  size_t cap1 = 0;
  double *ra = nullptr, *ia = nullptr, *rb = nullptr;
  double* buf[3] = {nullptr, nullptr, nullptr};  // old, psi, h
};

// Allocates (once) and initialises the Haydock buffers of nv chains from device
// psi0 planes (chain v: p0r + v*vstride, p0i + v*vstride), on the context stream.
int haydock_prepare(ocn_ctx* c, int nv, const double* p0r, const double* p0i, size_t vstride, int niter,
                    HayRun* R) {
  int rc = require(c);
  if (rc) return rc;
  const size_t n = c->npsi;
  const int hv = haydock_chains(c);
  if (nv < 1 || nv > hv) return set_err(c, OCN_ERR_ARG, "block size must be in 1..nvec");
  if (!c->hay_vec && (rc = dev_alloc(c, &c->hay_vec, 6 * n * hv))) return rc;
  if (!c->d_iter && (rc = dev_alloc(c, &c->d_iter, 1))) return rc;
  if (c->hay_cap < niter) {
    drop_haydock_graph(c);
    if (c->hay_coef) cudaFree(c->hay_coef);
    c->hay_coef = nullptr;
    c->hay_cap = 0;
    if ((rc = dev_alloc(c, &c->hay_coef, 3 * (size_t)(niter + 1) * hv))) return rc;
    c->hay_cap = niter;
  }
  // coefficients: [real_a of each chain | imag_a of each chain | real_b of each chain]
  R->nv = nv;
  R->niter = niter;
  R->hv = hv;
  R->cap1 = (size_t)c->hay_cap + 1;
  R->ra = c->hay_coef;
  R->ia = c->hay_coef + hv * R->cap1;
  R->rb = c->hay_coef + 2 * hv * R->cap1;
  R->buf[0] = c->hay_vec;
  R->buf[1] = c->hay_vec + 2 * n * hv;
  R->buf[2] = c->hay_vec + 4 * n * hv;
  cudaError_t e = cudaMemsetAsync(c->hay_coef, 0, 3 * hv * R->cap1 * sizeof(double), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_iter, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(R->buf[0], 0, 2 * n * nv * sizeof(double), c->stream);
  for (int v = 0; v < nv && e == cudaSuccess; ++v) {
    e = cudaMemcpyAsync(R->buf[1] + 2 * v * n, p0r + v * vstride, n * sizeof(double), cudaMemcpyDeviceToDevice,
                        c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R->buf[1] + 2 * v * n + n, p0i + v * vstride, n * sizeof(double),
                          cudaMemcpyDeviceToDevice, c->stream);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "ocn_haydock setup");
  if (c->conv_on && nv == 1) {  // early-exit test buffers (relArea per iteration, two spectra)
    if (c->conv_cap_ne < c->conv.ne || c->conv_cap_iter < c->hay_cap) {
      drop_haydock_graph(c);
      if (c->d_conv_sp) cudaFree(c->d_conv_sp);
      if (c->d_conv_rel) cudaFree(c->d_conv_rel);
      c->d_conv_sp = c->d_conv_rel = nullptr;
      c->conv_cap_ne = c->conv_cap_iter = 0;
      if ((rc = dev_alloc(c, &c->d_conv_sp, 2 * (size_t)c->conv.ne)) ||
          (rc = dev_alloc(c, &c->d_conv_rel, (size_t)c->hay_cap + 1)))
        return rc;
      c->conv_cap_ne = c->conv.ne;
      c->conv_cap_iter = c->hay_cap;
    }
    OCN_CUDA(c, cudaMemsetAsync(c->d_conv_rel, 0, ((size_t)c->hay_cap + 1) * sizeof(double), c->stream));
  }
  if (mixed_parts(c)) {
    mixed_take_advance(c);  // no request of an earlier, failed step carries over
    // first psi operand from the FP64 start vectors, then the loop's double-float form
    if ((rc = mixed_prep_b1(c, R->buf[1], R->buf[1] + n, 2 * n, nv))) return rc;
    if (!c->d_er_df && ((rc = dev_alloc(c, &c->d_er_df, n)) || (rc = dev_alloc(c, &c->d_ei_df, n)) ||
                        (rc = dev_alloc(c, &c->d_allow_f, n)) ||
                        (rc = dev_alloc(c, &c->d_so_f, (size_t)c->na * c->na))))
      return rc;
    if ((rc = haydock_to_df(c, R->buf[1], nv))) return rc;
  }
  return OCN_OK;
}

// The early-exit rule (OCEAN_haydock.f90:268-292) over relArea values of
// iterations from..to (rel indexed by iteration); prev carries prevConv
// across calls.  Returns the stopping iteration or 0.
int conv_stop(const ocn_ctx* c, const std::vector<double>& rel, int from, int to, bool* prev) {
  for (int it = from; it <= to; ++it) {
    if (it <= c->conv.spacing) continue;
    if (rel[it] < c->conv.threshold) {
      if (*prev) return it;
      *prev = true;
    } else {
      *prev = false;
    }
  }
  return 0;
}

// Captures three iterations, which rotate (old, psi, h) back to their starting
// roles, into a graph: one graph serves every launch.
int haydock_capture(ocn_ctx* c, const HayRun& R, cudaGraph_t* out) {
  *out = nullptr;
  OCN_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  c->capturing = true;
  const long long l0 = c->launches;
  double* b[3] = {R.buf[0], R.buf[1], R.buf[2]};
  int rc = OCN_OK;
  for (int r = 0; r < 3 && rc == OCN_OK; ++r) {
    rc = haydock_iteration(c, R.nv, b[0], b[1], b[2], R.ra, R.ia, R.rb, R.cap1);
    double* t = b[0];
    b[0] = b[1];
    b[1] = b[2];
    b[2] = t;
  }
  c->capturing = false;
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
  c->hay_graph_kernels = c->launches - l0;
  c->launches = l0;
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ce != cudaSuccess) return cuda_fail(c, ce, "cudaStreamEndCapture");
  *out = graph;
  return OCN_OK;
}

// Iterations first+1 .. niter launched directly (after 3*k graph iterations the
// buffers are back in their starting roles).
int haydock_remainder(ocn_ctx* c, const HayRun& R, int first, int* done) {
  double* buf[3] = {R.buf[0], R.buf[1], R.buf[2]};
  *done = first;
  for (int it = first + 1; it <= R.niter; ++it) {
    int rc = haydock_iteration(c, R.nv, buf[0], buf[1], buf[2], R.ra, R.ia, R.rb, R.cap1);
    if (rc) return rc;
    double* t = buf[0];
    buf[0] = buf[1];  // old <- psi
    buf[1] = buf[2];  // psi <- h / b
    buf[2] = t;
    *done = it;
  }
  return OCN_OK;
}

// Waits for the run, copies the coefficients of each chain into the host
// arrays (+ v*(niter+1)) and applies the reference's NaN check per chain.
int haydock_finish(ocn_ctx* c, const HayRun& R, int done, bool graph_timing, double* real_a, double* imag_a,
                   double* real_b, int* niter_done) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  std::vector<double> host(3 * R.hv * R.cap1);
  if (e == cudaSuccess)
    e = cudaMemcpy(host.data(), c->hay_coef, host.size() * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "ocn_haydock");
  if (c->timing.on && graph_timing) {  // event pairs of the last graph replay
    for (auto& ge : c->graph_events) {
      float t = 0.0f;
      if (cudaEventElapsedTime(&t, ge.second.first, ge.second.second) == cudaSuccess) {
        c->timing.total_ms[ge.first] += t;
        c->timing.count[ge.first] += 1;
      }
    }
    (void)cudaGetLastError();  // a failed timing query must not poison later calls
  }
  int rc;
  if (c->mixed && (rc = mixed_check(c))) return rc;
  const size_t out1 = (size_t)R.niter + 1;
  for (int v = 0; v < R.nv; ++v)
    for (int i = 0; i <= R.niter; ++i) {
      real_a[v * out1 + i] = host[v * R.cap1 + i];
      if (imag_a) imag_a[v * out1 + i] = host[(R.hv + v) * R.cap1 + i];
      real_b[v * out1 + i] = host[(2 * R.hv + v) * R.cap1 + i];
    }
  // NaN check on a (OCEAN_haydock.f90:913-920): the reference stops at the first
  // NaN; report the iteration count up to it.
  rc = OCN_OK;
  for (int v = 0; v < R.nv; ++v) {
    int dv = done;
    for (int i = 0; i < done; ++i)
      if (std::isnan(real_a[v * out1 + i])) {
        dv = i + 1;
        rc = set_err(c, OCN_ERR_NAN, "NaN detected in Lanczos a");
        break;
      }
    if (niter_done) niter_done[v] = dv;
  }
  return rc;
}

// nv Lanczos chains from device psi0 planes (chain v: p0r + v*vstride, p0i + v*vstride).
// Coefficients land in host arrays real_a/imag_a/real_b + v*(niter+1).
int haydock_run(ocn_ctx* c, int nv, const double* p0r, const double* p0i, size_t vstride, int niter,
                double* real_a, double* imag_a, double* real_b, int* niter_done, bool allow_conv = false) {
  const bool conv_saved = c->conv_on;
  c->conv_on = conv_saved && allow_conv && nv == 1;  // the early exit is for single-chain runs
  struct Restore {
    ocn_ctx* c;
    bool v;
    ~Restore() { c->conv_on = v; }
  } restore{c, conv_saved};
  HayRun R;
  int rc = haydock_prepare(c, nv, p0r, p0i, vstride, niter, &R);
  if (rc) return rc;
  const int ngraph = c->use_graphs ? niter / 3 : 0;
  if (ngraph > 0) {
    const unsigned long long key = haydock_key(c, nv);
    if (!c->hay_exec || key != c->hay_key) {
      drop_haydock_graph(c);
      cudaGraph_t graph = nullptr;
      if ((rc = haydock_capture(c, R, &graph))) return rc;
      cudaError_t ce = cudaGraphInstantiate(&c->hay_exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        c->hay_exec = nullptr;
        return cuda_fail(c, ce, "cudaGraphInstantiate");
      }
      c->hay_key = key;
    }
  }
  const bool conv = c->conv_on && nv == 1;
  std::vector<double> rel(conv ? (size_t)niter + 1 : 0, 0.0);
  bool prev = false;
  int checked = 0, stop = 0;
  // early exit: read the relArea of the steps so far and apply the rule
  auto poll = [&](int upto) -> int {
    OCN_CUDA(c, cudaMemcpyAsync(rel.data() + checked + 1, c->d_conv_rel + checked + 1,
                                (size_t)(upto - checked) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    OCN_CUDA(c, cudaStreamSynchronize(c->stream));
    stop = conv_stop(c, rel, checked + 1, upto, &prev);
    checked = upto;
    return OCN_OK;
  };
  int done = 0;
  for (int g = 0; g < ngraph && !stop; ++g) {
    OCN_CUDA(c, cudaGraphLaunch(c->hay_exec, c->stream));
    c->launches += c->hay_graph_kernels;
    done += 3;
    if (conv && (g % 10 == 9 || g == ngraph - 1) && (rc = poll(done))) return rc;
  }
  if (!stop) {
    rc = haydock_remainder(c, R, done, &done);
    if (rc == OCN_OK && conv && done > checked) rc = poll(done);
  }
  const int rf = haydock_finish(c, R, stop ? stop : done, ngraph > 0, real_a, imag_a, real_b, niter_done);
  if (stop && rf == OCN_OK && rc == OCN_OK)  // the steps computed past the stop are not part of the run
    for (int i = stop; i <= niter; ++i) {
      real_a[i] = 0.0;
      if (imag_a) imag_a[i] = 0.0;
      if (i > stop) real_b[i] = 0.0;
    }
  return rc ? rc : rf;
}

// Block Haydock on device psi0 planes; FP64 contexts run the chains one by one.
int haydock_block_impl(ocn_ctx* c, int nv, const double* d_psi0, int niter, double* real_a, double* imag_a,
                       double* real_b, int* niter_done) {
  const size_t n = c->npsi;
  if (nv < 1 || nv > std::max(c->nvec, 1)) return set_err(c, OCN_ERR_ARG, "block size must be in 1..nvec");
  if (haydock_chains(c) >= nv)
    return haydock_run(c, nv, d_psi0, d_psi0 + n, 2 * n, niter, real_a, imag_a, real_b, niter_done);
  const size_t out1 = (size_t)niter + 1;
  int rc = OCN_OK;
  for (int v = 0; v < nv; ++v) {
    const int r = haydock_run(c, 1, d_psi0 + 2 * v * n, d_psi0 + 2 * v * n + n, 0, niter, real_a + v * out1,
                              imag_a ? imag_a + v * out1 : nullptr, real_b + v * out1,
                              niter_done ? niter_done + v : nullptr);
    if (r == OCN_ERR_NAN) rc = r;
    else if (r) return r;
  }
  return rc;
}

}  // namespace

int ocn_set_haydock_conv(ocn_ctx* c, const ocn_haydock_conv* p) {
  if (!c) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  if (!p || !(p->threshold > 0.0)) {
    if (c->conv_on) drop_haydock_graph(c);
    c->conv_on = false;
    return OCN_OK;
  }
  if (p->spacing < 1 || p->ne < 1 || !(p->eh > p->el) || !(p->gam0 >= 0.0))
    return set_err(c, OCN_ERR_ARG, "ocn_set_haydock_conv: spacing >= 1, ne >= 1, eh > el, gam0 >= 0 required");
  OCN_CUDA(c, cudaStreamSynchronize(c->stream));
  drop_haydock_graph(c);
  c->conv = *p;
  c->conv_on = true;
  return OCN_OK;
}

int ocn_haydock_dev(ocn_ctx* c, const double* p0r, const double* p0i, int niter, double* real_a,
                    double* imag_a, double* real_b, int* niter_done) {
  if (!c || !p0r || !p0i || niter < 1 || !real_a || !real_b) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  return haydock_run(c, 1, p0r, p0i, 0, niter, real_a, imag_a, real_b, niter_done, true);
}

int ocn_haydock(ocn_ctx* c, const double* p0r, const double* p0i, int niter, double* real_a,
                double* imag_a, double* real_b, int* niter_done) {
  if (!c || !p0r || !p0i) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  double* d = nullptr;
  int rc = dev_alloc(c, &d, 2 * n);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(d, p0r, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d + n, p0i, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_fail(c, e, "ocn_haydock upload");
  }
  rc = ocn_haydock_dev(c, d, d + n, niter, real_a, imag_a, real_b, niter_done);
  cudaFree(d);
  return rc;
}

int ocn_haydock_block_dev(ocn_ctx* c, int nv, const double* d_psi0, int niter, double* real_a, double* imag_a,
                          double* real_b, int* niter_done) {
  if (!c || !d_psi0 || niter < 1 || !real_a || !real_b) return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  return haydock_block_impl(c, nv, d_psi0, niter, real_a, imag_a, real_b, niter_done);
}

int ocn_haydock_block(ocn_ctx* c, int nv, const double* p0r, const double* p0i, int niter, double* real_a,
                      double* imag_a, double* real_b, int* niter_done) {
  if (!c || !p0r || !p0i || niter < 1 || !real_a || !real_b) return OCN_ERR_ARG;
  if (nv < 1 || nv > std::max(c->nvec, 1)) return set_err(c, OCN_ERR_ARG, "block size must be in 1..nvec");
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  double* d = nullptr;
  int rc = dev_alloc(c, &d, 2 * n * nv);
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  for (int v = 0; v < nv && e == cudaSuccess; ++v) {
    e = cudaMemcpyAsync(d + 2 * v * n, p0r + v * n, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d + 2 * v * n + n, p0i + v * n, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  }
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_fail(c, e, "ocn_haydock_block upload");
  }
  rc = haydock_block_impl(c, nv, d, niter, real_a, imag_a, real_b, niter_done);
  cudaFree(d);
  return rc;
}

int ocn_haydock_batch(ocn_ctx* const* ctxs, int nctx, const int* nv, const double* const* d_psi0, int niter,
                      double* const* real_a, double* const* imag_a, double* const* real_b,
                      int* const* niter_done) {
  if (!ctxs || nctx < 1 || !nv || !d_psi0 || niter < 1 || !real_a || !real_b) return OCN_ERR_ARG;
  for (int i = 0; i < nctx; ++i) {
    if (!ctxs[i] || !d_psi0[i] || !real_a[i] || !real_b[i]) return OCN_ERR_ARG;
    if (ctxs[i]->device != ctxs[0]->device)
      return set_err(ctxs[i], OCN_ERR_ARG, "ocn_haydock_batch: contexts must share one device");
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == ctxs[i]) return set_err(ctxs[i], OCN_ERR_ARG, "ocn_haydock_batch: context listed twice");
  }
  cudaSetDevice(ctxs[0]->device);
  std::vector<HayRun> R(nctx);
  for (int i = 0; i < nctx; ++i) {
    ocn_ctx* c = ctxs[i];
    const int rc = haydock_prepare(c, nv[i], d_psi0[i], d_psi0[i] + c->npsi, 2 * c->npsi, niter, &R[i]);
    if (rc) return rc;
  }
  // One graph holds three iterations of every context, so a single launch
  // advances all of them.  Contexts that can share launches (mixed precision,
  // long-range term, no multiplet; batch_group_refusal) run as one branch of
  // grouped launches: each stage of the step is one persistent launch over the
  // tiles or vectors of all of them.  The others run as their own branches.
  const int ngraph = niter / 3;
  ocn_ctx* c0 = ctxs[0];
  std::vector<cudaEvent_t> ev(nctx, nullptr);
  cudaGraph_t parent = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<long long> kernels(nctx, 0);
  std::vector<int> grouped, own;
  for (int i = 0; i < nctx; ++i) (batch_group_refusal(ctxs[i]).empty() ? grouped : own).push_back(i);
  const char* nogroup = std::getenv("OCN_BATCH_BRANCHES");  // "1": every context as its own branch
  if (grouped.size() < 2 || (nogroup && nogroup[0] == '1')) {  // one context gains nothing from grouping
    own.insert(own.end(), grouped.begin(), grouped.end());
    grouped.clear();
  }
  LzGroup* lz = nullptr;
  LrGroup* lr = nullptr;
  auto cleanup = [&]() {
    if (exec) cudaGraphExecDestroy(exec);
    if (parent) cudaGraphDestroy(parent);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    lz_group_destroy(lz);
    lr_group_destroy(lr);
  };
  int rc = OCN_OK;
  if (ngraph > 0) {
    cudaError_t e = cudaGraphCreate(&parent, 0);
    if (!grouped.empty() && e == cudaSuccess) {
      std::vector<BatchMember> mem;
      for (int i : grouped)
        mem.push_back(BatchMember{ctxs[i], nv[i], {R[i].buf[0], R[i].buf[1], R[i].buf[2]}, R[i].ra, R[i].ia,
                                  R[i].rb, R[i].cap1});
      ocn_ctx* cg = ctxs[grouped[0]];
      rc = lz_group_create(mem, &lz);
      if (rc == OCN_OK) rc = lr_group_create(mem, &lr);
      if (rc == OCN_OK) {
        cudaGraph_t child = nullptr;
        e = cudaStreamBeginCapture(cg->stream, cudaStreamCaptureModeThreadLocal);
        for (int r = 0; r < 3 && e == cudaSuccess && rc == OCN_OK; ++r) {
          if ((rc = lz_group_advance(lz, cg->stream)) || (rc = lr_group_apply(lr, cg->stream)) ||
              (rc = lz_group_step(lz, r, cg->stream)) || (rc = lr_group_norm(lr, r, cg->stream)))
            rc = set_err(cg, rc, "grouped batched launch failed");
        }
        const cudaError_t ee = cudaStreamEndCapture(cg->stream, &child);
        if (e == cudaSuccess) e = ee;
        if (e == cudaSuccess && rc == OCN_OK) {
          cudaGraphNode_t node;
          e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, child);
          kernels[grouped[0]] = 3 * (lz_group_launches(lz) + lr_group_launches(lr));
        }
        if (child) cudaGraphDestroy(child);
      }
    }
    for (int i : own) {
      if (e != cudaSuccess || rc != OCN_OK) break;
      ocn_ctx* c = ctxs[i];
      const bool timing = c->timing.on;  // event-record nodes stay out of the batch graph
      const long long saved = c->hay_graph_kernels;
      c->timing.on = false;
      cudaGraph_t child = nullptr;
      rc = haydock_capture(c, R[i], &child);
      c->timing.on = timing;
      kernels[i] = c->hay_graph_kernels;
      c->hay_graph_kernels = saved;
      if (rc == OCN_OK) {
        cudaGraphNode_t node;
        e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, child);
        cudaGraphDestroy(child);
      }
    }
    if (rc == OCN_OK && e == cudaSuccess) e = cudaGraphInstantiate(&exec, parent, 0);
    // the launch stream (context 0's) waits for every context's set-up
    for (int i = 0; i < nctx && rc == OCN_OK && e == cudaSuccess; ++i) {
      e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(ev[i], ctxs[i]->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c0->stream, ev[i], 0);
    }
    for (int g = 0; g < ngraph && rc == OCN_OK && e == cudaSuccess; ++g) e = cudaGraphLaunch(exec, c0->stream);
    // and every context continues after the last replay
    if (rc == OCN_OK && e == cudaSuccess) e = cudaEventRecord(ev[0], c0->stream);
    for (int i = 1; i < nctx && rc == OCN_OK && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(ctxs[i]->stream, ev[0], 0);
    if (rc == OCN_OK && e != cudaSuccess) rc = cuda_fail(c0, e, "ocn_haydock_batch graph");
    if (rc == OCN_OK)
      for (int i = 0; i < nctx; ++i) ctxs[i]->launches += (long long)ngraph * kernels[i];
  }
  // remaining iterations on each context's own stream, then the read-backs
  std::vector<int> done(nctx, 3 * ngraph);
  for (int i = 0; i < nctx && rc == OCN_OK; ++i) rc = haydock_remainder(ctxs[i], R[i], 3 * ngraph, &done[i]);
  int worst = rc;
  for (int i = 0; i < nctx; ++i) {
    const int rf = haydock_finish(ctxs[i], R[i], done[i], false, real_a[i], imag_a ? imag_a[i] : nullptr,
                                  real_b[i], niter_done ? niter_done[i] : nullptr);
    if (rf && (worst == OCN_OK || worst == OCN_ERR_NAN)) worst = rf;  // a NaN yields to a harder error
  }
  cleanup();
  return worst;
}

int ocn_apply_H_block(ocn_ctx* c, int nv, const double* ir, const double* ii, double* orr, double* oi,
                      const int* hflag, int backwards) {
  if (!c || !ir || !ii || !orr || !oi) return OCN_ERR_ARG;
  if (nv < 1 || nv > std::max(c->nvec, 1)) return set_err(c, OCN_ERR_ARG, "block size must be in 1..nvec");
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  double* buf = nullptr;
  int rc = dev_alloc(c, &buf, 4 * n * nv);
  if (rc) return rc;
  double* in = buf;
  double* out = buf + 2 * n * nv;
  cudaError_t e = cudaSuccess;
  for (int v = 0; v < nv && e == cudaSuccess; ++v) {
    e = cudaMemcpyAsync(in + 2 * v * n, ir + v * n, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(in + 2 * v * n + n, ii + v * n, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  }
  if (e == cudaSuccess) rc = apply_H_block_impl(c, nv, in, out, hflag, backwards);
  for (int v = 0; v < nv && e == cudaSuccess && rc == OCN_OK; ++v) {
    e = cudaMemcpyAsync(orr + v * n, out + 2 * v * n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(oi + v * n, out + 2 * v * n + n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(c, e, "ocn_apply_H_block");
  if (rc == OCN_OK && c->mixed) rc = mixed_check(c);
  return rc;
}

int ocn_psi_pnorm(int n, int nkpts, double celvol, double* pr, double* pi, double* kpref) {
  if (n < 1 || !pr || !pi || !kpref || nkpts < 1 || celvol <= 0.0) return OCN_ERR_ARG;
  double val = 0.0;
  for (int i = 0; i < n; ++i) val += pr[i] * pr[i] + pi[i] * pi[i];
  val = std::sqrt(val);
  const double pi_ = 3.1415926535897932384626433832795028841971693993751;
  *kpref = 4.0 * pi_ * val * val / ((double)nkpts * celvol * celvol);
  const double inv = 1.0 / val;
  for (int i = 0; i < n; ++i) {
    pr[i] *= inv;
    pi[i] *= inv;
  }
  return OCN_OK;
}

// The two-sided Lanczos of OCEAN_haydock_nonHerm_do (OCEAN_haydock.f90:53-164),
// its step (haydock_abc_1, :1250-1433) written as Saad's algorithm that the
// routine's comments cite; see the header for the stored convention.
int ocn_haydock_nonherm(ocn_ctx* c, const double* psi0_r, const double* psi0_i, int niter, double* real_a,
                        double* imag_a, double* real_b, double* imag_b, double* real_c, double* imag_c,
                        int* niter_done) {
  if (!c || !psi0_r || !psi0_i || niter < 1 || !real_a || !imag_a || !real_b || !imag_b || !real_c || !imag_c)
    return OCN_ERR_ARG;
  cudaSetDevice(c->device);
  int rc = require(c);
  if (rc) return rc;
  const size_t n = c->npsi;
  double* pool = nullptr;
  if ((rc = dev_alloc(c, &pool, 6 * 2 * n))) return rc;
  // three blocks of two adjacent vectors (right, left): current, old, new;
  // with nvec >= 2 the mixed path applies H and H^dagger as one block
  double *cur = pool, *old = pool + 4 * n, *nxt = pool + 8 * n;
  const bool pair = c->dims.precision == OCN_PREC_MIXED && c->mixed && c->nvec >= 2;
  const int back_each[2] = {0, 1};
  for (int i = 0; i <= niter; ++i) real_a[i] = imag_a[i] = real_b[i] = imag_b[i] = real_c[i] = imag_c[i] = 0.0;
  if (niter_done) *niter_done = 0;
  cudaError_t e = cudaMemcpyAsync(cur, psi0_r, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cur + n, psi0_i, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(cur + 2 * n, cur, 2 * n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(old, 0, 4 * n * sizeof(double), c->stream);
  if (e != cudaSuccess) {
    cudaFree(pool);
    return cuda_fail(c, e, "ocn_haydock_nonherm setup");
  }
  auto dot = [&](const double* p, const double* q, double* r, double* i) -> int {  // sum conj(p) q
    int q_ = vec_dot_dev(c, p, q, c->d_scal);
    if (q_) return q_;
    double h[2];
    OCN_CUDA(c, cudaMemcpyAsync(h, c->d_scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    OCN_CUDA(c, cudaStreamSynchronize(c->stream));
    *r = h[0];
    *i = h[1];
    return OCN_OK;
  };
  int done = 0;
  for (int it = 1; it <= niter && rc == OCN_OK; ++it) {
    double* v = cur;
    double* w = cur + 2 * n;
    double* ov = old;
    double* ow = old + 2 * n;
    double* hv = nxt;
    double* hw = nxt + 2 * n;
    double ar = 0, ai = 0, zr = 0, zi = 0;
    if ((rc = vec_mask_inplace(c, v)) || (rc = vec_mask_inplace(c, w))) break;
    if (pair) {
      rc = apply_H_block_impl(c, 2, cur, nxt, nullptr, 0, back_each);
    } else if ((rc = apply_H_impl(c, v, v + n, hv, hv + n, nullptr, 0)) == OCN_OK) {
      rc = apply_H_impl(c, w, w + n, hw, hw + n, nullptr, 1);  // A^H
    }
    if (rc || (rc = vec_mask_inplace(c, hv)) || (rc = vec_mask_inplace(c, hw)) || (rc = dot(w, hv, &ar, &ai)))
      break;
    // beta_j = conj(b_j), conj(delta_j) = c_j
    if ((rc = vec_axpy(c, -real_b[it - 1], imag_b[it - 1], ov, hv)) ||
        (rc = vec_axpy(c, -real_c[it - 1], -imag_c[it - 1], ow, hw)) || (rc = vec_axpy(c, -ar, -ai, v, hv)) ||
        (rc = vec_axpy(c, -ar, ai, w, hw)))
      break;
    real_a[it - 1] = ar;
    imag_a[it - 1] = ai;
    if ((rc = vec_mask_inplace(c, hv)) || (rc = vec_mask_inplace(c, hw)) || (rc = dot(hw, hv, &zr, &zi))) break;
    const double az = std::sqrt(zr * zr + zi * zi);
    const double dr = std::sqrt((az + zr) / 2.0), di = std::copysign(std::sqrt((az - zr) / 2.0), zi);
    // beta = z / delta (Smith's division)
    double br, bi;
    if (std::fabs(dr) >= std::fabs(di)) {
      const double r = di / dr, t = 1.0 / (dr + di * r);
      br = (zr + zi * r) * t;
      bi = (zi - zr * r) * t;
    } else {
      const double r = dr / di, t = 1.0 / (dr * r + di);
      br = (zr * r + zi) * t;
      bi = (zi * r - zr) * t;
    }
    real_b[it] = br;
    imag_b[it] = -bi;
    real_c[it] = dr;
    imag_c[it] = -di;
    if ((rc = vec_divide(c, hw, br, -bi)) || (rc = vec_divide(c, hv, dr, di))) break;  // w^/conj(beta), v^/delta
    double* t = old;  // old <- current, current <- new
    old = cur;
    cur = nxt;
    nxt = t;
    done = it;
    if (std::isnan(ar)) {
      rc = set_err(c, OCN_ERR_NAN, "NaN in the Lanczos a_n");
      break;
    }
  }
  e = cudaStreamSynchronize(c->stream);
  cudaFree(pool);
  if (niter_done) *niter_done = done;
  if (rc == OCN_OK && e != cudaSuccess) rc = cuda_fail(c, e, "ocn_haydock_nonherm");
  if (rc == OCN_OK && c->mixed) rc = mixed_check(c);
  return rc;
}

int ocn_spectrum_cf_bc(const double* real_a, const double* imag_a, const double* real_b, const double* imag_b,
                       const double* real_c, const double* imag_c, int iter, double kpref,
                       const ocn_cf_params* p, double* out) {
  if (!real_a || !real_b || !p || !out) return set_err(nullptr, OCN_ERR_ARG, "null argument");
  std::string err;
  int rc = cf_eval(real_a, imag_a, real_b, iter, kpref, p, out, &err, imag_b, real_c, imag_c);
  if (rc) set_err(nullptr, rc, err);
  return rc;
}

int ocn_val_spectrum(const double* real_a, const double* imag_a, const double* real_b, const double* imag_b,
                     const double* real_c, const double* imag_c, int iter, const ocn_val_cf_params* p, double* out) {
  if (!real_a || !real_b || !p || !out) return set_err(nullptr, OCN_ERR_ARG, "null argument");
  std::string err;
  int rc = val_spectrum_eval(real_a, imag_a, real_b, imag_b, real_c, imag_c, iter, p, out, &err);
  if (rc) set_err(nullptr, rc, err);
  return rc;
}

int ocn_val_optical_constants(int n, const double* omega, const double* eps_re, const double* eps_im, double* out) {
  if (n < 0 || (n > 0 && (!omega || !eps_re || !eps_im || !out)))
    return set_err(nullptr, OCN_ERR_ARG, "ocn_val_optical_constants: bad argument");
  for (int i = 0; i < n; ++i) val_optical_host(omega[i], eps_re[i], eps_im[i], out + 8 * (size_t)i);
  return OCN_OK;
}

int ocn_spectrum_cf(const double* real_a, const double* imag_a, const double* real_b, int iter,
                    double kpref, const ocn_cf_params* p, double* out) {
  if (!real_a || !real_b || !p || !out) return set_err(nullptr, OCN_ERR_ARG, "null argument");
  std::string err;
  int rc = cf_eval(real_a, imag_a, real_b, iter, kpref, p, out, &err);
  if (rc) set_err(nullptr, rc, err);
  return rc;
}

int ocn_spectrum_cf_noalloc(const double* real_a, const double* imag_a, const double* real_b, int iter,
                            double kpref, const ocn_cf_params* p, double* out) {
  if (!real_a || !real_b || !p || !out) return set_err(nullptr, OCN_ERR_ARG, "null argument");
  std::string err;
  int rc = cf_eval_noalloc(real_a, imag_a, real_b, iter, kpref, p, out, &err);
  if (rc) set_err(nullptr, rc, err);
  return rc;
}

int ocn_redtrid(int n, const double* real_a, const double* real_b, double* w) {
  if (n < 0 || !real_a || !real_b || !w) return OCN_ERR_ARG;
  return redtrid_eigs(n, real_a, real_b, w) ? OCN_ERR_SOLVE : OCN_OK;
}

int ocn_gmres_set_lanes(ocn_ctx* c, int nlanes) {
  if (!c) return OCN_ERR_ARG;
  if (nlanes < 1 || nlanes > 64) return set_err(c, OCN_ERR_ARG, "ocn_gmres_set_lanes: nlanes must be in 1..64");
  c->gmres_lanes = nlanes;
  return OCN_OK;
}

namespace {
int gmres_check(ocn_ctx* c, const double* elist, int nomega, const ocn_gmres_params* p) {
  if (!elist || nomega < 1 || !p || p->depth < 1) return set_err(c, OCN_ERR_ARG, "ocn_gmres: bad argument");
  if (p->depth > 1024) return set_err(c, OCN_ERR_ARG, "gmres depth must be <= 1024");
  cudaSetDevice(c->device);
  return require(c);
}
}  // namespace

int ocn_gmres(ocn_ctx* c, const double* hay_r, const double* hay_i, double kpref, const double* elist,
              int nomega, const ocn_gmres_params* p, double* out_re, double* out_im, double* rel_err,
              int* iters) {
  if (!c || !hay_r || !hay_i) return OCN_ERR_ARG;
  int rc = gmres_check(c, elist, nomega, p);
  if (rc) return rc;
  const size_t n = c->npsi;
  double* d_hay = nullptr;
  if ((rc = dev_alloc(c, &d_hay, 2 * n))) return rc;
  cudaError_t e = cudaMemcpyAsync(d_hay, hay_r, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_hay + n, hay_i, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    cudaFree(d_hay);
    return cuda_fail(c, e, "ocn_gmres upload");
  }
  rc = gmres_solve(c, d_hay, kpref, elist, nomega, p, c->gmres_lanes, out_re, out_im, rel_err, iters, nullptr,
                   false);
  cudaStreamSynchronize(c->stream);
  cudaFree(d_hay);
  return rc;
}

int ocn_gmres_dev(ocn_ctx* c, const double* d_hay, double kpref, const double* elist, int nomega,
                  const ocn_gmres_params* p, double* out_re, double* out_im, double* rel_err, int* iters,
                  double* d_x) {
  if (!c || !d_hay) return OCN_ERR_ARG;
  int rc = gmres_check(c, elist, nomega, p);
  if (rc) return rc;
  const size_t n = c->npsi;
  GmresHook keep = [&](int step, const double* x) -> int {
    OCN_CUDA(c, cudaMemcpyAsync(d_x + (size_t)step * 2 * n, x, 2 * n * sizeof(double), cudaMemcpyDeviceToDevice,
                                c->stream));
    return OCN_OK;
  };
  return gmres_solve(c, d_hay, kpref, elist, nomega, p, c->gmres_lanes, out_re, out_im, rel_err, iters,
                     d_x ? &keep : nullptr, false);
}

int ocn_gmres_vjp(ocn_ctx* c, const double* d_hay, double kpref, const double* elist, int nomega,
                  const ocn_gmres_params* p, const double* d_x, const double* grad_re, const double* grad_im,
                  double* g_gamma, double* g_scissor, double* d_gW) {
  if (!c || !d_hay || !elist || nomega < 1 || !p || !d_x || !g_gamma || !g_scissor || !d_gW) return OCN_ERR_ARG;
  if (c->ei_nonzero || c->have_so || c->have_mult)
    return set_err(c, OCN_ERR_UNSUPPORTED, "ocn_gmres_vjp: needs real energies and no multiplet / spin-orbit term");
  if (!lr_wgrad_supported(c))
    return set_err(c, OCN_ERR_UNSUPPORTED, "ocn_gmres_vjp: W gradient needs a cubic k-mesh of 2,3,4,5,6 or 8");
  cudaSetDevice(c->device);
  const size_t n = c->npsi;
  const size_t nkx = (size_t)c->nk * c->nx;
  double2* phi = nullptr;
  int rc = dev_alloc(c, &phi, 2 * nkx * c->na);
  if (rc) return rc;
  cudaError_t e = cudaMemsetAsync(d_gW, 0, nkx * sizeof(double), c->stream);
  if (e != cudaSuccess) {
    cudaFree(phi);
    return cuda_fail(c, e, "ocn_gmres_vjp");
  }
  double gg = 0.0, gs = 0.0;
  // adjoint solve (conj(z) - H) y = rhs: the same recycled GMRES at -Gamma
  GmresHook pair = [&](int step, const double* y) -> int {
    const double* x = d_x + (size_t)step * 2 * n;
    const double a = -kpref * (grad_re ? grad_re[step] : 0.0);
    const double b = -kpref * (grad_im ? grad_im[step] : 0.0);
    int q;
    if ((q = vec_dot_dev(c, y, x, c->d_scal))) return q;
    double yx[2];
    OCN_CUDA(c, cudaMemcpyAsync(yx, c->d_scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    OCN_CUDA(c, cudaStreamSynchronize(c->stream));
    // dF/dGamma = -i <y|x>, dF/d(scissor) = <y|x>  (F = <rhs|x>)
    gg += a * yx[1] - b * yx[0];
    gs += a * yx[0] + b * yx[1];
    return lr_wgrad_fp64(c, x, y, phi, a, b, d_gW);
  };
  rc = gmres_check(c, elist, nomega, p);
  if (rc == OCN_OK)
    rc = gmres_solve(c, d_hay, kpref, elist, nomega, p, c->gmres_lanes, nullptr, nullptr, nullptr, nullptr, &pair,
                     true);
  e = cudaStreamSynchronize(c->stream);
  cudaFree(phi);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(c, e, "ocn_gmres_vjp");
  *g_gamma = gg;
  *g_scissor = gs;
  return OCN_OK;
}

int ocn_mult_exchange(int lc, int lv, int np, int kfl, int kfh, const double* fk, const double* scfk, int kgl,
                      int kgh, const double* gk, const double* scgk, double scfac, double* mhr, double* mhi) {
  if (lc < 0 || lc > 3 || lv < 0 || lv > 5 || np < 1 || !mhr || !mhi)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_mult_exchange: lc in 0..3, lv in 0..5, np >= 1 required");
  if (kfh >= kfl && (kfl < 0 || (kfl & 1) || ((kfh - kfl) & 1) || !fk || !scfk))
    return set_err(nullptr, OCN_ERR_ARG, "ocn_mult_exchange: F^k range must be even with fk and scfk given");
  if (kgh >= kgl && (kgl < 0 || ((kgh - kgl) & 1) || !gk || !scgk))
    return set_err(nullptr, OCN_ERR_ARG, "ocn_mult_exchange: G^k range must step by 2 with gk and scgk given");
  mult_exchange_matrix(lc, lv, np, kfl, kfh, fk, scfk, kgl, kgh, gk, scgk, scfac, mhr, mhi);
  return OCN_OK;
}

double ocn_threey(int ll, int ml, int lm, int mm, int lr, int mr, int conjug) {
  return gaunt_threey(ll, ml, lm, mm, lr, mr, conjug);
}

int ocn_w2_vjp(const ocn_dims* d, const ocn_lr_params* p, const double* G, double* g_ptab, double* g_scale) {
  if (!d || !p || !p->rtab || !p->ptab || p->nptab < 2 || p->epsilon0 <= 0.0 || !G || !g_ptab || !g_scale)
    return set_err(nullptr, OCN_ERR_ARG, "ocn_w2_vjp: bad argument");
  for (int i = 0; i < 3; ++i)
    if (d->kmesh[i] < 1 || d->xmesh[i] < 1) return set_err(nullptr, OCN_ERR_ARG, "bad mesh");
  double tau[3] = {p->tau[0], p->tau[1], p->tau[2]};
  int xs[3];
  const int ovr[3] = {p->xshift_override[0], p->xshift_override[1], p->xshift_override[2]};
  lrload_shift(*d, tau, ovr, xs);
  w2_vjp(*d, *p, tau, xs, G, g_ptab, g_scale);
  return OCN_OK;
}

}  // extern "C"
