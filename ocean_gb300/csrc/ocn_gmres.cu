// ocn_gmres.cu -- OCEAN_gmres_do_recycle (OCEAN_gmres.f90:508-908) on the GPU.
//
// The reference solves ((w + i Gamma) - H) x = b for one energy after another
// with a GCR-type minimal-residual iteration: u_i = P g (Lorentzian
// preconditioner), au_i = (w + i Gamma) u_i - H u_i, and each step solves the
// normal equations C c = -<au|g> with C_ij = <au_i|au_j> (update_gmres,
// :241-344).  At a new energy it keeps the basis, shifts au_i += dw u_i
// (make_recycle, :207-239) and re-runs the P updates one by one (:667-677),
// which costs O(P^2) passes over the basis per energy.
//
// Here the same iteration runs with three small matrices kept on the host for
// the current basis,
//     C_ij = <au_i|au_j>,  A_ij = <au_i|u_j>,  S_ij = <u_i|u_j>,
// filled one row per inner step by one fused pass over the basis.  An energy
// shift dw is then host algebra (C += dw (A + A^H) + dw^2 S, A += dw S), and
// the recycled solve is one P x P solve against r_j = <au_j|g0> (one pass) plus
// one update pass: O(P) passes per energy.  In exact arithmetic this is the
// reference's result: after the j-th of its P updates the residual is
// orthogonal to au_1..au_j, so the P sequential projections equal the one
// projection onto span(au_1..au_P).
//
// The solution is kept as x + sum_j gamma_j u_j (gamma on the host) and formed
// only where it is read: at a convergence test, before H x at a restart or at
// the next energy, and before the basis is dropped.  The residual g is updated
// explicitly every step (g = ax - b of :823 is kept current by g += sum c au).
//
// Precision.  FP64 contexts keep the basis in FP64 (complex interleaved) and
// form every dot and update in FP64.  Mixed-precision contexts keep it as
// double-float pairs (hi + lo, two binary32 per real: 48 significant bits) and
// form the Gram dots and updates with binary32 FMAs and compensated sums, which
// GB300 runs at 64x its FP64 rate; the normal equations, the solve and the
// residual norms stay FP64.
//
// Energy lanes.  With ocn_gmres_set_lanes the energy list is split into
// contiguous chunks, one per lane; each lane runs the reference's recycled
// sweep over its chunk and the lanes advance in lockstep, so one block action
// (one read of the Bloch functions) serves every lane that needs H in a round.
// One lane is the reference's single sweep.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <vector>

#include "ocn_df.cuh"
#include "ocn_internal.h"

namespace ocn {

namespace {

typedef std::complex<double> cd;
constexpr double EV2HA = 0.036749322175666;
constexpr int GM_THREADS = 256;
constexpr int GM_CTAS_PER_SM = 4;  // target CTAs per SM of the Gram and recycle passes
constexpr int GM_NQ = 10;          // real sums per basis vector in the Gram pass

// double-float helpers: ocn_df.cuh

// Element and accumulator policies of the two basis formats.
template <bool DF>
struct Pol;

template <>
struct Pol<false> {  // FP64, complex interleaved
  typedef double2 E;
  typedef double R;
  struct Acc {
    double v;
    __device__ __forceinline__ void zero() { v = 0.0; }
    __device__ __forceinline__ void fma(R a, R b) { v = __fma_rn(a, b, v); }
    __device__ __forceinline__ double value() const { return v; }
    __device__ __forceinline__ void shfl_add(int o) { v += __shfl_down_sync(0xffffffffu, v, o); }
  };
  static __device__ __forceinline__ E pack(double re, double im) { return make_double2(re, im); }
  static __device__ __forceinline__ R re(const E& e) { return e.x; }
  static __device__ __forceinline__ R im(const E& e) { return e.y; }
  static __device__ __forceinline__ R neg(R r) { return -r; }
  // a + d b, d real (make_recycle's axpy)
  static __device__ __forceinline__ E axpy(const E& a, double d, const E& b) {
    return make_double2(__fma_rn(d, b.x, a.x), __fma_rn(d, b.y, a.y));
  }
};

template <>
struct Pol<true> {  // double-float: (re hi, re lo, im hi, im lo)
  typedef float4 E;
  typedef df R;
  struct Acc {
    float h, l;
    __device__ __forceinline__ void zero() { h = l = 0.0f; }
    __device__ __forceinline__ void fma(R a, R b) { df_fma(h, l, a, b); }
    __device__ __forceinline__ double value() const { return (double)h + (double)l; }
    __device__ __forceinline__ void shfl_add(int o) {
      const float bh = __shfl_down_sync(0xffffffffu, h, o);
      const float bl = __shfl_down_sync(0xffffffffu, l, o);
      df_add(h, l, bh, bl);
    }
  };
  static __device__ __forceinline__ E pack(double re, double im) {
    const df a = df_split(re), b = df_split(im);
    return make_float4(a.h, a.l, b.h, b.l);
  }
  static __device__ __forceinline__ R re(const E& e) { return {e.x, e.y}; }
  static __device__ __forceinline__ R im(const E& e) { return {e.z, e.w}; }
  static __device__ __forceinline__ R neg(R r) { return {-r.h, -r.l}; }
  static __device__ __forceinline__ E axpy(const E& a, double d, const E& b) {
    const df dd = df_split(d);
    float rh = a.x, rl = a.y, ih = a.z, il = a.w;
    df_fma(rh, rl, dd, df{b.x, b.y});
    df_fma(ih, il, dd, df{b.z, b.w});
    const float rs = __fadd_rn(rh, rl), is = __fadd_rn(ih, il);
    return make_float4(rs, __fsub_rn(rl, __fsub_rn(rs, rh)), is, __fsub_rn(il, __fsub_rn(is, ih)));
  }
};

// acc_re + i acc_im += conj(a) b
template <bool DF>
__device__ __forceinline__ void cdot(typename Pol<DF>::Acc& sr, typename Pol<DF>::Acc& si,
                                     const typename Pol<DF>::E& a, const typename Pol<DF>::E& b) {
  typedef Pol<DF> P;
  sr.fma(P::re(a), P::re(b));
  sr.fma(P::im(a), P::im(b));
  si.fma(P::re(a), P::im(b));
  si.fma(P::neg(P::im(a)), P::re(b));
}
// acc_re + i acc_im += c v
template <bool DF>
__device__ __forceinline__ void caxpy(typename Pol<DF>::Acc& sr, typename Pol<DF>::Acc& si,
                                      const typename Pol<DF>::E& c, const typename Pol<DF>::E& v) {
  typedef Pol<DF> P;
  sr.fma(P::re(c), P::re(v));
  sr.fma(P::neg(P::im(c)), P::im(v));
  si.fma(P::re(c), P::im(v));
  si.fma(P::im(c), P::re(v));
}

// Block reduction of K accumulators per thread into K doubles written by
// threads 0..K-1 to out[0..K-1] (fixed order: shuffle tree, then warps in order).
template <bool DF, int K>
__device__ __forceinline__ void block_reduce_out(typename Pol<DF>::Acc (&acc)[K], double* sh, double* out,
                                                 int kvalid) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    for (int o = 16; o > 0; o >>= 1) acc[q].shfl_add(o);
    if (l == 0) sh[w * K + q] = acc[q].value();
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  for (int q = threadIdx.x; q < kvalid; q += blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += sh[i * K + q];
    out[q] = s;
  }
}

// ------------------------------------------------------------------ kernels

// pg = g o pcdiv (OCEAN_psi_3element_mult, OCEAN_gmres.f90:689); the new basis
// vector u = pg and the residual g in basis format.
template <bool DF>
__global__ void __launch_bounds__(GM_THREADS)
    k_gm_prec(const double* __restrict__ g, const double* __restrict__ pcdiv, size_t n, double* __restrict__ pg,
              typename Pol<DF>::E* __restrict__ u, typename Pol<DF>::E* __restrict__ gs) {
  typedef Pol<DF> P;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double a = g[e], b = g[n + e], c = pcdiv[e], d = pcdiv[n + e];
    const double zr = a * c - b * d, zi = a * d + b * c;
    pg[e] = zr;
    pg[n + e] = zi;
    u[e] = P::pack(zr, zi);
    gs[e] = P::pack(a, b);
  }
}

// au = (er + i ei) pg - t   (OCEAN_psi_axmy order, OCEAN_psi.f90:1515-1522)
template <bool DF>
__global__ void __launch_bounds__(GM_THREADS)
    k_gm_form(const double* __restrict__ pg, const double* __restrict__ t, size_t n, double er, double ei,
              typename Pol<DF>::E* __restrict__ au) {
  typedef Pol<DF> P;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double xr = pg[e], xi = pg[n + e];
    const double br = er * xr - t[e];
    const double bi = er * xi - t[n + e];
    au[e] = P::pack(br - ei * xi, bi + ei * xr);
  }
}

// Gram pass of inner step m (0-based basis index of the new vector): for the
// basis vector j = blockIdx.y <= m and the element chunk blockIdx.x, partial
// sums of
//   <au_j|au_m>, <au_j|u_m>, <au_m|u_j>, <u_j|u_m>, <au_j|g>   (re, im each)
// into part[(chunk*(m+1) + j)*10 + q].  u_m and au_m were stored by the two
// kernels before this one; for j == m their values are reused.  The next
// element's five loads are issued before the current element's products (the
// pass is bound by issue and load latency; measured on the 8^3 k / 100-band
// 1s case: 177 us for 60 basis vectors against 385 us with four vectors per
// CTA and no prefetch).
template <bool DF>
__global__ void __launch_bounds__(GM_THREADS, 3)
    k_gm_gram(const typename Pol<DF>::E* __restrict__ ub, const typename Pol<DF>::E* __restrict__ aub, int m,
              size_t n, size_t chunk, const typename Pol<DF>::E* __restrict__ gs, double* __restrict__ part) {
  typedef Pol<DF> P;
  typedef typename P::E E;
  __shared__ double sh[(GM_THREADS / 32) * GM_NQ];
  const int j = blockIdx.y;
  const bool self = j == m;
  const size_t e0 = blockIdx.x * chunk;
  const size_t e1 = min(n, e0 + chunk);
  typename P::Acc acc[GM_NQ];
#pragma unroll
  for (int q = 0; q < GM_NQ; ++q) acc[q].zero();
  const E* __restrict__ um = ub + (size_t)m * n;
  const E* __restrict__ aum = aub + (size_t)m * n;
  const E* __restrict__ uj = ub + (size_t)j * n;
  const E* __restrict__ auj = aub + (size_t)j * n;
  size_t e = e0 + threadIdx.x;
  E U, A, G, Uj, Aj;
  if (e < e1) {
    U = um[e];
    A = aum[e];
    G = gs[e];
    Uj = self ? U : uj[e];
    Aj = self ? A : auj[e];
  }
  for (; e < e1; e += blockDim.x) {
    const size_t en = e + blockDim.x;
    E U2, A2, G2, Uj2, Aj2;
    if (en < e1) {
      U2 = um[en];
      A2 = aum[en];
      G2 = gs[en];
      Uj2 = self ? U2 : uj[en];
      Aj2 = self ? A2 : auj[en];
    }
    cdot<DF>(acc[0], acc[1], Aj, A);
    cdot<DF>(acc[2], acc[3], Aj, U);
    cdot<DF>(acc[4], acc[5], A, Uj);
    cdot<DF>(acc[6], acc[7], Uj, U);
    cdot<DF>(acc[8], acc[9], Aj, G);
    U = U2;
    A = A2;
    G = G2;
    Uj = Uj2;
    Aj = Aj2;
  }
  block_reduce_out<DF, GM_NQ>(acc, sh, part + ((size_t)blockIdx.x * (m + 1) + j) * GM_NQ, GM_NQ);
}

// make_recycle (au_j += dw u_j, OCEAN_gmres.f90:233-236) fused with the
// recycled right-hand side r_j = <au_j|g0>, j = blockIdx.y: part[(chunk*P + j)*2 + q].
template <bool DF>
__global__ void __launch_bounds__(GM_THREADS)
    k_gm_recycle(const typename Pol<DF>::E* __restrict__ ub, typename Pol<DF>::E* __restrict__ aub, int P,
                 size_t n, size_t chunk, double dw, const typename Pol<DF>::E* __restrict__ gs,
                 double* __restrict__ part) {
  typedef Pol<DF> Po;
  typedef typename Po::E E;
  __shared__ double sh[(GM_THREADS / 32) * 2];
  const int j = blockIdx.y;
  const size_t e0 = blockIdx.x * chunk;
  const size_t e1 = min(n, e0 + chunk);
  typename Po::Acc acc[2];
  acc[0].zero();
  acc[1].zero();
  for (size_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const size_t o = (size_t)j * n + e;
    const E A = Po::axpy(aub[o], dw, ub[o]);
    aub[o] = A;
    cdot<DF>(acc[0], acc[1], A, gs[e]);
  }
  block_reduce_out<DF, 2>(acc, sh, part + ((size_t)blockIdx.x * P + j) * 2, 2);
}

// y += sum_j c_j v_j over nvec basis vectors (coefficients in basis format),
// then partial sums over this CTA's elements of |y|^2 and <rhs|y> into
// red[block*3 + q] (when red != NULL).
template <bool DF>
__global__ void __launch_bounds__(GM_THREADS)
    k_gm_combine(const typename Pol<DF>::E* __restrict__ vb, int nvec, const typename Pol<DF>::E* __restrict__ coef,
                 double* __restrict__ y, size_t n, const double* __restrict__ rhs, double* __restrict__ red) {
  typedef Pol<DF> P;
  typedef typename P::E E;
  extern __shared__ __align__(16) unsigned char gm_sm[];
  E* sc = reinterpret_cast<E*>(gm_sm);
  for (int j = threadIdx.x; j < nvec; j += blockDim.x) sc[j] = coef[j];
  __syncthreads();
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    typename P::Acc ar, ai;
    ar.zero();
    ai.zero();
#pragma unroll 4
    for (int j = 0; j < nvec; ++j) caxpy<DF>(ar, ai, sc[j], vb[(size_t)j * n + e]);
    const double yr = y[e] + ar.value();
    const double yi = y[n + e] + ai.value();
    if (nvec > 0) {
      y[e] = yr;
      y[n + e] = yi;
    }
    if (red) {
      s0 += yr * yr + yi * yi;
      if (rhs) {
        const double br = rhs[e], bi = rhs[n + e];
        s1 += br * yr + bi * yi;
        s2 += br * yi - bi * yr;
      }
    }
  }
  if (!red) return;
  __shared__ double shr[(GM_THREADS / 32) * 3];
  typename Pol<false>::Acc acc[3];
  acc[0].v = s0;
  acc[1].v = s1;
  acc[2].v = s2;
  block_reduce_out<false, 3>(acc, shr, red + (size_t)blockIdx.x * 3, 3);
}

// g = (er + i ei) x - t - rhs  (set_initial_vector: ax = (w + i G) x - H x,
// g = ax - b, OCEAN_gmres.f90:1232-1260,823); x == NULL means x = 0 (t unused).
// Optionally the residual in basis format, and |g|^2 partials.
template <bool DF>
__global__ void __launch_bounds__(GM_THREADS)
    k_gm_resid(const double* __restrict__ x, const double* __restrict__ t, const double* __restrict__ rhs, size_t n,
               double er, double ei, double* __restrict__ g, typename Pol<DF>::E* __restrict__ gs,
               double* __restrict__ red) {
  typedef Pol<DF> P;
  double s0 = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    double axr = 0.0, axi = 0.0;
    if (x) {
      const double xr = x[e], xi = x[n + e];
      const double br = er * xr - t[e];
      const double bi = er * xi - t[n + e];
      axr = br - ei * xi;
      axi = bi + ei * xr;
    }
    const double gr = axr - rhs[e], gi = axi - rhs[n + e];
    g[e] = gr;
    g[n + e] = gi;
    if (gs) gs[e] = P::pack(gr, gi);
    s0 += gr * gr + gi * gi;
  }
  __shared__ double shr[(GM_THREADS / 32) * 3];
  typename Pol<false>::Acc acc[3];
  acc[0].v = s0;
  acc[1].v = 0.0;
  acc[2].v = 0.0;
  block_reduce_out<false, 3>(acc, shr, red + (size_t)blockIdx.x * 3, 3);
}

// pcdiv = (E - (h_r + i(h_i + g))) / ((E - h)^2 + g^2), the Lorentzian
// preconditioner of OCEAN_psi_min_set_prec (OCEAN_psi.f90:2961-2965), h = H*1.
__global__ void k_gm_set_prec(double energy, double gprc, const double* __restrict__ h, double* __restrict__ out,
                              size_t n) {
  const double g2 = gprc * gprc;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double hr = h[e], hi = h[n + e];
    const double er = energy - hr, ei = -hi;
    const double dr = er * er - ei * ei + g2, di = 2.0 * er * ei;
    const double nr = energy - hr, ni = -(hi + gprc);
    const double den = dr * dr + di * di;
    out[e] = (nr * dr + ni * di) / den;
    out[n + e] = (ni * dr - nr * di) / den;
  }
}
// out = allow o in (both planes); in == NULL: out = allow o (1, 0)
__global__ void k_gm_mask(const double* __restrict__ in, const double* __restrict__ allow, double* __restrict__ out,
                          size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double m = allow[e];
    out[e] = in ? m * in[e] : m;
    out[n + e] = in ? m * in[n + e] : 0.0;
  }
}
__global__ void k_gm_ones(double* __restrict__ out, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    out[e] = 1.0;
    out[n + e] = 0.0;
  }
}

// out[i] = sum_b part[b*nout + i] for i < nout, one warp per output (lanes take
// b = lane, lane+32, ... in order, then a fixed shuffle tree).
__global__ void k_gm_reduce(const double* __restrict__ part, int nblk, int nout, double* __restrict__ out) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= nout) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += part[(size_t)b * nout + i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) out[i] = s;
}

// ------------------------------------------------------------- host helpers

// Cholesky factor L (L L^H = C) of the Hermitian positive-definite Gram matrix,
// one row at a time (row i needs C(i, 0..i)); L_ij = (C_ij - sum_{k<j} L_ik
// conj(L_jk)) / L_jj with k ascending.
struct Chol {
  int depth = 0;
  std::vector<cd> L;
  void init(int d) {
    depth = d;
    L.assign((size_t)d * d, cd(0.0, 0.0));
  }
  // C: row-major depth x depth with C(i,j) = <au_i|au_j>
  int add_row(int i, const std::vector<cd>& C) {
    cd* Li = L.data() + (size_t)i * depth;
    for (int j = 0; j < i; ++j) {
      cd v = C[(size_t)i * depth + j];
      const cd* Lj = L.data() + (size_t)j * depth;
      for (int k = 0; k < j; ++k) v -= Li[k] * std::conj(Lj[k]);
      Li[j] = v / Lj[j].real();
    }
    double d = C[(size_t)i * depth + i].real();
    for (int k = 0; k < i; ++k) d -= std::norm(Li[k]);
    if (!(d > 0.0)) return i + 1;
    Li[i] = std::sqrt(d);
    return 0;
  }
  // C x = b with the first n rows of L
  void solve(int n, std::vector<cd>& b) const {
    for (int i = 0; i < n; ++i) {
      cd s = b[i];
      for (int k = 0; k < i; ++k) s -= L[(size_t)i * depth + k] * b[k];
      b[i] = s / L[(size_t)i * depth + i].real();
    }
    for (int i = n - 1; i >= 0; --i) {
      cd s = b[i];
      for (int k = i + 1; k < n; ++k) s -= std::conj(L[(size_t)k * depth + i]) * b[k];
      b[i] = s / L[(size_t)i * depth + i].real();
    }
  }
};

// Host split of a complex coefficient into the basis format of the kernels.
struct Coef16 {
  unsigned char b[16];
};
Coef16 pack_coef(bool dfmt, cd c) {
  Coef16 o;
  if (dfmt) {
    float v[4];
    v[0] = (float)c.real();
    v[1] = (float)(c.real() - (double)v[0]);
    v[2] = (float)c.imag();
    v[3] = (float)(c.imag() - (double)v[2]);
    std::memcpy(o.b, v, 16);
  } else {
    double v[2] = {c.real(), c.imag()};
    std::memcpy(o.b, v, 16);
  }
  return o;
}

int grid_n(int sm_count, size_t n) {
  const size_t b = (n + GM_THREADS - 1) / GM_THREADS;
  return (int)std::max<size_t>(1, std::min<size_t>(b, (size_t)4 * sm_count));
}

enum LaneWait { LW_RUN, LW_H, LW_RB, LW_DONE };

enum LanePhase {
  LP_BEGIN,
  LP_INIT_H,      // H x of set_initial_vector arrived
  LP_REC_H,       // H x of a recycled energy arrived
  LP_REC_RB,      // recycled right-hand side read back
  LP_REC_G_RB,    // |g|^2 after the recycled solve read back
  LP_ITER,        // start an inner step
  LP_ITER_H,      // H pg arrived
  LP_ITER_RB,     // Gram row read back
  LP_RESTART_H,   // H x at the restart depth arrived
  LP_G_RB,        // |g|^2 after an inner step read back
  LP_CONV_RB,     // <rhs|x> for the convergence test read back
};

struct Lane {
  int s0 = 0, s1 = 0, s = 0;
  LanePhase ph = LP_BEGIN;
  LaneWait wait = LW_RUN;
  // device
  double *x = nullptr, *g = nullptr, *pcdiv = nullptr;
  unsigned char *ub = nullptr, *aub = nullptr, *gs = nullptr, *coef = nullptr;
  double *part = nullptr, *out = nullptr;
  double* host = nullptr;   // pinned read-back area
  Coef16* hcoef = nullptr;  // pinned coefficient staging
  // H slot of the current round
  int slot = -1;
  double *hin = nullptr, *hout = nullptr;
  // solver state (OCEAN_gmres_do_recycle's locals)
  int P = 0;        // basis vectors in use (prev_iter, then the current step)
  int it = 0;       // current inner step (1-based)
  bool restarted = false;
  bool after_recycle = false;
  double ener = 0.0, prev_energy = -1.0e308;
  int complete_iter = 0, restarts = 0;
  double gval = 0.0, rval = 0.0, ival = 0.0;
  bool xpend = false;  // x + sum gamma_j u_j not yet formed
  std::vector<cd> C, A, S, gam, r;
  Chol chol;
};

}  // namespace

#define GM_CUDA(call)                                                                          \
  do {                                                                                         \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess) return op.err(OCN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Multi-lane recycled GMRES over energies (see the file comment) for any action.
int gmres_solve_op(const GmresOp& op, const double* d_rhs_in, double kpref, const double* elist, int nomega,
                   const ocn_gmres_params* p, int nlanes, double* out_re, double* out_im, double* rel_err,
                   int* iters, const GmresHook* on_x, bool adjoint) {
  const double zs = adjoint ? -1.0 : 1.0;
  const double res = zs * p->resolution, gprc = zs * p->preconditioner;
  const size_t n = op.n;
  const int depth = p->depth;
  const bool dfmt = op.dfmt;
  const int L = std::max(1, std::min(nlanes, nomega));
  const int SM = op.sm_count;
  cudaStream_t stream = op.stream;
  // Gram / recycle chunking: about GM_CTAS_PER_SM CTAs per SM over all basis vectors
  const size_t nchunk_max =
      std::max<size_t>(8, std::min<size_t>((n + 255) / 256, (size_t)GM_CTAS_PER_SM * SM));
  const size_t part_doubles = std::max<size_t>(nchunk_max * (size_t)depth * GM_NQ, (size_t)4 * SM * 3);
  const size_t rb_doubles = (size_t)depth * GM_NQ + 8;
  const size_t host_bytes = rb_doubles * sizeof(double) + (size_t)depth * sizeof(Coef16);

  std::vector<void*> owned;
  unsigned char* host_pool = nullptr;
  auto cleanup = [&]() {
    for (void* q : owned) cudaFree(q);
    if (host_pool) cudaFreeHost(host_pool);
  };
  auto alloc = [&](size_t bytes, void** q) -> int {
    cudaError_t e = cudaMalloc(q, bytes);
    if (e != cudaSuccess) return op.err(OCN_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    owned.push_back(*q);
    return OCN_OK;
  };
  int rc = OCN_OK;
  double *rhs = nullptr, *hpsi1 = nullptr, *ones = nullptr, *hin = nullptr, *hout = nullptr;
  if ((rc = alloc(3 * 2 * n * sizeof(double), (void**)&rhs)) ||
      (rc = alloc((size_t)L * 2 * 2 * n * sizeof(double), (void**)&hin))) {
    cleanup();
    return rc;
  }
  hpsi1 = rhs + 2 * n;
  ones = rhs + 4 * n;
  hout = hin + (size_t)L * 2 * n;
  std::vector<Lane> lanes(L);
  for (int l = 0; l < L && rc == OCN_OK; ++l) {
    Lane& ln = lanes[l];
    ln.s0 = (int)((long long)nomega * l / L);
    ln.s1 = (int)((long long)nomega * (l + 1) / L);
    ln.s = ln.s0;
    unsigned char* q = nullptr;
    const size_t vb = 2 * n * sizeof(double), eb = n * 16;
    const size_t bytes = 3 * vb + (2 * (size_t)depth + 1) * eb + (size_t)depth * 16 +
                         (part_doubles + rb_doubles) * sizeof(double);
    if ((rc = alloc(bytes, (void**)&q))) break;
    ln.x = reinterpret_cast<double*>(q);
    ln.g = ln.x + 2 * n;
    ln.pcdiv = ln.g + 2 * n;
    ln.ub = q + 3 * vb;
    ln.aub = ln.ub + (size_t)depth * eb;
    ln.gs = ln.aub + (size_t)depth * eb;
    ln.coef = ln.gs + eb;
    ln.part = reinterpret_cast<double*>(ln.coef + (size_t)depth * 16);
    ln.out = ln.part + part_doubles;
    ln.C.assign((size_t)depth * depth, cd(0.0, 0.0));
    ln.A = ln.C;
    ln.S = ln.C;
    ln.gam.assign(depth, cd(0.0, 0.0));
    ln.chol.init(depth);
  }
  if (rc == OCN_OK) {
    cudaError_t e = cudaMallocHost((void**)&host_pool, (size_t)L * host_bytes);
    if (e != cudaSuccess) {
      host_pool = nullptr;
      rc = op.err(OCN_ERR_ALLOC, "cudaMallocHost (GMRES read-back)");
    }
  }
  if (rc) {
    cleanup();
    return rc;
  }
  for (int l = 0; l < L; ++l) {
    lanes[l].host = reinterpret_cast<double*>(host_pool + (size_t)l * host_bytes);
    lanes[l].hcoef = reinterpret_cast<Coef16*>(host_pool + (size_t)l * host_bytes + rb_doubles * sizeof(double));
  }

  auto launched = [&]() -> int {
    ++*op.launches;
    GM_CUDA(cudaGetLastError());
    return OCN_OK;
  };
  auto reduce_to = [&](const double* part, int nblk, int nout, double* dout) -> int {
    k_gm_reduce<<<(nout * 32 + 255) / 256, 256, 0, stream>>>(part, nblk, nout, dout);
    return launched();
  };
  auto readback = [&](Lane& ln, const double* dsrc, int count) -> int {
    GM_CUDA(cudaMemcpyAsync(ln.host, dsrc, count * sizeof(double), cudaMemcpyDeviceToHost, stream));
    ln.wait = LW_RB;
    return OCN_OK;
  };
  // y += sum_j coef_j v_j (coefficients staged through this lane's pinned
  // buffer; every path syncs the stream between two of a lane's calls, so the
  // previous copy out of it has completed); want: |y|^2 and <rhs|y> to ln.out
  auto combine_into = [&](Lane& ln, const unsigned char* vb, const std::vector<cd>& cf, int nvec, double* y,
                          bool want) -> int {
    if (nvec > 0) {
      for (int j = 0; j < nvec; ++j) ln.hcoef[j] = pack_coef(dfmt, cf[j]);
      GM_CUDA(cudaMemcpyAsync(ln.coef, ln.hcoef, nvec * sizeof(Coef16), cudaMemcpyHostToDevice, stream));
    }
    const int gb = grid_n(SM, n);
    double* red = want ? ln.part : nullptr;
    const size_t smem = (size_t)std::max(1, nvec) * 16;
    if (dfmt)
      k_gm_combine<true><<<gb, GM_THREADS, smem, stream>>>(reinterpret_cast<const float4*>(vb), nvec,
                                                             reinterpret_cast<const float4*>(ln.coef), y, n,
                                                             rhs, red);
    else
      k_gm_combine<false><<<gb, GM_THREADS, smem, stream>>>(reinterpret_cast<const double2*>(vb), nvec,
                                                              reinterpret_cast<const double2*>(ln.coef), y, n,
                                                              rhs, red);
    int q = launched();
    if (q || !want) return q;
    return reduce_to(ln.part, gb, 3, ln.out);
  };
  // x += sum gamma_j u_j, gamma = 0 (the pending solution formed)
  auto form_x = [&](Lane& ln, bool want) -> int {
    int q = combine_into(ln, ln.ub, ln.gam, ln.xpend ? ln.P : 0, ln.x, want);
    std::fill(ln.gam.begin(), ln.gam.end(), cd(0.0, 0.0));
    ln.xpend = false;
    return q;
  };
  auto resid = [&](Lane& ln, const double* t, bool zero_x, bool want_gs) -> int {
    const int gb = grid_n(SM, n);
    const double* xp = zero_x ? nullptr : ln.x;
    if (dfmt)
      k_gm_resid<true><<<gb, GM_THREADS, 0, stream>>>(xp, t, rhs, n, ln.ener, res, ln.g,
                                                         want_gs ? reinterpret_cast<float4*>(ln.gs) : nullptr,
                                                         ln.part);
    else
      k_gm_resid<false><<<gb, GM_THREADS, 0, stream>>>(xp, t, rhs, n, ln.ener, res, ln.g,
                                                          want_gs ? reinterpret_cast<double2*>(ln.gs) : nullptr,
                                                          ln.part);
    int q = launched();
    if (q) return q;
    return reduce_to(ln.part, gb, 3, ln.out);
  };
  auto set_prec = [&](Lane& ln) -> int {
    ln.prev_energy = ln.ener;
    k_gm_set_prec<<<grid_n(SM, n), GM_THREADS, 0, stream>>>(ln.ener, gprc, hpsi1, ln.pcdiv, n);
    return launched();
  };
  int nreq = 0;
  std::vector<Lane*> hq;
  auto request_H = [&](Lane& ln, const double* src) -> int {
    ln.slot = nreq++;
    ln.hin = hin + (size_t)ln.slot * 2 * n;
    ln.hout = hout + (size_t)ln.slot * 2 * n;
    if (src)
      GM_CUDA(cudaMemcpyAsync(ln.hin, src, 2 * n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    hq.push_back(&ln);
    ln.wait = LW_H;
    return OCN_OK;
  };
  auto finish_energy = [&](Lane& ln) -> int {
    const int st = ln.s;
    if (out_re) out_re[st] = 1.0 - ln.rval * kpref;
    if (out_im) out_im[st] = -ln.ival * kpref;
    if (rel_err) rel_err[st] = -ln.gval / ln.ival;
    if (iters) iters[st] = ln.complete_iter;
    if (on_x) {
      int q = (*on_x)(st, ln.x);
      if (q) return q;
    }
    ++ln.s;
    ln.ph = LP_BEGIN;
    if (ln.s >= ln.s1) ln.wait = LW_DONE;
    return OCN_OK;
  };
  // gval < tol: form x and read <rhs|x> for the relative-error test (:826-842)
  auto conv_test = [&](Lane& ln) -> int {
    int q = form_x(ln, true);
    if (q) return q;
    ln.ph = LP_CONV_RB;
    return readback(ln, ln.out, 3);
  };
  // after an inner step's residual is known and the test did not pass
  auto inner_continue = [&](Lane& ln) -> int {
    if (ln.restarted) {
      ln.restarted = false;
      if (++ln.restarts > std::max(0, p->max_restarts))
        return op.err(OCN_ERR_NOCONV, "GMRES restart cap reached");
    }
    ln.ph = LP_ITER;
    return OCN_OK;
  };
  // the basis is dropped (prev_iter = 0): the pending solution is formed first
  auto drop_basis = [&](Lane& ln) -> int {
    if (ln.xpend) {
      int q = form_x(ln, false);
      if (q) return q;
    }
    ln.P = 0;
    return OCN_OK;
  };

  // One lane until it waits (for H, a read-back) or is done.
  auto advance = [&](Lane& ln) -> int {
    int q;
    for (;;) {
      switch (ln.ph) {
        case LP_BEGIN: {
          ln.ener = elist[ln.s] * EV2HA;
          ln.complete_iter = 0;
          ln.restarts = 0;
          ln.restarted = false;
          if (ln.P == 0 && (q = set_prec(ln))) return q;
          if (ln.P == 0) {
            if (ln.s == ln.s0) {  // set_initial_vector at the lane's first energy: x = 0, g = -b
              GM_CUDA(cudaMemsetAsync(ln.x, 0, 2 * n * sizeof(double), stream));
              if ((q = resid(ln, nullptr, true, false))) return q;
              ln.xpend = false;
              ln.ph = LP_ITER;
              continue;
            }
            ln.ph = LP_INIT_H;  // force_reuse_x: keep x, ax = (w + iG) x - H x (:1232-1260)
            return request_H(ln, ln.x);
          }
          ln.ph = LP_REC_H;
          return request_H(ln, ln.x);
        }
        case LP_INIT_H:
          if ((q = resid(ln, ln.hout, false, false))) return q;
          ln.ph = LP_ITER;
          continue;
        case LP_REC_H: {
          // g0 = (w + iG) x - H x - b, then au_j += dw u_j and r_j = <au_j|g0> in one pass
          if ((q = resid(ln, ln.hout, false, true))) return q;
          const double dw = elist[ln.s] * EV2HA - elist[ln.s - 1] * EV2HA;
          const int ng = ln.P;
          const size_t nch =
              std::max<size_t>(1, std::min<size_t>(nchunk_max, ((size_t)GM_CTAS_PER_SM * SM + ng - 1) / ng));
          const size_t chunk = (n + nch - 1) / nch;
          const dim3 grid((unsigned)nch, (unsigned)ng);
          if (dfmt)
            k_gm_recycle<true><<<grid, GM_THREADS, 0, stream>>>(
                reinterpret_cast<const float4*>(ln.ub), reinterpret_cast<float4*>(ln.aub), ln.P, n, chunk, dw,
                reinterpret_cast<const float4*>(ln.gs), ln.part);
          else
            k_gm_recycle<false><<<grid, GM_THREADS, 0, stream>>>(
                reinterpret_cast<const double2*>(ln.ub), reinterpret_cast<double2*>(ln.aub), ln.P, n, chunk, dw,
                reinterpret_cast<const double2*>(ln.gs), ln.part);
          if ((q = launched()) || (q = reduce_to(ln.part, (int)nch, 2 * ln.P, ln.out))) return q;
          // the same shift on the host matrices: C += dw (A + A^H) + dw^2 S, A += dw S
          for (int i = 0; i < ln.P; ++i)
            for (int j = 0; j < ln.P; ++j) {
              const size_t ij = (size_t)i * depth + j, ji = (size_t)j * depth + i;
              ln.C[ij] += dw * (ln.A[ij] + std::conj(ln.A[ji])) + dw * dw * ln.S[ij];
            }
          for (int i = 0; i < ln.P; ++i)
            for (int j = 0; j < ln.P; ++j) ln.A[(size_t)i * depth + j] += dw * ln.S[(size_t)i * depth + j];
          ln.ph = LP_REC_RB;
          return readback(ln, ln.out, 2 * ln.P);
        }
        case LP_REC_RB: {
          // the recycled solve (the P updates of :667-677 in one projection)
          for (int i = 0; i < ln.P; ++i)
            if (ln.chol.add_row(i, ln.C))
              return op.err(OCN_ERR_SOLVE, "GMRES Gram matrix not positive definite");
          ln.r.assign(ln.P, cd(0.0, 0.0));
          for (int j = 0; j < ln.P; ++j) ln.r[j] = -cd(ln.host[2 * j], ln.host[2 * j + 1]);
          ln.chol.solve(ln.P, ln.r);
          for (int j = 0; j < ln.P; ++j) ln.gam[j] += ln.r[j];
          ln.xpend = true;
          if ((q = combine_into(ln, ln.aub, ln.r, ln.P, ln.g, true))) return q;
          ln.ph = LP_REC_G_RB;
          return readback(ln, ln.out, 1);
        }
        case LP_REC_G_RB:
          ln.gval = ln.host[0];
          if (ln.gval < p->convergence) {
            ln.after_recycle = true;
            return conv_test(ln);
          }
          // PRECONDITIONER OUT OF RANGE (:691-704)
          if (std::fabs(ln.prev_energy - ln.ener) > p->preconditioner / 4.0) {
            if ((q = drop_basis(ln)) || (q = set_prec(ln))) return q;
          }
          ln.ph = LP_ITER;
          continue;
        case LP_CONV_RB: {
          ln.rval = ln.host[1];
          ln.ival = ln.host[2];
          const double rel = -zs * ln.gval / ln.ival;
          if (rel < 0.001 || ln.gval < p->convergence / 10.0) {
            if (!ln.after_recycle && ln.it == depth) ln.P = 0;  // prev_iter = 0 after a restart
            ln.after_recycle = false;
            if ((q = finish_energy(ln))) return q;
            if (ln.wait == LW_DONE) return OCN_OK;
            ln.ph = LP_BEGIN;
            continue;
          }
          if (ln.after_recycle) {
            ln.after_recycle = false;
            if (std::fabs(ln.prev_energy - ln.ener) > p->preconditioner / 4.0) {
              if ((q = drop_basis(ln)) || (q = set_prec(ln))) return q;
            }
            ln.ph = LP_ITER;
            continue;
          }
          if ((q = inner_continue(ln))) return q;
          continue;
        }
        case LP_ITER: {
          ln.it = ln.P + 1;
          ++ln.complete_iter;
          const int m = ln.it - 1;
          const size_t eb = n * 16;
          // the preconditioned residual goes straight into this lane's H slot
          double* pg = hin + (size_t)nreq * 2 * n;
          const int gb = grid_n(SM, n);
          if (dfmt)
            k_gm_prec<true><<<gb, GM_THREADS, 0, stream>>>(ln.g, ln.pcdiv, n, pg,
                                                              reinterpret_cast<float4*>(ln.ub + (size_t)m * eb),
                                                              reinterpret_cast<float4*>(ln.gs));
          else
            k_gm_prec<false><<<gb, GM_THREADS, 0, stream>>>(ln.g, ln.pcdiv, n, pg,
                                                               reinterpret_cast<double2*>(ln.ub + (size_t)m * eb),
                                                               reinterpret_cast<double2*>(ln.gs));
          if ((q = launched())) return q;
          ln.ph = LP_ITER_H;
          return request_H(ln, nullptr);
        }
        case LP_ITER_H: {
          const int m = ln.it - 1;
          const size_t eb = n * 16;
          const int gb = grid_n(SM, n);
          if (dfmt)
            k_gm_form<true><<<gb, GM_THREADS, 0, stream>>>(ln.hin, ln.hout, n, ln.ener, res,
                                                              reinterpret_cast<float4*>(ln.aub + (size_t)m * eb));
          else
            k_gm_form<false><<<gb, GM_THREADS, 0, stream>>>(ln.hin, ln.hout, n, ln.ener, res,
                                                               reinterpret_cast<double2*>(ln.aub + (size_t)m * eb));
          if ((q = launched())) return q;
          const int ng = m + 1;
          const size_t nch =
              std::max<size_t>(1, std::min<size_t>(nchunk_max, ((size_t)GM_CTAS_PER_SM * SM + ng - 1) / ng));
          const size_t chunk = (n + nch - 1) / nch;
          const dim3 grid((unsigned)nch, (unsigned)ng);
          if (dfmt)
            k_gm_gram<true><<<grid, GM_THREADS, 0, stream>>>(
                reinterpret_cast<const float4*>(ln.ub), reinterpret_cast<const float4*>(ln.aub), m, n, chunk,
                reinterpret_cast<const float4*>(ln.gs), ln.part);
          else
            k_gm_gram<false><<<grid, GM_THREADS, 0, stream>>>(
                reinterpret_cast<const double2*>(ln.ub), reinterpret_cast<const double2*>(ln.aub), m, n, chunk,
                reinterpret_cast<const double2*>(ln.gs), ln.part);
          if ((q = launched()) || (q = reduce_to(ln.part, (int)nch, (m + 1) * GM_NQ, ln.out))) return q;
          ln.ph = LP_ITER_RB;
          return readback(ln, ln.out, (m + 1) * GM_NQ);
        }
        case LP_ITER_RB: {
          const int m = ln.it - 1;
          const double* h = ln.host;
          for (int j = 0; j <= m; ++j) {
            const double* v = h + (size_t)j * GM_NQ;
            const cd cjm(v[0], v[1]), ajm(v[2], v[3]), amj(v[4], v[5]), sjm(v[6], v[7]);
            ln.C[(size_t)j * depth + m] = cjm;
            ln.C[(size_t)m * depth + j] = std::conj(cjm);
            ln.A[(size_t)j * depth + m] = ajm;
            ln.A[(size_t)m * depth + j] = amj;
            ln.S[(size_t)j * depth + m] = sjm;
            ln.S[(size_t)m * depth + j] = std::conj(sjm);
          }
          ln.C[(size_t)m * depth + m] = cd(ln.C[(size_t)m * depth + m].real(), 0.0);
          ln.S[(size_t)m * depth + m] = cd(ln.S[(size_t)m * depth + m].real(), 0.0);
          if (ln.chol.add_row(m, ln.C)) return op.err(OCN_ERR_SOLVE, "GMRES Gram matrix not positive definite");
          ln.r.assign(m + 1, cd(0.0, 0.0));
          for (int j = 0; j <= m; ++j) ln.r[j] = -cd(h[(size_t)j * GM_NQ + 8], h[(size_t)j * GM_NQ + 9]);
          ln.chol.solve(m + 1, ln.r);
          for (int j = 0; j <= m; ++j) ln.gam[j] += ln.r[j];
          ln.xpend = true;
          ln.P = ln.it;
          if (ln.it == depth) {  // restart: ax = (w + iG) x - H x from the formed x (:779-819)
            if ((q = form_x(ln, false))) return q;
            ln.ph = LP_RESTART_H;
            return request_H(ln, ln.x);
          }
          if ((q = combine_into(ln, ln.aub, ln.r, m + 1, ln.g, true))) return q;
          ln.ph = LP_G_RB;
          return readback(ln, ln.out, 1);
        }
        case LP_RESTART_H:
          if ((q = resid(ln, ln.hout, false, false))) return q;
          if (ln.ener != ln.prev_energy && (q = set_prec(ln))) return q;
          ln.P = 0;
          ln.restarted = true;
          ln.ph = LP_G_RB;
          return readback(ln, ln.out, 1);
        case LP_G_RB:
          ln.gval = ln.host[0];
          if (ln.gval < p->convergence) return conv_test(ln);
          if ((q = inner_continue(ln))) return q;
          continue;
      }
    }
  };

  // ---- the sweep
  auto run = [&]() -> int {
    int q;
    // rhs = allow o hay (OCEAN_gmres.f90:586); hpsi1 = H (1, 0) (:600-608), with
    // the valence run's allow on the ones first (:603-606)
    k_gm_mask<<<grid_n(SM, n), GM_THREADS, 0, stream>>>(d_rhs_in, op.allow, rhs, n);
    if ((q = launched())) return q;
    if (op.mask_ones)
      k_gm_mask<<<grid_n(SM, n), GM_THREADS, 0, stream>>>(nullptr, op.allow, ones, n);
    else
      k_gm_ones<<<grid_n(SM, n), GM_THREADS, 0, stream>>>(ones, n);
    if ((q = launched())) return q;
    if ((q = op.H(ones, hpsi1))) return q;
    for (;;) {
      bool any_rb = false, all_done = true;
      for (Lane& ln : lanes) {
        if (ln.wait == LW_RUN) {
          if ((q = advance(ln))) return q;
        }
        any_rb = any_rb || ln.wait == LW_RB;
        all_done = all_done && ln.wait == LW_DONE;
      }
      if (all_done) break;
      if (any_rb) {
        GM_CUDA(cudaStreamSynchronize(stream));
        for (Lane& ln : lanes)
          if (ln.wait == LW_RB) ln.wait = LW_RUN;
        continue;
      }
      // every lane waits for H (or is done): one block action over the slots
      if (hq.empty()) return op.err(OCN_ERR_STATE, "GMRES scheduler stalled");
      const int nv = (int)hq.size();
      if (nv == 1 || !op.Hblock) {
        for (int v = 0; v < nv; ++v)
          if ((q = op.H(hin + (size_t)v * 2 * n, hout + (size_t)v * 2 * n))) return q;
      } else {
        for (int v0 = 0; v0 < nv; v0 += op.nvec) {
          const int nb = std::min(op.nvec, nv - v0);
          if ((q = op.Hblock(nb, hin + (size_t)v0 * 2 * n, hout + (size_t)v0 * 2 * n))) return q;
        }
      }
      for (Lane* lp : hq) lp->wait = LW_RUN;
      hq.clear();
      nreq = 0;
    }
    return OCN_OK;
  };
  rc = run();
  cudaError_t e = cudaStreamSynchronize(stream);
  cleanup();
  if (rc) return rc;
  if (e != cudaSuccess) return op.err(OCN_ERR_CUDA, std::string("ocn_gmres: ") + cudaGetErrorString(e));
  if (op.finish) rc = op.finish();
  return rc;
}

int gmres_solve(ocn_ctx* c, const double* d_rhs, double kpref, const double* elist, int nomega,
                const ocn_gmres_params* p, int nlanes, double* out_re, double* out_im, double* rel_err,
                int* iters, const GmresHook* on_x, bool adjoint) {
  GmresOp op;
  op.n = c->npsi;
  op.dfmt = c->dims.precision == OCN_PREC_MIXED;
  op.sm_count = c->sm_count;
  op.stream = c->stream;
  op.launches = &c->launches;
  op.nvec = c->nvec;
  op.allow = c->d_allow;
  op.mask_ones = false;
  const size_t n = c->npsi;
  op.H = [c, n](const double* in, double* out) { return apply_H_impl(c, in, in + n, out, out + n, nullptr, 0); };
  op.Hblock = [c](int nv, const double* in, double* out) { return apply_H_block_impl(c, nv, in, out, nullptr, 0); };
  op.err = [c](int code, const std::string& msg) { return set_err(c, code, msg); };
  if (c->mixed) op.finish = [c]() { return mixed_check(c); };
  return gmres_solve_op(op, d_rhs, kpref, elist, nomega, p, nlanes, out_re, out_im, rel_err, iters, on_x, adjoint);
}

}  // namespace ocn
